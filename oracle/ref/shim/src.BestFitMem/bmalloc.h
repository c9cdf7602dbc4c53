/* The reference's bump allocator (src.BestFitMem/bmalloc.h) is not in the
 * published tree.  Only its declarations are needed to compile the host
 * code; the harness never calls into it. */
#pragma once
void* bmalloc(int size);
void add_pool(void* pool, int size);
