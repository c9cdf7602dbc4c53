/* src/Rle4.cpp:1 includes <windows.h> for MessageBox only. */
#pragma once
static inline int MessageBoxA(void*, const char*, const char*, int) { return 0; }
static inline int MessageBox(void*, const char*, const char*, int) { return 0; }
