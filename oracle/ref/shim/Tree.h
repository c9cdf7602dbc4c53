/* Case shim: src/Rle4.cpp includes "Tree.h"; the file is src/tree.h. */
#include "tree.h"
