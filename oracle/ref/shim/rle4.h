/* Case shim: src/tree.h includes "rle4.h"; the file is src/Rle4.h. */
#include "Rle4.h"
