/* Case shim: src/Rle4.cpp includes "bmp.h"; the file is src/Bmp.h. */
#include "Bmp.h"
