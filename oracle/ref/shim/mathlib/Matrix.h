/* Case shim: src/VecMath.h includes "mathlib/Matrix.h"; the file is inc/mathlib/matrix.h. */
#include "mathlib/matrix.h"
