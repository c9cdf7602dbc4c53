/* Case shim: src/VecMath.h includes "mathlib/Vector.h"; the file is inc/mathlib/vector.h. */
#include "mathlib/vector.h"
