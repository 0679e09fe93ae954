/* Force-included when compiling the reference's src/GeneralUtilities.c (test infrastructure).
 * That file applies isnan to int arrays, which Apple's C library accepts and glibc's type-generic
 * isnan rejects at compile time; for an int the answer is always "not NaN", as here. */
#include <math.h>
#undef isnan
#define isnan(x) ((x) != (x))
