/*
 * Stand-in for GSL's gsl_math.h (written for this project): the reference only
 * needs M_PI and friends from <cmath>. TEST INFRASTRUCTURE ONLY.
 */
#ifndef PSPH_SHIM_GSL_MATH_H
#define PSPH_SHIM_GSL_MATH_H
#include <cmath>
#ifndef M_PI
#define M_PI 3.14159265358979323846264338328
#endif
#endif
