/*
 * real8.h -- TEST INFRASTRUCTURE: forced in front of the oracle's sources
 * (gcc -include) to build liboracle_r8.so, the same restatement with every
 * REAL in double precision -- what the reference's own build with
 * -fdefault-real-8 does (the FP64 error reference of the FP32 step).
 *
 * The parameter block (g3m3_types.h) is read first and keeps its FP32
 * fields: both the FP32 and the FP64 runs start from the same rounded
 * parameters, as the reference's FP64 build does when it is given the FP32
 * run's inputs.  After it, every `float` of the oracle is a double and the
 * single-precision math calls are their double forms.  FP32 literals
 * (1.e-6f and the like) keep their FP32 values promoted.
 */
#ifndef G3M3_ORACLE_REAL8_H
#define G3M3_ORACLE_REAL8_H
#include <math.h>
#include "../include/g3m3_types.h"
#define float double
#define sqrtf sqrt
#define fabsf fabs
#define floorf floor
#endif
