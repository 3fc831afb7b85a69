/*
 * cgfd_oracle_f64.c -- the oracle's time loop evaluated in double precision.
 *
 * TEST INFRASTRUCTURE ONLY (like cgfd_oracle.c): tests/ load it to measure
 * how far the single-precision runs -- the reference's own CPU build (to
 * which cgfd_oracle.c is bit-identical) and the GPU library -- drift from
 * the same discrete scheme evaluated with 53-bit arithmetic.
 *
 * The file compiles cgfd_oracle.c a second time with every `float` of it
 * and of the flat problem description (include/cgfd3d_gpu.h) read as
 * `double`: the problem's arrays, the wavefield, the PML auxiliaries, the
 * seismograms and every intermediate are doubles.  Literal constants keep
 * their single-precision values (the operator coefficients are float
 * literals in cgfd_oracle.c), so the scheme -- operators, RK weights of
 * the float build up to their exact fractions, inputs -- is the one the
 * FP32 runs evaluate, and the difference of an FP32 run from this one is
 * that run's rounding error.  The system headers come first, so that only
 * the oracle's own declarations change type.
 */
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define float double
#define sqrtf sqrt
#define expf exp
#define fabsf fabs
#define fmaxf fmax
#define fminf fmin

#include "cgfd_oracle.c"
