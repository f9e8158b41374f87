/*
 * ref_stub.h — lets the reference's CUDA kernel sections compile as host C++.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref).  The CUDA qualifiers become empty,
 * threadIdx / blockIdx / blockDim become thread-local host variables that the
 * harness sets before calling a kernel body once per emulated thread, and
 * device printf is dropped.  Every standard header the reference includes is
 * included here first, so that its own #include lines are no-ops inside the
 * namespace the harness wraps around it.
 */
#ifndef BDREF_STUB_H
#define BDREF_STUB_H
#define _USE_MATH_DEFINES
#include <cmath>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <iostream>
#include <fstream>

#define __global__
#define __device__
#define __constant__
#define __host__

struct bdref_uint3 { unsigned int x, y, z; };
extern thread_local bdref_uint3 threadIdx;
extern thread_local bdref_uint3 blockIdx;
extern thread_local bdref_uint3 blockDim;

typedef struct { float x, y; } cufftComplex;

inline int cudaDeviceSynchronize() { return 0; }

#endif
