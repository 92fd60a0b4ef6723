/*
 * Host stand-ins for the CUDA built-ins that the reference's delay-and-sum
 * kernels use (pycbf/gpu/__engines__.cu), so that g++ compiles that file for
 * the CPU where it lies (and pycbf/gpu/__advanced_engines__.cu, the DMAS
 * kernel).  Test infrastructure only.
 *
 * The reference files need: the __global__ and __device__ qualifiers, the
 * launch coordinates threadIdx / blockIdx / blockDim / gridDim (three
 * unsigned ints each, as CUDA's uint3 / dim3), atomicAdd on float, and the
 * C++ float overloads of
 * abs, sqrt, acos, sin and tan that CUDA's headers provide.  The atomic add
 * becomes a plain add: refgpu_driver.cpp runs the emulated threads one after
 * another, in thread order.  The math functions are the host library's, so
 * trigonometric results may differ from the device's in the last place.
 */
#ifndef REFGPU_SHIM_H
#define REFGPU_SHIM_H

#include <math.h>
#include <stdlib.h>

#include <cmath>

struct rg_coord {
    unsigned int x, y, z;
};

/* launch coordinates of the thread being emulated (set by the driver) */
static rg_coord threadIdx, blockIdx, blockDim, gridDim;

#define __global__
#define __device__

static inline float atomicAdd(float *address, float val)
{
    const float old = *address;
    *address = old + val;
    return old;
}

using std::abs;
using std::acos;
using std::sin;
using std::sqrt;
using std::tan;

#endif
