/* Included before the reference's own .cu sources (mermake/maxima.cu,
 * mermake/blur.cu) so that g++ compiles them unchanged as C++ for the CPU.
 * The kernels use no shared memory and no barriers, so running each CUDA
 * thread index in turn (ref_driver.cpp) reproduces a launch exactly, apart from
 * the order of atomicAdd slots and the last-ulp behaviour of expf.
 * Test infrastructure only: the built library lands in oracle/_ref/. */
#pragma once
#include <cmath>
#include <algorithm>
struct mm_ref_dim3 { unsigned x, y, z; };
extern mm_ref_dim3 threadIdx, blockIdx, blockDim;
#define __global__
#define __restrict__ __restrict
static inline unsigned atomicAdd(unsigned *p, unsigned v) { unsigned o = *p; *p += v; return o; }
using std::max;
using std::min;
