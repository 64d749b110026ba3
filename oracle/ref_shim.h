/*
 * ref_shim.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets the reference's own CUDA kernel source (src/core/cg_solver.cuh,
 * implicit_euler.cuh, newmark_beta.cuh) compile as host C++ so that its
 * kernels can be run as plain loops over particles.  Each kernel thread of
 * the reference writes only its own particle's data, so a loop over the
 * particle index reproduces the kernel exactly.
 *
 * The reference headers (definitions.h, parameters.h, helper_math.h,
 * cutil_math_ext.h, kdtree.h) are included in place from the reference tree
 * (-I<reference>/src/core); nothing from it is copied.  See build_ref.sh.
 */
#ifndef PD_REF_SHIM_H
#define PD_REF_SHIM_H

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>

#include <cuda_runtime.h>   /* host-side vector types and make_* helpers */

#undef __global__
#undef __device__
#undef __host__
#undef __forceinline__
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline

/* one "thread" per particle: blockIdx.x = p, blockDim.x = 1, threadIdx.x = 0 */
static thread_local uint3 blockIdx;
static thread_local uint3 blockDim;
static thread_local uint3 threadIdx;
static inline int __umul24(unsigned a, unsigned b) { return (int)(a * b); }
static inline int __mul24(int a, int b) { return a * b; }
static inline void __syncthreads() {}

#include "helper_math.h"
#include "cutil_math_ext.h"
#include "definitions.h"
#include "parameters.h"
#include "kdtree.h"

#endif
