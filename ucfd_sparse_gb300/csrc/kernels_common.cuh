// kernels_common.cuh -- helpers shared by the kernel headers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "bulk_copy.cuh"
#include "kargs.h"

#ifndef UCFD_KNS
#error "UCFD_KNS (kernel namespace) must be defined by the including translation unit"
#endif

#ifndef UCFD_KEXACT
#define UCFD_KEXACT 0
#endif

namespace UCFD_KNS {

constexpr int kBlock = 256;

// Block LU-SGS storage of the two builds.  The exact build keeps the
// reference's arithmetic: off-diagonal blocks J as given, each face's
// product multiplied by fv = face_area * rcp_vol, LU pivots divided by.
// The fast build (FP32 sweeps and the FP64 fused multiply-add mode) folds fv
// into the stored sweep blocks (J fv, formed once per Prepare in FP64) and
// stores reciprocal pivots in the LU diagonal, so a sweep does no division
// and no per-face scaling, and reads no face areas; its block products go
// straight into the right-hand side (one fused multiply-add per entry).
constexpr bool kFold = !UCFD_KEXACT;

__host__ __device__ inline unsigned grid_for(long long n, int block = kBlock) {
    long long g = (n + block - 1) / block;
    return (unsigned)(g > 0 ? g : 1);
}

// Block-wide sum of a double (blockDim.x multiple of 32, <= 1024); result
// valid in thread 0.
__device__ inline double block_sum(double v) {
    __shared__ double warp_part[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) warp_part[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? warp_part[threadIdx.x] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    }
    return v;
}

}  // namespace UCFD_KNS
