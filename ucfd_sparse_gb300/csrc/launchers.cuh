// launchers.cuh -- definitions of the launch.h declarations for the
// namespace UCFD_KNS; included once by each kernel translation unit.
#pragma once

#include "launch.h"
#include "kernels_lusgs.cuh"
#include "kernels_blusgs.cuh"
#include "kernels_krylov.cuh"
#include "kernels_adjoint.cuh"
#include "ucfd_internal.h"

namespace UCFD_KNS {

// ---- adjoint of the colored LU-SGS step --------------------------------------
template <typename T>
void adj_upper(const ::ucfd::AdjArgs &a, int nfv, int ndims, T gamma, T pmin, const T *fnv, const T *vec,
               const T *fspr, const T *upts, const T *diag, const T *dub, const T *dq, const T *gdq, T *qbar, T *dbar,
               T *gfspr, cudaStream_t s) {
    const int n = a.t1 - a.t0;
    if (n <= 0) return;
    if (nfv == 5 && ndims == 3)
        adj_upper_kernel<T, 5, 5, 3><<<grid_for(n), kBlock, 0, s>>>(a, gamma, pmin, fnv, vec, fspr, upts, diag, dub,
                                                                     dq, gdq, qbar, dbar, gfspr);
    else if (nfv == 4 && ndims == 2)
        adj_upper_kernel<T, 4, 4, 2><<<grid_for(n), kBlock, 0, s>>>(a, gamma, pmin, fnv, vec, fspr, upts, diag, dub,
                                                                     dq, gdq, qbar, dbar, gfspr);
    else
        ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "adjoint built for nfvars/ndims 5/3 and 4/2 only");
}

template <typename T>
void adj_lower(const ::ucfd::AdjArgs &a, int nfv, int ndims, T gamma, T pmin, T factor, const T *fnv, const T *vec,
               const T *fspr, const T *dt, const T *upts, const T *diag, const T *dub, const T *qbar, T *wbuf,
               const T *dbar, T *grhs, T *gdt, T *gfspr, cudaStream_t s) {
    const int n = a.t1 - a.t0;
    if (n <= 0) return;
    if (nfv == 5 && ndims == 3)
        adj_lower_kernel<T, 5, 5, 3><<<grid_for(n), kBlock, 0, s>>>(a, gamma, pmin, factor, fnv, vec, fspr, dt, upts,
                                                                     diag, dub, qbar, wbuf, dbar, grhs, gdt, gfspr);
    else if (nfv == 4 && ndims == 2)
        adj_lower_kernel<T, 4, 4, 2><<<grid_for(n), kBlock, 0, s>>>(a, gamma, pmin, factor, fnv, vec, fspr, dt, upts,
                                                                     diag, dub, qbar, wbuf, dbar, grhs, gdt, gfspr);
    else
        ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "adjoint built for nfvars/ndims 5/3 and 4/2 only");
}

// ---- scalar LU-SGS ---------------------------------------------------------
template <typename T>
void face_list_geo(long long E, long long ld, int ndims, const int *q, const T *nrm, const T *fa, const T *rv,
                   T *geo, cudaStream_t s) {
    if (E <= 0) return;
    const long long g = (E + kBlock - 1) / kBlock;
    face_list_geo_kernel<T><<<(unsigned)(g < 65535 * 16 ? g : 65535 * 16), kBlock, 0, s>>>(E, ld, ndims, q, nrm, fa,
                                                                                          rv, geo);
}

void pack_geo4(long long N, int P, int ndims, const float *nrm, const float *fa, const float *rv, void *geo4,
               cudaStream_t s) {
    const long long n = (long long)P * N;
    if (n <= 0) return;
    const long long g = (n + kBlock - 1) / kBlock;
    pack_geo4_kernel<<<(unsigned)(g < 65535 * 16 ? g : 65535 * 16), kBlock, 0, s>>>(N, P, ndims, nrm, fa, rv,
                                                                                   static_cast<float4 *>(geo4));
}

void pack_lam2(long long n, const float *lam, const float *tlam, void *lam2, cudaStream_t s) {
    if (n <= 0) return;
    const long long g = (n + kBlock - 1) / kBlock;
    pack_lam2_kernel<<<(unsigned)(g < 65535 * 16 ? g : 65535 * 16), kBlock, 0, s>>>(n, lam, tlam,
                                                                                   static_cast<float2 *>(lam2));
}

template <typename T, int NV, int NFV, int NDIMS, bool RANS>
static void sweep_go(const ::ucfd::ScalarSweepArgs<T> &a, int block, cudaStream_t s) {
    const long long n = a.t1 - a.t0;
    if (n <= 0) return;
    if (a.facelist) {
        constexpr int DNV = RANS ? NV - NFV : NFV;
        ::ucfd::ScalarSweepArgs<T> b = a;
        if (b.cpb <= 0 || b.cpb > block) b.cpb = block / 3 > 0 ? block / 3 : 1;
        const size_t smem = (size_t)b.cpb * (a.nface > 0 ? a.nface : 1) * DNV * sizeof(T);
        if (smem > 48 * 1024) ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "face-list sweep: %zu bytes of shared memory", smem);
        scalar_sweep_faces_kernel<T, NV, NFV, NDIMS, RANS><<<grid_for(n, b.cpb), block, smem, s>>>(b);
        return;
    }
    if (a.pair && a.nface <= 6) {
        if (a.regcap == 4)
            scalar_sweep_pair_kernel<T, NV, NFV, NDIMS, RANS, 4><<<grid_for(2 * n, block), block, 0, s>>>(a);
        else
            scalar_sweep_pair_kernel<T, NV, NFV, NDIMS, RANS, 1><<<grid_for(2 * n, block), block, 0, s>>>(a);
        return;
    }
    if (a.regcap == 4)
        scalar_sweep_kernel<T, NV, NFV, NDIMS, RANS, 4><<<grid_for(n, block), block, 0, s>>>(a);
    else if (a.regcap == 3)
        scalar_sweep_kernel<T, NV, NFV, NDIMS, RANS, 3><<<grid_for(n, block), block, 0, s>>>(a);
    else
        scalar_sweep_kernel<T, NV, NFV, NDIMS, RANS, 1><<<grid_for(n, block), block, 0, s>>>(a);
}

// Both systems in one launch per level (one thread per cell; the register
// caps of the single-system kernels).
template <typename T, int NV, int NFV, int NDIMS>
static void sweep_both_go(const ::ucfd::ScalarSweepArgs<T> &a, int block, cudaStream_t s) {
    const long long n = a.t1 - a.t0;
    if (n <= 0) return;
    if (a.facelist || a.pair)
        ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "both-system sweep: one thread per cell only");
    if (a.regcap == 4)
        scalar_sweep_both_kernel<T, NV, NFV, NDIMS, 4><<<grid_for(n, block), block, 0, s>>>(a);
    else if (a.regcap == 3)
        scalar_sweep_both_kernel<T, NV, NFV, NDIMS, 3><<<grid_for(n, block), block, 0, s>>>(a);
    else
        scalar_sweep_both_kernel<T, NV, NFV, NDIMS, 1><<<grid_for(n, block), block, 0, s>>>(a);
}

// rans: 0 mean-flow system, 1 turbulence system, 2 both in one launch.
template <typename T>
void scalar_sweep(const ::ucfd::ScalarSweepArgs<T> &a, int nv, int nfv, int ndims, int rans,
                  int block, cudaStream_t s) {
    if (block <= 0) block = kBlock;
#define UCFD_SW(NV, NFV, ND)                                                   \
    if (nv == NV && nfv == NFV && ndims == ND) {                               \
        if (rans == 2) {                                                       \
            if constexpr (NV > NFV) return sweep_both_go<T, NV, NFV, ND>(a, block, s); \
        } else if (rans) {                                                     \
            if constexpr (NV > NFV) return sweep_go<T, NV, NFV, ND, true>(a, block, s); \
        } else {                                                               \
            return sweep_go<T, NV, NFV, ND, false>(a, block, s);               \
        }                                                                      \
    }
    UCFD_SW(5, 5, 3)
    UCFD_SW(6, 5, 3)
    UCFD_SW(7, 5, 3)
    UCFD_SW(4, 4, 2)
    UCFD_SW(5, 4, 2)
    UCFD_SW(6, 4, 2)
#undef UCFD_SW
    ::ucfd::fail(UCFD_ERR_UNSUPPORTED,
                 "scalar sweep for nvars=%d nfvars=%d ndims=%d (%s) is not built (supported: "
                 "ndims 3 with nfvars 5, ndims 2 with nfvars 4, up to 2 turbulence variables)",
                 nv, nfv, ndims, rans ? "RANS" : "NS");
}

template <typename T, int NV, int NFV, int NDIMS, bool RANS, int MINB, bool BOTH = false>
static void persistent_minb_go(const ::ucfd::ScalarSweepArgs<T> &a, const int *lev_off, int nlev, unsigned *bar,
                               int *err, long long max_spin, cudaStream_t s) {
    auto kern = scalar_sweep_persistent_kernel<T, NV, NFV, NDIMS, RANS, MINB, BOTH>;
    static int grid = 0;  // per instantiation: blocks that fit co-resident
    if (!grid) {
        int per_sm = 0, dev = 0, sms = 0;
        UCFD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kBlock, 0));
        UCFD_CUDA(cudaGetDevice(&dev));
        UCFD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        grid = per_sm * sms;
        if (grid <= 0) ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "persistent sweep kernel does not fit on the device");
    }
    ::ucfd::ScalarSweepArgs<T> aa = a;
    void *args[] = {(void *)&aa, (void *)&lev_off, (void *)&nlev, (void *)&bar, (void *)&err, (void *)&max_spin};
    UCFD_CUDA(cudaLaunchCooperativeKernel((const void *)kern, dim3(grid), dim3(kBlock), args, 0, s));
}

template <typename T, int NV, int NFV, int NDIMS, bool RANS, bool BOTH = false>
static void persistent_go(const ::ucfd::ScalarSweepArgs<T> &a, const int *lev_off, int nlev, unsigned *bar,
                          int *err, long long max_spin, cudaStream_t s) {
    if (a.regcap == 4)
        persistent_minb_go<T, NV, NFV, NDIMS, RANS, 4, BOTH>(a, lev_off, nlev, bar, err, max_spin, s);
    else if (a.regcap == 3)
        persistent_minb_go<T, NV, NFV, NDIMS, RANS, 3, BOTH>(a, lev_off, nlev, bar, err, max_spin, s);
    else
        persistent_minb_go<T, NV, NFV, NDIMS, RANS, 2, BOTH>(a, lev_off, nlev, bar, err, max_spin, s);
}

// Whole sweep (all nlev levels) as one cooperative launch with a bounded
// grid barrier between levels; lev_off is a device array.
template <typename T>
void scalar_sweep_persistent(const ::ucfd::ScalarSweepArgs<T> &a, int nv, int nfv, int ndims, int rans,
                             const int *lev_off, int nlev, unsigned *bar, int *err, long long max_spin,
                             cudaStream_t s) {
#define UCFD_PSW(NV, NFV, ND)                                                                              \
    if (nv == NV && nfv == NFV && ndims == ND) {                                                           \
        if (rans == 2) {                                                                                   \
            if constexpr (NV > NFV) return persistent_go<T, NV, NFV, ND, true, true>(a, lev_off, nlev, bar, \
                                                                                      err, max_spin, s);   \
        } else if (rans) {                                                                                 \
            if constexpr (NV > NFV) return persistent_go<T, NV, NFV, ND, true>(a, lev_off, nlev, bar, err, \
                                                                                max_spin, s);              \
        } else {                                                                                           \
            return persistent_go<T, NV, NFV, ND, false>(a, lev_off, nlev, bar, err, max_spin, s);          \
        }                                                                                                  \
    }
    UCFD_PSW(5, 5, 3)
    UCFD_PSW(6, 5, 3)
    UCFD_PSW(7, 5, 3)
    UCFD_PSW(4, 4, 2)
    UCFD_PSW(5, 4, 2)
    UCFD_PSW(6, 4, 2)
#undef UCFD_PSW
    ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "persistent sweep for nvars=%d nfvars=%d ndims=%d is not built", nv, nfv,
                 ndims);
}

template <typename T>
void legacy_pre(int neles, int nface, T factor, const T *fnorm_vol, const T *dt, T *diag,
                const T *fspr, cudaStream_t s) {
    if (neles <= 0) return;
    legacy_pre_kernel<T><<<grid_for(neles), kBlock, 0, s>>>(neles, nface, factor, fnorm_vol, dt, diag, fspr);
}

template <typename T>
void legacy_update(int neles, int k0, int k1, T *upts, const T *rhs, cudaStream_t s) {
    if (neles <= 0 || k1 <= k0) return;
    legacy_update_kernel<T><<<grid_for(neles), kBlock, 0, s>>>(neles, k0, k1, upts, rhs);
}

template <typename T>
void fs_lusgs_pack(int neles, int nvars, int nfvars, long long N, double turb_factor, double a0,
                   const int *cell_ids, const int *iperm, const double *upts, const double *rhs,
                   const double *dt, const double *dsrc, T *u, T *du, T *diag, cudaStream_t s) {
    if (neles <= 0) return;
    fs_lusgs_pack_kernel<T><<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, nfvars, N, turb_factor, a0,
                                                                cell_ids, iperm, upts, rhs, dt, dsrc, u,
                                                                du, diag);
}

template <typename T>
void fs_lusgs_update(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,
                     const T *du, double *upts, int assign, cudaStream_t s) {
    if (neles <= 0) return;
    fs_lusgs_update_kernel<T><<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, N, cell_ids, iperm, du, upts, assign);
}

template <typename T>
void fs_lusgs_prepare(long long N, int maxdeg, int nv0, int nv1, T kappa, const int *nei,
                      const T *fa, const T *rv, const T *lam, const T *base, T *diag, cudaStream_t s) {
    if (N <= 0) return;
    fs_lusgs_prepare_kernel<T><<<grid_for(N), kBlock, 0, s>>>(N, maxdeg, nv0, nv1, kappa, nei, fa, rv, lam,
                                                              base, diag);
}

template <typename T>
void fs_lusgs_prepare_both(long long N, int maxdeg, int nfv, int nv, T kappa, const int *nei, const T *fa,
                           const T *rv, const T *lam, const T *tlam, const T *base, T *diag, cudaStream_t s) {
    if (N <= 0) return;
    fs_lusgs_prepare_both_kernel<T><<<grid_for(N), kBlock, 0, s>>>(N, maxdeg, nfv, nv, kappa, nei, fa, rv, lam,
                                                                   tlam, base, diag);
}

template <typename Td>
void gather_idx(long long n, const int *idx, const double *src, Td *dst, cudaStream_t s) {
    if (n <= 0) return;
    gather_idx_kernel<Td><<<grid_for(n < (1ll << 24) ? n : (1ll << 24)), kBlock, 0, s>>>(n, idx, src, dst);
}

__global__ void __launch_bounds__(1024) pair_reduce_kernel(int nblocks, const double *part, double *out) {
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        a += part[2 * i];
        b += part[2 * i + 1];
    }
    a = block_sum(a);
    b = block_sum(b);
    if (threadIdx.x == 0) {
        out[0] = a;
        out[1] = b;
    }
}

// out[0], out[1] = sums of the (r^2, rhs^2) pairs written by the residual kernel.
void pair_reduce(int nblocks, const double *part, double *out, cudaStream_t s) {
    pair_reduce_kernel<<<1, 1024, 0, s>>>(nblocks, part, out);
}

// ---- block LU-SGS ----------------------------------------------------------
#define UCFD_BSW(B, CALL)                 \
    switch (B) {                          \
        case 1: { constexpr int BB = 1; CALL; break; } \
        case 2: { constexpr int BB = 2; CALL; break; } \
        case 4: { constexpr int BB = 4; CALL; break; } \
        case 5: { constexpr int BB = 5; CALL; break; } \
        default: ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "block size %d not built (1, 2, 4, 5)", B); \
    }

template <typename S>
void fs_blusgs_pack(int neles, int nvars, int B, long long N, double a0, const int *cell_ids,
                    const int *iperm, const double *rhs, const double *dt, S *rhs_s, double *rhs64,
                    double *D, cudaStream_t s) {
    if (neles <= 0) return;
    fs_blusgs_pack_kernel<S><<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, B, N, a0, cell_ids, iperm,
                                                                 rhs, dt, rhs_s, rhs64, D);
}

void fs_tblusgs_pack(int model, int neles, int nvars, int nt, long long N, double a0, double factor,
                     double betast, const int *cell_ids, const int *iperm, const double *uptsb,
                     const double *dsrc, const double *dt, double *D, cudaStream_t s) {
    if (neles <= 0) return;
    fs_tblusgs_pack_kernel<<<grid_for(neles), kBlock, 0, s>>>(model, neles, nvars, nt, N, a0, factor, betast,
                                                              cell_ids, iperm, uptsb, dsrc, dt, D);
}

template <typename S>
void fs_blusgs_prepare(int B, long long N, int P, long long nF, const int *nei, const int *slot,
                       const int8_t *side, const double *fa, const double *rv, const double *jmat,
                       const double *dd, double *D, double *LU64, S *LU_s, S *J_s, double *J64,
                       double *jt, cudaStream_t s) {
    if (N <= 0) return;
    const unsigned gt = (unsigned)((nF + 31) / 32);
    UCFD_BSW(B, (jmat_face_major_kernel<BB><<<gt, 256, 0, s>>>(nF, jmat, jt)));
    UCFD_BSW(B, (fs_blusgs_prepare_kernel<S, BB><<<grid_for(N, 128), 128, 0, s>>>(
                    N, P, nei, slot, side, fa, rv, jt, dd, D, LU64, LU_s, J_s, J64)));
}

// Bulk-copy sweep: NST buffers per warp, 4 (NST 2) or 8 (NST 1) warps per
// block; grid capped at the blocks that fit on the device at once.
template <int B, int PW, int NST>
static void sweep_bulk_go(int t0, int t1, long long N, int var0, const int *nei, const float *fa,
                          const float *rv, const float *J, const float *LU, const float *rhs, float *du,
                          int *err, long long max_spin, const ::ucfd::SweepSplit<float> &sp, cudaStream_t s) {
    auto kern = fs_blusgs_sweep_bulk_kernel<B, PW, NST>;
    constexpr int threads = NST == 2 ? 128 : 256;
    constexpr int tiles_per_buf = kFold ? PW : PW + 1;  // J (and, in the exact build, LU) tiles
    constexpr size_t smem = (size_t)(threads / 32) * NST * (tiles_per_buf * B * B * 32 * sizeof(float) + 8);
    static int cap = 0;  // per instantiation: co-resident blocks on the device
    if (!cap) {
        UCFD_CUDA(cudaFuncSetAttribute((const void *)kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0, dev = 0, sms = 0;
        UCFD_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem));
        UCFD_CUDA(cudaGetDevice(&dev));
        UCFD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        if (per_sm <= 0) ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "bulk-copy sweep kernel does not fit on the device");
        cap = per_sm * sms;
    }
    const long long tiles = (((long long)t1 + 31) >> 5) - (t0 >> 5);
    const long long want = (tiles + threads / 32 - 1) / (threads / 32);
    const unsigned g = (unsigned)(want < cap ? want : cap);
    kern<<<g, threads, smem, s>>>(t0, t1, N, var0, nei, fa, rv, J, LU, rhs, du, err, max_spin, sp);
}

// Unrolled sweep launched as a programmatic dependent of the previous
// launch on the stream (cudaLaunchAttributeProgrammaticStreamSerialization).
template <typename S, int B, int PW>
static void sweep_dep_go(unsigned g, int block, cudaStream_t s, int t0, int t1, long long N, int P, int var0,
                         const int *nei, const S *fa, const S *rv, const S *J, const S *LU, const S *rhs, S *du,
                         const ::ucfd::SweepSplit<S> &sp) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(g);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UCFD_CUDA(cudaLaunchKernelEx(&cfg, fs_blusgs_sweep_kernel<S, B, PW, true>, t0, t1, N, P, var0, nei, fa, rv, J,
                                 LU, rhs, du, sp));
}

// Levels with at most this many cells take the register-hoisted kernel in
// the dependent-launch variant (FP32): they are bound by one thread's
// memory latency, not by bandwidth.
constexpr int kSmallLevel = 16384;

template <int B, int PW>
static void sweep_small_go(cudaStream_t s, int t0, int t1, long long N, int var0, const int *nei, const float *J,
                           const float *rhs, float *du, const ::ucfd::SweepSplit<float> &sp) {
    constexpr int threads = 128;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid_for(t1 - (t0 & ~31), threads));
    cfg.blockDim = dim3(threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UCFD_CUDA(cudaLaunchKernelEx(&cfg, fs_blusgs_sweep_small_kernel<B, PW>, t0, t1, N, var0, nei, J, rhs, du, sp));
}

template <typename S>
void fs_blusgs_sweep(int B, int t0, int t1, long long N, int P, int var0, const int *nei, const S *fa,
                     const S *rv, const S *J, const S *LU, const S *rhs, S *du, int block,
                     int variant, int *err, long long max_spin, const ::ucfd::SweepSplit<S> &sp,
                     cudaStream_t s) {
    if (t1 <= t0) return;
    if (block <= 0) block = kBlock;
    // threads start at the tile boundary below t0 (see the kernel)
    const unsigned g = grid_for(t1 - (t0 & ~31), block);
    // variant 0: faces unrolled to the ELL width (6 or 4) when it matches;
    // variant 1: the face loop that stops at the first padding slot;
    // variants 2 / 3: FP32, ELL width 6 or 4, block 5: J and LU tiles staged
    // in shared memory by bulk copies, 2 / 1 buffers per warp;
    // variant 4: variant 0 launched as a programmatic dependent of the
    // previous launch (its start overlaps the previous colour's tail).
    // All apply the faces in the same order with the same operations.
    if (variant == 4 && (P == 6 || P == 4)) {
        if constexpr (std::is_same<S, float>::value) {
            if (kFold && B == 5 && t1 - t0 <= kSmallLevel) {
                if (P == 6) sweep_small_go<5, 6>(s, t0, t1, N, var0, nei, J, rhs, du, sp);
                else sweep_small_go<5, 4>(s, t0, t1, N, var0, nei, J, rhs, du, sp);
                return;
            }
        }
        if (P == 6) {
            UCFD_BSW(B, (sweep_dep_go<S, BB, 6>(g, block, s, t0, t1, N, P, var0, nei, fa, rv, J, LU, rhs, du, sp)));
        } else {
            UCFD_BSW(B, (sweep_dep_go<S, BB, 4>(g, block, s, t0, t1, N, P, var0, nei, fa, rv, J, LU, rhs, du, sp)));
        }
        return;
    }
    if constexpr (std::is_same<S, float>::value) {
        if ((variant == 2 || variant == 3) && B == 5 && (P == 6 || P == 4)) {
            if (!err) ::ucfd::fail(UCFD_ERR_ARGUMENT, "bulk-copy sweep needs an error flag");
            if (P == 6) {
                if (variant == 2) sweep_bulk_go<5, 6, 2>(t0, t1, N, var0, nei, fa, rv, J, LU, rhs, du, err, max_spin, sp, s);
                else sweep_bulk_go<5, 6, 1>(t0, t1, N, var0, nei, fa, rv, J, LU, rhs, du, err, max_spin, sp, s);
            } else {
                if (variant == 2) sweep_bulk_go<5, 4, 2>(t0, t1, N, var0, nei, fa, rv, J, LU, rhs, du, err, max_spin, sp, s);
                else sweep_bulk_go<5, 4, 1>(t0, t1, N, var0, nei, fa, rv, J, LU, rhs, du, err, max_spin, sp, s);
            }
            return;
        }
    }
    if (variant == 1) {
        UCFD_BSW(B, (fs_blusgs_sweep_kernel<S, BB, 0><<<g, block, 0, s>>>(t0, t1, N, P, var0, nei, fa, rv, J, LU,
                                                                          rhs, du, sp)));
    } else if (P == 6) {
        UCFD_BSW(B, (fs_blusgs_sweep_kernel<S, BB, 6><<<g, block, 0, s>>>(t0, t1, N, P, var0, nei, fa, rv, J, LU,
                                                                          rhs, du, sp)));
    } else if (P == 4) {
        UCFD_BSW(B, (fs_blusgs_sweep_kernel<S, BB, 4><<<g, block, 0, s>>>(t0, t1, N, P, var0, nei, fa, rv, J, LU,
                                                                          rhs, du, sp)));
    } else {
        UCFD_BSW(B, (fs_blusgs_sweep_kernel<S, BB, 0><<<g, block, 0, s>>>(t0, t1, N, P, var0, nei, fa, rv, J, LU,
                                                                          rhs, du, sp)));
    }
}

template <typename S>
void fs_blusgs_rhs_solve(int B, long long N, int var0, const S *LU, const S *b, S *c, cudaStream_t s) {
    if (N <= 0) return;
    UCFD_BSW(B, (fs_blusgs_rhs_solve_kernel<S, BB><<<grid_for(N), kBlock, 0, s>>>(N, var0, LU, b, c)));
}

template <typename Sx, typename R>
void fs_blusgs_residual(int B, long long N, int P, int var0, int nvars, const int *nei,
                        const double *fa, const double *rv, const double *J64, const double *D,
                        const double *rhs64, const Sx *x, R *r_out, double *part, int nblocks_max,
                        int *nblocks_used, cudaStream_t s) {
    const unsigned g = grid_for(N);
    if ((int)g > nblocks_max) ::ucfd::fail(UCFD_ERR_ARGUMENT, "residual partial buffer too small");
    *nblocks_used = (int)g;
    UCFD_BSW(B, (fs_blusgs_residual_kernel<Sx, R, BB><<<g, kBlock, 0, s>>>(
                    N, P, var0, nvars, nei, fa, rv, J64, D, rhs64, x, r_out, part)));
}

template <typename S>
void fs_blusgs_subres(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,
                      const double *vol, const S *du, S *dup, double *res, cudaStream_t s) {
    if (neles <= 0) return;
    fs_blusgs_subres_kernel<S><<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, N, cell_ids, iperm, vol, du,
                                                                   dup, res);
}

template <typename S>
void fs_blusgs_update(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,
                      const S *du, double *upts, cudaStream_t s) {
    if (neles <= 0) return;
    fs_blusgs_update_kernel<S><<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, N, cell_ids, iperm, du, upts);
}

// ---- Krylov ----------------------------------------------------------------
#define UCFD_KSW(B, CALL)                 \
    switch (B) {                          \
        case 1: { constexpr int BB = 1; CALL; break; } \
        case 2: { constexpr int BB = 2; CALL; break; } \
        case 3: { constexpr int BB = 3; CALL; break; } \
        case 4: { constexpr int BB = 4; CALL; break; } \
        case 5: { constexpr int BB = 5; CALL; break; } \
        case 6: { constexpr int BB = 6; CALL; break; } \
        case 7: { constexpr int BB = 7; CALL; break; } \
        default: ::ucfd::fail(UCFD_ERR_UNSUPPORTED, "block size %d not built (1..7)", B); \
    }

template <typename Tv, typename Ta>
void bsr_spmv(int B, int bn, int P, const int *col, const Tv *val, double alpha, const double *x,
              double beta, double *y, int block, cudaStream_t s) {
    if (bn <= 0) return;
    if (block <= 0) block = kBlock;
    const unsigned g = grid_for(bn, block);
    // unrolled rows for the 5x5 systems (tets: diag + 4 faces; hexes: + 6)
    if (B == 5 && P <= 5) {
        bsr_spmv_kernel<Tv, Ta, 5, 5><<<g, block, 0, s>>>(bn, P, col, val, alpha, x, beta, y);
        return;
    }
    if (B == 5 && P <= 7) {
        bsr_spmv_kernel<Tv, Ta, 5, 7><<<g, block, 0, s>>>(bn, P, col, val, alpha, x, beta, y);
        return;
    }
    UCFD_KSW(B, (bsr_spmv_kernel<Tv, Ta, BB, 0><<<g, block, 0, s>>>(bn, P, col, val, alpha, x, beta, y)));
}

template <typename Tl>
void pc_prepare(int B, int bn, const int *perm, const long long *dslot, const double *values,
                double *LU64, Tl *LU_l, int factor, cudaStream_t s) {
    if (bn <= 0) return;
    UCFD_KSW(B, (pc_prepare_kernel<Tl, BB><<<grid_for(bn, 128), 128, 0, s>>>(bn, perm, dslot, values, LU64,
                                                                             LU_l, factor)));
}

template <typename T>
void ell_gather(int B, int bn, int P, const int *src, const double *vals, T *out, cudaStream_t s) {
    const long long n = (long long)P * bn;
    if (n <= 0) return;
    UCFD_KSW(B, (ell_gather_kernel<T, BB><<<grid_for(n), kBlock, 0, s>>>(bn, P, src, vals, out)));
}

void fingerprint(long long n, const int *a, unsigned long long *out, cudaStream_t s) {
    if (n <= 0) return;
    fingerprint_kernel<<<grid_for(n < (1ll << 22) ? n : (1ll << 22)), kBlock, 0, s>>>(n, a, out);
}

// Triangular steps, mode PC_BLUSGS / PC_BILU / PC_ILU (kernels_krylov.cuh).
template <typename T, int MODE, bool LOWER>
static void pc_step_go(int B, unsigned g, int block, cudaStream_t s, int t0, int t1, int bn, int P,
                       const int *col, const T *val, const T *LU, T *b) {
    if constexpr (MODE == PC_ILU) {
        if (B != 1) ::ucfd::fail(UCFD_ERR_ARGUMENT, "scalar ILU needs block size 1 (got %d)", B);
        if constexpr (LOWER) pc_lower_kernel<T, 1, 0, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
        else pc_upper_kernel<T, 1, 0, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
        return;
    } else {
        if (B == 5 && P <= 6) {
            if (P <= 4) {
                if constexpr (LOWER) pc_lower_kernel<T, 5, 4, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
                else pc_upper_kernel<T, 5, 4, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
            } else {
                if constexpr (LOWER) pc_lower_kernel<T, 5, 6, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
                else pc_upper_kernel<T, 5, 6, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b);
            }
            return;
        }
        if constexpr (LOWER) {
            UCFD_KSW(B, (pc_lower_kernel<T, BB, 0, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b)));
        } else {
            UCFD_KSW(B, (pc_upper_kernel<T, BB, 0, MODE><<<g, block, 0, s>>>(t0, t1, bn, P, col, val, LU, b)));
        }
    }
}

template <typename T, bool LOWER>
static void pc_step(int B, int t0, int t1, int bn, int P, const int *col, const T *val, const T *LU, T *b,
                    int block, int mode, cudaStream_t s) {
    if (t1 <= t0) return;
    if (block <= 0) block = kBlock;
    const unsigned g = grid_for(t1 - t0, block);
    if (mode == PC_BILU) pc_step_go<T, PC_BILU, LOWER>(B, g, block, s, t0, t1, bn, P, col, val, LU, b);
    else if (mode == PC_ILU) pc_step_go<T, PC_ILU, LOWER>(B, g, block, s, t0, t1, bn, P, col, val, LU, b);
    else pc_step_go<T, PC_BLUSGS, LOWER>(B, g, block, s, t0, t1, bn, P, col, val, LU, b);
}

template <typename T>
void pc_lower(int B, int t0, int t1, int bn, int PL, const int *Lcol, const T *Lval, const T *LU, T *b,
              int block, int mode, cudaStream_t s) {
    pc_step<T, true>(B, t0, t1, bn, PL, Lcol, Lval, LU, b, block, mode, s);
}

template <typename T>
void pc_upper(int B, int t0, int t1, int bn, int PU, const int *Ucol, const T *Uval, const T *LU, T *b,
              int block, int mode, cudaStream_t s) {
    pc_step<T, false>(B, t0, t1, bn, PU, Ucol, Uval, LU, b, block, mode, s);
}

// One level of the ILU(0) factorisation (rows[t], t in [t0, t1)).
void ilu_factor(int B, int scalar, int t0, int t1, const int *rows, const int *rowptr, const int *colidx,
                const int *diagslots, double *vals, cudaStream_t s) {
    if (t1 <= t0) return;
    const unsigned g = grid_for(t1 - t0, 128);
    if (scalar) {
        if (B != 1) ::ucfd::fail(UCFD_ERR_ARGUMENT, "scalar ILU needs block size 1 (got %d)", B);
        ilu_factor_kernel<1, true><<<g, 128, 0, s>>>(t0, t1, rows, rowptr, colidx, diagslots, vals);
        return;
    }
    UCFD_KSW(B, (ilu_factor_kernel<BB, false><<<g, 128, 0, s>>>(t0, t1, rows, rowptr, colidx, diagslots, vals)));
}

template <typename Ts, typename Td>
void gather_rows(int bn, int B, const int *perm, const Ts *src, Td *dst, cudaStream_t s) {
    const long long n = (long long)bn * B;
    if (n <= 0) return;
    gather_rows_kernel<Ts, Td><<<grid_for(n), kBlock, 0, s>>>(bn, B, perm, src, dst);
}

template <typename Ts, typename Td>
void scatter_rows(int bn, int B, const int *perm, const Ts *src, Td *dst, cudaStream_t s) {
    const long long n = (long long)bn * B;
    if (n <= 0) return;
    scatter_rows_kernel<Ts, Td><<<grid_for(n), kBlock, 0, s>>>(bn, B, perm, src, dst);
}

template <typename Ts, typename Td>
__global__ void convert_kernel(long long n, const Ts *src, Td *dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = (Td)src[i];
}

template <typename Ts, typename Td>
void convert(long long n, const Ts *src, Td *dst, cudaStream_t s) {
    if (n <= 0) return;
    convert_kernel<Ts, Td><<<grid_for(n < (1ll << 24) ? n : (1ll << 24)), kBlock, 0, s>>>(n, src, dst);
}

template <typename Ts>
__global__ void axpy_into_kernel(long long n, const Ts *x, double *y) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] += (double)x[i];
}

template <typename Ts>
void axpy_into(long long n, const Ts *x, double *y, cudaStream_t s) {
    if (n <= 0) return;
    axpy_into_kernel<Ts><<<grid_for(n < (1ll << 24) ? n : (1ll << 24)), kBlock, 0, s>>>(n, x, y);
}

// y += x and out = ||x||_2 accumulated in FP64 (pseudo-time update).
template <typename S>
__global__ void axpy_norm_kernel(long long n, const S *x, S *y, double *part) {
    double t = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const S xv = x[i];
        y[i] += xv;
        t += (double)xv * (double)xv;
    }
    t = block_sum(t);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(1024) sqrt_sum_kernel(int nb, const double *part, double *out) {
    double t = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) t += part[b];
    t = block_sum(t);
    if (threadIdx.x == 0) *out = sqrt(t);
}

// ---- GMRES pieces ----------------------------------------------------------
int gm_blocks(long long n) { return gm_grid(n); }

// gm_dots / gm_update: gm_launchers.cuh (their own translation unit, kern_gm.cu)

void gm_reduce(int nblocks, int K, const double *part, double *out, int accumulate, cudaStream_t s) {
    if (K <= 0) return;
    gm_reduce_kernel<<<K, kBlock, 0, s>>>(nblocks, part, out, accumulate);
}

void gm_sumsq(long long n, const double *x, double *part, cudaStream_t s) {
    gm_sumsq_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, x, part);
}

void gm_cycle_begin(int nblocks, const double *part, void *st, double *y, double *out_norm, cudaStream_t s) {
    gm_cycle_begin_kernel<<<1, kBlock, 0, s>>>(nblocks, part, (GmState *)st, y, out_norm);
}

void gm_scale(long long n, const void *st, const double *src, double *dst, cudaStream_t s) {
    gm_scale_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, (const GmState *)st, src, dst);
}

void gm_givens(int j, int ld, int nblocks, const double *part_norm, double *H, const double *h2, double *cs,
               double *sn, double *y, double haptol, double rel_floor, void *st, cudaStream_t s) {
    gm_givens_kernel<<<1, kBlock, 0, s>>>(j, ld, nblocks, part_norm, H, h2, cs, sn, y, haptol, rel_floor,
                                          (GmState *)st);
}

void gm_backsub(int ld, const double *H, double *y, const void *st, cudaStream_t s) {
    gm_backsub_kernel<<<1, 1, 0, s>>>(ld, H, y, (const GmState *)st);
}

void gm_solution(long long n, const double *V, long long ldv, const double *y, const void *st, double *x,
                 cudaStream_t s) {
    gm_solution_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, V, ldv, y, (const GmState *)st, x);
}

size_t gm_state_bytes() { return sizeof(GmState); }

template <typename S>
void axpy_norm(long long n, const S *x, S *y, double *part, double *out, cudaStream_t s) {
    const int nb = gm_blocks(n);
    axpy_norm_kernel<S><<<nb, kBlock, 0, s>>>(n, x, y, part);
    sqrt_sum_kernel<<<1, 1024, 0, s>>>(nb, part, out);
}

// The FP32 pseudo-time loop's state u += x, kept as a float-float pair: the
// working FP32 state hi (what the sweeps read) and a low part lo, together
// 48 significant bits, so an increment far below hi's rounding unit is kept
// in lo instead of being rounded away at every iteration.  The pair is
// updated by an error-free sum (Knuth's TwoSum of hi and x, the error added
// to lo) and renormalised (Dekker's Fast2Sum), all on the FP32 pipe: an FP64
// master would put four FP64 operations per value on GB300's narrow FP64
// pipe.  out = ||x||_2: each thread sums x^2 exactly split (x*x rounded plus
// its fma remainder) into a float-float accumulator, the thread sums are
// added in FP64.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bp = s - a;
    e = (a - (s - bp)) + (b - bp);
}

__global__ void axpy_master_kernel(long long n, const float *x, float *hi, float *lo, double *part) {
    float ah = 0.f, al = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float xv = x[i];
        float sh, se;
        two_sum(hi[i], xv, sh, se);
        const float t = lo[i] + se;
        const float nh = sh + t;
        hi[i] = nh;
        lo[i] = t - (nh - sh);
        const float p = __fmul_rn(xv, xv);
        const float pe = fmaf(xv, xv, -p);
        float qh, qe;
        two_sum(ah, p, qh, qe);
        const float ql = al + (qe + pe);
        ah = qh + ql;
        al = ql - (ah - qh);
    }
    double t = (double)ah + (double)al;
    t = block_sum(t);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

void axpy_master(long long n, const float *x, float *hi, float *lo, double *part, double *out, cudaStream_t s) {
    const int nb = gm_blocks(n);
    axpy_master_kernel<<<nb, kBlock, 0, s>>>(n, x, hi, lo, part);
    sqrt_sum_kernel<<<1, 1024, 0, s>>>(nb, part, out);
}

// Low part of the packed state (lusgs_pack's state, lusgs.c:8-37): with
// hi = (float)upts as fs_lusgs_pack rounds it, lo = (float)(upts - hi).
__global__ void state_lo_pack_kernel(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,
                                     const double *upts, float *lo) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) {
        const double x = upts[idx + (long long)v * neles];
        lo[k + v * N] = (float)(x - (double)(float)x);
    }
}

void state_lo_pack(int neles, int nvars, long long N, const int *cell_ids, const int *iperm, const double *upts,
                   float *lo, cudaStream_t s) {
    if (neles <= 0) return;
    state_lo_pack_kernel<<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, N, cell_ids, iperm, upts, lo);
}

// rank_lusgs_update's write-back (lusgs.c:54-70) of the float-float state:
// upts = hi + lo in FP64.
__global__ void state_ff_update_kernel(int neles, int nvars, long long N, const int *cell_ids, const int *iperm,
                                       const float *hi, const float *lo, double *upts) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v)
        upts[idx + (long long)v * neles] = (double)hi[k + v * N] + (double)lo[k + v * N];
}

void state_ff_update(int neles, int nvars, long long N, const int *cell_ids, const int *iperm, const float *hi,
                     const float *lo, double *upts, cudaStream_t s) {
    if (neles <= 0) return;
    state_ff_update_kernel<<<grid_for(neles), kBlock, 0, s>>>(neles, nvars, N, cell_ids, iperm, hi, lo, upts);
}

__global__ void __launch_bounds__(256) norm_finalize_kernel(int nblocks, const double *part, double *out) {
    const double t = block_sum_partials(part, nblocks, kMaxK);
    if (threadIdx.x == 0) *out = sqrt(t);
}

// out = ||x||_2 (two-pass, fixed order).
void norm2_to(long long n, const double *x, double *part, double *out, cudaStream_t s) {
    gm_sumsq_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, x, part);
    norm_finalize_kernel<<<1, kBlock, 0, s>>>(gm_blocks(n), part, out);
}

// ---- BiCGSTAB ----------------------------------------------------------------
size_t bc_state_bytes() { return sizeof(BcState); }

void bc_dot(long long n, const double *x, const double *y, double *part, const void *st, cudaStream_t s) {
    bc_dot_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, x, y, part, (const BcState *)st);
}
void bc_start(int nb, const double *part, void *st, int maxiter, cudaStream_t s) {
    bc_start_kernel<<<1, 1, 0, s>>>(nb, part, (BcState *)st, maxiter);
}
void bc_direction(long long n, const void *st, const double *r, const double *v, double *p, double *pt,
                  cudaStream_t s) {
    bc_direction_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, (const BcState *)st, r, v, p, pt);
}
void bc_alpha(int nb, const double *part, void *st, cudaStream_t s) {
    bc_alpha_kernel<<<1, 1, 0, s>>>(nb, part, (BcState *)st);
}
void bc_s(long long n, const void *st, const double *r, const double *v, double *sv, double *shat,
          cudaStream_t s) {
    bc_s_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, (const BcState *)st, r, v, sv, shat);
}
void bc_fused5(long long n, const double *rt, const double *sv, const double *t, double *part, const void *st,
               cudaStream_t s) {
    bc_fused5_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, rt, sv, t, part, (const BcState *)st);
}
void bc_omega(int nb, const double *part, void *st, double tol, double *hist, cudaStream_t s) {
    bc_omega_kernel<<<1, 1, 0, s>>>(nb, part, (BcState *)st, tol, hist);
}
void bc_update(long long n, const void *st, const double *pt, const double *shat, const double *sv,
               const double *t, double *x, double *r, cudaStream_t s) {
    bc_update_kernel<<<gm_blocks(n), kBlock, 0, s>>>(n, (const BcState *)st, pt, shat, sv, t, x, r);
}
void bc_advance(void *st, int maxiter, cudaStream_t s) {
    bc_advance_kernel<<<1, 1, 0, s>>>((BcState *)st, maxiter);
}

}  // namespace UCFD_KNS
