// kernels_krylov.cuh -- BSR matvec, BLU-SGS preconditioner, GMRES(m) pieces.
//
// Matrices are held on the device in an ELL-of-blocks layout: entry p of
// block row i has column col[p*bn + i] (-1 = padding) and its row-major
// block value (r, c) at val[(p*B*B + r*B + c)*bn + i], so one thread per
// block row reads every value with coalesced loads.  Vectors are AoS
// [bn][B] as in the reference (sparsemat.c:57-101).
#pragma once

#include "kernels_common.cuh"
#include "kernels_blusgs.cuh"

namespace UCFD_KNS {

// A read-only load: streaming (evict-first, ld.global.cs) when CS, else
// through the read-only cache.
template <bool CS, typename T>
__device__ __forceinline__ T ld_once(const T *p) {
    if constexpr (CS) return __ldcs(p);
    else return __ldg(p);
}

// acc[r] += SGN * sum over the ELL row k of (block_p x_{col_p})[r], entries in
// stored order, each block product summed over its columns first (the
// reference's order, sparsemat.c:82-97, blusgs.c:113-124).  PW > 0: the
// row width is at most PW and the loop is unrolled so that every column
// index, then every gathered x and block value, is requested up front;
// PW == 0: runtime-width loop.  Padding entries (column < 0) end the row.
// CS: columns and block values, read once per product, are loaded with the
// streaming (evict-first) policy so that the gathered vector x, which every
// row reads at its neighbours, stays in L2 (the matvec; the preconditioner
// sweeps keep cached loads, which measured faster there: the last colour of
// the lower sweep is the first of the upper one).
template <typename Tv, typename Tx, typename Ta, int B, int PW, int SGN, bool CS = false>
__device__ __forceinline__ void ell_row_products(long long k, int bn, int P, const int *col, const Tv *val,
                                                 const Tx *x, Ta *acc) {
    constexpr int B2 = B * B;
    if constexpr (PW > 0) {
        int c[PW];
#pragma unroll
        for (int p = 0; p < PW; ++p) c[p] = p < P ? ld_once<CS>(col + (long long)p * bn + k) : -1;
        Ta xv[PW][B];
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            const long long g = c[p] >= 0 ? c[p] : 0;  // padding: any valid address
#pragma unroll
            for (int cc = 0; cc < B; ++cc) xv[p][cc] = (Ta)x[g * B + cc];
        }
        bool live = true;
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            live = live && c[p] >= 0;
            if (live) {
                const Tv *vp = val + (long long)p * B2 * bn + k;
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    Ta v = Ta(0);
#pragma unroll
                    for (int cc = 0; cc < B; ++cc) v += (Ta)ld_once<CS>(vp + (long long)(r * B + cc) * bn) * xv[p][cc];
                    if (SGN > 0) acc[r] += v;
                    else acc[r] -= v;
                }
            }
        }
    } else {
        for (int p = 0; p < P; ++p) {
            const int c = ld_once<CS>(col + (long long)p * bn + k);
            if (c < 0) break;
            Ta xv[B];
#pragma unroll
            for (int cc = 0; cc < B; ++cc) xv[cc] = (Ta)x[(long long)c * B + cc];
            const Tv *vp = val + (long long)p * B2 * bn + k;
#pragma unroll
            for (int r = 0; r < B; ++r) {
                Ta v = Ta(0);
#pragma unroll
                for (int cc = 0; cc < B; ++cc) v += (Ta)ld_once<CS>(vp + (long long)(r * B + cc) * bn) * xv[cc];
                if (SGN > 0) acc[r] += v;
                else acc[r] -= v;
            }
        }
    }
}

// SpMV_BSR: sparsemat.c:57-101 -- y = alpha*A*x + beta*y.  Tv is the type
// of the stored values, Ta the accumulation type.  With beta == 0 y is not
// read (the BLAS convention): the reference forms beta*y regardless, which
// turns an uninitialised y holding NaN or Inf into NaN; for a finite y the
// results agree (up to the sign of a zero).
template <typename Tv, typename Ta, int B, int PW>
__global__ void __launch_bounds__(256) bsr_spmv_kernel(int bn, int P, const int *col, const Tv *val,
                                                       double alpha, const double *x, double beta,
                                                       double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bn) return;
    Ta acc[B];
#pragma unroll
    for (int r = 0; r < B; ++r) acc[r] = Ta(0);
    ell_row_products<Tv, double, Ta, B, PW, +1, true>(i, bn, P, col, val, x, acc);
#pragma unroll
    for (int r = 0; r < B; ++r) {
        const long long o = (long long)i * B + r;
        y[o] = beta == 0.0 ? alpha * (double)acc[r] : alpha * (double)acc[r] + beta * y[o];
    }
}

// Values of a CSR-of-blocks array (row-major B x B blocks in slot order)
// into the ELL-of-blocks layout: ELL entry (p, k) takes the block at slot
// src[p*bn + k] (src < 0: padding, zeros).  One thread per ELL entry: the
// writes coalesce over k, and a thread's B*B reads are one contiguous block
// requested all at once.  T = float rounds the FP64 values.
template <typename T, int B>
__global__ void __launch_bounds__(256) ell_gather_kernel(int bn, int P, const int *src, const double *vals,
                                                         T *out) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)P * bn) return;
    constexpr int B2 = B * B;
    const int p = (int)(t / bn);
    const int k = (int)(t - (long long)p * bn);
    const int q = __ldg(src + t);
    T *o = out + (long long)p * B2 * bn + k;
    double v[B2];
    if (q >= 0) {
        const double *blk = vals + (long long)q * B2;
#pragma unroll
        for (int e = 0; e < B2; ++e) v[e] = __ldg(blk + e);
    } else {
#pragma unroll
        for (int e = 0; e < B2; ++e) v[e] = 0.0;
    }
#pragma unroll
    for (int e = 0; e < B2; ++e) o[(long long)e * bn] = (T)v[e];
}

// Order-independent 64-bit fingerprint of an int array: out += sum over i
// of fingerprint_mix(i, a[i]) (wrapping), so a structure cached from an
// earlier call can be recognised without copying the array to the host.
__global__ void __launch_bounds__(256) fingerprint_kernel(long long n, const int *a, unsigned long long *out) {
    unsigned long long h = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        h += ::ucfd::fingerprint_mix(i, a[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) h += __shfl_down_sync(0xffffffffu, h, o);
    if ((threadIdx.x & 31) == 0 && h) atomicAdd(out, h);
}

// BLUSGSPreconPrepare: precon/blusgs.c:7-26 -- copy each diagonal block and
// LU-factor it (FP64), optionally rounding the factors to Tl.  The fast
// build (kFold) stores reciprocal pivots, so that the applies multiply
// instead of dividing (FP64 division is a long sequence on GB300's narrow
// FP64 pipe); the exact build keeps the reference's factors.
template <typename Tl, int B>
__global__ void pc_prepare_kernel(int bn, const int *perm, const long long *dslot,
                                  const double *values, double *LU64, Tl *LU_l, int factor) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= bn) return;
    constexpr int B2 = B * B;
    const long long s = dslot[perm ? perm[k] : k];
    double d[B2];
#pragma unroll
    for (int e = 0; e < B2; ++e) d[e] = values[s * B2 + e];
    // factor == 0: the diagonal block is already factorised (block ILU) or
    // kept as it is (scalar ILU)
    if (factor) ludcmp_dev<double, B, kFold, kFold>(d);
#pragma unroll
    for (int e = 0; e < B2; ++e) {
        LU64[(long long)e * bn + k] = d[e];
        if (LU_l) LU_l[(long long)e * bn + k] = (Tl)d[e];
    }
}

// Triangular steps of the preconditioners for the rows [t0, t1) of one
// level, in place on b.  MODE:
//   0 block SGS (precon/blusgs.c): lower b_i = inv(D_i)(b_i - sum L_ij b_j)
//     (104-130), upper b_i -= inv(D_i) sum U_ij b_j (132-161);
//   1 block ILU(0) (precon/bilu.c:64-129): lower b_i -= sum L_ij b_j,
//     upper b_i = inv(LU_ii)(b_i - sum U_ij b_j) with the factored diagonal;
//   2 scalar ILU(0) (precon/ilu.c:49-85): as 1 with B = 1, dividing by the
//     kept diagonal a_ii (LU holds a_ii, not its reciprocal).
enum { PC_BLUSGS = 0, PC_BILU = 1, PC_ILU = 2 };

template <typename T, int B, int PW, int MODE>
__global__ void __launch_bounds__(256) pc_lower_kernel(int t0, int t1, int bn, int PL, const int *Lcol,
                                                       const T *Lval, const T *LU, T *b) {
    const int k = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t1) return;
    constexpr int B2 = B * B;
    T arr[B];
#pragma unroll
    for (int r = 0; r < B; ++r) arr[r] = b[(long long)k * B + r];
    ell_row_products<T, T, T, B, PW, -1>(k, bn, PL, Lcol, Lval, b, arr);
    if constexpr (MODE == PC_BLUSGS) {
        T lu[B2];
#pragma unroll
        for (int e = 0; e < B2; ++e) lu[e] = __ldg(LU + (long long)e * bn + k);
        lusub_dev<T, B, kFold>(lu, arr);  // reciprocal pivots in the fast build (pc_prepare)
    }
#pragma unroll
    for (int r = 0; r < B; ++r) b[(long long)k * B + r] = arr[r];
}

template <typename T, int B, int PW, int MODE>
__global__ void __launch_bounds__(256) pc_upper_kernel(int t0, int t1, int bn, int PU, const int *Ucol,
                                                       const T *Uval, const T *LU, T *b) {
    const int k = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t1) return;
    constexpr int B2 = B * B;
    T arr[B];
    if constexpr (MODE == PC_BLUSGS) {
#pragma unroll
        for (int r = 0; r < B; ++r) arr[r] = T(0);
        ell_row_products<T, T, T, B, PW, +1>(k, bn, PU, Ucol, Uval, b, arr);
    } else {
#pragma unroll
        for (int r = 0; r < B; ++r) arr[r] = b[(long long)k * B + r];
        ell_row_products<T, T, T, B, PW, -1>(k, bn, PU, Ucol, Uval, b, arr);
    }
    if constexpr (MODE == PC_ILU) {
        static_assert(B == 1, "scalar ILU is B = 1");
        arr[0] = arr[0] / __ldg(LU + k);
    } else {
        T lu[B2];
#pragma unroll
        for (int e = 0; e < B2; ++e) lu[e] = __ldg(LU + (long long)e * bn + k);
        // the BLU-SGS factors carry reciprocal pivots in the fast build; the
        // ILU factors come from the factorisation, as the reference stores them
        if constexpr (MODE == PC_BLUSGS) lusub_dev<T, B, kFold>(lu, arr);
        else lusub_dev<T, B>(lu, arr);
    }
#pragma unroll
    for (int r = 0; r < B; ++r) {
        if constexpr (MODE == PC_BLUSGS) b[(long long)k * B + r] -= arr[r];
        else b[(long long)k * B + r] = arr[r];
    }
}

// One level of the ILU(0) factorisation in place on the caller's BSR
// values (row-major B x B blocks in CSR slot order), one thread per row
// (rows[t] for t in [t0, t1), every lower neighbour already final):
// precon/bilu.c:5-62 (SCALAR false) or precon/ilu.c:4-47 (SCALAR, B = 1).
// For each lower slot k of row i in order: A_ik := A_ik inv(A_kk)
// (lusubmattrans; A_ik / a_kk when SCALAR), then A_ij -= A_ik A_kj for
// every later slot j whose column row k holds (the last such slot of row k,
// as the reference's column map keeps); finally the diagonal block is
// LU-factorised (block ILU only).
template <int B, bool SCALAR>
__global__ void ilu_factor_kernel(int t0, int t1, const int *rows, const int *rowptr, const int *colidx,
                                  const int *diagslots, double *vals) {
    const int t = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= t1) return;
    constexpr int B2 = B * B;
    const int i = rows ? rows[t] : t;
    const int st = rowptr[i], ed = diagslots[i], jed = rowptr[i + 1];
    for (int kd = st; kd < ed; ++kd) {
        const int ck = colidx[kd], kk = diagslots[ck], kst = rowptr[ck], ked = rowptr[ck + 1];
        double aik[B2];
#pragma unroll
        for (int e = 0; e < B2; ++e) aik[e] = vals[(long long)kd * B2 + e];
        if constexpr (SCALAR) {
            aik[0] = aik[0] / vals[kk];
        } else {
            double lu[B2];
#pragma unroll
            for (int e = 0; e < B2; ++e) lu[e] = vals[(long long)kk * B2 + e];
            lusubmattrans_dev<double, B>(lu, aik);
        }
#pragma unroll
        for (int e = 0; e < B2; ++e) vals[(long long)kd * B2 + e] = aik[e];
        for (int jj = kd + 1; jj < jed; ++jj) {
            const int cj = colidx[jj];
            int iwj = -1;
            for (int q = kst; q < ked; ++q)
                if (colidx[q] == cj) iwj = q;
            if (iwj < 0) continue;
            const double *akj = vals + (long long)iwj * B2;
            double *aij = vals + (long long)jj * B2;
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
                for (int c = 0; c < B; ++c) {
                    double v = 0.0;
#pragma unroll
                    for (int e = 0; e < B; ++e) v += aik[r * B + e] * akj[e * B + c];
                    aij[r * B + c] -= v;
                }
        }
    }
    if constexpr (!SCALAR) {
        double d[B2];
#pragma unroll
        for (int e = 0; e < B2; ++e) d[e] = vals[(long long)ed * B2 + e];
        ludcmp_dev<double, B>(d);
#pragma unroll
        for (int e = 0; e < B2; ++e) vals[(long long)ed * B2 + e] = d[e];
    }
}

// Vector permutation / precision change between the caller's order and
// the level-major order of a preconditioner: dst[k] = src[perm[k]].
template <typename Ts, typename Td>
__global__ void gather_rows_kernel(int bn, int B, const int *perm, const Ts *src, Td *dst) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)bn * B) return;
    const long long k = t / B, r = t - k * B;
    const long long s = perm ? (long long)perm[k] : k;
    dst[t] = (Td)src[s * B + r];
}

template <typename Ts, typename Td>
__global__ void scatter_rows_kernel(int bn, int B, const int *perm, const Ts *src, Td *dst) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)bn * B) return;
    const long long k = t / B, r = t - k * B;
    const long long d = perm ? (long long)perm[k] : k;
    dst[d * B + r] = (Td)src[t];
}

// ---- GMRES(m) device pieces (gmres.c:4-129) --------------------------------
constexpr int kMaxK = 32;  // restart length + 1 <= kMaxK

// Grid of the reduction kernels: capped so the per-block partial buffers
// stay small (8 blocks x 152 SMs).
constexpr int kRedBlocks = 1216;
__host__ __device__ inline int gm_grid(long long n) {
    const long long g = (n + kBlock - 1) / kBlock;
    return (int)(g < kRedBlocks ? (g > 0 ? g : 1) : kRedBlocks);
}

// Per-block partial dots h[k] = sum_i V[k][i] * w[i], k < K.
// Block partials of KM accumulators (only the first KK meaningful) into
// part[block][k].
template <int KM>
__device__ __forceinline__ void gm_block_partials(const double *acc, int KK, double *part) {
    __shared__ double sm[KM][9];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < KM; ++k) {
        if (k < KK) {
            double v = acc[k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
            if (lane == 0) sm[k][wid] = v;
        }
    }
    __syncthreads();
    if (threadIdx.x < KK) {
        double s = 0.0;
        const int nw = blockDim.x >> 5;
        for (int q = 0; q < nw; ++q) s += sm[threadIdx.x][q];
        part[(long long)blockIdx.x * kMaxK + threadIdx.x] = s;
    }
}

// Basis vectors whose entries a thread of the orthogonalisation kernels
// holds in registers at once (all K when K <= 16, else chunks of 8).
template <int KM>
__host__ __device__ constexpr int gm_chunk() { return KM <= 16 ? KM : 8; }

__device__ __forceinline__ double2 ld_pair(const double *row, long long j) {
    return reinterpret_cast<const double2 *>(row)[j];
}

// Per-block partial dots h[k] = sum_i V[k][i] * w[i], k < K <= KM.  A thread
// takes two adjacent entries per step with 16-byte loads (every basis row
// starts on a 32-entry boundary) and requests the pair of every vector of a
// chunk before the first product, so each thread keeps many loads in flight;
// an odd last entry is added by the first thread.  (A layout spreading the
// vectors over the warps of a block, with the sums meeting in shared memory,
// measured slower: its barriers and idle warps at small K cost more than the
// occupancy it gains.)
template <int KM>
__global__ void __launch_bounds__(256, 2) gm_dots_kernel(long long n, int K, const double *V, long long ldv,
                                                         const double *w, double *part) {
    constexpr int CH = gm_chunk<KM>();
    double acc[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) acc[k] = 0.0;
    const long long n2 = n >> 1;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n2;
         j += (long long)gridDim.x * blockDim.x) {
        const double2 wi = ld_pair(w, j);
#pragma unroll
        for (int k0 = 0; k0 < KM; k0 += CH) {
            double2 v[CH];
#pragma unroll
            for (int c = 0; c < CH; ++c) v[c] = k0 + c < K ? ld_pair(V + (k0 + c) * ldv, j) : make_double2(0.0, 0.0);
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                acc[k0 + c] += v[c].x * wi.x;
                acc[k0 + c] += v[c].y * wi.y;
            }
        }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const double wi = w[n - 1];
#pragma unroll
        for (int k = 0; k < KM; ++k)
            if (k < K) acc[k] += V[k * ldv + n - 1] * wi;
    }
    gm_block_partials<KM>(acc, K, part);
}

// w_out = w - V h (gemvcol with alpha -1, beta 1), then either the partial
// dots V^T w_out (mode 0) or the partial sum of w_out^2 (mode 1).  Two
// adjacent entries per thread and step, as in gm_dots_kernel, the loaded
// entries of V staying in registers for the second product; for more than 16
// vectors one entry per thread, so that all of them still fit.  With more
// than 8 vectors one block per SM (up to 255 registers, no spills) still
// keeps over 100 KB of loads in flight per SM.
template <int KM>
__global__ void __launch_bounds__(256, (KM > 8 ? 1 : 2)) gm_update_kernel(long long n, int K, const double *V,
                                                                          long long ldv, const double *h, double *w,
                                                                          int mode, double *part) {
    constexpr int CH = gm_chunk<KM>();
    double acc[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) acc[k] = 0.0;
    __shared__ double hs[KM];
    if (threadIdx.x < KM) hs[threadIdx.x] = threadIdx.x < K ? h[threadIdx.x] : 0.0;
    __syncthreads();
    if constexpr (KM > 16) {
        // one entry per thread: all K values of V stay in registers for the
        // second product (pairs of 32 vectors would not fit)
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
             i += (long long)gridDim.x * blockDim.x) {
            double v[KM];
#pragma unroll
            for (int k = 0; k < KM; ++k) v[k] = k < K ? V[k * ldv + i] : 0.0;
            double sq = 0.0;
#pragma unroll
            for (int k = 0; k < KM; ++k) sq += v[k] * hs[k];
            const double wn = -1.0 * sq + 1.0 * w[i];
            w[i] = wn;
            if (mode == 0) {
#pragma unroll
                for (int k = 0; k < KM; ++k) acc[k] += v[k] * wn;
            } else {
                acc[0] += wn * wn;
            }
        }
        gm_block_partials<KM>(acc, mode == 0 ? K : 1, part);
        return;
    }
    const long long n2 = n >> 1;
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < n2;
         j += (long long)gridDim.x * blockDim.x) {
        double sx = 0.0, sy = 0.0;
        double2 v[CH];
#pragma unroll
        for (int k0 = 0; k0 < KM; k0 += CH) {
#pragma unroll
            for (int c = 0; c < CH; ++c) v[c] = k0 + c < K ? ld_pair(V + (k0 + c) * ldv, j) : make_double2(0.0, 0.0);
#pragma unroll
            for (int c = 0; c < CH; ++c) {
                sx += v[c].x * hs[k0 + c];
                sy += v[c].y * hs[k0 + c];
            }
        }
        const double2 wo = ld_pair(w, j);
        double2 wn;
        wn.x = -1.0 * sx + 1.0 * wo.x;
        wn.y = -1.0 * sy + 1.0 * wo.y;
        reinterpret_cast<double2 *>(w)[j] = wn;
        if (mode == 0) {
#pragma unroll
            for (int k0 = 0; k0 < KM; k0 += CH) {
                if (CH < KM) {
#pragma unroll
                    for (int c = 0; c < CH; ++c)
                        v[c] = k0 + c < K ? ld_pair(V + (k0 + c) * ldv, j) : make_double2(0.0, 0.0);
                }
#pragma unroll
                for (int c = 0; c < CH; ++c) {
                    acc[k0 + c] += v[c].x * wn.x;
                    acc[k0 + c] += v[c].y * wn.y;
                }
            }
        } else {
            acc[0] += wn.x * wn.x;
            acc[0] += wn.y * wn.y;
        }
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
        const long long i = n - 1;
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < KM; ++k)
            if (k < K) s += V[k * ldv + i] * hs[k];
        const double wn = -1.0 * s + 1.0 * w[i];
        w[i] = wn;
        if (mode == 0) {
#pragma unroll
            for (int k = 0; k < KM; ++k)
                if (k < K) acc[k] += V[k * ldv + i] * wn;
        } else {
            acc[0] += wn * wn;
        }
    }
    gm_block_partials<KM>(acc, mode == 0 ? K : 1, part);
}

// Sum of part[b * stride] over b < nb by a whole block: a fixed assignment
// of partials to threads and a fixed tree, so every call gives the same
// value; valid in thread 0.
__device__ __forceinline__ double block_sum_partials(const double *part, int nb, long long stride) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b * stride];
    return block_sum(s);
}

// Sum the per-block partials: out[k] = sum_b part[b][k] (block k, fixed order).
__global__ void __launch_bounds__(256) gm_reduce_kernel(int nblocks, const double *part, double *out,
                                                        int accumulate) {
    const int k = blockIdx.x;
    const double s = block_sum_partials(part + k, nblocks, kMaxK);
    if (threadIdx.x == 0) {
        if (accumulate) out[k] += 1.0 * s;
        else out[k] = s;
    }
}

// Sum of squares partials (one value per block) into *out (sqrt applied).
__global__ void __launch_bounds__(256) gm_sumsq_kernel(long long n, const double *x, double *part) {
    double s = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        s += x[i] * x[i];
    s = block_sum(s);
    if (threadIdx.x == 0) part[(long long)blockIdx.x * kMaxK] = s;
}

// State shared by the device-side Givens step (one per solve).
struct GmState {
    int k;        // Arnoldi steps completed in this cycle
    int stop;     // happy breakdown seen in this cycle
    int total;    // Arnoldi steps over the whole solve
    int pad;
    double beta;  // ||M^-1 r|| of this cycle
    double inv;   // 1 / (latest subdiagonal), applied to the next basis vector
};

// Cycle start: beta = sqrt(sum), y[0] = beta, inv = 1/beta, flags reset.
__global__ void __launch_bounds__(256) gm_cycle_begin_kernel(int nblocks, const double *part, GmState *st,
                                                             double *y, double *out_norm) {
    const double s = block_sum_partials(part, nblocks, kMaxK);
    if (threadIdx.x != 0) return;
    const double beta = sqrt(s);
    st->beta = beta;
    st->inv = 1.0 / beta;
    st->k = 0;
    st->stop = 0;
    y[0] = beta;
    if (out_norm) *out_norm = beta;
}

// dst = inv * src (dcopy + dscal(1/h), gmres.c:75-77 / 122-123); skipped
// after a breakdown.
__global__ void gm_scale_kernel(long long n, const GmState *st, const double *src, double *dst) {
    if (st->stop) return;
    const double inv = st->inv;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        dst[i] = inv * src[i];
}

// Arnoldi step j tail: H[:,j] = h1 + h2, H[j+1,j] = ||w||, previous
// rotations, new rotation, y update and happy-breakdown test
// (gmres.c:81-107 and 86-103).
// rel_floor > 0 (mixed precision only): the cycle also ends (stop = 2) once
// the Givens residual estimate |y[j+1]| falls below rel_floor * beta, the
// accuracy an FP32 operator can deliver; the FP64 restart then refreshes the
// true residual.
__global__ void __launch_bounds__(256) gm_givens_kernel(int j, int ld, int nblocks, const double *part_norm,
                                                        double *H, const double *h2, double *cs, double *sn,
                                                        double *y, double haptol, double rel_floor, GmState *st) {
    if (st->stop) return;  // the same for every thread of the block
    const double s = block_sum_partials(part_norm, nblocks, kMaxK);
    if (threadIdx.x != 0) return;
    double *Hc = H + (long long)j * ld;
    for (int i = 0; i <= j; ++i) Hc[i] += 1.0 * h2[i];
    const double hsub = sqrt(s);
    Hc[j + 1] = hsub;
    st->inv = 1.0 / hsub;
    for (int i = 0; i < j; ++i) {
        const double c = cs[i], sv = sn[i];
        const double t = c * Hc[i] + sv * Hc[i + 1];
        Hc[i + 1] = -sv * Hc[i] + c * Hc[i + 1];
        Hc[i] = t;
    }
    const double h1v = Hc[j], h2v = Hc[j + 1];
    const double rr = hypot(h1v, h2v);
    cs[j] = h1v / rr;
    sn[j] = h2v / rr;
    Hc[j] = cs[j] * Hc[j] + sn[j] * Hc[j + 1];
    Hc[j + 1] = 0.0;
    y[j + 1] = -sn[j] * y[j];
    y[j] = cs[j] * y[j];
    st->k = j + 1;
    st->total += 1;
    if (hsub < haptol * st->beta) st->stop = 1;
    else if (rel_floor > 0.0 && fabs(y[j + 1]) <= rel_floor * st->beta) st->stop = 2;
}

// Back substitution of the k x k triangle (gmres.c:111-117).
__global__ void gm_backsub_kernel(int ld, const double *H, double *y, const GmState *st) {
    const int k = st->k;
    for (int i = k - 1; i >= 0; --i) {
        double s = y[i];
        for (int jj = i + 1; jj < k; ++jj) s -= H[i + (long long)jj * ld] * y[jj];
        y[i] = s / H[i + (long long)i * ld];
    }
}

// x += V[:, :k] y (gemvcol with alpha 1, beta 1, gmres.c:120).
__global__ void __launch_bounds__(256) gm_solution_kernel(long long n, const double *V, long long ldv,
                                                          const double *y, const GmState *st,
                                                          double *x) {
    __shared__ double ys[kMaxK];
    const int k = st->k;
    if (threadIdx.x < kMaxK) ys[threadIdx.x] = threadIdx.x < k ? y[threadIdx.x] : 0.0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < k; ++q) s += V[q * ldv + i] * ys[q];
        x[i] = 1.0 * s + 1.0 * x[i];
    }
}

// ---- BiCGSTAB ----------------------------------------------------------------
// BICGSTABSolve (src/krylov/solver/bicgstab.c:24-128) with every scalar on
// the device: an iteration is a fixed sequence of launches with no host
// round trip.  Once a breakdown, convergence or the iteration limit is
// recorded (stop), every later kernel of the sequence returns at once, so
// the host may queue several iterations between its checks.
struct BcState {
    double rho, rhoprev, alpha, omega, rho_new, resnorm;
    int iter, stop, stat, conv;
};

// Per-block partial sums of (x, y) into part[block] (grid-stride).
__global__ void __launch_bounds__(256) bc_dot_kernel(long long n, const double *x, const double *y, double *part,
                                                     const BcState *st) {
    if (st && st->stop) return;
    double t = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        t += x[i] * y[i];
    t = block_sum(t);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// rho_0 = (r~, r_0), rhoprev = alpha = omega = 1 (bicgstab.c:52-56); a
// rho breakdown (|rho| < 1e-30, bicgstab.c:59-62) ends the solve.
__global__ void bc_start_kernel(int nb, const double *part, BcState *st, int maxiter) {
    double rho = 0.0;
    for (int b = 0; b < nb; ++b) rho += part[b];
    st->rho = rho;
    st->rhoprev = 1.0;
    st->alpha = 1.0;
    st->omega = 1.0;
    st->rho_new = 0.0;
    st->resnorm = 0.0;
    st->iter = 0;
    st->stop = 0;
    st->stat = -1;
    st->conv = 0;
    if (fabs(rho) < 1e-30) {
        st->stat = 3;
        st->stop = 1;
    } else if (maxiter <= 0) {
        st->stop = 1;
    }
}

// p := r (first iteration) or r + beta (p - omega v) as daxpy, dscal, daxpy
// (bicgstab.c:68-75); pt := p (the preconditioner then works on pt).
__global__ void __launch_bounds__(256) bc_direction_kernel(long long n, const BcState *st, const double *r,
                                                           const double *v, double *p, double *pt) {
    if (st->stop) return;
    const bool first = st->iter == 0;
    const double omega = st->omega;
    const double beta = first ? 0.0 : (st->rho / st->rhoprev) * (st->alpha / st->omega);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double q;
        if (first) {
            q = r[i];
        } else {
            q = p[i] + (-omega) * v[i];
            q = beta * q;
            q = q + 1.0 * r[i];
        }
        p[i] = q;
        pt[i] = q;
    }
}

// pi = (r~, v); alpha = rho / pi, or a pi breakdown (bicgstab.c:81-86).
__global__ void bc_alpha_kernel(int nb, const double *part, BcState *st) {
    if (st->stop) return;
    double pi = 0.0;
    for (int b = 0; b < nb; ++b) pi += part[b];
    if (fabs(pi) < 1e-30) {
        st->stat = 4;
        st->stop = 1;
    } else {
        st->alpha = st->rho / pi;
    }
}

// s := r - alpha v, shat := s (bicgstab.c:89-94).
__global__ void __launch_bounds__(256) bc_s_kernel(long long n, const BcState *st, const double *r,
                                                   const double *v, double *sv, double *shat) {
    if (st->stop) return;
    const double a = st->alpha;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double q = r[i] + (-a) * v[i];
        sv[i] = q;
        shat[i] = q;
    }
}

// The fused five-term reduction of bicgstab.c:5-22: per-block partials of
// (r~,s), (r~,t), (t,s), (t,t), (s,s) into part[5*block + j].
__global__ void __launch_bounds__(256) bc_fused5_kernel(long long n, const double *rt, const double *sv,
                                                        const double *t, double *part, const BcState *st) {
    if (st->stop) return;
    double a = 0.0, b = 0.0, c = 0.0, d = 0.0, e = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double sk = sv[i], tk = t[i], rk = rt[i];
        a += rk * sk;
        b += rk * tk;
        c += tk * sk;
        d += tk * tk;
        e += sk * sk;
    }
    a = block_sum(a);
    b = block_sum(b);
    c = block_sum(c);
    d = block_sum(d);
    e = block_sum(e);
    if (threadIdx.x == 0) {
        double *q = part + 5ll * blockIdx.x;
        q[0] = a;
        q[1] = b;
        q[2] = c;
        q[3] = d;
        q[4] = e;
    }
}

// omega = (t,s)/(t,t), rho_new = phi - omega (r~,t) and the residual
// estimate sqrt|ss - 2 omega ts + omega^2 tt| (bicgstab.c:101-118);
// conv when it is below tol.
__global__ void bc_omega_kernel(int nb, const double *part, BcState *st, double tol, double *hist) {
    if (st->stop) return;
    double phi = 0.0, rtt = 0.0, ts = 0.0, tt = 0.0, ss = 0.0;
    for (int b = 0; b < nb; ++b) {
        const double *q = part + 5ll * b;
        phi += q[0];
        rtt += q[1];
        ts += q[2];
        tt += q[3];
        ss += q[4];
    }
    // (t, t) == 0 means s == 0 (t = A inv(M) s): x + alpha pt already solves
    // the system.  The reference divides regardless (0/0 = NaN, after which
    // it never converges); omega = 0 gives r = s = 0 and a zero estimate.
    const double omega = tt != 0.0 ? ts / tt : 0.0;
    st->omega = omega;
    st->rho_new = phi - omega * rtt;
    const double res = sqrt(fabs(ss - 2.0 * omega * ts + omega * omega * tt));
    st->resnorm = res;
    if (hist) hist[st->iter] = res;
    st->conv = res < tol ? 1 : 0;
}

// x += alpha pt; x += omega shat; r := s - omega t (bicgstab.c:106-112).
__global__ void __launch_bounds__(256) bc_update_kernel(long long n, const BcState *st, const double *pt,
                                                        const double *shat, const double *sv, const double *t,
                                                        double *x, double *r) {
    if (st->stop) return;
    const double a = st->alpha, w = st->omega;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double xi = x[i] + a * pt[i];
        x[i] = xi + w * shat[i];
        r[i] = sv[i] + (-w) * t[i];
    }
}

// Converged, or rhoprev = rho, rho = rho_new, iter++ (bicgstab.c:120-128).
__global__ void bc_advance_kernel(BcState *st, int maxiter) {
    if (st->stop) return;
    if (st->conv) {
        st->stat = 0;
        st->stop = 1;
        return;
    }
    st->rhoprev = st->rho;
    st->rho = st->rho_new;
    st->iter += 1;
    if (st->iter >= maxiter) st->stop = 1;
}

}  // namespace UCFD_KNS
