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

// acc[r] += SGN * sum over the ELL row k of (block_p x_{col_p})[r], entries in
// stored order, each block product summed over its columns first (the
// reference's order, sparsemat.c:82-97, blusgs.c:113-124).  PW > 0: the
// row width is at most PW and the loop is unrolled so that every column
// index, then every gathered x and block value, is requested up front;
// PW == 0: runtime-width loop.  Padding entries (column < 0) end the row.
template <typename Tv, typename Tx, typename Ta, int B, int PW, int SGN>
__device__ __forceinline__ void ell_row_products(long long k, int bn, int P, const int *col, const Tv *val,
                                                 const Tx *x, Ta *acc) {
    constexpr int B2 = B * B;
    if constexpr (PW > 0) {
        int c[PW];
#pragma unroll
        for (int p = 0; p < PW; ++p) c[p] = p < P ? __ldg(col + (long long)p * bn + k) : -1;
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
                    for (int cc = 0; cc < B; ++cc) v += (Ta)__ldg(vp + (long long)(r * B + cc) * bn) * xv[p][cc];
                    if (SGN > 0) acc[r] += v;
                    else acc[r] -= v;
                }
            }
        }
    } else {
        for (int p = 0; p < P; ++p) {
            const int c = __ldg(col + (long long)p * bn + k);
            if (c < 0) break;
            Ta xv[B];
#pragma unroll
            for (int cc = 0; cc < B; ++cc) xv[cc] = (Ta)x[(long long)c * B + cc];
            const Tv *vp = val + (long long)p * B2 * bn + k;
#pragma unroll
            for (int r = 0; r < B; ++r) {
                Ta v = Ta(0);
#pragma unroll
                for (int cc = 0; cc < B; ++cc) v += (Ta)__ldg(vp + (long long)(r * B + cc) * bn) * xv[cc];
                if (SGN > 0) acc[r] += v;
                else acc[r] -= v;
            }
        }
    }
}

// SpMV_BSR: sparsemat.c:57-101 -- y = alpha*A*x + beta*y.  Tv is the type
// of the stored values, Ta the accumulation type.
template <typename Tv, typename Ta, int B, int PW>
__global__ void __launch_bounds__(256) bsr_spmv_kernel(int bn, int P, const int *col, const Tv *val,
                                                       double alpha, const double *x, double beta,
                                                       double *y) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bn) return;
    Ta acc[B];
#pragma unroll
    for (int r = 0; r < B; ++r) acc[r] = Ta(0);
    ell_row_products<Tv, double, Ta, B, PW, +1>(i, bn, P, col, val, x, acc);
#pragma unroll
    for (int r = 0; r < B; ++r) {
        const long long o = (long long)i * B + r;
        y[o] = alpha * (double)acc[r] + beta * y[o];
    }
}

// BLUSGSPreconPrepare: precon/blusgs.c:7-26 -- copy each diagonal block and
// LU-factor it (FP64), optionally rounding the factors to Tl.
template <typename Tl, int B>
__global__ void pc_prepare_kernel(int bn, const int *perm, const long long *dslot,
                                  const double *values, double *LU64, Tl *LU_l) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= bn) return;
    constexpr int B2 = B * B;
    const long long s = dslot[perm ? perm[k] : k];
    double d[B2];
#pragma unroll
    for (int e = 0; e < B2; ++e) d[e] = values[s * B2 + e];
    ludcmp_dev<double, B>(d);
#pragma unroll
    for (int e = 0; e < B2; ++e) {
        LU64[(long long)e * bn + k] = d[e];
        if (LU_l) LU_l[(long long)e * bn + k] = (Tl)d[e];
    }
}

// Forward (lower) step of the block SGS apply for rows [t0, t1) of one
// level: precon/blusgs.c:104-130 (b -> x' in place).
template <typename T, int B, int PW>
__global__ void __launch_bounds__(256) pc_lower_kernel(int t0, int t1, int bn, int PL, const int *Lcol,
                                                       const T *Lval, const T *LU, T *b) {
    const int k = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t1) return;
    constexpr int B2 = B * B;
    T arr[B];
#pragma unroll
    for (int r = 0; r < B; ++r) arr[r] = b[(long long)k * B + r];
    ell_row_products<T, T, T, B, PW, -1>(k, bn, PL, Lcol, Lval, b, arr);
    T lu[B2];
#pragma unroll
    for (int e = 0; e < B2; ++e) lu[e] = __ldg(LU + (long long)e * bn + k);
    lusub_dev<T, B>(lu, arr);
#pragma unroll
    for (int r = 0; r < B; ++r) b[(long long)k * B + r] = arr[r];
}

// Backward (upper) step: precon/blusgs.c:132-161 (x = x' - inv(D) U x).
template <typename T, int B, int PW>
__global__ void __launch_bounds__(256) pc_upper_kernel(int t0, int t1, int bn, int PU, const int *Ucol,
                                                       const T *Uval, const T *LU, T *b) {
    const int k = t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= t1) return;
    constexpr int B2 = B * B;
    T arr[B];
#pragma unroll
    for (int r = 0; r < B; ++r) arr[r] = T(0);
    ell_row_products<T, T, T, B, PW, +1>(k, bn, PU, Ucol, Uval, b, arr);
    T lu[B2];
#pragma unroll
    for (int e = 0; e < B2; ++e) lu[e] = __ldg(LU + (long long)e * bn + k);
    lusub_dev<T, B>(lu, arr);
#pragma unroll
    for (int r = 0; r < B; ++r) b[(long long)k * B + r] -= arr[r];
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

// Per-block partial dots h[k] = sum_i V[k][i] * w[i], k < K <= KM.
template <int KM>
__global__ void __launch_bounds__(256, (KM > 8 ? 3 : 4)) gm_dots_kernel(long long n, int K, const double *V, long long ldv,
                                                      const double *w, double *part) {
    double acc[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) acc[k] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double wi = w[i];
#pragma unroll
        for (int k = 0; k < KM; ++k)
            if (k < K) acc[k] += V[k * ldv + i] * wi;
    }
    gm_block_partials<KM>(acc, K, part);
}

// w_out = w - V h (gemvcol with alpha -1, beta 1), then either the partial
// dots V^T w_out (mode 0) or the partial sum of w_out^2 (mode 1).  The
// second pass over V re-reads the values this thread just loaded (L1).
template <int KM>
__global__ void __launch_bounds__(256, (KM > 8 ? 2 : 4)) gm_update_kernel(long long n, int K, const double *V, long long ldv,
                                                        const double *h, double *w, int mode,
                                                        double *part) {
    double acc[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) acc[k] = 0.0;
    __shared__ double hs[KM];
    if (threadIdx.x < KM) hs[threadIdx.x] = threadIdx.x < K ? h[threadIdx.x] : 0.0;
    __syncthreads();
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
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

// Sum the per-block partials: out[k] = sum_b part[b][k] (one block, fixed order).
__global__ void gm_reduce_kernel(int nblocks, int K, const double *part, double *out, int accumulate) {
    const int k = threadIdx.x;
    if (k >= K) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(long long)b * kMaxK + k];
    if (accumulate) out[k] += 1.0 * s;
    else out[k] = s;
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
__global__ void gm_cycle_begin_kernel(int nblocks, const double *part, GmState *st, double *y,
                                      double *out_norm) {
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[(long long)b * kMaxK];
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
__global__ void gm_givens_kernel(int j, int ld, int nblocks, const double *part_norm, double *H,
                                 const double *h2, double *cs, double *sn, double *y, double haptol,
                                 double rel_floor, GmState *st) {
    if (st->stop) return;
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part_norm[(long long)b * kMaxK];
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

}  // namespace UCFD_KNS
