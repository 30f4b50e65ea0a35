// kernels_blusgs.cuh -- block LU-SGS kernels on the level-major internal layout.
//
// Internal arrays (N = internal cells, P = ELL width, B = block size):
//   nei [P][N] (-1 padding), fa [P][N], rv [N]
//   J   tiled, m = P*B*B (element p*B*B + r*B + c): the off-diagonal block
//                    each cell-face multiplies its neighbour increment with
//                    (jmat half 1 when side == 1, minus half 0 otherwise,
//                    blusgs.c:307-310)
//   D   tiled, m = B*B   unfactored diagonal block (FP64)
//   LU  tiled, m = B*B   its in-place LU factors (ludcmp, inverse.h:13-45)
//   rhs, du [nvars][N]
// "tiled" is the cell-tile layout of kargs.h (tile_index).
#pragma once

#include "kernels_common.cuh"

namespace UCFD_KNS {

// ludcmp: src/lusgs/inverse.h:13-45 (Doolittle, no pivoting, row by row).
// RCP: multiply by the reciprocal of each pivot (B - 1 divisions instead of
// B(B-1)/2 + B - 1) -- used in the fast build: x * (1/p) differs from x / p
// by at most a rounding at the 1e-16 level.  RSTORE (with RCP): the
// diagonal then holds the reciprocal pivots 1/p instead of p, for
// lusub_dev<..., true>.  The exact build keeps the reference's divisions.
template <typename T, int B, bool RCP = false, bool RSTORE = false>
__device__ __forceinline__ void ludcmp_dev(T *A) {
    static_assert(RCP || !RSTORE, "reciprocal pivots are stored by the RCP form");
    if constexpr (B == 1) {
        A[0] = T(1) / A[0];
    } else if constexpr (RCP) {
        T ip[B];
        ip[0] = T(1) / A[0];
#pragma unroll
        for (int row = 1; row < B; ++row) {
            const int nr = B * row;
            A[nr] *= ip[0];
#pragma unroll
            for (int col = 1; col < B; ++col) {
                T v = T(0);
                if (row > col) {
#pragma unroll
                    for (int k = 0; k < col; ++k) v += A[nr + k] * A[col + B * k];
                    A[nr + col] = (A[nr + col] - v) * ip[col];
                } else {
#pragma unroll
                    for (int k = 0; k < row; ++k) v += A[nr + k] * A[B * k + col];
                    A[nr + col] -= v;
                }
            }
            // the row's pivot is final now (pivots are read only through ip)
            if (row + 1 < B || RSTORE) ip[row] = T(1) / A[(B + 1) * row];
        }
        if constexpr (RSTORE) {
#pragma unroll
            for (int row = 0; row < B; ++row) A[(B + 1) * row] = ip[row];
        }
    } else {
#pragma unroll
        for (int row = 1; row < B; ++row) {
            const int nr = B * row;
            A[nr] /= A[0];
#pragma unroll
            for (int col = 1; col < B; ++col) {
                T v = T(0);
                if (row > col) {
#pragma unroll
                    for (int k = 0; k < col; ++k) v += A[nr + k] * A[col + B * k];
                    A[nr + col] = (A[nr + col] - v) / A[(B + 1) * col];
                } else {
#pragma unroll
                    for (int k = 0; k < row; ++k) v += A[nr + k] * A[B * k + col];
                    A[nr + col] -= v;
                }
            }
        }
    }
}

// lusub: src/lusgs/inverse.h:51-80 (unit-lower forward, upper backward).
// RCP: the diagonal holds reciprocal pivots (ludcmp_dev RSTORE): multiply.
// (B == 1 stores the reciprocal in both forms, inverse.h:16.)
template <typename T, int B, bool RCP = false>
__device__ __forceinline__ void lusub_dev(const T *LU, T *b) {
    if constexpr (B == 1) {
        b[0] *= LU[0];
    } else {
#pragma unroll
        for (int row = 1; row < B; ++row) {
            T v = T(0);
#pragma unroll
            for (int col = 0; col < row; ++col) v += LU[row * B + col] * b[col];
            b[row] -= v;
        }
        if constexpr (RCP) b[B - 1] *= LU[B * B - 1];
        else b[B - 1] /= LU[B * B - 1];
#pragma unroll
        for (int row = B - 2; row > -1; --row) {
            T v = T(0);
#pragma unroll
            for (int col = row + 1; col < B; ++col) v += LU[row * B + col] * b[col];
            if constexpr (RCP) b[row] = (b[row] - v) * LU[row * B + row];
            else b[row] = (b[row] - v) / LU[row * B + row];
        }
    }
}

// lusubmattrans: src/krylov/utils/inverse.c:79-108.  X := X inv(LU) for a
// row-major B x B block X and factors LU from ludcmp_dev: Y U = X column
// by column, then X L = Y.
template <typename T, int B>
__device__ __forceinline__ void lusubmattrans_dev(const T *LU, T *X) {
    if constexpr (B == 1) {
        X[0] *= LU[0];
    } else {
#pragma unroll
        for (int s = 0; s < B; ++s) X[s * B] /= LU[0];
#pragma unroll
        for (int row = 1; row < B; ++row)
#pragma unroll
            for (int s = 0; s < B; ++s) {
                T v = T(0);
#pragma unroll
                for (int col = 0; col < row; ++col) v += X[s * B + col] * LU[col * B + row];
                X[s * B + row] = (X[s * B + row] - v) / LU[row * B + row];
            }
#pragma unroll
        for (int row = B - 2; row > -1; --row)
#pragma unroll
            for (int s = 0; s < B; ++s) {
                T v = T(0);
#pragma unroll
                for (int col = row + 1; col < B; ++col) v += X[s * B + col] * LU[col * B + row];
                X[s * B + row] -= v;
            }
    }
}

// rank_blusgs_pack: blusgs.c:17-45.  rhs goes to the internal SoA arrays;
// the NS diagonal block starts as (1/dt + a0) I, of which only the scalar
// dd = 1/dt + a0 is stored (the prepare kernel expands it).
template <typename S>
__global__ void fs_blusgs_pack_kernel(int neles, int nvars, int B, long long N, double a0,
                                      const int *cell_ids, const int *iperm, const double *rhs,
                                      const double *dt, S *rhs_s, double *rhs64, double *dd) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) {
        const double x = rhs[idx + (long long)v * neles];
        rhs_s[k + v * N] = (S)x;
        if (rhs64) rhs64[k + v * N] = x;
    }
    dd[k] = 1 / dt[idx] + a0;
}

// rank_tblusgs_pack + kwsst/sa source Jacobians: blusgs.c:60-120,
// source_jacobian.c:6-18.  model 0 = k-omega SST, 1 = Spalart-Allmaras.
__global__ void fs_tblusgs_pack_kernel(int model, int neles, int nvars, int nt, long long N,
                                       double a0, double factor, double betast,
                                       const int *cell_ids, const int *iperm, const double *uptsb,
                                       const double *dsrc, const double *dt, double *D) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    double A[4] = {0.0, 0.0, 0.0, 0.0};
    const double u0 = uptsb[idx];
    if (model == 0) {
        const double kk = uptsb[idx + (long long)(nvars - 2) * neles] / u0;
        A[0] += dsrc[idx + (long long)(nvars - 2) * neles];
        const double bk = betast * kk;
        A[1] += bk > 0.0 ? bk : 0.0;
        A[1 + nt] = dsrc[idx + (long long)(nvars - 1) * neles];
    } else {
        A[0] += dsrc[idx + (long long)(nvars - 1) * neles];
    }
    for (int row = 0; row < nt; ++row) A[row + row * nt] += 1 / (dt[idx] * factor) + a0;
    for (int e = 0; e < nt * nt; ++e) D[::ucfd::tile_index(k, e, nt * nt)] = A[e];
}

// Face Jacobians from the caller's layout jmat[2][B][B][nF] (face index
// fastest) to one contiguous record per face, jt[f][2*B*B], through a
// shared-memory tile: both the reads and the writes are coalesced.  The
// prepare kernel then reads a cell-face's two blocks as 2*B*B*8 contiguous
// bytes instead of 2*B*B separate 8-byte words nF apart.
template <int B>
__global__ void __launch_bounds__(256) jmat_face_major_kernel(long long nF, const double *__restrict__ jmat,
                                                              double *__restrict__ jt) {
    constexpr int R = 2 * B * B;
    constexpr int FT = 32;         // faces per tile
    constexpr int LD = R + 1;      // padded row: fewer shared-memory bank conflicts
    __shared__ double tile[FT * LD];
    const long long f0 = (long long)blockIdx.x * FT;
    const int nf = (int)(nF - f0 < FT ? nF - f0 : FT);
    for (int q = threadIdx.x; q < R * FT; q += blockDim.x) {
        const int e = q / FT, j = q % FT;
        if (j < nf) tile[j * LD + e] = __ldg(jmat + (long long)e * nF + f0 + j);
    }
    __syncthreads();
    double *out = jt + f0 * R;
    for (int q = threadIdx.x; q < nf * R; q += blockDim.x) out[q] = tile[(q / R) * LD + q % R];
}

// x with its sign bit XORed with the top bit of hi_mask (0 or 0x80000000):
// x or -x, bit for bit.  Done as an integer XOR of the high word in PTX so
// the flip stays an integer operation instead of a floating-point negation
// that would occupy the FP64 pipe.
__device__ __forceinline__ double xor_sign(double x, unsigned hi_mask) {
    unsigned hi;
    asm("xor.b32 %0, %1, %2;" : "=r"(hi) : "r"((unsigned)__double2hiint(x)), "r"(hi_mask));
    return __hiloint2double((int)hi, __double2loint(x));
}

// pre_blusgs: blusgs.c:200-246, plus the gather of each cell-face's
// off-diagonal block (the half the sweeps use) into the ELL layout.  The
// fast build (kFold) stores reciprocal pivots and, as the sweep blocks J_s,
// M = D^-1 J fv; J64, the FP64 copy the FP32 mode's residual reads, always
// holds the unscaled blocks.
// The block starts from dd[k] I when dd is given (NS pack), else from D.
// jt holds the face-major records written by jmat_face_major_kernel.
// The side's sign goes into the face factor once per face: the diagonal
// term (side == 1 ? h0 : -h1) * fv is computed as (side == 1 ? h0 : h1) *
// (side == 1 ? fv : -fv), the same value bit for bit (a product's sign is
// the XOR of its operands' signs, its magnitude rounds the same), and the
// stored off-diagonal value -h0 is a sign-bit flip.
template <typename S, int B>
__global__ void fs_blusgs_prepare_kernel(long long N, int P, const int *nei, const int *slot,
                                         const int8_t *side, const double *fa, const double *rv,
                                         const double *jt, const double *dd, double *D, double *LU64,
                                         S *LU_s, S *J_s, double *J64) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= N) return;
    constexpr int B2 = B * B;
    constexpr int R = 2 * B2;  // even: a record is a whole number of 16-byte pairs
    double dm[B2];
    if (dd) {
        const double d = dd[k];
#pragma unroll
        for (int e = 0; e < B2; ++e) dm[e] = (e % (B + 1) == 0) ? d : 0.0;
    } else {
#pragma unroll
        for (int e = 0; e < B2; ++e) dm[e] = D[::ucfd::tile_index(k, e, B2)];
    }
    const long long jbase = ::ucfd::tile_index(k, 0, (long long)P * B2);
    if constexpr (kFold) {
        // Fast build, two passes over the faces.  First the diagonal
        // block from each record's diagonal half (side == 1: half 0, else
        // half 1) only; then, with the block factored, each face's
        // off-diagonal half becomes M = D^-1 J fv in registers and is
        // stored once (no FP32 J stored, read back and rewritten).  Same
        // values as forming J first.
        for (int p = 0; p < P; ++p) {
            if (nei[p * N + k] < 0) break;
            const long long s = slot[p * N + k];
            const bool pos = side[p * N + k] == 1;
            const double fv = fa[p * N + k] * rv[k];
            const double fvs = pos ? fv : -fv;
            const double *hd = jt + s * R + (pos ? 0 : B2);
#pragma unroll
            for (int e = 0; e < B2; ++e) dm[e] += __ldg(hd + e) * fvs;  // == (pos ? h0 : -h1) * fv
        }
        const long long dbase = ::ucfd::tile_index(k, 0, B2);
#pragma unroll
        for (int e = 0; e < B2; ++e) D[dbase + (e << 5)] = dm[e];
        ludcmp_dev<double, B, true, true>(dm);
#pragma unroll
        for (int e = 0; e < B2; ++e) {
            if (LU64) LU64[dbase + (e << 5)] = dm[e];
            if (LU_s) LU_s[dbase + (e << 5)] = (S)dm[e];
        }
        S lu[B2];
#pragma unroll
        for (int e = 0; e < B2; ++e) lu[e] = (S)dm[e];
        for (int p = 0; p < P; ++p) {
            if (nei[p * N + k] < 0) break;
            const long long s = slot[p * N + k];
            const bool pos = side[p * N + k] == 1;
            const double fv = fa[p * N + k] * rv[k];
            const unsigned neg = pos ? 0u : 0x80000000u;
            const double *ho = jt + s * R + (pos ? B2 : 0);
            S m[B2];
#pragma unroll
            for (int e = 0; e < B2; ++e) {
                const double jv = xor_sign(__ldg(ho + e), neg);  // == pos ? h1 : -h0
                const long long o = jbase + ((long long)(p * B2 + e) << 5);
                if (J64) J64[o] = jv;
                m[e] = (S)(jv * fv);
            }
            // M = D^-1 (J fv), column by column through the factors just
            // formed (in the sweep precision)
#pragma unroll
            for (int c = 0; c < B; ++c) {
                S col[B];
#pragma unroll
                for (int r = 0; r < B; ++r) col[r] = m[r * B + c];
                lusub_dev<S, B, true>(lu, col);
#pragma unroll
                for (int r = 0; r < B; ++r) m[r * B + c] = col[r];
            }
#pragma unroll
            for (int e = 0; e < B2; ++e) J_s[jbase + ((long long)(p * B2 + e) << 5)] = m[e];
        }
        return;
    }
    for (int p = 0; p < P; ++p) {
        if (nei[p * N + k] < 0) break;
        const long long s = slot[p * N + k];
        const bool pos = side[p * N + k] == 1;
        const double fv = fa[p * N + k] * rv[k];
        const double fvs = pos ? fv : -fv;
        const unsigned neg = pos ? 0u : 0x80000000u;
        double h[R];
        const double2 *rec = reinterpret_cast<const double2 *>(jt + s * R);
#pragma unroll
        for (int q = 0; q < R / 2; ++q) {
            const double2 v = __ldg(rec + q);
            h[2 * q] = v.x;
            h[2 * q + 1] = v.y;
        }
#pragma unroll
        for (int r = 0; r < B; ++r) {
#pragma unroll
            for (int c = 0; c < B; ++c) {
                const double h0 = h[r * B + c], h1 = h[B2 + r * B + c];
                dm[c + r * B] += (pos ? h0 : h1) * fvs;    // == (pos ? h0 : -h1) * fv
                const double jv = xor_sign(pos ? h1 : h0, neg);  // == pos ? h1 : -h0
                const long long o = jbase + ((long long)(p * B2 + r * B + c) << 5);
                J_s[o] = (S)jv;
                if (J64) J64[o] = jv;
            }
        }
    }
    const long long dbase = ::ucfd::tile_index(k, 0, B2);
#pragma unroll
    for (int e = 0; e < B2; ++e) D[dbase + (e << 5)] = dm[e];
    ludcmp_dev<double, B>(dm);
#pragma unroll
    for (int e = 0; e < B2; ++e) {
        if (LU64) LU64[dbase + (e << 5)] = dm[e];
        if (LU_s) LU_s[dbase + (e << 5)] = (S)dm[e];
    }
}

// c = D^-1 b for the fast build's sweeps (variables var0 .. var0 + B - 1 of
// every cell, through the factors LU with reciprocal pivots); c may be b.
template <typename S, int B>
__global__ void fs_blusgs_rhs_solve_kernel(long long N, int var0, const S *LU, const S *b, S *c) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= N) return;
    constexpr int B2 = B * B;
    S lu[B2], v[B];
    const S *LUk = LU + ::ucfd::tile_index(k, 0, B2);
#pragma unroll
    for (int e = 0; e < B2; ++e) lu[e] = LUk[e << 5];
#pragma unroll
    for (int r = 0; r < B; ++r) v[r] = b[(var0 + r) * N + k];
    lusub_dev<S, B, true>(lu, v);
#pragma unroll
    for (int r = 0; r < B; ++r) c[(var0 + r) * N + k] = v[r];
}

// ---- split sums of the fast build's sweeps (see SweepSplit in kargs.h) ----
template <typename S>
using SweepSplit = ::ucfd::SweepSplit<S>;

// Side of a face whose neighbour is g, for a cell of the level [lo, hi) in
// the level-major layout: 0 an earlier level, 1 a later level, 2 the cell
// itself.
__device__ __forceinline__ int split_side(int g, int lo, int hi) { return g < lo ? 0 : (g >= hi ? 1 : 2); }

// Whether a sweep uses the face at all: its own side always, the other side
// (and a face to the cell itself) in full mode only.  A mesh with faces to
// the cell itself always sweeps in full mode (the host sees to it): such a
// term changes with the cell's own increment, so it is never stored.
template <typename S>
__device__ __forceinline__ bool split_uses(const SweepSplit<S> &sp, int side) {
    return side == sp.upper || sp.full != 0;
}

// One face's product M x (M(r, c) its block) added to the sum of its side:
// ta the sweep's own side, to the other side (with the cell itself).  The
// entries go in row by row, columns in order, one fused multiply-add each.
template <typename S, int B, typename MF>
__device__ __forceinline__ void split_add(const SweepSplit<S> &sp, int side, const S *x, MF m, S *ta, S *to) {
    if (side == sp.upper) {
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
            for (int c = 0; c < B; ++c) ta[r] += m(r, c) * x[c];
    } else {
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
            for (int c = 0; c < B; ++c) to[r] += m(r, c) * x[c];
    }
}

// The other side's sum to start from: stored by the previous sweep in
// partial mode (issued early, with the cell's other inputs), zero in full
// mode.  In a dependent launch only after griddepcontrol.wait.
template <typename S, int B>
__device__ __forceinline__ void split_start(const SweepSplit<S> &sp, long long N, int var0, long long k, S *ta,
                                            S *to) {
#pragma unroll
    for (int r = 0; r < B; ++r) {
        ta[r] = S(0);
        to[r] = sp.full ? S(0) : sp.part[(var0 + r) * N + k];
    }
}

// b = c - S_lo - S_up in that order (S_lo the lower side's sum, S_up the
// upper side's; faces to the cell itself are in the other side's sum); the
// sweep's own side is written to part.
template <typename S, int B>
__device__ __forceinline__ void split_finish(const SweepSplit<S> &sp, long long N, int var0, long long k, S *b,
                                             const S *ta, const S *to) {
#pragma unroll
    for (int r = 0; r < B; ++r) {
        const S slo = sp.upper ? to[r] : ta[r];
        const S sup = sp.upper ? ta[r] : to[r];
        b[r] = (b[r] - slo) - sup;
    }
#pragma unroll
    for (int r = 0; r < B; ++r) sp.part[(var0 + r) * N + k] = ta[r];
}

// lower_sweep / upper_sweep of blusgs.c:273-373 for one level: every
// neighbour contributes with its current value (lower levels already
// updated, higher levels not yet), then the cell solves with its LU.
//
// PW > 0: the ELL width is the compile-time constant PW and the face loop
// is fully unrolled: every neighbour index, then every neighbour increment
// and block value, is requested before the first product, so one thread
// keeps all of its memory traffic in flight (the reference's per-face
// order of the products and subtractions is kept; padding entries only
// skip their contribution).  PW == 0 is the generic runtime-width loop.
//
// Everything but the neighbour increments du is read once per sweep (the
// J and LU tiles, rhs, nei, fa) and is loaded with the streaming
// (evict-first) policy, so that du, gathered at every neighbour, keeps L2.
//
// DEP (PW > 0 only): launched as a programmatic dependent of the previous
// sweep launch (one colour after the other).  The grid lets its own
// dependent start at once, then loads every input the previous launch
// does not write (rhs, rv, nei, fa) before it waits for that launch to
// complete (griddepcontrol.wait); the neighbour increments du are read
// after the wait.  This overlaps a launch's start with the previous
// launch's tail, which pays where levels are small.  Results are those of
// DEP == false.  (An L2 bulk prefetch of each warp's J and LU tiles in
// front of the wait measured slower at 2.1M cells: the early grids'
// prefetches evict the running grid's data.)
//
// Fast build (kFold): the face products are split by side (split_add /
// split_finish; SweepSplit in kargs.h).  In partial mode the faces of the
// other side are neither loaded nor multiplied.
template <typename S, int B, int PW, bool DEP = false>
__global__ void __launch_bounds__(256) fs_blusgs_sweep_kernel(int t0, int t1, long long N, int P,
                                                              int var0, const int *nei, const S *fa,
                                                              const S *rv, const S *J, const S *LU,
                                                              const S *rhs, S *du, SweepSplit<S> sp) {
    static_assert(!DEP || PW > 0, "the dependent-launch form is the unrolled one");
    if constexpr (DEP) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    // threads start at the tile boundary below t0, so every warp reads
    // whole tiles; the cells of the tile outside [t0, t1) do nothing
    const int k = (t0 & ~31) + blockIdx.x * blockDim.x + threadIdx.x;
    if (k < t0 || k >= t1) return;
    constexpr int B2 = B * B;
    const S *Jk = J + ::ucfd::tile_index(k, 0, (long long)P * B2);
    S b[B];
#pragma unroll
    for (int r = 0; r < B; ++r) b[r] = __ldcs(rhs + (var0 + r) * N + k);
    if constexpr (kFold) {
        S ta[B], to[B];
        if constexpr (!DEP) split_start<S, B>(sp, N, var0, k, ta, to);
        if constexpr (PW > 0) {
            // the faces the sweep uses, as bits (own: those of its own side)
            int nb[PW];
            unsigned use = 0u, own = 0u;
#pragma unroll
            for (int p = 0; p < PW; ++p) {
                nb[p] = __ldcs(nei + p * N + k);
                const int sd = nb[p] >= 0 ? split_side(nb[p], t0, t1) : -1;
                use |= (sd >= 0 && split_uses(sp, sd)) ? 1u << p : 0u;
                own |= (sd == sp.upper) ? 1u << p : 0u;
            }
            if constexpr (DEP) {
                asm volatile("griddepcontrol.wait;" ::: "memory");
                split_start<S, B>(sp, N, var0, k, ta, to);
            }
            // KB used faces at a time, in face order: the step's neighbour
            // increments are all requested before its products
            constexpr int KB = sizeof(S) == 8 ? 2 : 3;
#pragma unroll 1
            while (use) {
                int pk[KB];
                bool on[KB];
#pragma unroll
                for (int q = 0; q < KB; ++q) {
                    on[q] = use != 0u;
                    pk[q] = on[q] ? __ffs(use) - 1 : 0;
                    use &= on[q] ? use - 1u : use;
                }
                S x[KB][B];
#pragma unroll
                for (int q = 0; q < KB; ++q) {
                    if (!on[q]) continue;
                    int g = nb[0];
#pragma unroll
                    for (int p = 1; p < PW; ++p) g = pk[q] == p ? nb[p] : g;
#pragma unroll
                    for (int c = 0; c < B; ++c) x[q][c] = du[(var0 + c) * N + g];
                }
#pragma unroll
                for (int q = 0; q < KB; ++q) {
                    if (!on[q]) continue;
                    const S *Jp = Jk + ((long long)pk[q] * B2 << 5);
                    const int sd = (own >> pk[q]) & 1u ? sp.upper : 2;
                    split_add<S, B>(sp, sd, x[q], [&](int r, int c) { return __ldcs(Jp + ((r * B + c) << 5)); }, ta,
                                    to);
                }
            }
        } else {
            for (int p = 0; p < P; ++p) {
                const int g = __ldcs(nei + p * N + k);
                if (g < 0) break;
                const int sd = split_side(g, t0, t1);
                if (!split_uses(sp, sd)) continue;
                S x[B];
#pragma unroll
                for (int c = 0; c < B; ++c) x[c] = du[(var0 + c) * N + g];
                const S *Jp = Jk + ((long long)p * B2 << 5);
                split_add<S, B>(sp, sd, x, [&](int r, int c) { return __ldcs(Jp + ((r * B + c) << 5)); }, ta, to);
            }
        }
        split_finish<S, B>(sp, N, var0, k, b, ta, to);
#pragma unroll
        for (int r = 0; r < B; ++r) du[(var0 + r) * N + k] = b[r];
        return;
    }
    // exact build: the reference's per-face products (blusgs.c:298-314),
    // scaled by fv, then the LU solve of the diagonal block
    const S rvk = rv[k];
    if constexpr (PW > 0) {
        int nb[PW];
        S fv[PW];
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            nb[p] = __ldcs(nei + p * N + k);
            fv[p] = __ldcs(fa + p * N + k) * rvk;
        }
        if constexpr (DEP) asm volatile("griddepcontrol.wait;" ::: "memory");
        S x[PW][B];
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            const int g = nb[p] >= 0 ? nb[p] : k;  // padding: any valid address
#pragma unroll
            for (int c = 0; c < B; ++c) x[p][c] = du[(var0 + c) * N + g];
        }
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            const S *Jp = Jk + ((long long)p * B2 << 5);
            S jv[B2];
#pragma unroll
            for (int e = 0; e < B2; ++e) jv[e] = __ldcs(Jp + (e << 5));
            if (nb[p] >= 0) {
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    S val = S(0);
#pragma unroll
                    for (int c = 0; c < B; ++c) val += jv[r * B + c] * x[p][c];
                    b[r] -= val * fv[p];
                }
            }
        }
    } else {
        for (int p = 0; p < P; ++p) {
            const int nb = __ldcs(nei + p * N + k);
            if (nb < 0) break;
            const S fv = __ldcs(fa + p * N + k) * rvk;
            S x[B];
#pragma unroll
            for (int c = 0; c < B; ++c) x[c] = du[(var0 + c) * N + nb];
            const S *Jp = Jk + ((long long)p * B2 << 5);
#pragma unroll
            for (int r = 0; r < B; ++r) {
                S val = S(0);
#pragma unroll
                for (int c = 0; c < B; ++c) val += __ldcs(Jp + ((r * B + c) << 5)) * x[c];
                b[r] -= val * fv;
            }
        }
    }
    S lu[B2];
    const S *LUk = LU + ::ucfd::tile_index(k, 0, B2);
#pragma unroll
    for (int e = 0; e < B2; ++e) lu[e] = __ldcs(LUk + (e << 5));
    lusub_dev<S, B>(lu, b);
#pragma unroll
    for (int r = 0; r < B; ++r) du[(var0 + r) * N + k] = b[r];
}

// FP32 sweep of a small level (a colour of a few thousand cells), where a
// launch costs one thread's chain of dependent memory round trips rather
// than bandwidth.  Launched like the DEP form of fs_blusgs_sweep_kernel,
// but every input the previous launch does not write -- rhs, nei and the
// blocks of the faces the sweep uses -- is loaded into registers before
// griddepcontrol.wait, so after the wait only the neighbour increments
// (and, in partial mode, the other side's sums) are fetched.  The fast
// build's split sums, formed as fs_blusgs_sweep_kernel forms them.
template <int B, int PW>
__global__ void __launch_bounds__(128) fs_blusgs_sweep_small_kernel(int t0, int t1, long long N, int var0,
                                                                    const int *nei, const float *J,
                                                                    const float *rhs, float *du,
                                                                    SweepSplit<float> sp) {
    static_assert(kFold || B < 0, "the small-level kernel is the fast build's");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const int k = (t0 & ~31) + blockIdx.x * blockDim.x + threadIdx.x;
    if (k < t0 || k >= t1) return;
    constexpr int B2 = B * B;
    const float *Jk = J + ::ucfd::tile_index(k, 0, (long long)PW * B2);
    float b[B], jv[PW][B2];
    int nb[PW], side[PW];
#pragma unroll
    for (int r = 0; r < B; ++r) b[r] = __ldcs(rhs + (var0 + r) * N + k);
#pragma unroll
    for (int p = 0; p < PW; ++p) {
        nb[p] = __ldcs(nei + p * N + k);
        side[p] = nb[p] >= 0 ? split_side(nb[p], t0, t1) : -1;
        if (side[p] >= 0 && split_uses(sp, side[p])) {
#pragma unroll
            for (int e = 0; e < B2; ++e) jv[p][e] = __ldcs(Jk + ((p * B2 + e) << 5));
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    float ta[B], to[B];
    split_start<float, B>(sp, N, var0, k, ta, to);
    float x[PW][B];
#pragma unroll
    for (int p = 0; p < PW; ++p) {
        if (side[p] >= 0 && split_uses(sp, side[p])) {
#pragma unroll
            for (int c = 0; c < B; ++c) x[p][c] = du[(var0 + c) * N + nb[p]];
        }
    }
#pragma unroll
    for (int p = 0; p < PW; ++p) {
        if (side[p] >= 0 && split_uses(sp, side[p]))
            split_add<float, B>(sp, side[p], x[p], [&](int r, int c) { return jv[p][r * B + c]; }, ta, to);
    }
    split_finish<float, B>(sp, N, var0, k, b, ta, to);
#pragma unroll
    for (int r = 0; r < B; ++r) du[(var0 + r) * N + k] = b[r];
}

// FP32 block sweep with each tile's J and LU staged in shared memory by
// bulk asynchronous copies (cp.async.bulk, completed on an mbarrier).
// Every warp owns a ring of NST tile buffers and walks the level's tiles
// with a grid stride; one tile's J and LU (PW*B*B + B*B values for each of
// its 32 cells) are two contiguous blocks of the tiled layout, so each is
// one copy.  With NST == 2 the copy of the warp's next tile is in flight
// while it gathers the neighbour increments of the current tile and
// computes it; with NST == 1 twice as many warps fit, each with one
// buffer.  Per cell the arithmetic is that of fs_blusgs_sweep_kernel
// (same products and subtractions, same order); in the fast build the
// blocks are M = D^-1 J fv and the LU tile is not needed.  A copy that has
// not landed after max_spin polls sets *err; the warp then waits (bounded)
// for its other copy and returns.
template <int B, int PW, int NST>
__global__ void __launch_bounds__(NST == 2 ? 128 : 256)
    fs_blusgs_sweep_bulk_kernel(int t0, int t1, long long N, int var0, const int *__restrict__ nei,
                                const float *__restrict__ fa, const float *__restrict__ rv,
                                const float *__restrict__ J, const float *__restrict__ LU,
                                const float *__restrict__ rhs, float *du, int *err, long long max_spin,
                                SweepSplit<float> sp) {
    constexpr int B2 = B * B;
    constexpr int JT = PW * B2 * 32;  // floats of J in one tile
    constexpr int LT = kFold ? 0 : B2 * 32;  // floats of LU in one tile (the fast build's blocks need none)
    constexpr int ST = JT + LT;       // floats per buffer
    constexpr unsigned JBYTES = JT * 4, LBYTES = LT * 4;
    static_assert(JBYTES % 16 == 0 && LBYTES % 16 == 0, "bulk copies move multiples of 16 bytes");
    static_assert(JBYTES + LBYTES < (1u << 20), "mbarrier transaction count");
    extern __shared__ __align__(16) float smem_f[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    float *buf = smem_f + (size_t)warp * NST * ST;
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem_f + (size_t)nwarps * NST * ST) + NST * warp;
    const long long tile1 = ((long long)t1 + 31) >> 5;
    const long long step = (long long)gridDim.x * nwarps;
    long long t = (t0 >> 5) + (long long)blockIdx.x * nwarps + warp;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NST; ++q) ::ucfd::dev::mbar_init(&bar[q], 1);
        ::ucfd::dev::fence_mbar_init();
    }
    __syncwarp();
    // lane 0 starts the copies of tile tt into buffer q
    auto issue = [&](long long tt, int q) {
        if (lane == 0) {
            ::ucfd::dev::fence_proxy_async_smem();
            ::ucfd::dev::mbar_arrive_expect_tx(&bar[q], JBYTES + LBYTES);
            ::ucfd::dev::bulk_copy_g2s(buf + q * ST, J + tt * JT, JBYTES, &bar[q]);
            if constexpr (LBYTES > 0) ::ucfd::dev::bulk_copy_g2s(buf + q * ST + JT, LU + tt * LT, LBYTES, &bar[q]);
        }
    };
    if (t < tile1) issue(t, 0);
    for (unsigned it = 0; t < tile1; t += step, ++it) {
        const int q = NST == 2 ? (int)(it & 1) : 0;
        const unsigned parity = (NST == 2 ? (it >> 1) : it) & 1;
        const long long tn = t + step;
        if (NST == 2 && tn < tile1) issue(tn, q ^ 1);
        const long long k = (t << 5) + lane;
        const bool act = k >= t0 && k < t1;
        const long long kk = act ? k : t0;  // any valid cell for the idle lanes
        float b[B];
#pragma unroll
        for (int r = 0; r < B; ++r) b[r] = rhs[(var0 + r) * N + kk];
        const float rvk = kFold ? 1.f : rv[kk];
        int nb[PW], side[PW];
        float fv[PW];
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            nb[p] = act ? __ldg(nei + p * N + kk) : -1;
            side[p] = nb[p] >= 0 ? split_side(nb[p], t0, t1) : -1;
            if constexpr (!kFold) fv[p] = __ldg(fa + p * N + kk) * rvk;
        }
        float x[PW][B];
#pragma unroll
        for (int p = 0; p < PW; ++p) {
            const bool use = kFold ? side[p] >= 0 && split_uses(sp, side[p]) : nb[p] >= 0;
            const long long g = use ? nb[p] : kk;
#pragma unroll
            for (int c = 0; c < B; ++c) x[p][c] = use ? du[(var0 + c) * N + g] : 0.f;
        }
        const bool ok = __all_sync(0xffffffffu, ::ucfd::dev::mbar_wait_bounded(&bar[q], parity, max_spin));
        if (!ok) {
            if (lane == 0) atomicExch(err, 1);
            if (NST == 2 && tn < tile1)
                (void)::ucfd::dev::mbar_wait_bounded(&bar[q ^ 1], ((it + 1) >> 1) & 1, max_spin);
            (void)::ucfd::dev::mbar_wait_bounded(&bar[q], parity, max_spin);
            return;
        }
        const float *sJ = buf + q * ST + lane;
        if constexpr (kFold) {
            float ta[B], to[B];
            split_start<float, B>(sp, N, var0, kk, ta, to);
#pragma unroll
            for (int p = 0; p < PW; ++p) {
                if (side[p] >= 0 && split_uses(sp, side[p]))
                    split_add<float, B>(sp, side[p], x[p], [&](int r, int c) { return sJ[(p * B2 + r * B + c) << 5]; },
                                        ta, to);
            }
            if (act) split_finish<float, B>(sp, N, var0, k, b, ta, to);
        } else {
#pragma unroll
            for (int p = 0; p < PW; ++p) {
                if (nb[p] >= 0) {
#pragma unroll
                    for (int r = 0; r < B; ++r) {
                        float val = 0.f;
#pragma unroll
                        for (int c = 0; c < B; ++c) val += sJ[(p * B2 + r * B + c) << 5] * x[p][c];
                        b[r] -= val * fv[p];
                    }
                }
            }
            float lu[B2];
#pragma unroll
            for (int e = 0; e < B2; ++e) lu[e] = sJ[JT + (e << 5)];
            lusub_dev<float, B>(lu, b);
        }
        if (act) {
#pragma unroll
            for (int r = 0; r < B; ++r) du[(var0 + r) * N + k] = b[r];
        }
        __syncwarp();
        if (NST == 1 && tn < tile1) issue(tn, 0);
    }
}

// FP64 residual of the packed system: r = rhs - D x - sum_f J x_nb fv.
// fa == nullptr: J64 holds the FP64 fused multiply-add mode's sweep blocks
// M = D^-1 J fv, so r = rhs - D (x + sum_f M x_nb).
// Writes r (as R) when r_out != nullptr and accumulates per-block partial
// sums of r^2 and rhs^2 into part[2*blockIdx.x + {0,1}].
template <typename Sx, typename R, int B>
__global__ void fs_blusgs_residual_kernel(long long N, int P, int var0, int nvars, const int *nei,
                                          const double *fa, const double *rv, const double *J64,
                                          const double *D, const double *rhs64, const Sx *x,
                                          R *r_out, double *part) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double rr = 0.0, bb = 0.0;
    if (k < N) {
        constexpr int B2 = B * B;
        double res[B];
        double xk[B];
        // x == nullptr: x is known to be zero, r = rhs (no matrix reads)
#pragma unroll
        for (int c = 0; c < B; ++c) xk[c] = x ? (double)x[(var0 + c) * N + k] : 0.0;
        // M form: t = x + sum_f M x_nb, then r = rhs - D t (below)
        double t[B];
#pragma unroll
        for (int r = 0; r < B; ++r) {
            t[r] = xk[r];
            double v = rhs64[(var0 + r) * N + k];
            bb += v * v;
            if (x && fa) {
#pragma unroll
                for (int c = 0; c < B; ++c) v -= D[::ucfd::tile_index(k, r * B + c, B2)] * xk[c];
            }
            res[r] = v;
        }
        // fixed trip count (6 = hex ELL width) so all gathers are issued
        // up front; padding entries contribute nothing
        constexpr int PU = 6;
        for (int p0 = 0; x && p0 < P; p0 += PU) {
            int nbv[PU];
            double xn[PU][B];
#pragma unroll
            for (int q = 0; q < PU; ++q) {
                const int p = p0 + q;
                nbv[q] = p < P ? nei[p * N + k] : -1;
            }
#pragma unroll
            for (int q = 0; q < PU; ++q) {
                const int g = nbv[q] >= 0 ? nbv[q] : (int)k;
#pragma unroll
                for (int c = 0; c < B; ++c) xn[q][c] = (double)x[(var0 + c) * N + g];
            }
#pragma unroll
            for (int q = 0; q < PU; ++q) {
                if (nbv[q] < 0) continue;
                const int p = p0 + q;
                const double fv = fa ? fa[p * N + k] * rv[k] : 1.0;
#pragma unroll
                for (int r = 0; r < B; ++r) {
                    double val = 0.0;
#pragma unroll
                    for (int c = 0; c < B; ++c)
                        val += J64[::ucfd::tile_index(k, (long long)p * B2 + r * B + c, (long long)P * B2)] * xn[q][c];
                    if (fa) res[r] -= val * fv;
                    else t[r] += val;
                }
            }
        }
        if (x && !fa) {
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
                for (int c = 0; c < B; ++c) res[r] -= D[::ucfd::tile_index(k, r * B + c, B2)] * t[c];
        }
#pragma unroll
        for (int r = 0; r < B; ++r) {
            rr += res[r] * res[r];
            if (r_out) r_out[(var0 + r) * N + k] = (R)res[r];
        }
    }
    rr = block_sum(rr);
    bb = block_sum(bb);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = rr;
        part[2 * blockIdx.x + 1] = bb;
    }
}

// rank_sub_residual: blusgs.c:161-185 (per element, SoA internal state).
template <typename S>
__global__ void fs_blusgs_subres_kernel(int neles, int nvars, long long N, const int *cell_ids,
                                        const int *iperm, const double *vol, const S *du, S *dup,
                                        double *res) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) {
        const S diff = du[k + v * N] - dup[k + v * N];
        res[idx + (long long)v * neles] = (double)(diff * diff) * vol[idx];
        dup[k + v * N] = du[k + v * N];
    }
}

// rank_blusgs_update: blusgs.c:126-143.
template <typename S>
__global__ void fs_blusgs_update_kernel(int neles, int nvars, long long N, const int *cell_ids,
                                        const int *iperm, const S *du, double *upts) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) upts[idx + (long long)v * neles] += (double)du[k + v * N];
}

}  // namespace UCFD_KNS
