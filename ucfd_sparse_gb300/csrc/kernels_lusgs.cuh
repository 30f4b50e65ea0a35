// kernels_lusgs.cuh -- scalar (colored / level-scheduled) LU-SGS kernels.
//
// Included by kern_exact.cu (namespace kexact, built with -fmad=false: the
// FP64 arithmetic of every cell is the reference's, operation by
// operation) and kern_fast.cu (namespace kfast, FMA contraction on; FP64
// and FP32 instantiations).
//
// One thread per cell.  All per-cell arrays are [..][ld] with the cell
// index fastest, so a warp's loads of one face/variable are coalesced.
#pragma once

#include "kernels_common.cuh"
#include "kargs.h"

namespace UCFD_KNS {

// a / b.  FP32: one approximate reciprocal and a product (at most two ulp
// off, __fdividef); the FP32 sweeps are not bit-matched to the reference,
// and the division is a long instruction sequence in a kernel that is
// bound by its instruction issue.  FP64 keeps the correctly rounded
// division of the reference.
__device__ __forceinline__ float div_sweep(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double div_sweep(double a, double b) { return a / b; }

// ns_flux_container: flux.c:29-67.  The pressure floor rewrites the energy
// of the local copy u (flux.c:51-56), exactly as the reference does.  In
// FP32 the two divisions by rho are products with one reciprocal.
template <typename T, int NFV, int NDIMS>
__device__ __forceinline__ void ns_flux(T gamma, T pmin, T *u, const T *nf, T *f) {
    T rho = u[0];
    T et = u[NFV - 1];
    T temp = T(0), contrav = T(0);
#pragma unroll
    for (int i = 0; i < NDIMS; ++i) {
        contrav += u[i + 1] * nf[i];
        temp += u[i + 1] * u[i + 1];
    }
    T ke;  // 0.5 * temp / rho
    if constexpr (sizeof(T) == 4) {
        const T irho = div_sweep(T(1), rho);
        contrav *= irho;
        ke = T(0.5) * temp * irho;
    } else {
        contrav /= rho;
        ke = T(0.5) * temp / rho;
    }
    T p = (gamma - T(1)) * (et - ke);
    if (p < pmin) {
        p = pmin;
        et = p / (gamma - T(1)) + ke;
        u[NFV - 1] = et;
    }
    T ht = et + p;
    f[0] = rho * contrav;
#pragma unroll
    for (int i = 0; i < NDIMS; ++i) f[i + 1] = u[i + 1] * contrav + nf[i] * p;
    f[NFV - 1] = ht * contrav;
}

// rans_flux_container: flux.c:77-90
template <typename T, int NFV, int NDIMS, int NT>
__device__ __forceinline__ void rans_flux(const T *u, const T *nf, T *f) {
    T rho = u[0];
    T contrav = T(0);
#pragma unroll
    for (int i = 0; i < NDIMS; ++i) contrav += u[i + 1] * nf[i];
    contrav = div_sweep(contrav, rho);
#pragma unroll
    for (int i = 0; i < NT; ++i) f[i] = u[NFV + i] * contrav;
}

// F(u + dn; n) - F(u; n) of ns_flux in difference form, for FP32: the
// reference subtracts two whole fluxes (lusgs.c:143-155), which in single
// precision cancels most of the digits when |dn| << |u| (an increment of
// 1e-6 on a state of order 1 is below half an FP32 ulp of the energy).
// With c = m.n / rho, ke = |m|^2 / (2 rho), p = (gamma - 1)(E - ke) and the
// primed values at u + dn, the same difference is, exactly in real numbers,
//   dc  = (dm.n - c drho) / rho',  dke = (m.dm + |dm|^2 / 2 - ke drho) / rho',
//   dp  = (gamma - 1)(dE - dke),
//   dF0 = dm.n,  dFi = dm_i c' + m_i dc + n_i dp,  dF4 = (dE + dp) c' + (E + p) dc,
// each term formed from the increments themselves.  Where the pressure floor
// acts on either state (p or p' below pmin, flux.c:51-56) the two fluxes
// are subtracted as the reference does.
template <int NFV, int NDIMS>
__device__ __forceinline__ void ns_flux_diff(float gamma, float pmin, const float *u, const float *dn,
                                             const float *nf, float *dfl) {
    const float rho = u[0], drho = dn[0], rho1 = rho + drho;
    const float E = u[NFV - 1], dE = dn[NFV - 1];
    float mn = 0.f, dmn = 0.f, m2 = 0.f, mdm = 0.f, dm2 = 0.f;
#pragma unroll
    for (int i = 0; i < NDIMS; ++i) {
        const float m = u[i + 1], dm = dn[i + 1];
        mn += m * nf[i];
        dmn += dm * nf[i];
        m2 += m * m;
        mdm += m * dm;
        dm2 += dm * dm;
    }
    const float ir = __fdividef(1.f, rho), ir1 = __fdividef(1.f, rho1);
    const float c = mn * ir;
    const float dc = (dmn - c * drho) * ir1;
    const float c1 = c + dc;
    const float ke = 0.5f * m2 * ir;
    const float dke = (mdm + 0.5f * dm2 - ke * drho) * ir1;
    const float p = (gamma - 1.f) * (E - ke);
    const float dp = (gamma - 1.f) * (dE - dke);
    if (p < pmin || p + dp < pmin) {
        float uu[NFV], u1[NFV], f0[NFV], f1[NFV];
#pragma unroll
        for (int v = 0; v < NFV; ++v) {
            uu[v] = u[v];
            u1[v] = u[v] + dn[v];
        }
        ns_flux<float, NFV, NDIMS>(gamma, pmin, uu, nf, f0);
        ns_flux<float, NFV, NDIMS>(gamma, pmin, u1, nf, f1);
#pragma unroll
        for (int v = 0; v < NFV; ++v) dfl[v] = f1[v] - f0[v];
        return;
    }
    dfl[0] = dmn;
#pragma unroll
    for (int i = 0; i < NDIMS; ++i) dfl[i + 1] = dn[i + 1] * c1 + u[i + 1] * dc + nf[i] * dp;
    dfl[NFV - 1] = (dE + dp) * c1 + (E + p) * dc;
}

template <typename T>
using ScalarSweepArgs = ::ucfd::ScalarSweepArgs<T>;

// lower_sweep / upper_sweep of lusgs.c:157-257 for one level (or colour):
// every cell of the range is independent of the others.
template <typename T, int NV, int NFV, int NDIMS, bool RANS, bool COHERENT = false>
__device__ __forceinline__ void scalar_sweep_cell(const ScalarSweepArgs<T> &a, int t, int lo, int hi);

// Both systems of one level in one pass (the mean-flow variables with the
// spectral radius lam, the turbulence variables with tlam): the two sweeps
// are independent of each other, since each reads only the state u and its
// own increments, so this gives every value the separate sweeps give.
// FB: active faces gathered per step (fewer for the register-capped builds).
template <typename T, int NV, int NFV, int NDIMS, bool COHERENT = false, int FB = 3>
__device__ __forceinline__ void scalar_sweep_cell_both(const ScalarSweepArgs<T> &a, int t, int lo, int hi);

// MINB: minimum resident blocks of 256 threads per SM the compiler must
// allow (1: no register cap, about 106 registers; 3 / 4: at most 80 / 64
// registers, more warps to cover the gathers' latency for a few spilled
// bytes).  The autotuner picks.
template <typename T, int NV, int NFV, int NDIMS, bool RANS, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) scalar_sweep_kernel(ScalarSweepArgs<T> a) {
    const int t = a.t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.t1) return;
    scalar_sweep_cell<T, NV, NFV, NDIMS, RANS>(a, t, a.lo, a.hi);
}

// Grid-wide barrier for a cooperative launch (all blocks co-resident).
// Every wait is bounded: after max_spin polls the block records a timeout
// in *err and leaves the barrier; the kernel then stops at once.  Returns
// false after a timeout (also when another block reported one).
__device__ inline bool grid_barrier_bounded(unsigned *count, unsigned *gen, int *err, long long max_spin) {
    __shared__ int ok_sh;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        volatile unsigned *vgen = gen;
        const unsigned g = *vgen;
        __threadfence();
        const unsigned arrived = atomicAdd(count, 1u);
        if (arrived == gridDim.x - 1) {
            *count = 0u;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            long long spins = 0;
            while (*vgen == g) {
                if (*(volatile int *)err) {
                    ok = 0;
                    break;
                }
                if (++spins > max_spin) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        ok_sh = ok;
    }
    __syncthreads();
    return ok_sh != 0;
}

// One whole sweep (every level, ascending or descending) in one
// cooperative launch: the blocks stride over the cells of a level, then
// meet at the bounded grid barrier before the next level.
// BOTH: both systems per cell (scalar_sweep_cell_both).
template <typename T, int NV, int NFV, int NDIMS, bool RANS, int MINB = 1, bool BOTH = false>
__global__ void __launch_bounds__(256, MINB) scalar_sweep_persistent_kernel(ScalarSweepArgs<T> a, const int *lev_off,
                                                                      int nlev, unsigned *bar, int *err,
                                                                      long long max_spin) {
    // the level's bounds are passed on their own: a copy of the whole
    // argument struct per level would live in registers
    for (int q = 0; q < nlev; ++q) {
        const int l = a.upper ? nlev - 1 - q : q;
        const int t0 = lev_off[l], t1 = lev_off[l + 1];
        for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
            if constexpr (BOTH) scalar_sweep_cell_both<T, NV, NFV, NDIMS, true, (MINB >= 3 ? 2 : 3)>(a, t, t0, t1);
            else scalar_sweep_cell<T, NV, NFV, NDIMS, RANS, true>(a, t, t0, t1);
        }
        if (q + 1 < nlev && !grid_barrier_bounded(bar, bar + 1, err, max_spin)) return;
    }
}

// x * y rounded on its own (never fused into a following add), so that
// every sweep kernel forms the same per-face term whatever the compiler
// contracts; with contraction off this is the plain product.
__device__ __forceinline__ float mul_rn(float x, float y) { return __fmul_rn(x, y); }
__device__ __forceinline__ double mul_rn(double x, double y) { return __dmul_rn(x, y); }

// Active faces among the NB face slots f0 .. f0+NB-1 of a cell (neighbours
// nb[q], -1 for none): bit q is set when the neighbour of slot q belongs to
// this sweep (a lower colour / level for the lower sweep, a higher one for
// the upper sweep).
template <typename T, int NB>
__device__ __forceinline__ unsigned active_faces(const ScalarSweepArgs<T> &a, int lo, int hi, int ci,
                                                 const int *nb) {
    unsigned m = 0;
#pragma unroll
    for (int q = 0; q < NB; ++q) {
        bool act;
        if (a.lcolor) {
            const int cn = nb[q] >= 0 ? __ldg(a.lcolor + nb[q]) : ci;
            act = a.upper ? (cn > ci) : (cn < ci);
        } else {
            act = nb[q] >= 0 && (a.upper ? (nb[q] >= hi) : (nb[q] < lo));
        }
        m |= act ? (1u << q) : 0u;
    }
    return m;
}

// One active face's term ((F(u+dn) - F(u)) - kappa lam dn) * fvk of
// lusgs.c:143-205 (fvk = face area * rcp_vol), u the neighbour's state (only
// the variables the flux reads need be set; the pressure floor may rewrite
// u's energy), dn the neighbour's increment.  FP64 follows the reference's
// operations (du += u before either flux); FP32 forms the flux difference in
// difference form.  Every sweep kernel forms its terms here.
template <typename T, int NV, int NFV, int NDIMS, bool RANS>
__device__ __forceinline__ void face_term(const ScalarSweepArgs<T> &a, T *u, const T *dn, const T *nf, T fvk, T kl,
                                          T *term) {
    constexpr int NV0 = RANS ? NFV : 0;
    constexpr int DNV = RANS ? NV - NFV : NFV;
    T dfl[DNV];
    if constexpr (sizeof(T) == 4) {
        if constexpr (RANS) {
            // only the turbulence variables move: dF_j = dn_j * m.n / rho
            T mn = T(0);
#pragma unroll
            for (int d = 0; d < NDIMS; ++d) mn += u[d + 1] * nf[d];
            const T c = div_sweep(mn, u[0]);
#pragma unroll
            for (int j = 0; j < DNV; ++j) dfl[j] = dn[j] * c;
        } else {
            ns_flux_diff<NFV, NDIMS>(a.gamma, a.pmin, u, dn, nf, dfl);
        }
    } else {
        T du[NV], f0v[DNV], f1v[DNV];
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] = T(0);
#pragma unroll
        for (int j = 0; j < DNV; ++j) du[j + NV0] = dn[j];
        // diff_flux: lusgs.c:143-155 (du += u before either flux)
#pragma unroll
        for (int v = 0; v < NV; ++v) du[v] += u[v];
        if constexpr (RANS) {
            rans_flux<T, NFV, NDIMS, NV - NFV>(u, nf, f0v);
            rans_flux<T, NFV, NDIMS, NV - NFV>(du, nf, f1v);
        } else {
            ns_flux<T, NFV, NDIMS>(a.gamma, a.pmin, u, nf, f0v);
            ns_flux<T, NFV, NDIMS>(a.gamma, a.pmin, du, nf, f1v);
        }
#pragma unroll
        for (int j = 0; j < DNV; ++j) dfl[j] = f1v[j] - f0v[j];
    }
    const T klk = a.kappa * kl;
#pragma unroll
    for (int j = 0; j < DNV; ++j) term[j] = mul_rn(dfl[j] - klk * dn[j], fvk);
}

// Whether a flux of this kind reads state variable v of the neighbour.
template <typename T, int NV, int NFV, int NDIMS, bool RANS>
__device__ __forceinline__ constexpr bool flux_reads(int v) {
    return RANS ? (v <= NDIMS || (v >= NFV && sizeof(T) == 8)) : (v < NFV);
}

// Terms of the next (up to) KB active faces of a cell, taken from the mask
// m of its slots f0 + q (neighbours nb[q], NB slots) lowest slot first, so
// the k-th term is that of the k-th active face in face order; the faces
// taken are cleared from m and their number is returned.  Every lane of a
// warp works on its own k-th active face at step k, so a warp runs as many
// face steps as its busiest lane has active faces (not one per slot that
// any lane has active).  All gathers of the step's faces are issued before
// any flux is evaluated (latency hiding).  (The geometry stays on cached
// loads: at step k the lanes of a warp read different face rows of the same
// cells, which later steps find in L1; streaming loads measured slower.)
// Each face's term
// ((F(u+du) - F(u)) - kappa lam du) * area * rcp_vol (lusgs.c:143-205) is
// added to df in order (ACC) or stored in c[k] for the caller to add.
template <typename T, int NV, int NFV, int NDIMS, bool RANS, bool COHERENT, int NB, int KB, bool ACC>
__device__ __forceinline__ int face_terms(const ScalarSweepArgs<T> &a, int i, T rvi, int f0, const int *nb,
                                          unsigned &m, T (*c)[RANS ? NV - NFV : NFV], T *df) {
    constexpr int NV0 = RANS ? NFV : 0;
    constexpr int DNV = RANS ? NV - NFV : NFV;
    const long long ld = a.ld;
    bool on[KB];
    int fk[KB], gk[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        on[k] = m != 0u;
        const int q = on[k] ? __ffs(m) - 1 : 0;
        m &= m - 1u;
        int g = nb[0];
#pragma unroll
        for (int r = 1; r < NB; ++r) g = (q == r) ? nb[r] : g;
        fk[k] = f0 + q;
        gk[k] = g;
    }
    T uu[KB][NV], dn[KB][DNV], nf[KB][NDIMS], fv[KB], kl[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        if (!on[k]) continue;
        const int g = gk[k];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            // only the variables the flux reads are loaded
            uu[k][v] = flux_reads<T, NV, NFV, NDIMS, RANS>(v) ? __ldg(a.u + v * ld + g) : T(0);
        }
#pragma unroll
        for (int j = 0; j < DNV; ++j)
            dn[k][j] = COHERENT ? __ldcg(a.nbsrc + (j + NV0) * ld + g) : a.nbsrc[(j + NV0) * ld + g];
        const int f = fk[k];
#pragma unroll
        for (int d = 0; d < NDIMS; ++d) nf[k][d] = __ldg(a.nrm + (f * NDIMS + d) * ld + i);
        fv[k] = __ldg(a.fa + f * ld + i);
        kl[k] = __ldg(a.lam + f * ld + i);
    }
    int n = 0;
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        if (!on[k]) continue;
        ++n;
        const T fvk = a.rv ? fv[k] * rvi : fv[k];
        T term[DNV];
        face_term<T, NV, NFV, NDIMS, RANS>(a, uu[k], dn[k], nf[k], fvk, kl[k], term);
#pragma unroll
        for (int j = 0; j < DNV; ++j) {
            if constexpr (ACC) df[j] += term[j];
            else c[k][j] = term[j];
        }
    }
    return n;
}

// In the level-major layout the first level of a lower sweep and the last
// of an upper sweep have no active face at all.
template <typename T>
__device__ __forceinline__ bool no_active_face(const ScalarSweepArgs<T> &a, int lo, int hi) {
    return !a.lcolor && (a.upper ? hi >= a.ld : lo <= 0);
}

// The cell's new increment from its own input, diagonal and df.
template <typename T>
__device__ __forceinline__ T sweep_result(bool upper, T own, T df, T dg) {
    return !upper ? div_sweep(own - T(0.5) * df, dg) : own - div_sweep(T(0.5) * df, dg);
}

template <typename T, int NV, int NFV, int NDIMS, bool RANS, bool COHERENT>
__device__ __forceinline__ void scalar_sweep_cell(const ScalarSweepArgs<T> &a, int t, int lo, int hi) {
    constexpr int NV0 = RANS ? NFV : 0;
    constexpr int DNV = RANS ? NV - NFV : NFV;
    const long long ld = a.ld;
    const int i = a.cells ? __ldg(a.cells + t) : t;
    const int ci = a.lcolor ? __ldg(a.lcolor + i) : 0;

    // the cell's own inputs first (independent of every gather)
    T own[DNV], dg[DNV], df[DNV];
#pragma unroll
    for (int k = 0; k < DNV; ++k) {
        own[k] = a.own_in[(k + NV0) * ld + i];
        dg[k] = a.diag[(k + NV0) * a.diag_vs + i];
        df[k] = T(0);
    }
    const T rvi = a.rv ? __ldg(a.rv + i) : T(1);

    // Active faces three at a time (about 80 registers: occupancy for the
    // gathers' latency); the terms are added to df in the reference's face
    // order.
    constexpr int FB = 3;
    if (no_active_face(a, lo, hi)) {
    } else if (a.nface <= 2 * FB) {
        // every neighbour index of the cell up front, then its active faces
        int nba[2 * FB];
#pragma unroll
        for (int p = 0; p < 2 * FB; ++p) nba[p] = p < a.nface ? __ldg(a.nei + p * ld + i) : -1;
        unsigned m = active_faces<T, 2 * FB>(a, lo, hi, ci, nba);
        face_terms<T, NV, NFV, NDIMS, RANS, COHERENT, 2 * FB, FB, true>(a, i, rvi, 0, nba, m, nullptr, df);
        if (m) face_terms<T, NV, NFV, NDIMS, RANS, COHERENT, 2 * FB, FB, true>(a, i, rvi, 0, nba, m, nullptr, df);
    } else {
        for (int f0 = 0; f0 < a.nface; f0 += FB) {
            int nb[FB];
#pragma unroll
            for (int q = 0; q < FB; ++q) nb[q] = (f0 + q < a.nface) ? __ldg(a.nei + (f0 + q) * ld + i) : -1;
            unsigned m = active_faces<T, FB>(a, lo, hi, ci, nb);
            face_terms<T, NV, NFV, NDIMS, RANS, COHERENT, FB, FB, true>(a, i, rvi, f0, nb, m, nullptr, df);
        }
    }
#pragma unroll
    for (int k = 0; k < DNV; ++k) a.own_out[(k + NV0) * ld + i] = sweep_result(a.upper != 0, own[k], df[k], dg[k]);
}

// face_terms for both systems at once: each active face's neighbour index,
// normal, area and mean-flow state are loaded once and give the face's
// mean-flow term (spectral radius lam) and turbulence term (tlam), each
// added to its own sums in face order.  The terms are formed by face_term
// exactly as the single-system sweeps form them.  FP64 also loads the
// turbulence state, which its flux difference reads; in FP32 only the
// increments of the turbulence variables move.
template <typename T, int NV, int NFV, int NDIMS, bool COHERENT, int NB, int KB>
__device__ __forceinline__ void face_terms_both(const ScalarSweepArgs<T> &a, int i, T rvi, int f0, const int *nb,
                                                unsigned &m, T *df) {
    const long long ld = a.ld;
    bool on[KB];
    int fk[KB], gk[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        on[k] = m != 0u;
        const int q = on[k] ? __ffs(m) - 1 : 0;
        m &= m - 1u;
        int g = nb[0];
#pragma unroll
        for (int r = 1; r < NB; ++r) g = (q == r) ? nb[r] : g;
        fk[k] = f0 + q;
        gk[k] = g;
    }
    T uu[KB][NV], dn[KB][NV], nf[KB][NDIMS], fv[KB], kl[KB], klt[KB];
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        if (!on[k]) continue;
        const int g = gk[k];
#pragma unroll
        for (int v = 0; v < NV; ++v)
            uu[k][v] = (v < NFV || sizeof(T) == 8) ? __ldg(a.u + v * ld + g) : T(0);
#pragma unroll
        for (int j = 0; j < NV; ++j) dn[k][j] = COHERENT ? __ldcg(a.nbsrc + j * ld + g) : a.nbsrc[j * ld + g];
        const int f = fk[k];
        if constexpr (sizeof(T) == 4) {
            if (a.geo4) {
                // packed per cell-face: (normal, fa * rv) and (lam, tlam),
                // two vector loads instead of six
                const float4 gq = __ldg(static_cast<const float4 *>(a.geo4) + f * ld + i);
                const float2 l = __ldg(static_cast<const float2 *>(a.lam2) + f * ld + i);
                nf[k][0] = gq.x;
                if constexpr (NDIMS > 1) nf[k][1] = gq.y;
                if constexpr (NDIMS > 2) nf[k][2] = gq.z;
                fv[k] = gq.w;
                kl[k] = l.x;
                klt[k] = l.y;
                continue;
            }
        }
#pragma unroll
        for (int d = 0; d < NDIMS; ++d) nf[k][d] = __ldg(a.nrm + (f * NDIMS + d) * ld + i);
        fv[k] = __ldg(a.fa + f * ld + i);
        kl[k] = __ldg(a.lam + f * ld + i);
        klt[k] = __ldg(a.tlam + f * ld + i);
    }
#pragma unroll
    for (int k = 0; k < KB; ++k) {
        if (!on[k]) continue;
        // packed geometry holds the product fa * rv itself (the same rounding)
        const T fvk = a.rv && !a.geo4 ? fv[k] * rvi : fv[k];
        T tn[NFV], tt[NV - NFV];
        // the mean-flow flux may raise the energy of uu[k] to the pressure
        // floor (as its own sweep does to its copy); the turbulence flux
        // does not read the energy
        face_term<T, NV, NFV, NDIMS, false>(a, uu[k], dn[k], nf[k], fvk, kl[k], tn);
        face_term<T, NV, NFV, NDIMS, true>(a, uu[k], dn[k] + NFV, nf[k], fvk, klt[k], tt);
#pragma unroll
        for (int j = 0; j < NFV; ++j) df[j] += tn[j];
#pragma unroll
        for (int j = 0; j < NV - NFV; ++j) df[NFV + j] += tt[j];
    }
}

template <typename T, int NV, int NFV, int NDIMS, bool COHERENT, int FB>
__device__ __forceinline__ void scalar_sweep_cell_both(const ScalarSweepArgs<T> &a, int t, int lo, int hi) {
    const long long ld = a.ld;
    const int i = a.cells ? __ldg(a.cells + t) : t;
    const int ci = a.lcolor ? __ldg(a.lcolor + i) : 0;
    T own[NV], dg[NV], df[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        own[k] = a.own_in[k * ld + i];
        dg[k] = a.diag[k * a.diag_vs + i];
        df[k] = T(0);
    }
    const T rvi = a.rv && !a.geo4 ? __ldg(a.rv + i) : T(1);  // packed geometry carries fa * rv
    if (no_active_face(a, lo, hi)) {
    } else if (a.nface <= 2 * FB) {
        int nba[2 * FB];
#pragma unroll
        for (int p = 0; p < 2 * FB; ++p) nba[p] = p < a.nface ? __ldg(a.nei + p * ld + i) : -1;
        unsigned m = active_faces<T, 2 * FB>(a, lo, hi, ci, nba);
        face_terms_both<T, NV, NFV, NDIMS, COHERENT, 2 * FB, FB>(a, i, rvi, 0, nba, m, df);
        if (m) face_terms_both<T, NV, NFV, NDIMS, COHERENT, 2 * FB, FB>(a, i, rvi, 0, nba, m, df);
    } else {
        for (int f0 = 0; f0 < a.nface; f0 += FB) {
            int nb[FB];
#pragma unroll
            for (int q = 0; q < FB; ++q) nb[q] = (f0 + q < a.nface) ? __ldg(a.nei + (f0 + q) * ld + i) : -1;
            unsigned m = active_faces<T, FB>(a, lo, hi, ci, nb);
            face_terms_both<T, NV, NFV, NDIMS, COHERENT, FB, FB>(a, i, rvi, f0, nb, m, df);
        }
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) a.own_out[k * ld + i] = sweep_result(a.upper != 0, own[k], df[k], dg[k]);
}

// One level of both systems' sweeps, one thread per cell.  The builds
// capped at 80 / 64 registers gather two active faces per step (three
// otherwise), which keeps the 80-register build free of spills; the terms
// are added in face order either way.
template <typename T, int NV, int NFV, int NDIMS, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) scalar_sweep_both_kernel(ScalarSweepArgs<T> a) {
    const int t = a.t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.t1) return;
    scalar_sweep_cell_both<T, NV, NFV, NDIMS, false, (MINB >= 3 ? 2 : 3)>(a, t, a.lo, a.hi);
}

// One level of the sweep with one thread per active face.  A block owns
// a.cpb consecutive cells of the level; their active faces are consecutive
// entries of the face list.  Every thread forms the terms of the entries
// e0 + tid, e0 + tid + blockDim, ... (neighbour gathers and two flux
// evaluations each, all independent), parks them in shared memory, and
// after the barrier the first a.cpb threads add their cell's terms in face
// order and write the cell: the terms and their order are those of
// scalar_sweep_cell.  Each thread holds one face's data instead of a whole
// cell's, so many more warps fit to cover the gathers' latency, and no lane
// idles on a face that is active for a neighbouring cell only.
template <typename T, int NV, int NFV, int NDIMS, bool RANS>
__global__ void __launch_bounds__(256) scalar_sweep_faces_kernel(ScalarSweepArgs<T> a) {
    constexpr int NV0 = RANS ? NFV : 0;
    constexpr int DNV = RANS ? NV - NFV : NFV;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *terms = reinterpret_cast<T *>(smem_raw);
    const long long ld = a.ld;
    const int c0 = a.t0 + blockIdx.x * a.cpb;
    const int c1 = min(a.t1, c0 + a.cpb);
    const int e0 = __ldg(a.fl_off + c0), e1 = __ldg(a.fl_off + c1);
    const int k = c0 + (int)threadIdx.x;
    const bool owner = (int)threadIdx.x < a.cpb && k < c1;
    T own[DNV], dg[DNV];
    int f0 = 0, f1 = 0;
    if (owner) {
#pragma unroll
        for (int j = 0; j < DNV; ++j) {
            own[j] = a.own_in[(j + NV0) * ld + k];
            dg[j] = a.diag[(j + NV0) * a.diag_vs + k];
        }
        f0 = __ldg(a.fl_off + k);
        f1 = __ldg(a.fl_off + k + 1);
    }
    for (int e = e0 + (int)threadIdx.x; e < e1; e += blockDim.x) {
        const int g = __ldcs(a.fl_nb + e);
        T geo[4];
        if constexpr (sizeof(T) == 4) {
            const float4 v = __ldcs(reinterpret_cast<const float4 *>(a.fl_geo) + e);
            geo[0] = v.x, geo[1] = v.y, geo[2] = v.z, geo[3] = v.w;
        } else {
            const double2 v0 = __ldcs(reinterpret_cast<const double2 *>(a.fl_geo) + 2 * (long long)e);
            const double2 v1 = __ldcs(reinterpret_cast<const double2 *>(a.fl_geo) + 2 * (long long)e + 1);
            geo[0] = v0.x, geo[1] = v0.y, geo[2] = v1.x, geo[3] = v1.y;
        }
        const T kl = __ldg(a.lam + __ldcs(a.fl_q + e));
        T u[NV], dn[DNV];
#pragma unroll
        for (int v = 0; v < NV; ++v) u[v] = flux_reads<T, NV, NFV, NDIMS, RANS>(v) ? __ldg(a.u + v * ld + g) : T(0);
#pragma unroll
        for (int j = 0; j < DNV; ++j) dn[j] = a.nbsrc[(j + NV0) * ld + g];
        T term[DNV];
        face_term<T, NV, NFV, NDIMS, RANS>(a, u, dn, geo, geo[3], kl, term);
#pragma unroll
        for (int j = 0; j < DNV; ++j) terms[(e - e0) * DNV + j] = term[j];
    }
    __syncthreads();
    if (!owner) return;
    T df[DNV];
#pragma unroll
    for (int j = 0; j < DNV; ++j) df[j] = T(0);
    for (int e = f0; e < f1; ++e)
#pragma unroll
        for (int j = 0; j < DNV; ++j) df[j] += terms[(e - e0) * DNV + j];
#pragma unroll
    for (int j = 0; j < DNV; ++j) a.own_out[(j + NV0) * ld + k] = sweep_result(a.upper != 0, own[j], df[j], dg[j]);
}

// Face list geometry: per entry the outward normal of its ELL slot q
// (nrm [nface][ndims][ld], zero-padded to 3 components) and fa * rv, the
// same product the per-cell kernels form.
template <typename T>
__global__ void face_list_geo_kernel(long long E, long long ld, int ndims, const int *q, const T *nrm, const T *fa,
                                     const T *rv, T *geo) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < E;
         e += (long long)gridDim.x * blockDim.x) {
        const long long qq = q[e];
        const long long p = qq / ld, k = qq - p * ld;
        for (int d = 0; d < 3; ++d) geo[4 * e + d] = d < ndims ? nrm[(p * ndims + d) * ld + k] : T(0);
        geo[4 * e + 3] = rv ? fa[qq] * rv[k] : fa[qq];
    }
}

// Packed geometry of the FP32 run loop with both systems, per cell-face
// (p, k): (outward normal, zero-padded to 3 components; fa * rv).
__global__ void pack_geo4_kernel(long long N, int P, int ndims, const float *nrm, const float *fa, const float *rv,
                                 float4 *geo4) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)P * N;
         e += (long long)gridDim.x * blockDim.x) {
        const long long p = e / N, k = e - p * N;
        float4 g;
        g.x = nrm[(p * ndims + 0) * N + k];
        g.y = ndims > 1 ? nrm[(p * ndims + 1) * N + k] : 0.f;
        g.z = ndims > 2 ? nrm[(p * ndims + 2) * N + k] : 0.f;
        g.w = rv ? fa[e] * rv[k] : fa[e];
        geo4[e] = g;
    }
}

// (lam, tlam) per cell-face for the same loop.
__global__ void pack_lam2_kernel(long long n, const float *lam, const float *tlam, float2 *lam2) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        lam2[e] = make_float2(lam[e], tlam[e]);
}

// Two threads per cell (ELL width <= 6, level-major or coloured): the even
// lane takes faces 0-2, the odd lane faces 3-5, each with its gathers and
// fluxes; the odd lane hands its three terms to the even lane (warp
// shuffles), which adds all six in face order and writes the cell.  Half
// the dependent memory chain per thread and twice the threads in flight.
// Same terms, same order as scalar_sweep_cell.
template <typename T, int NV, int NFV, int NDIMS, bool RANS, int MINB = 1>
__global__ void __launch_bounds__(256, MINB) scalar_sweep_pair_kernel(ScalarSweepArgs<T> a) {
    constexpr int NV0 = RANS ? NFV : 0;
    constexpr int DNV = RANS ? NV - NFV : NFV;
    constexpr int FB = 3;
    const long long ld = a.ld;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int h = (int)(tid & 1);
    const long long t = a.t0 + (tid >> 1);
    const bool live = t < a.t1;  // both lanes of a pair agree
    const int i = live ? (a.cells ? __ldg(a.cells + t) : (int)t) : 0;
    const int ci = live && a.lcolor ? __ldg(a.lcolor + i) : 0;
    T own[DNV], dg[DNV];
    if (live && h == 0) {
#pragma unroll
        for (int k = 0; k < DNV; ++k) {
            own[k] = a.own_in[(k + NV0) * ld + i];
            dg[k] = a.diag[(k + NV0) * a.diag_vs + i];
        }
    }
    int n = 0;  // active faces of this lane, terms in c[0 .. n-1] in face order
    T c[FB][DNV];
    if (live && !no_active_face(a, a.lo, a.hi)) {
        const T rvi = a.rv ? __ldg(a.rv + i) : T(1);
        int nb[FB];
#pragma unroll
        for (int q = 0; q < FB; ++q) {
            const int p = h * FB + q;
            nb[q] = p < a.nface ? __ldg(a.nei + p * ld + i) : -1;
        }
        unsigned m = active_faces<T, FB>(a, a.lo, a.hi, ci, nb);
        n = face_terms<T, NV, NFV, NDIMS, RANS, false, FB, FB, false>(a, i, rvi, h * FB, nb, m, c, nullptr);
    }
    // the odd lane's terms to the even lane
    const int n_hi = __shfl_down_sync(0xffffffffu, n, 1);
    T chi[FB][DNV];
#pragma unroll
    for (int q = 0; q < FB; ++q)
#pragma unroll
        for (int k = 0; k < DNV; ++k) chi[q][k] = __shfl_down_sync(0xffffffffu, q < n ? c[q][k] : T(0), 1);
    if (!live || h != 0) return;
    T df[DNV];
#pragma unroll
    for (int k = 0; k < DNV; ++k) df[k] = T(0);
#pragma unroll
    for (int q = 0; q < FB; ++q)
        if (q < n)
#pragma unroll
            for (int k = 0; k < DNV; ++k) df[k] += c[q][k];
#pragma unroll
    for (int q = 0; q < FB; ++q)
        if (q < n_hi)
#pragma unroll
            for (int k = 0; k < DNV; ++k) df[k] += chi[q][k];
#pragma unroll
    for (int k = 0; k < DNV; ++k) a.own_out[(k + NV0) * ld + i] = sweep_result(a.upper != 0, own[k], df[k], dg[k]);
}

// {serial,parallel}_pre_lusgs (array layout): lusgs.c:8-37 + 87-113 with
// kappa = 1, a0 = dsrc = 0, rcp_vol = 1.
template <typename T>
__global__ void legacy_pre_kernel(int neles, int nface, T factor, const T *fnorm_vol, const T *dt,
                                  T *diag, const T *fspr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= neles) return;
    T sd = T(0);
    for (int f = 0; f < nface; ++f) {
        const T lamf = fspr[(long long)f * neles + i];
        sd += T(0.5) * lamf * fnorm_vol[(long long)f * neles + i];
    }
    diag[i] = T(1) / (dt[i] * factor) + sd;
}

template <typename T>
__global__ void legacy_update_kernel(int neles, int k0, int k1, T *upts, const T *rhs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= neles) return;
    for (int k = k0; k < k1; ++k) upts[(long long)k * neles + i] += rhs[(long long)k * neles + i];
}

// ---- FlowSys scalar LU-SGS on the level-major internal layout ---------------

// lusgs_pack: lusgs.c:8-37.  Element idx -> internal cell pos[cell_ids[idx]].
template <typename T>
__global__ void fs_lusgs_pack_kernel(int neles, int nvars, int nfvars, long long N,
                                     double turb_factor, double a0, const int *cell_ids,
                                     const int *iperm, const double *upts, const double *rhs,
                                     const double *dt, const double *dsrc, T *u, T *du, T *diag) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) {
        const long long e = idx + (long long)v * neles;
        const double factor = v < nfvars ? 1.0 : turb_factor;
        u[k + v * N] = (T)upts[e];
        du[k + v * N] = (T)rhs[e];
        diag[k + v * N] = (T)(1.0 / (dt[idx] * factor) + a0 + dsrc[e]);
    }
}

// rank_lusgs_update: lusgs.c:54-70 (uptsb += du over all nvars).  With
// assign != 0 the element state is overwritten by src instead (writing the
// device-resident state of a pseudo-time loop back).
template <typename T>
__global__ void fs_lusgs_update_kernel(int neles, int nvars, long long N, const int *cell_ids,
                                       const int *iperm, const T *src, double *upts, int assign) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= neles) return;
    const long long k = iperm[cell_ids[idx]];
    for (int v = 0; v < nvars; ++v) {
        if (assign) upts[idx + (long long)v * neles] = (double)src[k + v * N];
        else upts[idx + (long long)v * neles] += (double)src[k + v * N];
    }
}

// pre_lusgs's sum over a cell's faces (lusgs.c:87-113): slots p in order,
// up to the first padding slot, of 0.5 * (lam * kappa) * fa * rv, for one
// spectral radius (sd) or two (sd from lam, st from tlam).  Rows of up to 8
// slots issue every load before the first sum (one round trip instead of
// one per face, the same sums in the same order); wider rows loop.
template <typename T, bool TWO>
__device__ __forceinline__ void prepare_sums(long long N, int maxdeg, long long k, T kappa, const int *nei,
                                             const T *fa, const T *rv, const T *lam, const T *tlam, T &sd,
                                             T &st) {
    sd = T(0);
    st = T(0);
    const T r = rv[k];
    constexpr int PM = 8;
    if (maxdeg <= PM) {
        int nb[PM];
        T f[PM], l[PM], lt[PM];
#pragma unroll
        for (int p = 0; p < PM; ++p) {
            const bool in = p < maxdeg;
            nb[p] = in ? nei[p * N + k] : -1;
            f[p] = in ? fa[p * N + k] : T(0);
            l[p] = in ? lam[p * N + k] : T(0);
            if constexpr (TWO) lt[p] = in ? tlam[p * N + k] : T(0);
        }
        bool live = true;
#pragma unroll
        for (int p = 0; p < PM; ++p) {
            live = live && nb[p] >= 0;
            if (live) {
                const T lamf = l[p] * kappa;
                sd += T(0.5) * lamf * f[p] * r;
                if constexpr (TWO) {
                    const T lamt = lt[p] * kappa;
                    st += T(0.5) * lamt * f[p] * r;
                }
            }
        }
        return;
    }
    for (int p = 0; p < maxdeg; ++p) {
        if (nei[p * N + k] < 0) break;
        const T f = fa[p * N + k];
        const T lamf = lam[p * N + k] * kappa;
        sd += T(0.5) * lamf * f * r;
        if constexpr (TWO) {
            const T lamt = tlam[p * N + k] * kappa;
            st += T(0.5) * lamt * f * r;
        }
    }
}

// pre_lusgs: lusgs.c:87-113.  lam is the per cell-face copy of lambdaf.
// With base != nullptr the result is base + sd (a pseudo-time loop
// re-preparing from the packed diagonal), otherwise diag += sd.
template <typename T>
__global__ void fs_lusgs_prepare_kernel(long long N, int maxdeg, int nv0, int nv1, T kappa,
                                        const int *nei, const T *fa, const T *rv, const T *lam,
                                        const T *base, T *diag) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= N) return;
    T sd, st;
    prepare_sums<T, false>(N, maxdeg, k, kappa, nei, fa, rv, lam, nullptr, sd, st);
    if (base)
        for (int v = nv0; v < nv1; ++v) diag[k + v * N] = base[k + v * N] + sd;
    else
        for (int v = nv0; v < nv1; ++v) diag[k + v * N] += sd;
}

// pre_lusgs of both systems in one pass over the faces: the mean-flow
// variables [0, nfv) from lam, the turbulence variables [nfv, nv) from
// tlam, each sum formed as fs_lusgs_prepare_kernel forms it;
// diag = base + sum, or diag += sum without base.
template <typename T>
__global__ void fs_lusgs_prepare_both_kernel(long long N, int maxdeg, int nfv, int nv, T kappa, const int *nei,
                                             const T *fa, const T *rv, const T *lam, const T *tlam, const T *base,
                                             T *diag) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= N) return;
    T sd, st;
    prepare_sums<T, true>(N, maxdeg, k, kappa, nei, fa, rv, lam, tlam, sd, st);
    if (base)
        for (int v = 0; v < nv; ++v) diag[k + v * N] = base[k + v * N] + (v < nfv ? sd : st);
    else
        for (int v = 0; v < nv; ++v) diag[k + v * N] += v < nfv ? sd : st;
}

// dst[i] = src[idx[i]] (0 where idx[i] < 0): per cell-face copies of
// face-indexed arrays.
template <typename Td>
__global__ void gather_idx_kernel(long long n, const int *idx, const double *src, Td *dst) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int j = idx[i];
        dst[i] = j >= 0 ? (Td)src[j] : Td(0);
    }
}

}  // namespace UCFD_KNS
