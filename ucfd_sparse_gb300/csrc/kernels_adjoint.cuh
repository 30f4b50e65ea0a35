// kernels_adjoint.cuh -- reverse-mode derivative of one colored LU-SGS step
// (array layout), as transposed sweeps.
//
// Forward (lusgs.c:87-257 on the colour-renumbered mesh):
//   D_i    = 1/(dt_i f) + 1/2 sum_f lam_fi s_fi
//   lower  dQ*_i = (R_i - 1/2 sum_{f in L(i)} G_fi(dQ*_j)) / D_i
//   upper  dQ_i  = dQ*_i - 1/2 D_i^-1 sum_{f in U(i)} G_fi(dQ_j)
//   G_fi(d) = [F(u_j + d; n_fi) - F(u_j; n_fi) - lam_fi d] s_fi
// Reverse: first the upper sweep transposed (colours ascending), then the
// lower sweep transposed (colours descending), then the diagonal.  Each
// thread owns one cell and *pulls* the contributions of the neighbours
// that used it (through the reverse-face map rface), so no atomics are
// needed and every output element has one writer.
#pragma once

#include "kernels_common.cuh"
#include "kargs.h"

namespace UCFD_KNS {

// out = J^T v, J = dF(w; n)/dw of the Euler flux (flux.c:29-67), including
// the branch where the pressure floor replaces the energy.
template <typename T, int NFV, int NDIMS>
__device__ __forceinline__ void ns_flux_jt(T gamma, T pmin, const T *w, const T *n, const T *v, T *out) {
    const T rho = w[0];
    const T E = w[NFV - 1];
    T th = T(0), q = T(0);
#pragma unroll
    for (int d = 0; d < NDIMS; ++d) {
        th += w[d + 1] * n[d];
        q += w[d + 1] * w[d + 1];
    }
    const T ir = T(1) / rho;
    const T c = th * ir;
    const T gm1 = gamma - T(1);
    T p = gm1 * (E - T(0.5) * q * ir);
    const bool clamp = p < pmin;
    T Ee = E;
    if (clamp) {
        p = pmin;
        Ee = p / gm1 + T(0.5) * q * ir;
    }
    // partial derivatives of c, p, Ee
    const T dc_dr = -th * ir * ir;
    T dp_dr = clamp ? T(0) : gm1 * T(0.5) * q * ir * ir;
    T dp_dE = clamp ? T(0) : gm1;
    const T dEe_dr = clamp ? -T(0.5) * q * ir * ir : T(0);
    const T dEe_dE = clamp ? T(0) : T(1);
    const T H = Ee + p;
    const T vL = v[NFV - 1];
    // rho column
    T o0 = T(0);
#pragma unroll
    for (int a = 0; a < NDIMS; ++a) o0 += (w[a + 1] * dc_dr + n[a] * dp_dr) * v[a + 1];
    o0 += ((dEe_dr + dp_dr) * c + H * dc_dr) * vL;
    out[0] = o0;
    // momentum columns
#pragma unroll
    for (int d = 0; d < NDIMS; ++d) {
        const T dp_dm = clamp ? T(0) : -gm1 * w[d + 1] * ir;
        const T dEe_dm = clamp ? w[d + 1] * ir : T(0);
        T o = n[d] * v[0];
#pragma unroll
        for (int a = 0; a < NDIMS; ++a) {
            T jad = w[a + 1] * n[d] * ir + n[a] * dp_dm;
            if (a == d) jad += c;
            o += jad * v[a + 1];
        }
        o += ((dEe_dm + dp_dm) * c + H * n[d] * ir) * vL;
        out[d + 1] = o;
    }
    // energy column
    T oE = T(0);
#pragma unroll
    for (int a = 0; a < NDIMS; ++a) oE += n[a] * dp_dE * v[a + 1];
    oE += ((dEe_dE + dp_dE) * c) * vL;
    out[NFV - 1] = oE;
}

using AdjArgs = ::ucfd::AdjArgs;

// Transposed upper sweep for one colour.  qbar = adjoint of dQ (final for
// this cell once its lower-coloured neighbours are done), dbar = adjoint of
// D (upper part), gfspr initialised for every face of the cell.
template <typename T, int NV, int NFV, int NDIMS>
__global__ void adj_upper_kernel(AdjArgs a, T gamma, T pmin, const T *fnv, const T *vec, const T *fspr,
                                 const T *upts, const T *diag, const T *dub, const T *dq, const T *gdq, T *qbar,
                                 T *dbar, T *gfspr) {
    const int t = a.t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.t1) return;
    const long long N = a.neles;
    const int i = a.icolor[t];
    const int ci = a.lcolor[i];
    T qb[NFV], st[NFV];
#pragma unroll
    for (int v = 0; v < NFV; ++v) {
        qb[v] = gdq[v * N + i];
        st[v] = upts[v * N + i] + dq[v * N + i];  // state u_i + dQ_i
    }
    for (int f = 0; f < a.nface; ++f) {
        const int k = a.nei[f * N + i];
        if (k == i || a.lcolor[k] >= ci) continue;
        // i is the upper neighbour of k through k's face fp
        const int fp = a.rface[f * N + i];
        const T s = fnv[fp * N + k], lam = fspr[fp * N + k], Dk = diag[k];
        T n[NDIMS], w[NFV], y[NFV];
#pragma unroll
        for (int d = 0; d < NDIMS; ++d) n[d] = vec[(fp * NDIMS + d) * N + k];
#pragma unroll
        for (int v = 0; v < NFV; ++v) w[v] = qbar[v * N + k];
        ns_flux_jt<T, NFV, NDIMS>(gamma, pmin, st, n, w, y);
        const T sc = -T(0.5) * s / Dk;
#pragma unroll
        for (int v = 0; v < NFV; ++v) qb[v] += sc * (y[v] - lam * w[v]);
    }
    const T Di = diag[i];
    T db = T(0);
#pragma unroll
    for (int v = 0; v < NFV; ++v) {
        qbar[v * N + i] = qb[v];
        db += qb[v] * (-(dq[v * N + i] - dub[v * N + i]) / Di);
    }
    dbar[i] = db;
    for (int f = 0; f < a.nface; ++f) {
        const int j = a.nei[f * N + i];
        T g = T(0);
        if (j != i && a.lcolor[j] > ci) {
            T dot = T(0);
#pragma unroll
            for (int v = 0; v < NFV; ++v) dot += dq[v * N + j] * qb[v];
            g = T(0.5) * fnv[f * N + i] / Di * dot;
        }
        gfspr[f * N + i] = g;
    }
}

// Transposed lower sweep for one colour, then the diagonal: grhs, gdt and
// the rest of gfspr.  wbuf = qstar / D of cells already processed.
template <typename T, int NV, int NFV, int NDIMS>
__global__ void adj_lower_kernel(AdjArgs a, T gamma, T pmin, T factor, const T *fnv, const T *vec, const T *fspr,
                                 const T *dt, const T *upts, const T *diag, const T *dub, const T *qbar, T *wbuf,
                                 const T *dbar, T *grhs, T *gdt, T *gfspr) {
    const int t = a.t0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= a.t1) return;
    const long long N = a.neles;
    const int i = a.icolor[t];
    const int ci = a.lcolor[i];
    T qs[NFV], st[NFV];
#pragma unroll
    for (int v = 0; v < NFV; ++v) {
        qs[v] = qbar[v * N + i];
        st[v] = upts[v * N + i] + dub[v * N + i];  // state u_i + dQ*_i
    }
    for (int f = 0; f < a.nface; ++f) {
        const int k = a.nei[f * N + i];
        if (k == i || a.lcolor[k] <= ci) continue;
        // i is a lower neighbour of k through k's face fp
        const int fp = a.rface[f * N + i];
        const T s = fnv[fp * N + k], lam = fspr[fp * N + k];
        T n[NDIMS], w[NFV], y[NFV];
#pragma unroll
        for (int d = 0; d < NDIMS; ++d) n[d] = vec[(fp * NDIMS + d) * N + k];
#pragma unroll
        for (int v = 0; v < NFV; ++v) w[v] = wbuf[v * N + k];
        ns_flux_jt<T, NFV, NDIMS>(gamma, pmin, st, n, w, y);
        const T sc = -T(0.5) * s;
#pragma unroll
        for (int v = 0; v < NFV; ++v) qs[v] += sc * (y[v] - lam * w[v]);
    }
    const T Di = diag[i];
    T wi[NFV];
    T db = dbar[i];
#pragma unroll
    for (int v = 0; v < NFV; ++v) {
        wi[v] = qs[v] / Di;
        wbuf[v * N + i] = wi[v];
        grhs[v * N + i] = wi[v];
        db -= wi[v] * dub[v * N + i];
    }
    // D_i = 1/(dt_i f) + 1/2 sum_f lam_fi s_fi
    const T dti = dt[i];
    gdt[i] = -db / (dti * dti * factor);
    for (int f = 0; f < a.nface; ++f) {
        const int j = a.nei[f * N + i];
        const T s = fnv[f * N + i];
        T g = gfspr[f * N + i] + T(0.5) * s * db;
        if (j != i && a.lcolor[j] < ci) {
            T dot = T(0);
#pragma unroll
            for (int v = 0; v < NFV; ++v) dot += dub[v * N + j] * wi[v];
            g += T(0.5) * s * dot;
        }
        gfspr[f * N + i] = g;
    }
}

}  // namespace UCFD_KNS
