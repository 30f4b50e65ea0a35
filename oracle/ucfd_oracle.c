/*
 * ucfd_oracle.c -- CPU restatement of the reference's LU-SGS / BLU-SGS /
 * Krylov hot path.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke
 * check and the bench's CPU-baseline leg call it as the checker; the product
 * library (libucfd_gb300.so) never links or calls it.
 *
 * Every function restates one reference routine and keeps its arithmetic
 * order (loop order, association of each product and sum) so that, built
 * with -ffp-contract=off, its results are bit-identical to the reference's
 * own compiled sources on the same inputs.  That identity is checked by
 * tests/test_oracle_pin.py against oracle/_ref (where the reference source
 * is present) and against the committed golden vectors in tests/golden/.
 *
 * Citations are path:line inside the reference project (UCFD_SPARSE).
 * Types: ints are int32 (UCFDInt), reals are double (UCFDReal), as in the
 * reference's default configuration (src/krylov/include/config.h:15-28).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define OR_PARFOR _Pragma("omp parallel for schedule(static)")
#else
#define OR_PARFOR
#endif

typedef int32_t oint;
typedef double oreal;

/* Physical constants: src/lusgs/flux.h:18-26 (double build). */
static oreal g_gamma = 1.4;
static oreal g_pmin = 1e-13;

void oracle_set_constants(double gamma, double pmin)
{
    g_gamma = gamma;
    g_pmin = pmin;
}

/* ------------------------------------------------------------------------
 * Flux containers: src/lusgs/flux.c:29-67 (Euler/NS, with the pressure
 * floor that rewrites the energy of the *local copy* u) and 77-90 (RANS).
 * ---------------------------------------------------------------------- */
static void or_ns_flux(oint nfvars, oint ndims, oreal *u, const oreal *nf, oreal *f)
{
    oreal rho = u[0];
    oreal et = u[nfvars - 1];
    oreal temp = 0.0, contrav = 0.0;
    for (oint i = 0; i < ndims; ++i) {
        contrav += u[i + 1] * nf[i];
        temp += u[i + 1] * u[i + 1];
    }
    contrav /= rho;
    oreal p = (g_gamma - 1.0) * (et - 0.5 * temp / rho);
    if (p < g_pmin) {
        p = g_pmin;
        et = p / (g_gamma - 1.0) + 0.5 * temp / rho;
        u[nfvars - 1] = et;
    }
    oreal ht = et + p;
    f[0] = rho * contrav;
    for (oint i = 0; i < ndims; ++i) f[i + 1] = u[i + 1] * contrav + nf[i] * p;
    f[nfvars - 1] = ht * contrav;
}

static void or_rans_flux(oint nfvars, oint nturbvars, oint ndims, oreal *u, const oreal *nf, oreal *f)
{
    oreal rho = u[0];
    oreal contrav = 0.0;
    for (oint i = 0; i < ndims; ++i) contrav += u[i + 1] * nf[i];
    contrav /= rho;
    for (oint i = 0; i < nturbvars; ++i) f[i] = u[nfvars + i] * contrav;
}

/* diff_flux: src/lusgs/lusgs.c:143-155.  du += u first, then F(u), F(u+du). */
static void or_diff_flux(oint nvars, oint nfvars, oint ndims, oint dnv, int rans,
                         oreal *u, oreal *du, oreal *df, const oreal *nf)
{
    oreal f[16];
    for (oint i = 0; i < nvars; ++i) du[i] += u[i];
    if (rans) {
        or_rans_flux(nfvars, nvars - nfvars, ndims, u, nf, f);
        or_rans_flux(nfvars, nvars - nfvars, ndims, du, nf, df);
    } else {
        or_ns_flux(nfvars, ndims, u, nf, f);
        or_ns_flux(nfvars, ndims, du, nf, df);
    }
    for (oint i = 0; i < dnv; ++i) df[i] -= f[i];
}

/* ========================================================================
 * Scalar LU-SGS, FlowSys form (src/lusgs/lusgs.c).
 * All state arrays are SoA [nvars][nlocal] (rank order).
 * ====================================================================== */

/* lusgs_pack: src/lusgs/lusgs.c:8-37 */
void oracle_lusgs_pack(oint nlocal, oint neles, oint nvars, oint nfvars,
                       double turb_factor, double a0, const oint *cell_ids,
                       const oreal *upts, const oreal *rhs, const oreal *dt,
                       const oreal *dsrc, oreal *u, oreal *du, oreal *diag)
{
    OR_PARFOR
    for (oint idx = 0; idx < neles; ++idx) {
        oint ridx = cell_ids[idx];
        for (oint k = 0; k < nvars; ++k) {
            oint r = ridx + k * nlocal, e = idx + k * neles;
            oreal factor = k < nfvars ? 1.0 : turb_factor;
            u[r] = upts[e];
            du[r] = rhs[e];
            diag[r] = 1.0 / (dt[idx] * factor) + a0 + dsrc[e];
        }
    }
}

/* rank_lusgs_update: src/lusgs/lusgs.c:54-70 */
void oracle_lusgs_update(oint nlocal, oint neles, oint nvars, const oint *cell_ids,
                         const oreal *du, oreal *upts)
{
    OR_PARFOR
    for (oint idx = 0; idx < neles; ++idx) {
        oint ridx = cell_ids[idx];
        for (oint k = 0; k < nvars; ++k) upts[idx + k * neles] += du[ridx + k * nlocal];
    }
}

/* pre_lusgs: src/lusgs/lusgs.c:87-113 (NS: [0,nfvars), RANS: [nfvars,nvars)) */
void oracle_lusgs_prepare(oint nlocal, oint nv0, oint nv1, double kappa,
                          const oint *rowptr, const oint *slots, const oreal *face_area,
                          const oreal *rcp_vol, const oreal *lambdaf, oreal *diag)
{
    OR_PARFOR
    for (oint r = 0; r < nlocal; ++r) {
        oreal sd = 0.0;
        for (oint pos = rowptr[r]; pos < rowptr[r + 1]; ++pos) {
            oint slot = slots[pos];
            oreal lamf = lambdaf[slot] * kappa;
            sd += 0.5 * lamf * face_area[slot] * rcp_vol[r];
        }
        for (oint k = nv0; k < nv1; ++k) diag[r + k * nlocal] += sd;
    }
}

/* lower_sweep / upper_sweep: src/lusgs/lusgs.c:157-205 and 207-257.
 * dir = +1: lower (ascending rank order, neighbours with smaller index);
 * dir = -1: upper (descending order, neighbours with larger index). */
static void or_lusgs_sweep(int dir, int rans, oint nv0, oint nv1, double kappa,
                           const oreal *lambdaf, oint nlocal, oint nvars, oint nfvars,
                           oint ndims, oint nfaces, const oint *rowptr, const oint *colidx,
                           const int8_t *sides, const oint *slots, const oreal *face_area,
                           const oreal *face_normal, const oreal *rcp_vol,
                           const oreal *diag, const oreal *u_rank, oreal *du_rank)
{
    const oint dnv = nv1 - nv0;
    oreal du[16], dfj[16], df[16], u[16], nf[3];
    for (oint it = 0; it < nlocal; ++it) {
        oint r = dir > 0 ? it : nlocal - 1 - it;
        for (oint k = 0; k < dnv; ++k) df[k] = 0.0;
        for (oint pos = rowptr[r]; pos < rowptr[r + 1]; ++pos) {
            oint nb = colidx[pos];
            if (dir > 0 ? (nb < r) : (nb > r)) {
                oint slot = slots[pos];
                for (oint k = 0; k < nvars; ++k) u[k] = u_rank[nb + k * nlocal];
                int8_t side = sides[pos];
                for (oint d = 0; d < ndims; ++d) nf[d] = side * face_normal[slot + d * nfaces];
                oreal fv = face_area[slot] * rcp_vol[r];
                for (oint k = 0; k < nvars; ++k) du[k] = 0.0;
                for (oint k = nv0; k < nv1; ++k) du[k] = du_rank[nb + k * nlocal];
                or_diff_flux(nvars, nfvars, ndims, dnv, rans, u, du, dfj, nf);
                for (oint k = 0; k < dnv; ++k)
                    df[k] += (dfj[k] - kappa * lambdaf[slot] * du_rank[nb + (k + nv0) * nlocal]) * fv;
            }
        }
        for (oint k = 0; k < dnv; ++k) {
            oint l = r + (k + nv0) * nlocal;
            if (dir > 0)
                du_rank[l] = (du_rank[l] - 0.5 * df[k]) / diag[l];
            else
                du_rank[l] -= (0.5 * df[k] / diag[l]);
        }
    }
}

void oracle_lusgs_lower(int rans, oint nv0, oint nv1, double kappa, const oreal *lambdaf,
                        oint nlocal, oint nvars, oint nfvars, oint ndims, oint nfaces,
                        const oint *rowptr, const oint *colidx, const int8_t *sides,
                        const oint *slots, const oreal *face_area, const oreal *face_normal,
                        const oreal *rcp_vol, const oreal *diag, const oreal *u, oreal *du)
{
    or_lusgs_sweep(+1, rans, nv0, nv1, kappa, lambdaf, nlocal, nvars, nfvars, ndims, nfaces,
                   rowptr, colidx, sides, slots, face_area, face_normal, rcp_vol, diag, u, du);
}

void oracle_lusgs_upper(int rans, oint nv0, oint nv1, double kappa, const oreal *lambdaf,
                        oint nlocal, oint nvars, oint nfvars, oint ndims, oint nfaces,
                        const oint *rowptr, const oint *colidx, const int8_t *sides,
                        const oint *slots, const oreal *face_area, const oreal *face_normal,
                        const oreal *rcp_vol, const oreal *diag, const oreal *u, oreal *du)
{
    or_lusgs_sweep(-1, rans, nv0, nv1, kappa, lambdaf, nlocal, nvars, nfvars, ndims, nfaces,
                   rowptr, colidx, sides, slots, face_area, face_normal, rcp_vol, diag, u, du);
}

/* ========================================================================
 * Colored array ("legacy") LU-SGS: the entry points the reference examples
 * bind (examples/omp3d.py:22-35, examples/mpi3d.py:21-34), whose semantics
 * are given by README.md:15-50, doc/1_introduction.md:16-26 and
 * doc/3.1_lusgs.md:79-127.  The C source of this API is not part of the
 * reference snapshot; each routine below is the FlowSys routine above
 * specialised to the array layout with kappa = 1, rcp_vol = 1,
 * face_area = fnorm_vol, lambdaf = fspr, sides = +1 and "lower neighbour"
 * meaning "lower colour" (lcolor[nb] < lcolor[i]).  Under that mapping the
 * arithmetic of every cell is identical (multiplying by 1.0 / adding 0.0
 * are exact), which tests/test_oracle_pin.py checks bit-for-bit against
 * the reference FlowSys library on a colour-renumbered mesh.
 * Arrays: fnorm_vol, fspr, nei_ele [nface][neles]; vec_fnorm
 * [nface][ndims][neles]; upts, rhs, dub [nvars][neles]; dt, diag [neles].
 * ====================================================================== */

/* {serial,parallel}_pre_lusgs: lusgs.c:8-37 (diag = 1/(dt*factor)) plus
 * lusgs.c:87-113 (spectral-radius sum). */
void oracle_legacy_pre(oint neles, oint nface, double factor, const oreal *fnorm_vol,
                       const oreal *dt, oreal *diag, const oreal *fspr)
{
    OR_PARFOR
    for (oint i = 0; i < neles; ++i) {
        oreal sd = 0.0;
        for (oint f = 0; f < nface; ++f) {
            oreal lamf = fspr[f * neles + i];
            sd += 0.5 * lamf * fnorm_vol[f * neles + i];
        }
        diag[i] = 1.0 / (dt[i] * factor) + sd;
    }
}

/* One colour range [n0, ne) of icolor.  upper = 0: lower sweep reading rhs
 * and dub, writing dub.  upper = 1: upper sweep reading dub and rhs,
 * writing rhs (README.md:41-50).  rans selects the turbulence variables
 * [nfvars, nvars) and the RANS flux, otherwise [0, nfvars) and the NS flux.
 * lusgs.c:157-257 restated per colour. */
void oracle_legacy_sweep(int upper, int rans, oint n0, oint ne, oint neles, oint nface,
                         oint nvars, oint nfvars, oint ndims, const oint *nei_ele,
                         const oint *icolor, const oint *lcolor, const oreal *fnorm_vol,
                         const oreal *vec_fnorm, const oreal *upts, oreal *rhs, oreal *dub,
                         const oreal *diag, const oreal *fspr)
{
    const oint nv0 = rans ? nfvars : 0, nv1 = rans ? nvars : nfvars, dnv = nv1 - nv0;
    /* lower: neighbour increments live in dub, the result goes to dub;
     * upper: neighbour increments live in rhs, the result goes to rhs. */
    oreal *nbsrc = upper ? rhs : dub;
    oreal *own_in = upper ? dub : rhs;
    oreal *own_out = upper ? rhs : dub;
    OR_PARFOR
    for (oint t = n0; t < ne; ++t) {
        oreal du[16], dfj[16], df[16], u[16], nf[3];
        oint i = icolor[t];
        oint ci = lcolor[i];
        for (oint k = 0; k < dnv; ++k) df[k] = 0.0;
        for (oint f = 0; f < nface; ++f) {
            oint nb = nei_ele[f * neles + i];
            oint cn = lcolor[nb];
            if (upper ? (cn > ci) : (cn < ci)) {
                for (oint k = 0; k < nvars; ++k) u[k] = upts[k * neles + nb];
                for (oint d = 0; d < ndims; ++d) nf[d] = vec_fnorm[(f * ndims + d) * neles + i];
                oreal fv = fnorm_vol[f * neles + i];
                for (oint k = 0; k < nvars; ++k) du[k] = 0.0;
                for (oint k = nv0; k < nv1; ++k) du[k] = nbsrc[k * neles + nb];
                or_diff_flux(nvars, nfvars, ndims, dnv, rans, u, du, dfj, nf);
                for (oint k = 0; k < dnv; ++k)
                    df[k] += (dfj[k] - fspr[f * neles + i] * nbsrc[(k + nv0) * neles + nb]) * fv;
            }
        }
        for (oint k = 0; k < dnv; ++k) {
            oint l = (k + nv0) * neles + i;
            if (!upper)
                own_out[l] = (own_in[l] - 0.5 * df[k]) / diag[i];
            else
                own_out[l] = own_in[l] - (0.5 * df[k] / diag[i]);
        }
    }
}

/* Natural-order ("serial") sweeps: the same routine with lcolor = identity
 * ranks, i.e. neighbour index compared with cell index (lusgs.c:184,236). */
void oracle_legacy_serial_sweep(int upper, int rans, oint neles, oint nface, oint nvars,
                                oint nfvars, oint ndims, const oint *nei_ele,
                                const oreal *fnorm_vol, const oreal *vec_fnorm,
                                const oreal *upts, oreal *rhs, oreal *dub,
                                const oreal *diag, const oreal *fspr)
{
    oint *ord = (oint *)malloc(sizeof(oint) * (size_t)neles);
    for (oint i = 0; i < neles; ++i) ord[i] = i;
    /* cells must be visited one at a time in order: colour i+1 for cell i,
     * processed as neles single-cell colour ranges */
    oint *rank = (oint *)malloc(sizeof(oint) * (size_t)neles);
    for (oint i = 0; i < neles; ++i) rank[i] = i;
    for (oint it = 0; it < neles; ++it) {
        oint t = upper ? neles - 1 - it : it;
        oracle_legacy_sweep(upper, rans, t, t + 1, neles, nface, nvars, nfvars, ndims, nei_ele,
                            ord, rank, fnorm_vol, vec_fnorm, upts, rhs, dub, diag, fspr);
    }
    free(ord);
    free(rank);
}

/* lusgs_{serial,parallel}_{ns,rans}_update: lusgs.c:54-70, upts += dQ on
 * the variable range of the equation set. */
void oracle_legacy_update(int rans, oint neles, oint nvars, oint nfvars, oreal *upts,
                          const oreal *rhs)
{
    oint k0 = rans ? nfvars : 0, k1 = rans ? nvars : nfvars;
    OR_PARFOR
    for (oint i = 0; i < neles; ++i)
        for (oint k = k0; k < k1; ++k) upts[k * neles + i] += rhs[k * neles + i];
}

/* ========================================================================
 * Small dense LU without pivoting: src/lusgs/inverse.h:13-80 (identical to
 * src/krylov/utils/inverse.c:7-75).  Row-major, unit-lower L and U share
 * the buffer; a 1x1 block stores its reciprocal.
 * ====================================================================== */
void oracle_ludcmp(oint n, oreal *A)
{
    if (n == 1) {
        A[0] = 1.0 / A[0];
        return;
    }
    for (oint row = 1; row < n; ++row) {
        oint nr = n * row;
        A[nr] /= A[0];
        for (oint col = 1; col < n; ++col) {
            oreal v = 0.0;
            if (row > col) {
                for (oint k = 0; k < col; ++k) v += A[nr + k] * A[col + n * k];
                A[nr + col] = (A[nr + col] - v) / A[(n + 1) * col];
            } else {
                for (oint k = 0; k < row; ++k) v += A[nr + k] * A[n * k + col];
                A[nr + col] -= v;
            }
        }
    }
}

void oracle_lusub(oint n, const oreal *LU, oreal *b)
{
    if (n == 1) {
        b[0] *= LU[0];
        return;
    }
    for (oint row = 1; row < n; ++row) {
        oreal v = 0.0;
        for (oint col = 0; col < row; ++col) v += LU[row * n + col] * b[col];
        b[row] -= v;
    }
    b[n - 1] /= LU[n * n - 1];
    for (oint row = n - 2; row > -1; --row) {
        oreal v = 0.0;
        for (oint col = row + 1; col < n; ++col) v += LU[row * n + col] * b[col];
        b[row] = (b[row] - v) / LU[row * n + row];
    }
}

/* ========================================================================
 * Block LU-SGS, FlowSys form (src/lusgs/blusgs.c).  rhs/du/dup are AoS
 * [nlocal][nvars]; diag is [nlocal][nv][nv]; jmat is [2][nv][nv][nfaces].
 * ====================================================================== */

/* rank_blusgs_pack: blusgs.c:17-45 */
void oracle_blusgs_pack(oint nlocal, oint neles, oint nvars, oint nfvars, double a0,
                        const oint *cell_ids, const oreal *rhs, const oreal *dt,
                        oreal *rank_rhs, oreal *diag)
{
    const oint d2 = nfvars * nfvars;
    for (oint idx = 0; idx < neles; ++idx) {
        oint r = cell_ids[idx];
        for (oint k = 0; k < nvars; ++k) rank_rhs[k + r * nvars] = rhs[idx + k * neles];
        for (oint row = 0; row < nfvars; ++row) {
            oint off = row * nfvars + r * d2;
            for (oint col = 0; col < nfvars; ++col) diag[col + off] = 0.0;
            diag[row + off] = 1 / dt[idx] + a0;
        }
    }
}

/* rank_tblusgs_pack with kwsst / sa source Jacobians: blusgs.c:60-120,
 * src/lusgs/source_jacobian.c:6-18.  model 0 = k-omega SST, 1 = SA. */
void oracle_tblusgs_pack(int model, oint nlocal, oint neles, oint nvars, oint nfvars,
                         double a0, double factor, const oint *cell_ids, const oreal *uptsb,
                         const oreal *dsrc, const oreal *dt, oreal *tdiag)
{
    const oint nt = nvars - nfvars, d2 = nt * nt;
    oreal u[16], d[16];
    for (oint idx = 0; idx < neles; ++idx) {
        oint r = cell_ids[idx];
        oreal *A = &tdiag[r * d2];
        for (oint i = 0; i < d2; ++i) A[i] = 0.0;
        for (oint k = 0; k < nvars; ++k) {
            u[k] = uptsb[idx + k * neles];
            d[k] = dsrc[idx + k * neles];
        }
        if (model == 0) {
            oreal kk = u[nvars - 2] / u[0];
            A[0] += d[nvars - 2];
            oreal bk = 0.09 * kk; /* BETAST, flux.h:16 */
            A[1] += bk > 0.0 ? bk : 0.0;
            A[1 + nt] = d[nvars - 1];
        } else {
            A[0] += d[nvars - 1];
        }
        for (oint row = 0; row < nt; ++row) A[row + row * nt] += 1 / (dt[idx] * factor) + a0;
    }
}

/* rank_blusgs_update: blusgs.c:126-143 */
void oracle_blusgs_update(oint nlocal, oint neles, oint nvars, const oint *cell_ids,
                          const oreal *du, oreal *upts)
{
    for (oint idx = 0; idx < neles; ++idx) {
        oint r = cell_ids[idx];
        for (oint k = 0; k < nvars; ++k) upts[idx + k * neles] += du[k + r * nvars];
    }
}

/* rank_sub_residual: blusgs.c:161-185 */
void oracle_blusgs_sub_residual(oint nlocal, oint neles, oint nvars, const oint *cell_ids,
                                const oreal *vol, const oreal *du, oreal *dup, oreal *res)
{
    for (oint idx = 0; idx < neles; ++idx) {
        oint r = cell_ids[idx];
        for (oint k = 0; k < nvars; ++k) {
            oint o = k + r * nvars;
            oreal diff = du[o] - dup[o];
            res[idx + k * neles] = diff * diff * vol[idx];
            dup[o] = du[o];
        }
    }
}

/* pre_blusgs: blusgs.c:200-246.  side == 1 adds jmat half 0, else
 * subtracts half 1; then the block is LU-factored in place. */
void oracle_blusgs_prepare(oint nlocal, oint nv, oint nfaces, const oint *rowptr,
                           const oint *slots, const int8_t *sides, const oreal *face_area,
                           const oreal *rcp_vol, oreal *diag, const oreal *jmat)
{
    const oint d2 = nv * nv;
    oreal dm[64];
    for (oint r = 0; r < nlocal; ++r) {
        for (oint i = 0; i < d2; ++i) dm[i] = diag[i + r * d2];
        for (oint pos = rowptr[r]; pos < rowptr[r + 1]; ++pos) {
            oint slot = slots[pos];
            int8_t side = sides[pos];
            oreal fv = face_area[slot] * rcp_vol[r];
            for (oint row = 0; row < nv; ++row)
                for (oint col = 0; col < nv; ++col) {
                    oreal val;
                    if (side == 1)
                        val = jmat[slot + col * nfaces + row * nfaces * nv];
                    else
                        val = -jmat[slot + col * nfaces + row * nfaces * nv + d2 * nfaces];
                    dm[col + row * nv] += val * fv;
                }
        }
        oracle_ludcmp(nv, dm);
        for (oint i = 0; i < d2; ++i) diag[i + r * d2] = dm[i];
    }
}

/* lower_sweep / upper_sweep: blusgs.c:273-373.  Every CSR neighbour
 * contributes (Gauss-Seidel: already-visited cells hold new values);
 * side == 1 uses jmat half 1, else minus half 0. */
static void or_blusgs_sweep(int dir, oint var0, oint nv, oint nlocal, oint nvars,
                            oint nfaces, const oint *rowptr, const oint *colidx,
                            const int8_t *sides, const oint *slots, const oreal *face_area,
                            const oreal *rcp_vol, const oreal *rhsb, const oreal *diag,
                            const oreal *jmat, oreal *dub)
{
    const oint d2 = nv * nv;
    oreal rhs[16], dm[64];
    for (oint it = 0; it < nlocal; ++it) {
        oint r = dir > 0 ? it : nlocal - 1 - it;
        for (oint row = 0; row < nv; ++row) {
            rhs[row] = rhsb[var0 + row + r * nvars];
            for (oint col = 0; col < nv; ++col) dm[col + nv * row] = diag[col + nv * row + r * d2];
        }
        for (oint pos = rowptr[r]; pos < rowptr[r + 1]; ++pos) {
            oint nb = colidx[pos], slot = slots[pos];
            int8_t side = sides[pos];
            oreal fv = face_area[slot] * rcp_vol[r];
            for (oint row = 0; row < nv; ++row) {
                oreal val = 0.0;
                for (oint col = 0; col < nv; ++col) {
                    oreal jv;
                    if (side == 1)
                        jv = jmat[slot + col * nfaces + row * nv * nfaces + d2 * nfaces];
                    else
                        jv = -jmat[slot + col * nfaces + row * nv * nfaces];
                    val += jv * dub[var0 + col + nb * nvars];
                }
                rhs[row] -= val * fv;
            }
        }
        oracle_lusub(nv, dm, rhs);
        for (oint row = 0; row < nv; ++row) dub[var0 + row + r * nvars] = rhs[row];
    }
}

void oracle_blusgs_lower(oint var0, oint nv, oint nlocal, oint nvars, oint nfaces,
                         const oint *rowptr, const oint *colidx, const int8_t *sides,
                         const oint *slots, const oreal *face_area, const oreal *rcp_vol,
                         const oreal *rhsb, const oreal *diag, const oreal *jmat, oreal *dub)
{
    or_blusgs_sweep(+1, var0, nv, nlocal, nvars, nfaces, rowptr, colidx, sides, slots,
                    face_area, rcp_vol, rhsb, diag, jmat, dub);
}

void oracle_blusgs_upper(oint var0, oint nv, oint nlocal, oint nvars, oint nfaces,
                         const oint *rowptr, const oint *colidx, const int8_t *sides,
                         const oint *slots, const oreal *face_area, const oreal *rcp_vol,
                         const oreal *rhsb, const oreal *diag, const oreal *jmat, oreal *dub)
{
    or_blusgs_sweep(-1, var0, nv, nlocal, nvars, nfaces, rowptr, colidx, sides, slots,
                    face_area, rcp_vol, rhsb, diag, jmat, dub);
}

/* ========================================================================
 * Krylov: BSR SpMV, BLU-SGS preconditioner, GMRES(m).
 * ====================================================================== */

/* SpMV_BSR: src/krylov/matrix/sparsemat.c:57-101.  y = alpha*A*x + beta*y
 * with row-major b x b blocks and AoS vectors. */
void oracle_bsr_spmv(oint bn, oint blk, const oint *rowptr, const oint *colidx,
                     const oreal *values, double alpha, const oreal *x, double beta, oreal *y)
{
    const oint b2 = blk * blk;
    OR_PARFOR
    for (oint i = 0; i < bn; ++i) {
        oreal arr[16];
        for (oint k = 0; k < blk; ++k) arr[k] = 0.0;
        for (oint j = rowptr[i]; j < rowptr[i + 1]; ++j) {
            oint c = colidx[j];
            for (oint row = 0; row < blk; ++row) {
                oreal v = 0.0;
                for (oint col = 0; col < blk; ++col)
                    v += values[(size_t)j * b2 + row * blk + col] * x[(size_t)c * blk + col];
                arr[row] += v;
            }
        }
        for (oint k = 0; k < blk; ++k)
            y[(size_t)i * blk + k] = alpha * arr[k] + beta * y[(size_t)i * blk + k];
    }
}

/* BLUSGSPreconPrepare: src/krylov/precon/blusgs.c:7-26 */
void oracle_blusgs_precon_prepare(oint bn, oint blk, const oint *diagslots,
                                  const oreal *values, oreal *diagvalues)
{
    const oint b2 = blk * blk;
    OR_PARFOR
    for (oint i = 0; i < bn; ++i) {
        oreal *d = &diagvalues[(size_t)i * b2];
        memcpy(d, &values[(size_t)diagslots[i] * b2], sizeof(oreal) * b2);
        oracle_ludcmp(blk, d);
    }
}

/* One block row of the forward solve (D+L)x' = b: precon/blusgs.c:104-130 */
static void or_pc_lower_row(oint i, oint blk, const oint *rowptr, const oint *colidx,
                            const oint *diagslots, const oreal *values,
                            const oreal *diagvalues, oreal *b)
{
    const oint b2 = blk * blk;
    oreal arr[16];
    for (oint k = 0; k < blk; ++k) arr[k] = b[k + (size_t)i * blk];
    for (oint j = rowptr[i]; j < diagslots[i]; ++j) {
        oint c = colidx[j];
        for (oint row = 0; row < blk; ++row) {
            oreal v = 0.0;
            for (oint col = 0; col < blk; ++col)
                v += values[col + row * blk + (size_t)j * b2] * b[col + (size_t)c * blk];
            arr[row] -= v;
        }
    }
    oracle_lusub(blk, &diagvalues[(size_t)i * b2], arr);
    for (oint k = 0; k < blk; ++k) b[k + (size_t)i * blk] = arr[k];
}

/* One block row of the backward step x = x' - inv(D) U x:
 * precon/blusgs.c:132-161 */
static void or_pc_upper_row(oint i, oint blk, const oint *rowptr, const oint *colidx,
                            const oint *diagslots, const oreal *values,
                            const oreal *diagvalues, oreal *b)
{
    const oint b2 = blk * blk;
    oreal arr[16];
    for (oint k = 0; k < blk; ++k) arr[k] = 0.0;
    for (oint j = diagslots[i] + 1; j < rowptr[i + 1]; ++j) {
        oint c = colidx[j];
        for (oint row = 0; row < blk; ++row) {
            oreal v = 0.0;
            for (oint col = 0; col < blk; ++col)
                v += values[col + row * blk + (size_t)j * b2] * b[col + (size_t)c * blk];
            arr[row] += v;
        }
    }
    oracle_lusub(blk, &diagvalues[(size_t)i * b2], arr);
    for (oint k = 0; k < blk; ++k) b[k + (size_t)i * blk] -= arr[k];
}

/* BLUSGSPreconApply: precon/blusgs.c:28-100 (natural order, in place) */
void oracle_blusgs_precon_apply(oint bn, oint blk, const oint *rowptr, const oint *colidx,
                                const oint *diagslots, const oreal *values,
                                const oreal *diagvalues, oreal *b)
{
    for (oint i = 0; i < bn; ++i)
        or_pc_lower_row(i, blk, rowptr, colidx, diagslots, values, diagvalues, b);
    for (oint i = bn - 1; i > -1; --i)
        or_pc_upper_row(i, blk, rowptr, colidx, diagslots, values, diagvalues, b);
}

/* PBLUSGSPreconApply: precon/pblusgs.c:90-104, colours as contiguous row
 * ranges icolors[c]..icolors[c+1], lower in ascending colour order, upper
 * in descending order.  The lower apply indexes the diagonal block at
 * idx*blkdim (pblusgs.c:41 writes idx+blkdim, which reads the wrong block;
 * this restatement follows the intended, natural-order routine). */
void oracle_pblusgs_precon_apply(oint bn, oint blk, oint ncolors, const oint *icolors,
                                 const oint *rowptr, const oint *colidx,
                                 const oint *diagslots, const oreal *values,
                                 const oreal *diagvalues, oreal *b)
{
    for (oint c = 0; c < ncolors; ++c) {
        OR_PARFOR
        for (oint i = icolors[c]; i < icolors[c + 1]; ++i)
            or_pc_lower_row(i, blk, rowptr, colidx, diagslots, values, diagvalues, b);
    }
    for (oint c = ncolors - 1; c >= 0; --c) {
        OR_PARFOR
        for (oint i = icolors[c]; i < icolors[c + 1]; ++i)
            or_pc_upper_row(i, blk, rowptr, colidx, diagslots, values, diagvalues, b);
    }
}

/* BLAS kernels: src/krylov/utils/blas_basic.c:4-61 (serial sums; the
 * reference's OpenMP reductions equal these with one thread). */
static oreal or_nrm2(oint n, const oreal *a)
{
    oreal s = 0.0;
    for (oint i = 0; i < n; ++i) s += a[i] * a[i];
    return sqrt(s);
}

static void or_gemvcol(oint m, oint n, oint lda, oreal alpha, const oreal *a, const oreal *x,
                       oreal beta, oreal *y)
{
    OR_PARFOR
    for (oint i = 0; i < m; ++i) {
        oreal s = 0.0;
        for (oint j = 0; j < n; ++j) s += a[i + (size_t)j * lda] * x[j];
        y[i] = alpha * s + beta * y[i];
    }
}

static void or_gemvcoltrans(oint m, oint n, oint lda, oreal alpha, const oreal *a,
                            const oreal *x, oreal beta, oreal *y)
{
    for (oint j = 0; j < n; ++j) {
        oreal s = 0.0;
        for (oint i = 0; i < m; ++i) s += a[i + (size_t)j * lda] * x[i];
        y[j] = alpha * s + beta * y[j];
    }
}

/* Preconditioner selector for GMRES: 0 none, 1 natural-order BLU-SGS,
 * 2 coloured BLU-SGS (colour ranges). */
typedef struct {
    int kind;
    oint bn, blk, ncolors;
    const oint *rowptr, *colidx, *diagslots, *icolors;
    const oreal *values, *diagvalues;
} or_precon;

static void or_pc_apply(const or_precon *pc, oreal *b)
{
    if (pc->kind == 1)
        oracle_blusgs_precon_apply(pc->bn, pc->blk, pc->rowptr, pc->colidx, pc->diagslots,
                                   pc->values, pc->diagvalues, b);
    else if (pc->kind == 2)
        oracle_pblusgs_precon_apply(pc->bn, pc->blk, pc->ncolors, pc->icolors, pc->rowptr,
                                    pc->colidx, pc->diagslots, pc->values, pc->diagvalues, b);
}

/* GMRESSolve + arnoldi_cgs2: src/krylov/solver/gmres.c:4-129.
 * Left-preconditioned restarted GMRES(m), classical Gram-Schmidt with one
 * re-orthogonalisation, Givens rotations, absolute stopping test
 * ||b - A x|| <= tol.  Returns the status code of ucfdtypes.h:22-30
 * (0 converged, 1 happy breakdown, 2 iteration limit) and writes the
 * outer-iteration count and last true residual. */
int oracle_gmres(oint bn, oint blk, const oint *rowptr, const oint *colidx,
                 const oreal *values, int pc_kind, oint ncolors, const oint *icolors,
                 const oint *diagslots, const oreal *diagvalues, oint m, oint maxiter,
                 double tol, double haptol, oreal *x, const oreal *b, oint *iters,
                 double *resid, double *hist)
{
    const oint n = bn * blk, ld = m + 1;
    or_precon pc = {pc_kind, bn, blk, ncolors, rowptr, colidx, diagslots, icolors, values, diagvalues};
    oreal *H = (oreal *)calloc((size_t)(m + 1) * m, sizeof(oreal));
    oreal *V = (oreal *)calloc((size_t)n * (m + 1), sizeof(oreal));
    oreal *y = (oreal *)calloc((size_t)(m + 1), sizeof(oreal));
    oreal *w = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *sn = (oreal *)calloc((size_t)(m + 1), sizeof(oreal));
    oreal *cs = (oreal *)calloc((size_t)(m + 1), sizeof(oreal));
    oreal *h2 = (oreal *)calloc((size_t)(m + 1), sizeof(oreal));
    oreal *r = (oreal *)calloc((size_t)n, sizeof(oreal));
    int stat = -1;
    oint iter = 0;
    oreal abeta = 0.0;
    while (iter < maxiter) {
        /* r = b - A x (solverimpl.h:45-50) */
        memcpy(r, b, sizeof(oreal) * n);
        oracle_bsr_spmv(bn, blk, rowptr, colidx, values, -1.0, x, 1.0, r);
        abeta = or_nrm2(n, r);
        if (hist) hist[iter] = abeta;
        if (abeta <= tol) {
            stat = 0;
            break;
        }
        or_pc_apply(&pc, r);
        oreal beta = or_nrm2(n, r);
        y[0] = beta;
        for (oint i = 0; i < n; ++i) V[i] = r[i];
        for (oint i = 0; i < n; ++i) V[i] = (1.0 / beta) * V[i];
        oint k = 0;
        for (oint j = 0; j < m; ++j) {
            const oint kk = j + 1;
            oreal *vj = V + (size_t)j * n;
            oreal *Hc = H + (size_t)j * ld;
            oracle_bsr_spmv(bn, blk, rowptr, colidx, values, 1.0, vj, 0.0, w);
            or_pc_apply(&pc, w);
            or_gemvcoltrans(n, kk, n, 1.0, V, w, 0.0, Hc);
            or_gemvcol(n, kk, n, -1.0, V, Hc, 1.0, w);
            or_gemvcoltrans(n, kk, n, 1.0, V, w, 0.0, h2);
            or_gemvcol(n, kk, n, -1.0, V, h2, 1.0, w);
            for (oint i = 0; i < kk; ++i) Hc[i] += 1.0 * h2[i];
            oreal hsub = or_nrm2(n, w);
            Hc[j + 1] = hsub;
            oreal *vn = V + (size_t)(j + 1) * n;
            for (oint i = 0; i < n; ++i) vn[i] = w[i];
            for (oint i = 0; i < n; ++i) vn[i] = (1.0 / hsub) * vn[i];
            /* Givens rotations: gmres.c:87-102 */
            for (oint i = 0; i < j; ++i) {
                oreal c = cs[i], s = sn[i];
                oreal t = c * Hc[i] + s * Hc[i + 1];
                Hc[i + 1] = -s * Hc[i] + c * Hc[i + 1];
                Hc[i] = t;
            }
            oreal h1v = Hc[j], h2v = Hc[j + 1];
            oreal rr = hypot(h1v, h2v);
            cs[j] = h1v / rr;
            sn[j] = h2v / rr;
            Hc[j] = cs[j] * Hc[j] + sn[j] * Hc[j + 1];
            Hc[j + 1] = 0.0;
            y[j + 1] = -sn[j] * y[j];
            y[j] = cs[j] * y[j];
            k = j + 1;
            if (hsub < haptol * beta) {
                stat = 1;
                break;
            }
        }
        /* back substitution: gmres.c:111-117 */
        for (oint i = k - 1; i >= 0; --i) {
            oreal s = y[i];
            for (oint jj = i + 1; jj < k; ++jj) s -= H[i + (size_t)jj * ld] * y[jj];
            y[i] = s / H[i + (size_t)i * ld];
        }
        or_gemvcol(n, k, n, 1.0, V, y, 1.0, x);
        iter++;
    }
    if (iter == maxiter) stat = 2;
    *iters = iter;
    *resid = abeta;
    free(H); free(V); free(y); free(w); free(sn); free(cs); free(h2); free(r);
    return stat;
}

/* ========================================================================
 * Incomplete factorisations and BiCGSTAB (src/krylov/precon/{ilu,bilu,
 * pbilu}.c, src/krylov/solver/bicgstab.c).
 * ====================================================================== */

/* lusubmattrans: src/krylov/utils/inverse.c:79-108.  B := B inv(LU) for an
 * n x n row-major B and the in-place factors LU of oracle_ludcmp: first
 * Y U = B column by column, then X L = Y. */
void oracle_lusubmattrans(oint n, const oreal *LU, oreal *B)
{
    if (n == 1) {
        B[0] *= LU[0];
        return;
    }
    for (oint s = 0; s < n; ++s) B[s * n] /= LU[0];
    for (oint row = 1; row < n; ++row)
        for (oint s = 0; s < n; ++s) {
            oreal v = 0.0;
            for (oint col = 0; col < row; ++col) v += B[s * n + col] * LU[col * n + row];
            B[s * n + row] = (B[s * n + row] - v) / LU[row * n + row];
        }
    for (oint row = n - 2; row > -1; --row)
        for (oint s = 0; s < n; ++s) {
            oreal v = 0.0;
            for (oint col = row + 1; col < n; ++col) v += B[s * n + col] * LU[col * n + row];
            B[s * n + row] -= v;
        }
}

/* BILUPreconPrepare: src/krylov/precon/bilu.c:5-62.  Block ILU(0) in
 * natural row order, in place on values: for each lower entry (i,k) in
 * slot order, A_ik := A_ik inv(A_kk), then A_ij -= A_ik A_kj for every
 * later slot j of row i whose column row k also holds; finally the
 * diagonal block is LU-factorised.  iw maps a column of row k to its slot
 * (the last slot if a column repeats).  PBILUPreconPrepare (pbilu.c:5-79)
 * computes the same per colour, which on a colour-ordered matrix equals
 * this natural order. */
void oracle_bilu_prepare(oint bn, oint blk, const oint *rowptr, const oint *colidx,
                         const oint *diagslots, oreal *values)
{
    const oint b2 = blk * blk;
    oint *iw = (oint *)malloc(sizeof(oint) * (size_t)bn);
    oreal aik[256];
    for (oint i = 0; i < bn; ++i) iw[i] = -1;
    for (oint i = 0; i < bn; ++i) {
        const oint st = rowptr[i], ed = diagslots[i], jed = rowptr[i + 1];
        for (oint kd = st; kd < ed; ++kd) {
            const oint ck = colidx[kd], kk = diagslots[ck], kst = rowptr[ck], ked = rowptr[ck + 1];
            oracle_lusubmattrans(blk, &values[(size_t)kk * b2], &values[(size_t)kd * b2]);
            memcpy(aik, &values[(size_t)kd * b2], sizeof(oreal) * b2);
            for (oint jj = kst; jj < ked; ++jj) iw[colidx[jj]] = jj;
            for (oint jj = kd + 1; jj < jed; ++jj) {
                const oint iwj = iw[colidx[jj]];
                if (iwj == -1) continue;
                for (oint row = 0; row < blk; ++row)
                    for (oint col = 0; col < blk; ++col) {
                        oreal v = 0.0;
                        for (oint e = 0; e < blk; ++e)
                            v += aik[row * blk + e] * values[(size_t)iwj * b2 + e * blk + col];
                        values[(size_t)jj * b2 + row * blk + col] -= v;
                    }
            }
            for (oint jj = kst; jj < ked; ++jj) iw[colidx[jj]] = -1;
        }
        oracle_ludcmp(blk, &values[(size_t)ed * b2]);
    }
    free(iw);
}

/* BILUPreconApply: src/krylov/precon/bilu.c:64-129 (natural order, in
 * place): forward b_i -= sum_{j<i} L_ij b_j, then backward
 * b_i = inv(LU_ii) (b_i - sum_{j>i} U_ij b_j).  PBILUPreconApply
 * (pbilu.c:81-200) equals it on a colour-ordered matrix. */
void oracle_bilu_apply(oint bn, oint blk, const oint *rowptr, const oint *colidx,
                       const oint *diagslots, const oreal *values, oreal *b)
{
    const oint b2 = blk * blk;
    oreal arr[16];
    for (oint i = 0; i < bn; ++i) {
        for (oint k = 0; k < blk; ++k) arr[k] = b[k + (size_t)i * blk];
        for (oint j = rowptr[i]; j < diagslots[i]; ++j) {
            const oint c = colidx[j];
            for (oint row = 0; row < blk; ++row) {
                oreal v = 0.0;
                for (oint col = 0; col < blk; ++col)
                    v += values[col + row * blk + (size_t)j * b2] * b[col + (size_t)c * blk];
                arr[row] -= v;
            }
        }
        for (oint k = 0; k < blk; ++k) b[k + (size_t)i * blk] = arr[k];
    }
    for (oint i = bn - 1; i > -1; --i) {
        for (oint k = 0; k < blk; ++k) arr[k] = b[k + (size_t)i * blk];
        for (oint j = diagslots[i] + 1; j < rowptr[i + 1]; ++j) {
            const oint c = colidx[j];
            for (oint row = 0; row < blk; ++row) {
                oreal v = 0.0;
                for (oint col = 0; col < blk; ++col)
                    v += values[col + row * blk + (size_t)j * b2] * b[col + (size_t)c * blk];
                arr[row] -= v;
            }
        }
        oracle_lusub(blk, &values[(size_t)diagslots[i] * b2], arr);
        for (oint k = 0; k < blk; ++k) b[(size_t)i * blk + k] = arr[k];
    }
}

/* ILUPreconPrepare: src/krylov/precon/ilu.c:4-47 (scalar ILU(0), in
 * place; the diagonal is kept, not inverted). */
void oracle_ilu_prepare(oint n, const oint *rowptr, const oint *colidx, const oint *diagslots,
                        oreal *values)
{
    oint *iw = (oint *)malloc(sizeof(oint) * (size_t)n);
    for (oint i = 0; i < n; ++i) iw[i] = -1;
    for (oint i = 0; i < n; ++i) {
        const oint st = rowptr[i], ed = diagslots[i], jed = rowptr[i + 1];
        for (oint kd = st; kd < ed; ++kd) {
            const oint ck = colidx[kd], kk = diagslots[ck], kst = rowptr[ck], ked = rowptr[ck + 1];
            values[kd] /= values[kk];
            const oreal aik = values[kd];
            for (oint jj = kst; jj < ked; ++jj) iw[colidx[jj]] = jj;
            for (oint jj = kd + 1; jj < jed; ++jj) {
                const oint iwj = iw[colidx[jj]];
                if (iwj != -1) values[jj] -= aik * values[iwj];
            }
            for (oint jj = kst; jj < ked; ++jj) iw[colidx[jj]] = -1;
        }
    }
    free(iw);
}

/* ILUPreconApply: src/krylov/precon/ilu.c:49-85, with the backward loop
 * starting after the diagonal slot.  ilu.c:78 starts it at the diagonal
 * slot itself, which subtracts a_ii b_i before dividing by a_ii; the
 * intended triangular solve, restated here, excludes it. */
void oracle_ilu_apply(oint n, const oint *rowptr, const oint *colidx, const oint *diagslots,
                      const oreal *values, oreal *b)
{
    for (oint i = 0; i < n; ++i) {
        oreal v = b[i];
        for (oint j = rowptr[i]; j < diagslots[i]; ++j) v -= values[j] * b[colidx[j]];
        b[i] = v;
    }
    for (oint i = n - 1; i > -1; --i) {
        const oint dd = diagslots[i];
        oreal v = b[i];
        for (oint j = dd + 1; j < rowptr[i + 1]; ++j) v -= values[j] * b[colidx[j]];
        b[i] = v / values[dd];
    }
}

/* Preconditioner of oracle_bicgstab: 0 none, 1 BLU-SGS (natural), 2
 * coloured BLU-SGS (colour ranges), 3 BILU / PBILU with factored values
 * (fvalues from oracle_bilu_prepare), 4 ILU with factored values. */
static void or_pc_apply_any(int kind, oint bn, oint blk, oint ncolors, const oint *icolors,
                            const oint *rowptr, const oint *colidx, const oint *diagslots,
                            const oreal *values, const oreal *diagvalues, const oreal *fvalues, oreal *b)
{
    if (kind == 1)
        oracle_blusgs_precon_apply(bn, blk, rowptr, colidx, diagslots, values, diagvalues, b);
    else if (kind == 2)
        oracle_pblusgs_precon_apply(bn, blk, ncolors, icolors, rowptr, colidx, diagslots, values, diagvalues, b);
    else if (kind == 3)
        oracle_bilu_apply(bn, blk, rowptr, colidx, diagslots, fvalues, b);
    else if (kind == 4)
        oracle_ilu_apply(bn * blk, rowptr, colidx, diagslots, fvalues, b);
}

static oreal or_dot(oint n, const oreal *x, const oreal *y)
{
    oreal s = 0.0;
    for (oint i = 0; i < n; ++i) s += x[i] * y[i];
    return s;
}

static void or_axpy(oint n, oreal a, const oreal *x, oreal *y)
{
    for (oint i = 0; i < n; ++i) y[i] += a * x[i];
}

/* BICGSTABSolve: src/krylov/solver/bicgstab.c:24-128.  Right-preconditioned
 * BiCGSTAB with the fused five-term reduction of bicgstab.c:5-22 and the
 * residual-norm estimate sqrt|ss - 2 w ts + w^2 tt|; stops when it drops
 * below tol (absolute).  Returns the status of ucfdtypes.h:22-30 (0
 * converged, 2 iteration limit, 3 rho breakdown, 4 pi breakdown) and
 * writes the iteration count, the last estimate and (if hist) the
 * estimate of every iteration. */
int oracle_bicgstab(oint bn, oint blk, const oint *rowptr, const oint *colidx, const oreal *values,
                    int pc_kind, oint ncolors, const oint *icolors, const oint *diagslots,
                    const oreal *diagvalues, const oreal *fvalues, oint maxiter, double tol, oreal *x,
                    const oreal *b, oint *iters, double *resid, double *hist)
{
    const oint n = bn * blk;
    oreal *r = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *rt = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *p = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *pt = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *v = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *s = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *sh = (oreal *)calloc((size_t)n, sizeof(oreal));
    oreal *t = (oreal *)calloc((size_t)n, sizeof(oreal));
    int stat = -1;
    oint iter = 0;
    oreal rho, rhoprev = 1.0, alpha = 1.0, omega = 1.0, resnorm = 0.0;
    memcpy(r, b, sizeof(oreal) * n);
    oracle_bsr_spmv(bn, blk, rowptr, colidx, values, -1.0, x, 1.0, r);
    memcpy(rt, r, sizeof(oreal) * n);
    rho = or_dot(n, rt, r);
    if (fabs(rho) < 1e-30) {
        stat = 3;
        goto done;
    }
    while (iter < maxiter) {
        if (iter == 0) {
            memcpy(p, r, sizeof(oreal) * n);
        } else {
            const oreal beta = (rho / rhoprev) * (alpha / omega);
            or_axpy(n, -omega, v, p);
            for (oint i = 0; i < n; ++i) p[i] = beta * p[i];
            or_axpy(n, 1.0, r, p);
        }
        memcpy(pt, p, sizeof(oreal) * n);
        or_pc_apply_any(pc_kind, bn, blk, ncolors, icolors, rowptr, colidx, diagslots, values, diagvalues,
                        fvalues, pt);
        oracle_bsr_spmv(bn, blk, rowptr, colidx, values, 1.0, pt, 0.0, v);
        const oreal pi = or_dot(n, rt, v);
        if (fabs(pi) < 1e-30) {
            stat = 4;
            break;
        }
        alpha = rho / pi;
        memcpy(s, r, sizeof(oreal) * n);
        or_axpy(n, -alpha, v, s);
        memcpy(sh, s, sizeof(oreal) * n);
        or_pc_apply_any(pc_kind, bn, blk, ncolors, icolors, rowptr, colidx, diagslots, values, diagvalues,
                        fvalues, sh);
        oracle_bsr_spmv(bn, blk, rowptr, colidx, values, 1.0, sh, 0.0, t);
        oreal phi = 0.0, rtt = 0.0, ts = 0.0, tt = 0.0, ss = 0.0;
        for (oint k = 0; k < n; ++k) {
            const oreal sk = s[k], tk = t[k], rk = rt[k];
            phi += rk * sk;
            rtt += rk * tk;
            ts += tk * sk;
            tt += tk * tk;
            ss += sk * sk;
        }
        omega = ts / tt;
        or_axpy(n, alpha, pt, x);
        or_axpy(n, omega, sh, x);
        memcpy(r, s, sizeof(oreal) * n);
        or_axpy(n, -omega, t, r);
        const oreal rho_new = phi - omega * rtt;
        resnorm = sqrt(fabs(ss - 2.0 * omega * ts + omega * omega * tt));
        if (hist) hist[iter] = resnorm;
        if (resnorm < tol) {
            stat = 0;
            goto done;
        }
        rhoprev = rho;
        rho = rho_new;
        iter++;
    }
done:
    if (iter == maxiter) stat = 2;
    *iters = iter;
    *resid = resnorm;
    free(r); free(rt); free(p); free(pt); free(v); free(s); free(sh); free(t);
    return stat;
}

/* ========================================================================
 * Greedy first-fit colouring of a CSR graph, cells visited in index order.
 * The reference has no general colouring (its examples use the checkerboard
 * of examples/utils/pbutils.py:39-56); this is the colouring the GB300
 * library defines for jittered / permuted meshes, restated here so that the
 * CPU legs can colour a mesh without the product library.  A cell takes the
 * smallest colour that no already coloured neighbour holds, an edge counting
 * in both directions (the graph is used as if symmetric; negative and
 * self entries are ignored).  color[] gets
 * 0-based colours; returns the number of colours (-1 on allocation failure).
 * ====================================================================== */
int oracle_greedy_coloring_csr(oint n, const oint *rowptr, const oint *colidx, oint *color)
{
    const oint nnz = rowptr[n];
    oint *trp = (oint *)calloc((size_t)n + 1, sizeof(oint));
    oint *tci = (oint *)malloc(sizeof(oint) * (size_t)(nnz > 0 ? nnz : 1));
    oint maxdeg = 0;
    if (!trp || !tci) {
        free(trp); free(tci);
        return -1;
    }
    /* transpose: the cells that list i as a neighbour */
    for (oint i = 0; i < n; ++i)
        for (oint p = rowptr[i]; p < rowptr[i + 1]; ++p)
            if (colidx[p] >= 0 && colidx[p] != i) trp[colidx[p] + 1]++;
    for (oint i = 0; i < n; ++i) trp[i + 1] += trp[i];
    {
        oint *fill = (oint *)malloc(sizeof(oint) * (size_t)(n > 0 ? n : 1));
        if (!fill) {
            free(trp); free(tci);
            return -1;
        }
        memcpy(fill, trp, sizeof(oint) * (size_t)n);
        for (oint i = 0; i < n; ++i)
            for (oint p = rowptr[i]; p < rowptr[i + 1]; ++p)
                if (colidx[p] >= 0 && colidx[p] != i) tci[fill[colidx[p]]++] = i;
        free(fill);
    }
    for (oint i = 0; i < n; ++i) {
        oint d = (rowptr[i + 1] - rowptr[i]) + (trp[i + 1] - trp[i]);
        if (d > maxdeg) maxdeg = d;
    }
    oint *mark = (oint *)malloc(sizeof(oint) * (size_t)(maxdeg + 2));
    if (!mark) {
        free(trp); free(tci);
        return -1;
    }
    for (oint c = 0; c < maxdeg + 2; ++c) mark[c] = -1;
    oint nc = 0;
    for (oint i = 0; i < n; ++i) color[i] = -1;
    for (oint i = 0; i < n; ++i) {
        for (oint p = rowptr[i]; p < rowptr[i + 1]; ++p) {
            const oint j = colidx[p];
            if (j >= 0 && j != i && color[j] >= 0) mark[color[j]] = i;
        }
        for (oint p = trp[i]; p < trp[i + 1]; ++p) {
            const oint j = tci[p];
            if (color[j] >= 0) mark[color[j]] = i;
        }
        oint c = 0;
        while (mark[c] == i) ++c;
        color[i] = c;
        if (c + 1 > nc) nc = c + 1;
    }
    free(mark); free(trp); free(tci);
    return nc;
}
