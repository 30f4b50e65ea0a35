// krylov.cpp -- SpMat / Precon / Solver objects (ucfdmat.h, ucfdprecon.h,
// ucfdsolver.h) on the GPU.
//
// Matrices and preconditioners live on the device in the ELL-of-blocks
// layout of kernels_krylov.cuh.  Their structure (schedule, columns, the CSR
// slot behind every ELL entry) is built on the host once and kept while the
// fingerprints of rowptr / colidx / diagslots stay the same; new values are
// gathered, factorised and LU-factored on the device.  GMRES(m) keeps every
// vector, the Hessenberg matrix and the Givens state on the device; the host
// reads one residual norm (and the cycle state) per restart.  BiCGSTAB keeps
// its scalars on the device and reads its stop flag every few iterations.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>

#include "../../include/ucfdsolver.h"
#include "graph.h"
#include "launch.h"
#include "ucfd_internal.h"

using namespace ucfd;

namespace {

cudaStream_t kstream() {
    static cudaStream_t s = nullptr;
    if (!s) {
        ensure_device();
        UCFD_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    }
    return s;
}

// Row-major CSR-of-blocks -> ELL-of-blocks (device).  The structure -- each
// ELL entry's column and the CSR slot whose block it holds -- is built on
// the host once; the values are gathered on the device from the caller's
// block array (ell_gather), so a new set of values costs one device pass.
struct EllBlocks {
    int bn = 0, B = 0, P = 0;
    DevBuf<int> col, src;
    DevBuf<double> val;
    DevBuf<float> val32;

    // rows: internal row k takes original row perm[k] (perm null: identity);
    // entries [first[k], last[k]) of that row; columns mapped through iperm.
    void build(int bn_, int B_, const std::vector<int> &rp, const std::vector<int> &ci, const int *perm,
               const int *iperm, const std::vector<int> *lo, const std::vector<int> *hi, cudaStream_t s) {
        bn = bn_;
        B = B_;
        P = 0;
        for (int k = 0; k < bn; ++k) {
            const int r = perm ? perm[k] : k;
            const int a = lo ? (*lo)[r] : rp[r], b = hi ? (*hi)[r] : rp[r + 1];
            P = std::max(P, b - a);
        }
        const size_t slots = (size_t)std::max(P, 1) * bn;
        std::vector<int> c(slots, -1), q(slots, -1);
        for (int k = 0; k < bn; ++k) {
            const int r = perm ? perm[k] : k;
            const int a = lo ? (*lo)[r] : rp[r], b = hi ? (*hi)[r] : rp[r + 1];
            for (int p = 0; p < b - a; ++p) {
                c[(size_t)p * bn + k] = iperm ? iperm[ci[a + p]] : ci[a + p];
                q[(size_t)p * bn + k] = a + p;
            }
        }
        col.upload(c.data(), c.size(), s);
        src.upload(q.data(), q.size(), s);
        UCFD_CUDA(cudaStreamSynchronize(s));
    }

    // Blocks of the caller's values (device, [nnzb][B][B]) into val (FP64)
    // and/or val32 (rounded to FP32).
    void gather(const double *vals, bool fp64, bool fp32, cudaStream_t s) {
        const size_t n = (size_t)std::max(P, 1) * B * B * bn;
        if (fp64) {
            val.ensure(n);
            kfast::ell_gather<double>(B, bn, P, src.p, vals, val.p, s);
        }
        if (fp32) {
            val32.ensure(n);
            kfast::ell_gather<float>(B, bn, P, src.p, vals, val32.p, s);
        }
    }
};

// Fingerprints (kargs.h fingerprint_mix) of up to three int arrays in host
// or device memory; arrays with n <= 0 give 0.
struct Fingerprint {
    unsigned long long h[3] = {0, 0, 0};
    bool operator==(const Fingerprint &o) const { return h[0] == o.h[0] && h[1] == o.h[1] && h[2] == o.h[2]; }
};

Fingerprint fingerprint_arrays(const int *const a[3], const long long n[3], DevBuf<unsigned long long> &acc,
                               cudaStream_t s) {
    Fingerprint f;
    bool any_dev = false;
    for (int j = 0; j < 3; ++j) {
        if (!a[j] || n[j] <= 0) continue;
        if (is_device_ptr(a[j])) {
            if (!any_dev) acc.zero(3, s);
            any_dev = true;
            kfast::fingerprint(n[j], a[j], acc.p + j, s);
        } else {
            for (long long i = 0; i < n[j]; ++i) f.h[j] += fingerprint_mix(i, a[j][i]);
        }
    }
    if (any_dev) {
        unsigned long long d[3];
        UCFD_CUDA(cudaMemcpyAsync(d, acc.p, sizeof d, cudaMemcpyDeviceToHost, s));
        UCFD_CUDA(cudaStreamSynchronize(s));
        for (int j = 0; j < 3; ++j)
            if (a[j] && n[j] > 0 && is_device_ptr(a[j])) f.h[j] = d[j];
    }
    return f;
}

// One int of a caller array (host or device).
int read_int(const int *p) {
    int v = 0;
    if (is_device_ptr(p)) UCFD_CUDA(cudaMemcpy(&v, p, sizeof v, cudaMemcpyDeviceToHost));
    else v = *p;
    return v;
}

}  // namespace

// ===========================================================================
// SpMat
// ===========================================================================
struct _SpMat {
    const char *type_name = nullptr;
    int bn = 0, blk = 0;
    int *rowptr = nullptr, *colidx = nullptr;
    double *values = nullptr;
    EllBlocks ell;
    bool ready = false;
    DevBuf<double> sx, sy;

    DevBuf<double> vstage;
    DevBuf<unsigned long long> fpacc;
    Fingerprint fp;
    int nnzb = -1;

    // Structure (host, validated) and values (device gather).  The structure
    // is rebuilt only when the fingerprints of rowptr / colidx differ from the
    // ones it was built from.
    void load(bool fp32) {
        cudaStream_t s = kstream();
        const int nnz_now = read_int(rowptr + bn);
        UCFD_REQUIRE(nnz_now >= 0, "rowptr[bn] = %d is negative", nnz_now);
        const int *arr[3] = {rowptr, colidx, nullptr};
        const long long len[3] = {(long long)bn + 1, (long long)nnz_now, 0};
        const Fingerprint f = fingerprint_arrays(arr, len, fpacc, s);
        if (!ready || nnz_now != nnzb || !(f == fp)) {
            std::vector<int> rp, ci;
            to_host(rowptr, (size_t)bn + 1, rp);
            UCFD_REQUIRE(rp[0] == 0, "rowptr[0] must be 0");
            for (int i = 0; i < bn; ++i) UCFD_REQUIRE(rp[i + 1] >= rp[i], "rowptr must be non-decreasing");
            to_host(colidx, (size_t)rp[bn], ci);
            for (size_t q = 0; q < ci.size(); ++q)
                UCFD_REQUIRE(ci[q] >= 0 && ci[q] < bn, "colidx[%zu] = %d out of range", q, ci[q]);
            ell.build(bn, blk, rp, ci, nullptr, nullptr, nullptr, nullptr, s);
            nnzb = rp[bn];
            fp = f;
        }
        const double *vd = device_view<double>(values, (size_t)nnzb * blk * blk, vstage, s);
        ell.gather(vd, true, fp32, s);
        UCFD_CHECK_LAUNCH();
        UCFD_CUDA(cudaStreamSynchronize(s));
        ready = true;
    }
    void ensure32() {
        if (!ell.val32.p) {
            const long long n = (long long)std::max(ell.P, 1) * blk * blk * bn;
            ell.val32.ensure(n);
            kfast::convert<double, float>(n, ell.val.p, ell.val32.p, kstream());
            UCFD_CHECK_LAUNCH();
            UCFD_CUDA(cudaStreamSynchronize(kstream()));
        }
    }
    // y = alpha A x + beta y on device vectors.  kind: UCFD_PREC_FP64 the
    // reference's arithmetic (separate multiply and add, bit-exact),
    // UCFD_PREC_FP64_FMA the same sums with fused multiply-adds (half the FP64
    // instructions), UCFD_PREC_FP32 FP32 values and accumulation.
    void mult(double alpha, const double *x, double beta, double *y, int kind, cudaStream_t s) {
        if (kind == UCFD_PREC_FP32) {
            ensure32();
            kfast::bsr_spmv<float, float>(blk, bn, ell.P, ell.col.p, ell.val32.p, alpha, x, beta, y, 0, s);
        } else if (kind == UCFD_PREC_FP64_FMA) {
            kfast::bsr_spmv<double, double>(blk, bn, ell.P, ell.col.p, ell.val.p, alpha, x, beta, y, 0, s);
        } else {
            kexact::bsr_spmv<double, double>(blk, bn, ell.P, ell.col.p, ell.val.p, alpha, x, beta, y, 0, s);
        }
    }
};

// ===========================================================================
// Precon
// ===========================================================================
struct _Precon {
    const char *type_name = nullptr;
    int *rowptr = nullptr, *colidx = nullptr, *diagslots = nullptr;
    double *values = nullptr;
    int bn = 0, blk = 0, ncolors = 0;
    int kind = 0;  // PC_BLUSGS (0), PC_BILU (1), PC_ILU (2) of kernels_krylov.cuh
    std::vector<int> icolors;
    bool colored = false, none = false;
    int prec = UCFD_PREC_FP64;
    bool prepared = false;
    Schedule sch;
    bool identity = true;
    DevBuf<int> perm;
    DevBuf<long long> dslot;
    EllBlocks L, U;
    DevBuf<double> LU64, tmp64;
    DevBuf<float> LU32, tmp32;
    DevBuf<double> stage_b;

    // Structure cache: built from rowptr / colidx / diagslots (and the
    // colours) at the first Prepare, rebuilt when their fingerprints change
    // or a Set call resets it.
    bool have_structure = false;
    Fingerprint fp;
    int nnzb = -1;
    DevBuf<unsigned long long> fpacc;
    DevBuf<int> d_rp, d_ci, d_ds, d_rows;  // ILU factorisation
    DevBuf<double> vstage;

    void build_structure(cudaStream_t s) {
        std::vector<int> rp, ci, ds;
        to_host(rowptr, (size_t)bn + 1, rp);
        UCFD_REQUIRE(rp[0] == 0, "rowptr[0] must be 0");
        for (int i = 0; i < bn; ++i) UCFD_REQUIRE(rp[i + 1] >= rp[i], "rowptr must be non-decreasing");
        to_host(colidx, (size_t)rp[bn], ci);
        to_host(diagslots, (size_t)bn, ds);
        for (size_t q = 0; q < ci.size(); ++q)
            UCFD_REQUIRE(ci[q] >= 0 && ci[q] < bn, "colidx[%zu] = %d out of range", q, ci[q]);
        for (int i = 0; i < bn; ++i) {
            UCFD_REQUIRE(ds[i] >= rp[i] && ds[i] < rp[i + 1], "diagslots[%d] = %d outside row %d", i, ds[i], i);
            UCFD_REQUIRE(ci[ds[i]] == i, "diagslots[%d] does not point at the diagonal block", i);
        }
        if (kind != 0) {
            // the ILU types pair "before the diagonal slot" with "lower row"
            for (int i = 0; i < bn; ++i)
                for (int q = rp[i]; q < rp[i + 1]; ++q)
                    UCFD_REQUIRE(q == ds[i] || (q < ds[i]) == (ci[q] < i),
                                 "row %d: an ILU preconditioner needs columns below the diagonal before its slot "
                                 "and columns above it after", i);
        }
        if (colored) {
            // colour c = rows [icolors[c], icolors[c+1]); no row may reference
            // another row of its own colour (otherwise the reference result
            // depends on thread timing)
            UCFD_REQUIRE((int)icolors.size() == ncolors + 1 && icolors[0] == 0 && icolors[ncolors] == bn,
                         "icolors must run from 0 to bn over ncolors+1 entries");
            std::vector<int> col(bn);
            for (int c = 0; c < ncolors; ++c) {
                UCFD_REQUIRE(icolors[c + 1] >= icolors[c], "icolors must be non-decreasing");
                for (int i = icolors[c]; i < icolors[c + 1]; ++i) col[i] = c;
            }
            sch = schedule_colored(bn, rp.data(), ci.data(), col.data());
        } else {
            sch = schedule_natural(bn, rp.data(), ci.data());
        }
        identity = true;
        for (int k = 0; k < bn; ++k)
            if (sch.perm[k] != k) identity = false;
        if (!identity) perm.upload(sch.perm.data(), bn, s);
        std::vector<int> lo(bn), mid(bn), hi(bn);
        for (int i = 0; i < bn; ++i) {
            lo[i] = rp[i];
            mid[i] = ds[i];
            hi[i] = ds[i] + 1;
        }
        std::vector<int> end(rp.begin() + 1, rp.end());
        const int *pm = identity ? nullptr : sch.perm.data();
        const int *ip = identity ? nullptr : sch.iperm.data();
        L.build(bn, blk, rp, ci, pm, ip, &lo, &mid, s);
        U.build(bn, blk, rp, ci, pm, ip, &hi, &end, s);
        std::vector<long long> dsl(ds.begin(), ds.end());
        dslot.upload(dsl.data(), bn, s);
        if (kind != 0) {
            d_rp.upload(rp.data(), rp.size(), s);
            d_ci.upload(ci.data(), ci.size(), s);
            d_ds.upload(ds.data(), ds.size(), s);
            d_rows.upload(sch.perm.data(), sch.perm.size(), s);
        }
        UCFD_CUDA(cudaStreamSynchronize(s));
        nnzb = rp[bn];
        have_structure = true;
    }

    void prepare() {
        if (none) {
            prepared = true;
            return;
        }
        UCFD_REQUIRE(bn > 0 && blk > 0, "preconditioner type not set (UCFDPreconSetBLUSGS / SetPBLUSGS)");
        cudaStream_t s = kstream();
        const int nnz_now = read_int(rowptr + bn);
        UCFD_REQUIRE(nnz_now >= 0, "rowptr[bn] = %d is negative", nnz_now);
        const int *arr[3] = {rowptr, colidx, diagslots};
        const long long len[3] = {(long long)bn + 1, (long long)nnz_now, (long long)bn};
        const Fingerprint f = fingerprint_arrays(arr, len, fpacc, s);
        if (!have_structure || nnz_now != nnzb || !(f == fp)) {
            have_structure = false;
            build_structure(s);
            fp = f;
        }
        const bool fp32 = prec == UCFD_PREC_FP32;
        const long long B2 = (long long)blk * blk;
        const size_t nv = (size_t)nnzb * B2;
        // the caller's values on the device (the ILU types factorise them in
        // place there and, for a host array, copy the factors back)
        const bool vdev = is_device_ptr(values);
        double *vd = values;
        if (!vdev) {
            vstage.upload(values, nv, s);
            vd = vstage.p;
        }
        if (kind != 0) {
            factorize(vd, s);
            if (!vdev) copy_d2h(values, vd, nv * sizeof(double), s);
        }
        L.gather(vd, !fp32, fp32, s);
        U.gather(vd, !fp32, fp32, s);
        LU64.ensure(B2 * bn);
        const int fac = kind == 0 ? 1 : 0;  // the ILU types arrive factored
        if (fp32) {
            LU32.ensure(B2 * bn);
            kfast::pc_prepare<float>(blk, bn, identity ? nullptr : perm.p, dslot.p, vd, LU64.p, LU32.p, fac, s);
        } else if (prec == UCFD_PREC_FP64) {
            kexact::pc_prepare<double>(blk, bn, identity ? nullptr : perm.p, dslot.p, vd, LU64.p, nullptr, fac, s);
        } else {
            kfast::pc_prepare<double>(blk, bn, identity ? nullptr : perm.p, dslot.p, vd, LU64.p, nullptr, fac, s);
        }
        UCFD_CHECK_LAUNCH();
        UCFD_CUDA(cudaStreamSynchronize(s));
        prepared = true;
    }

    // ILU(0) factorisation in place on the device values v (FP64), level by
    // level of the schedule (each row once its lower neighbours are final:
    // the sequential result).
    void factorize(double *v, cudaStream_t s) {
        const int scalar = kind == 2 ? 1 : 0;
        for (int l = 0; l < sch.nlev; ++l) {
            if (prec == UCFD_PREC_FP64)
                kexact::ilu_factor(blk, scalar, sch.lev_off[l], sch.lev_off[l + 1], d_rows.p, d_rp.p, d_ci.p, d_ds.p,
                                   v, s);
            else
                kfast::ilu_factor(blk, scalar, sch.lev_off[l], sch.lev_off[l + 1], d_rows.p, d_rp.p, d_ci.p, d_ds.p,
                                  v, s);
        }
        UCFD_CHECK_LAUNCH();
    }

    // In-place apply to a device vector b [bn*blk] (FP64).
    void apply(double *b, cudaStream_t s) {
        if (none) return;
        UCFD_REQUIRE(prepared, "UCFDPreconPrepare has not been called");
        const long long n = (long long)bn * blk;
        const int L_ = sch.nlev;
        if (prec == UCFD_PREC_FP32) {
            float *x = tmp32.ensure(n);
            kfast::gather_rows<double, float>(bn, blk, identity ? nullptr : perm.p, b, x, s);
            for (int l = 0; l < L_; ++l)
                kfast::pc_lower<float>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, L.P, L.col.p, L.val32.p, LU32.p, x,
                                       0, kind, s);
            for (int l = L_ - 1; l >= 0; --l)
                kfast::pc_upper<float>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, U.P, U.col.p, U.val32.p, LU32.p, x,
                                       0, kind, s);
            kfast::scatter_rows<float, double>(bn, blk, identity ? nullptr : perm.p, x, b, s);
        } else {
            double *x = b;
            if (!identity) {
                x = tmp64.ensure(n);
                kfast::gather_rows<double, double>(bn, blk, perm.p, b, x, s);
            }
            const bool ex = prec == UCFD_PREC_FP64;
            for (int l = 0; l < L_; ++l) {
                if (ex)
                    kexact::pc_lower<double>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, L.P, L.col.p, L.val.p,
                                             LU64.p, x, 0, kind, s);
                else
                    kfast::pc_lower<double>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, L.P, L.col.p, L.val.p,
                                            LU64.p, x, 0, kind, s);
            }
            for (int l = L_ - 1; l >= 0; --l) {
                if (ex)
                    kexact::pc_upper<double>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, U.P, U.col.p, U.val.p,
                                             LU64.p, x, 0, kind, s);
                else
                    kfast::pc_upper<double>(blk, sch.lev_off[l], sch.lev_off[l + 1], bn, U.P, U.col.p, U.val.p,
                                            LU64.p, x, 0, kind, s);
            }
            if (!identity) kfast::scatter_rows<double, double>(bn, blk, perm.p, x, b, s);
        }
    }
};

// ===========================================================================
// Solver (GMRES)
// ===========================================================================
struct _Solver {
    const char *type_name = nullptr;
    double tol = 1e-5, haptol = 1e-12;  // solver.c:10-11
    int maxiter = -1, itnum = 0;
    double residual = 0.0;
    int stat = INITIALIZED;
    bool trace = false;
    std::vector<double> hist;
    int n = 0, m = 0;
    int prec = UCFD_PREC_FP64;
    // mixed precision: a cycle ends when its residual estimate drops below
    // this fraction of the cycle's start (FP32 operator accuracy)
    double mixed_floor = 1e-6;
    // FP64 modes, on request: a cycle also ends once its residual estimate
    // has fallen by the factor the true residual still needs (x 0.1), instead
    // of always building m vectors (UCFDSolverSetCycleExit)
    bool cycle_exit = false;
    long long arnoldi = 0;
    long long ldv = 0;
    DevBuf<double> V, w, r, H, cs, sn, y, h2, part, abeta;
    DevBuf<unsigned char> st;
    DevBuf<double> sx, sb;
    PinnedBuf<double> h_abeta;
    PinnedBuf<unsigned char> h_st;
    // BiCGSTAB (bicgstab.h:6-9): r, r~, p, pt, v, s, shat, t, reductions, state
    bool bicg = false;
    DevBuf<double> br, brt, bp, bpt, bv, bs, bsh, bt, bpart, bhist;
    DevBuf<unsigned char> bst;
    PinnedBuf<unsigned char> h_bst;

    void alloc() {
        ldv = ((long long)n + 31) / 32 * 32;
        V.ensure((size_t)ldv * (m + 1));
        w.ensure(n);
        r.ensure(n);
        H.ensure((size_t)(m + 1) * m);
        cs.ensure(m + 1);
        sn.ensure(m + 1);
        y.ensure(m + 1);
        h2.ensure(m + 1);
        part.ensure((size_t)kfast::gm_blocks(n) * 32 + 64);
        abeta.ensure(2);
        st.ensure(kfast::gm_state_bytes());
        h_abeta.ensure(2);
        h_st.ensure(kfast::gm_state_bytes());
    }

    // bicgstab.c:24-128 on the device: every scalar lives in a device state
    // (kernels_krylov.cuh BcState); the host queues kChunk iterations between
    // its reads of the stop flag, the kernels of iterations queued after a
    // stop return at once (the preconditioner and matvec of those only touch
    // scratch vectors).
    void solve_bicgstab(SpMat A, Precon pc, double *x, const double *b, cudaStream_t s) {
        // iterations queued between two reads of the device stop flag: the
        // matvec and preconditioner of an iteration queued after convergence
        // still run, which costs more than a host read once n is large
        const long long nn = n;
        const int kChunk = nn >= (1ll << 20) ? 1 : 4;
        // the reference's products (bit-exact) unless the solver runs with FMA
        const int mk = prec == UCFD_PREC_FP64_FMA ? UCFD_PREC_FP64_FMA : UCFD_PREC_FP64;
        const int nb = kfast::gm_blocks(nn);
        for (DevBuf<double> *v : {&br, &brt, &bp, &bpt, &bv, &bs, &bsh, &bt}) v->ensure((size_t)n);
        bpart.ensure((size_t)5 * nb);
        bst.ensure(kfast::bc_state_bytes());
        h_bst.ensure(kfast::bc_state_bytes());
        double *hist_d = nullptr;
        if (trace && maxiter > 0) {
            hist.assign(maxiter, 0.0);
            hist_d = bhist.ensure((size_t)maxiter);
            UCFD_CUDA(cudaMemsetAsync(hist_d, 0, (size_t)maxiter * sizeof(double), s));
        }
        // r = b - A x, r~ = r, rho = (r~, r)
        UCFD_CUDA(cudaMemcpyAsync(br.p, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        A->mult(-1.0, x, 1.0, br.p, mk, s);
        UCFD_CUDA(cudaMemcpyAsync(brt.p, br.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        kfast::bc_dot(nn, brt.p, br.p, bpart.p, nullptr, s);
        kfast::bc_start(nb, bpart.p, bst.p, maxiter, s);
        struct HostState {
            double rho, rhoprev, alpha, omega, rho_new, resnorm;
            int iter, stop, stat, conv;
        };
        static_assert(sizeof(HostState) == 64, "device state layout");
        HostState h{};
        int queued = 0;
        for (;;) {
            for (int q = 0; q < kChunk && queued < maxiter; ++q, ++queued) {
                kfast::bc_direction(nn, bst.p, br.p, bv.p, bp.p, bpt.p, s);
                pc->apply(bpt.p, s);
                A->mult(1.0, bpt.p, 0.0, bv.p, mk, s);
                kfast::bc_dot(nn, brt.p, bv.p, bpart.p, bst.p, s);
                kfast::bc_alpha(nb, bpart.p, bst.p, s);
                kfast::bc_s(nn, bst.p, br.p, bv.p, bs.p, bsh.p, s);
                pc->apply(bsh.p, s);
                A->mult(1.0, bsh.p, 0.0, bt.p, mk, s);
                kfast::bc_fused5(nn, brt.p, bs.p, bt.p, bpart.p, bst.p, s);
                kfast::bc_omega(nb, bpart.p, bst.p, tol, hist_d, s);
                kfast::bc_update(nn, bst.p, bpt.p, bsh.p, bs.p, bt.p, x, br.p, s);
                kfast::bc_advance(bst.p, maxiter, s);
            }
            UCFD_CHECK_LAUNCH();
            UCFD_CUDA(cudaMemcpyAsync(h_bst.p, bst.p, sizeof(HostState), cudaMemcpyDeviceToHost, s));
            UCFD_CUDA(cudaStreamSynchronize(s));
            std::memcpy(&h, h_bst.p, sizeof(HostState));
            if (h.stop || queued >= maxiter) break;
        }
        itnum = h.iter;
        residual = h.resnorm;
        stat = h.stat;
        if (h.iter == maxiter) stat = REACH_ITERMAX;
        if (hist_d)
            UCFD_CUDA(cudaMemcpy(hist.data(), hist_d, (size_t)maxiter * sizeof(double), cudaMemcpyDeviceToHost));
    }

    // gmres.c:42-129 on the device.
    void solve(SpMat A, Precon pc, double *x, const double *b, cudaStream_t s) {
        if (bicg) {
            solve_bicgstab(A, pc, x, b, s);
            return;
        }
        const int ld = m + 1;
        const int nb = kfast::gm_blocks(n);
        const bool mixed = prec == UCFD_PREC_FP32;
        UCFD_CUDA(cudaMemsetAsync(st.p, 0, kfast::gm_state_bytes(), s));
        int iter = 0;
        double ab = 0.0;
        bool breakdown = false;
        if (trace) hist.assign(std::max(maxiter, 0), 0.0);
        stat = INITIALIZED;
        while (iter < maxiter) {
            // r = b - A x, abeta = ||r||  (true residual, FP64 values; with FMA in
            // the FMA and mixed modes, which are not bit-matched to the reference)
            UCFD_CUDA(cudaMemcpyAsync(r.p, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            A->mult(-1.0, x, 1.0, r.p, prec == UCFD_PREC_FP64 ? UCFD_PREC_FP64 : UCFD_PREC_FP64_FMA, s);
            kfast::norm2_to(n, r.p, part.p, abeta.p, s);
            UCFD_CUDA(cudaMemcpyAsync(h_abeta.p, abeta.p, sizeof(double), cudaMemcpyDeviceToHost, s));
            UCFD_CUDA(cudaStreamSynchronize(s));
            ab = h_abeta.p[0];
            if (trace && iter < (int)hist.size()) hist[iter] = ab;
            if (ab <= tol) {
                stat = CONVERGED;
                break;
            }
            // the cycle's floor on its (preconditioned) residual estimate,
            // relative to the cycle's start
            const double floor = mixed ? mixed_floor : cycle_exit ? std::min(0.5, 0.1 * tol / ab) : 0.0;
            pc->apply(r.p, s);
            kfast::gm_sumsq(n, r.p, part.p, s);
            kfast::gm_cycle_begin(nb, part.p, st.p, y.p, nullptr, s);
            kfast::gm_scale(n, st.p, r.p, V.p, s);
            for (int j = 0; j < m; ++j) {
                const double *vj = V.p + (size_t)j * ldv;
                A->mult(1.0, vj, 0.0, w.p, prec, s);
                pc->apply(w.p, s);
                const int K = j + 1;
                double *Hc = H.p + (size_t)j * ld;
                kfast::gm_dots(n, K, V.p, ldv, w.p, part.p, s);
                kfast::gm_reduce(nb, K, part.p, Hc, 0, s);
                kfast::gm_update(n, K, V.p, ldv, Hc, w.p, 0, part.p, s);
                kfast::gm_reduce(nb, K, part.p, h2.p, 0, s);
                kfast::gm_update(n, K, V.p, ldv, h2.p, w.p, 1, part.p, s);
                kfast::gm_givens(j, ld, nb, part.p, H.p, h2.p, cs.p, sn.p, y.p, haptol, floor, st.p, s);
                kfast::gm_scale(n, st.p, w.p, V.p + (size_t)(j + 1) * ldv, s);
                if (floor > 0.0) {
                    // an FP32 operator cannot resolve the cycle below its floor: stop
                    // launching once the device reports it (one host read per step)
                    UCFD_CUDA(cudaMemcpyAsync(h_st.p, st.p, kfast::gm_state_bytes(), cudaMemcpyDeviceToHost, s));
                    UCFD_CUDA(cudaStreamSynchronize(s));
                    if (((const int *)h_st.p)[1]) break;
                }
            }
            kfast::gm_backsub(ld, H.p, y.p, st.p, s);
            kfast::gm_solution(n, V.p, ldv, y.p, st.p, x, s);
            UCFD_CHECK_LAUNCH();
            UCFD_CUDA(cudaMemcpyAsync(h_st.p, st.p, kfast::gm_state_bytes(), cudaMemcpyDeviceToHost, s));
            UCFD_CUDA(cudaStreamSynchronize(s));
            const int *sti = (const int *)h_st.p;  // {k, stop, total}
            if (sti[1] == 1) breakdown = true;
            arnoldi = sti[2];
            iter++;
        }
        if (iter == maxiter) stat = REACH_ITERMAX;
        else if (stat != CONVERGED && breakdown) stat = HAPPYBREAKDOWN;
        residual = ab;
        itnum = iter;
    }
};

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

// ---- SpMat -------------------------------------------------------------------
ucfd_status_t UCFDMatInit(SpMat *mat) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mat, "null SpMat pointer");
    *mat = new _SpMat();
    UCFD_API_END
}

ucfd_status_t UCFDMatDestroy(SpMat *mat) {
    UCFD_API_BEGIN
    if (!mat || !*mat) return UCFD_SUCCESS;
    delete *mat;
    *mat = nullptr;
    UCFD_API_END
}

static ucfd_status_t mat_create(SpMat *mat, const char *type, UCFDInt bn, UCFDInt blk, UCFDInt *rowptr,
                                UCFDInt *colidx, UCFDReal *values) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mat, "null SpMat pointer");
    UCFD_REQUIRE(bn > 0 && blk > 0 && blk <= 7, "bad sizes bn=%d blk=%d (blk 1..7)", bn, blk);
    UCFD_REQUIRE(rowptr && colidx && values, "null matrix array");
    std::unique_ptr<_SpMat> m(new _SpMat());
    m->type_name = type;
    m->bn = bn;
    m->blk = blk;
    m->rowptr = rowptr;
    m->colidx = colidx;
    m->values = values;
    m->load(false);
    *mat = m.release();
    UCFD_API_END
}

ucfd_status_t UCFDMatCreateCSR(SpMat *mat, UCFDInt n, UCFDInt *rowptr, UCFDInt *colidx, UCFDReal *values) {
    return mat_create(mat, CSR, n, 1, rowptr, colidx, values);
}
ucfd_status_t UCFDMatCreateBSR(SpMat *mat, UCFDInt bn, UCFDInt blk, UCFDInt *rowptr, UCFDInt *colidx,
                               UCFDReal *values) {
    return mat_create(mat, BSR, bn, blk, rowptr, colidx, values);
}
ucfd_status_t UCFDMatCreateCUDACSR(SpMat *mat, UCFDInt n, UCFDInt *rowptr, UCFDInt *colidx, UCFDReal *values) {
    return mat_create(mat, CSRCUDA, n, 1, rowptr, colidx, values);
}
ucfd_status_t UCFDMatCreateCUDABSR(SpMat *mat, UCFDInt bn, UCFDInt blk, UCFDInt *rowptr, UCFDInt *colidx,
                                   UCFDReal *values) {
    return mat_create(mat, BSRCUDA, bn, blk, rowptr, colidx, values);
}

ucfd_status_t UCFDMatUpdateValues(SpMat mat) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mat && mat->type_name, "matrix not created");
    const bool had32 = mat->ell.val32.p != nullptr;
    mat->load(had32);
    UCFD_API_END
}

ucfd_status_t UCFDMatGetType(SpMat mat, const char **type_name) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mat && type_name, "null argument");
    *type_name = mat->type_name;
    UCFD_API_END
}

static ucfd_status_t mat_mult(UCFDReal alpha, SpMat mat, UCFDReal *x, UCFDReal beta, UCFDReal *y, int prec) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(mat && mat->type_name && mat->ready, "Matrix type must be set");
    UCFD_REQUIRE(x && y, "null vector");
    cudaStream_t s = kstream();
    const size_t n = (size_t)mat->bn * mat->blk;
    const double *xd = device_view<double>(x, n, mat->sx, s);
    const bool ydev = is_device_ptr(y);
    double *yd = ydev ? y : const_cast<double *>(device_view<double>(y, n, mat->sy, s));
    mat->mult(alpha, xd, beta, yd, prec, s);
    UCFD_CHECK_LAUNCH();
    if (!ydev) copy_d2h(y, yd, n * sizeof(double), s);
    UCFD_CUDA(cudaStreamSynchronize(s));
    UCFD_API_END
}

ucfd_status_t UCFDMatMult(UCFDReal alpha, SpMat mat, UCFDReal *x, UCFDReal beta, UCFDReal *y) {
    return mat_mult(alpha, mat, x, beta, y, UCFD_PREC_FP64);
}
ucfd_status_t UCFDMatMultFP32(UCFDReal alpha, SpMat mat, UCFDReal *x, UCFDReal beta, UCFDReal *y) {
    return mat_mult(alpha, mat, x, beta, y, UCFD_PREC_FP32);
}
ucfd_status_t UCFDMatMultPrecision(UCFDReal alpha, SpMat mat, UCFDReal *x, UCFDReal beta, UCFDReal *y,
                                   int precision) {
    if (precision != UCFD_PREC_FP64 && precision != UCFD_PREC_FP64_FMA && precision != UCFD_PREC_FP32) {
        ucfd::set_error("UCFDMatMultPrecision: unknown precision %d", precision);
        return UCFD_ERR_ARGUMENT;
    }
    return mat_mult(alpha, mat, x, beta, y, precision);
}

// ---- Precon ------------------------------------------------------------------
ucfd_status_t UCFDPreconCreatefromArrays(Precon *pc, UCFDInt *rowptr, UCFDInt *colidx, UCFDInt *diagslots,
                                         UCFDReal *values) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc, "null Precon pointer");
    UCFD_REQUIRE(rowptr && colidx && diagslots && values, "null preconditioner array");
    std::unique_ptr<_Precon> p(new _Precon());
    p->rowptr = rowptr;
    p->colidx = colidx;
    p->diagslots = diagslots;
    p->values = values;
    *pc = p.release();
    UCFD_API_END
}

ucfd_status_t UCFDPreconCreateNone(Precon *pc) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc, "null Precon pointer");
    std::unique_ptr<_Precon> p(new _Precon());
    p->type_name = NONE;
    p->none = true;
    *pc = p.release();
    UCFD_API_END
}

ucfd_status_t UCFDPreconDestroy(Precon *pc) {
    UCFD_API_BEGIN
    if (!pc || !*pc) return UCFD_SUCCESS;
    delete *pc;
    *pc = nullptr;
    UCFD_API_END
}

static ucfd_status_t pc_set(Precon *pc, const char *type, UCFDInt bn, UCFDInt block, UCFDInt ncolors,
                            UCFDInt *icolors) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc && *pc, "Preconditioner must be initialized");
    UCFD_REQUIRE(bn > 0 && block > 0 && block <= 7, "bad sizes bn=%d block=%d", bn, block);
    Precon p = *pc;
    p->type_name = type;
    p->kind = 0;
    p->bn = bn;
    p->blk = block;
    p->colored = icolors != nullptr;
    if (icolors) {
        UCFD_REQUIRE(ncolors > 0, "ncolors must be positive");
        to_host(icolors, (size_t)ncolors + 1, p->icolors);
        p->ncolors = ncolors;
    }
    p->prepared = false;
    p->have_structure = false;
    UCFD_API_END
}

ucfd_status_t UCFDPreconSetBLUSGS(Precon *pc, UCFDInt bn, UCFDInt block) {
    return pc_set(pc, BLUSGS, bn, block, 0, nullptr);
}
ucfd_status_t UCFDPreconSetPBLUSGS(Precon *pc, UCFDInt bn, UCFDInt block, UCFDInt ncolors, UCFDInt *icolors) {
    if (!icolors) return UCFD_ERR_ARGUMENT;
    return pc_set(pc, PBLUSGS, bn, block, ncolors, icolors);
}
ucfd_status_t UCFDPreconSetCUDABLUSGS(Precon *pc, UCFDInt bn, UCFDInt block, UCFDInt ncolors, UCFDInt *icolors) {
    if (!icolors) return UCFD_ERR_ARGUMENT;
    return pc_set(pc, CUDABLUSGS, bn, block, ncolors, icolors);
}

static ucfd_status_t pc_set_ilu(Precon *pc, const char *type, int kind, UCFDInt bn, UCFDInt block,
                                UCFDInt ncolors, UCFDInt *icolors) {
    const ucfd_status_t st = pc_set(pc, type, bn, block, ncolors, icolors);
    if (st == UCFD_SUCCESS) (*pc)->kind = kind;
    return st;
}
ucfd_status_t UCFDPreconSetILU(Precon *pc, UCFDInt n) { return pc_set_ilu(pc, ILU, 2, n, 1, 0, nullptr); }
ucfd_status_t UCFDPreconSetBILU(Precon *pc, UCFDInt bn, UCFDInt block) {
    return pc_set_ilu(pc, BILU, 1, bn, block, 0, nullptr);
}
ucfd_status_t UCFDPreconSetPBILU(Precon *pc, UCFDInt bn, UCFDInt block, UCFDInt ncolors, UCFDInt *icolors) {
    if (!icolors) return UCFD_ERR_ARGUMENT;
    return pc_set_ilu(pc, PBILU, 1, bn, block, ncolors, icolors);
}
ucfd_status_t UCFDPreconSetCUDABILU(Precon *pc, UCFDInt bn, UCFDInt block, UCFDInt ncolors, UCFDInt *icolors) {
    if (!icolors) return UCFD_ERR_ARGUMENT;
    return pc_set_ilu(pc, CUDABILU, 1, bn, block, ncolors, icolors);
}

ucfd_status_t UCFDPreconSetPrecision(Precon pc, int precision) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc, "null Precon");
    UCFD_REQUIRE(precision == UCFD_PREC_FP64 || precision == UCFD_PREC_FP64_FMA || precision == UCFD_PREC_FP32,
                 "unknown precision %d", precision);
    pc->prec = precision;
    pc->prepared = false;
    UCFD_API_END
}

ucfd_status_t UCFDPreconPrepare(Precon pc) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc && pc->type_name, "Preconditioner type must be set");
    pc->prepare();
    UCFD_API_END
}

ucfd_status_t UCFDPreconGetLevels(Precon pc, UCFDInt *nlevels) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc && nlevels, "null argument");
    UCFD_REQUIRE(pc->prepared, "UCFDPreconPrepare has not been called");
    *nlevels = pc->sch.nlev;
    UCFD_API_END
}

ucfd_status_t UCFDPreconApply(Precon pc, UCFDReal *b) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(pc && pc->type_name, "Preconditioner type must be set");
    UCFD_REQUIRE(b, "null vector");
    if (pc->none) return UCFD_SUCCESS;
    cudaStream_t s = kstream();
    const size_t n = (size_t)pc->bn * pc->blk;
    const bool dev = is_device_ptr(b);
    double *bd = dev ? b : const_cast<double *>(device_view<double>(b, n, pc->stage_b, s));
    pc->apply(bd, s);
    UCFD_CHECK_LAUNCH();
    if (!dev) copy_d2h(b, bd, n * sizeof(double), s);
    UCFD_CUDA(cudaStreamSynchronize(s));
    UCFD_API_END
}

// ---- Solver ------------------------------------------------------------------
ucfd_status_t UCFDSolverInit(Solver *solver) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver pointer");
    *solver = new _Solver();
    UCFD_API_END
}

ucfd_status_t UCFDSolverDestroy(Solver *solver) {
    UCFD_API_BEGIN
    if (!solver || !*solver) return UCFD_SUCCESS;
    delete *solver;
    *solver = nullptr;
    UCFD_API_END
}

static ucfd_status_t gmres_create(Solver *solver, UCFDInt n, UCFDInt m, UCFDInt maxiter, UCFDReal tol) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver pointer");
    UCFD_REQUIRE(n > 0 && m > 0 && m < 32 && maxiter >= 0, "bad GMRES sizes n=%d m=%d (m < 32) maxiter=%d", n, m,
                 maxiter);
    ensure_device();
    std::unique_ptr<_Solver> s(new _Solver());
    s->type_name = GMRES;
    s->n = n;
    s->m = m;
    s->maxiter = maxiter;
    s->tol = tol;
    s->alloc();
    *solver = s.release();
    UCFD_API_END
}

ucfd_status_t UCFDSolverCreateGMRES(Solver *solver, UCFDInt n, UCFDInt m, UCFDInt maxiter, UCFDReal tol) {
    return gmres_create(solver, n, m, maxiter, tol);
}

ucfd_status_t UCFDSolverCreateBICGSTAB(Solver *solver, UCFDInt n, UCFDInt maxiter, UCFDReal tol) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver pointer");
    UCFD_REQUIRE(n > 0 && maxiter >= 0, "bad BiCGSTAB sizes n=%d maxiter=%d", n, maxiter);
    ensure_device();
    std::unique_ptr<_Solver> s(new _Solver());
    s->type_name = BICGSTAB;
    s->bicg = true;
    s->n = n;
    s->maxiter = maxiter;
    s->tol = tol;
    *solver = s.release();
    UCFD_API_END
}
ucfd_status_t UCFDSolverCreateCUDAGMRES(Solver *solver, UCFDInt n, UCFDInt m, UCFDInt maxiter, UCFDReal tol) {
    return gmres_create(solver, n, m, maxiter, tol);
}

ucfd_status_t UCFDSolverSetPrecision(Solver solver, int precision) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver");
    UCFD_REQUIRE(precision == UCFD_PREC_FP64 || precision == UCFD_PREC_FP64_FMA || precision == UCFD_PREC_FP32,
                 "unknown precision %d", precision);
    solver->prec = precision;
    UCFD_API_END
}

ucfd_status_t UCFDSolverSetHappyTol(Solver solver, UCFDReal haptol) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver");
    solver->haptol = haptol;
    UCFD_API_END
}

ucfd_status_t UCFDSolverSetCycleExit(Solver solver, int on) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver");
    solver->cycle_exit = on != 0;
    UCFD_API_END
}

ucfd_status_t UCFDSolve(Solver solver, Precon pc, SpMat A, UCFDReal *x, UCFDReal *b) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver && solver->type_name, "Solver must be initialized");
    UCFD_REQUIRE(pc && pc->type_name, "Preconditioner must be initialized");
    UCFD_REQUIRE(A && A->type_name && A->ready, "Matrix must be constructed");
    UCFD_REQUIRE(x && b, "null vector");
    UCFD_REQUIRE((long long)A->bn * A->blk == solver->n, "matrix size %lld != solver size %d",
                 (long long)A->bn * A->blk, solver->n);
    if (!pc->none) {
        UCFD_REQUIRE(pc->bn == A->bn && pc->blk == A->blk, "preconditioner and matrix sizes differ");
        if (!pc->prepared) pc->prepare();
    }
    cudaStream_t s = kstream();
    const size_t n = solver->n;
    const bool xdev = is_device_ptr(x);
    double *xd = xdev ? x : const_cast<double *>(device_view<double>(x, n, solver->sx, s));
    const double *bd = device_view<double>(b, n, solver->sb, s);
    solver->solve(A, pc, xd, bd, s);
    if (!xdev) copy_d2h(x, xd, n * sizeof(double), s);
    UCFD_CUDA(cudaStreamSynchronize(s));
    UCFD_API_END
}

ucfd_status_t UCFDSolverGetResult(Solver solver, UCFDInt *stat, UCFDInt *iter, UCFDReal *residual) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver");
    if (stat) *stat = solver->stat;
    if (iter) *iter = solver->itnum;
    if (residual) *residual = solver->residual;
    UCFD_API_END
}

ucfd_status_t UCFDSolverGetArnoldiSteps(Solver solver, UCFDInt *steps) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver && steps, "null argument");
    *steps = (UCFDInt)solver->arnoldi;
    UCFD_API_END
}

ucfd_status_t UCFDSolverTraceResidualHistory(Solver solver) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver, "null Solver");
    solver->trace = true;
    solver->hist.assign(std::max(solver->maxiter, 0), 0.0);
    UCFD_API_END
}

ucfd_status_t UCFDSolverGetResidualHistory(Solver solver, UCFDReal *hist) {
    UCFD_API_BEGIN
    UCFD_REQUIRE(solver && hist, "null argument");
    UCFD_REQUIRE(solver->trace, "Tracing residual unset");
    std::memcpy(hist, solver->hist.data(), solver->hist.size() * sizeof(double));
    UCFD_API_END
}

}  // extern "C"
