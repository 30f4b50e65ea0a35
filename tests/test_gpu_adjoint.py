"""The hand-written adjoint of one colored LU-SGS step.

Forward: bit-identical to the oracle's colored step.  Backward: gradients
with respect to rhs, dt and fspr against central finite differences of the
FP64 oracle (h = 1e-6, relative agreement 1e-6), a dot-product test of the
transposed sweeps, torch.autograd.gradcheck, and FP32 against FP64."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

FD_H = 1e-6
FD_REL = 1e-6


def setup(m=6, jitter=0.2, permute=True, seed=0):
    from ucfd_sparse_gb300 import meshgen as mg
    from ucfd_sparse_gb300.adjoint import ColoredMesh
    c = mg.lusgs_case(m, jitter=jitter, permute=permute, seed=seed)
    icolor, ranges, lcolor = mg.greedy_coloring_np(c["nei_ele"])
    c["lcolor"] = lcolor.astype(np.int32)
    mesh = ColoredMesh(c["nei_ele"], c["fnorm_vol"], c["vec_fnorm"], icolor, ranges)
    return c, icolor.astype(np.int32), [int(r) for r in ranges], mesh


def T(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda().to(dtype)


def oracle_dq(port, c, icolor, ranges, rhs, dt, fspr):
    cc = dict(c, rhs=rhs, dt=dt, fspr=fspr)
    up, rhs_out, dub, diag = port.legacy_step(cc, icolor, ranges, c["lcolor"], nsteps=1)
    return rhs_out  # dQ after the upper sweep


def test_forward_bitexact(port, ucfd):
    from ucfd_sparse_gb300.adjoint import lusgs_step
    c, icolor, ranges, mesh = setup()
    dq = lusgs_step(T(c["rhs"]), T(c["dt"]), T(c["fspr"]), mesh, T(c["upts"]))
    ref = oracle_dq(port, c, icolor, ranges, c["rhs"], c["dt"], c["fspr"])
    np.testing.assert_array_equal(dq.cpu().numpy(), ref)


def test_gradients_match_central_differences(port, ucfd):
    from ucfd_sparse_gb300.adjoint import lusgs_step
    c, icolor, ranges, mesh = setup(m=6, seed=3)
    rng = np.random.default_rng(11)
    g = rng.standard_normal(c["rhs"].shape)
    rhs, dt, fspr = (T(c[k]).requires_grad_() for k in ("rhs", "dt", "fspr"))
    dq = lusgs_step(rhs, dt, fspr, mesh, T(c["upts"]))
    (dq * T(g)).sum().backward()
    grads = {"rhs": rhs.grad.cpu().numpy(), "dt": dt.grad.cpu().numpy(), "fspr": fspr.grad.cpu().numpy()}
    base = {k: c[k] for k in ("rhs", "dt", "fspr")}
    for name in ("rhs", "dt", "fspr"):
        for trial in range(3):
            v = rng.standard_normal(base[name].shape) * np.abs(base[name])   # relative perturbation direction
            args_p = dict(base)
            args_m = dict(base)
            args_p[name] = base[name] + FD_H * v
            args_m[name] = base[name] - FD_H * v
            lp = float((oracle_dq(port, c, icolor, ranges, **args_p) * g).sum())
            lm = float((oracle_dq(port, c, icolor, ranges, **args_m) * g).sum())
            fd = (lp - lm) / (2 * FD_H)
            ad = float((grads[name] * v).sum())
            assert abs(ad - fd) <= FD_REL * max(abs(fd), 1e-30), (name, trial, ad, fd)


def test_dot_product_transpose(ucfd):
    """<J^T g, v> == <g, J v>, J v by central differences of the GPU forward."""
    from ucfd_sparse_gb300.adjoint import lusgs_step
    c, icolor, ranges, mesh = setup(m=5, seed=5)
    rng = np.random.default_rng(2)
    g = T(rng.standard_normal(c["rhs"].shape))
    up = T(c["upts"])
    x = {k: T(c[k]) for k in ("rhs", "dt", "fspr")}
    v = {k: T(rng.standard_normal(c[k].shape) * np.abs(c[k])) for k in x}
    xs = {k: x[k].clone().requires_grad_() for k in x}
    (lusgs_step(xs["rhs"], xs["dt"], xs["fspr"], mesh, up) * g).sum().backward()
    lhs = sum(float((xs[k].grad * v[k]).sum()) for k in x)
    h = 1e-6
    fp = lusgs_step(*(x[k] + h * v[k] for k in ("rhs", "dt", "fspr")), mesh, up)
    fm = lusgs_step(*(x[k] - h * v[k] for k in ("rhs", "dt", "fspr")), mesh, up)
    rhs_ = float((g * (fp - fm)).sum()) / (2 * h)
    assert abs(lhs - rhs_) <= 1e-7 * abs(rhs_)


def test_gradcheck_small(ucfd):
    from ucfd_sparse_gb300.adjoint import lusgs_step
    c, icolor, ranges, mesh = setup(m=3, seed=7)
    up = T(c["upts"])
    rhs, dt, fspr = (T(c[k]).requires_grad_() for k in ("rhs", "dt", "fspr"))
    f = lambda r, d, s: lusgs_step(r, d, s, mesh, up)
    assert torch.autograd.gradcheck(f, (rhs, dt, fspr), eps=1e-6, atol=1e-7, rtol=1e-5)


def test_fp32_gradients_track_fp64(ucfd):
    from ucfd_sparse_gb300.adjoint import lusgs_step
    c, icolor, ranges, mesh = setup(m=8, seed=9)
    g = np.random.default_rng(4).standard_normal(c["rhs"].shape)
    out = {}
    for dt_ in (torch.float64, torch.float32):
        xs = {k: T(c[k], dt_).requires_grad_() for k in ("rhs", "dt", "fspr")}
        (lusgs_step(xs["rhs"], xs["dt"], xs["fspr"], mesh, T(c["upts"], dt_)) * T(g, dt_)).sum().backward()
        out[dt_] = {k: xs[k].grad.double().cpu().numpy() for k in xs}
    for k in ("rhs", "dt", "fspr"):
        a, b = out[torch.float32][k], out[torch.float64][k]
        assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max(), k
