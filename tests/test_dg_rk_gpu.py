"""Runge-Kutta stages and LSRK(5,4) time steps of the DG advection operator
on the GPU (through the C ABI) against the reference's own do_rk_stage /
do_time_step (golden vectors), the oracle, and the exact travelling wave."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.gpu_util import FP32_TOL, FP64_TOL, rel, to_dev, to_np, torch_cuda

pytestmark = pytest.mark.gpu
VEL = (1.0, 0.15, -0.05)


def _sf():
    from sum_factorization_kernels_gb300 import sfgpu
    return sfgpu


def _op(sf, g, p):
    nc = tuple(int(v) for v in g["nc_%d" % p])
    h = g["h_%d" % p]
    return sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=nc,
                       length=tuple(float(n) * float(hh) for n, hh in zip(nc, h)),
                       velocity=VEL, inverse_mass=1)


@pytest.mark.parametrize("p", [1, 2, 4, 5])
@pytest.mark.parametrize("case", ["a", "b"])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_rk_stage_golden(golden, p, case, prec):
    """one fused stage, distinct vectors and then with upd aliasing the
    output that do_time_step aliases it with"""
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_rk.npz")
    op = _op(sf, g, p)
    dt = torch.float64 if prec == "fp64" else torch.float32
    tol = FP64_TOL if prec == "fp64" else 4 * FP32_TOL[p]
    c_np, c_tm = (float(v) for v in g["c_%s_%d" % (case, p)])
    src = to_dev(torch, g["src_%d" % p], dt)
    upd = to_dev(torch, g["upd_%d" % p], dt)
    vnp = torch.full_like(src, float("nan"))
    vtm = to_dev(torch, g["tm0_%d" % p], dt)
    op.rk_stage(src, upd, vnp, vtm, c_np, c_tm)
    assert rel(to_np(vnp), g["np_%s_%d" % (case, p)]) < tol
    assert rel(to_np(vtm), g["tm_%s_%d" % (case, p)]) < tol  # untouched when c_tm == 0
    u = to_dev(torch, g["upd_%d" % p], dt)
    if case == "a":   # upd is vec_tm (stages 2 and 3 of do_time_step)
        op.rk_stage(src, u, vnp, u, c_np, c_tm)
        assert rel(to_np(u), g["tm_a_%d" % p]) < tol
    else:             # upd is vec_np (stage 5)
        op.rk_stage(src, u, u, None, c_np, c_tm)
        assert rel(to_np(u), g["np_b_%d" % p]) < tol
    assert op.device_status() == 0


@pytest.mark.parametrize("p", [1, 2, 4, 5])
def test_lsrk_steps_golden(golden, p):
    """three LSRK(5,4) steps against the reference's do_time_step"""
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_rk.npz")
    op = _op(sf, g, p)
    ref = g["steps3_%d" % p]
    for prec, dt, tol in (("fp64", torch.float64, FP64_TOL), ("fp32", torch.float32, 20 * FP32_TOL[p])):
        x = to_dev(torch, g["x0_%d" % p], dt)
        old, tmp = torch.zeros_like(x), torch.zeros_like(x)
        for _ in range(3):
            op.lsrk_step(x, old, tmp, float(g["dt_%d" % p]))
        assert rel(to_np(x), ref) < tol, prec
    assert op.device_status() == 0


def test_rk_stage_batched_and_errors(golden):
    """8 right-hand sides in one launch equal 8 single stages; invalid
    aliasing and operator kinds are rejected with a status"""
    torch = torch_cuda()
    sf = _sf()
    g = golden("dg_rk.npz")
    p = 4
    op = _op(sf, g, p)
    N = op.n_dofs
    gen = torch.Generator(device="cuda:0").manual_seed(3)
    src = torch.rand(8 * N, dtype=torch.float64, device="cuda:0", generator=gen) - 0.5
    upd = torch.rand(8 * N, dtype=torch.float64, device="cuda:0", generator=gen) - 0.5
    vnp, vtm = torch.empty_like(src), torch.empty_like(src)
    op.rk_stage(src, upd, vnp, vtm, 0.02, -0.01, nrhs=8)
    for r in range(8):
        s_ = slice(r * N, (r + 1) * N)
        a, b = torch.empty(N, dtype=torch.float64, device="cuda:0"), torch.empty(N, dtype=torch.float64,
                                                                                device="cuda:0")
        op.rk_stage(src[s_].contiguous(), upd[s_].contiguous(), a, b, 0.02, -0.01)
        assert float((vnp[s_] - a).abs().max()) == 0.0
        assert float((vtm[s_] - b).abs().max()) == 0.0
    with pytest.raises(sf.SFError):
        op.rk_stage(src, upd, src, vtm, 0.02, -0.01, nrhs=8)      # src written
    with pytest.raises(sf.SFError):
        op.rk_stage(src, upd, vnp, vnp, 0.02, -0.01, nrhs=8)      # vec_np == vec_tm
    with pytest.raises(sf.SFError):
        op.lsrk_step(vnp, vnp, vtm, 0.01, nrhs=8)                 # registers must differ
    # partial overlaps (views one right-hand side apart in one buffer)
    big = torch.zeros(10 * N, dtype=torch.float64, device="cuda:0")
    for call in (lambda: op.rk_stage(src, upd, big[:8 * N], big[N:9 * N], 0.02, -0.01, nrhs=8),
                 lambda: op.rk_stage(big[N:9 * N], upd, big[:8 * N], vtm, 0.02, -0.01, nrhs=8),
                 lambda: op.rk_stage(src, big[N:9 * N], big[:8 * N], vtm, 0.02, -0.01, nrhs=8),
                 lambda: op.lsrk_step(big[:8 * N], big[N:9 * N], vtm, 0.01, nrhs=8)):
        with pytest.raises(sf.SFError) as e:
            call()
        assert e.value.code == sf.SF_ERR_INVALID and "overlap" in str(e.value)
    op.rk_stage(src, vnp, vnp, vtm, 0.02, -0.01, nrhs=8)          # upd is vec_np itself: allowed
    assert op.device_status() == 0
    lap = sf.Operator(sf.OP_LAPLACE, degree=2, n_cells=(2, 2, 2))
    x = torch.zeros(lap.n_dofs, dtype=torch.float64, device="cuda:0")
    with pytest.raises(sf.SFError):
        lap.rk_stage(x, x, torch.empty_like(x), None, 0.1, 0.0)


def _gll(p):
    from numpy.polynomial import legendre as L
    c = np.zeros(p + 1)
    c[-1] = 1
    r = np.real(L.legroots(L.legder(c))) if p > 1 else np.array([])
    return np.concatenate([[0.0], 0.5 + 0.5 * np.sort(r), [1.0]])


def _wave(p, nc, t):
    """the reference's ExactSolution (evaluation_dg_advect.h:36-95) at the GLL
    nodes of the cell-major DG vector on [0, 2]^3"""
    g = _gll(p)
    h = 2.0 / nc
    i = np.arange(nc)
    X = (i[None, None, :, None, None, None] + g[None, None, None, None, None, :]) * h - t * VEL[0]
    Y = (i[None, :, None, None, None, None] + g[None, None, None, None, :, None]) * h - t * VEL[1]
    Z = (i[:, None, None, None, None, None] + g[None, None, None, :, None, None]) * h - t * VEL[2]
    return (np.sin(4 * np.pi * X) * np.cos(4 * np.pi * Y) * np.cos(4 * np.pi * Z)).reshape(-1)


def test_lsrk_travelling_wave_full_size():
    """48^3 cells, p=4 (13.8 M DoF per vector): 10 LSRK(5,4) steps of the
    exact wave at the reference's time step, FP64 and FP32: the FP64 error
    against the exact wave stays small (9e-5 at 24^3 in the oracle, less at
    48^3) and FP32 follows FP64"""
    torch = torch_cuda()
    sf = _sf()
    p, nc, steps = 4, 48, 10
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=(nc,) * 3, length=(2.0, 2.0, 2.0), velocity=VEL,
                     inverse_mass=1)
    dt = 0.2 / (nc / 2.0) / np.linalg.norm(VEL) / p
    u0 = _wave(p, nc, 0.0)
    res = {}
    for prec, tdt in (("fp64", torch.float64), ("fp32", torch.float32)):
        x = to_dev(torch, u0, tdt)
        old, tmp = torch.zeros_like(x), torch.zeros_like(x)
        for _ in range(steps):
            op.lsrk_step(x, old, tmp, dt)
        res[prec] = to_np(x)
    err64 = np.abs(res["fp64"] - _wave(p, nc, steps * dt)).max()
    assert err64 < 1e-4
    assert np.abs(res["fp32"] - res["fp64"]).max() < 1e-4
    assert op.device_status() == 0


def test_lsrk_matches_oracle_16c():
    """16^3 cells, p=4: 20 steps of the exact wave, GPU FP64 against the
    oracle's LSRK(5,4)"""
    torch = torch_cuda()
    sf = _sf()
    p, nc, steps = 4, 16, 20
    op = sf.Operator(sf.OP_DG_ADVECT, degree=p, n_cells=(nc,) * 3, length=(2.0, 2.0, 2.0), velocity=VEL,
                     inverse_mass=1)
    dt = 0.2 / (nc / 2.0) / np.linalg.norm(VEL) / p
    u0 = _wave(p, nc, 0.0)
    x = to_dev(torch, u0, torch.float64)
    old, tmp = torch.zeros_like(x), torch.zeros_like(x)
    for _ in range(steps):
        op.lsrk_step(x, old, tmp, dt)
    d = O.dg(p, (nc,) * 3, (2.0 / nc,) * 3, velocity=VEL, inverse_mass=1)
    xo, oo, to = u0.copy(), np.zeros_like(u0), np.zeros_like(u0)
    for _ in range(steps):
        O.dg_lsrk_step(d, dt, xo, oo, to)
    assert rel(to_np(x), xo) < FP64_TOL
    assert np.abs(xo - _wave(p, nc, steps * dt)).max() < 2e-3
