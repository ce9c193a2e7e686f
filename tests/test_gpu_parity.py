"""GPU parity: every stage of the hot path through the C ABI against the CPU
oracle on the same seeded inputs.

Tolerances (max-norm relative error, max|gpu - oracle| / max|oracle|):
  FP64 plain form: 1e-12 (projections, convolved fields, energy, gradient);
  FP32 mixed form: 1e-4 for the fields, 1e-6 for the excess energy (the
  mixed form's accuracy target is stated on the excess free energy).
"""
import numpy as np
import pytest

import oracle as O
from mini_mdft_gb300 import inputs as I

from _util import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-4


def _t(x, dtype):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).to(device="cuda", dtype=dtype)


def _np(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _dtypes(prec):
    import torch
    return (torch.float32, torch.complex64) if prec == "f32" else (torch.float64, torch.complex128)


def _tol(prec):
    # f64 and f64df (FP64 fields, double-float arithmetic) share the 1e-12 bound
    return TOL32 if prec == "f32" else TOL64


PRECS = ["f64", "f32", "f64df"]


OPT_CASES = [((2, 2, 2), 10, 10), ((3, 2, 2), 3, 2), ((2, 2, 1), 5, 1), ((2, 1, 2), 4, 3),
             ((2, 2, 2), 1, 2), ((1, 1, 3), 2, 1), ((8, 8, 8), 3, 2), ((5, 6, 7), 5, 2),
             ((9, 7, 5), 4, 2), ((4, 4, 4), 6, 1)]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,mmax,mrso", OPT_CASES)
def test_angl2proj(gpu_lib, n, mmax, mrso, prec):
    import torch
    M = gpu_lib
    o = O.Oracle(n, (1.0, 1.0, 1.0), mmax, mrso)
    rng = np.random.default_rng(12345)
    x = rng.uniform(0, 1, size=(o.N, o.ntheta, o.nphi, o.npsi))
    ref = o.angl2proj(x)
    sg, ag = M.SpatialGrid(n, (1.0, 1.0, 1.0)), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    rd, cd = _dtypes(prec)
    xo = _t(x, rd)
    p = torch.zeros((o.np,) + tuple(n), dtype=cd, device="cuda")
    opt.angl2proj(xo, p)
    assert rel_err(_np(p), ref) < _tol(prec)
    # get_delta_rho fused into the load
    rho0 = 0.3
    opt.angl2proj_from_xi(xo, rho0, p)
    ref2 = o.angl2proj(O.delta_rho(x, rho0))
    assert rel_err(_np(p), ref2) < _tol(prec)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,mmax,mrso", OPT_CASES)
def test_proj2angl(gpu_lib, n, mmax, mrso, prec):
    import torch
    M = gpu_lib
    o = O.Oracle(n, (1.0, 1.0, 1.0), mmax, mrso)
    rng = np.random.default_rng(12345)
    shp = (o.np,) + tuple(n)
    p = rng.uniform(0, 1, shp) + 1j * rng.uniform(0, 1, shp)
    ref = o.proj2angl(p)
    sg, ag = M.SpatialGrid(n, (1.0, 1.0, 1.0)), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    rd, cd = _dtypes(prec)
    out = torch.zeros((o.N, o.ntheta, o.nphi, o.npsi), dtype=rd, device="cuda")
    pt = _t(p, cd)
    opt.proj2angl(pt, out)
    assert rel_err(_np(out), ref) < _tol(prec)
    # p is read only
    assert np.array_equal(_np(pt), p.astype(_np(pt).dtype))


@pytest.mark.parametrize("n,mmax,mrso", OPT_CASES[:7])
def test_round_trip_identity(gpu_lib, n, mmax, mrso):
    # Test_OrientationProjectionTransform.cpp:312-348 plus the band-limited
    # subspace where proj2angl . angl2proj is the identity
    import torch
    M = gpu_lib
    sg, ag = M.SpatialGrid(n, (1.0, 1.0, 1.0)), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag))
    N = int(np.prod(n))
    shape_o = (N, ag.m_ntheta, ag.m_nphi, ag.m_npsi)
    p = torch.zeros((ag.m_np,) + tuple(n), dtype=torch.complex128, device="cuda")
    ones = torch.ones(shape_o, dtype=torch.float64, device="cuda")
    back = torch.zeros_like(ones)
    opt.angl2proj(ones, p)
    opt.proj2angl(p, back)
    assert rel_err(_np(back), _np(ones)) < 1e-13
    rng = np.random.default_rng(7)
    pr = rng.standard_normal(p.shape) + 1j * rng.standard_normal(p.shape)
    o1 = torch.zeros_like(ones)
    opt.proj2angl(_t(pr, torch.complex128), o1)
    opt.angl2proj(o1, p)
    opt.proj2angl(p, back)
    assert rel_err(_np(back), _np(o1)) < 1e-12


FFT_SHAPES = [(2, 4, 5), (8, 8, 8), (6, 10, 12), (3, 5, 7), (32, 48, 5), (16, 16, 16),
              (20, 24, 30), (64, 32, 4), (1, 1, 9), (11, 13, 2), (128, 2, 2), (4, 96, 3),
              (80, 2, 3)]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n", FFT_SHAPES)
def test_fft3d_vs_numpy_and_cufft(gpu_lib, n, prec):
    import torch
    M = gpu_lib
    sg, ag = M.SpatialGrid(n, (10.0, 10.0, 10.0)), M.AngularGrid(1, 2)
    nq = I.nq_for(n, (10.0, 10.0, 10.0), 0.01)
    idx, tab = I.synthetic_cq(1, 2, nq, 0.01)
    conv = M.Convolution.from_table(idx, tab, 0.01, sg, ag, precision=prec)
    rng = np.random.default_rng(3)
    shp = (ag.m_np,) + tuple(n)
    x = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    rd, cd = _dtypes(prec)
    tol = {"f64": 1e-13, "f64df": 1e-13, "f32": 2e-6}[prec]
    for sign in (-1, 1):
        t = _t(x, cd)
        conv.fft(t, sign)
        ref = np.fft.fftn(x, axes=(1, 2, 3)) if sign < 0 else \
            np.fft.ifftn(x, axes=(1, 2, 3)) * np.prod(n)
        assert rel_err(_np(t), ref) < tol
        # cuFFT (through torch.fft) as the comparator only
        cu = torch.fft.fftn(_t(x, cd), dim=(1, 2, 3)) if sign < 0 else \
            torch.fft.ifftn(_t(x, cd), dim=(1, 2, 3), norm="forward")
        assert rel_err(_np(t), _np(cu)) < 10 * tol


CONV_CASES = [((4, 4, 4), (10., 10., 10.), 3, 2), ((5, 5, 5), (1., 1., 1.), 3, 2),
              ((4, 3, 6), (8., 7., 9.), 2, 1), ((2, 4, 5), (5., 6., 7.), 1, 2),
              ((8, 6, 10), (12., 9., 15.), 4, 2), ((6, 6, 6), (9., 9., 9.), 5, 2),
              ((6, 5, 4), (9., 8., 7.), 6, 3), ((16, 16, 16), (20., 20., 20.), 3, 2),
              ((10, 10, 10), (1., 1., 1.), 3, 2)]


def _conv_pair(M, n, box, mmax, mrso, prec):
    o = O.Oracle(n, box, mmax, mrso)
    dq = 0.01
    nq = o.nq_for_dq(dq)
    idx, tab = I.synthetic_cq(mmax, mrso, nq + 2, dq)
    o.set_luc(idx, tab, dq)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    conv = M.Convolution.from_table(idx, tab, dq, sg, ag, precision=prec)
    return o, conv, idx, tab


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,box,mmax,mrso", CONV_CASES)
def test_conv_execute(gpu_lib, n, box, mmax, mrso, prec):
    M = gpu_lib
    o, conv, _, _ = _conv_pair(M, n, box, mmax, mrso, prec)
    rng = np.random.default_rng(12345)
    shp = (o.np,) + tuple(n)
    p = rng.uniform(0, 1, shp) + 1j * rng.uniform(0, 1, shp)
    ref = o.conv_execute(p)
    rd, cd = _dtypes(prec)
    t = _t(p, cd)
    conv.execute(t)
    assert rel_err(_np(t), ref) < _tol(prec)


@pytest.mark.parametrize("prec", PRECS)
def test_conv_execute_timed_equals_execute(gpu_lib, prec):
    """The stage-timed execute runs the same kernels: bit-identical output,
    and its four events come in stream order."""
    import torch
    M = gpu_lib
    n = (16, 12, 10)
    o, conv, _, _ = _conv_pair(M, n, (20., 15., 12.), 3, 2, prec)
    rng = np.random.default_rng(7)
    shp = (o.np,) + tuple(n)
    p = rng.uniform(0, 1, shp) + 1j * rng.uniform(0, 1, shp)
    rd, cd = _dtypes(prec)
    a, b = _t(p, cd), _t(p, cd)
    conv.execute(a)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    conv.execute_timed(b, ev)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert all(ev[i].elapsed_time(ev[i + 1]) >= 0.0 for i in range(3))
    with pytest.raises(ValueError):
        conv.execute_timed(b, ev[:3])


def test_conv_tables_match_oracle(gpu_lib):
    M = gpu_lib
    o, conv, _, _ = _conv_pair(M, (6, 5, 4), (9., 8., 7.), 5, 2, "f64")
    assert np.array_equal(conv.gamma_p_map(), o.gamma_p_map())
    assert np.array_equal(conv.mnmunukhi_q(), o.mnmunukhi_q())
    assert conv.nq == o.nq and conv.dq() == 0.01


def test_conv_from_file_equals_from_table(gpu_lib, tmp_path):
    M = gpu_lib
    n, box, mmax, mrso = (8, 8, 8), (10., 10., 10.), 3, 2
    path = I.write_luc_if_missing(str(tmp_path), mmax, mrso, n, box)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    c1 = M.Convolution(path, sg, ag, M.OrientationProjectionMap(ag), I.NPLUC[mmax])
    idx, tab, dq = I.read_luc_file(path, I.NPLUC[mmax])
    c2 = M.Convolution.from_table(idx, tab, dq, sg, ag)
    assert abs(c1.dq() - c2.dq()) < 1e-15
    assert np.allclose(c1.mnmunukhi_q(), c2.mnmunukhi_q(), rtol=0, atol=1e-15)
    rng = np.random.default_rng(1)
    shp = (ag.m_np,) + n
    p = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
    import torch
    a, b = _t(p, torch.complex128), _t(p, torch.complex128)
    c1.execute(a)
    c2.execute(b)
    assert rel_err(_np(a), _np(b)) < 1e-13


def test_conv_errors(gpu_lib, tmp_path):
    M = gpu_lib
    sg, ag = M.SpatialGrid((8, 8, 8), (10., 10., 10.)), M.AngularGrid(3, 2)
    with pytest.raises(M.MdftError, match="does not exist"):
        M.Convolution(str(tmp_path / "nope"), sg, ag, None, 252)
    idx, tab = I.synthetic_cq(3, 2, 10, 0.01)  # far too few q rows
    with pytest.raises(M.MdftError, match="rows"):
        M.Convolution.from_table(idx, tab, 0.01, sg, ag)
    with pytest.raises(M.MdftError, match="mmax <= 6"):
        M.Convolution.from_table(idx, tab, 0.01, sg, M.AngularGrid(7, 2))


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_energy(gpu_lib, prec):
    # unit_test/Test_Solvent.cpp:127-211 shapes, then a grid-sized case
    import torch
    M = gpu_lib
    rd, _ = _dtypes(prec)
    for shape in [(2, 3, 4, 5), (16, 16, 16, 84), (7, 5, 3, 330)]:
        rng = np.random.default_rng(12345)
        xi = rng.uniform(0, 1, shape)
        vexc = rng.uniform(-1, 1, shape)
        w = rng.uniform(0, 1, shape[-1])
        rho0, pref = 0.3, 0.334
        dr = torch.zeros(shape, dtype=rd, device="cuda")
        M.get_delta_rho(_t(xi, rd), dr, rho0)
        tol = 1e-15 if prec == "f64" else 1e-6
        assert rel_err(_np(dr), O.delta_rho(xi, rho0)) < tol * 10
        df_ref, ff_ref = O.delta_f(xi, vexc, w, rho0, pref)
        df = torch.zeros(shape, dtype=rd, device="cuda")
        ff = M.get_delta_f(_t(xi, rd), _t(vexc, rd), torch.from_numpy(w), df, rho0, pref)
        assert rel_err(_np(df), df_ref) < tol * 10
        if prec == "f64":
            assert abs(ff - ff_ref) <= 1e-12 * abs(ff_ref)
            ff2 = M.get_delta_f(_t(xi, rd), _t(vexc, rd), torch.from_numpy(w), df, rho0, pref)
            assert ff2 == ff  # deterministic reduction
        else:
            # inputs rounded to FP32; the sum itself is FP64
            xi32 = xi.astype(np.float32).astype(np.float64)
            v32 = vexc.astype(np.float32).astype(np.float64)
            _, ff_ref32 = O.delta_f(xi32, v32, w, rho0, pref)
            assert abs(ff - ff_ref32) <= 1e-12 * abs(ff_ref32)


@pytest.mark.parametrize("prec", PRECS)
def test_energy_cproj_pipeline_32cubed(gpu_lib, prec):
    """The five stages of Solver::energy_cproj_mrso (src/mini-mdft.hpp:137-183)
    on the 32^3 / 20 A / mmax 3 / mrso 2 configuration, against the oracle:
    projections, convolved projections, vexc, gradient and energy."""
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (32, 32, 32), (20., 20., 20.), 3, 2
    o, conv, _, _ = _conv_pair(M, n, box, mmax, mrso, prec)
    N = o.N
    xi = I.synthetic_xi(N, mmax, mrso)
    rho0, pref = I.tip3p_constants(mrso)
    # oracle
    dr = O.delta_rho(xi, rho0)
    p_ref = o.angl2proj(dr)
    pc_ref = o.conv_execute(p_ref)
    vexc_ref = o.proj2angl(pc_ref)
    _, _, w = o.angular()
    df_ref, ff_ref = O.delta_f(xi, vexc_ref, w, rho0, pref)
    # GPU through the C ABI
    rd, cd = _dtypes(prec)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    xt = _t(xi, rd)
    drt = torch.zeros_like(xt)
    M.get_delta_rho(xt, drt, rho0)
    p = torch.zeros((o.np,) + n, dtype=cd, device="cuda")
    opt.angl2proj(drt, p)
    tol = _tol(prec)
    assert rel_err(_np(p), p_ref) < tol
    conv.execute(p)
    assert rel_err(_np(p), pc_ref) < tol
    vexc = torch.zeros_like(xt)
    opt.proj2angl(p, vexc)
    assert rel_err(_np(vexc), vexc_ref) < tol
    df = torch.zeros_like(xt)
    ff = M.get_delta_f(xt, vexc, torch.from_numpy(w), df, rho0, pref)
    assert rel_err(_np(df), df_ref) < tol
    assert abs(ff - ff_ref) <= (1e-6 if prec == "f32" else 1e-12) * abs(ff_ref)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("n,box,mmax,mrso", [((12, 10, 8), (12., 10., 9.), 3, 2),
                                             ((6, 7, 8), (9., 9., 9.), 2, 1),
                                             ((8, 6, 10), (12., 9., 15.), 5, 2)])
def test_batched_plans_equal_single_fields(gpu_lib, n, box, mmax, mrso, prec):
    """A batched plan (B same-shape fields per call: o stored back to back, p
    as (np, B, nx, ny, nz)) gives every field exactly what the single-field
    plan gives it."""
    import torch
    M = gpu_lib
    B = 3
    o = O.Oracle(n, box, mmax, mrso)
    dq = 0.01
    idx, tab = I.synthetic_cq(mmax, mrso, o.nq_for_dq(dq) + 2, dq)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt1 = M.OrientationProjectionTransform(sg, ag, precision=prec)
    conv1 = M.Convolution.from_table(idx, tab, dq, sg, ag, precision=prec)
    optb = M.OrientationProjectionTransform(sg, ag, precision=prec, batch=B)
    convb = M.Convolution.from_table(idx, tab, dq, sg, ag, precision=prec, batch=B)
    rd, cd = _dtypes(prec)
    rng = np.random.default_rng(5)
    fields = [_t(rng.uniform(-0.1, 0.1, (o.N, o.ntheta, o.nphi, o.npsi)), rd) for _ in range(B)]
    singles_p, singles_v = [], []
    for f in fields:
        p = torch.zeros((o.np,) + tuple(n), dtype=cd, device="cuda")
        v = torch.zeros_like(f)
        opt1.angl2proj(f, p)
        conv1.execute(p)
        opt1.proj2angl(p, v)
        singles_p.append(p)
        singles_v.append(v)
    ob = torch.cat(fields)
    pb = torch.zeros((o.np, B) + tuple(n), dtype=cd, device="cuda")
    vb = torch.zeros_like(ob)
    optb.angl2proj(ob, pb)
    convb.execute(pb)
    optb.proj2angl(pb, vb)
    torch.cuda.synchronize()
    for b in range(B):
        assert torch.equal(pb[:, b], singles_p[b])
        assert torch.equal(vb[b * o.N:(b + 1) * o.N], singles_v[b])


def test_no_copy_wait_timed_out(gpu_lib):
    """Every asynchronous tile copy of the FFTs above landed in time (a wait
    that runs out leaves its tile untouched and is counted)."""
    assert gpu_lib.wait_timeouts() == 0
