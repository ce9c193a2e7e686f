"""The workload configurations at full size (64^3 / 30 A / mmax 3,
96^3 / 40 A / mmax 4, 128^3 / 50 A / mmax 5, all mrso 2), where the CPU oracle
would take too long, through properties that do not depend on size:

* the three forms agree: the double-float form with the FP64 form within the
  FP64 parity bound (1e-12, max-norm relative) and the mixed form within the
  FP32 field bound (1e-4); the FP64 form itself is checked against the oracle
  at the smaller sizes of test_gpu_parity.py;
* Convolution::execute is linear;
* proj2angl . angl2proj is the identity on the band-limited subspace (the
  range of proj2angl), as in test_round_trip_identity.
Inputs are seeded and drawn on the device; sizes follow the reference's
c(q) reader (nq = int(q_max/dq + 0.5) + 2)."""
import gc

import numpy as np
import pytest

from mini_mdft_gb300 import inputs as I

pytestmark = pytest.mark.gpu

CONFIGS = [((64, 64, 64), (30., 30., 30.), 3), ((96, 96, 96), (40., 40., 40.), 4),
           ((128, 128, 128), (50., 50., 50.), 5)]
MRSO = 2
DQ = 0.01


def _rel(a, b):
    import torch
    return (torch.max(torch.abs(a - b)) / torch.max(torch.abs(b))).item()


def _handles(M, n, box, mmax, prec):
    idx, tab = I.synthetic_cq(mmax, MRSO, I.nq_for(n, box, DQ), DQ)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, MRSO)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    conv = M.Convolution.from_table(idx, tab, DQ, sg, ag, precision=prec)
    return ag, opt, conv


def _free():
    import torch
    gc.collect()
    torch.cuda.empty_cache()


@pytest.mark.parametrize("n,box,mmax", CONFIGS)
def test_round_trip_forms_agree(gpu_lib, n, box, mmax):
    """angl2proj + execute + proj2angl (the bench step) in all three forms."""
    import torch
    M = gpu_lib
    N = n[0] * n[1] * n[2]
    nt, nphi, npsi, _, _ = I.angular_counts(mmax, MRSO)
    g = torch.Generator(device="cuda").manual_seed(0)
    dr = (torch.rand((N, nt, nphi, npsi), generator=g, device="cuda", dtype=torch.float64) - 0.5) * 0.2
    out = {}
    for prec in ("f64", "f64df", "f32"):
        ag, opt, conv = _handles(M, n, box, mmax, prec)
        rd, cd = (torch.float32, torch.complex64) if prec == "f32" else (torch.float64, torch.complex128)
        p = torch.zeros((ag.m_np,) + tuple(n), dtype=cd, device="cuda")
        vexc = torch.zeros(dr.shape, dtype=rd, device="cuda")
        opt.angl2proj(dr.to(rd), p)
        conv.execute(p)
        opt.proj2angl(p, vexc)
        torch.cuda.synchronize()
        out[prec] = vexc.double()
        del opt, conv, p, vexc
        _free()
    assert torch.isfinite(out["f64"]).all()
    assert torch.max(torch.abs(out["f64"])).item() > 0
    assert _rel(out["f64df"], out["f64"]) < 1e-12
    assert _rel(out["f32"], out["f64"]) < 1e-4


@pytest.mark.parametrize("n,box,mmax", CONFIGS)
def test_execute_is_linear(gpu_lib, n, box, mmax):
    """execute(x + 2 y) = execute(x) + 2 execute(y) (double-float form)."""
    import torch
    M = gpu_lib
    ag, _, conv = _handles(M, n, box, mmax, "f64df")
    g = torch.Generator(device="cuda").manual_seed(1)
    shp = (ag.m_np,) + tuple(n)
    x = torch.randn(shp, generator=g, device="cuda", dtype=torch.complex128)
    y = torch.randn(shp, generator=g, device="cuda", dtype=torch.complex128)
    z = x + 2 * y
    for t in (x, y, z):
        conv.execute(t)
    torch.cuda.synchronize()
    assert _rel(z, x + 2 * y) < 1e-12
    del x, y, z, conv
    _free()


@pytest.mark.parametrize("n,box,mmax", CONFIGS)
def test_band_limited_round_trip(gpu_lib, n, box, mmax):
    """o' = proj2angl(p) is band-limited, so proj2angl(angl2proj(o')) = o'."""
    import torch
    M = gpu_lib
    ag, opt, _ = _handles(M, n, box, mmax, "f64df")
    N = n[0] * n[1] * n[2]
    g = torch.Generator(device="cuda").manual_seed(2)
    p = torch.randn((ag.m_np,) + tuple(n), generator=g, device="cuda", dtype=torch.complex128)
    o1 = torch.zeros((N, ag.m_ntheta, ag.m_nphi, ag.m_npsi), dtype=torch.float64, device="cuda")
    back = torch.zeros_like(o1)
    opt.proj2angl(p, o1)
    opt.angl2proj(o1, p)
    opt.proj2angl(p, back)
    torch.cuda.synchronize()
    assert _rel(back, o1) < 1e-12
    del p, o1, back, opt
    _free()
