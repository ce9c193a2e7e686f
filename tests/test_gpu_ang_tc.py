"""The tensor-core angular transforms (MDFT_ANG_TC=1 at create time: dense
per-point matrices as tcgen05 GEMMs with exact BF16 digit slicing) against
the oracle's angl2proj / proj2angl
(MDFT_OrientationProjectionTransform.hpp:270-380, :391-484): double-float
form within 1e-12, FP32 form within 1e-4 (max-norm relative), on grids with
partial tiles and unaligned plane strides (plain-load path) and whole tiles
(bulk-copy path), and the 32^3 pipeline energy within the FP32 bound."""
import os

import numpy as np
import pytest

import oracle as O
from mini_mdft_gb300 import inputs as I
from tests._util import rel_err

pytestmark = pytest.mark.gpu

CASES = [((8, 8, 8), 3, 2), ((5, 6, 7), 3, 2), ((16, 16, 16), 2, 2), ((9, 7, 5), 1, 2), ((32, 32, 32), 3, 2)]


@pytest.fixture
def tc_on():
    old = os.environ.get("MDFT_ANG_TC")
    os.environ["MDFT_ANG_TC"] = "1"
    yield
    if old is None:
        del os.environ["MDFT_ANG_TC"]
    else:
        os.environ["MDFT_ANG_TC"] = old


@pytest.mark.parametrize("prec", ["f64df", "f32"])
@pytest.mark.parametrize("n,mmax,mrso", CASES)
def test_tensor_core_transforms_vs_oracle(gpu_lib, tc_on, n, mmax, mrso, prec):
    import torch
    M = gpu_lib
    o = O.Oracle(n, (10.0, 10.0, 10.0), mmax, mrso)
    rng = np.random.default_rng(7)
    x = rng.uniform(-0.1, 0.1, (o.N, o.ntheta, o.nphi, o.npsi))
    p_ref = o.angl2proj(x)
    q = rng.normal(size=(o.np,) + tuple(n)) + 1j * rng.normal(size=(o.np,) + tuple(n))
    o_ref = o.proj2angl(q)
    sg, ag = M.SpatialGrid(n, (10.0, 10.0, 10.0)), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    rd, cd = (torch.float32, torch.complex64) if prec == "f32" else (torch.float64, torch.complex128)
    tol = 1e-4 if prec == "f32" else 1e-12
    p = torch.zeros((o.np,) + tuple(n), dtype=cd, device="cuda")
    opt.angl2proj(torch.from_numpy(x).to("cuda", rd), p)
    assert rel_err(p.cpu().numpy(), p_ref) < tol
    out = torch.zeros(x.shape, dtype=rd, device="cuda")
    opt.proj2angl(torch.from_numpy(q).to("cuda", cd), out)
    assert rel_err(out.cpu().numpy(), o_ref) < tol


def test_tensor_core_pipeline_energy_32cubed(gpu_lib, tc_on):
    """get_delta_rho -> angl2proj -> execute -> proj2angl -> get_delta_f at
    32^3 / 20 A / mmax 3 in the FP32 form with the tensor-core transforms:
    the energy within 1e-6 of the oracle's."""
    import torch
    M = gpu_lib
    n, box, mmax, mrso, dq = (32, 32, 32), (20., 20., 20.), 3, 2, 0.01
    o = O.Oracle(n, box, mmax, mrso)
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, dq), dq)
    o.set_luc(idx, tab, dq)
    xi = I.synthetic_xi(o.N, mmax, mrso)
    rho0, pref = I.tip3p_constants(mrso)
    _, _, w = o.angular()
    vexc_ref = o.proj2angl(o.conv_execute(o.angl2proj(O.delta_rho(xi, rho0))))
    _, ff_ref = O.delta_f(xi, vexc_ref, w, rho0, pref)
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision="f32")
    conv = M.Convolution.from_table(idx, tab, dq, sg, ag, precision="f32")
    xt = torch.from_numpy(xi).to("cuda", torch.float32)
    dr = torch.zeros_like(xt)
    M.get_delta_rho(xt, dr, rho0)
    p = torch.zeros((o.np,) + n, dtype=torch.complex64, device="cuda")
    opt.angl2proj(dr, p)
    conv.execute(p)
    vexc = torch.zeros_like(xt)
    opt.proj2angl(p, vexc)
    ff = M.get_delta_f(xt, vexc, torch.from_numpy(w), torch.zeros_like(xt), rho0, pref)
    assert abs(ff - ff_ref) <= 1e-6 * abs(ff_ref)
