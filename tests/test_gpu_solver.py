"""The solute external potential and the L-BFGS minimiser on the GPU
(mdft_vext_lj_coulomb, mdft_solver_*), through the C ABI:

* vext (double-float arithmetic) equals the oracle's FP64 values
  (oracle/solver.py) within 1e-13 of the sum of the magnitudes of each
  value's terms;
* the energy terms and gradient equal the oracle's on the same xi, with
  vexc from the convolution oracle: FP64 and double-float within 1e-12,
  FP32 within 1e-5 (its convolution is FP32);
* without the excess term the minimiser reaches the Boltzmann density
  xi^2 = exp(-vext / kT);
* the gradient matches central differences of the energy (isotropic c(q),
  for which it is exact);
* with a 12-site solute the energies never rise (FP32: not beyond its
  noise band), the gradient falls, and the three forms reach the same
  minimum;
* on a water-like c(q) the FP32 form reaches the same gradient tolerance
  as the FP64-accurate form (its line search also accepts by the slope)."""
import numpy as np
import pytest

import oracle as O
from oracle import solver as OS
from mini_mdft_gb300 import inputs as I

pytestmark = pytest.mark.gpu

FORMS = ("f64", "f64df", "f32")
DQ = 0.05


def _handles(M, n, box, mmax, mrso, prec, idx, tab):
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, M.OrientationProjectionMap(ag), precision=prec)
    conv = M.Convolution.from_table(idx, tab, DQ, sg, ag, precision=prec)
    return sg, ag, opt, conv


def test_vext_matches_oracle(gpu_lib):
    M = gpu_lib
    n, box, mmax, mrso = (10, 12, 14), (14., 15., 16.), 3, 2
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    su = I.synthetic_solute(12, box, seed=3)
    vmax = 100 * I.kT()
    v = M.solute_vext(sg, ag, I.SPCE_SITES, su, vmax).cpu().numpy().reshape(-1, ag.m_no)
    vo, size = OS.vext_lj_coulomb(n, box, ag.m_thetaofntheta, ag.m_nphi, ag.m_npsi, mrso, I.SPCE_SITES, su, vmax,
                                  with_size=True)
    # double-float on the GPU: each value within 1e-13 of the sum of the
    # magnitudes of its terms (LJ repulsion and Coulomb attraction can cancel
    # to 1e-4 of that sum; 1.5e-14 measured)
    assert np.all(np.abs(v - vo) <= 1e-13 * size)
    assert (v == vmax).any() and (np.abs(v) < vmax).mean() > 0.5  # cores capped, the rest not


@pytest.mark.parametrize("prec", FORMS)
def test_energy_and_gradient_match_oracle(gpu_lib, prec):
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (8, 8, 8), (10., 10., 10.), 2, 2
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ)
    sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, prec, idx, tab)
    g = O.Oracle(n, box, mmax, mrso)
    g.set_luc(idx, tab, DQ)
    _, _, w = g.angular()
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    su = I.synthetic_solute(4, box, seed=4)
    vext = OS.vext_lj_coulomb(n, box, ag.m_thetaofntheta, ag.m_nphi, ag.m_npsi, mrso, I.SPCE_SITES, su, 20 * kT)
    xi = np.random.default_rng(6).uniform(0.8, 1.2, (g.N, g.no))
    vexc = g.proj2angl(g.conv_execute(g.angl2proj(O.delta_rho(xi, rho0)))).reshape(g.N, g.no)
    dv = float(np.prod(np.array(box) / np.array(n)))
    t_o, g_o = OS.energy_terms(xi, vexc, vext, w, kT, rho0, dv, pref)
    solver = M.Solver(opt, conv, torch.from_numpy(vext).cuda(), kT=kT, rho0=rho0, prefactor=pref)
    xt = torch.from_numpy(xi).cuda()
    grad = torch.empty_like(xt)
    t = solver.energy(xt, grad)
    tol = 1e-5 if prec == "f32" else 1e-12
    scale = max(abs(t_o[1]), abs(t_o[2]), abs(t_o[3]))
    for k, name in enumerate(M.Solver.TERMS[:4]):
        assert abs(t[name] - t_o[k]) <= tol * scale, name
    assert np.abs(grad.cpu().numpy() - g_o).max() <= tol * np.abs(g_o).max()
    assert abs(t["gmax"] - t_o[4]) <= tol * t_o[4]


@pytest.mark.parametrize("prec", ("f64df", "f32"))
def test_energy_over_the_whole_xi_range(gpu_lib, prec):
    """The ideal and external terms for xi from 1e-30 to 1e8 (both signs,
    0, +-1, the sqrt 2 and 2^+-20 boundaries of the double-float logarithm),
    element by element: |g - g_oracle| within 1e-12 of the sizes of the
    gradient's terms before they cancel; the mixed form computes them in
    FP32 (sums in double-float), within 2e-6."""
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (6, 6, 6), (9., 9., 9.), 2, 2
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ)
    tab[:] = 0  # vexc = 0: the excess term is checked above
    sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, prec, idx, tab)
    rng = np.random.default_rng(11)
    N, no = 216, ag.m_no
    xi = np.exp(rng.uniform(np.log(1e-30), np.log(1e8), N * no)) * rng.choice([-1.0, 1.0], N * no)
    special = [0.0, 1.0, -1.0, 2 ** -20, 2 ** 20, -(2 ** -20), 2 ** -20 * (1 - 2 ** -52), 2 ** 20 * (1 + 2 ** -52),
               2 ** 0.25, 2 ** -0.25, 2 ** 0.25 * (1 + 1e-15), 1 + 1e-9, 1 - 1e-12, 0.7, 1.3, 1e-7, 3e5]
    xi[: len(special)] = special
    xi[len(special): 2000] = rng.uniform(0.5, 1.5, 2000 - len(special))
    xi = xi.reshape(N, no)
    kT = I.kT()
    vext = rng.uniform(-50, 50, (N, no))
    vext[:, ::3] = 0.0
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    w = ag.m_w
    dv = 1.5 ** 3
    t_o, g_o = OS.energy_terms(xi, np.zeros_like(xi), vext, w, kT, rho0, dv, pref)
    solver = M.Solver(opt, conv, torch.from_numpy(vext).cuda(), kT=kT, rho0=rho0, prefactor=pref)
    grad = torch.empty((N, no), dtype=torch.float64, device="cuda")
    t = solver.energy(torch.from_numpy(xi).cuda(), grad)
    scale = max(abs(t_o[1]), abs(t_o[2]))
    tol = 2e-6 if prec == "f32" else 1e-12
    for k, name in enumerate(M.Solver.TERMS[:3]):
        assert abs(t[name] - t_o[k]) <= tol * scale, name
    x2 = xi * xi
    lx = np.where(x2 > 0, np.log(np.where(x2 > 0, x2, 1.0)), 0.0)
    size = 2 * np.abs(xi) * w[None, :] * rho0 * dv * (kT * np.abs(lx) + np.abs(vext))
    err = np.abs(grad.cpu().numpy() - g_o)
    assert np.all(err <= tol * size + 1e-300), float((err / np.maximum(size, 1e-300)).max())


def test_minimizer_reaches_boltzmann_density_without_excess(gpu_lib):
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (8, 8, 8), (12., 12., 12.), 2, 2
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ)
    tab[:] = 0  # no excess term
    sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, "f64", idx, tab)
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    su = I.synthetic_solute(6, box, seed=5)
    vext = M.solute_vext(sg, ag, I.SPCE_SITES, su, 5 * kT)
    xi = torch.ones_like(vext)
    solver = M.Solver(opt, conv, vext, kT=kT, rho0=rho0, prefactor=pref)
    # near max |g| ~ 1e-7 the energy decrease of a step (~1e-12) reaches the
    # rounding of E (~2e3 here, spacing 4.5e-13), so the run may stop there
    # before gtol; 1e-6 bounds |ln xi - ln xi_B| by ~1e-4
    assert solver.status() == -1  # never run
    trace = solver.minimize(xi, max_iter=300, gtol=1e-10)
    assert trace[-1, 4] <= 1e-6
    # it ends at gtol or at the rounding floor, not at the iteration cap
    assert M.Solver.STATUS[solver.status()] in ("gtol", "flat", "no_decrease")
    if solver.status() == 0:
        assert trace[-1, 4] <= 1e-10
    assert len(trace) - 1 < 300
    solver.minimize(xi, max_iter=1, gtol=0.0)
    assert M.Solver.STATUS[solver.status()] in ("max_iter", "flat", "no_decrease")
    assert np.all(np.diff(trace[:, 0]) <= 0)
    # E depends on xi^2 only (rho = rho0 xi^2): a step may cross to -xi
    xb = torch.exp(-vext / (2 * kT))
    assert torch.max(torch.abs(torch.abs(xi) - xb) / xb).item() < 1e-4
    assert abs(trace[-1, 3]) < 1e-300  # no excess term


@pytest.mark.parametrize("prec", ("f64", "f64df"))
def test_gradient_matches_finite_differences(gpu_lib, prec):
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (12, 12, 12), (14., 14., 14.), 3, 2
    idx, tab = I.isotropic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ, amplitude=1e-3)
    sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, prec, idx, tab)
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    vext = M.solute_vext(sg, ag, I.SPCE_SITES, I.synthetic_solute(4, box, seed=8), 20 * kT)
    solver = M.Solver(opt, conv, vext, kT=kT, rho0=rho0, prefactor=pref)
    gen = torch.Generator(device="cuda").manual_seed(9)
    xi = 0.8 + 0.4 * torch.rand(vext.shape, generator=gen, device="cuda", dtype=torch.float64)
    d = torch.randn(vext.shape, generator=gen, device="cuda", dtype=torch.float64)
    grad = torch.empty_like(xi)
    e0 = solver.energy(xi, grad)
    assert abs(e0["exc"]) > 1e-3 * abs(e0["id"])  # the excess term takes part
    an = torch.sum(grad * d).item()
    h = 1e-5
    fp = solver.energy(xi + h * d)["total"]
    fm = solver.energy(xi - h * d)["total"]
    assert abs((fp - fm) / (2 * h) - an) <= 1e-6 * abs(an)


def test_minimizer_with_solute_descends_and_forms_agree(gpu_lib):
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (16, 16, 16), (16., 16., 16.), 3, 2
    idx, tab = I.isotropic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ, amplitude=1e-3)
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    su = I.synthetic_solute(12, box, seed=3)
    final = {}
    for prec in FORMS:
        sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, prec, idx, tab)
        vext = M.solute_vext(sg, ag, I.SPCE_SITES, su, 100 * kT)
        solver = M.Solver(opt, conv, vext, kT=kT, rho0=rho0, prefactor=pref, history=7)
        xi = torch.ones_like(vext)
        trace = solver.minimize(xi, max_iter=300, gtol=1e-9)
        # the FP32 convolution's energies carry ~1e-7 relative noise: there
        # the line search also accepts a step by its slope (approximate
        # Wolfe) when E is within 1e-6 |E| of the current value, so E may
        # rise by that much; the FP64 forms descend monotonically
        band = 1e-6 if prec == "f32" else 1e-12
        assert np.all(np.diff(trace[:, 0]) <= band * np.abs(trace[:, 0]).max()), prec
        assert trace[-1, 4] <= (1e-2 if prec == "f32" else 1e-3) * trace[0, 4], prec
        assert torch.isfinite(xi).all()
        final[prec] = trace[-1]
    assert abs(final["f64df"][0] - final["f64"][0]) <= 1e-9 * abs(final["f64"][0])
    assert abs(final["f32"][0] - final["f64"][0]) <= 1e-5 * abs(final["f64"][0])


def test_solver_argument_errors(gpu_lib):
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (4, 4, 4), (8., 8., 8.), 1, 1
    idx, tab = I.synthetic_cq(mmax, mrso, I.nq_for(n, box, DQ), DQ)
    sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, "f64", idx, tab)
    _, _, opt32, _ = _handles(M, n, box, mmax, mrso, "f32", idx, tab)
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    with pytest.raises(M.MdftError):
        M.Solver(opt, conv, None, kT=I.kT(), rho0=rho0, prefactor=pref, history=0)
    with pytest.raises(M.MdftError):
        M.Solver(opt32, conv, None, kT=I.kT(), rho0=rho0, prefactor=pref)
    with pytest.raises(M.MdftError):
        M.solute_vext(sg, ag, I.SPCE_SITES, I.synthetic_solute(2, box), vmax=-1.0)
    s = M.Solver(opt, conv, None, kT=I.kT(), rho0=rho0, prefactor=pref)
    with pytest.raises(M.MdftError):
        s.energy(torch.ones(3, dtype=torch.float64, device="cuda"))


def test_mixed_form_reaches_the_fp64_gradient_tolerance(gpu_lib):
    """The serving stream's tolerance, max |dE/dxi| <= 1e-5, on a 24^3 grid
    in a 20 A box with a water-like c(q) (amplitude 3e-6) and a 12-site
    solute: the FP32
    form ends by gtol (not by E going flat at its noise), in about as many
    iterations as the double-float form, at an energy within 1e-6 of it."""
    import torch
    M = gpu_lib
    n, box, mmax, mrso = (24, 24, 24), (20., 20., 20.), 3, 2
    idx, tab = I.isotropic_cq(mmax, mrso, I.nq_for(n, box, DQ) + 2, DQ, amplitude=3e-6)
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    su = I.synthetic_solute(12, box, seed=11)
    out = {}
    for prec in ("f64df", "f32"):
        sg, ag, opt, conv = _handles(M, n, box, mmax, mrso, prec, idx, tab)
        vext = M.solute_vext(sg, ag, I.SPCE_SITES, su, 100 * kT)
        solver = M.Solver(opt, conv, vext, kT=kT, rho0=rho0, prefactor=pref, history=5)
        trace = solver.minimize(torch.ones_like(vext), max_iter=300, gtol=1e-5)
        out[prec] = (M.Solver.STATUS[solver.status()], len(trace) - 1, trace[-1])
    st_df, it_df, last_df = out["f64df"]
    st_32, it_32, last_32 = out["f32"]
    assert st_df == "gtol" and st_32 == "gtol", (st_df, st_32)
    assert last_32[4] <= 1e-5
    assert it_32 <= 1.5 * it_df + 10
    assert abs(last_32[0] - last_df[0]) <= 1e-6 * abs(last_df[0])
