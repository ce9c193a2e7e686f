"""The oracle of the minimiser's functional (oracle/solver.py) on the CPU:
the orientation rotations, the external potential against direct loops,
and the gradient formula -- the ideal and external terms against finite
differences and their Boltzmann minimum, and the excess term's
2 prefactor w df against finite differences of get_delta_f's ff through the
convolution oracle for a symmetric (isotropic) c(q).  No reference
implementation of these terms exists, so they are pinned by identities."""
import math

import numpy as np
import pytest

import oracle as O
from oracle import solver as OS
from mini_mdft_gb300 import inputs as I


def test_orientation_rotations_are_rotations():
    g = O.Oracle((2, 2, 2), (5., 5., 5.), 3, 2)
    th, _, _ = g.angular()
    R = OS.orientation_rotations(th, g.nphi, g.npsi, g.mrso)
    assert R.shape == (g.no, 3, 3)
    for r in R:
        assert np.abs(r @ r.T - np.eye(3)).max() < 1e-14
        assert abs(np.linalg.det(r) - 1.0) < 1e-14
    # the molecular z axis goes to the orientation's direction (sin t cos p, sin t sin p, cos t)
    io = 0
    for t in th:
        for i in range(g.nphi):
            for k in range(g.npsi):
                p = 2 * math.pi * i / g.nphi
                assert np.abs(R[io] @ [0, 0, 1] - [math.sin(t) * math.cos(p), math.sin(t) * math.sin(p),
                                                   math.cos(t)]).max() < 1e-15
                io += 1


def test_vext_matches_direct_loops():
    n, box, mmax, mrso = (4, 3, 5), (9., 8., 10.), 2, 2
    g = O.Oracle(n, box, mmax, mrso)
    th, _, _ = g.angular()
    su = I.synthetic_solute(5, box, seed=7)
    vmax = 1e3
    v = OS.vext_lj_coulomb(n, box, th, g.nphi, g.npsi, mrso, I.SPCE_SITES, su, vmax)
    R = OS.orientation_rotations(th, g.nphi, g.npsi, mrso)
    qf = OS.qfact()
    L = np.array(box)
    rng = np.random.default_rng(0)
    for _ in range(40):
        r, o = int(rng.integers(v.shape[0])), int(rng.integers(v.shape[1]))
        ix, iy, iz = r // (n[1] * n[2]), (r // n[2]) % n[1], r % n[2]
        p = np.array([ix * box[0] / n[0], iy * box[1] / n[1], iz * box[2] / n[2]])
        tot = 0.0
        for a in I.SPCE_SITES:
            sa = p + R[o] @ a[3:6]
            for s in su:
                dd = sa - s[3:6]
                dd -= L * np.rint(dd / L)
                d = math.sqrt(max(dd @ dd, 1e-12))
                eps, sig = math.sqrt(a[2] * s[2]), 0.5 * (a[1] + s[1])
                if eps:
                    tot += 4 * eps * ((sig / d) ** 12 - (sig / d) ** 6)
                tot += qf * a[0] * s[0] / d
        tot = min(max(tot, -vmax), vmax)
        assert abs(v[r, o] - tot) <= 1e-11 * max(1.0, abs(tot))


def test_qfact_value():
    # e^2 / (4 pi eps0 A) in kJ/mol
    assert abs(OS.qfact() - 1389.3545) < 1e-3


def _setup(n=(6, 6, 6), box=(12., 12., 12.), mmax=1, mrso=1):
    g = O.Oracle(n, box, mmax, mrso)
    th, _, w = g.angular()
    return g, th, w


def test_ideal_and_external_gradient_and_boltzmann_minimum():
    g, th, w = _setup()
    rho0, pref = I.solvent_constants(I.SPCE_N0, g.mrso)
    kT = I.kT()
    dv = (12. / 6) ** 3
    su = I.synthetic_solute(3, (12., 12., 12.), seed=1)
    vext = OS.vext_lj_coulomb((6, 6, 6), (12., 12., 12.), th, g.nphi, g.npsi, g.mrso, I.SPCE_SITES, su, 20 * kT)
    rng = np.random.default_rng(2)
    xi = rng.uniform(0.5, 1.5, (g.N, g.no))
    zero = np.zeros_like(xi)
    t, grad = OS.energy_terms(xi, zero, vext, w, kT, rho0, dv, pref)
    d = rng.standard_normal(xi.shape)
    for h in (1e-4, 1e-5):
        fp, _ = OS.energy_terms(xi + h * d, zero, vext, w, kT, rho0, dv, pref)
        fm, _ = OS.energy_terms(xi - h * d, zero, vext, w, kT, rho0, dv, pref)
        fd = (fp[0] - fm[0]) / (2 * h)
        assert abs(fd - (grad * d).sum()) <= 1e-7 * abs(fd)
    # without the excess term the minimum is rho = rho0 exp(-vext / kT)
    xb = np.exp(-vext / (2 * kT))
    _, gb = OS.energy_terms(xb, zero, vext, w, kT, rho0, dv, pref)
    assert np.abs(gb).max() <= 1e-12 * np.abs(grad).max()


def test_excess_gradient_is_exact_for_a_symmetric_cq():
    n, box, mmax, mrso, dq = (8, 8, 8), (10., 10., 10.), 2, 2, 0.05
    g = O.Oracle(n, box, mmax, mrso)
    idx, tab = I.isotropic_cq(mmax, mrso, I.nq_for(n, box, dq), dq, amplitude=1e-3)
    g.set_luc(idx, tab, dq)
    _, _, w = g.angular()
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    rng = np.random.default_rng(5)
    xi = rng.uniform(0.9, 1.1, (g.N, g.no))

    def ff_and_grad(x):
        p = g.conv_execute(g.angl2proj(O.delta_rho(x, rho0)))
        vexc = g.proj2angl(p).reshape(g.N, g.no)
        df, ff = O.delta_f(x, vexc, w, rho0, pref)
        t, gr = OS.energy_terms(x, vexc, None, w, 1.0, rho0, 0.0, pref)  # dv = 0: excess only
        assert abs(t[3] - ff) <= 1e-12 * abs(ff)
        assert np.abs(gr - 2 * pref * w[None, :] * df).max() <= 1e-13 * np.abs(gr).max()
        return ff, gr

    ff, gr = ff_and_grad(xi)
    assert ff > 0  # convex: c(q) <= 0
    d = rng.standard_normal(xi.shape)
    errs = []
    for h in (1e-4, 1e-5):
        fp, _ = ff_and_grad(xi + h * d)
        fm, _ = ff_and_grad(xi - h * d)
        fd = (fp - fm) / (2 * h)
        errs.append(abs(fd - (gr * d).sum()) / abs(fd))
    assert errs[1] < 1e-6 and errs[1] < errs[0] / 50  # second-order convergence


def test_synthetic_solute_follows_its_recipe():
    box = (30.0, 30.0, 30.0)
    su = I.synthetic_solute(12, box, seed=3)
    assert su.shape == (12, 6)
    assert abs(su[:, 0].sum()) < 1e-14  # neutral
    assert np.all((su[:, 1] >= 2.5) & (su[:, 1] <= 4.0))
    assert np.all((su[:, 2] >= 0.1) & (su[:, 2] <= 1.0))
    assert np.all(np.abs(su[:, 3:6] - 15.0) <= 5.0)  # central 10 A cube
    assert np.array_equal(su, I.synthetic_solute(12, box, seed=3))
    assert not np.array_equal(su, I.synthetic_solute(12, box, seed=4))


def test_isotropic_cq_has_only_the_zero_entry():
    idx, tab = I.isotropic_cq(3, 2, 50, 0.05, amplitude=2e-3, s=1.5)
    zero = (idx == 0).all(axis=0)
    assert zero.sum() == 1
    q = np.arange(50) * 0.05
    assert np.allclose(tab[zero][0], -2e-3 * np.exp(-1.5 * q * q), rtol=0, atol=1e-18)
    assert not np.any(tab[~zero])


def test_solvent_constants_match_the_tip3p_helper():
    assert I.solvent_constants(I.TIP3P_N0, 2) == pytest.approx(I.tip3p_constants(2), rel=1e-15)
    rho0, pref = I.solvent_constants(I.SPCE_N0, 2)
    assert pref == pytest.approx(-I.kT() / rho0, rel=1e-14)  # -2 kT 4 pi^2 / (mrso n0) = -kT / rho0
