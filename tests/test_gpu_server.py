"""The job server (mdft_server_*): jobs of several shapes and uneven lengths,
submitted from several host threads, must return exactly what the same
steps give through the operator API one field at a time (the server batches
same-shape jobs, replays captured graphs and compacts finished slots, none of
which may change a job's numbers), and the latency statistics must cover
every job."""
import threading

import numpy as np
import pytest

from mini_mdft_gb300 import inputs as I

pytestmark = pytest.mark.gpu

DQ = 0.01
# (grid, box, mmax, mrso): two shapes share a solvent, one has its own
SHAPES = [((12, 10, 8), (12., 10., 9.), 3, 2), ((8, 8, 8), (10., 10., 10.), 3, 2),
          ((6, 7, 5), (9., 9., 8.), 2, 1)]


def _solvent_table(mmax, mrso):
    nq = max(I.nq_for(n, box, DQ) for n, box, m, r in SHAPES if (m, r) == (mmax, mrso))
    return I.synthetic_cq(mmax, mrso, nq + 2, DQ)


def _direct(M, n, box, mmax, mrso, table, rho0, pref, xi0, n_steps, step, prec):
    """The job's steps through the operator API, one field."""
    import torch
    idx, tab = table
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, precision=prec)
    conv = M.Convolution.from_table(idx, tab, DQ, sg, ag, precision=prec)
    rd, cd = (torch.float32, torch.complex64) if prec == "f32" else (torch.float64, torch.complex128)
    xi = torch.from_numpy(xi0).to("cuda", rd)
    w = torch.from_numpy(ag.m_w)
    p = torch.zeros((ag.m_np,) + tuple(n), dtype=cd, device="cuda")
    vexc, df = torch.zeros_like(xi), torch.zeros_like(xi)
    ffs = []
    for _ in range(n_steps):
        opt.angl2proj_from_xi(xi, rho0, p)
        conv.execute(p)
        opt.proj2angl(p, vexc)
        ffs.append(M.get_delta_f(xi, vexc, w, df, rho0, pref))
        xi = xi - step * df
    torch.cuda.synchronize()
    return xi.cpu().numpy(), np.array(ffs)


@pytest.mark.parametrize("prec", ["f64", "f64df", "f32"])
def test_server_jobs_match_operator_api(gpu_lib, prec):
    M = gpu_lib
    rho0, pref = I.tip3p_constants(2)
    srv = M.Server(precision=prec, max_batch=3)
    tables = {}
    solvent = {}
    for n, box, mmax, mrso in SHAPES:
        if (mmax, mrso) not in solvent:
            tables[(mmax, mrso)] = _solvent_table(mmax, mrso)
            idx, tab = tables[(mmax, mrso)]
            solvent[(mmax, mrso)] = srv.add_solvent(mmax, mrso, idx, tab, DQ, rho0, pref)
    rng = np.random.default_rng(11)
    jobs = []
    for i in range(9):  # shape 0 gets 5 jobs: more than one batch of 3
        n, box, mmax, mrso = SHAPES[[0, 0, 1, 0, 2, 0, 1, 0, 2][i]]
        nt, nphi, npsi, _, _ = I.angular_counts(mmax, mrso)
        xi0 = rng.uniform(0.9, 1.1, (n[0] * n[1] * n[2], nt, nphi, npsi))
        if prec == "f32":
            xi0 = xi0.astype(np.float32)
        jobs.append(dict(shape=(n, box, mmax, mrso), xi0=xi0, n_steps=int(rng.integers(2, 7)),
                         step=float(rng.uniform(1e-3, 5e-3))))
    ids = [None] * len(jobs)

    def submit(lo, hi):
        for i in range(lo, hi):
            j = jobs[i]
            n, box, mmax, mrso = j["shape"]
            ids[i] = srv.submit(solvent[(mmax, mrso)], n, box, j["xi0"], j["n_steps"], j["step"])

    threads = [threading.Thread(target=submit, args=(a, a + 3)) for a in (0, 3, 6)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    tol_xi, tol_ff = (1e-5, 1e-5) if prec == "f32" else (1e-12, 1e-12)
    for i, j in enumerate(jobs):
        xi, ff, lat = srv.wait(ids[i])
        n, box, mmax, mrso = j["shape"]
        xr, fr = _direct(M, n, box, mmax, mrso, tables[(mmax, mrso)], rho0, pref, j["xi0"],
                         j["n_steps"], j["step"], prec)
        assert lat > 0
        assert np.all(np.isfinite(ff)) and len(ff) == j["n_steps"]
        assert np.max(np.abs(ff - fr)) <= tol_ff * np.max(np.abs(fr))
        assert np.max(np.abs(xi - xr)) <= tol_xi * np.max(np.abs(xr))
    st = srv.stats()
    assert st["done"] == len(jobs)
    assert 0 < st["p50_s"] <= st["p99_s"]
    assert st["solves_per_s"] > 0 and st["groups"] == len(SHAPES) and st["peak_bytes"] > 0
    # every active count's step graph is captured when its group is made:
    # steps replay graphs
    assert st["graph_steps"] > 0 and st["direct_steps"] == 0
    srv.close()


def test_server_budget_too_small(gpu_lib):
    M = gpu_lib
    rho0, pref = I.tip3p_constants(2)
    srv = M.Server(precision="f64", max_batch=2, hbm_budget_bytes=1 << 20)
    idx, tab = _solvent_table(3, 2)
    sid = srv.add_solvent(3, 2, idx, tab, DQ, rho0, pref)
    n, box = (12, 10, 8), (12., 10., 9.)
    xi0 = np.ones((n[0] * n[1] * n[2], 4, 7, 3))
    jid = srv.submit(sid, n, box, xi0, 2, 1e-3)
    with pytest.raises(M.MdftError, match="budget"):
        srv.wait(jid)
    with pytest.raises(M.MdftError, match="unknown job"):
        srv.wait(jid)
    srv.close()


# solute jobs: (grid, box, mmax, mrso, solute sites, solute seed)
SOLUTE_JOBS = [((12, 10, 8), (12., 10., 9.), 2, 2, 5, 11), ((12, 10, 8), (12., 10., 9.), 2, 2, 8, 12),
               ((8, 8, 8), (10., 10., 10.), 2, 2, 7, 13), ((10, 12, 8), (11., 12., 10.), 1, 1, 4, 14),
               ((10, 12, 8), (11., 12., 10.), 1, 1, 9, 15)]
SOLUTE_DQ = 0.05


def _solute_alone(M, n, box, mmax, mrso, table, su, max_iter, gtol, prec):
    """The job alone: the single-field minimiser (mdft_solver_minimize)."""
    import torch
    idx, tab = table
    rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
    kT = I.kT()
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    opt = M.OrientationProjectionTransform(sg, ag, precision=prec)
    conv = M.Convolution.from_table(idx, tab, SOLUTE_DQ, sg, ag, precision=prec)
    vext = M.solute_vext(sg, ag, I.SPCE_SITES, su, 100 * kT)
    solver = M.Solver(opt, conv, vext, kT=kT, rho0=rho0, prefactor=pref, history=5)
    xi = torch.ones_like(vext)
    trace = solver.minimize(xi, max_iter=max_iter, gtol=gtol)
    return xi.cpu().numpy().reshape(-1), trace


@pytest.mark.parametrize("prec", ["f64df", "f32"])
def test_solute_jobs_match_the_single_minimiser(gpu_lib, prec):
    """Solute jobs of three shapes and two angular grids, submitted from three
    threads to a server with two slots per group (so finished jobs' slots are
    refilled and compacted mid-run): every job's trace and final field equal
    the same job run alone through the single-field minimiser."""
    M = gpu_lib
    kT = I.kT()
    max_iter, gtol = 12, 1e-9
    tables, alone = {}, []
    for n, box, mmax, mrso, ns, seed in SOLUTE_JOBS:
        if (mmax, mrso) not in tables:
            nq = max(I.nq_for(n2, b2, SOLUTE_DQ) for n2, b2, m2, r2, _, _ in SOLUTE_JOBS if (m2, r2) == (mmax, mrso))
            tables[(mmax, mrso)] = I.isotropic_cq(mmax, mrso, nq + 2, SOLUTE_DQ, amplitude=1e-3)
        su = I.synthetic_solute(ns, box, seed=seed)
        alone.append(_solute_alone(M, n, box, mmax, mrso, tables[(mmax, mrso)], su, max_iter, gtol, prec))
    srv = M.Server(precision=prec, max_batch=2)
    solvent = {}
    for (mmax, mrso), (idx, tab) in tables.items():
        rho0, pref = I.solvent_constants(I.SPCE_N0, mrso)
        sid = srv.add_solvent(mmax, mrso, idx, tab, SOLUTE_DQ, rho0, pref)
        srv.set_solvent_model(sid, I.SPCE_SITES, kT, 100 * kT)
        solvent[(mmax, mrso)] = sid
    ids = [None] * len(SOLUTE_JOBS)

    def submit(part):
        for i in part:
            n, box, mmax, mrso, ns, seed = SOLUTE_JOBS[i]
            ids[i] = srv.submit_solute(solvent[(mmax, mrso)], n, box, I.synthetic_solute(ns, box, seed=seed),
                                       max_iter=max_iter, gtol=gtol)

    threads = [threading.Thread(target=submit, args=(part,)) for part in ([0, 3], [1, 4], [2])]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, jid in enumerate(ids):
        xi, trace, status, lat = srv.wait_solute(jid)
        xa, ta = alone[i]
        assert trace.shape == ta.shape, i
        assert np.array_equal(trace, ta), (i, np.abs(trace - ta).max())
        assert np.array_equal(xi.reshape(-1), xa), i
        assert lat > 0
        assert np.all(np.diff(trace[:, 0]) <= 0)
    st = srv.stats()
    assert st["done"] == len(SOLUTE_JOBS)
    srv.close()


def test_solute_job_needs_a_solvent_model(gpu_lib):
    M = gpu_lib
    idx, tab = I.isotropic_cq(1, 1, 40, SOLUTE_DQ)
    srv = M.Server(precision="f64", max_batch=2)
    rho0, pref = I.solvent_constants(I.SPCE_N0, 1)
    sid = srv.add_solvent(1, 1, idx, tab, SOLUTE_DQ, rho0, pref)
    with pytest.raises(M.MdftError):
        srv.submit_solute(sid, (4, 4, 4), (8., 8., 8.), I.synthetic_solute(2, (8., 8., 8.)))
    srv.close()
