"""get_delta_f (common/MDFT_Solvent.hpp:617-660) on grids that do not divide
evenly among the energy kernel's CTAs.  Each CTA takes one contiguous run of
grid points and leaves one partial sum, so these cases exercise:

- a last run shorter than the others;
- fewer grid points than CTAs of one wave;
- one grid point;
- more orientations than threads per CTA;
- a single orientation.

All three forms go through the C ABI and are checked against the oracle.
A repeated call must give the same ff bit for bit."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from _util import rel_err

pytestmark = pytest.mark.gpu

# (grid points, orientations)
CASES = [(1, 84), (33, 5), (1217, 84), (45007, 84), (2503, 330), (300001, 1)]
DF_TOL = {0: 1e-14, 1: 1e-6, 2: 1e-13}  # MDFT_F64, MDFT_F32, MDFT_F64_DF


def _p(t):
    return C.c_void_p(t.data_ptr())


@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("nxyz,no", CASES)
def test_delta_f_on_uneven_runs(gpu_lib, nxyz, no, prec):
    import torch
    L = gpu_lib.lib()
    rng = np.random.default_rng(7 * nxyz + no)
    xi = rng.uniform(0.0, 1.0, (nxyz, no))
    vexc = rng.uniform(-1.0, 1.0, (nxyz, no))
    w = rng.uniform(0.0, 1.0, no)
    rho0, pref = 0.3, 0.334
    dt = torch.float32 if prec == 1 else torch.float64
    if prec == 1:  # FP32 fields: the oracle sees the rounded inputs; its sum stays FP64
        xi = xi.astype(np.float32).astype(np.float64)
        vexc = vexc.astype(np.float32).astype(np.float64)
    df_ref, ff_ref = O.delta_f(xi, vexc, w, rho0, pref)
    xt = torch.from_numpy(xi).to("cuda", dt)
    vt = torch.from_numpy(vexc).to("cuda", dt)
    wt = torch.from_numpy(w).to("cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    ffs = []
    for _ in range(2):
        df = torch.full_like(xt, 7.0)  # every element must be written
        ff = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
        rc = L.mdft_get_delta_f(_p(xt), _p(vt), _p(wt), _p(df), _p(ff), nxyz, no, rho0, pref, prec, stream)
        assert rc == 0, L.mdft_last_error()
        torch.cuda.synchronize()
        assert rel_err(df.double().cpu().numpy(), df_ref) < DF_TOL[prec]
        ffs.append(float(ff.item()))
    assert abs(ffs[0] - ff_ref) <= 1e-12 * abs(ff_ref)
    assert ffs[1] == ffs[0]  # deterministic reduction
