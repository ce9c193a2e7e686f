"""The dense angular matrices the tensor-core path multiplies by
(mdft_grid_ang_matrices, host-only) reproduce the oracle's angl2proj and
proj2angl (MDFT_OrientationProjectionTransform.hpp:270-380, :391-484) at one
grid point: p = A o and o = B p for random o and p, on the angular grids of
the GPU parity tests."""
import numpy as np
import pytest

import oracle as O
from mini_mdft_gb300 import api as A
from tests._util import rel_err

GRIDS = [(1, 1), (2, 1), (2, 2), (3, 1), (3, 2), (3, 3), (4, 2), (5, 2), (6, 2), (5, 3)]


@pytest.mark.parametrize("mmax,mrso", GRIDS)
def test_dense_matrices_equal_oracle(mmax, mrso):
    ag = A.AngularGrid(mmax, mrso)
    a2p, p2a = A.OrientationProjectionMap(ag).dense_matrices()
    o = O.Oracle((1, 1, 1), (1.0, 1.0, 1.0), mmax, mrso)
    rng = np.random.default_rng(mmax * 10 + mrso)
    x = rng.uniform(-1, 1, (1, o.ntheta, o.nphi, o.npsi))
    p_ref = o.angl2proj(x).reshape(o.np)
    p = a2p @ x.ravel()
    assert rel_err(p[0::2] + 1j * p[1::2], p_ref) < 1e-14
    q = rng.normal(size=o.np) + 1j * rng.normal(size=o.np)
    qq = np.zeros(2 * o.np)
    qq[0::2], qq[1::2] = q.real, q.imag
    o_ref = o.proj2angl(q.reshape(o.np, 1, 1, 1)).ravel()
    assert rel_err(p2a @ qq, o_ref) < 1e-14
