"""The C-ABI library on a machine without a GPU: it loads, exports every
entry point include/mdft_gb300.h declares, and its host-side set-up (grids,
orientation/projection map, Wigner table) equals the oracle's.  No compute
entry point is called here."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from mini_mdft_gb300 import _lib
from mini_mdft_gb300 import inputs as I


@pytest.fixture(scope="module")
def L():
    from mini_mdft_gb300 import build
    build.build()
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    declared = _lib.header_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(_lib.SIGNATURES), "binding table out of sync with the header"
    assert L.mdft_abi_version() == 1


@pytest.mark.parametrize("n,box,mmax,mrso", [((8, 6, 5), (10., 12., 9.), 3, 2),
                                             ((2, 2, 2), (1., 1., 1.), 10, 10),
                                             ((64, 64, 64), (30., 30., 30.), 3, 2),
                                             ((5, 4, 3), (1., 2., 3.), 5, 1)])
def test_host_tables_equal_oracle(L, n, box, mmax, mrso):
    import mini_mdft_gb300 as M
    sg, ag = M.SpatialGrid(n, box), M.AngularGrid(mmax, mrso)
    mp = M.OrientationProjectionMap(ag)
    o = O.Oracle(n, box, mmax, mrso)
    kx, ky, kz = o.kvectors()
    assert np.array_equal(sg.m_kx, kx) and np.array_equal(sg.m_ky, ky) and np.array_equal(sg.m_kz, kz)
    th, wth, w = o.angular()
    assert np.array_equal(ag.m_thetaofntheta, th)
    assert np.array_equal(ag.m_wthetaofntheta, wth)
    assert np.array_equal(ag.m_w, w)
    om = o.opmap()
    for k, v in (("p", mp.p()), ("m", mp.m()), ("mup", mp.mup()), ("mu", mp.mu()), ("mu2", mp.mu2())):
        assert np.array_equal(v, om[k]), k
    assert np.abs(mp.wigner_small_d() - om["wigner"]).max() <= 2e-16


@pytest.mark.parametrize("args,msg", [
    ((4, 4, 4, 1.0, 1.0, 1.0, 0, 2), "mmax must be greater than zero"),
    ((4, 4, 4, 1.0, 1.0, 1.0, 3, 0), "molrotsymorder must be greater than zero"),
    ((4, 4, 4, -1.0, 1.0, 1.0, 3, 2), "negative length"),
    ((0, 4, 4, 1.0, 1.0, 1.0, 3, 2), "grid nodes"),
    ((4, 4, 4, 1.0, 1.0, 1.0, 11, 2), "not supported"),
])
def test_grid_errors_are_status_codes(L, args, msg):
    h = C.c_void_p()
    rc = L.mdft_grid_create(C.byref(h), *args)
    assert rc != 0
    assert msg in L.mdft_last_error().decode()
    assert not h.value


def test_null_arguments_rejected_without_gpu(L):
    assert L.mdft_grid_info(None, None) == 1
    assert b"NULL" in L.mdft_last_error()
    assert L.mdft_opt_angl2proj(None, None, None, None) == 1
    assert L.mdft_conv_execute(None, None, None) == 1
    assert L.mdft_get_delta_rho(None, None, 0, 0.3, 7, None) == 1
    assert b"precision" in L.mdft_last_error()
    assert L.mdft_get_delta_f(None, None, None, None, None, 0, 0, 0.3, 0.3, 0, None) == 1


def test_luc_index_counts_match_npluc():
    # npluc per mmax of the 3-site water models (common/MDFT_Solvent.hpp:433)
    for mmax, npl in enumerate(I.NPLUC):
        idx = I.luc_index(mmax, 2)
        assert idx.shape == (5, npl)
        assert tuple(idx[:, 0]) == (mmax, mmax, (mmax // 2) * 2, (mmax // 2) * 2, mmax)
        assert tuple(idx[:, -1]) == (0, 0, 0, 0, 0)


def test_nq_formula_matches_oracle():
    for n, box, nq in [((32,) * 3, (20.,) * 3, 873), ((64,) * 3, (30.,) * 3, 1163),
                       ((96,) * 3, (40.,) * 3, 1308), ((128,) * 3, (50.,) * 3, 1395)]:
        assert I.nq_for(n, box, 0.01) == nq
        o = O.Oracle(n if n[0] < 64 else (4, 4, 4), box, 3, 2)
        if n[0] < 64:
            assert o.nq_for_dq(0.01) == nq


def test_luc_file_round_trip(tmp_path):
    idx, tab = I.synthetic_cq(3, 2, 50, 0.01)
    path = str(tmp_path / "ck")
    I.write_luc_file(path, idx, tab, 0.01)
    idx2, tab2, dq = I.read_luc_file(path, idx.shape[1])
    assert np.array_equal(idx, idx2)
    assert np.array_equal(tab, tab2)
    assert abs(dq - 0.01) < 1e-15


def test_generators_are_seeded():
    a = I.synthetic_delta_rho(10, 3, 2)
    b = I.synthetic_delta_rho(10, 3, 2)
    assert np.array_equal(a, b) and a.shape == (10, 4, 7, 3)
    assert a.min() >= -0.1 and a.max() <= 0.1
    x = I.synthetic_xi(10, 3, 2)
    assert x.min() >= 0.9 and x.max() <= 1.1


def test_luc_write_read_round_trip(L, tmp_path):
    """C++ Luc writer and reader (host only): the written file is the one the
    Python writer produces, byte for byte, both readers get the table back
    exactly, and a smaller |q_max| keeps int(qmax/dq + 0.5) + 2 rows."""
    import mini_mdft_gb300 as M
    idx, tab = I.synthetic_cq(3, 2, 40, 0.01)
    a, b = tmp_path / "cpp.luc", tmp_path / "py.luc"
    M.luc_write(a, idx, tab, 0.01, header="synthetic c(q) table")
    I.write_luc_file(str(b), idx, tab, 0.01, header="synthetic c(q) table")
    assert a.read_bytes() == b.read_bytes()
    i2, t2, dq2 = I.read_luc_file(str(a), idx.shape[1])
    assert np.array_equal(i2, idx) and np.array_equal(t2, tab) and abs(dq2 - 0.01) < 1e-15
    qmax = 0.37
    i3, t3, dq3 = M.luc_read(a, idx.shape[1], qmax)
    nq = int(qmax / dq3 + 0.5) + 2
    assert np.array_equal(i3, idx) and t3.shape == (idx.shape[1], nq)
    assert np.array_equal(t3, tab[:, :nq])
    with pytest.raises(M.MdftError, match="does not exist") as e:
        M.luc_read(tmp_path / "missing", idx.shape[1], qmax)
    assert e.value.code == 3
    with pytest.raises(M.MdftError, match="fewer q rows"):
        M.luc_read(a, idx.shape[1], 1.0)
