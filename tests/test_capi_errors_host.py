"""Error paths of the C ABI that need no GPU: every entry point below checks
its arguments before its first CUDA call.  Each check must return a status
code and leave the reference's kind of message in mdft_last_error().

Covered: get_delta_f and its allocation-free variant (including the fixed
scratch limit), the external potential, the minimiser and the job server.
Errors cross the ABI as status codes, never as exceptions, and a NULL
handle passed to a destroy call is a no-op, as for free()."""
import ctypes as C

import numpy as np
import pytest

from mini_mdft_gb300 import _lib
from mini_mdft_gb300 import inputs as I

FAKE = C.c_void_p(256)  # a non-NULL device address that no failing check dereferences
MAX_NOALLOC_POINTS = 1 << 21


@pytest.fixture(scope="module")
def L():
    from mini_mdft_gb300 import build
    build.build()
    return _lib.lib()


def _err(L):
    return L.mdft_last_error().decode()


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def test_get_delta_f_argument_checks(L):
    assert L.mdft_get_delta_f(FAKE, FAKE, FAKE, FAKE, FAKE, 10, 84, 0.3, 0.3, 3, None) == 1
    assert "precision must be" in _err(L)
    assert L.mdft_get_delta_f(FAKE, FAKE, FAKE, FAKE, FAKE, 10, 0, 0.3, 0.3, 0, None) == 1
    assert "angular grid size must be positive" in _err(L)
    assert L.mdft_get_delta_f(None, FAKE, FAKE, FAKE, FAKE, 10, 84, 0.3, 0.3, 2, None) == 1
    assert "NULL argument" in _err(L)


def test_noalloc_rejects_grids_beyond_the_fixed_scratch_before_touching_the_gpu(L):
    rc = L.mdft_get_delta_f_noalloc(FAKE, FAKE, FAKE, FAKE, FAKE, MAX_NOALLOC_POINTS + 1, 1, 0.3, 0.3, 0, None)
    assert rc == 4  # MDFT_ERR_UNSUPPORTED
    assert "fixed scratch limit" in _err(L)
    assert L.mdft_get_delta_f_noalloc(FAKE, FAKE, FAKE, FAKE, FAKE, 10, 84, 0.3, 0.3, -1, None) == 1
    assert "precision must be" in _err(L)
    assert L.mdft_get_delta_f_noalloc(FAKE, FAKE, FAKE, FAKE, None, 10, 84, 0.3, 0.3, 0, None) == 1
    assert "NULL argument" in _err(L)


def test_scratch_pool_argument_check(L):
    assert L.mdft_scratch_pool(None) == 1
    assert "NULL argument" in _err(L)


def test_vext_argument_checks(L):
    g = C.c_void_p()
    assert L.mdft_grid_create(C.byref(g), 4, 4, 4, 10.0, 10.0, 10.0, 3, 2) == 0
    try:
        sv = np.ascontiguousarray(I.SPCE_SITES)
        su = I.synthetic_solute(3, (10.0, 10.0, 10.0), seed=1)
        assert L.mdft_vext_lj_coulomb(None, _dp(sv), 3, _dp(su), 3, 100.0, FAKE, None) == 1
        assert "NULL argument" in _err(L)
        assert L.mdft_vext_lj_coulomb(g, _dp(sv), 3, _dp(su), 3, 100.0, None, None) == 1
        assert "NULL argument" in _err(L)
        assert L.mdft_vext_lj_coulomb(g, _dp(sv), 3, None, 3, 100.0, FAKE, None) == 1
        assert "NULL argument" in _err(L)
        assert L.mdft_vext_lj_coulomb(g, _dp(sv), 0, _dp(su), 3, 100.0, FAKE, None) == 1
        assert "site counts" in _err(L)
        assert L.mdft_vext_lj_coulomb(g, _dp(sv), 3, _dp(su), -1, 100.0, FAKE, None) == 1
        assert "site counts" in _err(L)
        assert L.mdft_vext_lj_coulomb(g, _dp(sv), 3, _dp(su), 3, 0.0, FAKE, None) == 1
        assert "vmax must be positive" in _err(L)
    finally:
        assert L.mdft_grid_destroy(g) == 0


def test_solver_argument_checks(L):
    h = C.c_void_p()
    assert L.mdft_solver_create(None, FAKE, FAKE, FAKE, 2.5, 0.001, -1.0, 5) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_solver_create(C.byref(h), None, FAKE, FAKE, 2.5, 0.001, -1.0, 5) == 1
    assert "NULL argument" in _err(L) and not h.value
    terms = np.zeros(5)
    assert L.mdft_solver_energy(None, FAKE, FAKE, _dp(terms), None) == 1
    assert "NULL argument" in _err(L)
    trace = np.zeros(10)
    it = C.c_int()
    assert L.mdft_solver_minimize(None, FAKE, 1, 0.0, 0.0, _dp(trace), C.byref(it), None) == 1
    assert "NULL argument" in _err(L)
    st = C.c_int(7)
    assert L.mdft_solver_status(None, C.byref(st)) == 1
    assert "NULL argument" in _err(L) and st.value == 7
    assert L.mdft_solver_destroy(None) == 0


def test_server_argument_checks(L):
    h = C.c_void_p()
    assert L.mdft_server_create(None, 0, 1, 0) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_server_create(C.byref(h), 3, 1, 0) == 1
    assert "precision must be" in _err(L) and not h.value
    assert L.mdft_server_create(C.byref(h), 0, 0, 0) == 1
    assert "max_batch must be 1..1024" in _err(L) and not h.value
    assert L.mdft_server_create(C.byref(h), 2, 1025, 0) == 1
    assert "max_batch must be 1..1024" in _err(L) and not h.value
    jid = C.c_longlong()
    sid = C.c_int()
    assert L.mdft_server_add_solvent(None, 3, 2, None, None, 252, 100, 0.01, 0.3, 0.3, C.byref(sid)) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_server_submit(None, 0, 4, 4, 4, 1.0, 1.0, 1.0, FAKE, 2, 1e-3, C.byref(jid)) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_server_wait(None, 0, None, None, None) == 1
    assert "NULL argument" in _err(L)
    sites = np.ascontiguousarray(I.SPCE_SITES)
    assert L.mdft_server_set_solvent_model(None, 0, _dp(sites), 3, 2.5, 100.0) == 1
    assert "NULL argument" in _err(L)
    xi0 = np.ones(8)
    assert L.mdft_server_submit_solute(None, 0, 4, 4, 4, 1.0, 1.0, 1.0, None, 0, _dp(xi0), 10, 1e-5,
                                       C.byref(jid)) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_server_wait_solute(None, 0, None, None, None, None, None) == 1
    assert "NULL argument" in _err(L)
    out = np.zeros(8)
    assert L.mdft_server_stats(None, _dp(out)) == 1
    assert "NULL argument" in _err(L)
    assert L.mdft_server_destroy(None) == 0
