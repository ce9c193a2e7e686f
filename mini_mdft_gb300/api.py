"""Python mirror of the reference's operator API for the convolution hot path.

Names, argument order and meaning follow the reference's C++ classes so the
tests read like the reference's own unit tests:

* ``SpatialGrid(n_nodes, length)``        -- common/MDFT_Grid.hpp:158-239
* ``AngularGrid(mmax, molrotsymorder)``   -- common/MDFT_Grid.hpp:241-470
* ``OrientationProjectionMap(ag)``        -- common/MDFT_OrientationProjectionTransform.hpp:20-156
* ``OrientationProjectionTransform(sg, ag, map)`` with ``angl2proj(o, p)`` and
  ``proj2angl(p, o)``                     -- :161-485
* ``Convolution(filename, sg, ag, map, np_luc)`` with ``execute(p)``,
  ``gamma_p_map()``, ``mnmunukhi_q()``, ``dq()`` -- common/MDFT_Convolution.hpp:20-549
* ``get_delta_rho(xi, delta_rho, rho0)`` and
  ``get_delta_f(xi, vexc, w, delta_f, rho0, prefactor) -> ff``
                                           -- common/MDFT_Solvent.hpp:578-660

Fields are torch CUDA tensors in the reference layouts (o: (N, ntheta, nphi,
npsi) real; p: (np, nx, ny, nz) complex).  float64/complex128 selects the
plain FP64 form, float32/complex64 the mixed form (the reference's
ScalarType=float instantiation with FP64 recursions and energy sum).  Work
goes to torch's current CUDA stream and is asynchronous, as Kokkos kernels
are; errors raise ``MdftError`` (a RuntimeError, like Throw_If).
Every call goes through the C ABI of ``libmdft_gb300.so``.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import MDFT_F32, MDFT_F64, MDFT_F64_DF, MdftError, check, lib

__all__ = [
    "SpatialGrid", "AngularGrid", "OrientationProjectionMap",
    "OrientationProjectionTransform", "Convolution", "get_delta_rho",
    "get_delta_f", "MdftError", "MDFT_F64", "MDFT_F32", "MDFT_F64_DF",
]

_PRECISIONS = {"f64": MDFT_F64, "f32": MDFT_F32, "f64df": MDFT_F64_DF,
               MDFT_F64: MDFT_F64, MDFT_F32: MDFT_F32, MDFT_F64_DF: MDFT_F64_DF}


def _precision_arg(precision):
    try:
        return _PRECISIONS[precision]
    except (KeyError, TypeError):
        raise MdftError(1, "precision must be 'f64', 'f32' or 'f64df'")


def _torch():
    import torch
    return torch


def _stream():
    torch = _torch()
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dptr(t):
    return C.c_void_p(t.data_ptr())


def _np_d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _np_i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class _GridHandle:
    def __init__(self, n, box, mmax, mrso):
        h = C.c_void_p()
        check(lib().mdft_grid_create(C.byref(h), int(n[0]), int(n[1]), int(n[2]),
                                     float(box[0]), float(box[1]), float(box[2]),
                                     int(mmax), int(mrso)))
        self.h = h
        v = np.zeros(11, np.int32)
        check(lib().mdft_grid_info(h, _np_i(v)))
        (self.nx, self.ny, self.nz, self.mmax, self.mrso, self.ntheta, self.nphi,
         self.npsi, self.no, self.np, self.np_new) = [int(x) for x in v]

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mdft_grid_destroy(self.h)
            self.h = None


class SpatialGrid:
    """SpatialGrid<ExecutionSpace, ScalarType>(n_nodes, length)."""

    def __init__(self, n_nodes, length):
        self.m_n_nodes = tuple(int(v) for v in n_nodes)
        self.m_length = tuple(float(v) for v in length)
        self.m_nx, self.m_ny, self.m_nz = self.m_n_nodes
        self.m_lx, self.m_ly, self.m_lz = self.m_length
        g = _GridHandle(self.m_n_nodes, self.m_length, 1, 1)
        kx, ky, kz = np.zeros(self.m_nx), np.zeros(self.m_ny), np.zeros(self.m_nz)
        check(lib().mdft_grid_kvectors(g.h, _np_d(kx), _np_d(ky), _np_d(kz)))
        self.m_kx, self.m_ky, self.m_kz = kx, ky, kz
        self.m_dl = tuple(l / n for l, n in zip(self.m_length, self.m_n_nodes))
        self.m_v = float(np.prod(self.m_length))
        self.m_dv = float(np.prod(self.m_dl))


class AngularGrid:
    """AngularGrid<ExecutionSpace, ScalarType>(mmax, molrotsymorder)."""

    def __init__(self, mmax, molrotsymorder):
        g = _GridHandle((1, 1, 1), (1.0, 1.0, 1.0), mmax, molrotsymorder)
        self.m_mmax, self.m_molrotsymorder = g.mmax, g.mrso
        self.m_ntheta, self.m_nphi, self.m_npsi = g.ntheta, g.nphi, g.npsi
        self.m_no, self.m_np = g.no, g.np
        th, wth, w = np.zeros(g.ntheta), np.zeros(g.ntheta), np.zeros(g.no)
        check(lib().mdft_grid_angular(g.h, _np_d(th), _np_d(wth), _np_d(w)))
        self.m_thetaofntheta, self.m_wthetaofntheta, self.m_w = th, wth, w
        self.m_quadrature_norm = 8.0 * np.pi * np.pi


class OrientationProjectionMap:
    """OrientationProjectionMap(angular_grid) with its getters."""

    def __init__(self, angular_grid):
        ag = angular_grid
        g = _GridHandle((1, 1, 1), (1.0, 1.0, 1.0), ag.m_mmax, ag.m_molrotsymorder)
        K = g.mmax // g.mrso
        self._p = np.zeros((g.mmax + 1, 2 * g.mmax + 1, K + 1), np.int32)
        self._arr = [np.zeros(g.np, np.int32) for _ in range(4)]
        self._wig = np.zeros((g.ntheta, g.np))
        check(lib().mdft_grid_opmap(g.h, _np_i(self._p), *[_np_i(a) for a in self._arr],
                                    _np_d(self._wig)))
        self.angular_grid = ag

    def p(self):
        return self._p

    def m(self):
        return self._arr[0]

    def mup(self):
        return self._arr[1]

    def mu(self):
        return self._arr[2]

    def mu2(self):
        return self._arr[3]

    def wigner_small_d(self):
        return self._wig

    def dense_matrices(self):
        """(a2p, p2a): the angular transforms at one grid point as dense
        real FP64 matrices, a2p (2 np, no) and p2a (no, 2 np); row 2 ip + c
        of a2p (column of p2a) is the real (c = 0) or imaginary (c = 1)
        part of projection ip (mdft_grid_ang_matrices).  No counterpart in
        the reference."""
        ag = self.angular_grid
        g = _GridHandle((1, 1, 1), (1.0, 1.0, 1.0), ag.m_mmax, ag.m_molrotsymorder)
        a2p = np.zeros((2 * g.np, g.no))
        p2a = np.zeros((g.no, 2 * g.np))
        check(lib().mdft_grid_ang_matrices(g.h, _np_d(a2p), _np_d(p2a)))
        return a2p, p2a


def _precision_of(dtype):
    torch = _torch()
    if dtype in (torch.float64, torch.complex128):
        return MDFT_F64
    if dtype in (torch.float32, torch.complex64):
        return MDFT_F32
    raise MdftError(1, "unsupported dtype %s" % dtype)


def _check_field(t, shape_numel, dtypes, name):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise MdftError(1, "%s must be a CUDA tensor" % name)
    if t.dtype not in dtypes:
        raise MdftError(1, "%s has dtype %s, expected one of %s" % (name, t.dtype, dtypes))
    if not t.is_contiguous():
        raise MdftError(1, "%s must be contiguous (LayoutRight)" % name)
    if t.numel() != shape_numel:
        raise MdftError(1, "%s has %d elements, expected %d" % (name, t.numel(), shape_numel))


class OrientationProjectionTransform:
    """OrientationProjectionTransform(spatial_grid, angular_grid, map).

    ``precision`` is "f64" (plain form), "f32" (mixed form) or "f64df" (FP64
    fields, double-float arithmetic on the FP32 pipes); the dtype of the
    tensors passed to angl2proj/proj2angl must match it (float64/complex128
    for "f64" and "f64df")."""

    def __init__(self, spatial_grid, angular_grid, map=None, precision="f64", batch=1):
        sg, ag = spatial_grid, angular_grid
        self._g = _GridHandle(sg.m_n_nodes, sg.m_length, ag.m_mmax, ag.m_molrotsymorder)
        self.precision = _precision_arg(precision)
        self.batch = int(batch)
        h = C.c_void_p()
        # batch > 1: `batch` same-shape fields per call, stored back to back
        # (mdft_opt_create_batched; no counterpart in the reference)
        check(lib().mdft_opt_create_batched(C.byref(h), self._g.h, self.precision, self.batch))
        self.h = h
        g = self._g
        self.N = g.nx * g.ny * g.nz
        self.ntheta, self.nphi, self.npsi, self.np, self.no = g.ntheta, g.nphi, g.npsi, g.np, g.no

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mdft_opt_destroy(self.h)
            self.h = None

    def _dtypes(self):
        torch = _torch()
        if self.precision == MDFT_F32:
            return (torch.float32,), (torch.complex64,)
        return (torch.float64,), (torch.complex128,)

    def angl2proj(self, o, p):
        rd, cd = self._dtypes()
        _check_field(o, self.N * self.batch * self.no, rd, "o")
        _check_field(p, self.N * self.batch * self.np, cd, "p")
        check(lib().mdft_opt_angl2proj(self.h, _dptr(o), _dptr(p), _stream()))

    def angl2proj_from_xi(self, xi, rho0, p):
        """get_delta_rho fused into angl2proj (delta_rho never stored)."""
        rd, cd = self._dtypes()
        _check_field(xi, self.N * self.batch * self.no, rd, "xi")
        _check_field(p, self.N * self.batch * self.np, cd, "p")
        check(lib().mdft_opt_angl2proj_from_xi(self.h, _dptr(xi), float(rho0), _dptr(p), _stream()))

    def proj2angl(self, p, o):
        rd, cd = self._dtypes()
        _check_field(o, self.N * self.batch * self.no, rd, "o")
        _check_field(p, self.N * self.batch * self.np, cd, "p")
        check(lib().mdft_opt_proj2angl(self.h, _dptr(p), _dptr(o), _stream()))


class Convolution:
    """Convolution(filename, spatial_grid, angular_grid, map, np_luc)."""

    def __init__(self, filename, spatial_grid, angular_grid, map=None, np_luc=None,
                 precision="f64", _table=None, batch=1):
        sg, ag = spatial_grid, angular_grid
        self._g = _GridHandle(sg.m_n_nodes, sg.m_length, ag.m_mmax, ag.m_molrotsymorder)
        self.precision = _precision_arg(precision)
        self.batch = int(batch)
        h = C.c_void_p()
        if _table is not None:
            idx, tab, dq = _table
            idx = np.ascontiguousarray(idx, np.int32)
            tab = np.ascontiguousarray(tab, np.complex128)
            np_luc_, nq = tab.shape
            check(lib().mdft_conv_create_batched(C.byref(h), self._g.h, _np_i(idx),
                                                 tab.ctypes.data_as(C.POINTER(C.c_double)),
                                                 np_luc_, nq, float(dq), self.precision,
                                                 self.batch))
        else:
            if self.batch != 1:
                raise ValueError("batched plans are built from a table (Convolution.from_table)")
            check(lib().mdft_conv_create_from_file(C.byref(h), self._g.h,
                                                   str(filename).encode(), int(np_luc),
                                                   self.precision))
        self.h = h
        v = np.zeros(3, np.int32)
        d = C.c_double()
        check(lib().mdft_conv_info(h, _np_i(v), C.byref(d)))
        self.npairs, self.np_new, self.nq = [int(x) for x in v]
        self._dq = d.value
        g = self._g
        self.N = g.nx * g.ny * g.nz
        self.np = g.np

    @classmethod
    def from_table(cls, luc_index, table, dq, spatial_grid, angular_grid, map=None,
                   precision="f64", batch=1):
        """Same operator from a c(q) table already in memory (Luc layout).
        batch > 1: p holds `batch` same-shape fields, (np, batch, nx, ny, nz)
        (mdft_conv_create_batched; no counterpart in the reference)."""
        return cls(None, spatial_grid, angular_grid, map, None, precision,
                   _table=(luc_index, table, dq), batch=batch)

    def __del__(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mdft_conv_destroy(self.h)
            self.h = None

    def _cdt(self):
        torch = _torch()
        return (torch.complex64,) if self.precision == MDFT_F32 else (torch.complex128,)

    def execute(self, deltarho_p):
        _check_field(deltarho_p, self.N * self.batch * self.np, self._cdt(), "deltarho_p")
        check(lib().mdft_conv_execute(self.h, _dptr(deltarho_p), _stream()))

    def execute_timed(self, deltarho_p, events):
        """execute() with its stages timed: ``events`` are four
        torch.cuda.Event(enable_timing=True), recorded on the current stream
        before the forward FFT and after the forward FFT, the k-space step and
        the inverse FFT (mdft_conv_execute_timed).  No counterpart in the
        reference; it times the kernels execute() itself runs."""
        _check_field(deltarho_p, self.N * self.batch * self.np, self._cdt(), "deltarho_p")
        if len(events) != 4:
            raise ValueError("execute_timed needs four events")
        for e in events:
            if not e.cuda_event:  # torch creates the CUDA event on first record
                e.record()
        arr = (C.c_void_p * 4)(*[C.c_void_p(e.cuda_event) for e in events])
        check(lib().mdft_conv_execute_timed(self.h, _dptr(deltarho_p), _stream(), arr))

    def execute_timed_passes(self, deltarho_p, events):
        """execute() timed per kernel: ``events`` are eight
        torch.cuda.Event(enable_timing=True), recorded on the current stream
        before the forward FFT, after each of its axis passes (z, y, x), after
        the k-space step and after each inverse pass (x, y, z)
        (mdft_conv_execute_timed_passes).  No counterpart in the reference."""
        _check_field(deltarho_p, self.N * self.batch * self.np, self._cdt(), "deltarho_p")
        if len(events) != 8:
            raise ValueError("execute_timed_passes needs eight events")
        for e in events:
            if not e.cuda_event:
                e.record()
        arr = (C.c_void_p * 8)(*[C.c_void_p(e.cuda_event) for e in events])
        check(lib().mdft_conv_execute_timed_passes(self.h, _dptr(deltarho_p), _stream(), arr))

    def fft(self, p, sign):
        _check_field(p, self.N * self.batch * self.np, self._cdt(), "p")
        check(lib().mdft_conv_fft(self.h, _dptr(p), int(sign), _stream()))

    def kspace(self, p):
        _check_field(p, self.N * self.batch * self.np, self._cdt(), "p")
        check(lib().mdft_conv_kspace(self.h, _dptr(p), _stream()))

    def gamma_p_map(self):
        m = np.zeros((self.npairs, 3), np.int32)
        check(lib().mdft_conv_gamma_p_map(self.h, _np_i(m)))
        return m

    def mnmunukhi_q(self):
        t = np.zeros((self.np_new, self.nq), np.complex128)
        check(lib().mdft_conv_mnmunukhi_q(self.h, t.ctypes.data_as(C.POINTER(C.c_double))))
        return t

    def dq(self):
        return self._dq


def get_delta_rho(xi, delta_rho, rho0):
    """delta_rho = rho0 (xi^2 - 1) (MDFT_Solvent.hpp:578-596)."""
    torch = _torch()
    if xi.numel() != delta_rho.numel():
        raise MdftError(1, "size of delta_rho must be the same as the size of xi")
    _check_field(xi, xi.numel(), (torch.float64, torch.float32), "xi")
    _check_field(delta_rho, xi.numel(), (xi.dtype,), "delta_rho")
    check(lib().mdft_get_delta_rho(_dptr(xi), _dptr(delta_rho), xi.numel(), float(rho0),
                                   _precision_of(xi.dtype), _stream()))


def get_delta_f(xi, vexc, w, delta_f, rho0, prefactor, ff_out=None):
    """delta_f = 2 rho0 xi vexc; returns ff = sum rho0 prefactor vexc w (xi^2-1)
    (MDFT_Solvent.hpp:617-660).  xi, vexc, delta_f are (nx, ny, nz, no) (or any
    shape whose last axis is no); w is (no,).  Like the reference, which
    returns ff through a host reference after a blocking reduction, this
    synchronises and returns a Python float unless ``ff_out`` (a CUDA float64
    tensor of one element) is given, in which case it stays asynchronous."""
    torch = _torch()
    no = int(w.numel())
    if xi.shape != vexc.shape:
        raise MdftError(1, "angular grid size of xi and vexc must be the same")
    n = xi.numel()
    if no <= 0 or n % no:
        raise MdftError(1, "last axis of xi must be the orientation axis of w")
    _check_field(xi, n, (torch.float64, torch.float32), "xi")
    _check_field(vexc, n, (xi.dtype,), "vexc")
    _check_field(delta_f, n, (xi.dtype,), "delta_f")
    wd = w.to(device=xi.device, dtype=torch.float64).contiguous()
    ff = ff_out if ff_out is not None else torch.zeros(1, dtype=torch.float64, device=xi.device)
    check(lib().mdft_get_delta_f(_dptr(xi), _dptr(vexc), _dptr(wd), _dptr(delta_f), _dptr(ff),
                                 n // no, no, float(rho0), float(prefactor),
                                 _precision_of(xi.dtype), _stream()))
    if ff_out is not None:
        return ff_out
    return float(ff.item())


class Server:
    """Job server (mdft_server_*; no counterpart in the reference).

    Jobs (one field xi on one grid with one registered solvent) run n_steps
    steps of the cproj excess energy and gradient followed by
    xi <- xi - step * gradient; same-shape jobs advance together in batched,
    graph-replayed steps on the server's worker thread.  Fields are numpy
    arrays of the server's precision (float64 for "f64"/"f64df", float32 for
    "f32")."""

    def __init__(self, precision="f64df", max_batch=8, hbm_budget_bytes=0):
        self.precision = _precision_arg(precision)
        self._dt = np.float32 if self.precision == MDFT_F32 else np.float64
        h = C.c_void_p()
        check(lib().mdft_server_create(C.byref(h), self.precision, int(max_batch),
                                       int(hbm_budget_bytes)))
        self.h = h
        self._solvents = {}
        self._jobs = {}

    def close(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mdft_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def add_solvent(self, mmax, mrso, luc_index, table, dq, rho0, prefactor):
        idx = np.ascontiguousarray(luc_index, np.int32)
        tab = np.ascontiguousarray(table, np.complex128)
        np_luc, nq = tab.shape
        sid = C.c_int()
        check(lib().mdft_server_add_solvent(self.h, int(mmax), int(mrso), _np_i(idx),
                                            tab.ctypes.data_as(C.POINTER(C.c_double)), np_luc, nq,
                                            float(dq), float(rho0), float(prefactor), C.byref(sid)))
        ntheta, nphi, npsi = mmax + 1, 2 * mmax + 1, 2 * (mmax // mrso) + 1
        self._solvents[sid.value] = (ntheta, nphi, npsi)
        return sid.value

    def submit(self, solvent, n_nodes, length, xi0, n_steps, step):
        """Queues a job and returns its id at once."""
        nx, ny, nz = (int(v) for v in n_nodes)
        ntheta, nphi, npsi = self._solvents[solvent]
        x = np.ascontiguousarray(xi0, self._dt)
        if x.size != nx * ny * nz * ntheta * nphi * npsi:
            raise ValueError("xi0 has %d values, the job needs %d"
                             % (x.size, nx * ny * nz * ntheta * nphi * npsi))
        jid = C.c_longlong()
        check(lib().mdft_server_submit(self.h, int(solvent), nx, ny, nz, *(float(v) for v in length),
                                       x.ctypes.data_as(C.c_void_p), int(n_steps), float(step),
                                       C.byref(jid)))
        self._jobs[jid.value] = (x.shape, int(n_steps))
        return jid.value

    def wait(self, job):
        """(final xi, energies of every step, latency in s) of a job."""
        shape, n_steps = self._jobs.pop(job, (None, 0))[:2]
        lat = C.c_double()
        if shape is None:  # not submitted here, or already waited for: the server says which
            check(lib().mdft_server_wait(self.h, C.c_longlong(job), None, None, C.byref(lat)))
            return None, None, lat.value
        xi = np.empty(shape, self._dt)
        ff = np.empty(n_steps, np.float64)
        check(lib().mdft_server_wait(self.h, C.c_longlong(job), xi.ctypes.data_as(C.c_void_p),
                                     ff.ctypes.data_as(C.POINTER(C.c_double)), C.byref(lat)))
        return xi, ff, lat.value

    def set_solvent_model(self, solvent, sites, kT, vmax):
        """The solvent's molecular model for solute jobs: sites (q, sigma,
        epsilon, x, y, z) in the molecular frame, kT and vmax in kJ/mol."""
        sv = np.ascontiguousarray(sites, np.float64).reshape(-1, 6)
        check(lib().mdft_server_set_solvent_model(self.h, int(solvent), _np_d(sv), sv.shape[0], float(kT),
                                                  float(vmax)))

    def submit_solute(self, solvent, n_nodes, length, solute_sites, max_iter=100, gtol=1e-5, xi0=None):
        """Queues a solute job: minimise the full functional from xi0 (None:
        xi = 1) with the solute's external potential; returns its id."""
        nx, ny, nz = (int(v) for v in n_nodes)
        ntheta, nphi, npsi = self._solvents[solvent]
        su = np.ascontiguousarray(solute_sites, np.float64).reshape(-1, 6)
        x = None
        if xi0 is not None:
            x = np.ascontiguousarray(xi0, np.float64)
            if x.size != nx * ny * nz * ntheta * nphi * npsi:
                raise ValueError("xi0 has the wrong size")
        jid = C.c_longlong()
        check(lib().mdft_server_submit_solute(self.h, int(solvent), nx, ny, nz, *(float(v) for v in length),
                                              _np_d(su), su.shape[0], _np_d(x) if x is not None else None,
                                              int(max_iter), float(gtol), C.byref(jid)))
        self._jobs[jid.value] = ((nx * ny * nz, ntheta, nphi, npsi), int(max_iter), "solute")
        return jid.value

    def wait_solute(self, job):
        """(final xi, trace (iterations + 1, 5): E_total, E_id, E_ext, E_exc,
        max |dE/dxi|, status, latency in s) of a solute job; status 0: gtol
        reached, 1: E flat, 2: max_iter, 3: no decrease along the direction."""
        shape, max_iter, _ = self._jobs.pop(job)
        xi = np.empty(shape, np.float64)
        trace = np.zeros((max_iter + 1, 5), np.float64)
        it, st, lat = C.c_int(), C.c_int(), C.c_double()
        check(lib().mdft_server_wait_solute(self.h, C.c_longlong(job), _np_d(xi), _np_d(trace), C.byref(it),
                                            C.byref(st), C.byref(lat)))
        return xi, trace[: it.value + 1], st.value, lat.value

    def stats(self):
        """dict: done, solves_per_s, p50_s, p99_s, groups, peak_bytes,
        graph_steps, direct_steps."""
        out = np.zeros(8, np.float64)
        check(lib().mdft_server_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        keys = ("done", "solves_per_s", "p50_s", "p99_s", "groups", "peak_bytes", "graph_steps",
                "direct_steps")
        return dict(zip(keys, out.tolist()))


def solute_vext(spatial_grid, angular_grid, solvent_sites, solute_sites, vmax=100.0, out=None):
    """External potential of a solute at every grid point and orientation
    (mdft_vext_lj_coulomb; no counterpart in the reference, which defines the
    sites but not the potential): LJ 12-6 with Lorentz-Berthelot mixing plus
    Coulomb (qfact) between every solvent site and every solute site, minimum
    image, clamped to [-vmax, vmax] kJ/mol.  Sites are rows (q, sigma,
    epsilon, x, y, z): solvent sites in the molecular frame, solute sites in
    box coordinates.  Returns (N, ntheta, nphi, npsi) float64 on the GPU."""
    torch = _torch()
    sg, ag = spatial_grid, angular_grid
    g = _GridHandle(sg.m_n_nodes, sg.m_length, ag.m_mmax, ag.m_molrotsymorder)
    sv = np.ascontiguousarray(solvent_sites, np.float64).reshape(-1, 6)
    su = np.ascontiguousarray(solute_sites, np.float64).reshape(-1, 6)
    shape = (g.nx * g.ny * g.nz, g.ntheta, g.nphi, g.npsi)
    if out is None:
        out = torch.empty(shape, dtype=torch.float64, device="cuda")
    _check_field(out, int(np.prod(shape)), (torch.float64,), "vext")
    check(lib().mdft_vext_lj_coulomb(g.h, _np_d(sv), sv.shape[0], _np_d(su), su.shape[0],
                                     float(vmax), _dptr(out), _stream()))
    return out


class Solver:
    """L-BFGS minimiser of the MDFT functional in xi = sqrt(rho/rho0)
    (mdft_solver_*): E = E_id + E_ext + E_exc, the excess term being the
    cproj energy of get_delta_f computed by ``opt`` and ``conv`` (single-field
    handles of one grid and precision).  xi, vext and gradients are float64
    CUDA tensors (N, ntheta, nphi, npsi) in every precision."""

    TERMS = ("total", "id", "ext", "exc", "gmax")

    def __init__(self, opt, conv, vext=None, kT=None, rho0=None, prefactor=None, history=5):
        torch = _torch()
        if kT is None or rho0 is None or prefactor is None:
            raise MdftError(1, "kT, rho0 and prefactor are required")
        self._keep = (opt, conv)
        self.N, self.no = opt.N, opt.no
        if vext is not None:
            _check_field(vext, self.N * self.no, (torch.float64,), "vext")
        h = C.c_void_p()
        check(lib().mdft_solver_create(C.byref(h), opt.h, conv.h,
                                       _dptr(vext) if vext is not None else None,
                                       float(kT), float(rho0), float(prefactor), int(history)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and _lib._lib is not None:
            _lib._lib.mdft_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def energy(self, xi, grad=None):
        """dict of E_total, E_id, E_ext, E_exc and max |dE/dxi| at xi; the
        gradient goes to ``grad`` when given."""
        torch = _torch()
        _check_field(xi, self.N * self.no, (torch.float64,), "xi")
        if grad is not None:
            _check_field(grad, self.N * self.no, (torch.float64,), "grad")
        t = np.zeros(5, np.float64)
        check(lib().mdft_solver_energy(self.h, _dptr(xi), _dptr(grad) if grad is not None else None,
                                       _np_d(t), _stream()))
        return dict(zip(self.TERMS, t.tolist()))

    def minimize(self, xi, max_iter=50, gtol=1e-5, ftol=0.0):
        """Minimises in place from xi; returns the (iterations + 1, 5) trace
        of the terms (row 0 at the start)."""
        torch = _torch()
        _check_field(xi, self.N * self.no, (torch.float64,), "xi")
        trace = np.zeros((int(max_iter) + 1, 5), np.float64)
        it = C.c_int()
        check(lib().mdft_solver_minimize(self.h, _dptr(xi), int(max_iter), float(gtol), float(ftol),
                                         _np_d(trace), C.byref(it), _stream()))
        return trace[: it.value + 1]

    STATUS = {0: "gtol", 1: "flat", 2: "max_iter", 3: "no_decrease", -1: "not_run"}

    def status(self):
        """How the last minimize ended (mdft_solver_status): 0 gtol reached,
        1 E flat (ftol), 2 max_iter, 3 no decrease along the direction, -1
        never run."""
        st = C.c_int()
        check(lib().mdft_solver_status(self.h, C.byref(st)))
        return st.value


def luc_read(path, np_luc, qmax):
    """IO::LucData: (luc_index (5, np_luc) int32, table (np_luc, nq) complex128,
    dq) with the first int(qmax/dq + 0.5) + 2 q rows (mdft_luc_read)."""
    nq, dq = C.c_int(), C.c_double()
    check(lib().mdft_luc_read(str(path).encode(), int(np_luc), float(qmax), None, None,
                              C.byref(nq), C.byref(dq)))
    idx = np.zeros((5, np_luc), np.int32)
    tab = np.zeros((np_luc, nq.value), np.complex128)
    check(lib().mdft_luc_read(str(path).encode(), int(np_luc), float(qmax), _np_i(idx),
                              tab.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nq), C.byref(dq)))
    return idx, tab, dq.value


def luc_write(path, luc_index, table, dq, header="c(q) table"):
    """Writes a c(q) table in the Luc text layout (mdft_luc_write)."""
    idx = np.ascontiguousarray(luc_index, np.int32)
    tab = np.ascontiguousarray(table, np.complex128)
    np_luc, nq = tab.shape
    check(lib().mdft_luc_write(str(path).encode(), _np_i(idx), tab.ctypes.data_as(C.POINTER(C.c_double)),
                               np_luc, nq, float(dq), header.encode()))


def wait_timeouts():
    """Bounded device waits (FFT tile copies, persistent-kernel flags) that
    ran out of time on the current device since the library was loaded
    (mdft_wait_timeouts); stays 0 unless wait_selftest ran."""
    c = C.c_int()
    check(lib().mdft_wait_timeouts(C.byref(c)))
    return c.value


def grid_barrier_selftest(missing, stream=None):
    """One cooperative launch meeting at the persistent L-BFGS kernel's grid
    barrier, which expects `missing` more arrivals than there are blocks
    (mdft_grid_barrier_selftest): missing = 0 passes; missing > 0 runs out
    after about a second and is recorded as a timed-out wait."""
    check(lib().mdft_grid_barrier_selftest(int(missing), _stream() if stream is None else C.c_void_p(stream)))


def wait_selftest(spins=1024, stream=None):
    """Launches one CTA whose bounded wait runs out (nothing completes its
    barrier) and is recorded as a timeout (mdft_wait_selftest): the next FFT
    launch on the device then raises MdftError with code MDFT_ERR_TIMEOUT."""
    check(lib().mdft_wait_selftest(int(spins), _stream() if stream is None else C.c_void_p(stream)))
