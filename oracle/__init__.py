"""CPU oracle for the Mini-MDFT convolution hot path -- TEST INFRASTRUCTURE.

This package is the checker, never the product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
it.  It wraps ``mdft_oracle.c`` (a C restatement of the reference's
OrientationProjectionTransform, Convolution, get_delta_rho and get_delta_f)
through ctypes with numpy arrays.

Parity status: pinned by the reference's known-answer tests (Gauss-Legendre
weight sum, Wigner-d quick returns/closed forms), numpy.fft convention checks
and identities; the reference itself cannot be built here (Kokkos and
kokkos-fft are absent), so end-to-end values are otherwise unpinned.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.mdfto_create.restype = vp
        L.mdfto_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_double, C.c_double, C.c_int, C.c_int]
        L.mdfto_destroy.argtypes = [vp]
        L.mdfto_set_threads.argtypes = [vp, C.c_int]
        L.mdfto_info.argtypes = [vp, ip]
        L.mdfto_kvectors.argtypes = [vp, dp, dp, dp]
        L.mdfto_angular.argtypes = [vp, dp, dp, dp]
        L.mdfto_opmap.argtypes = [vp, ip, ip, ip, ip, ip, dp]
        L.mdfto_wigner_small_d.restype = C.c_double
        L.mdfto_wigner_small_d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double]
        L.mdfto_gauss_legendre.argtypes = [C.c_int, dp, dp]
        L.mdfto_rotation_coeffs.argtypes = [dp, dp, dp, dp]
        L.mdfto_rotation_matrix.argtypes = [dp, C.c_int, dp]
        L.mdfto_set_luc.restype = C.c_int
        L.mdfto_set_luc.argtypes = [vp, ip, dp, C.c_int, C.c_int, C.c_double]
        L.mdfto_qmax.restype = C.c_double
        L.mdfto_qmax.argtypes = [vp]
        L.mdfto_nq_for_dq.restype = C.c_int
        L.mdfto_nq_for_dq.argtypes = [vp, C.c_double]
        L.mdfto_gamma_p_map.argtypes = [vp, ip]
        L.mdfto_ia_map.argtypes = [vp, ip]
        L.mdfto_mnmunukhi_q.argtypes = [vp, dp]
        L.mdfto_delta_rho.argtypes = [dp, dp, C.c_size_t, C.c_double]
        L.mdfto_angl2proj.argtypes = [vp, dp, dp]
        L.mdfto_proj2angl.argtypes = [vp, dp, dp]
        L.mdfto_conv_execute.argtypes = [vp, dp]
        L.mdfto_delta_f.restype = C.c_double
        L.mdfto_delta_f.argtypes = [dp, dp, dp, dp, C.c_size_t, C.c_int,
                                    C.c_double, C.c_double]
        L.mdfto_fft3d.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        L.mdfto_prefactor.restype = C.c_double
        L.mdfto_prefactor.argtypes = [C.c_double, C.c_int, C.c_double]
        _lib = L
    return _lib


def _d(a):
    assert a.dtype in (np.float64, np.complex128) and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int))


def wigner_small_d(m, mu, mup, theta):
    return lib().mdfto_wigner_small_d(int(m), int(mu), int(mup), float(theta))


def gauss_legendre(n):
    x = np.zeros(n)
    w = np.zeros(n)
    lib().mdfto_gauss_legendre(n, _d(x), _d(w))
    return x, w


def rotation_coeffs():
    a = np.zeros((5, 13, 13))
    b = np.zeros((5, 13, 13))
    c = np.zeros((5, 13))
    d = np.zeros((5, 13))
    lib().mdfto_rotation_coeffs(_d(a), _d(b), _d(c), _d(d))
    return a, b, c, d


def rotation_matrix(q, mmax):
    R = np.zeros((mmax + 1, 2 * mmax + 1, 2 * mmax + 1), np.complex128)
    qq = np.ascontiguousarray(q, dtype=np.float64)
    lib().mdfto_rotation_matrix(_d(qq), mmax, _d(R))
    return R


def fft3d(data, sign):
    """In-place unnormalised batched 3-D FFT of a (batch, nx, ny, nz) array."""
    b, nx, ny, nz = data.shape
    lib().mdfto_fft3d(_d(data), b, nx, ny, nz, sign)
    return data


def delta_rho(xi, rho0):
    xi = np.ascontiguousarray(xi, np.float64)
    out = np.empty_like(xi)
    lib().mdfto_delta_rho(_d(xi), _d(out), xi.size, rho0)
    return out


def delta_f(xi, vexc, w, rho0, prefactor):
    """Returns (delta_f, ff) for xi, vexc of shape (..., no) and w (no,)."""
    xi = np.ascontiguousarray(xi, np.float64)
    vexc = np.ascontiguousarray(vexc, np.float64)
    w = np.ascontiguousarray(w, np.float64)
    no = w.size
    df = np.empty_like(xi)
    ff = lib().mdfto_delta_f(_d(xi), _d(vexc), _d(w), _d(df), xi.size // no,
                             no, rho0, prefactor)
    return df, ff


def prefactor(temperature, mrso, n0):
    return lib().mdfto_prefactor(temperature, mrso, n0)


class Oracle:
    """Grid + OPT + Convolution state of one problem, on the CPU."""

    def __init__(self, n, box, mmax, mrso, threads=0):
        nx, ny, nz = n
        lx, ly, lz = box
        self._h = lib().mdfto_create(nx, ny, nz, lx, ly, lz, mmax, mrso)
        if not self._h:
            raise ValueError("invalid grid for the oracle")
        if threads:
            lib().mdfto_set_threads(self._h, threads)
        self._info()

    def _info(self):
        v = np.zeros(13, np.int32)
        lib().mdfto_info(self._h, _i(v))
        (self.nx, self.ny, self.nz, self.mmax, self.mrso, self.ntheta,
         self.nphi, self.npsi, self.no, self.np, self.npairs, self.np_new,
         self.nq) = [int(x) for x in v]
        self.N = self.nx * self.ny * self.nz

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.mdfto_destroy(h)
            self._h = None

    def kvectors(self):
        kx, ky, kz = np.zeros(self.nx), np.zeros(self.ny), np.zeros(self.nz)
        lib().mdfto_kvectors(self._h, _d(kx), _d(ky), _d(kz))
        return kx, ky, kz

    def angular(self):
        th, wth, w = np.zeros(self.ntheta), np.zeros(self.ntheta), np.zeros(self.no)
        lib().mdfto_angular(self._h, _d(th), _d(wth), _d(w))
        return th, wth, w

    def opmap(self):
        K = self.mmax // self.mrso
        p = np.zeros((self.mmax + 1, 2 * self.mmax + 1, K + 1), np.int32)
        arrs = [np.zeros(self.np, np.int32) for _ in range(4)]
        wig = np.zeros((self.ntheta, self.np))
        lib().mdfto_opmap(self._h, _i(p), *[_i(a) for a in arrs], _d(wig))
        return dict(p=p, m=arrs[0], mup=arrs[1], mu=arrs[2], mu2=arrs[3], wigner=wig)

    def qmax(self):
        return lib().mdfto_qmax(self._h)

    def nq_for_dq(self, dq):
        return lib().mdfto_nq_for_dq(self._h, dq)

    def set_luc(self, luc_index, luc, dq):
        luc_index = np.ascontiguousarray(luc_index, np.int32)
        luc = np.ascontiguousarray(luc, np.complex128)
        np_luc, nq = luc.shape
        assert luc_index.shape == (5, np_luc)
        rc = lib().mdfto_set_luc(self._h, _i(luc_index), _d(luc), np_luc, nq, dq)
        if rc:
            raise ValueError("c(q) table has too few rows for this grid")
        self._info()

    def gamma_p_map(self):
        m = np.zeros((self.npairs, 3), np.int32)
        lib().mdfto_gamma_p_map(self._h, _i(m))
        return m

    def ia_map(self):
        ia = np.zeros((self.np, self.mmax + 1, 2 * self.mmax // self.mrso + 1), np.int32)
        lib().mdfto_ia_map(self._h, _i(ia))
        return ia

    def mnmunukhi_q(self):
        t = np.zeros((self.np_new, self.nq), np.complex128)
        lib().mdfto_mnmunukhi_q(self._h, _d(t))
        return t

    def angl2proj(self, o):
        o = np.ascontiguousarray(o, np.float64)
        assert o.size == self.N * self.no
        p = np.zeros((self.np, self.nx, self.ny, self.nz), np.complex128)
        lib().mdfto_angl2proj(self._h, _d(o), _d(p))
        return p

    def proj2angl(self, p):
        p = np.ascontiguousarray(p, np.complex128)
        assert p.size == self.N * self.np
        o = np.zeros((self.N, self.ntheta, self.nphi, self.npsi))
        lib().mdfto_proj2angl(self._h, _d(p), _d(o))
        return o

    def conv_execute(self, p):
        """Returns the convolved copy of p (np, nx, ny, nz) complex128."""
        q = np.array(p, dtype=np.complex128, copy=True, order="C")
        assert q.size == self.N * self.np
        lib().mdfto_conv_execute(self._h, _d(q))
        return q
