"""The oracle against independent numpy restatements of the reference's
device-vs-host unit tests (small sizes; numpy.fft stands in for the
kokkos-fft host backend the reference tests use)."""
import math

import numpy as np
import pytest

import oracle as O
from mini_mdft_gb300 import inputs as I

from _util import rel_err


@pytest.mark.parametrize("shape", [(2, 4, 6, 5), (3, 8, 8, 8), (1, 10, 12, 7), (2, 64, 1, 3),
                                   (1, 32, 48, 5), (1, 2, 3, 11)])
def test_fft3d_matches_numpy(shape):
    rng = np.random.default_rng(5)
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    ref = np.fft.fftn(x, axes=(1, 2, 3))
    assert rel_err(O.fft3d(x.copy(), -1), ref) < 1e-14
    refi = np.fft.ifftn(x, axes=(1, 2, 3)) * np.prod(shape[1:])
    assert rel_err(O.fft3d(x.copy(), +1), refi) < 1e-14


def numpy_angl2proj(o, om, wth, mmax, mrso, nphi, npsi):
    """unit_test/Test_OrientationProjectionTransform.cpp:129-178 with
    numpy.fft.rfft2 (Normalization::forward = divide by nphi*npsi)."""
    N, nt = o.shape[0], o.shape[1]
    K = mmax // mrso
    fm = np.sqrt(2.0 * np.arange(mmax + 1) + 1.0)
    npj = len(om["m"])
    p = np.zeros((npj, N), np.complex128)
    for r in range(N):
        f = np.zeros((nt, K + 1, 2 * mmax + 1), np.complex128)
        for it in range(nt):
            c2d = np.fft.rfft2(o[r, it]) / (nphi * npsi)
            for imu2 in range(K + 1):
                for imup in range(mmax + 1):
                    f[it, imu2, imup + mmax] = np.conj(c2d[imup, imu2])
                for imup in range(mmax):
                    f[it, imu2, imup] = np.conj(c2d[imup + mmax + 1, imu2])
        for ip in range(npj):
            m, mup, mu2 = om["m"][ip], om["mup"][ip], om["mu2"][ip]
            p[ip, r] = np.sum(f[:, mu2, mup + mmax] * om["wigner"][:, ip] * wth * fm[m])
    return p


def numpy_proj2angl(p2d, om, mmax, mrso, nt, nphi, npsi):
    """unit_test/Test_OrientationProjectionTransform.cpp:249-306 with
    numpy.fft.irfft2 times nphi*npsi (Normalization::none)."""
    npj, N = p2d.shape
    K = mmax // mrso
    fm = np.sqrt(2.0 * np.arange(mmax + 1) + 1.0)
    o = np.zeros((N, nt, nphi, npsi))
    for r in range(N):
        f = np.zeros((nt, K + 1, 2 * mmax + 1), np.complex128)
        for imup in range(-mmax, mmax + 1):
            for imu2 in range(K + 1):
                for im in range(max(abs(imup), mrso * imu2), mmax + 1):
                    ip = om["p"][im, imup + mmax, imu2]
                    f[:, imu2, imup + mmax] += p2d[ip, r] * om["wigner"][:, ip] * fm[im]
        for it in range(nt):
            c2d = np.zeros((nphi, K + 1), np.complex128)
            for imu2 in range(K + 1):
                for imup in range(mmax + 1):
                    c2d[imup, imu2] = np.conj(f[it, imu2, imup + mmax])
                for imup in range(mmax):
                    c2d[imup + mmax + 1, imu2] = np.conj(f[it, imu2, imup])
            o[r, it] = np.fft.irfft2(c2d, s=(nphi, npsi)) * (nphi * npsi)
    return o


CASES = [((2, 2, 2), 10, 10), ((3, 2, 2), 3, 2), ((2, 2, 1), 5, 1), ((2, 1, 2), 4, 3),
         ((2, 2, 2), 1, 2), ((1, 1, 3), 2, 1)]


@pytest.mark.parametrize("n,mmax,mrso", CASES)
def test_angl2proj_matches_numpy(n, mmax, mrso):
    o = O.Oracle(n, (1.0, 1.0, 1.0), mmax, mrso)
    rng = np.random.default_rng(12345)
    x = rng.uniform(0, 1, size=(o.N, o.ntheta, o.nphi, o.npsi))
    _, wth, _ = o.angular()
    ref = numpy_angl2proj(x, o.opmap(), wth, mmax, mrso, o.nphi, o.npsi)
    got = o.angl2proj(x).reshape(o.np, o.N)
    # reference tolerance eps*1e3 (Test_OrientationProjectionTransform.cpp:184)
    assert rel_err(got, ref) < 1e-13


@pytest.mark.parametrize("n,mmax,mrso", CASES)
def test_proj2angl_matches_numpy(n, mmax, mrso):
    o = O.Oracle(n, (1.0, 1.0, 1.0), mmax, mrso)
    rng = np.random.default_rng(12345)
    p = rng.uniform(0, 1, (o.np, o.N)) + 1j * rng.uniform(0, 1, (o.np, o.N))
    ref = numpy_proj2angl(p, o.opmap(), mmax, mrso, o.ntheta, o.nphi, o.npsi)
    got = o.proj2angl(p.reshape(o.np, o.nx, o.ny, o.nz))
    assert rel_err(got, ref) < 1e-13


@pytest.mark.parametrize("n,mmax,mrso", CASES)
def test_round_trip_identity(n, mmax, mrso):
    # unit_test/Test_OrientationProjectionTransform.cpp:312-348 (constant o=1)
    o = O.Oracle(n, (1.0, 1.0, 1.0), mmax, mrso)
    ones = np.ones((o.N, o.ntheta, o.nphi, o.npsi))
    assert rel_err(o.proj2angl(o.angl2proj(ones)), ones) < 1e-13
    # band-limited subspace: o' = proj2angl(p) is reproduced, and p' =
    # angl2proj(o) is a fixed point of angl2proj . proj2angl
    rng = np.random.default_rng(7)
    p = rng.standard_normal((o.np, o.nx, o.ny, o.nz)) + 1j * rng.standard_normal((o.np, o.nx, o.ny, o.nz))
    o1 = o.proj2angl(p)
    assert rel_err(o.proj2angl(o.angl2proj(o1)), o1) < 1e-12
    x = rng.standard_normal((o.N, o.ntheta, o.nphi, o.npsi))
    p1 = o.angl2proj(x)
    assert rel_err(o.angl2proj(o.proj2angl(p1)), p1) < 1e-12


def numpy_conv_execute(o, p):
    """unit_test/Test_Convolution.cpp:107-331 restated with numpy, following
    the implementation where the test differs (no chop of R)."""
    mmax, mrso, npj = o.mmax, o.mrso, o.np
    nx, ny, nz = o.nx, o.ny, o.nz
    om = o.opmap()
    pm = om["p"]
    kx, ky, kz = o.kvectors()
    tab = o.mnmunukhi_q()
    dq = o._dq
    eps = np.finfo(np.float64).eps
    h = np.fft.fftn(p, axes=(1, 2, 3))
    done = np.zeros((nx, ny, nz), bool)
    for iz in range(nz // 2 + 1):
        for iy in range(ny):
            for ix in range(nx):
                mq = tuple(0 if i == 0 else n - i for i, n in ((ix, nx), (iy, ny), (iz, nz)))
                if done[ix, iy, iz] and done[mq]:
                    continue
                q = np.array([kx[ix], ky[iy], kz[iz]])
                R = O.rotation_matrix(q, mmax)
                gq = h[:, ix, iy, iz].copy()
                gmq = h[(slice(None),) + mq].copy()
                dqv = np.zeros(npj, np.complex128)
                dmq = np.zeros(npj, np.complex128)
                for ip in range(npj):
                    im, ikhi, imu2 = om["m"][ip], om["mup"][ip], om["mu2"][ip]
                    for imup in range(-im, im + 1):
                        j = pm[im, imup + mmax, imu2]
                        dqv[ip] += gq[j] * R[im, imup + mmax, ikhi + mmax]
                        dmq[ip] += gmq[j] * R[im, imup + mmax, -ikhi + mmax]
                    dmq[ip] *= (-1.0) ** im
                eiq = math.sqrt(q @ q) / dq
                iq = int(eiq)
                alpha = eiq - iq
                ceff = alpha * tab[:, iq + 1] + (1.0 - alpha) * tab[:, iq]
                gq[:] = 0
                gmq[:] = 0
                ia = 0
                for ip in range(npj):
                    ikhi = om["mup"][ip]
                    for n_ in range(abs(ikhi), mmax + 1):
                        for nu2 in range(-(n_ // mrso), n_ // mrso + 1):
                            c = ceff[ia]
                            if nu2 < 0:
                                j = pm[n_, ikhi + mmax, abs(nu2)]
                                gq[ip] += c * dqv[j]
                                gmq[ip] += c * dmq[j]
                            else:
                                j = pm[n_, ikhi + mmax, nu2]
                                gq[ip] += c * np.conj(dmq[j])
                                gmq[ip] += c * np.conj(dqv[j])
                            ia += 1
                for g in (gq, gmq):
                    g.real[np.abs(g.real) < eps] = 0
                    g.imag[np.abs(g.imag) < eps] = 0
                outq = np.zeros(npj, np.complex128)
                outmq = np.zeros(npj, np.complex128)
                for ip in range(npj):
                    im, imup, imu2 = om["m"][ip], om["mup"][ip], om["mu2"][ip]
                    for ikhi in range(-im, im + 1):
                        j = pm[im, ikhi + mmax, imu2]
                        outq[ip] += gq[j] * np.conj(R[im, imup + mmax, ikhi + mmax])
                        outmq[ip] += gmq[j] * np.conj(R[im, imup + mmax, -ikhi + mmax])
                    outmq[ip] *= (-1.0) ** im
                h[:, ix, iy, iz] = outq
                sing = (mq == (ix, iy, iz)) and (ix == nx // 2 or iy == ny // 2 or iz == nz // 2)
                h[(slice(None),) + mq] = np.conj(outmq) if sing else outmq
                done[ix, iy, iz] = True
                done[mq] = True
    return np.fft.ifftn(h, axes=(1, 2, 3)) * (nx * ny * nz)


@pytest.mark.parametrize("n,box,mmax,mrso", [((4, 4, 4), (10., 10., 10.), 3, 2),
                                             ((5, 5, 5), (1., 1., 1.), 3, 2),
                                             ((4, 3, 6), (8., 7., 9.), 2, 1),
                                             ((2, 4, 5), (5., 6., 7.), 1, 2)])
def test_conv_execute_matches_numpy(n, box, mmax, mrso):
    o = O.Oracle(n, box, mmax, mrso)
    dq = 0.01
    nq = o.nq_for_dq(dq)
    idx, tab = I.synthetic_cq(mmax, mrso, nq + 3, dq)
    o.set_luc(idx, tab, dq)
    o._dq = dq
    rng = np.random.default_rng(12345)
    p = rng.uniform(0, 1, (o.np,) + n) + 1j * rng.uniform(0, 1, (o.np,) + n)
    ref = numpy_conv_execute(o, p)
    got = o.conv_execute(p)
    # reference tolerance eps*1e3 (Test_Convolution.cpp:335)
    assert rel_err(got, ref) < 1e-13


def test_delta_rho_delta_f_match_numpy():
    # unit_test/Test_Solvent.cpp:127-211: shape (2,3,4,5), rho0 0.3,
    # prefactor 0.334, tolerance eps*100
    rng = np.random.default_rng(12345)
    xi = rng.uniform(0, 1, (2, 3, 4, 5))
    vexc = rng.uniform(0, 1, (2, 3, 4, 5))
    w = rng.uniform(0, 1, 5)
    rho0, pref = 0.3, 0.334
    dr = O.delta_rho(xi, rho0)
    assert np.allclose(dr, rho0 * (xi * xi - 1.0), rtol=2.3e-14, atol=0)
    df, ff = O.delta_f(xi, vexc, w, rho0, pref)
    assert np.allclose(df, 2.0 * rho0 * xi * vexc, rtol=2.3e-14, atol=0)
    ff_ref = np.sum(rho0 * (xi * xi - 1.0) * pref * w * vexc)
    assert abs(ff - ff_ref) <= 2.3e-14 * abs(ff_ref)


def test_prefactor_matches_reference_formula():
    rho0, pref = I.tip3p_constants()
    assert abs(pref - O.prefactor(298.0, 2, I.TIP3P_N0)) < 1e-15 * abs(pref)
    assert abs(rho0 - I.TIP3P_N0 / (8 * math.pi ** 2 / 2)) < 1e-18


def numpy_mnmunukhi_q(mmax, mrso, idx, tab, nq):
    """common/MDFT_Convolution.hpp:271-311 restated: reorder the Luc table
    into (m, khi, mu2, n, nu2) order and fold the (-1)^(khi+nu) / (-1)^n
    signs in."""
    K = mmax // mrso
    pos = {}
    for ip in range(idx.shape[1]):
        m, n, mu, nu, khi = (int(v) for v in idx[:, ip])
        pos[(m, n, mu // mrso + K, nu // mrso + K, khi + mmax)] = ip
    rows = []
    for im in range(mmax + 1):
        for ikhi in range(-im, im + 1):
            for imu2 in range(im // mrso + 1):
                for in_ in range(abs(ikhi), mmax + 1):
                    for inu2 in range(-(in_ // mrso), in_ // mrso + 1):
                        ip = pos.get((im, in_, imu2 + K, inu2 + K, ikhi + mmax), 0)
                        nu = inu2 * mrso
                        s = (-1.0) ** (ikhi + nu) if nu < 0 else (-1.0) ** in_
                        rows.append(s * tab[ip, :nq])
    return np.array(rows)


@pytest.mark.parametrize("mmax,mrso,extra", [(3, 2, 0), (3, 2, 7), (5, 2, 3), (2, 1, 1), (4, 3, 0)])
def test_luc_reorder_matches_numpy(mmax, mrso, extra):
    o = O.Oracle((6, 5, 4), (9., 8., 7.), mmax, mrso)
    nq = o.nq_for_dq(0.01)
    idx, tab = I.synthetic_cq(mmax, mrso, nq + extra, 0.01)
    o.set_luc(idx, tab, 0.01)
    assert o.nq == nq
    assert np.array_equal(o.mnmunukhi_q(), numpy_mnmunukhi_q(mmax, mrso, idx, tab, nq))
