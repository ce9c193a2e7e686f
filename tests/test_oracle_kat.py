"""The oracle against the reference's own known-answer tests.

Each test names the reference test it restates (paths relative to the
Mini_MDFT root).  These pin the CPU oracle before it is used as the checker.
"""
import math

import numpy as np
import pytest

import oracle as O

EPS = np.finfo(np.float64).eps


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 11, 20])
def test_gauss_legendre_weights_sum_to_one(n):
    # unit_test/Test_Math_Utils.cpp:30-44: sum(w) == 1 within eps*100
    x, w = O.gauss_legendre(n)
    assert abs(w.sum() - 1.0) < EPS * 100
    # nodes are the roots of P_n, symmetric
    assert np.allclose(x, -x[::-1], atol=1e-15)
    from numpy.polynomial import legendre
    roots = np.sort(legendre.legroots([0] * n + [1]))
    assert np.allclose(np.sort(x), roots, atol=1e-14)


@pytest.mark.parametrize("m", [0, 1, 2, 5, 10])
def test_wigner_quick_return(m):
    # unit_test/Test_Wigner.cpp:26-45
    for mu in range(-m - 1, m + 2):
        for mup in range(-m - 1, m + 2):
            d = O.wigner_small_d(m, mu, mup, 0.0)
            if abs(mu) > m or abs(mup) > m:
                assert abs(d) < EPS * 100
            elif m == 0:
                assert abs(d - 1.0) < EPS * 100
            assert d >= 0.0


def _fact(k):
    return float(math.factorial(k))


@pytest.mark.parametrize("m", [1, 2, 5, 10])
def test_wigner_closed_forms(m):
    # unit_test/Test_Wigner.cpp:47-130: the mu==0||mup==0 branch and the
    # general sum, restated independently here with exact factorials.
    theta = 0.5488135039273248  # a fixed draw in [0, 1)
    for mu in range(-m, m + 1):
        for mup in range(-m, m + 1):
            d = O.wigner_small_d(m, mu, mup, theta)
            if mu == 0 or mup == 0:
                mu0, th0 = (mup, -theta) if mu == 0 else (mu, theta)
                x = 1.0
                if mu0 < 0:
                    x = (-1.0) ** mu0
                    mu0 = -mu0
                cc = math.cos(th0)
                pm1, pm = 0.0, 1.0
                for l in range(mu0 + 1, m + 1):
                    pm2, pm1 = pm1, pm
                    pm = (cc * (2 * l - 1) * pm1 - (l + mu0 - 1) * pm2) / (l - mu0)
                ref = (x * (-1.0) ** mu0 * math.sqrt(_fact(m - mu0) / _fact(m + mu0))
                       * _fact(2 * mu0) / (2.0 ** mu0 * _fact(mu0)) * math.sin(th0) ** mu0 * pm)
            else:
                cc, ss = math.cos(0.5 * theta), math.sin(0.5 * theta)
                t = 0.0
                for it in range(max(0, mu - mup), min(m + mu, m - mup) + 1):
                    t += ((-1.0) ** it / (_fact(m + mu - it) * _fact(m - mup - it) * _fact(it)
                                         * _fact(it - mu + mup))
                          * cc ** (2 * m + mu - mup - 2 * it) * ss ** (2 * it - mu + mup))
                ref = math.sqrt(_fact(m + mu) * _fact(m - mu) * _fact(m + mup) * _fact(m - mup)) * t
            assert abs(d - ref) < EPS * 100


@pytest.mark.parametrize("m", [1, 2, 3, 5])
def test_wigner_orthogonality_and_legendre(m):
    # identities of the Wigner d-matrix: orthogonal rows, d^m_00 = P_m(cos)
    theta = 0.83
    D = np.array([[O.wigner_small_d(m, a, b, theta) for b in range(-m, m + 1)]
                  for a in range(-m, m + 1)])
    assert np.allclose(D @ D.T, np.eye(2 * m + 1), atol=1e-13)
    from numpy.polynomial import legendre
    assert abs(D[m, m] - legendre.legval(math.cos(theta), [0] * m + [1])) < 1e-14


def test_rotation_coeffs_shapes_and_values():
    # common/MDFT_Rotation.hpp:33-84 (RotationCoeffs ctor, no-throw test
    # unit_test/Test_Rotation.cpp:27-30)
    a, b, c, d = O.rotation_coeffs()
    assert a.shape == (5, 13, 13) and c.shape == (5, 13)
    # l=2, m=0, m1=0: a = sqrt(3)sqrt(3)/(sqrt(3)sqrt(3)) = 1
    assert abs(a[0, 6, 6] - 1.0) < 1e-15
    # d(l, m=l) = sqrt(2l+1) sqrt(2l) / (sqrt(2l+1) sqrt(2l)) = 1
    for l in range(2, 7):
        assert abs(d[l - 2, 6 + l] - 1.0) < 1e-15


@pytest.mark.parametrize("mmax", [1, 2, 3, 4, 5, 6])
def test_rotation_matrix_identity_at_q0(mmax):
    # q = 0 -> frame = identity -> R(l, m, m1) = delta(m, m1)
    # (unit_test/Test_Rotation.cpp:20-23 uses q = 0 as a test vector)
    R = O.rotation_matrix([0.0, 0.0, 0.0], mmax)
    for l in range(mmax + 1):
        blk = R[l, mmax - l:mmax + l + 1, mmax - l:mmax + l + 1]
        assert np.allclose(blk, np.eye(2 * l + 1), atol=1e-14)


@pytest.mark.parametrize("q", [[1.0, 2.0, 3.0], [0.209439510239320] * 3, [0.0, 0.0, 0.7],
                               [0.0, 0.3, 0.0], [-0.4, 0.1, -0.2]])
def test_rotation_matrix_unitary(q):
    # test vectors of unit_test/Test_Rotation.cpp:20-23 (plus axis cases):
    # each R(l) block is a unitary (2l+1)x(2l+1) matrix.
    mmax = 6
    R = O.rotation_matrix(q, mmax)
    for l in range(mmax + 1):
        blk = R[l, mmax - l:mmax + l + 1, mmax - l:mmax + l + 1]
        assert np.allclose(blk @ blk.conj().T, np.eye(2 * l + 1), atol=1e-13)


def test_rotation_matrix_l1_is_vector_rotation():
    # for l = 1 |R| entries follow the q-frame axes: R(1,0,0) = qz/|q|
    q = np.array([1.0, 2.0, 3.0])
    R = O.rotation_matrix(q, 1)
    assert abs(R[1, 1, 1].real - q[2] / np.linalg.norm(q)) < 1e-15
    assert abs(R[1, 1, 1].imag) == 0.0


@pytest.mark.parametrize("n", [5, 10, 4, 6])
def test_gamma_p_map_covers_each_pair_once(n):
    # unit_test/Test_Convolution.cpp:37-78
    o = O.Oracle((n, n, n), (1.0, 1.0, 1.0), 10, 10)
    gmap = o.gamma_p_map()
    seen = np.zeros((n, n, n), bool)
    for ix, iy, iz in gmap:
        mq = tuple(0 if i == 0 else n - i for i in (ix, iy, iz))
        assert not seen[ix, iy, iz]
        assert not seen[mq]
        seen[ix, iy, iz] = True
        seen[mq] = True
    assert seen.all()


@pytest.mark.parametrize("mmax,mrso", [(10, 10), (3, 2), (5, 2), (4, 1), (1, 2)])
def test_opmap_and_weights(mmax, mrso):
    # unit_test/Test_OrientationProjectionTransform.cpp:350-370 (no-throw init)
    # and common/MDFT_Grid.hpp:388-398 (sum w = 8 pi^2 / mrso)
    o = O.Oracle((2, 2, 2), (1.0, 1.0, 1.0), mmax, mrso)
    _, _, w = o.angular()
    assert abs(w.sum() - 8 * math.pi ** 2 / mrso) <= EPS * 100 * w.sum()
    om = o.opmap()
    assert len(om["m"]) == o.np
    assert (np.abs(om["mup"]) <= om["m"]).all()
    assert (om["mu"] == om["mu2"] * mrso).all()
    for ip in range(o.np):
        assert om["p"][om["m"][ip], om["mup"][ip] + mmax, om["mu2"][ip]] == ip


def test_sizes_of_the_named_configurations():
    # np / no / np_new for the 32^3..128^3 configurations (mrso = 2)
    for mmax, no, np_, np_new in [(3, 84, 28, 178), (4, 225, 55, 573), (5, 330, 88, 1268),
                                  (1, 6, 4, 6)]:
        o = O.Oracle((2, 2, 2), (1.0, 1.0, 1.0), mmax, 2)
        assert (o.no, o.np, o.np_new) == (no, np_, np_new)
