"""R(q) of the convolution's frame (common/MDFT_Rotation.hpp:103-283, the
frame r2 = q/|q|, r1 = z x r2 / |z x r2|, r0 = r1 x r2 of :112-160) factors as

    R^l(m, m1; q) = w^m d^l(m, m1; q),   d real,   w = r1_y + i r1_x = e^{-i phi}

(phi the azimuth of q; on the z axis r1 = (0, sign qz, 0), at q = 0 r1 =
(0, 1, 0)).  The split OZ kernels store d (the m1 >= 0 half, with
d(-m, -m1) = (-1)^(m+m1) d(m, m1)) and the powers of w in place of the
complex R; this pins the identity on the oracle's R at every k-point of a
cubic and of a non-cubic grid, the z axis and q = 0 included."""
import numpy as np
import pytest

import oracle as O


def _frame_phase(q):
    """w = e^{-i phi} from the frame vector r1 exactly as the frame is built."""
    r2 = np.array(q, dtype=np.float64)
    if not r2.any():
        r2 = np.array([0.0, 0.0, 1.0])
    if r2[0] != 0.0 or r2[1] != 0.0:
        r1 = np.array([-r2[1], r2[0], 0.0])
    else:
        r1 = np.array([0.0, r2[2], 0.0])
    r1 = r1 / np.sqrt(r1 @ r1)
    return complex(r1[1], r1[0])


@pytest.mark.parametrize("n,box,mmax", [((8, 8, 8), (10., 10., 10.), 5),
                                        ((6, 7, 10), (7., 9., 11.), 4)])
def test_rotation_factors_into_phase_and_real_block(n, box, mmax):
    g = O.Oracle(n, box, mmax, 1)
    kx, ky, kz = g.kvectors()
    worst_imag = worst_sym = 0.0
    for x in kx:
        for y in ky:
            for z in kz:
                q = (x, y, z)
                R = O.rotation_matrix(np.array(q), mmax)
                w = _frame_phase(q)
                assert abs(abs(w) - 1.0) < 1e-15
                for l in range(1, mmax + 1):
                    ms = np.arange(-l, l + 1)
                    B = R[l][mmax - l:mmax + l + 1, mmax - l:mmax + l + 1]
                    # d = w^-m R, row by row
                    d = (np.conj(w) ** ms)[:, None] * B
                    worst_imag = max(worst_imag, np.abs(d.imag).max())
                    sgn = (-1.0) ** (ms[:, None] + ms[None, :])
                    worst_sym = max(worst_sym, np.abs(d.real[::-1, ::-1] - sgn * d.real).max())
    assert worst_imag < 1e-14
    assert worst_sym < 1e-14
