"""Seeded synthetic inputs for the convolution hot path, and the Luc c(q) file.

The reference reads tip3p direct-correlation data from Luc's text files
(common/IO/MDFT_ReadCLuc.hpp:40-187); those files are not distributed with it.
This module generates stand-ins with the same shapes and index layout:

* delta_rho per grid point and orientation ~ U[-0.1, 0.1], seed 0, shape
  (N, ntheta, nphi, npsi) float64 (the layout of Solver::m_delta_rho,
  src/mini-mdft.hpp:100);
* xi ~ U[0.9, 1.1], seed 1, same shape (Solvent::m_xi viewed as
  (nx, ny, nz, no), common/MDFT_Solvent.hpp:287-297);
* c(|q|) in the Luc projection-index layout: for Luc index i,
  c_i(q) = a_i * exp(-s_i q^2), a_i ~ N(0,1), s_i ~ U(0.5, 4) (seed 2),
  q_k = k * dq, dq = 0.01 1/Angstrom, imaginary part 0, with
  nq = int(q_max/dq + 0.5) + 2 rows (ReadCLuc.hpp:65) so that every |q| of
  the grid is covered.

All draws use numpy's PCG64 generator, which gives identical streams on x86_64
and aarch64.
"""
import math
import os

import numpy as np

# npluc per mmax for the 3-site water models (common/MDFT_Solvent.hpp:433).
NPLUC = (1, 6, 75, 252, 877, 2002)

# tip3p bulk density and the energy prefactor inputs
# (common/MDFT_Solvent.hpp:483-485, MDFT_Thermo.hpp:60, MDFT_Constants.hpp).
TIP3P_N0 = 0.03349459
BOLTZ = 1.38064852e-23
NAVO = 6.02214129e23


def angular_counts(mmax, mrso):
    """(ntheta, nphi, npsi, no, np) as AngularGrid builds them
    (common/MDFT_Grid.hpp:270-287)."""
    ntheta = mmax + 1
    nphi = 2 * mmax + 1
    npsi = 2 * (mmax // mrso) + 1
    no = ntheta * nphi * npsi
    np_ = sum((2 * m + 1) * (m // mrso + 1) for m in range(mmax + 1))
    return ntheta, nphi, npsi, no, np_


def np_new_count(mmax, mrso):
    """Number of OZ coefficients (common/MDFT_Convolution.hpp:239-251)."""
    c = 0
    for m in range(mmax + 1):
        for khi in range(-m, m + 1):
            for _mu2 in range(m // mrso + 1):
                for n in range(abs(khi), mmax + 1):
                    c += 2 * (n // mrso) + 1
    return c


def kproj(n, length):
    """k-vector in FFT order (common/MDFT_Grid.hpp:222-238)."""
    d = 2.0 * math.pi / length
    n1, n2 = n // 2 + 1, (n - 1) // 2
    k = np.zeros(n)
    for i in range(n1):
        k[i] = float(i) * d
    for i in range(n2):
        k[i + n1] = float(i - n2) * d
    return k


def qmax(n, box):
    """|k_max| over the half space the convolution visits
    (common/MDFT_Convolution.hpp:214-231)."""
    kx, ky, kz = (kproj(n[i], box[i]) for i in range(3))
    kzm = kz[: n[2] // 2 + 1].max()
    return math.sqrt(kx.max() ** 2 + ky.max() ** 2 + kzm ** 2)


def nq_for(n, box, dq):
    return int(qmax(n, box) / dq + 0.5) + 2


def luc_index(mmax, mrso):
    """(5, np_luc) int32 rows m, n, mu, nu, khi, enumerated in descending
    order (the order of the tip3p files: first (mmax, mmax, .., .., mmax),
    last (0, 0, 0, 0, 0))."""
    rows = []
    for m in range(mmax, -1, -1):
        for n in range(mmax, -1, -1):
            mus = [mu for mu in range(m, -m - 1, -1) if mu % mrso == 0]
            nus = [nu for nu in range(n, -n - 1, -1) if nu % mrso == 0]
            for mu in mus:
                for nu in nus:
                    for khi in range(min(m, n), -min(m, n) - 1, -1):
                        rows.append((m, n, mu, nu, khi))
    return np.ascontiguousarray(np.array(rows, dtype=np.int32).T)


def synthetic_cq(mmax, mrso, nq, dq=0.01, seed=2):
    """Synthetic c(|q|) table: (luc_index (5, np_luc) int32,
    table (np_luc, nq) complex128)."""
    idx = luc_index(mmax, mrso)
    np_luc = idx.shape[1]
    rng = np.random.default_rng(seed)
    a = rng.standard_normal(np_luc)
    s = rng.uniform(0.5, 4.0, np_luc)
    q = np.arange(nq, dtype=np.float64) * dq
    tab = a[:, None] * np.exp(-s[:, None] * (q[None, :] ** 2))
    return idx, np.ascontiguousarray(tab.astype(np.complex128))


# Solvent site tables, rows (q [e], sigma [A], epsilon [kJ/mol], x, y, z [A])
# in the molecular frame (common/MDFT_Solvent.hpp:418-436 spce,
# :470-494 tip3p); bulk number densities n0 [1/A^3] beside them.
SPCE_SITES = np.array([[-0.8476, 3.166, 0.65, 0.0, 0.0, 0.0],
                       [0.4238, 0.0, 0.0, 0.816495, 0.0, 0.5773525],
                       [0.4238, 0.0, 0.0, -0.816495, 0.0, 0.5773525]])
SPCE_N0 = 0.0332891
TIP3P_SITES = np.array([[-0.834, 3.15061, 0.636386, 0.0, 0.0, 0.0],
                        [0.417, 0.0, 0.0, 0.756950, 0.0, 0.585882],
                        [0.417, 0.0, 0.0, -0.756950, 0.0, 0.585882]])


def kT(temperature=298.0):
    """kT in kJ/mol (common/MDFT_Thermo.hpp:60)."""
    return BOLTZ * NAVO * temperature * 1e-3


def solvent_constants(n0, mrso=2, temperature=298.0):
    """(rho0, prefactor) of a solvent of bulk density n0
    (common/MDFT_Solvent.hpp:366-368, :426-427)."""
    rho0 = n0 / (8 * math.pi * math.pi / mrso)
    prefactor = -2 * kT(temperature) * 4 * math.pi * math.pi / mrso / n0
    return rho0, prefactor


def synthetic_solute(n_sites, box, seed=3):
    """Seeded synthetic solute, rows (q, sigma, epsilon, x, y, z) in box
    coordinates: positions uniform in the central 10 A cube of the box,
    sigma ~ U(2.5, 4) A, epsilon ~ U(0.1, 1) kJ/mol, charges ~ N(0, 0.4) e
    shifted to sum to 0."""
    rng = np.random.default_rng(seed)
    pos = np.asarray(box, np.float64)[None, :] / 2 + rng.uniform(-5.0, 5.0, (n_sites, 3))
    sig = rng.uniform(2.5, 4.0, n_sites)
    eps = rng.uniform(0.1, 1.0, n_sites)
    q = rng.normal(0.0, 0.4, n_sites)
    q = q - q.mean()
    return np.ascontiguousarray(np.column_stack([q, sig, eps, pos]))


def isotropic_cq(mmax, mrso, nq, dq=0.01, amplitude=1e-4, s=1.0):
    """c(|q|) table with only the (m, n, mu, nu, khi) = 0 entry set, to
    -amplitude exp(-s q^2): an isotropic, symmetric (c(1,2) = c(2,1)) direct
    correlation function whose excess energy is convex in delta_rho."""
    idx = luc_index(mmax, mrso)
    keep = (idx == 0).all(axis=0)
    q = np.arange(nq, dtype=np.float64) * dq
    tab = np.zeros((idx.shape[1], nq), np.complex128)
    tab[keep, :] = -amplitude * np.exp(-s * q ** 2)
    return idx, tab


def synthetic_delta_rho(N, mmax, mrso, seed=0, dtype=np.float64):
    ntheta, nphi, npsi, _, _ = angular_counts(mmax, mrso)
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.1, 0.1, size=(N, ntheta, nphi, npsi)).astype(dtype)


def synthetic_xi(N, mmax, mrso, seed=1, dtype=np.float64):
    ntheta, nphi, npsi, _, _ = angular_counts(mmax, mrso)
    rng = np.random.default_rng(seed)
    return rng.uniform(0.9, 1.1, size=(N, ntheta, nphi, npsi)).astype(dtype)


def tip3p_constants(mrso=2, temperature=298.0):
    """(rho0, prefactor) for tip3p (common/MDFT_Solvent.hpp:483-485,
    :366-368; kT from common/MDFT_Thermo.hpp:60)."""
    n0 = TIP3P_N0
    pi = math.pi
    rho0 = n0 / (8 * pi * pi / mrso)
    kbt = BOLTZ * NAVO * temperature * 1e-3
    prefactor = -2 * kbt * 4 * pi * pi / mrso / n0
    return rho0, prefactor


def write_luc_file(path, idx, tab, dq, header="synthetic c(q) table"):
    """Writes a table in the text layout ReadCLuc.hpp:123-187 parses:
    10 free lines, a label line, five lines 'label v_1 .. v_np' for
    m, n, mu, nu, khi, one free line, then nq rows 'q (re,im) ...'."""
    np_luc, nq = tab.shape
    with open(path, "w") as f:
        f.write("# " + header + "\n")
        for i in range(9):
            f.write("#\n")
        f.write("# projection indices\n")
        for name, row in zip(("m", "n", "mu", "nu", "khi"), idx):
            f.write(name + " " + " ".join(str(int(v)) for v in row) + "\n")
        f.write("# q  c(q) for each projection\n")
        for iq in range(nq):
            vals = " ".join("(%.17g,%.17g)" % (z.real, z.imag) for z in tab[:, iq])
            f.write("%.17g %s\n" % (iq * dq, vals))


def read_luc_file(path, np_luc):
    """Pure-Python reader of the same layout: (idx, tab, dq)."""
    with open(path) as f:
        lines = f.read().splitlines()
    idx = []
    for row in lines[11:16]:
        parts = row.split()
        idx.append([int(v) for v in parts[1:1 + np_luc]])
    rows = []
    qs = []
    for row in lines[17:]:
        if not row.strip():
            continue
        parts = row.split()
        qs.append(float(parts[0]))
        vals = []
        for tok in parts[1:1 + np_luc]:
            re_, im_ = tok.strip("()").split(",")
            vals.append(complex(float(re_), float(im_)))
        rows.append(vals)
    tab = np.array(rows, dtype=np.complex128).T.copy()
    dq = qs[3] - qs[2] if len(qs) > 3 else qs[1] - qs[0]
    return np.array(idx, np.int32), tab, dq


def write_luc_if_missing(dirpath, mmax, mrso, n, box, dq=0.01):
    os.makedirs(dirpath, exist_ok=True)
    nq = nq_for(n, box, dq)
    path = os.path.join(dirpath, "synthetic-ck_mmax%d_mrso%d_nq%d" % (mmax, mrso, nq))
    if not os.path.exists(path):
        idx, tab = synthetic_cq(mmax, mrso, nq, dq)
        write_luc_file(path + ".tmp", idx, tab, dq)
        os.replace(path + ".tmp", path)
    return path
