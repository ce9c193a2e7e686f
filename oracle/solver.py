"""CPU oracle for the solute external potential and the functional the
minimiser descends -- TEST INFRASTRUCTURE (only ``tests/`` import it).

Parity status: **unpinned**.  The reference defines the data these terms use
-- solvent sites (common/MDFT_Solvent.hpp:418-494), solute sites
(common/MDFT_Solute.hpp:150-200), the rotation matrix of each orientation
(common/MDFT_Grid.hpp:283-310), qfact and kT (common/MDFT_Constants.hpp:46-47,
common/MDFT_Thermo.hpp:60) -- but computes neither vext, nor the ideal and
external energies, nor a minimiser step, so this module restates the
standard MDFT functional in plain numpy as the checker of the GPU code, and
pins it only by identities (the Boltzmann density is the minimum without
the excess term; gradients against finite differences):

    vext(r, o) = sum_a sum_s 4 eps_as [(sig_as/d)^12 - (sig_as/d)^6] + qfact q_a q_s / d
        d = |r + R(o) x_a - x_s| (minimum image), eps_as = sqrt(eps_a eps_s),
        sig_as = (sig_a + sig_s)/2, clamped to [-vmax, vmax]
    E_id  = kT rho0 dv sum w_o (xi^2 ln xi^2 - xi^2 + 1)
    E_ext =    rho0 dv sum w_o xi^2 vext
    E_exc = prefactor rho0 sum w_o vexc (xi^2 - 1)            (get_delta_f's ff)
    dE/dxi = 2 rho0 dv w_o xi (kT ln xi^2 + vext) + 4 prefactor rho0 w_o xi vexc
"""
import math

import numpy as np


def qfact():
    """q_i q_j / r in kJ/mol for e and Angstrom (common/MDFT_Constants.hpp:46-47)."""
    eps0, qunit, navo = 8.854187817e-12, 1.602176565e-19, 6.02214129e23
    return qunit * qunit * 1.0e-3 * navo / (4.0 * math.pi * eps0 * 1.0e-10)


def orientation_rotations(theta, nphi, npsi, mrso):
    """(no, 3, 3) rotation matrices, orientation index (theta, phi, psi) with
    psi fastest, phi = i 2pi/nphi, psi = k 2pi/(mrso npsi)
    (common/MDFT_Grid.hpp:224-238, 283-310)."""
    rows = []
    dphi, dpsi = 2 * math.pi / nphi, 2 * math.pi / mrso / npsi
    for th in theta:
        for i in range(nphi):
            for k in range(npsi):
                ct, st = math.cos(th), math.sin(th)
                cp, sp = math.cos(i * dphi), math.sin(i * dphi)
                cs, ss = math.cos(k * dpsi), math.sin(k * dpsi)
                rows.append([[ct * cp * cs - sp * ss, -ct * cp * ss - sp * cs, st * cp],
                             [ct * sp * cs + cp * ss, -ct * sp * ss + cp * cs, st * sp],
                             [-st * cs, st * ss, ct]])
    return np.array(rows)


def vext_lj_coulomb(n, box, theta, nphi, npsi, mrso, solvent_sites, solute_sites, vmax, with_size=False):
    """(N, no) external potential, N in (x, y, z) order with z fastest and
    grid node (i, j, k) at (i dx, j dy, k dz); with_size: also the sum of the
    magnitudes of its terms (the scale of its rounding error)."""
    nx, ny, nz = n
    L = np.asarray(box, np.float64)
    d = L / np.asarray(n, np.float64)
    R = orientation_rotations(theta, nphi, npsi, mrso)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pts = np.stack([ix.ravel() * d[0], iy.ravel() * d[1], iz.ravel() * d[2]], axis=1)  # (N, 3)
    sv = np.asarray(solvent_sites, np.float64).reshape(-1, 6)
    su = np.asarray(solute_sites, np.float64).reshape(-1, 6)
    qf = qfact()
    v = np.zeros((pts.shape[0], R.shape[0]))
    size = np.zeros_like(v)
    for a in range(sv.shape[0]):
        off = R @ sv[a, 3:6]                                        # (no, 3)
        pos = pts[:, None, :] + off[None, :, :]                     # (N, no, 3)
        for s in range(su.shape[0]):
            dd = pos - su[s, 3:6]
            dd = dd - L * np.rint(dd / L)
            d2 = np.maximum((dd * dd).sum(axis=2), 1e-12)
            eps = math.sqrt(sv[a, 2] * su[s, 2])
            if eps != 0.0:
                sig = 0.5 * (sv[a, 1] + su[s, 1])
                s6 = (sig * sig / d2) ** 3
                v += 4.0 * eps * (s6 * s6 - s6)
                size += 4.0 * eps * (s6 * s6 + s6)
            qq = qf * sv[a, 0] * su[s, 0]
            if qq != 0.0:
                v += qq / np.sqrt(d2)
                size += abs(qq) / np.sqrt(d2)
    v = np.where(np.isfinite(v), np.clip(v, -vmax, vmax), vmax)
    return (v, size) if with_size else v


def energy_terms(xi, vexc, vext, w, kT, rho0, dv, prefactor):
    """([E_total, E_id, E_ext, E_exc, max |g|], g) for fields of shape (N, no)."""
    xi = np.asarray(xi, np.float64).reshape(-1, w.size)
    vexc = np.asarray(vexc, np.float64).reshape(xi.shape)
    vext = np.zeros_like(xi) if vext is None else np.asarray(vext, np.float64).reshape(xi.shape)
    x2 = xi * xi
    lx = np.where(x2 > 0, np.log(np.where(x2 > 0, x2, 1.0)), 0.0)
    wo = w[None, :]
    e_id = kT * rho0 * dv * (wo * (x2 * lx - x2 + 1.0)).sum()
    e_ext = rho0 * dv * (wo * x2 * vext).sum()
    e_exc = prefactor * rho0 * (wo * vexc * (x2 - 1.0)).sum()
    g = 2.0 * xi * wo * (rho0 * dv * (kT * lx + vext) + 2.0 * prefactor * rho0 * vexc)
    return np.array([e_id + e_ext + e_exc, e_id, e_ext, e_exc, np.abs(g).max()]), g
