"""Solvent set-up of common/MDFT_Solvent.hpp:308-560 (struct Solvents): a
solvent model name, the number of solvent species and the angular grid give
each species its mole fraction, bulk densities n0 and rho0, and the
excess term's prefactor.  These are the constants that get_delta_rho,
get_delta_f, the minimiser and the job server take as arguments.

Like the reference:

- one model name serves every species (:409-411);
- the species get equal mole fractions (:375-405);
- each species' n0 is the model's pure-solvent density times its mole
  fraction, and rho0 = n0 / (8 pi^2 / mrso) (:426-427);
- the prefactor -2 kT 4 pi^2 / mrso / n0 uses species 0 (:366-368);
- the cproj term evaluates species 0 (src/mini-mdft.hpp:138).

Errors raise MdftError with the reference's Throw_If messages.

Site positions: the reference's Solvent::init (:199-203) puts site i at
(r0[i], r1[i], r2[i]), which would place the SPC/E oxygen at
(0, 0.816, -0.816) A.  Here the three vectors are the three sites'
positions: the oxygen at the origin, 1 A bonds, 109.47 degrees.  No
reference code reads the positions; the external potential here does.
"""
import math
import sys

import numpy as np

from . import inputs as I
from ._lib import MdftError

# npluc[mmax]: the number of Luc c(q) entries per mmax, and the c(q) file's
# line count (common/MDFT_Solvent.hpp:431-432, the same for every model)
NPLUC = (1, 6, 75, 252, 877, 2002)
N_LINE_CFILE = 1024


def _with_charges(sites, charges):
    s = np.array(sites, dtype=np.float64)
    s[:, 0] = charges
    return s


# model name -> (stored name, sites (q, sigma, epsilon, x, y, z), pure n0 [1/A^3],
# molrotsymorder, relative permittivity); common/MDFT_Solvent.hpp:415-530
MODELS = {
    "spce": ("spce", I.SPCE_SITES, I.SPCE_N0, 2, 71.0),
    "spce-h": ("spce", I.SPCE_SITES, I.SPCE_N0, 2, 71.0),
    "spce-m": ("spce", _with_charges(I.SPCE_SITES, (-1.0, 0.5, 0.5)), I.SPCE_N0, 2, 71.0),
    "tip3p": ("tip3p", I.TIP3P_SITES, I.TIP3P_N0, 2, 91.0),
    "tip3p-m": ("tip3p", _with_charges(I.TIP3P_SITES, (-0.95, 0.475, 0.475)), I.TIP3P_N0, 2, 91.0),
}


def _throw_if(cond, msg):
    if cond:
        raise MdftError(1, msg)


def mole_fractions(nb_solvent):
    """Equal mole fractions of nb_solvent species, checked as the reference
    checks them (common/MDFT_Solvent.hpp:375-405)."""
    if nb_solvent < 1:
        fr = []  # no species: the sum check fails, as in the reference
    else:
        fr = [1.0] if nb_solvent == 1 else [1.0 / float(nb_solvent)] * nb_solvent
    check_mole_fractions(fr)
    return fr


def check_mole_fractions(fractions):
    """Sum within 100 machine epsilons of one, each in [0, 1]
    (common/MDFT_Solvent.hpp:387-404)."""
    total = 0.0
    for f in fractions:
        total += f
    _throw_if(abs(total - 1.0) > sys.float_info.epsilon * 100,
              "Critial error. Sum of all mole fraction should be equal to one.")
    _throw_if(any(f < 0 or f > 1 for f in fractions),
              "Critical errror. Mole fractions should be between 0 and 1")


class Solvent:
    """One species (common/MDFT_Solvent.hpp:62-206, the members the path
    uses), with the reference's member names."""

    def __init__(self, name, sites, n0, rho0, molrotsymorder, relative_permittivity, mole_fraction):
        self.m_name = name
        self.m_sites = np.ascontiguousarray(sites, dtype=np.float64)
        self.m_nsite = len(self.m_sites)
        self.m_n0 = n0
        self.m_rho0 = rho0
        self.m_molrotsymorder = molrotsymorder
        self.m_relativePermittivity = relative_permittivity
        self.m_mole_fraction = mole_fraction
        self.m_npluc = NPLUC
        self.m_n_line_cfile = N_LINE_CFILE


class Solvents:
    """Solvents(solvent, nb_solvent, mmax, mrso, temperature): the species of
    one solvent model (common/MDFT_Solvent.hpp:343-372).  m_solvents[i] are
    the species; m_prefactor is the excess term's prefactor."""

    def __init__(self, solvent="spce", nb_solvent=1, mmax=3, mrso=2, temperature=298.0):
        self.m_solvents = []
        fractions = mole_fractions(nb_solvent)
        for fr in fractions:
            _throw_if(solvent not in MODELS, "Critical error. Solvent: " + solvent + " not recognized.")
            name, sites, n0_pure, mrso_model, eps_r = MODELS[solvent]
            n0 = n0_pure * fr
            rho0 = n0 / (8 * math.pi * math.pi / mrso_model)
            self.m_solvents.append(Solvent(name, sites, n0, rho0, mrso_model, eps_r, fr))
            _throw_if(mmax > 5 or mmax < 0, "solvent %s only avail with mmax between 0 and 5" % name)
        _throw_if(any(s.m_molrotsymorder != mrso for s in self.m_solvents),
                  "at least one solvent molrotsymorder is different from the grid molrotsymorder")
        kbt = I.kT(temperature)
        n00 = self.m_solvents[0].m_n0
        self.m_prefactor = -2 * kbt * 4 * math.pi * math.pi / mrso / n00
        self.m_kbt = kbt
        self.m_mmax = mmax

    def constants(self, i=0):
        """(rho0, prefactor) of species i: the arguments of get_delta_rho,
        get_delta_f and the minimiser."""
        return self.m_solvents[i].m_rho0, self.m_prefactor

    def np_luc(self, i=0):
        """np_luc of species i's c(q) file at this mmax (src/mini-mdft.hpp:125)."""
        return self.m_solvents[i].m_npluc[self.m_mmax]
