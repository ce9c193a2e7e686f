"""The solvent set-up (mini_mdft_gb300/solvent.py) against the reference's
Solvents (common/MDFT_Solvent.hpp:308-560) and its unit test
(unit_test/Test_Solvent.cpp:44-93): model constants, mole fractions,
per-species densities, the prefactor, and the Throw_If messages."""
import math

import numpy as np
import pytest

from mini_mdft_gb300 import MdftError, Solvents, check_mole_fractions, mole_fractions
from mini_mdft_gb300 import inputs as I


@pytest.mark.parametrize("mmax", [0, 3, 5])
def test_solvent_init_matches_the_reference_test_values(mmax):
    # unit_test/Test_Solvent.cpp:44-62 builds the expected spce solvent,
    # :85-100 compares it field by field with ASSERT_EQ
    s = Solvents("spce", 1, mmax, 2).m_solvents[0]
    n0 = 0.0332891
    assert s.m_name == "spce"
    assert s.m_molrotsymorder == 2
    assert s.m_nsite == 3
    assert s.m_n0 == n0
    assert s.m_rho0 == n0 / (8 * math.pi * math.pi / 2)
    assert s.m_relativePermittivity == 71
    assert tuple(s.m_npluc) == (1, 6, 75, 252, 877, 2002)
    assert s.m_n_line_cfile == 1024
    assert s.m_mole_fraction == 1.0
    assert np.array_equal(s.m_sites[:, 0], [-0.8476, 0.4238, 0.4238])
    assert np.array_equal(s.m_sites[:, 1], [3.166, 0.0, 0.0])
    assert np.array_equal(s.m_sites[:, 2], [0.65, 0.0, 0.0])


def test_single_species_constants_equal_the_path_helpers():
    assert Solvents("tip3p", 1, 3, 2).constants() == I.tip3p_constants(2)
    assert Solvents("spce", 1, 3, 2).constants() == I.solvent_constants(I.SPCE_N0, 2)
    assert Solvents("spce", 1, 3, 2).np_luc() == 252
    assert Solvents("spce", 1, 5, 2).np_luc() == 2002


def test_mole_fractions():
    assert mole_fractions(1) == [1.0]
    assert mole_fractions(2) == [0.5, 0.5]
    assert mole_fractions(3) == [1.0 / 3.0] * 3  # sum within 100 eps of one
    assert mole_fractions(7) == [1.0 / 7.0] * 7
    with pytest.raises(MdftError, match="Sum of all mole fraction should be equal to one"):
        mole_fractions(0)
    with pytest.raises(MdftError, match="Sum of all mole fraction should be equal to one"):
        check_mole_fractions([0.5, 0.6])
    with pytest.raises(MdftError, match="Mole fractions should be between 0 and 1"):
        check_mole_fractions([1.5, -0.5])


@pytest.mark.parametrize("model,pure_n0", [("spce", I.SPCE_N0), ("tip3p", I.TIP3P_N0)])
def test_species_densities_scale_with_the_mole_fraction(model, pure_n0):
    one = Solvents(model, 1, 3, 2)
    for nb in (2, 3, 4):
        many = Solvents(model, nb, 3, 2)
        assert len(many.m_solvents) == nb
        for s in many.m_solvents:
            assert s.m_mole_fraction == 1.0 / nb
            assert s.m_n0 == pure_n0 * (1.0 / nb)
            assert s.m_rho0 == s.m_n0 / (8 * math.pi * math.pi / 2)
        # the prefactor uses species 0's density, which includes its mole fraction
        assert many.m_prefactor == pytest.approx(one.m_prefactor * nb, rel=1e-15)
        rho0, pref = many.constants(0)
        assert rho0 == many.m_solvents[0].m_rho0 and pref == many.m_prefactor


def test_model_variants():
    m = Solvents("spce-m", 1, 3, 2).m_solvents[0]
    assert m.m_name == "spce" and np.array_equal(m.m_sites[:, 0], [-1.0, 0.5, 0.5])
    t = Solvents("tip3p-m", 1, 3, 2).m_solvents[0]
    assert t.m_name == "tip3p" and np.array_equal(t.m_sites[:, 0], [-0.95, 0.475, 0.475])
    assert t.m_relativePermittivity == 91 and t.m_n0 == 0.03349459
    h = Solvents("spce-h", 1, 3, 2).m_solvents[0]
    assert h.m_name == "spce" and np.array_equal(h.m_sites, I.SPCE_SITES)


@pytest.mark.parametrize("sites", [I.SPCE_SITES, I.TIP3P_SITES])
def test_site_geometry_is_the_water_model(sites):
    o, h1, h2 = (np.asarray(r[3:6]) for r in sites)
    assert not o.any()  # oxygen at the molecular origin
    b1, b2 = np.linalg.norm(h1), np.linalg.norm(h2)
    assert abs(b1 - b2) < 1e-15
    cos = h1 @ h2 / (b1 * b2)
    angle = math.degrees(math.acos(cos))
    if sites is I.SPCE_SITES:  # SPC/E: 1 A bonds, 109.47 degrees (coordinates to 6-7 digits)
        assert abs(b1 - 1.0) < 1e-6 and abs(angle - 109.47) < 1e-2
    else:  # TIP3P: 0.9572 A bonds, 104.52 degrees
        assert abs(b1 - 0.9572) < 1e-4 and abs(angle - 104.52) < 1e-2


def test_errors_carry_the_reference_messages():
    with pytest.raises(MdftError, match="Critical error. Solvent: water not recognized."):
        Solvents("water", 1, 3, 2)
    with pytest.raises(MdftError, match="solvent spce only avail with mmax between 0 and 5"):
        Solvents("spce-m", 1, 6, 2)
    with pytest.raises(MdftError, match="solvent tip3p only avail with mmax between 0 and 5"):
        Solvents("tip3p-m", 2, -1, 2)
    with pytest.raises(MdftError, match="molrotsymorder is different from the grid molrotsymorder"):
        Solvents("spce", 1, 3, 1)
