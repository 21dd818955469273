"""Field ionisation (physics_packages/ionise.F90) on the CPU: the constants
of initialise_ionisation computed by the product's host code equal the
oracle's bit for bit, they meet known answers, and an oracle run of the
reference's field_ionisation example deck ionises carbon with charge and
particle bookkeeping intact."""
import ctypes as C

import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi

oracle = pytest.importorskip("oracle.oracle")

HARTREE_EV = 27.211385  # atomic unit of energy in eV (CODATA 2010, the reference's constants)


def _product_constants(deck, model):
    lib = cg.load()
    out = np.zeros((len(deck.species), abi.ION_NCONST))
    omega = deck.lasers[0].omega if deck.lasers else 0.0
    abi.check("cyl_ionisation_constants",
              lib.cyl_ionisation_constants(deck.ionisation_descs(), deck.species_descs(), len(deck.species),
                                           model, omega, out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


@pytest.mark.parametrize("model", [0, abi.IONISE_BSI, abi.IONISE_MULTIPHOTON, abi.IONISE_BSI | abi.IONISE_MULTIPHOTON])
def test_constants_match_oracle(model):
    deck = cg.field_ionisation_deck(model=model)
    a = _product_constants(deck, model)
    orc = oracle.Oracle(deck)
    b = orc.ionisation_constants()
    assert np.array_equal(a, b), np.argwhere(a != b)


def test_constants_known_answers():
    """Carbon's first three levels in atomic units: the ADK field scale
    2 (2 Ip)^(3/2), the barrier-suppression threshold, which is the classical
    over-the-barrier field Ip^2 / (4 Z), and the exponent 2 n* - 1.5 with
    n* = Z / sqrt(2 Ip)."""
    deck = cg.field_ionisation_deck()
    c = _product_constants(deck, abi.IONISE_BSI | abi.IONISE_MULTIPHOTON)
    for k, ev in enumerate((11.2602880, 24.383154, 47.88778)):
        ip = ev / HARTREE_EV
        z = k + 1.0
        n_star = z / np.sqrt(2 * ip)
        assert c[k, 0] == pytest.approx(cg.deck.M0 / deck.species[k].mass, rel=1e-12)  # released mass fraction
        assert c[k, 1] == pytest.approx(2 * n_star - 1.5, rel=1e-6)
        assert c[k, 2] == pytest.approx(2 * (2 * ip) ** 1.5, rel=1e-6)
        assert c[k, 7] == pytest.approx(ip ** 2 / (4 * z), rel=1e-6)
        assert 0 < c[k, 10] < c[k, 8]  # Keldysh field below the ADK maximum
    assert np.all(c[3:] == 0.0)


def test_oracle_ionises_the_carbon_slab():
    """200 steps of the example deck on the oracle: the laser reaches the slab
    (x = 3.05 um) near step 160 and C+ appears; every ionisation releases one
    electron into its level's species with the parent's position and weight;
    the total charge sum(q w) stays zero."""
    deck = cg.field_ionisation_deck()
    lib = oracle.load()
    lib.orc_set_threads(4)
    orc = oracle.Oracle(deck, load_species=True)
    orc.initialise()
    orc.step(200)
    lib.orc_set_threads(1)
    n = [orc.state().n_live[i] for i in range(7)]
    assert n[1] > 0 and sum(n[:4]) == 30517
    # electrons of level k = ions that passed level k
    assert n[4] == n[1] + n[2] + n[3]
    assert n[5] == n[2] + n[3]
    assert n[6] == n[3]
    q = sum(deck.species[i].charge * orc.particles(i).w.sum() for i in range(7))
    scale = cg.deck.Q0 * orc.particles(0).w.sum()
    assert abs(q) <= 1e-12 * scale
    e = orc.particles(4)
    assert np.all(e.id >= (1 << 62))
