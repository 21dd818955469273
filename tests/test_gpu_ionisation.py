"""Field ionisation on the device (cyl_set_ionisation, the FP64 form)
against the oracle on the reference's field_ionisation example deck
(example_decks/field_ionisation.deck): carbon ionised by a 3e15 W/cm^2
laser up to C3+, one electron species per level, with the reference's
default model (multiphoton, tunnelling and barrier suppression) and with
plain tunnelling.  Particle counts of every species exact, the same ids in
every species, positions and momenta within 1e-12, fields within the
oracle's own summation-order spread (or 1e-10)."""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"]


@pytest.mark.parametrize("model", [abi.IONISE_MULTIPHOTON | abi.IONISE_BSI, 0])
def test_field_ionisation_parity(gpu_lib, model):
    from oracle.oracle import Oracle, load
    lib = load()
    deck = cg.field_ionisation_deck(model=model)
    parts, rng = cg.host_load(deck)
    gpu = cg.Run(deck, particles=parts, rng=rng)
    orc = Oracle(deck, particles=parts, rng=rng, atan2="shared")
    orc.initialise()
    lib.orc_set_threads(8)
    try:
        for chunk in (160, 40, 80):  # the laser reaches the slab near step 160
            gpu.step(chunk, graph=True)
            orc.step(chunk)
            sg, so = gpu.state(), orc.state()
            for isp in range(len(deck.species)):
                assert sg.n_live[isp] == so.n_live[isp], (chunk, isp, sg.n_live[isp], so.n_live[isp])
    finally:
        lib.orc_set_threads(1)
    assert so.n_live[1] + so.n_live[2] + so.n_live[3] > 1000 and so.n_live[4] > 1000
    for isp in range(len(deck.species)):
        if so.n_live[isp] == 0:
            continue
        a, b = match_by_id(gpu.particles(isp), orc.particles(isp))
        for k in ("x", "y", "z", "px", "py", "pz", "w"):
            assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12, (isp, k)
    for n in FIELDS:
        a, b = gpu.field(n), orc.field(n)
        for m in range(a.shape[0]):
            if np.all(b[m] == 0) and np.all(a[m] == 0):
                continue
            assert rel_l2(a[m], b[m]) < 1e-10, (n, m, rel_l2(a[m], b[m]))


def test_ionisation_refused_in_mixed_form(gpu_lib):
    deck = cg.field_ionisation_deck(precision=abi.PREC_MIXED)
    ion = deck.ionisation
    deck.ionisation = None
    run = cg.Run(deck, initialise=False)
    try:
        deck.ionisation = ion
        rc = run.lib.cyl_set_ionisation(run.h, deck.ionisation_descs(), len(deck.species), 3, 1)
        assert rc == abi.CYL_ERR_UNSUPPORTED
    finally:
        run.close()
