"""Field ionisation on the device (cyl_set_ionisation, both forms)
against the oracle on the reference's field_ionisation example deck
(example_decks/field_ionisation.deck): carbon ionised by a 3e15 W/cm^2
laser up to C3+, one electron species per level, with the reference's
default model (multiphoton, tunnelling and barrier suppression) and with
plain tunnelling.  Particle counts of every species exact, the same ids in
every species, positions and momenta within 1e-12, fields within the
oracle's own summation-order spread (or 1e-10); and the mixed form, whose
counts follow the oracle's within the FP32 fields' precision."""
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


def test_field_ionisation_mixed_form(gpu_lib):
    """The mixed form with field ionisation against the oracle on the same
    deck and load.  The ionisation probability of each trial follows |E| at
    the particle, which the FP32 fields carry to about 1e-4, so a few
    borderline trials can go the other way: each species' count within 2 %
    of the oracle's.  Exact in the run itself: carbon is conserved, and every
    level's electrons number the ions that passed that level."""
    from oracle.oracle import Oracle, load
    lib = load()
    d64 = cg.field_ionisation_deck()
    dmx = cg.field_ionisation_deck(precision=abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    gpu = cg.Run(dmx, particles=parts, rng=rng)
    orc = Oracle(d64, particles=parts, rng=rng, atan2="shared")
    orc.initialise()
    lib.orc_set_threads(8)
    try:
        gpu.step(280, graph=True)
        orc.step(280)
    finally:
        lib.orc_set_threads(1)
    sg, so = gpu.state(), orc.state()
    g = [sg.n_live[i] for i in range(7)]
    o = [so.n_live[i] for i in range(7)]
    print("mixed-form ionisation counts", g, "oracle", o)
    assert sum(g[:4]) == parts[0].n
    assert g[4] == g[1] + g[2] + g[3] and g[5] == g[2] + g[3] and g[6] == g[3]
    assert g[1] + g[2] + g[3] > 1000
    for i in range(1, 7):
        assert abs(g[i] - o[i]) <= 0.02 * max(o[i], 50), (i, g[i], o[i])
    for n in ("exm", "erm", "etm"):
        a, b = gpu.field(n), orc.field(n)
        print(n, [rel_l2(a[m], b[m]) for m in range(a.shape[0])])
    e1 = rel_l2(gpu.field("erm")[1], orc.field("erm")[1])
    assert e1 < 1e-3, e1


def test_batch_refuses_ionising_runs(gpu_lib):
    deck = cg.field_ionisation_deck(precision=abi.PREC_MIXED)
    runs = [cg.Run(deck), cg.Run(deck)]
    try:
        with cg.Batch(4) as b:
            with pytest.raises(abi.CylError) as e:
                b.step(runs, 16)
            assert e.value.code == abi.CYL_ERR_UNSUPPORTED
    finally:
        for r in runs:
            r.close()
