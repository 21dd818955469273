"""Generate tests/golden/oracle_wakefield_small.json from the CPU oracle.

The fixture freezes the oracle's output on a small windowed, laser-driven
wakefield deck (64 x 24 cells, modes 0..1, 2 particles per cell, the window
starting at step 10), 24 steps from t = 0, single-threaded.  It guards the
restatement against accidental change; the oracle's independent pins are in
tests/test_oracle_pins.py.

    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "oracle_wakefield_small.json")
STEPS = 24


def small_deck():
    import cylindrical_epoch_gb300 as cg
    deck = cg.wakefield(nx=64, ny=24, ppc=2, density=3.0e24, ramp=1.0e-6)
    deck.window_start_time = 10 * 5.0e-17
    return deck


def summarise(orc, deck):
    out = {}
    for name in ("exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"):
        a = orc.field(name)
        out[name] = {
            "l2": [float(np.sqrt(np.sum(np.abs(a[m]) ** 2))) for m in range(deck.n_mode)],
            "sum_re": [float(np.sum(a[m].real)) for m in range(deck.n_mode)],
            "sum_im": [float(np.sum(a[m].imag)) for m in range(deck.n_mode)],
        }
    p = orc.particles(0).sorted_by_id()
    s = orc.state()
    d = orc.diagnostics()
    out["n_live"] = int(p.n)
    out["n_shifts"] = int(s.n_shifts)
    out["x_grid_min"] = float(s.x_grid_min)
    out["kinetic_energy"] = float(d.kinetic_energy)
    out["first_particles"] = {k: [float(v) for v in getattr(p, k)[:16]] for k in ("x", "y", "z", "px", "py", "pz", "w")}
    out["first_ids"] = [int(v) for v in p.id[:16]]
    return out


def generate():
    from oracle.oracle import Oracle, load
    load().orc_set_threads(1)
    deck = small_deck()
    orc = Oracle(deck, load_species=True)  # the oracle's own loader and KISS stream
    orc.initialise()
    orc.step(STEPS)
    return {"deck": "wakefield 64x24 m=0..1 2 ppc, density 3e24, ramp 1 um, window from step 10",
            "steps": STEPS, "result": summarise(orc, deck)}


if __name__ == "__main__":
    with open(OUT, "w") as f:
        json.dump(generate(), f, indent=1)
    print(OUT)
