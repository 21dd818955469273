"""Full-size check of both GPU forms against the CPU oracle (not collected by
pytest: it needs a GPU and several minutes of the host's cores).

Runs the 2048 x 256, m = 0..1, 8 ppc laser wakefield deck for K steps (2000
by default) three times from the same loaded state: the oracle (FP64
restatement of the reference, OpenMP on all host threads), the plain FP64
GPU form and the mixed GPU form; then compares each GPU run with the oracle
(per-mode Ez relative L2, on-axis wake amplitude, electron kinetic-energy
moments, counts, window shifts, continuity residual of one further step).
Prints one JSON object.

    python tests/oracle_full_deck.py [K]
"""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    steps = int(sys.argv[1]) if len(sys.argv) > 1 else 2000
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    from cylindrical_epoch_gb300.diagnostics import compare_runs
    from oracle.oracle import Oracle, load

    lib = load()
    lib.orc_set_threads(os.cpu_count() or 1)
    d64 = cg.wakefield(precision=abi.PREC_FP64)
    d32 = cg.wakefield(precision=abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    out = {"deck": "wakefield 2048x256 m=0..1 8 ppc", "steps": steps, "oracle_threads": os.cpu_count()}
    t0 = time.perf_counter()
    orc = Oracle(d64, particles=parts, rng=rng)
    orc.initialise()
    orc.step(steps)
    out["oracle_seconds"] = time.perf_counter() - t0
    res = {}
    for name, deck in (("fp64", d64), ("mixed", d32)):
        run = cg.Run(deck, particles=parts, rng=rng)
        if deck.precision == abi.PREC_MIXED:
            run.tune_tiles()
        run.step(steps, graph=True)
        res[name] = compare_runs(run, orc, deck, residual=False)
        run.close()
    out["against_oracle"] = res
    print(json.dumps(out))


if __name__ == "__main__":
    main()
