"""The oracle against its committed golden fixture (CPU).

tests/golden/oracle_wakefield_small.json was written by
tests/golden/make_golden.py; this test re-runs the same deck and requires
the same summary, so any change of the restatement's results is seen.
"""
import json
import os

import numpy as np
import pytest

pytest.importorskip("oracle.oracle")

HERE = os.path.dirname(os.path.abspath(__file__))


def test_oracle_matches_golden_fixture():
    from tests.golden import make_golden
    with open(os.path.join(HERE, "golden", "oracle_wakefield_small.json")) as f:
        gold = json.load(f)
    now = make_golden.generate()
    assert now["steps"] == gold["steps"]
    a, b = now["result"], gold["result"]
    for k in ("n_live", "n_shifts", "first_ids"):
        assert a[k] == b[k], k
    assert a["x_grid_min"] == pytest.approx(b["x_grid_min"], rel=1e-14)
    assert a["kinetic_energy"] == pytest.approx(b["kinetic_energy"], rel=1e-11)
    for k, v in b["first_particles"].items():
        np.testing.assert_allclose(a["first_particles"][k], v, rtol=1e-12, atol=0, err_msg=k)
    for name in ("exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"):
        for key in ("l2", "sum_re", "sum_im"):
            ref = np.asarray(b[name][key])
            scale = max(np.max(np.abs(b[name]["l2"])), 1e-300)
            np.testing.assert_allclose(a[name][key], ref, rtol=1e-10, atol=1e-10 * scale, err_msg=f"{name}.{key}")


def test_full_deck_record():
    """The committed record of the whole 2000-step wakefield deck (written on
    a GB300 by the opt-in test_full_wakefield_deck_against_oracle): the FP64
    form against the oracle with equal counts and window shifts and per-mode
    Ez within 1e-9, the mixed form within its 1e-3 Ez bar."""
    with open(os.path.join(HERE, "golden", "full_deck_summary.json")) as f:
        rec = json.load(f)
    assert rec["steps"] == 2000
    fp, mx = rec["against_oracle"]["fp64"], rec["against_oracle"]["mixed"]
    assert fp["n_live"]["run"] == fp["n_live"]["against"]
    assert fp["n_shifts"]["run"] == fp["n_shifts"]["against"] > 500
    assert max(fp["ez_rel_l2_per_mode"]) < 1e-9
    assert max(mx["ez_rel_l2_per_mode"]) <= 1e-3
    assert mx["n_shifts"]["run"] == mx["n_shifts"]["against"]
