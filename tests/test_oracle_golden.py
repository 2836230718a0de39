"""The CPU oracle against snapshots of the reference binary (tests/golden).

Pins the oracle: pair sets and contact flags bit-exact at every snapshot
(including several neighbour rebuilds with history carry-over), per-step
forces/torques within FORCE_RTOL, trajectories within TRAJ_RTOL.
"""
import numpy as np
import pytest

from golden_io import (FORCE_RTOL, HIST_RTOL, canonical_pairs, compare_pairs, load_golden,
                       max_rel, sort_by_tag)
from oracle.binding import Oracle

CASES = ["dense_hertz", "poly_cdt", "hooke"]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    case, snaps = load_golden(name)
    o = Oracle(case)
    o.setup()
    prev = 0
    for st in sorted(snaps):
        if st > prev:
            o.run(st - prev)
            prev = st
        g = sort_by_tag(o.atoms())
        r = snaps[st]
        assert np.array_equal(g["tag"], r["tag"])
        # forces and torques of this step (reference: rounding-level agreement)
        tol = FORCE_RTOL if st <= 100 else 1e-9
        assert max_rel(g["f"], r["f"]) < tol, (name, st)
        assert max_rel(g["torque"], r["torque"]) < tol, (name, st)
        assert max_rel(g["x"], r["x"], scale=1.0) < 1e-12
        assert max_rel(g["v"], r["v"]) < (1e-9 if st <= 100 else 1e-8)
        pg = o.pairs()
        gp = canonical_pairs(pg["tag_i"], pg["tag_j"], pg["shift"], pg["flag"], pg["hist"])
        rp = canonical_pairs(r["pair_tag_i"], r["pair_tag_j"], r["pair_shift"], r["pair_flag"],
                             r["pair_hist"])
        missing, extra, flagmis, hm = compare_pairs(gp, rp)
        assert not missing and not extra, (name, st, len(missing), len(extra))
        assert not flagmis
        assert all(gp[k][0] == rp[k][0] for k in rp), "contact flag bits differ"
        assert hm < (HIST_RTOL if st <= 100 else 1e-8)
        wh = o.wall_history(0)[np.argsort(o.atoms()["tag"], kind="stable")]
        assert max_rel(wh, r["wall0_hist"]) < (HIST_RTOL if st <= 100 else 1e-8)
    assert o.nrebuilds >= 2, "fixture must exercise history carry-over across rebuilds"


def test_fixture_has_periodic_and_wall_contacts():
    case, snaps = load_golden("dense_hertz")
    s0 = snaps[0]
    assert (np.abs(s0["pair_shift"]).sum(axis=1) > 0).any(), "no periodic image pairs"
    assert (np.abs(snaps[100]["wall0_hist"]).sum(axis=1) > 0).any(), "no wall contacts"
