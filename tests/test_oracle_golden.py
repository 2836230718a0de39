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

CASES = ["dense_hertz", "poly_cdt", "hooke", "fibre_bond", "fibre_bond_stress", "silo_cyl"]


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
        order = np.argsort(o.atoms()["tag"], kind="stable")
        nw = len([k for k in r if k.startswith("wall") and k.endswith("_hist")])
        for w in range(nw):  # planes, then cylinders
            wh = o.wall_history(w)[order]
            assert max_rel(wh, r["wall%d_hist" % w]) < (HIST_RTOL if st <= 100 else 1e-8), (name, st, w)
    assert o.nrebuilds >= 2, "fixture must exercise history carry-over across rebuilds"


MESH_CASES = ["hopper_mesh", "hopper_mesh_cdt"]


def mesh_contact_map(tags, tris, slots, hists):
    return {(int(t), int(tr)): (int(sl), np.asarray(h)) for t, tr, sl, h in zip(tags, tris, slots, hists)}


@pytest.mark.parametrize("name", MESH_CASES)
def test_oracle_mesh_walls_match_reference(name):
    """Triangle-mesh walls: the derived edge/corner activity equals the
    reference's, and the mesh contact set, slot layout and histories match at
    every snapshot (including atoms leaving through the outlet)."""
    case, snaps = load_golden(name)
    o = Oracle(case)
    ea, ca = o.mesh_flags(0)
    assert np.array_equal(ea, snaps[0]["mesh0_edge_active"])
    assert np.array_equal(ca, snaps[0]["mesh0_corner_active"])
    o.setup()
    prev = 0
    for st in sorted(snaps):
        if st > prev:
            o.run(st - prev)
            prev = st
        g = sort_by_tag(o.atoms())
        r = snaps[st]
        assert np.array_equal(g["tag"], r["tag"])
        tol = FORCE_RTOL if st <= 100 else 1e-9
        assert max_rel(g["f"], r["f"]) < tol and max_rel(g["torque"], r["torque"]) < tol, (name, st)
        mc = o.mesh_contacts(0)
        gm = mesh_contact_map(mc["tag"], mc["tri"], mc["slot"], mc["hist"])
        rm = mesh_contact_map(r["mesh0_contact_tag"], r["mesh0_contact_tri"], r["mesh0_contact_slot"],
                              r["mesh0_contact_hist"])
        assert set(gm) == set(rm), (name, st)
        assert all(gm[k][0] == rm[k][0] for k in rm), "slot layout differs"
        hs = max([np.abs(v[1]).max() for v in rm.values()] + [1e-300])
        assert max([np.abs(gm[k][1] - rm[k][1]).max() for k in rm] + [0.0]) / hs < HIST_RTOL
    assert len(snaps[0]["mesh0_contact_tag"]) > 20, "fixture must start with wall contacts"


def test_fixture_has_periodic_and_wall_contacts():
    case, snaps = load_golden("dense_hertz")
    s0 = snaps[0]
    assert (np.abs(s0["pair_shift"]).sum(axis=1) > 0).any(), "no periodic image pairs"
    assert (np.abs(snaps[100]["wall0_hist"]).sum(axis=1) > 0).any(), "no wall contacts"


def test_oracle_moving_mesh_press_matches_reference():
    """fix move/mesh linear: a two-triangle plate pressing bonded fibres in a
    box of primitive walls.  Plate node positions bit-exact at every
    snapshot, rebuilds triggered by the plate's travel, forces, pair and bond
    sets, plate contact slots and histories as the reference's."""
    case, snaps = load_golden("fibre_press")
    o = Oracle(case)
    o.setup()
    prev = 0
    for st in sorted(snaps):
        if st > prev:
            o.run(st - prev)
            prev = st
        g = sort_by_tag(o.atoms())
        r = snaps[st]
        assert np.array_equal(o.mesh_nodes(0), r["mesh0_node"]), st
        assert np.array_equal(g["tag"], r["tag"])
        tol = FORCE_RTOL if st <= 100 else 1e-9
        assert max_rel(g["f"], r["f"]) < tol and max_rel(g["torque"], r["torque"]) < tol, st
        pg = o.pairs()
        gp = canonical_pairs(pg["tag_i"], pg["tag_j"], pg["shift"], pg["flag"], pg["hist"])
        rp = canonical_pairs(r["pair_tag_i"], r["pair_tag_j"], r["pair_shift"], r["pair_flag"],
                             r["pair_hist"])
        missing, extra, flagmis, hm = compare_pairs(gp, rp)
        assert not missing and not extra and not flagmis, st
        assert all(gp[k][0] == rp[k][0] for k in rp)
        assert hm < HIST_RTOL, (st, hm)
        mc = o.mesh_contacts(0)
        gm = mesh_contact_map(mc["tag"], mc["tri"], mc["slot"], mc["hist"])
        rm = mesh_contact_map(r["mesh0_contact_tag"], r["mesh0_contact_tri"], r["mesh0_contact_slot"],
                              r["mesh0_contact_hist"])
        assert set(gm) == set(rm) and all(gm[k][0] == rm[k][0] for k in rm), st
        for w in range(5):
            wh = o.wall_history(w)[np.argsort(o.atoms()["tag"], kind="stable")]
            assert max_rel(wh, r["wall%d_hist" % w]) < HIST_RTOL
    assert len(snaps[600]["mesh0_contact_tag"]) >= 5
    assert o.nrebuilds >= 4, o.nrebuilds


def test_oracle_rotating_mesh_matches_reference():
    """fix move/mesh rotate: a paddle stirring a lattice.  Paddle nodes
    bit-exact at every snapshot (quaternion arithmetic in the reference's
    order), rebuilds forced by the paddle's travel, forces, pair sets and
    paddle contact slots and histories as the reference's."""
    case, snaps = load_golden("mixer_rotate")
    o = Oracle(case)
    o.setup()
    prev = 0
    for st in sorted(snaps):
        if st > prev:
            o.run(st - prev)
            prev = st
        g = sort_by_tag(o.atoms())
        r = snaps[st]
        assert np.array_equal(o.mesh_nodes(0), r["mesh0_node"]), st
        assert np.array_equal(g["tag"], r["tag"])
        tol = FORCE_RTOL if st <= 100 else 1e-9
        assert max_rel(g["f"], r["f"]) < tol and max_rel(g["torque"], r["torque"]) < tol, st
        pg = o.pairs()
        gp = canonical_pairs(pg["tag_i"], pg["tag_j"], pg["shift"], pg["flag"], pg["hist"])
        rp = canonical_pairs(r["pair_tag_i"], r["pair_tag_j"], r["pair_shift"], r["pair_flag"],
                             r["pair_hist"])
        missing, extra, flagmis, hm = compare_pairs(gp, rp)
        assert not missing and not extra and not flagmis, st
        assert hm < HIST_RTOL, (st, hm)
        mc = o.mesh_contacts(0)
        gm = mesh_contact_map(mc["tag"], mc["tri"], mc["slot"], mc["hist"])
        rm = mesh_contact_map(r["mesh0_contact_tag"], r["mesh0_contact_tri"], r["mesh0_contact_slot"],
                              r["mesh0_contact_hist"])
        assert set(gm) == set(rm), st
        assert all(gm[k][0] == rm[k][0] for k in rm), st
    assert o.nrebuilds >= 4


def test_oracle_insertion_joins_after_initial_integrate():
    """orc_insert_atoms: staged atoms join at the next step after its initial
    integration (they are not drifted at that step), and that step rebuilds."""
    case, _ = load_golden("dense_hertz")
    o = Oracle(case)
    o.setup()
    o.run(5)
    nreb = o.nrebuilds
    n0 = len(o.atoms()["tag"])
    x = np.array([[1e-3, 1e-3, 0.013]])
    new = dict(tag=np.array([100000], np.int32), type=np.array([1], np.int32), x=x,
               v=np.array([[0.0, 0.0, -1.0]]), omega=np.zeros((1, 3)), radius=np.array([0.9e-3]),
               rmass=np.array([4.0 / 3.0 * np.pi * 0.9e-3 ** 3 * 2500.0]))
    o.insert(new)
    o.run(1)
    a = o.atoms()
    assert len(a["tag"]) == n0 + 1
    assert o.nrebuilds == nreb + 1
    i = int(np.nonzero(a["tag"] == 100000)[0][0])
    # no drift at the insertion step; the final half-kick used the step's forces
    assert np.array_equal(a["x"][i], x[0])
    assert a["v"][i][2] < -1.0
