"""Batched ensemble runner (gb300dem.ensemble): packing on the CPU, and on
the GPU each packed system against the oracle running that system alone.

Every system takes its own neighbour decision, as it would alone, so under
the default `neigh_modify every 1 delay 0 check yes` as well as with a
rebuild every step (`check no`) every system must match its standalone run:
its rebuild count, forces within FORCE_RTOL per step while the trajectories
agree to rounding, pair sets bit-exact and histories within 1e-9."""
import numpy as np
import pytest

from golden_io import FORCE_RTOL, TRAJ_RTOL, canonical_pairs, compare_pairs, max_rel, sort_by_tag


def _systems(n=5, neigh=(1, 0, 0)):
    from gb300dem import ensemble
    sy = ensemble.settling_systems(11, n, nmin=150, nmax=500)
    for k, s in enumerate(sy):
        s["neigh"] = neigh
        rng = np.random.default_rng(100 + k)
        s["atoms"]["v"] = rng.uniform(-0.5, 0.5, size=s["atoms"]["x"].shape)
    return sy


def test_pack_layout():
    from gb300dem import ensemble
    sy = _systems()
    case, lay = ensemble.pack(sy)
    a = case["atoms"]
    assert len(np.unique(a["tag"])) == len(a["tag"])
    assert case["ntypes"] == len(sy) == case["ensemble"]
    for k, s in enumerate(sy):
        t = k + 1
        sel = a["type"] == t
        assert sel.sum() == len(s["atoms"]["tag"])
        for name in ("Yeff", "Geff", "betaeff", "coeffFrict"):
            assert case[name][t, t] == s[name][1, 1]
        # every system keeps its own coordinates, bit for bit
        assert np.array_equal(a["x"][sel], s["atoms"]["x"])
        assert np.array_equal(a["tag"][sel] - lay["offsets"][k], s["atoms"]["tag"])
        assert case["planes_per_type"][0][1][t] == s["planes"][0][1]


@pytest.mark.gpu
@pytest.mark.parametrize("neigh", [(1, 0, 0), (1, 0, 1)])
def test_ensemble_systems_match_standalone_oracle(neigh):
    from gb300dem import ensemble
    from oracle.binding import Oracle
    sy = _systems(neigh=neigh)
    if neigh[2]:  # faster systems rebuild more often than slower ones
        for k, s in enumerate(sy):
            s["atoms"]["v"] *= 1.0 + 3.0 * k
    e = ensemble.Ensemble(sy)
    e.setup()
    orcs = [Oracle(s) for s in sy]
    for o in orcs:
        o.setup()
    done = 0
    for chunk in ((1, 4, 5, 20) if not neigh[2] else (1, 4, 5, 20, 70)):
        e.step(chunk)
        for o in orcs:
            o.run(chunk)
        done += chunk
        allp = e.sys.pairs()
        for k, (s, o) in enumerate(zip(sy, orcs)):
            a, b = e.system_atoms(k), sort_by_tag(o.atoms())
            assert np.array_equal(a["tag"], b["tag"])
            ftol = FORCE_RTOL if done <= 10 else 1e-7
            assert max_rel(a["f"], b["f"]) < ftol, (k, done, max_rel(a["f"], b["f"]))
            assert max_rel(a["torque"], b["torque"]) < ftol, (k, done)
            assert max_rel(a["x"], b["x"], scale=0.05) < TRAJ_RTOL
            tag0 = e.layout["offsets"][k]
            ntag = len(s["atoms"]["tag"])
            sel = (allp["tag_i"] > tag0) & (allp["tag_i"] <= tag0 + ntag)
            gp = canonical_pairs(allp["tag_i"][sel] - tag0, allp["tag_j"][sel] - tag0, allp["shift"][sel],
                                 allp["flag"][sel], allp["hist"][sel])
            po = o.pairs()
            op = canonical_pairs(po["tag_i"], po["tag_j"], po["shift"], po["flag"], po["hist"])
            missing, extra, flagmis, hm = compare_pairs(gp, op)
            assert not missing and not extra and not flagmis, (k, done)
            assert hm < 1e-9, (k, done, hm)
        reb = e.rebuilds()
        assert [int(r) for r in reb] == [o.nrebuilds for o in orcs], (done, reb, [o.nrebuilds for o in orcs])
    if not neigh[2]:
        assert e.stats()["nrebuilds"] == done + 1
    else:  # the systems' schedules differ
        assert len(set(int(r) for r in e.rebuilds())) > 1
    e.close()


@pytest.mark.gpu
def test_ensemble_launch_shapes_give_identical_results():
    """The autotuner's launch-shape knobs (blocks per SM, threads per block of
    the per-particle kernel) change no result: each particle's sums run in
    one thread in a fixed order whatever the grid."""
    from gb300dem import ensemble
    sy = _systems(n=3)
    out = []
    for tuning in ((8, 1.0, 256), (4, 1.0, 128), (16, 1.0, 64)):
        e = ensemble.Ensemble(sy, tuning=tuning)
        e.setup()
        e.step(30)
        out.append([e.system_atoms(k) for k in range(len(sy))])
        e.close()
    for run in out[1:]:
        for a, b in zip(run, out[0]):
            for key in ("x", "v", "omega", "f", "torque"):
                assert np.array_equal(a[key], b[key]), key


def _run_modes(sy, monkeypatch, chunks):
    """The same ensemble under three rebuild settings: the whole-list path
    at every build (LIGGGHTS_GB300_ENS_FULL), the default (in place where
    possible), and segments without slack (LIGGGHTS_GB300_ENS_SLACK=0: a
    rebuilding system that gains one entry re-lays the list)."""
    from gb300dem import ensemble
    runs = {}
    for name, env in (("full", {"LIGGGHTS_GB300_ENS_FULL": "1"}), ("inplace", {}),
                      ("noslack", {"LIGGGHTS_GB300_ENS_SLACK": "0"})):
        for key in ("LIGGGHTS_GB300_ENS_FULL", "LIGGGHTS_GB300_ENS_SLACK"):
            monkeypatch.delenv(key, raising=False)
        for key, v in env.items():
            monkeypatch.setenv(key, v)
        e = ensemble.Ensemble(sy)
        for key in env:
            monkeypatch.delenv(key, raising=False)
        e.setup()
        out = []
        for chunk in chunks:
            e.step(chunk)
            out.append(([e.system_atoms(k) for k in range(len(sy))], e.sys.pairs(), e.rebuilds().copy(),
                        e.stats()))
        e.close()
        runs[name] = out
    return runs


@pytest.mark.gpu
def test_ensemble_in_place_rebuilds_match_whole_list_rebuilds(monkeypatch):
    """A build where only some systems rebuild runs over those systems'
    atoms, cells and list segments alone; the others stay where they are.
    That must change no bit: atoms, forces, pair sets, histories and the
    per-system build counts equal those of the whole-list path at every
    build, with the segments re-laid out (no slack) or not, and through a
    build at which a rebuilding system loses an atom (the whole-list path
    takes that one: the systems behind it move)."""
    sy = _systems(n=6, neigh=(1, 0, 1))
    for k, s in enumerate(sy):  # fast enough that new pairs form and segments overflow
        s["atoms"]["v"] *= 4.0 * (1.0 + 3.0 * k)
    # an atom of system 3 leaves through the open top of its box
    zhi = sy[3]["boxhi"][2]
    sy[3]["atoms"]["x"][0] = (sy[3]["atoms"]["x"][0, 0], sy[3]["atoms"]["x"][0, 1], zhi - 1e-4)
    sy[3]["atoms"]["v"][0] = (0.0, 0.0, 20.0)
    runs = _run_modes(sy, monkeypatch, (7, 30, 63))
    ref = runs["full"]
    for name in ("inplace", "noslack"):
        for (atoms, pairs, reb, st), (ratoms, rpairs, rreb, rst) in zip(runs[name], ref):
            assert np.array_equal(reb, rreb), name
            assert st["natoms"] == rst["natoms"] and st["nlost"] == rst["nlost"], name
            assert st["npairs"] == rst["npairs"], name
            for a, b in zip(atoms, ratoms):
                for key in ("tag", "x", "v", "omega", "f", "torque"):
                    assert np.array_equal(a[key], b[key]), (name, key)
            for key in rpairs:
                assert np.array_equal(pairs[key], rpairs[key]), (name, key)
    assert ref[-1][3]["nlost"] >= 1
    assert ref[-1][3]["ens_inplace_builds"] == 0 and ref[-1][3]["ens_relayout_builds"] == 0
    last = runs["inplace"][-1][3]
    assert last["ens_inplace_builds"] > 10, last
    assert runs["noslack"][-1][3]["ens_relayout_builds"] > 0
    # the schedules differ between systems, so most builds leave some system out
    assert len(set(int(r) for r in runs["inplace"][-1][2])) > 1
