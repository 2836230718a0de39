"""Loading of the golden fixtures and the comparison rules shared by tests.

Comparison rules (the parity contract):
  * pair sets: bit-exact as sets of (owner tag, partner tag, image shift);
    a pair of two owned atoms is canonicalised to (min tag, max tag) with its
    history negated when the orientation flips (the reference stores the
    j-side copy negated, src/fix_contact_history.cpp:400-413);
  * forces and torques: |a - b| <= FORCE_RTOL * max|F| per component
    (per-step, relative to the force norm);
  * trajectories: positions within TRAJ_ATOL_REL of the box size.
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

FORCE_RTOL = 1e-11      # per-step forces/torques, relative to max |F| (|T|)
HIST_RTOL = 1e-9        # shear history, relative to max |shear|
TRAJ_RTOL = 1e-9        # positions/velocities over <= 100 steps, relative


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    case = dict(meta)
    case["boxlo"] = tuple(meta["boxlo"])
    case["boxhi"] = tuple(meta["boxhi"])
    case["periodic"] = tuple(meta["periodic"])
    case["neigh"] = tuple(meta["neigh"])
    case["gravity"] = tuple(meta["gravity"]) if meta["gravity"] is not None else None
    case["planes"] = [tuple(p) for p in meta["planes"]]
    case["meshes"] = [dict(m, nodes=z["mesh%d_nodes" % k]) for k, m in enumerate(meta.get("meshes", []))]
    for k in ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRollFrict", "coeffRestLog"):
        case[k] = z[k]
    case["atoms"] = dict(tag=z["init_tag"], type=z["init_type"], x=z["init_x"], v=z["init_v"],
                         omega=z["init_omega"], radius=z["init_radius"], rmass=z["init_rmass"])
    if "bond_settings" in meta:
        case["bond"] = dict(tables=z["bond_tables"], settings=meta["bond_settings"])
    snaps = {}
    for st in meta["snaps"]:
        pre = "s%d_" % st
        snaps[st] = {k[len(pre):]: z[k] for k in z.files if k.startswith(pre)}
    return case, snaps


DIVERGED_RTOL = 1e-7    # forces after >10 steps of independently rounded trajectories


def newton_sign(dnum):
    """Sign of each history value in the partner's copy (newtonflag of
    add_history_value): shear[3] of tangential history flips; of the 28
    values of cohesion bond/nonlinear that precede it, ft[3], thetan[3] and
    thetat[3] (indices 5..13) flip, the rest keep their sign."""
    if dnum == 3:
        return -np.ones(3)
    sgn = np.ones(dnum)
    sgn[5:14] = -1.0
    sgn[28:31] = -1.0
    return sgn


def restart_from_snapshot(case, snap):
    """The reference's state at one snapshot as restart data.

    Returns (case_k, tag_owner, tag_partner, hist, wall_hists): atoms at that
    step plus the per-atom partner lists FixContactHistory::pre_exchange would
    write from the snapshot's neighbour list (src/fix_contact_history.cpp:
    305-425): every flagged pair gives an owner entry and, when both atoms are
    owned (no periodic image), a partner entry with negated history.
    """
    ck = dict(case)
    ck["atoms"] = dict(tag=snap["tag"], type=snap["type"], x=snap["x"], v=snap["v"],
                       omega=snap["omega"], radius=snap["radius"], rmass=snap["rmass"])
    to, tp, hs = [], [], []
    for p in range(len(snap["pair_flag"])):
        if snap["pair_flag"][p] == 0:
            continue
        ti, tj, h = int(snap["pair_tag_i"][p]), int(snap["pair_tag_j"][p]), snap["pair_hist"][p]
        to.append(ti); tp.append(tj); hs.append(h)
        if not np.any(snap["pair_shift"][p]):
            to.append(tj); tp.append(ti); hs.append(newton_sign(len(h)) * h)
    walls = [snap[k] for k in sorted(k for k in snap if k.startswith("wall") and k.endswith("_hist"))]
    dnum = snap["pair_hist"].shape[1]
    return ck, np.array(to, np.int32), np.array(tp, np.int32), np.array(hs).reshape(-1, dnum), walls


def canonical_pairs(tag_i, tag_j, shift, flag, hist):
    """dict key -> (flag, hist) with owned-owned pairs as (min, max) tags."""
    out = {}
    for p in range(len(tag_i)):
        ti, tj = int(tag_i[p]), int(tag_j[p])
        sh = tuple(int(t) for t in shift[p])
        h = np.asarray(hist[p], dtype=np.float64)
        if sh == (0, 0, 0) and ti > tj:
            ti, tj, h = tj, ti, newton_sign(len(h)) * h
        key = (ti, tj, sh)
        assert key not in out, "duplicate pair %r" % (key,)
        out[key] = (int(flag[p]), h)
    return out


def sort_by_tag(atoms):
    o = np.argsort(atoms["tag"], kind="stable")
    return {k: (v[o] if isinstance(v, np.ndarray) and v.shape[:1] == o.shape else v)
            for k, v in atoms.items()}


def max_rel(a, b, scale=None):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    s = np.max(np.abs(b)) if scale is None else scale
    if s == 0:
        return float(np.max(np.abs(a - b)))
    return float(np.max(np.abs(a - b)) / s)


def compare_pairs(got, ref, hist_rtol=HIST_RTOL):
    """Returns (missing, extra, flag_mismatch, max_hist_rel)."""
    ks_g, ks_r = set(got), set(ref)
    missing = ks_r - ks_g
    extra = ks_g - ks_r
    common = ks_g & ks_r
    flagmis = [k for k in common if (got[k][0] != 0) != (ref[k][0] != 0)]
    if not common:
        return missing, extra, flagmis, 0.0
    # each history value (column) relative to its own largest magnitude
    ks = sorted(common)
    G = np.array([got[k][1] for k in ks])
    R = np.array([ref[k][1] for k in ks])
    scale = np.max(np.abs(R), axis=0)
    d = np.max(np.abs(G - R), axis=0)
    rel = np.where(scale > 0, d / np.where(scale > 0, scale, 1.0), d)
    return missing, extra, flagmis, float(np.max(rel))
