"""Generate the golden fixtures in this folder from the reference itself.

Runs the LIGGGHTS-INL binary that oracle/ref/Makefile builds from the
reference sources (oracle/_ref/lmp_ref) on seeded synthetic inputs, with the
snapshot fix of oracle/ref registered, and stores tag-sorted per-atom state,
the granular half neighbour list (pair set, contact flags, shear history) and
the primitive-wall histories at selected steps as compressed .npz files.

This runs only where the reference sources are present (not on the GPU
machine); the .npz files it writes are committed and travel instead.

    python tests/golden/make_golden.py            # all cases
    python tests/golden/make_golden.py dense_hertz
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "liggghts-inl_gb300", "python"))
from gb300dem import workloads  # noqa: E402,F401
sys.path.insert(0, ROOT)
from oracle.lmp_input import DUMP_COLUMNS, fmt, write_inputs  # noqa: E402,F401

LMP = os.path.join(ROOT, "oracle", "_ref", "lmp_ref")


def cases():
    c = {}
    c["dense_hertz"] = (workloads.lattice_case(
        seed=11, nx=8, ny=8, nz=5, spacing=1.96e-3, radius=(1e-3, 1e-3), z0=0.99e-3,
        jitter=2e-5, vmax=2.0, wmax=100.0), 500, [0, 1, 2, 10, 50, 100, 200, 300, 500])
    c["poly_cdt"] = (workloads.lattice_case(
        seed=23, nx=7, ny=7, nz=5, spacing=2.1e-3, radius=(0.8e-3, 1.2e-3), z0=1.0e-3,
        jitter=3e-5, vmax=2.0, wmax=200.0, ntypes=2, E=(5e6, 1e7), nu=(0.45, 0.3),
        rest=((0.9, 0.7), (0.7, 0.5)), frict=((0.5, 0.4), (0.4, 0.6)),
        rollfrict=((0.3, 0.2), (0.2, 0.1)), rolling_model=1, density=1500.0),
        400, [0, 1, 2, 10, 50, 100, 200, 400])
    c["hooke"] = (workloads.lattice_case(
        seed=5, nx=6, ny=6, nz=4, spacing=1.97e-3, radius=(1e-3, 1e-3), z0=0.995e-3,
        jitter=2e-5, vmax=1.5, wmax=80.0, normal_model=1, charVel=0.5),
        300, [0, 1, 10, 100, 300])
    # conical hopper wall (triangle mesh), outlet open: atoms leave the box
    c["hopper_mesh"] = (workloads.hopper_case(
        seed=31, r_out=3e-3, r_top=14e-3, half_angle_deg=30.0, n_az=24, n_ax=5,
        spacing=2.05e-3, radius=(0.9e-3, 1.0e-3), jitter=3e-5, vmax=1.5, wmax=100.0,
        fill_height=12e-3, clearance=-0.6e-3), 600, [0, 1, 2, 10, 50, 100, 200, 400, 600])
    c["hopper_mesh_cdt"] = (workloads.hopper_case(
        seed=37, r_out=3e-3, r_top=14e-3, half_angle_deg=30.0, n_az=16, n_ax=4,
        spacing=2.05e-3, radius=(0.9e-3, 1.0e-3), jitter=3e-5, vmax=1.5, wmax=100.0,
        fill_height=12e-3, rollfrict=((0.3,),), rolling_model=1, density=1500.0, E=(1e7,),
        nu=(0.3,), rest=((0.5,),), frict=((0.6,),), clearance=-0.6e-3),
        400, [0, 1, 10, 100, 200, 400])
    # bonded fibres pressed by a moving two-triangle plate (fix move/mesh
    # linear) in a box of primitive walls; the plate's travel triggers rebuilds
    r = 0.5e-3
    bp = workloads.bond_params(
        2, [1], tsCreate=1.0, radiusMultiplier=0.5, K_fn1=200.0, Ku_fn1=400.0, Kc_fn1=100.0,
        K_fn2=1e12, Ku_fn2=2e12, Kc_fn2=5e11, K_ft=5e11, K_tn=5e11, Ku_tn=1e12, Kc_tn=2.5e11,
        K_tt=5e11, Ku_tt=1e12, Kc_tt=2.5e11, damp_fn=0.05, damp_ft=0.05, damp_tn=0.05,
        damp_tt=0.05, maxDistance=2 * r * 1.0035, createDistance=2 * r * 1.002)
    c["fibre_press"] = (workloads.press_case(
        47, nfib=60, nper=4, radius=r, box=(9e-3, 9e-3, 7e-3), plate_gap=0.1e-3,
        plate_vel=(0.0, 0.0, -6.0), gap=1.01, vmax=1.0, wmax=2000.0, bond=bp, skin=1e-4,
        max_fail=5000), 600, [0, 1, 2, 10, 50, 100, 200, 300, 400, 500, 600])
    # a lattice stirred by a rotating paddle mesh (fix move/mesh rotate)
    c["mixer_rotate"] = (workloads.mixer_case(
        53, nx=8, ny=8, nz=3, spacing=2.2e-3, radius=(0.95e-3, 1.0e-3), blade_half_len=6e-3,
        blade_height=7e-3, period=0.02, z0=1.0e-3, jitter=2e-5, vmax=0.5, wmax=50.0),
        600, [0, 1, 2, 10, 50, 100, 200, 300, 400, 500, 600])
    # a cylindrical silo (primitive zcylinder, contacts from inside) on a floor
    # plane with a horizontal bar through the bed (primitive xcylinder,
    # contacts from outside), CDT rolling on pairs and walls
    c["silo_cyl"] = (workloads.silo_case(
        81, rolling_model=1, rollfrict=((0.3,),), E=(1e7,), nu=(0.3,), rest=((0.6,),), frict=((0.5,),),
        density=2000.0), 500, [0, 1, 2, 10, 50, 100, 200, 300, 500])
    # fibres of bonded spheres (cohesion bond/nonlinear), floor of wall type 2
    for name, seed, stress in (("fibre_bond", 41, 0), ("fibre_bond_stress", 43, 1)):
        r = 0.5e-3
        bp = workloads.bond_params(
            2, [1], tsCreate=1.0, radiusMultiplier=0.5, K_fn1=200.0, Ku_fn1=400.0, Kc_fn1=100.0,
            K_fn2=1e12, Ku_fn2=2e12, Kc_fn2=5e11, K_ft=5e11, K_tn=5e11, Ku_tn=1e12, Kc_tn=2.5e11,
            K_tt=5e11, Ku_tt=1e12, Kc_tt=2.5e11, damp_fn=0.05, damp_ft=0.05, damp_tn=0.05,
            damp_tt=0.05, maxDistance=2 * r * 1.0035, maxSigma=6e6, maxTau=6e6, ratioTC=0.5,
            createDistance=2 * r * 1.002, stressBreak=stress, dampingBondSmooth=stress,
            ratioTCBond=stress)
        c[name] = (workloads.fibre_case(seed, nfib=60, nper=5, radius=r, box=(8e-3, 8e-3, 10e-3),
                                        gap=1.01, vmax=3.0, wmax=4000.0, bond=bp),
                   300, [0, 1, 2, 3, 10, 50, 100, 200, 300])
    return c


def read_snapshot(path):
    b = open(path, "rb").read()
    assert b[:8] == b"DEMSNAP1"
    off = 8
    def take(dt, cnt):
        nonlocal off
        a = np.frombuffer(b, dtype=dt, count=cnt, offset=off)
        off += a.nbytes
        return a
    step = int(take(np.int64, 1)[0])
    nlocal, nghost, dnum, nwall = [int(t) for t in take(np.int32, 4)]
    boxlo, boxhi = take(np.float64, 3), take(np.float64, 3)
    per = take(np.int32, 4)[:3]
    nall = nlocal + nghost
    tag, typ = take(np.int32, nall), take(np.int32, nall)
    vec = {k: take(np.float64, 3 * nall).reshape(nall, 3) for k in ("x", "v", "omega", "f", "torque")}
    radius, rmass = take(np.float64, nall), take(np.float64, nall)
    np_ = int(take(np.int32, 1)[0])
    pi, pj, pf = take(np.int32, np_), take(np.int32, np_), take(np.int32, np_)
    ph = take(np.float64, np_ * dnum).reshape(np_, dnum)
    walls = {}
    for _ in range(nwall):
        ln = int(take(np.int32, 1)[0])
        name = b[off:off + ln].decode(); off += ln
        wd = int(take(np.int32, 1)[0])
        walls[name] = take(np.float64, nlocal * wd).reshape(nlocal, wd)
    meshes = []
    if off < len(b):
        nm = int(take(np.int32, 1)[0])
        for _ in range(nm):
            ln = int(take(np.int32, 1)[0])
            name = b[off:off + ln].decode(); off += ln
            ntri = int(take(np.int32, 1)[0])
            ids = take(np.int32, ntri)
            mnodes = take(np.float64, 9 * ntri).reshape(ntri, 3, 3)
            act = np.frombuffer(b, dtype=np.uint8, count=6 * ntri, offset=off).reshape(ntri, 6)
            off += 6 * ntri
            md = int(take(np.int32, 1)[0])
            nslot = take(np.int32, nlocal)
            npart = take(np.int32, nlocal)
            ns = int(take(np.int32, 1)[0])
            part = take(np.int32, ns)
            mh = take(np.float64, ns * md).reshape(ns, md)
            meshes.append(dict(name=name, ids=ids, nodes=mnodes, edge_active=act[:, :3].copy(),
                               corner_active=act[:, 3:].copy(), nslot=nslot, npart=npart,
                               part=part, hist=mh))
    # canonical pairs: tags plus periodic image of j
    L = boxhi - boxlo
    owner = {int(t): i for i, t in enumerate(tag[:nlocal])}
    shift = np.zeros((np_, 3), np.int32)
    for p in range(np_):
        j = pj[p]
        if j >= nlocal:
            o = owner[int(tag[j])]
            shift[p] = np.rint((vec["x"][j] - vec["x"][o]) / L).astype(np.int32)
    order = np.argsort(tag[:nlocal], kind="stable")
    snap = dict(step=step, tag=tag[:nlocal][order], type=typ[:nlocal][order],
                radius=radius[:nlocal][order], rmass=rmass[:nlocal][order],
                pair_tag_i=tag[pi], pair_tag_j=tag[pj], pair_shift=shift, pair_flag=pf,
                pair_hist=ph)
    for k in vec:
        snap[k] = vec[k][:nlocal][order]
    for k, (name, w) in enumerate(sorted(walls.items())):
        snap["wall%d_hist" % k] = w[order]
    # mesh contacts as (atom tag, triangle id, history) triples, plus the
    # per-atom slot layout (for slot-order checks) and the mesh topology
    starts = None
    for k, m in enumerate(meshes):
        starts = np.concatenate([[0], np.cumsum(m["nslot"])])
        mt, mtri, mhist, mslot = [], [], [], []
        for i in range(nlocal):
            for s_ in range(m["nslot"][i]):
                pidx = starts[i] + s_
                if m["part"][pidx] >= 0:
                    mt.append(int(tag[i])); mtri.append(int(m["part"][pidx]))
                    mhist.append(m["hist"][pidx]); mslot.append(s_)
        snap["mesh%d_contact_tag" % k] = np.array(mt, np.int32)
        snap["mesh%d_contact_tri" % k] = np.array(mtri, np.int32)
        snap["mesh%d_contact_hist" % k] = np.array(mhist, np.float64).reshape(-1, 3)
        snap["mesh%d_contact_slot" % k] = np.array(mslot, np.int32)
        snap["mesh%d_nslot" % k] = m["nslot"][order]
        snap["mesh%d_ids" % k] = m["ids"]
        snap["mesh%d_edge_active" % k] = m["edge_active"]
        snap["mesh%d_corner_active" % k] = m["corner_active"]
        snap["mesh%d_node" % k] = m["nodes"]
    return snap


def run_case(name, case, nsteps, snaps):
    with tempfile.TemporaryDirectory() as d:
        write_inputs(case, d, nsteps, snaps)
        subprocess.check_call([LMP, "-in", "in.case", "-log", "log.case", "-screen", "screen.case"], cwd=d)
        out = {}
        for st in snaps:
            sn = read_snapshot(os.path.join(d, "snap.%d.bin" % st))
            for k, v in sn.items():
                if k != "step":
                    out["s%d_%s" % (st, k)] = v
        loop = [l for l in open(os.path.join(d, "log.case")) if l.startswith("Loop time")]
    meta = {k: v for k, v in case.items()
            if k not in ("atoms", "meshes", "bond") and not isinstance(v, np.ndarray)}
    if "bond" in case:
        meta["bond_settings"] = case["bond"]["settings"]
        out["bond_tables"] = case["bond"]["tables"]
    meta.update(nsteps=nsteps, snaps=snaps, loop=loop)
    meta["meshes"] = [dict(wall_type=m["wall_type"], rolling=m.get("rolling", 0), vel=m.get("vel"),
                           rotate=m.get("rotate")) for m in case.get("meshes", [])]
    for k, m in enumerate(case.get("meshes", [])):
        out["mesh%d_nodes" % k] = m["nodes"]
    a = case["atoms"]
    # the reference's rmass (identical formula) is what the runs start from
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta),
                        init_tag=a["tag"], init_type=a["type"], init_x=a["x"], init_v=a["v"],
                        init_omega=a["omega"], init_radius=a["radius"],
                        init_rmass=out["s0_rmass"], Yeff=case["Yeff"], Geff=case["Geff"],
                        betaeff=case["betaeff"], coeffFrict=case["coeffFrict"],
                        coeffRollFrict=case["coeffRollFrict"], coeffRestLog=case["coeffRestLog"],
                        **out)
    print(name, "atoms", len(a["tag"]), "pairs@0", len(out["s0_pair_flag"]), loop)


if __name__ == "__main__":
    allc = cases()
    sel = sys.argv[1:] or list(allc)
    for nm in sel:
        run_case(nm, *allc[nm])
