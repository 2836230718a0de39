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
from gb300dem import workloads  # noqa: E402

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


def fmt(v):
    return "%.17g" % v


DUMP_COLUMNS = ("id type x y z vx vy vz omegax omegay omegaz fx fy fz tqx tqy tqz radius")


def write_inputs(case, d, nsteps, snaps=None, dump_every=None, extra=(), run_style=False):
    """Writes data.case and in.case (plus mesh STL files) into d.

    snaps: steps at which the snapshot fix of the reference build writes its
    binary state (golden generation).  dump_every: instead or as well, a
    "dump custom" of every atom's id, type, x, v, omega, f, torque and
    radius in %.17g every that many steps, sorted by id (dump.<step>.txt).
    extra: further input lines placed after the integrator fix (insertion
    fixes, regions).  run_style: adds "run_style verlet", which selects the
    reference's default integrator explicitly; under "-sf gb300" that command
    selects verlet/gb300 (Update::create_integrate, src/update.cpp:342-377),
    while the integrator LAMMPS creates at start-up is never suffixed
    (src/update.cpp:103-106)."""
    a = case["atoms"]
    n = len(a["tag"])
    mat = case["material"]
    nt = case["ntypes"]
    lines = ["LIGGGHTS data file (seeded synthetic)", "", "%d atoms" % n, "%d atom types" % nt, ""]
    for k, ax in enumerate("xyz"):
        lines.append("%s %s %slo %shi" % (fmt(case["boxlo"][k]), fmt(case["boxhi"][k]), ax, ax))
    lines += ["", "Atoms", ""]
    for i in range(n):
        lines.append("%d %d %s %s %s %s %s" % (a["tag"][i], a["type"][i], fmt(2 * a["radius"][i]),
                                               fmt(mat["density"]), fmt(a["x"][i, 0]),
                                               fmt(a["x"][i, 1]), fmt(a["x"][i, 2])))
    lines += ["", "Velocities", ""]
    for i in range(n):
        lines.append("%d %s" % (a["tag"][i], " ".join(fmt(t) for t in
                                                       list(a["v"][i]) + list(a["omega"][i]))))
    open(os.path.join(d, "data.case"), "w").write("\n".join(lines) + "\n")

    bnd = " ".join("p" if p else "f" for p in case["periodic"])
    model = "model %s tangential history" % ("hooke" if case["normal_model"] == 1 else "hertz")
    if case["rolling_model"] == 1:
        model += " rolling_friction cdt"
    bond = case.get("bond") if case.get("cohesion_model", 0) == 1 else None
    if bond is not None:
        model += " cohesion bond/nonlinear"
        for f in workloads.BOND_FLAGS:
            if bond["settings"][f] != workloads.BOND_DEFAULTS[f]:
                model += " %s %s" % (workloads.BOND_KEYWORDS[f], "on" if bond["settings"][f] else "off")
    tpl = lambda m: " ".join(fmt(m[i][j]) for i in range(nt) for j in range(nt))  # noqa: E731
    s = ["atom_style granular", "atom_modify map array sort 0 0", "boundary %s" % bnd,
         "newton off", "communicate single vel yes", "units si",
         "read_data data.case", "neighbor %s bin" % fmt(case["skin"]), "neigh_modify delay 0",
         "fix m1 all property/global youngsModulus peratomtype %s" % " ".join(fmt(e) for e in mat["E"]),
         "fix m2 all property/global poissonsRatio peratomtype %s" % " ".join(fmt(e) for e in mat["nu"]),
         "fix m3 all property/global coefficientRestitution peratomtypepair %d %s" % (nt, tpl(mat["rest"])),
         "fix m4 all property/global coefficientFriction peratomtypepair %d %s" % (nt, tpl(mat["frict"]))]
    if case["rolling_model"] == 1:
        s.append("fix m5 all property/global coefficientRollingFriction peratomtypepair %d %s"
                 % (nt, tpl(mat["rollfrict"])))
    if case["normal_model"] == 1:
        s.append("fix m6 all property/global characteristicVelocity scalar %s" % fmt(case["charVel"]))
    if bond is not None:
        for k, name in enumerate(workloads.BOND_TABLES):
            s.append("fix b%d all property/global %s peratomtypepair %d %s"
                     % (k, name, nt, tpl(bond["tables"][k][1:, 1:])))
        s.append("fix bts all property/global tsCreateBondnonlinear scalar %s"
                 % fmt(bond["settings"]["tsCreate"]))
    s += ["pair_style gran %s" % model, "pair_coeff * *", "timestep %s" % fmt(case["dt"])]
    g = case["gravity"]
    s.append("fix gravi all gravity 9.81 vector 0.0 0.0 -1.0")
    assert tuple(g) == (0.0, 0.0, -9.81)
    for k, (axis, pos, wtype, roll) in enumerate(case["planes"]):
        wm = "model %s tangential history" % ("hooke" if case["normal_model"] == 1 else "hertz")
        if roll == 1:
            wm += " rolling_friction cdt"
        s.append("fix wall%d all wall/gran %s primitive type %d %splane %s"
                 % (k, wm, wtype, "xyz"[axis], fmt(pos)))
    for k, m in enumerate(case.get("meshes", [])):
        workloads.write_stl(os.path.join(d, "mesh%d.stl" % k), m["nodes"])
        s.append("fix cad%d all mesh/surface file mesh%d.stl type %d" % (k, k, m["wall_type"]))
        wm = "model %s tangential history" % ("hooke" if case["normal_model"] == 1 else "hertz")
        if m.get("rolling", 0) == 1:
            wm += " rolling_friction cdt"
        s.append("fix mwall%d all wall/gran %s mesh n_meshes 1 meshes cad%d" % (k, wm, k))
        if m.get("vel") is not None:
            s.append("fix mv%d all move/mesh mesh cad%d linear %s" % (k, k, " ".join(fmt(v) for v in m["vel"])))
        if m.get("rotate") is not None:
            ro = m["rotate"]
            s.append("fix mv%d all move/mesh mesh cad%d rotate origin %s axis %s period %s"
                     % (k, k, " ".join(fmt(v) for v in ro["origin"]), " ".join(fmt(v) for v in ro["axis"]),
                        fmt(ro["period"])))
    if not all(case["periodic"]):
        s.append("thermo_modify lost ignore")
    s.append("fix integr all nve/sphere")
    s += list(extra)
    if snaps is not None:
        s.append("fix snap all oracle/snapshot snap %s" % " ".join(str(t) for t in snaps))
    if dump_every:
        ncol = len(DUMP_COLUMNS.split())
        s += ["dump dmp all custom %d dump.*.txt %s" % (dump_every, DUMP_COLUMNS),
              'dump_modify dmp sort id format "%%d %%d%s"' % (" %.17g" * (ncol - 2))]
    if run_style:
        s.append("run_style verlet")
    s += ["thermo 100", "run %d" % nsteps]
    open(os.path.join(d, "in.case"), "w").write("\n".join(s) + "\n")


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
