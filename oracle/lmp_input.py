"""LIGGGHTS input scripts for the reference binaries of oracle/_ref (test
infrastructure: the golden-fixture generator, the suffix-style tests and the
CPU legs of bench.py use it; the GB300 library never does).

write_inputs(case, d, ...) writes a seeded synthetic case (the dicts of
gb300dem.workloads) as a LIGGGHTS data file, STL meshes and an input
script: atom_style granular, the material fixes (property/global), pair_style
gran with the case's model, gravity, fix wall/gran primitive planes and
meshes (fix mesh/surface), fix move/mesh, fix nve/sphere, and the requested
output and runs.  The commands are the reference's own (src/input.cpp,
src/read_data.cpp, src/fix_wall_gran.cpp, src/fix_mesh_surface.cpp,
src/fix_move_mesh.cpp, src/dump_custom.cpp).
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PY = os.path.join(ROOT, "liggghts-inl_gb300", "python")
if PY not in sys.path:
    sys.path.insert(0, PY)
from gb300dem import workloads  # noqa: E402


def fmt(v):
    return "%.17g" % v


DUMP_COLUMNS = ("id type x y z vx vy vz omegax omegay omegaz fx fy fz tqx tqy tqz radius")


def write_inputs(case, d, nsteps, snaps=None, dump_every=None, extra=(), run_style=False, runs=None,
                 atom_sort="0 0"):
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
    (src/update.cpp:103-106).  runs: several consecutive "run" commands
    (for instance a warm-up and a timed run) in place of "run nsteps".
    atom_sort: the "atom_modify sort" frequency and bin size: "0 0" for the
    parity runs (the atoms keep their order), "1000 0" (the reference's
    default, its fastest setting) for timing."""
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
    s = ["atom_style granular", "atom_modify map array sort %s" % atom_sort, "boundary %s" % bnd,
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
    npl = len(case["planes"])
    for k, (axis, rad, c1, c2, wtype, roll) in enumerate(case.get("cylinders", [])):
        wm = "model %s tangential history" % ("hooke" if case["normal_model"] == 1 else "hertz")
        if roll == 1:
            wm += " rolling_friction cdt"
        s.append("fix wall%d all wall/gran %s primitive type %d %scylinder %s %s %s"
                 % (npl + k, wm, wtype, "xyz"[axis], fmt(rad), fmt(c1), fmt(c2)))
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
    s.append("thermo 100")
    s += ["run %d" % r for r in (runs if runs else [nsteps])]
    open(os.path.join(d, "in.case"), "w").write("\n".join(s) + "\n")
