"""The drop-in boundary end to end: unchanged LIGGGHTS input scripts run
through the reference's own suffix lookup into the GB300 library.

oracle/ref/Makefile builds lmp_gb300: the unmodified reference sources
with the styles of liggghts-inl_gb300/styles registered and libdemgpu.so
linked.  Each case writes ONE input script (data file, material fixes,
pair_style gran, walls, meshes, movers, insertion, nve/sphere, a %.17g
"dump custom" every 10 steps, "run_style verlet", "run 100") and runs it
twice with the same binary:

  lmp_gb300 -in in.case             the reference's CPU path;
  lmp_gb300 -sf gb300 -in in.case   Force::new_pair, Modify::add_fix and
                                    Update::create_integrate pick
                                    gran/gb300, wall/gran/gb300,
                                    nve/sphere/gb300, gravity/gb300,
                                    move/mesh/gb300 and verlet/gb300
                                    (src/lammps.cpp:242-250,
                                    src/force.cpp:226-246,
                                    src/modify.cpp:833-848,
                                    src/update.cpp:342-377).

The dumps are compared with the parity bars of the C ABI tests: the same
atoms at every dump; forces and torques within 1e-11 of the force norm at
steps 0 and 10; positions (relative to the box), velocities and angular
velocities within 1e-9 over the 100 steps; later forces within 1e-7.
"""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from golden_io import DIVERGED_RTOL, FORCE_RTOL, TRAJ_RTOL, load_golden, max_rel

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

REF_OUT = os.path.join(ROOT, "oracle", "_ref")
LMP = os.path.join(REF_OUT, "lmp_gb300")
STAGED = os.path.join(REF_OUT, "src", "lammps.cpp")

needs_binary = pytest.mark.skipif(not os.path.exists(STAGED),
                                  reason="no reference sources staged in oracle/_ref/src")

NSTEPS = 100
EVERY = 10


def insertion_case():
    """A settled-lattice floor in a periodic box, with fix insert/pack
    filling a slab 20 mm up every 30 steps (particles_in_region 30, moving
    down at 5 m/s, so every insertion finds the slab empty again)."""
    from gb300dem import workloads
    c = workloads.lattice_case(seed=61, nx=6, ny=6, nz=2, spacing=2.1e-3, radius=(1e-3, 1e-3),
                               z0=1.0e-3, jitter=2e-5, vmax=0.5, wmax=50.0, zhi=30e-3, dt=1e-5)
    L = c["boxhi"][0]
    extra = [
        "region slab block %r %r %r %r 0.020 0.0222 units box" % (0.0, L, 0.0, c["boxhi"][1]),
        "fix pts1 all particletemplate/sphere 15485863 atom_type 1 density constant 2500 "
        "radius constant 0.001",
        "fix pdd1 all particledistribution/discrete 15485867 1 pts1 1.0",
        "fix ins all insert/pack seed 32452843 distributiontemplate pdd1 maxattempt 200 "
        "insert_every 30 overlapcheck yes all_in yes vel constant 0.0 0.0 -5.0 "
        "region slab particles_in_region 30 ntry_mc 10000",
    ]
    return c, extra


def _case(name):
    if name == "insert_pack":
        return insertion_case()
    case, _ = load_golden(name)
    return case, ()


def _read_dump(path):
    with open(path) as f:
        lines = f.readlines()
    n = int(lines[3])
    if n == 0:
        return np.zeros((0, 18))
    return np.loadtxt(lines[9:9 + n], ndmin=2)


def _run(case, extra, d, suffix):
    os.makedirs(d)
    make_golden.write_inputs(case, d, NSTEPS, dump_every=EVERY, extra=extra, run_style=True)
    # screen output to a file: parts of the reference (the STL reader) write
    # to it unconditionally, so "-screen none" is not an option
    cmd = [LMP] + (["-sf", "gb300"] if suffix else []) + ["-in", "in.case", "-log", "log.case",
                                                          "-screen", "screen.case"]
    r = subprocess.run(cmd, cwd=d, capture_output=True, text=True, timeout=600)
    log = open(os.path.join(d, "log.case")).read() if os.path.exists(os.path.join(d, "log.case")) else ""
    assert r.returncode == 0, (cmd, r.stdout[-2000:], r.stderr[-2000:], log[-3000:])
    return {st: _read_dump(os.path.join(d, "dump.%d.txt" % st)) for st in range(0, NSTEPS + 1, EVERY)}, log


CASES = ["dense_hertz", "poly_cdt", "hooke", "hopper_mesh_cdt", "fibre_bond", "fibre_press",
         "mixer_rotate", "silo_cyl", "insert_pack"]


@needs_binary
@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_unchanged_script_runs_through_suffix_styles(name, tmp_path):
    assert os.path.exists(LMP), "oracle/_ref/lmp_gb300 was not built (build())"
    case, extra = _case(name)
    plain, _ = _run(case, extra, str(tmp_path / "plain"), False)
    dev, log = _run(case, extra, str(tmp_path / "gb300"), True)
    # the suffixed run really ran the device integrator
    assert "resident on the GPU" in log, log[-2000:]
    box = float(np.max(np.asarray(case["boxhi"]) - np.asarray(case["boxlo"])))
    for st in sorted(plain):
        a, b = dev[st], plain[st]
        assert a.shape == b.shape, (name, st, a.shape, b.shape)
        if len(b) == 0:
            continue
        assert np.array_equal(a[:, 0], b[:, 0]) and np.array_equal(a[:, 1], b[:, 1]), (name, st)
        assert np.array_equal(a[:, 17], b[:, 17]), (name, st)           # radius
        ftol = FORCE_RTOL if st <= 10 else DIVERGED_RTOL
        assert max_rel(a[:, 11:14], b[:, 11:14]) < ftol, (name, st, max_rel(a[:, 11:14], b[:, 11:14]))
        assert max_rel(a[:, 14:17], b[:, 14:17]) < ftol, (name, st, max_rel(a[:, 14:17], b[:, 14:17]))
        assert max_rel(a[:, 2:5], b[:, 2:5], scale=box) < TRAJ_RTOL, (name, st)
        assert max_rel(a[:, 5:8], b[:, 5:8]) < TRAJ_RTOL, (name, st, max_rel(a[:, 5:8], b[:, 5:8]))
        assert max_rel(a[:, 8:11], b[:, 8:11]) < TRAJ_RTOL, (name, st)
    if name == "insert_pack":
        assert len(plain[NSTEPS]) > len(plain[0]) + 30, "insertion did not add atoms"
    if name == "hopper_mesh_cdt":
        assert len(plain[NSTEPS]) <= len(plain[0])


@needs_binary
def test_suffix_run_without_device_is_an_error_not_a_fallback(tmp_path):
    """Without a usable GPU the suffixed run stops with the library's
    no-device status: the styles never fall back to the host path."""
    if not os.path.exists(LMP):
        pytest.skip("lmp_gb300 not built")
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    case, _ = load_golden("dense_hertz")
    d = str(tmp_path / "c")
    os.makedirs(d)
    make_golden.write_inputs(case, d, 10, dump_every=EVERY, run_style=True)
    r = subprocess.run([LMP, "-sf", "gb300", "-in", "in.case", "-screen", "screen.case", "-log", "log.case"],
                       cwd=d, capture_output=True, text=True, timeout=120)
    log = open(os.path.join(d, "log.case")).read()
    assert r.returncode != 0
    assert "verlet/gb300: dem_create failed" in log, log[-2000:]
    assert not os.path.exists(os.path.join(d, "dump.10.txt"))
