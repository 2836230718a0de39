"""Long-run acceptance: packing fraction, kinetic-energy decay and wall force
of the GPU path within the seed-to-seed spread of the reference path.

Over many steps two independently rounded runs of a granular packing
decorrelate (the dynamics are chaotic), so step-by-step agreement is not the
bar there.  The bar is statistical.  For an ensemble of seeds, run by both
the oracle (the reference's CPU path) and the GPU, the GPU's mean of each
observable lies within the sampling error of the oracle's mean:

    |mean_gpu - mean_ref| <= 3 * sqrt(var_ref/n + var_gpu/n) + atol

Observables, from dem_get_diagnostics on the GPU and the oracle's atoms and
wall accumulators:
  * the packing fraction of the lower half of the bed;
  * the kinetic energy at several points of its decay;
  * the floor's normal force, which tends to the bed's weight.

The system is a loose jittered lattice of 288 polydisperse spheres settling
onto a floor, periodic in x/y, over 40,000 steps (0.2 s).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = (101, 102, 103, 104, 105, 106)
CHECKPOINTS = (2000, 10000, 20000, 40000)


def _case(seed):
    from gb300dem import workloads
    return workloads.lattice_case(seed=seed, nx=6, ny=6, nz=8, spacing=2.3e-3, radius=(0.9e-3, 1.1e-3),
                                  z0=1.2e-3, jitter=1e-4, vmax=0.3, wmax=50.0, E=(5e6,), nu=(0.45,),
                                  rest=((0.5,),), frict=((0.5,),), dt=5e-6, skin=4e-4)


def _region(case):
    lo = np.asarray(case["boxlo"], dtype=float)
    hi = np.asarray(case["boxhi"], dtype=float)
    return lo, np.array([hi[0], hi[1], lo[2] + 6e-3])


def _oracle_run(seed):
    from oracle.binding import Oracle
    case = _case(seed)
    lo, hi = _region(case)
    o = Oracle(case)
    o.setup()
    out, done = [], 0
    for cp in CHECKPOINTS:
        o.run(cp - done)
        done = cp
        a = o.atoms()
        m, r = a["rmass"], a["radius"]
        ke = 0.5 * np.sum(m * np.sum(a["v"] ** 2, axis=1))
        inside = np.all((a["x"] >= lo) & (a["x"] < hi), axis=1)
        pf = 4.0 * np.pi / 3.0 * np.sum(r[inside] ** 3) / np.prod(hi - lo)
        fz = o.diagnostics()["wall_force"][0][2]
        out.append((ke, pf, fz))
    return np.array(out)


def _gpu_run(seed):
    from gb300dem.api import DemSystem
    case = _case(seed)
    lo, hi = _region(case)
    g = DemSystem(case)
    g.setup()
    out, done = [], 0
    for cp in CHECKPOINTS:
        g.step(cp - done)
        done = cp
        d = g.diagnostics((lo, hi))
        out.append((d["ke_translational"], d["packing_fraction"], d["wall_force"][0][2]))
    g.close()
    return np.array(out)


def _within_spread(a, b, atol):
    n = len(a)
    ma, mb = a.mean(), b.mean()
    err = 3.0 * np.sqrt(a.var(ddof=1) / n + b.var(ddof=1) / n) + atol
    return abs(ma - mb) <= err, (ma, mb, err)


def test_long_run_statistics_match_reference():
    ref = np.stack([_oracle_run(s) for s in SEEDS])  # [seed, checkpoint, observable]
    gpu = np.stack([_gpu_run(s) for s in SEEDS])
    weight = None
    for k, cp in enumerate(CHECKPOINTS):
        # kinetic energy: compared in log space (it decays over decades)
        ok, info = _within_spread(np.log(gpu[:, k, 0]), np.log(ref[:, k, 0]), atol=0.05)
        assert ok, ("kinetic energy", cp, info)
        ok, info = _within_spread(gpu[:, k, 1], ref[:, k, 1], atol=2e-3)
        assert ok, ("packing fraction", cp, info)
        ok, info = _within_spread(gpu[:, k, 2], ref[:, k, 2], atol=1e-3 * np.abs(ref[:, k, 2]).mean())
        assert ok, ("floor force", cp, info)
    # the settled bed rests on the floor: its normal force approaches the weight
    case = _case(SEEDS[0])
    weight = 9.81 * np.sum(case["atoms"]["rmass"])
    assert abs(gpu[:, -1, 2].mean() - weight) < 0.05 * weight, (gpu[:, -1, 2].mean(), weight)
