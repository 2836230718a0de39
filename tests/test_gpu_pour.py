"""The plain FP64 pour that the reference's CPU build runs as it is:
10,000 monodisperse spheres (r 1 mm, density 2500 kg/m^3, E 5e6 Pa,
Poisson 0.45, restitution 0.9, friction 0.5), Hertz + tangential history,
gravity -9.81 z, a 0.1 x 0.1 x 0.2 m box periodic in x/y with a floor plane
(fix wall/gran primitive zplane 0), a 2.4 mm cubic lattice with uniform
+-0.1 mm jitter from a seed, zero velocities, dt 1e-6 s, skin 0.5 mm,
20,000 steps, run through the C ABI against the oracle.

The pour is not chaotic over its 20,000 steps: two oracle runs whose inputs
differ by one ulp in one coordinate stay within 7e-17 of the box in
position and 4e-14 of the largest speed in velocity, with the same 8
rebuilds.  So the whole run is held to the per-step bars: positions and
velocities within 1e-9, the same pair sets and flags, the same rebuild
steps, forces within 1e-11 over the first 10 steps (both sides from the same
state) and within 1e-7 afterwards.
"""
import numpy as np
import pytest

from golden_io import (DIVERGED_RTOL, FORCE_RTOL, HIST_RTOL, TRAJ_RTOL, canonical_pairs, compare_pairs,
                       max_rel, sort_by_tag)

pytestmark = pytest.mark.gpu


def _pour_case(seed=7, n=10000):
    from gb300dem import workloads
    sp = 2.4e-3
    nx = ny = int(0.1 / sp)
    c = workloads.lattice_case(seed=seed, nx=nx, ny=ny, nz=6, spacing=sp, radius=(1e-3, 1e-3), density=2500.0,
                               z0=1.2e-3, jitter=1e-4, E=(5e6,), nu=(0.45,), rest=((0.9,),), frict=((0.5,),),
                               periodic=(1, 1, 0), zhi=0.2, dt=1e-6, skin=5e-4, plane_z=0.0,
                               pad=(0.1 - nx * sp, 0.1 - ny * sp))
    a = c["atoms"]
    keep = np.arange(len(a["tag"])) < n
    c["atoms"] = {k: v[keep] for k, v in a.items()}
    return c


def _pairs(p):
    return canonical_pairs(p["tag_i"], p["tag_j"], p["shift"], p["flag"], p["hist"])


def test_gpu_pour_10k_matches_oracle():
    from gb300dem.api import DemSystem
    from oracle.binding import Oracle
    case = _pour_case()
    assert len(case["atoms"]["tag"]) == 10000
    assert tuple(case["boxhi"]) == pytest.approx((0.1, 0.1, 0.2))
    g = DemSystem(case)
    o = Oracle(case)
    g.setup()
    o.setup()
    done = 0
    for chunk in (1, 9, 90, 900, 4000, 5000, 10000):
        g.step(chunk)
        o.run(chunk)
        done += chunk
        a, b = sort_by_tag(g.atoms()), sort_by_tag(o.atoms())
        ftol = FORCE_RTOL if done <= 10 else DIVERGED_RTOL
        assert max_rel(a["f"], b["f"]) < ftol, (done, max_rel(a["f"], b["f"]))
        assert max_rel(a["torque"], b["torque"]) < ftol, (done, max_rel(a["torque"], b["torque"]))
        assert max_rel(a["x"], b["x"], scale=0.2) < TRAJ_RTOL, done
        assert max_rel(a["v"], b["v"]) < TRAJ_RTOL, done
        missing, extra, flagmis, hm = compare_pairs(_pairs(g.pairs()), _pairs(o.pairs()))
        assert not missing and not extra and not flagmis, done
        assert hm < (HIST_RTOL if done <= 10 else 1e-6), (done, hm)
        assert g.nrebuilds == o.nrebuilds, done
    assert done == 20000
    ke_g = 0.5 * np.sum(a["rmass"] * np.sum(a["v"] ** 2, axis=1))
    ke_o = 0.5 * np.sum(b["rmass"] * np.sum(b["v"] ** 2, axis=1))
    assert ke_g == pytest.approx(ke_o, rel=1e-9)
    g.close()
