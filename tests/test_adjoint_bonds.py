"""Discrete adjoint with cohesion bond/nonlinear (dem_adjoint_set_bonds).

A jittered lattice compressed between a floor and a ceiling plane, periodic
in x/y, with random velocities and spins; every nearest-neighbour pair bonds
at the first step (tsCreate 1, createDistance between the nearest and the
diagonal neighbour distance) while it also touches, so each bonded pair runs
the bond's normal law, shear force and twisting and bending torques together
with the tangential contact law whose friction cap the normal contact force
sets.

  * the adjoint engine's forward run matches the oracle (the reference's CPU
    path) with the same rebuild schedule within the trajectory bar;
  * its gradients of the kinetic-energy and bed-height losses with respect to
    Young's modulus, restitution, friction and per-particle radii match
    central finite differences of the oracle's loss within ADJ_RTOL.

Finite differences resolve a derivative only where the map is smooth across
the difference stencil.  The bond law's switch points (hysteresis branches,
the square-root compression law at zero displacement, the damping signs) are
crossed somewhere in 275 bonds x 100 steps for any useful stencil, and a
stencil across a kink measures a mix of both slopes.  The 1e-6 comparison
therefore runs the bond law with linear branches (loading = unloading
stiffness, tension only, no damping): every force is then smooth in the
state except at stick/slip transitions.  The branches themselves are checked
per pair against finite differences on the CPU (tests/test_adjoint_vjp.py);
the full law runs end to end here against the oracle's differences at the
accuracy those differences reach (FULL_RTOL).
"""
import numpy as np
import pytest

from golden_io import TRAJ_RTOL, max_rel, sort_by_tag

ADJ_RTOL = 1e-6
NSTEPS = 100
SEG = 10


def _case(E=1e7, rest=0.6, frict=0.5, radius=None, seed=9, law="linear"):
    from gb300dem import workloads
    sp = 1.97e-3
    nz = 4
    z0 = 0.985e-3
    c = workloads.lattice_case(seed=seed, nx=5, ny=5, nz=nz, spacing=sp, radius=(0.99e-3, 1.0e-3),
                               z0=z0, jitter=2e-6, vmax=5e-3, wmax=50.0, E=(E,), nu=(0.3,),
                               rest=((rest,),), frict=((frict,),), dt=1e-6, skin=5e-4,
                               zhi=z0 + (nz - 1) * sp + 3e-3)
    top = z0 + (nz - 1) * sp + 0.985e-3
    c["planes"] = [(2, 0.0, 1, 0), (2, top, 1, 0)]
    c["neigh"] = (SEG, 0, 0)
    common = dict(tsCreate=1.0, radiusMultiplier=1.0, maxDistance=2.2e-3, maxSigma=1e12, maxTau=1e12,
                  ratioTC=1.0, createDistance=2.1e-3)
    if law == "linear":
        c["bond"] = workloads.bond_params(
            1, (1,), K_fn1=20.0, Ku_fn1=20.0, Kc_fn1=40.0, K_fn2=5e9, Ku_fn2=5e9, Kc_fn2=1e10, K_ft=6e9,
            K_tn=1e9, Ku_tn=1e9, Kc_tn=2e9, K_tt=1e9, Ku_tt=1e9, Kc_tt=2e9, dampingBond=0,
            compressionStress=0, **common)
    else:  # hysteresis in every law, square-root compression, smooth force damping
        c["bond"] = workloads.bond_params(
            1, (1,), K_fn1=20.0, Ku_fn1=60.0, Kc_fn1=40.0, K_fn2=5e9, Ku_fn2=1.5e10, Kc_fn2=1e10, K_ft=6e9,
            K_tn=1e9, Ku_tn=3e9, Kc_tn=2e9, K_tt=1e9, Ku_tt=3e9, Kc_tt=2e9, damp_fn=0.2, damp_ft=0.1,
            dampingBondSmooth=1, **common)
    c["cohesion_model"] = 1
    if radius is not None:
        c["atoms"]["radius"] = np.asarray(radius, dtype=np.float64).copy()
        c["atoms"]["rmass"] = workloads.sphere_mass(c["atoms"]["radius"], c["material"]["density"])
    return c


def _oracle(case, nsteps=NSTEPS):
    from oracle.binding import Oracle
    o = Oracle(case)
    o.setup()
    o.run(nsteps)
    return o


def _oracle_loss(case, kind):
    a = sort_by_tag(_oracle(case).atoms())
    if kind == "ke":
        m, r = a["rmass"], a["radius"]
        return float(np.sum(0.5 * m[:, None] * a["v"] ** 2) + np.sum(0.5 * (0.4 * m * r * r)[:, None] * a["omega"] ** 2))
    return float((np.mean(a["x"][:, 2]) - 2.5e-3) ** 2)


def _spec(kind):
    from gb300dem.adjoint import make_loss
    return make_loss(w_ke=1.0) if kind == "ke" else make_loss(w_height=1.0, height_target=2.5e-3)


@pytest.mark.parametrize("law", ["linear", "full"])
def test_bonded_case_bonds_every_neighbour(law):
    """The case exercises what it claims (oracle only): after the first step
    every nearest neighbour pair holds a bond and touches, and no bond breaks
    within the window."""
    c = _case(law=law)
    o = _oracle(c, nsteps=1)
    p = o.pairs()
    bonded = (p["flag"] & 2) != 0
    # 5 x 5 columns periodic in x/y, 4 layers: the +x and +y neighbour of
    # every atom and the one above; a pair across a periodic boundary is held
    # by both atoms (2 x 20 such pairs)
    expected = 100 * 2 + 25 * 3 + 40
    assert int(bonded.sum()) == expected, (int(bonded.sum()), expected)
    assert np.all(p["flag"][bonded] == 7), "bonded pairs also touch (normal, tangential and cohesion bits)"
    o.run(NSTEPS - 1)
    assert int(((o.pairs()["flag"] & 2) != 0).sum()) == expected, "no bond breaks within the window"


@pytest.mark.gpu
@pytest.mark.parametrize("law", ["linear", "full"])
def test_adjoint_forward_with_bonds_matches_oracle(law):
    from gb300dem.adjoint import DemAdjoint
    c = _case(law=law)
    eng = DemAdjoint(c)
    eng.loss(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG)
    g = eng.final_state()
    o = sort_by_tag(_oracle(c).atoms())
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(g["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(g["v"], o["v"]) < TRAJ_RTOL
    assert max_rel(g["omega"], o["omega"]) < TRAJ_RTOL
    eng.close()


def _fd4(f, h):
    """fourth-order central difference: error O(h^4) instead of O(h^2), so
    steps large enough to stay clear of the rounding of the loss"""
    return (8.0 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12.0 * h)


# relative steps where the differences of the oracle's loss have converged
# (successive steps agree to 1e-7 or better); the height term's friction
# derivative is below what differences of the mean height resolve
FD_REL = {"ke": dict(E=1e-4, restitution=1e-4, friction=1e-3, radius=1e-6),
          "height": dict(E=3e-5, restitution=1e-4, radius=1e-6)}
# the full law: its kinks limit the differences to ~1e-4 (successive steps
# scatter by that much); no contact slides in this case, so friction has no
# gradient there
FD_FULL = dict(E=1e-6, restitution=3e-6, radius=3e-7)
FULL_RTOL = 1e-3


def _check(kind, law, rtol, nrad, steps):
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu, law=law)
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec(kind))
    assert np.isclose(val, _oracle_loss(c, kind), rtol=1e-8, atol=0)
    t = eng.times()
    print("bonded adjoint (%s, %s): forward %.2f ms, backward %.2f ms" % (law, kind, t["forward_ms"],
                                                                          t["backward_ms"]))
    for name, base in (("E", E), ("restitution", e), ("friction", mu)):
        if name not in steps:
            continue
        key = {"E": "E", "restitution": "rest", "friction": "frict"}[name]

        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu, law=law)
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), kind)

        fd = _fd4(f, steps[name] * base)
        assert abs(fd) > 0, name
        assert abs(g[name] - fd) <= rtol * abs(fd), (kind, law, name, g[name], fd)
    # radii: the atoms with the largest gradients (those against the planes),
    # whose differences are not swamped by the others' kinks
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:nrad]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(radius=r, law=law), kind)

        fdi = _fd4(f, steps["radius"] * r0[i])
        assert abs(gr[i] - fdi) <= rtol * abs(fdi), (kind, law, int(i), gr[i], fdi)
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ke", "height"])
def test_adjoint_with_bonds_matches_oracle_fd(kind):
    _check(kind, "linear", ADJ_RTOL, 4, FD_REL[kind])


@pytest.mark.gpu
def test_adjoint_with_full_bond_law_matches_oracle_fd():
    _check("ke", "full", FULL_RTOL, 2, FD_FULL)
