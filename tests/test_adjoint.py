"""Discrete adjoint (gb300dem.adjoint, dem_adjoint_* in the C ABI).

  * the adjoint engine's forward run is the reference model: its final state
    matches the oracle run with the same rebuild schedule
    (neigh_modify every <segment> delay 0 check no) within the trajectory bar;
  * its gradients with respect to Young's modulus, restitution, friction and
    per-particle radii match central finite differences of the oracle's loss
    (kinetic-energy, height and plane wall-force terms) within ADJ_RTOL, on
    the small case and at the calibration configuration's 20,000 spheres;
  * checkpoint segment length does not change the result beyond rounding;
  * the torch.autograd.Function returns the same gradients.

The case is a jittered lattice compressed between a floor and a ceiling plane,
periodic in x/y, with random spins: every contact stays closed over the
window (no contact opens or closes), a part of them slides.
"""
import numpy as np
import pytest

from golden_io import TRAJ_RTOL, max_rel, sort_by_tag

pytestmark = pytest.mark.gpu

ADJ_RTOL = 1e-6   # gradient vs central finite difference, relative
NSTEPS = 100
SEG = 10


def _case(E=1e7, rest=0.6, frict=0.5, radius=None, seed=5, rolling=None):
    """rolling: None, or the CDT rolling-friction coefficient of pairs and walls"""
    from gb300dem import workloads
    sp = 1.97e-3
    nz = 4
    z0 = 0.985e-3
    c = workloads.lattice_case(seed=seed, nx=6, ny=6, nz=nz, spacing=sp, radius=(0.99e-3, 1.0e-3),
                               z0=z0, jitter=2e-6, vmax=5e-3, wmax=50.0, E=(E,), nu=(0.3,),
                               rest=((rest,),), frict=((frict,),), dt=1e-6, skin=5e-4,
                               zhi=z0 + (nz - 1) * sp + 3e-3,
                               rollfrict=((rolling,),) if rolling is not None else None,
                               rolling_model=1 if rolling is not None else 0)
    top = z0 + (nz - 1) * sp + 0.985e-3
    rf = 1 if rolling is not None else 0
    c["planes"] = [(2, 0.0, 1, rf), (2, top, 1, rf)]
    c["neigh"] = (SEG, 0, 0)
    if radius is not None:
        c["atoms"]["radius"] = np.asarray(radius, dtype=np.float64).copy()
        c["atoms"]["rmass"] = workloads.sphere_mass(c["atoms"]["radius"], c["material"]["density"])
    return c


def _oracle_final(case, nsteps=NSTEPS):
    from oracle.binding import Oracle
    o = Oracle(case)
    o.setup()
    o.run(nsteps)
    return sort_by_tag(o.atoms())


def _oracle_loss(case, kind):
    a = _oracle_final(case)
    if kind == "ke":
        m, r = a["rmass"], a["radius"]
        return float(np.sum(0.5 * m[:, None] * a["v"] ** 2) + np.sum(0.5 * (0.4 * m * r * r)[:, None] * a["omega"] ** 2))
    if kind == "height":
        return float((np.mean(a["x"][:, 2]) - 2.5e-3) ** 2)
    raise ValueError(kind)


def _spec(kind):
    from gb300dem.adjoint import make_loss
    if kind == "ke":
        return make_loss(w_ke=1.0)
    if kind == "height":
        return make_loss(w_height=1.0, height_target=2.5e-3)
    if kind == "wall":
        return make_loss(w_wallforce=1.0, wallforce_target=0.0, wall_id=1)
    raise ValueError(kind)


def _close(g, fd, scale):
    return abs(g - fd) <= ADJ_RTOL * max(abs(fd), scale)


def test_adjoint_forward_matches_oracle():
    from gb300dem.adjoint import DemAdjoint
    c = _case()
    eng = DemAdjoint(c)
    eng.loss(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG)
    g = eng.final_state()
    o = _oracle_final(c)
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(g["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(g["v"], o["v"]) < TRAJ_RTOL
    assert max_rel(g["omega"], o["omega"]) < TRAJ_RTOL
    eng.close()


# relative central-difference steps per loss term and parameter, chosen where
# the difference quotient has converged (rounding noise ~ eps*L/h below 1e-7
# of the derivative, truncation ~ h^2 likewise): friction only acts through
# the sliding contacts, so d(loss)/d(mu) is small against loss/mu and needs
# larger steps; the mean-height term changes by ~1e-5 of its value for a unit
# relative change of E, so its differences need larger steps to stay above
# the rounding of the mean (sum of 144 heights), and its friction derivative
# (~1e-14) is below what a difference of that sum resolves (checked through
# the other terms instead)
FD_REL = {"ke": dict(E=1e-6, restitution=1e-6, friction=1e-4, radius=1e-6),
          "height": dict(E=1e-4, restitution=1e-4, radius=1e-5)}


@pytest.mark.parametrize("kind", ["ke", "height"])
def test_adjoint_gradients_match_oracle_fd(kind):
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu)
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec(kind))
    assert np.isclose(val, _oracle_loss(c, kind), rtol=1e-8, atol=0)
    fd = {}
    for name, base in (("E", E), ("restitution", e), ("friction", mu)):
        if name not in FD_REL[kind]:
            continue
        h = FD_REL[kind][name] * base
        kw_p = dict(E=E, rest=e, frict=mu)
        kw_m = dict(E=E, rest=e, frict=mu)
        key = {"E": "E", "restitution": "rest", "friction": "frict"}[name]
        kw_p[key] = base + h
        kw_m[key] = base - h
        fd[name] = (_oracle_loss(_case(**kw_p), kind) - _oracle_loss(_case(**kw_m), kind)) / (2 * h)
    # every parameter is active in this case
    assert all(abs(fd[k]) > 0 for k in fd), fd
    for k in fd:
        scale = abs(fd[k])
        assert _close(g[k], fd[k], scale), (kind, k, g[k], fd[k])
    # radii: a sample of atoms
    gr = g["radius"]
    rscale = float(np.max(np.abs(gr)))
    for i in (0, 7, 40, 77, 143):
        h = FD_REL[kind]["radius"] * r0[i]
        rp, rm = r0.copy(), r0.copy()
        rp[i] += h
        rm[i] -= h
        fdi = (_oracle_loss(_case(radius=rp), kind) - _oracle_loss(_case(radius=rm), kind)) / (2 * h)
        assert abs(gr[i] - fdi) <= ADJ_RTOL * max(abs(fdi), 1e-3 * rscale), (kind, i, gr[i], fdi)
    eng.close()


def _oracle_wallforce_loss(case, nsteps=NSTEPS):
    """(normal force of the ceiling plane, wall 1, at the last force pass)^2"""
    from oracle.binding import Oracle
    o = Oracle(case)
    o.setup()
    o.run(nsteps)
    return float(o.diagnostics()["wall_force"][1][2] ** 2)


def test_adjoint_wallforce_gradient_matches_oracle_fd():
    """The plane wall-force term against central differences of the
    oracle's own wall force (FixWallGran's force on the atoms, summed)."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu)
    eng = DemAdjoint(c)
    spec = _spec("wall")
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=spec)
    assert val > 0
    assert np.isclose(val, _oracle_wallforce_loss(c), rtol=1e-8, atol=0)
    rel = 1e-6
    args = dict(E=E, rest=e, frict=mu)
    # the normal wall force moves by less than one ulp of the loss for any
    # friction step that keeps the difference quotient accurate (its friction
    # derivative is ~1e-10): friction is checked through the kinetic-energy term
    for k, gk in (("E", "E"), ("rest", "restitution")):
        h = rel * args[k]
        ap, am = dict(args), dict(args)
        ap[k] += h
        am[k] -= h
        fd = (_oracle_wallforce_loss(_case(**ap)) - _oracle_wallforce_loss(_case(**am))) / (2 * h)
        assert _close(g[gk], fd, abs(fd)), (k, g[gk], fd)
    r0 = c["atoms"]["radius"]
    gr = g["radius"]
    for i in (3, 100, 140):
        h = rel * r0[i]
        rp, rm = r0.copy(), r0.copy()
        rp[i] += h
        rm[i] -= h
        fd = (_oracle_wallforce_loss(_case(radius=rp)) - _oracle_wallforce_loss(_case(radius=rm))) / (2 * h)
        assert abs(gr[i] - fd) <= ADJ_RTOL * max(abs(fd), 1e-3 * np.max(np.abs(gr))), (i, gr[i], fd)
    eng.close()


def _c5_case(E=1e7, rest=0.6, frict=0.5, radius=None):
    """The calibration configuration's size: 20,000 spheres (50 x 50 x 8),
    in the compressed-lattice form of _case so that the contact set stays
    fixed over the 100-step window (a settling column's contacts open and
    close inside the window, and differences across such events do not
    converge)."""
    from gb300dem import workloads
    sp, nz, z0 = 1.97e-3, 8, 0.985e-3
    c = workloads.lattice_case(seed=5, nx=50, ny=50, nz=nz, spacing=sp, radius=(0.99e-3, 1.0e-3), z0=z0,
                               jitter=2e-6, vmax=5e-3, wmax=50.0, E=(E,), nu=(0.3,), rest=((rest,),),
                               frict=((frict,),), dt=1e-6, skin=5e-4, zhi=z0 + (nz - 1) * sp + 3e-3)
    c["planes"] = [(2, 0.0, 1, 0), (2, z0 + (nz - 1) * sp + 0.985e-3, 1, 0)]
    c["neigh"] = (SEG, 0, 0)
    if radius is not None:
        c["atoms"]["radius"] = np.asarray(radius, dtype=np.float64).copy()
        c["atoms"]["rmass"] = workloads.sphere_mass(c["atoms"]["radius"], c["material"]["density"])
    return c


def test_adjoint_c5_size_matches_oracle_fd():
    """20,000 spheres, a 100-step window with sqrt(N) checkpoints: the
    kinetic-energy gradients with respect to E, restitution, friction and
    eight sampled radii match the oracle's central differences within 1e-6
    (steps: 1e-6 relative; friction 1e-5 and radii 3e-6, where those
    differences have converged)."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _c5_case()
    assert len(c["atoms"]["tag"]) == 20000
    eng = DemAdjoint(c)
    eng.set_tape(0)  # checkpoints + replay
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec("ke"))

    def L(**kw):
        return _oracle_loss_of(_c5_case(**kw))
    assert np.isclose(val, L(), rtol=1e-8, atol=0)
    for key, gk, base, rel in (("E", "E", E, 1e-6), ("rest", "restitution", e, 1e-6),
                               ("frict", "friction", mu, 1e-5)):
        h = rel * base
        fd = (L(**{key: base + h}) - L(**{key: base - h})) / (2 * h)
        assert fd != 0 and _close(g[gk], fd, abs(fd)), (gk, g[gk], fd)
    r0 = c["atoms"]["radius"]
    gr = g["radius"]
    for i in (0, 1234, 4567, 8000, 11111, 14000, 17777, 19999):
        h = 3e-6 * r0[i]  # where the quotient of the 20,000-term loss is settled (rounding scatter ~6e-7 at 1e-6)
        rp, rm = r0.copy(), r0.copy()
        rp[i] += h
        rm[i] -= h
        fd = (L(radius=rp) - L(radius=rm)) / (2 * h)
        assert abs(gr[i] - fd) <= ADJ_RTOL * max(abs(fd), 1e-3 * np.max(np.abs(gr))), (i, gr[i], fd)
    eng.close()


def _oracle_loss_of(case):
    a = _oracle_final(case)
    m, r = a["rmass"], a["radius"]
    return float(np.sum(0.5 * m[:, None] * a["v"] ** 2) + np.sum(0.5 * (0.4 * m * r * r)[:, None] * a["omega"] ** 2))


def test_adjoint_segment_length_and_determinism():
    from gb300dem.adjoint import DemAdjoint
    c = _case()
    eng = DemAdjoint(c)
    spec = _spec("ke")
    v1, g1 = eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG, loss=spec)
    v2, g2 = eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG, loss=spec)
    assert v1 == v2 and all(np.array_equal(g1[k], g2[k]) for k in g1)  # bitwise reproducible
    # another rebuild schedule is another (equally valid) discretisation of
    # the same physics: the same gradients to within the FD bar
    v3, g3 = eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=25, loss=spec)
    assert np.isclose(v3, v1, rtol=1e-9)
    for k in ("E", "restitution", "friction"):
        assert np.isclose(g3[k], g1[k], rtol=ADJ_RTOL), k
    assert max_rel(g3["radius"], g1["radius"]) < ADJ_RTOL
    t = eng.times()
    assert t["segments"] == NSTEPS // 25 + 1 and t["max_pairs"] > 0
    eng.close()


def _fd4(f, h):
    return (8.0 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12.0 * h)


def test_adjoint_with_cdt_rolling_matches_oracle():
    """CDT rolling friction on pairs and planes (coefficient 0.002: the
    rolling torque opposes the relative spin at constant magnitude and flips
    with it, so a spin reaching zero within the window would make the map
    non-smooth; at this coefficient no spin does).  Forward against the
    oracle, gradients against its fourth-order differences."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu, mur = 1e7, 0.6, 0.5, 0.002
    c = _case(E, e, mu, rolling=mur)
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec("ke"))
    st = eng.final_state()
    o = _oracle_final(c)
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(st["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(st["v"], o["v"]) < TRAJ_RTOL
    assert max_rel(st["omega"], o["omega"]) < TRAJ_RTOL
    assert np.isclose(val, _oracle_loss(c, "ke"), rtol=1e-8, atol=0)
    for name, base, key in (("E", E, "E"), ("restitution", e, "rest"), ("friction", mu, "frict")):
        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu, rolling=mur)
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), "ke")

        fd = _fd4(f, 1e-4 * base)
        assert abs(g[name] - fd) <= ADJ_RTOL * abs(fd), (name, g[name], fd)

    def fr(dv):  # the rolling-friction coefficient
        return _oracle_loss(_case(E, e, mu, rolling=mur + dv), "ke")

    fd = _fd4(fr, 1e-3 * mur)
    assert abs(g["rolling_friction"] - fd) <= ADJ_RTOL * abs(fd), (g["rolling_friction"], fd)
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:4]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(radius=r, rolling=mur), "ke")

        fdi = _fd4(f, 1e-6 * r0[i])
        assert abs(gr[i] - fdi) <= ADJ_RTOL * abs(fdi), (int(i), gr[i], fdi)
    eng.close()


@pytest.mark.parametrize("model", ["plain", "bonded", "mesh"])
def test_adjoint_recorded_and_replayed_tapes_agree(model):
    """The backward pass on a record taken in the forward pass and on one
    replayed from the sqrt(N) checkpoints: the same gradients bit for bit."""
    from gb300dem.adjoint import DemAdjoint
    if model == "bonded":
        import test_adjoint_bonds
        c = test_adjoint_bonds._case(law="full")
    elif model == "mesh":
        import test_adjoint_mesh
        c = test_adjoint_mesh._case(frict=0.9, floor="gapped")
    else:
        c = _case()
    eng = DemAdjoint(c)
    spec = _spec("ke")
    out = {}
    for mode in (0, 1, 2):
        eng.set_tape(mode)
        out[mode] = eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG, loss=spec)
        assert eng.tape_recorded() == (mode != 0), mode  # mode 2: this record fits
    for mode in (1, 2):
        assert out[mode][0] == out[0][0]
        for k in ("E", "restitution", "friction", "radius"):
            assert np.array_equal(out[mode][1][k], out[0][1][k]), (mode, k)
    eng.set_tape(2, max_bytes=1e3)  # a budget the record does not fit: replay
    eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG, loss=spec)
    assert not eng.tape_recorded()
    eng.close()


def test_adjoint_torch_function():
    torch = pytest.importorskip("torch")
    from gb300dem.adjoint import DemAdjoint, adjoint_loss
    c = _case()
    eng = DemAdjoint(c)
    spec = _spec("ke")
    E = torch.tensor(1e7, dtype=torch.float64, requires_grad=True)
    e = torch.tensor(0.6, dtype=torch.float64, requires_grad=True)
    mu = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    r = torch.tensor(c["atoms"]["radius"], dtype=torch.float64, requires_grad=True)
    L = adjoint_loss(E, e, mu, r, eng, NSTEPS, SEG, spec)
    L.backward()
    v, g = eng.gradient(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG, loss=spec)
    assert float(L.detach()) == v
    assert float(E.grad) == g["E"] and float(e.grad) == g["restitution"] and float(mu.grad) == g["friction"]
    assert np.array_equal(r.grad.numpy(), g["radius"])
    eng.close()
