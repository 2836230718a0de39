"""Discrete adjoint with static triangle-mesh walls (dem_adjoint_add_mesh).

The compressed lattice of tests/test_adjoint.py with its floor made of a
triangle mesh (a grid of squares, each split into two coplanar triangles)
instead of a primitive plane, and the ceiling a primitive plane: the bottom
layer's wall contacts run through the reference's sphere-triangle
resolution and history slots.

  * the adjoint engine's forward run matches the oracle (the reference's CPU
    path) with the same rebuild schedule within the trajectory bar;
  * its gradients of the kinetic-energy and bed-height losses with respect to
    Young's modulus, restitution, friction and the radii with the largest
    gradients match fourth-order central differences of the oracle's loss
    within ADJ_RTOL.
"""
import numpy as np
import pytest

from golden_io import TRAJ_RTOL, max_rel, sort_by_tag

ADJ_RTOL = 1e-6
NSTEPS = 100
SEG = 10


def floor_mesh(lx, ly, nx, ny, z=0.0):
    """nx x ny squares over [0, lx] x [0, ly] at height z, two triangles each,
    normals +z; nodes[2 nx ny, 3, 3]."""
    tris = []
    for i in range(nx):
        for j in range(ny):
            x0, x1 = lx * i / nx, lx * (i + 1) / nx
            y0, y1 = ly * j / ny, ly * (j + 1) / ny
            a, b, c, d = (x0, y0, z), (x1, y0, z), (x1, y1, z), (x0, y1, z)
            tris += [(a, b, c), (a, c, d)]
    return np.array(tris, dtype=np.float64)


def gapped_floor(lx, ly, period, gap, ny):
    """A flat floor of strips along y with gaps of width `gap` centred at
    x = (2k + 1/2) period: an atom above a gap touches the two strip edges
    beside it (edge contacts), the others a strip face.  Each strip is split
    along y into ny rectangles of two coplanar triangles."""
    cuts = [0.0]
    k = 0
    while (2 * k + 0.5) * period < lx:
        c = (2 * k + 0.5) * period
        cuts += [c - 0.5 * gap, c + 0.5 * gap]
        k += 1
    cuts.append(lx)
    tris = []
    for a0, a1 in zip(cuts[0::2], cuts[1::2]):
        for j in range(ny):
            y0, y1 = ly * j / ny, ly * (j + 1) / ny
            a, b, c_, d = (a0, y0, 0.0), (a1, y0, 0.0), (a1, y1, 0.0), (a0, y1, 0.0)
            tris += [(a, b, c_), (a, c_, d)]
    return np.array(tris, dtype=np.float64)


def _case(E=1e7, rest=0.6, frict=0.5, radius=None, seed=5, floor="flat", wmax=50.0):
    from gb300dem import workloads
    sp = 1.97e-3
    nz = 4
    z0 = 0.985e-3
    c = workloads.lattice_case(seed=seed, nx=6, ny=6, nz=nz, spacing=sp, radius=(0.99e-3, 1.0e-3),
                               z0=z0, jitter=2e-6, vmax=5e-3, wmax=wmax, E=(E,), nu=(0.3,),
                               rest=((rest,),), frict=((frict,),), dt=1e-6, skin=5e-4,
                               zhi=z0 + (nz - 1) * sp + 3e-3)
    top = z0 + (nz - 1) * sp + 0.985e-3
    c["planes"] = [(2, top, 1, 0)]
    lx, ly = c["boxhi"][0], c["boxhi"][1]
    if floor in ("flat", "rising"):
        nodes = floor_mesh(lx, ly, 3, 3)
    else:  # gaps under every other column of bottom atoms: edge contacts beside face contacts
        nodes = gapped_floor(lx, ly, sp, 0.05e-3, 3)
    c["meshes"] = [dict(nodes=nodes, wall_type=1)]
    if floor == "rising":  # fix move/mesh linear 0 0 0.02: the floor presses into the bed
        c["meshes"][0]["vel"] = (0.0, 0.0, 0.02)
    c["neigh"] = (SEG, 0, 0)
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
    if kind == "wall":  # z force of the floor mesh (walls: the ceiling plane, then the mesh) at the last step
        return float(_oracle(case).diagnostics()["wall_force"][1][2] ** 2)
    a = sort_by_tag(_oracle(case).atoms())
    if kind == "ke":
        m, r = a["rmass"], a["radius"]
        return float(np.sum(0.5 * m[:, None] * a["v"] ** 2) + np.sum(0.5 * (0.4 * m * r * r)[:, None] * a["omega"] ** 2))
    return float((np.mean(a["x"][:, 2]) - 2.5e-3) ** 2)


def _spec(kind):
    from gb300dem.adjoint import make_loss
    if kind == "wall":
        return make_loss(w_wallforce=1.0, wallforce_target=0.0, wall_id=1, wall_axis=2)
    return make_loss(w_ke=1.0) if kind == "ke" else make_loss(w_height=1.0, height_target=2.5e-3)


def _fd4(f, h):
    return (8.0 * (f(h) - f(-h)) - (f(2 * h) - f(-2 * h))) / (12.0 * h)


def test_mesh_case_has_mesh_contacts():
    """The case exercises what it claims (oracle only): the bottom layer
    touches the mesh floor throughout the window."""
    c = _case()
    o = _oracle(c, nsteps=1)
    mc = o.mesh_contacts(0)
    assert len(mc["tag"]) >= 36, len(mc["tag"])
    o.run(NSTEPS - 1)
    assert len(o.mesh_contacts(0)["tag"]) >= 36


@pytest.mark.gpu
def test_adjoint_forward_with_mesh_matches_oracle():
    from gb300dem.adjoint import DemAdjoint
    c = _case()
    eng = DemAdjoint(c)
    eng.loss(1e7, 0.6, 0.5, nsteps=NSTEPS, segment=SEG)
    g = eng.final_state()
    o = sort_by_tag(_oracle(c).atoms())
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(g["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(g["v"], o["v"]) < TRAJ_RTOL
    assert max_rel(g["omega"], o["omega"]) < TRAJ_RTOL
    eng.close()


# relative steps where the oracle's fourth-order differences have converged
FD_REL = {"ke": dict(E=1e-4, restitution=1e-4, friction=1e-3, radius=1e-6),
          "height": dict(E=1e-4, restitution=1e-4, radius=1e-6)}


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["ke", "height"])
def test_adjoint_with_mesh_matches_oracle_fd(kind):
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu)
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec(kind))
    assert np.isclose(val, _oracle_loss(c, kind), rtol=1e-8, atol=0)
    steps = FD_REL[kind]
    for name, base in (("E", E), ("restitution", e), ("friction", mu)):
        if name not in steps:
            continue
        key = {"E": "E", "restitution": "rest", "friction": "frict"}[name]

        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu)
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), kind)

        fd = _fd4(f, steps[name] * base)
        assert abs(fd) > 0, name
        assert abs(g[name] - fd) <= ADJ_RTOL * abs(fd), (kind, name, g[name], fd)
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:4]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(radius=r), kind)

        fdi = _fd4(f, steps["radius"] * r0[i])
        assert abs(gr[i] - fdi) <= ADJ_RTOL * abs(fdi), (kind, int(i), gr[i], fdi)
    eng.close()


def test_gapped_floor_case_has_edge_contacts():
    """Oracle only: above each gap an atom touches the two strip edges; the
    contact set stays the same over the window."""
    c = _case(frict=0.9, floor="gapped")
    o = _oracle(c, nsteps=1)
    n0 = len(o.mesh_contacts(0)["tag"])
    assert n0 == 18 * 2 + 18, n0  # 18 atoms above gaps (two edges each), 18 on strip faces
    o.run(NSTEPS - 1)
    assert len(o.mesh_contacts(0)["tag"]) == n0


@pytest.mark.gpu
def test_adjoint_with_mesh_edges_matches_oracle():
    """Edge contacts (closest feature on a strip edge, d moving as I - e e^T):
    forward against the oracle, gradients against its differences.  No
    contact slides at friction 0.9, so the friction gradient is zero on both
    sides."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.9
    c = _case(E, e, mu, floor="gapped")
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec("ke"))
    st = eng.final_state()
    o = sort_by_tag(_oracle(c).atoms())
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(st["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(st["v"], o["v"]) < TRAJ_RTOL
    assert np.isclose(val, _oracle_loss(c, "ke"), rtol=1e-8, atol=0)
    assert g["friction"] == 0.0
    for name, base, key, rel in (("E", E, "E", 1e-4), ("restitution", e, "rest", 1e-4)):
        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu, floor="gapped")
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), "ke")

        fd = _fd4(f, rel * base)
        assert abs(g[name] - fd) <= ADJ_RTOL * abs(fd), (name, g[name], fd)
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:4]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(frict=mu, radius=r, floor="gapped"), "ke")

        fdi = _fd4(f, 1e-6 * r0[i])
        assert abs(gr[i] - fdi) <= ADJ_RTOL * abs(fdi), (int(i), gr[i], fdi)
    eng.close()


@pytest.mark.gpu
def test_adjoint_with_moving_mesh_matches_oracle():
    """A translating mesh (fix move/mesh linear): the floor rises at 2 cm/s
    (2 um over the window, far below the skin, so no mesh-forced rebuild),
    its velocity entering the contacts' relative velocity.  Forward against
    the oracle, gradients against its differences."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu, floor="rising")
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec("ke"))
    st = eng.final_state()
    o = sort_by_tag(_oracle(c).atoms())
    box = float(np.max(np.asarray(c["boxhi"]) - np.asarray(c["boxlo"])))
    assert max_rel(st["x"], o["x"], scale=box) < TRAJ_RTOL
    assert max_rel(st["v"], o["v"]) < TRAJ_RTOL
    assert np.isclose(val, _oracle_loss(c, "ke"), rtol=1e-8, atol=0)
    for name, base, key in (("E", E, "E"), ("restitution", e, "rest")):
        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu, floor="rising")
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), "ke")

        fd = _fd4(f, 1e-4 * base)
        assert abs(g[name] - fd) <= ADJ_RTOL * abs(fd), (name, g[name], fd)
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:4]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(radius=r, floor="rising"), "ke")

        fdi = _fd4(f, 1e-6 * r0[i])
        assert abs(gr[i] - fdi) <= ADJ_RTOL * abs(fdi), (int(i), gr[i], fdi)
    eng.close()


@pytest.mark.gpu
def test_adjoint_mesh_wallforce_matches_oracle_fd():
    """The wall-force term on a mesh wall: the squared z force of the floor
    mesh on the bed at the last step (wall_id counts the planes first, then
    the meshes).  Its value against the oracle's per-wall force, its
    gradients against the oracle's differences."""
    from gb300dem.adjoint import DemAdjoint
    E, e, mu = 1e7, 0.6, 0.5
    c = _case(E, e, mu)
    r0 = c["atoms"]["radius"].copy()
    eng = DemAdjoint(c)
    val, g = eng.gradient(E, e, mu, nsteps=NSTEPS, segment=SEG, loss=_spec("wall"))
    assert val > 0
    assert np.isclose(val, _oracle_loss(c, "wall"), rtol=1e-8, atol=0)
    for name, base, key in (("E", E, "E"), ("restitution", e, "rest")):
        def f(dv, key=key, base=base):
            kw = dict(E=E, rest=e, frict=mu)
            kw[key] = base + dv
            return _oracle_loss(_case(**kw), "wall")

        fd = _fd4(f, 1e-4 * base)
        assert abs(fd) > 0, name
        assert abs(g[name] - fd) <= ADJ_RTOL * abs(fd), (name, g[name], fd)
    gr = g["radius"]
    for i in np.argsort(-np.abs(gr))[:4]:
        def f(dv, i=i):
            r = r0.copy()
            r[i] += dv
            return _oracle_loss(_case(radius=r), "wall")

        fdi = _fd4(f, 1e-6 * r0[i])
        assert abs(gr[i] - fdi) <= ADJ_RTOL * abs(fdi), (int(i), gr[i], fdi)
    eng.close()
