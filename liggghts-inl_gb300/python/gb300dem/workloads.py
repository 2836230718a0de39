"""Seeded synthetic DEM states and the material-table derivation.

The tables follow the reference's property registry:
  Yeff    = 1/((1-nu_i^2)/E_i + (1-nu_j^2)/E_j)        src/global_properties.cpp:449
  Geff    = 1/(2(2-nu_i)(1+nu_i)/E_i + 2(2-nu_j)(1+nu_j)/E_j)   :480
  betaeff = ln e / sqrt(ln^2 e + pi^2)                   :556
  coeffRestLog = ln e                                    :518
with the same operand order, so on the same libm the values are bit-identical
to the reference's MatrixProperty data.  Matrices are (ntypes+1)^2 with types
starting at 1 (row/column 0 unused).

A "case" is a plain dict describing one system: box, periodicity, dt, skin,
contact-model switches, material tables, primitive planes and the initial
atoms (tag, type, x, v, omega, radius, rmass).  The same dict drives the GPU
handle, the CPU oracle and the reference input scripts.
"""
import math

import numpy as np

MY_PI = 3.14159265358979323846


def derive_tables(E, nu, rest, frict, rollfrict=None):
    """E, nu: per type (length nt); rest, frict, rollfrict: nt x nt."""
    nt = len(E)
    Y = np.zeros((nt + 1, nt + 1))
    G = np.zeros((nt + 1, nt + 1))
    B = np.zeros((nt + 1, nt + 1))
    RL = np.zeros((nt + 1, nt + 1))
    MU = np.zeros((nt + 1, nt + 1))
    MUR = np.zeros((nt + 1, nt + 1))
    for i in range(1, nt + 1):
        for j in range(1, nt + 1):
            Yi, Yj, vi, vj = float(E[i - 1]), float(E[j - 1]), float(nu[i - 1]), float(nu[j - 1])
            Y[i, j] = 1. / ((1. - math.pow(vi, 2.)) / Yi + (1. - math.pow(vj, 2.)) / Yj)
            G[i, j] = 1. / (2. * (2. - vi) * (1. + vi) / Yi + 2. * (2. - vj) * (1. + vj) / Yj)
            lg = math.log(float(rest[i - 1][j - 1]))
            RL[i, j] = lg
            B[i, j] = lg / math.sqrt(math.pow(lg, 2.) + math.pow(math.pi, 2.))
            MU[i, j] = float(frict[i - 1][j - 1])
            MUR[i, j] = float(rollfrict[i - 1][j - 1]) if rollfrict is not None else 0.0
    return dict(Yeff=Y, Geff=G, betaeff=B, coeffRestLog=RL, coeffFrict=MU, coeffRollFrict=MUR)


def sphere_mass(radius, density):
    """rmass of atom_style granular, src/atom_vec_sphere.cpp:1076-1080."""
    r = np.asarray(radius, dtype=np.float64)
    return 4.0 * MY_PI / 3.0 * r * r * r * np.asarray(density, dtype=np.float64)


def cone_mesh(r_out, r_top, half_angle_deg, n_az, n_ax, z_out=0.0):
    """Triangles of a conical hopper wall (axis z, outlet at z_out).

    n_az x n_ax quads between rings of radius r(z) = r_out + (z - z_out) tan(a),
    each split into two triangles; returns nodes[ntri, 3, 3].
    """
    ta = math.tan(math.radians(half_angle_deg))
    z_top = z_out + (r_top - r_out) / ta
    zs = np.linspace(z_out, z_top, n_ax + 1)
    th = np.linspace(0.0, 2.0 * math.pi, n_az + 1)
    tri = []
    for k in range(n_ax):
        r0 = r_out + (zs[k] - z_out) * ta
        r1 = r_out + (zs[k + 1] - z_out) * ta
        for j in range(n_az):
            jn = (j + 1) % n_az  # the seam reuses the nodes of column 0 exactly
            c0, s0 = math.cos(th[j]), math.sin(th[j])
            c1, s1 = math.cos(th[jn]), math.sin(th[jn])
            a = (r0 * c0, r0 * s0, zs[k])
            b = (r0 * c1, r0 * s1, zs[k])
            c = (r1 * c1, r1 * s1, zs[k + 1])
            d = (r1 * c0, r1 * s0, zs[k + 1])
            tri.append((a, b, c))
            tri.append((a, c, d))
    return np.array(tri, dtype=np.float64), z_top


def write_stl(path, nodes):
    """ASCII STL of nodes[ntri, 3, 3] (facet normals from the node order)."""
    with open(path, "w") as f:
        f.write("solid mesh\n")
        for t in nodes:
            n = np.cross(t[1] - t[0], t[2] - t[0])
            nn = np.linalg.norm(n)
            n = n / nn if nn > 0 else n
            f.write("  facet normal %.17g %.17g %.17g\n    outer loop\n" % tuple(n))
            for p in t:
                f.write("      vertex %.17g %.17g %.17g\n" % tuple(p))
            f.write("    endloop\n  endfacet\n")
        f.write("endsolid mesh\n")


def hopper_case(seed, r_out, r_top, half_angle_deg, n_az, n_ax, spacing, radius=(1e-3, 1e-3),
                density=2500.0, fill_height=None, vmax=0.0, wmax=0.0, E=(5e6,), nu=(0.45,),
                rest=((0.9,),), frict=((0.5,),), rollfrict=None, rolling_model=0, dt=1e-6,
                skin=5e-4, gravity=(0.0, 0.0, -9.81), jitter=0.0, z_below=None, normal_model=0,
                charVel=0.0, max_atoms=None, clearance=None):
    """Conical hopper (triangle mesh, outlet open) filled with a jittered lattice.

    The box is non-periodic; atoms falling below z_below are lost at the next
    neighbour rebuild, as with `thermo_modify lost ignore` in the reference.
    """
    rng = np.random.default_rng(seed)
    nodes, z_top = cone_mesh(r_out, r_top, half_angle_deg, n_az, n_ax)
    ta = math.tan(math.radians(half_angle_deg))
    rmax = radius[1]
    if clearance is None:
        clearance = 0.25 * spacing  # negative: the outer ring overlaps the wall
    zf = z_top if fill_height is None else fill_height
    nxy = int(2 * r_top / spacing) + 2
    nz = int((zf - rmax) / spacing) + 1
    gx = -r_top + (np.arange(nxy) + 0.5) * spacing
    gz = rmax * 1.5 + np.arange(nz) * spacing
    zz, xx, yy = np.meshgrid(gz, gx, gx, indexing="ij")  # z-major, then x, then y
    R = r_out + zz * ta
    # inside the cone with one radius of clearance measured normal to the wall
    inside = (np.hypot(xx, yy) + rmax / math.cos(math.radians(half_angle_deg))) < R - clearance
    x = np.stack([xx[inside], yy[inside], zz[inside]], axis=1).astype(np.float64)
    if max_atoms is not None and len(x) > max_atoms:
        x = x[np.argsort(x[:, 2], kind="stable")[:max_atoms]]
    n = len(x)
    if jitter > 0:
        x += rng.uniform(-jitter, jitter, size=x.shape)
    r = rng.uniform(radius[0], radius[1], size=n) if radius[0] != radius[1] else np.full(n, radius[0])
    v = rng.uniform(-vmax, vmax, size=(n, 3)) if vmax > 0 else np.zeros((n, 3))
    w = rng.uniform(-wmax, wmax, size=(n, 3)) if wmax > 0 else np.zeros((n, 3))
    if z_below is None:
        z_below = -4 * rmax
    pad = 4 * rmax
    case = dict(
        boxlo=(-r_top - pad, -r_top - pad, z_below), boxhi=(r_top + pad, r_top + pad, z_top + pad),
        periodic=(0, 0, 0), dt=dt, skin=skin, cdf=1.0, neigh=(1, 0, 1), normal_model=normal_model,
        rolling_model=rolling_model, gravity=gravity, ntypes=1, charVel=charVel, planes=[],
        meshes=[dict(nodes=nodes, wall_type=1, rolling=rolling_model)],
        material=dict(E=list(E), nu=list(nu), rest=[list(q) for q in rest],
                      frict=[list(q) for q in frict],
                      rollfrict=[list(q) for q in rollfrict] if rollfrict is not None else None,
                      density=density),
        atoms=dict(tag=np.arange(1, n + 1, dtype=np.int32), type=np.ones(n, np.int32), x=x, v=v,
                   omega=w, radius=r, rmass=sphere_mass(r, density)),
    )
    case.update(derive_tables(E, nu, rest, frict, rollfrict))
    return case


def packed_bed_case(seed, nx, ny, nz, dnn=2.04e-3, radius=(0.97e-3, 1.03e-3), density=1500.0, dt=5e-6,
                    **kw):
    """Spheres on a face-centred cubic lattice (nearest-neighbour distance
    dnn, just above the mean diameter) in a box periodic in x/y above a floor:
    under gravity the polydisperse lattice collapses into a dense random bed
    with about five touching contacts per sphere.  4*nx*ny*nz spheres."""
    rng = np.random.default_rng(seed)
    a = dnn * math.sqrt(2.0)  # edge of the cubic FCC cell
    basis = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cells = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], 1).astype(np.float64)
    x = ((cells[:, None, :] + basis[None]) * a).reshape(-1, 3)
    x[:, 2] += radius[1] * 1.05
    n = len(x)
    c = lattice_case(seed, 1, 1, 1, 1.0, radius=radius, density=density, dt=dt, **kw)
    r = rng.uniform(radius[0], radius[1], n)
    c["boxhi"] = (nx * a, ny * a, float(x[:, 2].max() + 6 * radius[1]))
    c["atoms"] = dict(tag=np.arange(1, n + 1, dtype=np.int32), type=np.ones(n, np.int32), x=x,
                      v=np.zeros((n, 3)), omega=np.zeros((n, 3)), radius=r, rmass=sphere_mass(r, density))
    return c


def restart_state(sys_, case):
    """A resident system's state as the reference's restart data: atoms,
    the per-atom partner lists with their contact history (one entry per
    touching side; FixContactHistory::pre_exchange writes both sides of a
    pair of two owned atoms, the partner's with the newton sign) and the
    primitive-wall histories.  Returns (case with those atoms, owner tags,
    partner tags, histories, wall histories)."""
    a = sys_.atoms()
    ck = dict(case)
    ck["atoms"] = {k: np.array(a[k]) for k in ("tag", "type", "x", "v", "omega", "radius", "rmass")}
    p = sys_.pairs()
    on = p["flag"] != 0
    ti, tj, sh, hs = p["tag_i"][on], p["tag_j"][on], p["shift"][on], p["hist"][on]
    own = ~np.any(sh != 0, axis=1)
    # sign of each history value in the partner's copy (the newtonflag of
    # add_history_value): the shear flips; of the 28 bond values, ft,
    # thetan and thetat (5..13) flip
    if hs.shape[1] == 3:
        sgn = -np.ones(3)
    else:
        sgn = np.ones(hs.shape[1])
        sgn[5:14] = -1.0
        sgn[28:31] = -1.0
    to = np.concatenate([ti, tj[own]]).astype(np.int32)
    tp = np.concatenate([tj, ti[own]]).astype(np.int32)
    hh = np.concatenate([hs, hs[own] * sgn[None, :]])
    order = np.argsort(a["tag"], kind="stable")
    nprim = len(case.get("planes", [])) + len(case.get("cylinders", []))
    walls = [np.asarray(sys_.wall_history(w))[order] for w in range(nprim)]
    ck["atoms"] = {k: v[order] for k, v in ck["atoms"].items()}
    return ck, to, tp, hh, walls


def silo_case(seed, R=8e-3, nz=6, spacing=2.05e-3, radius=(0.9e-3, 1.0e-3), bar=(1.5e-3, 7e-3),
              vmax=0.5, wmax=80.0, **kw):
    """A jittered lattice filling a vertical cylinder (fix wall/gran
    primitive zcylinder R 0 0: contacts from inside) on a floor plane, with a
    horizontal bar through the bed (xcylinder of radius bar[0] at height
    bar[1]: contacts from outside), closed box."""
    rng = np.random.default_rng(seed)
    rmax = radius[1]
    m = int(2 * R / spacing) + 1
    g = (np.arange(m) - (m - 1) / 2.0) * spacing
    pts = []
    for k in range(nz):
        z = rmax + k * spacing
        for x0 in g:
            for y0 in g:
                if math.hypot(x0, y0) + rmax > R - spacing:
                    continue
                if math.hypot(y0, z - bar[1]) < bar[0] + spacing:
                    continue
                pts.append((x0, y0, z))
        # a ring just inside the wall (overlapping it slightly)
        nr = int(2 * math.pi * (R - rmax) / spacing)
        for q in range(nr):
            t = 2 * math.pi * (q + 0.5 * (k % 2)) / nr
            pts.append(((R - 0.97 * rmax) * math.cos(t), (R - 0.97 * rmax) * math.sin(t), z))
    # a row resting on the bar (touching it from outside)
    zb = bar[1] + bar[0] + 0.97 * rmax
    for x0 in g[1:-1]:
        pts.append((x0, 0.0, zb))
    x = np.asarray(pts, dtype=np.float64)
    keep = np.ones(len(x), bool)
    for a in range(len(x)):  # drop lattice sites that overlap a ring or bar atom
        if keep[a]:
            d = np.linalg.norm(x[a + 1:] - x[a], axis=1)
            keep[a + 1:][d < 0.95 * spacing] = False
    x = x[keep]
    x += rng.uniform(-0.01 * spacing, 0.01 * spacing, size=x.shape)
    n = len(x)
    c = lattice_case(seed, 1, 1, 1, 1.0, radius=radius, periodic=(0, 0, 0), **kw)
    r = rng.uniform(radius[0], radius[1], size=n) if radius[0] != radius[1] else np.full(n, radius[0])
    c["boxlo"] = (-R - 4 * rmax, -R - 4 * rmax, -2 * rmax)
    c["boxhi"] = (R + 4 * rmax, R + 4 * rmax, float(x[:, 2].max() + 6 * rmax))
    c["cylinders"] = [(2, R, 0.0, 0.0, 1, c["rolling_model"]), (0, bar[0], 0.0, bar[1], 1, c["rolling_model"])]
    c["atoms"] = dict(tag=np.arange(1, n + 1, dtype=np.int32), type=np.ones(n, np.int32), x=x,
                      v=rng.uniform(-vmax, vmax, size=(n, 3)), omega=rng.uniform(-wmax, wmax, size=(n, 3)),
                      radius=r, rmass=sphere_mass(r, c["material"]["density"]))
    return c


def fine_floor_case(seed, nx=6, ny=6, nz=2, spacing=2.1e-3, radius=(0.95e-3, 1.05e-3), tri=0.5e-3,
                    jitter=2e-5, vmax=0.1, wmax=50.0, **kw):
    """A jittered lattice resting on a finely tessellated floor mesh (squares
    of `tri`, two triangles each, at z = 0) in a closed box: every atom near
    the floor has tens of candidate triangles (FixNeighlistMesh), more than
    a fixed small per-atom page would hold."""
    c = lattice_case(seed, nx, ny, nz, spacing, radius=radius, z0=0.98 * radius[0], jitter=jitter,
                     vmax=vmax, wmax=wmax, periodic=(0, 0, 0), plane_z=None, **kw)
    Lx, Ly = c["boxhi"][0], c["boxhi"][1]
    mx, my = int(round(Lx / tri)), int(round(Ly / tri))
    gx, gy = np.linspace(0.0, Lx, mx + 1), np.linspace(0.0, Ly, my + 1)
    tris = []
    for i in range(mx):
        for j in range(my):
            a = (gx[i], gy[j], 0.0)
            b = (gx[i + 1], gy[j], 0.0)
            cc = (gx[i + 1], gy[j + 1], 0.0)
            d = (gx[i], gy[j + 1], 0.0)
            tris.append((a, b, cc))
            tris.append((a, cc, d))
    c["meshes"] = [dict(nodes=np.asarray(tris, dtype=np.float64), wall_type=1, rolling=c["rolling_model"])]
    c["boxlo"] = (0.0, 0.0, -2 * radius[1])
    return c


# property/global names of the 23 per-type-pair tables of cohesion
# bond/nonlinear (src/cohesion_model_bond_nonlinear.h:70-147), in the order
# the C ABI stacks them (DEM_BOND_* / ORC_BOND_*)
BOND_TABLES = ("radiusMultiplierBondnonlinear", "stiffnessPerUnitAreaK_fn1",
               "stiffnessPerUnitAreaKu_fn1", "stiffnessPerUnitAreaKc_fn1",
               "stiffnessPerUnitAreaK_fn2", "stiffnessPerUnitAreaKu_fn2",
               "stiffnessPerUnitAreaKc_fn2", "stiffnessPerUnitAreaK_ft",
               "stiffnessPerUnitAreaK_tn", "stiffnessPerUnitAreaKu_tn", "stiffnessPerUnitAreaKc_tn",
               "stiffnessPerUnitAreaK_tt", "stiffnessPerUnitAreaKu_tt", "stiffnessPerUnitAreaKc_tt",
               "dampingNormalForceBondnonlinear", "dampingTangentialForceBondnonlinear",
               "dampingNormalTorqueBondnonlinear", "dampingTangentialTorqueBondnonlinear",
               "maxDistanceBondnonlinear", "maxSigmaBondnonlinear", "maxTauBondnonlinear",
               "ratioTensionCompressionBondnonlinear", "createDistanceBondnonlinear")
BOND_FLAGS = ("stressBreak", "tensionStress", "compressionStress", "shearStress",
              "normalTorqueStress", "shearTorqueStress", "createBondAlways", "dampingBond",
              "dampingBondSmooth", "ratioTCBond")
# the model's defaults (registerSettings, src/cohesion_model_bond_nonlinear.h:231-243)
BOND_DEFAULTS = dict(stressBreak=0, tensionStress=1, compressionStress=1, shearStress=1,
                     normalTorqueStress=1, shearTorqueStress=1, createBondAlways=0,
                     dampingBond=1, dampingBondSmooth=0, ratioTCBond=0)
# the keywords of those settings on the pair_style line
BOND_KEYWORDS = dict(stressBreak="stressBreak", tensionStress="tensionStress",
                     compressionStress="compressionStress", shearStress="shearStress",
                     normalTorqueStress="normalTorqueStress", shearTorqueStress="shearTorqueStress",
                     createBondAlways="createBondAlways", dampingBond="dampingBond",
                     dampingBondSmooth="dampingBondSmooth", ratioTCBond="ratioTensionCompressionBond")


def bond_params(ntypes, bonded_types, tsCreate=1.0, **kw):
    """Tables for cohesion bond/nonlinear: every property takes one value for
    all type pairs, except radiusMultiplier, which is 0 outside the type
    pairs within ``bonded_types`` (so walls of other types never bond).  Keyword names are the property/global names without
    the common prefixes, e.g. K_fn1=..., radiusMultiplier=..., maxDistance=...;
    on/off settings by their names in BOND_FLAGS."""
    damp = {"dampingNormalForceBondnonlinear": "damp_fn", "dampingTangentialForceBondnonlinear": "damp_ft",
            "dampingNormalTorqueBondnonlinear": "damp_tn",
            "dampingTangentialTorqueBondnonlinear": "damp_tt"}
    short = {n: damp.get(n) or n.replace("stiffnessPerUnitArea", "").replace("Bondnonlinear", "")
             .replace("ratioTensionCompression", "ratioTC") for n in BOND_TABLES}
    tabs = np.zeros((len(BOND_TABLES), ntypes + 1, ntypes + 1))
    for k, n in enumerate(BOND_TABLES):
        v = kw.pop(short[n], 0.0)
        if k == 0:  # radiusMultiplier: 0 switches the model off for a type pair
            for i in bonded_types:
                for j in bonded_types:
                    tabs[k, i, j] = v
        else:
            tabs[k, 1:, 1:] = v
    settings = dict(BOND_DEFAULTS, tsCreate=float(tsCreate))
    for f in BOND_FLAGS:
        if f in kw:
            settings[f] = int(kw.pop(f))
    assert not kw, "unknown bond parameters: %s" % sorted(kw)
    return dict(tables=tabs, settings=settings)


def elastoplastic_bond_params(ntypes, bonded_types, E, yield_strain, hardening, radius, lam=0.5, nu=0.3,
                              ref_strain_factor=2.0, **kw):
    """cohesion bond/nonlinear tables for a bond of a bilinear elastoplastic
    material: elastic modulus E, yield strain, hardening ratio (plastic
    tangent / E), Poisson ratio nu, between touching spheres of `radius`
    (bond length L0 = 2 radius, bond radius lam*radius, area A = pi (lam r)^2).

    The reference's laws (src/cohesion_model_bond_nonlinear.h:582-615 for
    the normal force, :666-872 for twist and bend) load along an envelope
    through the origin of stiffness K, unload along Ku and continue past the
    origin along Kc; tension and shear/twist/bend are linear in the
    displacement or angle (force K*A*d, torque K*J*theta or K*I*theta, K per
    unit length), compression goes with K_fn1*sqrt(d) and no area factor.  A
    bilinear material cannot be followed by a line through the origin, so:
      * Ku and Kc take the elastic stiffness (E/L0; G/L0 for shear and
        twist, G = E/(2(1+nu))): the material unloads elastically;
      * K is the secant of the bilinear curve at the reference strain
        eps_r = ref_strain_factor * yield_strain:
        sigma(eps_r)/eps_r / L0 with sigma = E (eps_y + h (eps_r - eps_y));
        the unloading from eps_r then leaves the bilinear material's
        permanent set eps_r - sigma/E exactly (1 - K/Ku = 1 - sigma/(E eps_r));
      * compression: K_fn1 sqrt(eps_r L0) = A sigma(eps_r), and Ku_fn1 so
        that the sqrt-law unloading leaves the same permanent set
        ((1 - K/Ku)^2 = 1 - sigma/(E eps_r)); Kc_fn1 = Ku_fn1;
      * shear force (K_ft, no hysteresis in the reference): G/L0.
    Remaining keywords go to bond_params (damping, break and creation
    settings)."""
    L0 = 2.0 * radius
    A = math.pi * (lam * radius) ** 2
    G = E / (2.0 * (1.0 + nu))
    eps_r = ref_strain_factor * yield_strain
    sig = E * (yield_strain + hardening * (eps_r - yield_strain))
    sec = sig / (E * eps_r)  # secant / elastic modulus
    k_fn1 = A * sig / math.sqrt(eps_r * L0)
    ku_fn1 = k_fn1 / (1.0 - math.sqrt(1.0 - sec))
    return bond_params(ntypes, bonded_types, radiusMultiplier=lam,
                       K_fn1=k_fn1, Ku_fn1=ku_fn1, Kc_fn1=ku_fn1,
                       K_fn2=sec * E / L0, Ku_fn2=E / L0, Kc_fn2=E / L0,
                       K_ft=G / L0,
                       K_tn=sec * G / L0, Ku_tn=G / L0, Kc_tn=G / L0,
                       K_tt=sec * E / L0, Ku_tt=E / L0, Kc_tt=E / L0, **kw)


def fibre_case(seed, nfib, nper, radius, box, spacing=(0.999, 1.001), density=1000.0,
               E=(5e7, 5e7), nu=(0.3, 0.3), rest=((0.5, 0.5), (0.5, 0.5)),
               frict=((0.3, 0.3), (0.3, 0.3)), vmax=0.0, wmax=0.0, dt=1e-7, skin=2e-4,
               gravity=(0.0, 0.0, -9.81), bond=None, gap=1.3, max_tries=200000, z0=None,
               max_fail=None, periodic_xy=True):
    """Straight fibres of nper touching spheres (type 1) with directions
    uniform on the sphere, centres uniform in the box; a floor plane of wall
    type 2 at z = 0, periodic in x and y.  Sphere spacing along a fibre is
    spacing[0..1] x 2r (per fibre, uniform); spheres of different fibres stay
    more than gap x 2r apart, so only intra-fibre pairs bond at creation.
    Placement stops after max_tries trials or max_fail trials in a row
    without success.
    ``bond`` is a bond_params(...) dict (cohesion bond/nonlinear)."""
    rng = np.random.default_rng(seed)
    Lx, Ly, Lz = box
    d = 2.0 * radius
    pts = []
    # spatial hash of placed spheres (cell >= gap*d), periodic in x and y
    cs = gap * d
    ncx, ncy = max(1, int(Lx // cs)), max(1, int(Ly // cs))
    csx, csy = Lx / ncx, Ly / ncy
    grid = {}

    def key(p):
        return (int(p[0] // csx) % ncx, int(p[1] // csy) % ncy, int(p[2] // cs))

    def clear(chain):
        for p in chain:
            kx, ky, kz = key(p)
            for ox in (-1, 0, 1):
                for oy in (-1, 0, 1):
                    for oz in (-1, 0, 1):
                        for q in grid.get(((kx + ox) % ncx, (ky + oy) % ncy, kz + oz), ()):
                            dx = p[0] - q[0]
                            dy = p[1] - q[1]
                            if periodic_xy:
                                dx -= Lx * round(dx / Lx)
                                dy -= Ly * round(dy / Ly)
                            dz = p[2] - q[2]
                            if dx * dx + dy * dy + dz * dz < (gap * d) ** 2:
                                return False
        return True

    tries = fails = 0
    while len(pts) < nfib and tries < max_tries and (max_fail is None or fails < max_fail):
        tries += 1
        fails += 1
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        sp = d * rng.uniform(*spacing)
        half = 0.5 * (nper - 1) * sp
        lo = np.array([0.0, 0.0, (z0 if z0 is not None else radius) + half * abs(u[2]) + radius])
        hi = np.array([Lx, Ly, Lz - half * abs(u[2]) - radius])
        if not periodic_xy:  # whole fibre inside the side walls
            for ax in (0, 1):
                lo[ax] = half * abs(u[ax]) + radius
                hi[ax] = box[ax] - half * abs(u[ax]) - radius
        if np.any(hi <= lo):
            continue
        c = rng.uniform(lo, hi)
        chain = c + (np.arange(nper) - 0.5 * (nper - 1))[:, None] * sp * u
        if periodic_xy:
            chain[:, 0] %= Lx
            chain[:, 1] %= Ly
        if not clear(chain):
            continue
        for p in chain:
            grid.setdefault(key(p), []).append(p)
        pts.append(chain)
        fails = 0
    x = np.concatenate(pts).astype(np.float64)
    n = len(x)
    r = np.full(n, radius)
    v = rng.uniform(-vmax, vmax, size=(n, 3)) if vmax > 0 else np.zeros((n, 3))
    w = rng.uniform(-wmax, wmax, size=(n, 3)) if wmax > 0 else np.zeros((n, 3))
    case = dict(
        boxlo=(0.0, 0.0, 0.0), boxhi=(Lx, Ly, Lz), periodic=(1, 1, 0) if periodic_xy else (0, 0, 0),
        dt=dt, skin=skin, cdf=1.0,
        neigh=(1, 0, 1), normal_model=0, rolling_model=0, gravity=gravity, ntypes=2, charVel=0.0,
        planes=[(2, 0.0, 2, 0)], cohesion_model=1 if bond is not None else 0,
        material=dict(E=list(E), nu=list(nu), rest=[list(q) for q in rest],
                      frict=[list(q) for q in frict], rollfrict=None, density=density),
        atoms=dict(tag=np.arange(1, n + 1, dtype=np.int32), type=np.ones(n, np.int32), x=x, v=v,
                   omega=w, radius=r, rmass=sphere_mass(r, density)),
        nfibres=len(pts), nper=nper,
    )
    if bond is not None:
        case["bond"] = bond
    case.update(derive_tables(E, nu, rest, frict, None))
    return case


def fibre_bed_case(seed, n_target, radius=0.5e-3, nper=10, box_xy=(45e-3, 45e-3), along=1.0,
                   across=1.05, end_gap=1.2, density=1000.0, E=(5e7, 5e7), nu=(0.3, 0.3),
                   rest=((0.5, 0.5), (0.5, 0.5)), frict=((0.3, 0.3), (0.3, 0.3)), dt=1e-7, skin=2e-4,
                   vmax=0.05, bond=None, plate_vel=None, plate_gap=0.5e-3):
    """A bed of straight fibres of nper spheres, built layer by layer (no
    random placement, so it scales to 10^5-10^6 spheres): in each layer the
    fibres lie parallel, along x in even layers and along y in odd ones
    (plywood order).  Spheres of a fibre are along x 2r apart (touching), rows
    and layers across x 2r apart, and fibre ends end_gap x 2r apart, so with
    createDistance between 2r and across x 2r only intra-fibre neighbours bond.
    Periodic in x and y, floor plane of wall type 2 at z = 0, atoms type 1.
    With plate_vel, a closed box instead: floor and four side planes, and a
    two-triangle lid of wall type 2 plate_gap above the highest sphere
    surface, moving with velocity plate_vel (fix move/mesh ... linear)."""
    rng = np.random.default_rng(seed)
    d = 2.0 * radius
    Lx, Ly = box_xy
    flen = (nper - 1) * along * d + end_gap * d  # fibre pitch along its axis
    nfx = max(1, int(Lx // flen))
    nrow = max(1, int(Ly // (across * d)))
    Lx_eff, Ly_eff = nfx * flen, nrow * across * d
    L = min(Lx_eff, Ly_eff)
    nfx = max(1, int(L // flen))
    nrow = max(1, int(L // (across * d)))
    L = nfx * flen
    nrow = int(L // (across * d))
    per_layer = nfx * nrow * nper
    nlayer = (n_target + per_layer - 1) // per_layer
    k = np.arange(nper)
    pts = []
    for lay in range(nlayer):
        z = radius + lay * across * d
        fx, row = np.meshgrid(np.arange(nfx), np.arange(nrow), indexing="ij")
        a0 = (fx.ravel()[:, None] * flen + k[None, :] * along * d + 0.5 * end_gap * d)
        b0 = np.repeat((row.ravel()[:, None] + 0.5) * across * d, nper, axis=1)
        if lay % 2 == 0:
            xy = np.stack([a0.ravel(), b0.ravel()], axis=1)
        else:
            xy = np.stack([b0.ravel(), a0.ravel()], axis=1)
        pts.append(np.column_stack([xy, np.full(len(xy), z)]))
    x = np.concatenate(pts)[:n_target - n_target % nper].astype(np.float64)
    n = len(x)
    Lz = radius + nlayer * across * d + 20 * d
    r = np.full(n, radius)
    v = rng.uniform(-vmax, vmax, size=(n, 3)) if vmax > 0 else np.zeros((n, 3))
    case = dict(
        boxlo=(0.0, 0.0, 0.0), boxhi=(L, L, Lz), periodic=(1, 1, 0), dt=dt, skin=skin, cdf=1.0,
        neigh=(1, 0, 1), normal_model=0, rolling_model=0, gravity=(0.0, 0.0, -9.81), ntypes=2,
        charVel=0.0, planes=[(2, 0.0, 2, 0)], cohesion_model=1 if bond is not None else 0,
        material=dict(E=list(E), nu=list(nu), rest=[list(q) for q in rest],
                      frict=[list(q) for q in frict], rollfrict=None, density=density),
        atoms=dict(tag=np.arange(1, n + 1, dtype=np.int32), type=np.ones(n, np.int32), x=x, v=v,
                   omega=np.zeros((n, 3)), radius=r, rmass=sphere_mass(r, density)),
        nfibres=n // nper, nper=nper,
    )
    if bond is not None:
        case["bond"] = bond
    if plate_vel is not None:
        ztop = float(np.max(x[:, 2])) + radius + plate_gap
        case["periodic"] = (0, 0, 0)
        case["planes"] = [(2, 0.0, 2, 0), (0, 0.0, 2, 0), (0, L, 2, 0), (1, 0.0, 2, 0), (1, L, 2, 0)]
        inset = 0.1 * radius
        case["meshes"] = [dict(nodes=plate_mesh(inset, L - inset, inset, L - inset, ztop), wall_type=2,
                               rolling=0, vel=tuple(float(v) for v in plate_vel))]
    case.update(derive_tables(E, nu, rest, frict, None))
    return case


def plate_mesh(x0, x1, y0, y1, z):
    """Two triangles of a horizontal plate [x0,x1] x [y0,y1] at height z,
    normal +z; nodes[2, 3, 3]."""
    a, b, c, d = (x0, y0, z), (x1, y0, z), (x1, y1, z), (x0, y1, z)
    return np.array([(a, b, c), (a, c, d)], dtype=np.float64)


def press_case(seed, nfib, nper, radius, box, plate_gap, plate_vel, inset=None, fill_height=None,
               **kw):
    """Fibres of bonded spheres in a closed box: floor and four side walls are
    primitive planes of wall type 2, the lid is a two-triangle mesh plate of
    wall type 2 that starts plate_gap above the highest sphere surface and
    moves with velocity plate_vel (fix move/mesh ... linear).  Fibres fill
    the box up to fill_height (default 80 % of its height)."""
    Lx, Ly, Lz = box
    zf = 0.8 * Lz if fill_height is None else fill_height
    c = fibre_case(seed, nfib, nper, radius, (Lx, Ly, zf), periodic_xy=False, **kw)
    c["boxhi"] = (Lx, Ly, Lz)
    x = c["atoms"]["x"]
    ztop = float(np.max(x[:, 2])) + radius + plate_gap
    if inset is None:
        inset = 0.1 * radius
    c["planes"] = [(2, 0.0, 2, 0), (0, 0.0, 2, 0), (0, Lx, 2, 0), (1, 0.0, 2, 0), (1, Ly, 2, 0)]
    c["meshes"] = [dict(nodes=plate_mesh(inset, Lx - inset, inset, Ly - inset, ztop), wall_type=2,
                        rolling=0, vel=tuple(float(v) for v in plate_vel))]
    return c


def paddle_mesh(cx, cy, half_len, z0, z1):
    """A vertical two-triangle paddle through (cx, cy) spanning x in
    [cx - half_len, cx + half_len], z in [z0, z1] at y = cy; nodes[2, 3, 3]."""
    a, b, c, d = (cx - half_len, cy, z0), (cx + half_len, cy, z0), (cx + half_len, cy, z1), (cx - half_len, cy, z1)
    return np.array([(a, b, c), (a, c, d)], dtype=np.float64)


def mixer_case(seed, nx, ny, nz, spacing, radius, blade_half_len, blade_height, period, **kw):
    """A jittered lattice on a floor (periodic x/y) stirred by a vertical
    paddle mesh turning about the vertical axis through the box centre (fix
    move/mesh ... rotate origin O axis 0 0 1 period T).  The paddle lies in
    the gap between two lattice rows."""
    c = lattice_case(seed, nx, ny, nz, spacing, radius=radius, **kw)
    cx = 0.5 * nx * spacing
    cy = (ny // 2) * spacing
    c["meshes"] = [dict(nodes=paddle_mesh(cx, cy, blade_half_len, 0.0, blade_height), wall_type=1,
                        rolling=c.get("rolling_model", 0),
                        rotate=dict(origin=(cx, cy, 0.0), axis=(0.0, 0.0, 1.0), period=float(period)))]
    return c


def lattice_case(seed, nx, ny, nz, spacing, radius=(1e-3, 1e-3), density=2500.0,
                 z0=None, jitter=0.0, vmax=0.0, wmax=0.0, ntypes=1, E=(5e6,), nu=(0.45,),
                 rest=((0.9,),), frict=((0.5,),), rollfrict=None, periodic=(1, 1, 0),
                 zhi=None, dt=1e-6, skin=5e-4, gravity=(0.0, 0.0, -9.81), plane_z=0.0,
                 normal_model=0, rolling_model=0, charVel=0.0, pad=(0.0, 0.0)):
    """Jittered cubic lattice of spheres in a box periodic in x/y with a floor.

    Box x/y extents are nx*spacing, ny*spacing (exactly periodic lattice);
    z starts at z0 (default: radius_max) and the box top is zhi.
    """
    rng = np.random.default_rng(seed)
    n = nx * ny * nz
    Lx, Ly = nx * spacing + pad[0], ny * spacing + pad[1]
    rmax = radius[1]
    if z0 is None:
        z0 = rmax
    ii, jj, kk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    x = np.stack([(ii.ravel() + 0.5) * spacing, (jj.ravel() + 0.5) * spacing,
                  z0 + kk.ravel() * spacing], axis=1).astype(np.float64)
    if jitter > 0:
        x += rng.uniform(-jitter, jitter, size=x.shape)
        x[:, 2] = np.maximum(x[:, 2], z0 - jitter)
    if zhi is None:
        zhi = z0 + nz * spacing + 4 * rmax
    r = rng.uniform(radius[0], radius[1], size=n) if radius[0] != radius[1] else np.full(n, radius[0])
    typ = rng.integers(1, ntypes + 1, size=n).astype(np.int32)
    v = rng.uniform(-vmax, vmax, size=(n, 3)) if vmax > 0 else np.zeros((n, 3))
    w = rng.uniform(-wmax, wmax, size=(n, 3)) if wmax > 0 else np.zeros((n, 3))
    rmass = sphere_mass(r, density)
    case = dict(
        boxlo=(0.0, 0.0, 0.0), boxhi=(Lx, Ly, float(zhi)), periodic=tuple(periodic),
        dt=dt, skin=skin, cdf=1.0, neigh=(1, 0, 1), normal_model=normal_model,
        rolling_model=rolling_model, gravity=gravity, ntypes=ntypes, charVel=charVel,
        planes=[(2, plane_z, 1, rolling_model)] if plane_z is not None else [],
        material=dict(E=list(E), nu=list(nu), rest=[list(r_) for r_ in rest],
                      frict=[list(f_) for f_ in frict],
                      rollfrict=[list(f_) for f_ in rollfrict] if rollfrict is not None else None,
                      density=density),
        atoms=dict(tag=np.arange(1, n + 1, dtype=np.int32), type=typ, x=x, v=v, omega=w,
                   radius=r, rmass=rmass),
    )
    case.update(derive_tables(E, nu, rest, frict, rollfrict))
    return case
