"""Batched ensemble runner: many independent granular systems advanced
together on one GPU by one resident handle.

The reference runs one process per system.  Here the systems are packed into
one handle (dem_set_ensemble) and every kernel of a timestep covers all of
them at once (one graph-resident step loop, one conditional rebuild node),
which turns hundreds of launch-bound small systems into one large, FP64- and
bandwidth-bound one:

  * system k is the atoms of type k+1; the per-type-pair tables hold system
    k's Yeff/Geff/betaeff/friction on the diagonal (k+1, k+1); systems never
    touch, so off-diagonal entries are never read;
  * every system keeps its own coordinates in the shared box (same size and
    boundaries for all); the library gives each system its own block of
    neighbour cells, so pairs and periodic images never cross systems and
    each system sees exactly the coordinates of its standalone run;
  * each system's floor is a per-type primitive plane (dem_add_plane_per_type)
    at its own height, with wall type = the atom's type;
  * tags are offset per system so that they stay unique.

Each system takes its own neighbour decision, as it would running alone
(Neighbor::decide, src/neighbor.cpp:1362-1378): a system rebuilds when one
of its own atoms moved beyond skin/2, and the others keep their atom order,
list entries and histories.  A build touches only the rebuilding systems'
atoms and list segments.  Each system therefore evolves exactly as its
standalone run, rebuild steps included; the systems do not interact.

The autotuner times short runs of the packed ensemble over launch shapes
(blocks per SM, dem_set_tuning; threads per block of the per-particle
kernel, dem_set_particle_threads), neighbour-cell sizes and, when asked, the
neighbour skin, and keeps the fastest.  Launch shape and cell size change no
result beyond summation order.  The skin changes the rebuild schedule: a pair that
separates and touches again between two builds keeps its tangential
history, one rebuilt in between starts afresh (src/neigh_gran.cpp carry-over
rule), so a tuned skin gives an equally valid but not bit-identical run;
skins are therefore tuned only when the caller lists candidates.
"""
import itertools
import time

import numpy as np

from . import workloads


def pack(systems):
    """systems: list of single-type cases (workloads.lattice_case style, one
    primitive zplane floor each, the same box).  Returns (case, layout)."""
    if not systems:
        raise ValueError("empty ensemble")
    s0 = systems[0]
    keys = ("dt", "skin", "normal_model", "rolling_model", "periodic", "gravity", "neigh", "boxlo",
            "boxhi", "cdf")
    for s in systems:
        for k in keys:
            if tuple(np.atleast_1d(s.get(k))) != tuple(np.atleast_1d(s0.get(k))):
                raise ValueError("ensemble systems differ in %s" % k)
        if s["ntypes"] != 1:
            raise ValueError("ensemble systems must be single-type")
        if len(s["planes"]) != 1:
            raise ValueError("each system needs exactly one primitive floor")
        if s.get("meshes"):
            raise ValueError("mesh walls are not supported in ensembles")
    nsys = len(systems)
    nt = nsys
    tabs = {k: np.zeros((nt + 1, nt + 1)) for k in
            ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRollFrict", "coeffRestLog")}
    floor = np.zeros(nt + 1)
    parts = {k: [] for k in ("tag", "type", "x", "v", "omega", "radius", "rmass")}
    offsets, counts = [], []
    tag0 = 0
    for k, s in enumerate(systems):
        t = k + 1
        for name in tabs:
            tabs[name][t, t] = np.asarray(s[name])[1, 1]
        floor[t] = float(s["planes"][0][1])
        a = s["atoms"]
        n = len(a["tag"])
        parts["tag"].append(np.asarray(a["tag"], np.int32) + tag0)
        parts["type"].append(np.full(n, t, np.int32))
        for name in ("x", "v", "omega", "radius", "rmass"):
            parts[name].append(np.asarray(a[name], dtype=np.float64))
        offsets.append(tag0)
        counts.append(n)
        tag0 += int(np.max(a["tag"]))
    floor[0] = floor[1]
    axis, _, _, roll = s0["planes"][0]
    case = dict(
        boxlo=tuple(s0["boxlo"]), boxhi=tuple(s0["boxhi"]), periodic=tuple(s0["periodic"]),
        dt=s0["dt"], skin=s0["skin"], cdf=s0.get("cdf", 1.0), neigh=s0.get("neigh", (1, 0, 1)),
        normal_model=s0["normal_model"], rolling_model=s0["rolling_model"], gravity=s0["gravity"],
        ntypes=nt, charVel=s0.get("charVel", 0.0), planes=[],
        planes_per_type=[(axis, floor, roll)], ensemble=nsys,
        atoms={k: np.concatenate(v) for k, v in parts.items()},
    )
    case.update(tabs)
    layout = dict(nsys=nsys, offsets=offsets, counts=counts)
    return case, layout


class Ensemble:
    """One handle running a packed ensemble."""

    def __init__(self, systems, tuning=None, skin=None):
        from .api import DemSystem
        if skin is not None:
            systems = [dict(s, skin=float(skin)) for s in systems]
        self.case, self.layout = pack(systems)
        if tuning is not None:
            self.case["tuning"] = tuning
        self.sys = DemSystem(self.case)

    def setup(self):
        self.sys.setup()

    def step(self, n):
        self.sys.step(n)

    def stats(self):
        return self.sys.stats()

    def rebuilds(self):
        """Neighbour list builds of every system (dem_ensemble_rebuilds)."""
        from .api import _p, load
        out = np.zeros(self.layout["nsys"], np.int32)
        self.sys._check(load().dem_ensemble_rebuilds(self.sys.h, _p(out)))
        return out

    def system_atoms(self, k):
        """Atoms of system k with its own tags and coordinates (sorted by tag)."""
        a = self.sys.atoms()
        sel = a["type"] == k + 1
        tag0 = self.layout["offsets"][k]
        out = {key: (v[sel] if isinstance(v, np.ndarray) and len(v) == len(sel) else v)
               for key, v in a.items()}
        out["tag"] = out["tag"] - tag0
        out["type"] = np.ones_like(out["type"])
        order = np.argsort(out["tag"], kind="stable")
        return {key: v[order] for key, v in out.items()}

    def close(self):
        self.sys.close()


def autotune(systems, steps=30, blocks_per_sm=(4, 8, 16), cell_scale=(1.0, 1.25, 1.5), warm=5, skins=None,
             particle_threads=(256,)):
    """Times `steps` steps of the packed ensemble for each (blocks_per_sm,
    cell_scale, skin, particle_threads) and returns the fastest as (best,
    table); best is (blocks_per_sm, cell_scale, skin, particle_threads) with
    skin None unless skins lists candidates.  The timed steps include the
    rebuilds they trigger, so a skin is judged by its rebuild rate as well as
    its list length."""
    table = []
    for bps, cs, sk, pt in itertools.product(blocks_per_sm, cell_scale, skins or (None,), particle_threads):
        e = Ensemble(systems, tuning=(bps, cs, pt), skin=sk)
        e.setup()
        e.step(warm)
        t0 = time.perf_counter()
        e.step(steps)
        ms = e.stats()["last_step_ms"]
        table.append(((bps, cs, sk, pt), ms / steps, time.perf_counter() - t0))
        e.close()
    best = min(table, key=lambda r: r[1])[0]
    return best, table


def settling_systems(seed, nsys, nmin=2000, nmax=20000, spacing=2.2e-3, box=(0.05, 0.05, 0.3),
                     radius=(0.9e-3, 1.1e-3), density=2500.0, dt=1e-6, skin=5e-4):
    """The batched settling-column ensemble: per system N ~ U[nmin, nmax]
    spheres on a jittered lattice above a floor, radii U[0.9, 1.1] mm, in a
    0.05 x 0.05 x 0.3 m box periodic in x/y; E log-uniform in [1e6, 1e8] Pa,
    restitution U[0.3, 0.95], friction U[0.1, 0.9] per system; Hertz +
    tangential history; seeded."""
    rng = np.random.default_rng(seed)
    nx = int(box[0] / spacing)
    ny = int(box[1] / spacing)
    out = []
    for k in range(nsys):
        n = int(rng.integers(nmin, nmax + 1))
        E = float(np.exp(rng.uniform(np.log(1e6), np.log(1e8))))
        e = float(rng.uniform(0.3, 0.95))
        mu = float(rng.uniform(0.1, 0.9))
        nz = (n + nx * ny - 1) // (nx * ny)
        c = workloads.lattice_case(
            seed=int(rng.integers(1 << 30)), nx=nx, ny=ny, nz=nz, spacing=spacing, radius=radius,
            density=density, z0=1.2 * radius[1], jitter=0.05 * spacing, E=(E,), nu=(0.3,),
            rest=((e,),), frict=((mu,),), dt=dt, skin=skin, zhi=box[2], pad=(box[0] - nx * spacing,
                                                                             box[1] - ny * spacing))
        a = c["atoms"]
        keep = np.arange(len(a["tag"])) < n
        c["atoms"] = {key: v[keep] for key, v in a.items()}
        c["material_summary"] = dict(E=E, restitution=e, friction=mu, n=n)
        out.append(c)
    return out
