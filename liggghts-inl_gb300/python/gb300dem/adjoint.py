"""Discrete adjoint of the sphere-DEM timestep (dem_adjoint_* in the C ABI).

``DemAdjoint`` owns one adjoint handle: an initial granular state (one atom
type, one material, primitive planes, static triangle meshes, gravity,
optionally cohesion bond/nonlinear) and a run length.  ``loss()``
runs the forward model only; ``gradient()`` also runs the backward pass and
returns d(loss)/d(E, restitution, friction, radius_i).  ``AdjointLoss`` is a
``torch.autograd.Function`` over the same call, so the parameters can sit in
a torch optimisation loop (the simulation itself runs in the library's CUDA
kernels, not in torch).

The forward model is the reference's: Verlet::setup, then N Verlet steps of
FixNVESphere + PairGran (Hertz, tangential history, cohesion bond/nonlinear
when the case has bonds) + FixGravity + FixWallGran primitive planes, with
the neighbour list rebuilt every
`segment` steps (neigh_modify every <segment> delay 0 check no).
"""
import ctypes

import numpy as np

from . import api

P = ctypes.c_void_p
D = ctypes.c_double


class DemAdjointConfig(ctypes.Structure):
    _fields_ = [("boxlo", D * 3), ("boxhi", D * 3), ("periodic", ctypes.c_int * 3), ("dt", D),
                ("skin", D), ("density", D), ("poisson", D), ("gravity_on", ctypes.c_int),
                ("gravity", D * 3), ("nplanes", ctypes.c_int), ("plane_axis", ctypes.c_int * 8),
                ("plane_pos", D * 8)]


class DemAdjointLoss(ctypes.Structure):
    _fields_ = [("w_ke", D), ("w_height", D), ("height_target", D), ("w_wallforce", D),
                ("wallforce_target", D), ("wall_id", ctypes.c_int), ("wall_axis", ctypes.c_int)]


def _bind(L):
    if getattr(L, "_adjoint_bound", False):
        return L
    I = ctypes.c_int
    L.dem_adjoint_create.argtypes = [ctypes.POINTER(DemAdjointConfig), ctypes.POINTER(P)]
    L.dem_adjoint_destroy.argtypes = [P]
    L.dem_adjoint_set_state.argtypes = [P, I, P, P, P, P]
    L.dem_adjoint_set_bonds.argtypes = [P, P, ctypes.POINTER(api.DemBondSettings)]
    L.dem_adjoint_add_mesh.argtypes = [P, I, P, P, P]
    L.dem_adjoint_set_rolling.argtypes = [P, D]
    L.dem_adjoint_set_mesh_motion.argtypes = [P, I, P]
    L.dem_adjoint_rolling_gradient.argtypes = [P, P]
    L.dem_adjoint_forward.argtypes = [P, D, D, D, P, I, I, ctypes.POINTER(DemAdjointLoss), P]
    L.dem_adjoint_gradient.argtypes = [P, D, D, D, P, I, I, ctypes.POINTER(DemAdjointLoss), P, P, P, P, P]
    L.dem_adjoint_download.argtypes = [P, P, P, P]
    L.dem_adjoint_times.argtypes = [P, P, P, P, P]
    L.dem_adjoint_set_tape.argtypes = [P, I, D]
    L.dem_adjoint_tape_recorded.argtypes = [P, P]
    L.dem_adjoint_last_error.argtypes = [P]
    L.dem_adjoint_last_error.restype = ctypes.c_char_p
    L._adjoint_bound = True
    return L


def make_loss(w_ke=0.0, w_height=0.0, height_target=0.0, w_wallforce=0.0, wallforce_target=0.0,
              wall_id=-1, wall_axis=2):
    """wall_id: planes first, then meshes; wall_axis: the force component of a
    mesh (a plane takes its normal)"""
    return DemAdjointLoss(w_ke, w_height, height_target, w_wallforce, wallforce_target, wall_id, wall_axis)


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a


class DemAdjoint:
    """One adjoint handle.  `case`: a single-type granular case
    (workloads.lattice_case style: box, dt, skin, gravity, primitive planes,
    material with E/nu/rest/frict, atoms with x/v/omega/radius); the atoms'
    rmass must be 4/3 pi r^3 rho of material['density']."""

    def __init__(self, case):
        if case.get("ntypes", 1) != 1:
            raise ValueError("the adjoint covers one atom type")
        if case.get("normal_model", 0) != 0:
            raise ValueError("the adjoint covers Hertz")
        rolling = case.get("rolling_model", 0)
        if rolling not in (0, 1):
            raise ValueError("the adjoint covers no rolling friction or CDT")
        if any(int(pl[3]) != rolling for pl in case.get("planes", [])):
            raise ValueError("the adjoint's walls use the pairs' rolling model")
        if case.get("cylinders"):
            raise ValueError("the adjoint covers primitive planes and meshes, not cylinders")
        for m in case.get("meshes", []):
            if m.get("rotate") is not None:
                raise ValueError("the adjoint covers static and translating meshes")
            if int(m["wall_type"]) != 1 or int(m.get("rolling", 0)) != rolling:
                raise ValueError("the adjoint's meshes are of the atoms' material (wall type 1) and rolling model")
        bonded = case.get("cohesion_model", 0) == 1
        if float(case.get("cdf", 1.0)) != 1.0:
            raise ValueError("the adjoint takes the contact distance factor of its bonds, else 1")
        self.L = _bind(api.load())
        mat = case["material"]
        cfg = DemAdjointConfig()
        for d in range(3):
            cfg.boxlo[d] = case["boxlo"][d]
            cfg.boxhi[d] = case["boxhi"][d]
            cfg.periodic[d] = int(case["periodic"][d])
            cfg.gravity[d] = case["gravity"][d] if case.get("gravity") is not None else 0.0
        cfg.dt = case["dt"]
        cfg.skin = case["skin"]
        cfg.density = float(mat["density"])
        cfg.poisson = float(mat["nu"][0])
        cfg.gravity_on = 1 if case.get("gravity") is not None else 0
        planes = case.get("planes", [])
        if len(planes) > 8:
            raise ValueError("at most 8 planes")
        cfg.nplanes = len(planes)
        for w, pl in enumerate(planes):
            cfg.plane_axis[w] = int(pl[0])
            cfg.plane_pos[w] = float(pl[1])
        self.params = dict(E=float(mat["E"][0]), restitution=float(mat["rest"][0][0]),
                           friction=float(mat["frict"][0][0]))
        h = P()
        rc = self.L.dem_adjoint_create(ctypes.byref(cfg), ctypes.byref(h))
        if rc != 0:
            raise api.DemError("dem_adjoint_create: %s" % api.STATUS.get(rc, rc))
        self.h = h
        if bonded:
            b = case["bond"]
            vals = np.ascontiguousarray(np.asarray(b["tables"], dtype=np.float64)[:, 1, 1])
            st = api.DemBondSettings()
            st.tsCreate = float(b["settings"]["tsCreate"])
            for k in api.BOND_FLAGS:
                setattr(st, k, int(b["settings"][k]))
            self._call("dem_adjoint_set_bonds", self.h, api._p(vals), ctypes.byref(st))
        if rolling == 1:
            self._call("dem_adjoint_set_rolling", self.h, float(mat["rollfrict"][0][0]))
        self._meshkeep = []
        for mi, m in enumerate(case.get("meshes", [])):
            nodes = _f64(m["nodes"])
            ea, ca = m.get("edge_active"), m.get("corner_active")
            ea = np.ascontiguousarray(ea, dtype=np.uint8) if ea is not None else None
            ca = np.ascontiguousarray(ca, dtype=np.uint8) if ca is not None else None
            self._meshkeep += [nodes, ea, ca]
            self._call("dem_adjoint_add_mesh", self.h, len(nodes), api._p(nodes), api._p(ea), api._p(ca))
            if m.get("vel") is not None:
                vel = _f64(m["vel"])
                self._meshkeep.append(vel)
                self._call("dem_adjoint_set_mesh_motion", self.h, mi, api._p(vel))
        a = case["atoms"]
        self.n = len(a["radius"])
        self.radius = _f64(a["radius"]).copy()
        self._call("dem_adjoint_set_state", self.h, self.n, api._p(_f64(a["x"], (-1, 3))),
                   api._p(_f64(a["v"], (-1, 3))), api._p(_f64(a["omega"], (-1, 3))), api._p(self.radius))

    def _call(self, name, *args):
        rc = getattr(self.L, name)(*args)
        if rc != 0:
            msg = self.L.dem_adjoint_last_error(self.h).decode() if getattr(self, "h", None) else ""
            raise api.DemError("%s: %s %s" % (name, api.STATUS.get(rc, rc), msg))

    def loss(self, E, restitution, friction, radius=None, nsteps=100, segment=10, loss=None):
        out = D()
        r = None if radius is None else _f64(radius)
        self._call("dem_adjoint_forward", self.h, E, restitution, friction, api._p(r), nsteps, segment,
                   ctypes.byref(loss or make_loss(w_ke=1.0)), ctypes.byref(out))
        return out.value

    def gradient(self, E, restitution, friction, radius=None, nsteps=100, segment=10, loss=None):
        out, gE, ge, gmu = D(), D(), D(), D()
        r = None if radius is None else _f64(radius)
        gr = np.zeros(self.n)
        self._call("dem_adjoint_gradient", self.h, E, restitution, friction, api._p(r), nsteps, segment,
                   ctypes.byref(loss or make_loss(w_ke=1.0)), ctypes.byref(out), ctypes.byref(gE),
                   ctypes.byref(ge), ctypes.byref(gmu), api._p(gr))
        gmr = D()
        self._call("dem_adjoint_rolling_gradient", self.h, ctypes.byref(gmr))
        return out.value, dict(E=gE.value, restitution=ge.value, friction=gmu.value, radius=gr,
                               rolling_friction=gmr.value)

    def set_tape(self, mode, max_bytes=0.0):
        """Where the backward pass takes each step's record: 0 replay from
        checkpoints (O(sqrt(N)) memory), 1 record every step in the forward
        pass, 2 record when it fits max_bytes (default: half the free device
        memory)."""
        self._call("dem_adjoint_set_tape", self.h, int(mode), float(max_bytes))

    def tape_recorded(self):
        r = ctypes.c_int()
        self._call("dem_adjoint_tape_recorded", self.h, ctypes.byref(r))
        return bool(r.value)

    def final_state(self):
        x, v, w = (np.zeros((self.n, 3)) for _ in range(3))
        self._call("dem_adjoint_download", self.h, api._p(x), api._p(v), api._p(w))
        return dict(x=x, v=v, omega=w)

    def times(self):
        f, b = D(), D()
        ns, mp = ctypes.c_int(), ctypes.c_int()
        self._call("dem_adjoint_times", self.h, ctypes.byref(f), ctypes.byref(b), ctypes.byref(ns),
                   ctypes.byref(mp))
        return dict(forward_ms=f.value, backward_ms=b.value, segments=ns.value, max_pairs=mp.value)

    def close(self):
        if getattr(self, "h", None):
            self.L.dem_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _autograd_function():
    import torch

    class AdjointLoss(torch.autograd.Function):
        """loss = AdjointLoss.apply(E, restitution, friction, radius, engine,
        nsteps, segment, loss_spec): scalar fp64 tensors E, restitution,
        friction and an (n,) fp64 tensor of radii (CPU tensors; the
        simulation runs on the GPU through the engine)."""

        @staticmethod
        def forward(ctx, E, restitution, friction, radius, engine, nsteps, segment, spec):
            r = radius.detach().cpu().double().numpy()
            val, g = engine.gradient(float(E), float(restitution), float(friction), r, nsteps, segment, spec)
            ctx.save_for_backward(torch.tensor(g["E"], dtype=torch.float64),
                                  torch.tensor(g["restitution"], dtype=torch.float64),
                                  torch.tensor(g["friction"], dtype=torch.float64),
                                  torch.from_numpy(g["radius"]))
            return torch.tensor(val, dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            gE, ge, gmu, gr = ctx.saved_tensors
            return gout * gE, gout * ge, gout * gmu, gout * gr, None, None, None, None

    return AdjointLoss


_AF = None


def adjoint_loss(E, restitution, friction, radius, engine, nsteps=100, segment=10, spec=None):
    """Differentiable loss of the final state (torch tensors in, scalar out)."""
    global _AF
    if _AF is None:
        _AF = _autograd_function()
    return _AF.apply(E, restitution, friction, radius, engine, nsteps, segment, spec or make_loss(w_ke=1.0))
