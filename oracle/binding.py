"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes binding of ``dem_oracle.c`` (the CPU restatement of the reference's
sphere timestep).  ``build()`` compiles it with ``-ffp-contract=off`` so that
the arithmetic is plain IEEE double on x86-64 and on aarch64 alike.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle_dem.so")

NORMAL_HERTZ, NORMAL_HOOKE = 0, 1
ROLLING_OFF, ROLLING_CDT = 0, 1
COHESION_OFF, COHESION_BOND_NONLINEAR = 0, 1
# on/off settings of cohesion bond/nonlinear, in orc_bond_settings order
BOND_FLAGS = ("stressBreak", "tensionStress", "compressionStress", "shearStress",
              "normalTorqueStress", "shearTorqueStress", "createBondAlways", "dampingBond",
              "dampingBondSmooth", "ratioTCBond")


def build(force=False):
    src = os.path.join(HERE, "dem_oracle.c")
    deps = [os.path.join(HERE, f) for f in os.listdir(HERE) if f.endswith((".c", ".h"))]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(map(os.path.getmtime, deps)):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp"
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", src,
                           "-o", tmp, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class OrcConfig(ctypes.Structure):
    _fields_ = [("boxlo", ctypes.c_double * 3), ("boxhi", ctypes.c_double * 3),
                ("periodic", ctypes.c_int * 3), ("dt", ctypes.c_double),
                ("skin", ctypes.c_double), ("contact_distance_factor", ctypes.c_double),
                ("neigh_every", ctypes.c_int), ("neigh_delay", ctypes.c_int),
                ("neigh_check", ctypes.c_int), ("normal_model", ctypes.c_int),
                ("rolling_model", ctypes.c_int), ("cohesion_model", ctypes.c_int),
                ("tangential_damping", ctypes.c_int), ("limit_force", ctypes.c_int),
                ("gravity_on", ctypes.c_int), ("gravity", ctypes.c_double * 3)]


class OrcBondSettings(ctypes.Structure):
    _fields_ = [("tsCreate", ctypes.c_double)] + [(k, ctypes.c_int) for k in BOND_FLAGS]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.POINTER(OrcConfig)]
        L.orc_destroy.argtypes = [P]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_last_error.argtypes = [P]
        L.orc_set_pair_params.argtypes = [P, ctypes.c_int] + [P] * 6 + [ctypes.c_double]
        L.orc_set_bond_params.argtypes = [P, P, ctypes.POINTER(OrcBondSettings)]
        L.orc_add_plane.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int]
        L.orc_add_cylinder.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int, ctypes.c_int]
        L.orc_set_atoms.argtypes = [P, ctypes.c_int] + [P] * 7
        L.orc_setup.argtypes = [P]
        L.orc_run.argtypes = [P, ctypes.c_int]
        for fn in ("orc_natoms", "orc_npairs", "orc_dnum"):
            getattr(L, fn).argtypes = [P]
        L.orc_nrebuilds.restype = ctypes.c_long
        L.orc_nrebuilds.argtypes = [P]
        L.orc_ntimestep.restype = ctypes.c_long
        L.orc_ntimestep.argtypes = [P]
        L.orc_get_atoms.argtypes = [P] + [P] * 9
        L.orc_get_pairs.argtypes = [P] + [P] * 5
        L.orc_get_wall_history.argtypes = [P, ctypes.c_int, P]
        L.orc_set_contact_history.argtypes = [P, ctypes.c_int, P, P, P]
        L.orc_set_wall_history.argtypes = [P, ctypes.c_int, P]
        L.orc_add_mesh.argtypes = [P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_get_mesh_flags.argtypes = [P, ctypes.c_int, P, P]
        L.orc_set_mesh_motion.argtypes = [P, ctypes.c_int] + [ctypes.c_double] * 3
        L.orc_get_mesh_nodes.argtypes = [P, ctypes.c_int, P]
        L.orc_set_mesh_rotation.argtypes = [P, ctypes.c_int, P, P, ctypes.c_double]
        L.orc_get_mesh_contacts.argtypes = [P, ctypes.c_int, P, P, P, P]
        L.orc_insert_atoms.argtypes = [P, ctypes.c_int] + [P] * 7
        L.orc_ncontacts.restype = ctypes.c_longlong
        L.orc_ncontacts.argtypes = [P]
        L.orc_get_wall_forces.argtypes = [P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


class Oracle:
    """One system of the CPU restatement; mirrors the GPU handle's methods."""

    def __init__(self, case):
        L = lib()
        c = OrcConfig()
        c.boxlo[:] = case["boxlo"]
        c.boxhi[:] = case["boxhi"]
        c.periodic[:] = case["periodic"]
        c.dt = case["dt"]
        c.skin = case["skin"]
        c.contact_distance_factor = case.get("cdf", 1.0)
        c.neigh_every, c.neigh_delay, c.neigh_check = case.get("neigh", (1, 0, 1))
        c.normal_model = case.get("normal_model", NORMAL_HERTZ)
        c.rolling_model = case.get("rolling_model", ROLLING_OFF)
        c.cohesion_model = case.get("cohesion_model", COHESION_OFF)
        c.tangential_damping = 1
        c.limit_force = 0
        g = case.get("gravity")
        c.gravity_on = 1 if g is not None else 0
        c.gravity[:] = g if g is not None else (0.0, 0.0, 0.0)
        self._keep = []
        self.h = L.orc_create(ctypes.byref(c))
        nt = int(case["ntypes"])
        tabs = []
        for k in ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRollFrict", "coeffRestLog"):
            a = np.ascontiguousarray(case[k], dtype=np.float64).reshape(nt + 1, nt + 1)
            tabs.append(a)
        self._keep += tabs
        L.orc_set_pair_params(self.h, nt, *[_p(a) for a in tabs], float(case.get("charVel", 0.0)))
        if c.cohesion_model == COHESION_BOND_NONLINEAR:
            b = case["bond"]
            bt = np.ascontiguousarray(b["tables"], dtype=np.float64)
            assert bt.shape == (23, nt + 1, nt + 1)
            st = OrcBondSettings()
            st.tsCreate = float(b["settings"]["tsCreate"])
            for k in BOND_FLAGS:
                setattr(st, k, int(b["settings"][k]))
            self._keep.append(bt)
            self._check(L.orc_set_bond_params(self.h, _p(bt), ctypes.byref(st)))
        for (axis, pos, wtype, roll) in case.get("planes", []):
            L.orc_add_plane(self.h, int(axis), float(pos), int(wtype), int(roll))
        for (axis, rad, c1, c2, wtype, roll) in case.get("cylinders", []):
            L.orc_add_cylinder(self.h, int(axis), float(rad), float(c1), float(c2), int(wtype), int(roll))
        self.nmesh = 0
        self._mesh_nodes = []
        for m in case.get("meshes", []):
            nodes = np.ascontiguousarray(m["nodes"], dtype=np.float64)
            ea = m.get("edge_active")
            ca = m.get("corner_active")
            ea = np.ascontiguousarray(ea, dtype=np.uint8) if ea is not None else None
            ca = np.ascontiguousarray(ca, dtype=np.uint8) if ca is not None else None
            self._keep += [nodes, ea, ca]
            self._mesh_nodes.append(nodes)
            self._check(L.orc_add_mesh(self.h, len(nodes), _p(nodes), int(m["wall_type"]),
                                       int(m.get("rolling", 0)), _p(ea), _p(ca)))
            if m.get("vel") is not None:
                self._check(L.orc_set_mesh_motion(self.h, self.nmesh, *[float(v) for v in m["vel"]]))
            if m.get("rotate") is not None:
                ro = m["rotate"]
                org = np.ascontiguousarray(ro["origin"], dtype=np.float64)
                axv = np.ascontiguousarray(ro["axis"], dtype=np.float64)
                self._keep += [org, axv]
                self._check(L.orc_set_mesh_rotation(self.h, self.nmesh, _p(org), _p(axv), float(ro["period"])))
            self.nmesh += 1
        a = case["atoms"]
        n = len(a["tag"])
        arrs = [np.ascontiguousarray(a[k], dtype=t) for k, t in
                (("tag", np.int32), ("type", np.int32), ("x", np.float64), ("v", np.float64),
                 ("omega", np.float64), ("radius", np.float64), ("rmass", np.float64))]
        L.orc_set_atoms(self.h, n, *[_p(x) for x in arrs])

    def set_restart(self, tag_owner, tag_partner, hist, wall_hist=()):
        """Contact/wall history as restored by read_restart (see dem_oracle.h)."""
        to = np.ascontiguousarray(tag_owner, dtype=np.int32)
        tp = np.ascontiguousarray(tag_partner, dtype=np.int32)
        h = np.ascontiguousarray(hist, dtype=np.float64)
        self._check(lib().orc_set_contact_history(self.h, len(to), _p(to), _p(tp), _p(h)))
        for w, wh in enumerate(wall_hist):
            wh = np.ascontiguousarray(wh, dtype=np.float64)
            self._check(lib().orc_set_wall_history(self.h, w, _p(wh)))

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(lib().orc_last_error(self.h).decode())

    def setup(self):
        self._check(lib().orc_setup(self.h))

    def run(self, n):
        self._check(lib().orc_run(self.h, int(n)))

    @property
    def nrebuilds(self):
        return lib().orc_nrebuilds(self.h)

    def atoms(self):
        L = lib()
        n = L.orc_natoms(self.h)
        out = dict(tag=np.zeros(n, np.int32), type=np.zeros(n, np.int32),
                   x=np.zeros((n, 3)), v=np.zeros((n, 3)), omega=np.zeros((n, 3)),
                   f=np.zeros((n, 3)), torque=np.zeros((n, 3)), radius=np.zeros(n),
                   rmass=np.zeros(n))
        L.orc_get_atoms(self.h, *[_p(out[k]) for k in
                                  ("tag", "type", "x", "v", "omega", "f", "torque", "radius", "rmass")])
        return out

    def pairs(self):
        L = lib()
        n = L.orc_npairs(self.h)
        d = L.orc_dnum(self.h)
        out = dict(tag_i=np.zeros(n, np.int32), tag_j=np.zeros(n, np.int32),
                   shift=np.zeros((n, 3), np.int32), flag=np.zeros(n, np.int32),
                   hist=np.zeros((n, d)))
        L.orc_get_pairs(self.h, *[_p(out[k]) for k in ("tag_i", "tag_j", "shift", "flag", "hist")])
        return out

    def mesh_flags(self, k):
        ntri = len(self._keep_mesh_nodes(k))
        ea = np.zeros((ntri, 3), np.uint8)
        ca = np.zeros((ntri, 3), np.uint8)
        lib().orc_get_mesh_flags(self.h, int(k), _p(ea), _p(ca))
        return ea, ca

    def _keep_mesh_nodes(self, k):
        return self._mesh_nodes[k]

    def mesh_nodes(self, k):
        nodes = np.zeros_like(self._keep_mesh_nodes(k))
        lib().orc_get_mesh_nodes(self.h, int(k), _p(nodes))
        return nodes

    def mesh_contacts(self, k):
        L = lib()
        n = L.orc_get_mesh_contacts(self.h, int(k), None, None, None, None)
        out = dict(tag=np.zeros(n, np.int32), tri=np.zeros(n, np.int32), slot=np.zeros(n, np.int32),
                   hist=np.zeros((n, 3)))
        L.orc_get_mesh_contacts(self.h, int(k), *[_p(out[q]) for q in ("tag", "tri", "slot", "hist")])
        return out

    def insert(self, a):
        """Atoms (dict as in the case's "atoms") that join at the next step."""
        arrs = [np.ascontiguousarray(a[k], dtype=t) for k, t in
                (("tag", np.int32), ("type", np.int32), ("x", np.float64), ("v", np.float64),
                 ("omega", np.float64), ("radius", np.float64), ("rmass", np.float64))]
        self._check(lib().orc_insert_atoms(self.h, len(arrs[0]), *[_p(x) for x in arrs]))

    def diagnostics(self):
        """Entries with a contact force and the per-wall total forces of the
        last force pass (planes, then meshes)."""
        L = lib()
        out = np.zeros((16, 3))
        nw = L.orc_get_wall_forces(self.h, _p(out))
        return dict(ncontacts=int(L.orc_ncontacts(self.h)), wall_force=out[:nw].copy())

    def wall_history(self, w):
        L = lib()
        n = L.orc_natoms(self.h)
        h = np.zeros((n, 3))
        L.orc_get_wall_history(self.h, int(w), _p(h))
        return h

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None
