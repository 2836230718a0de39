"""ctypes binding of the C ABI in include/liggghts_gb300.h (libdemgpu.so).

``DemSystem`` mirrors the reference's run semantics: ``setup()`` is
Verlet::setup (neighbour build + forces without history update) and
``step(n)`` runs n Verlet iterations.  It raises if the CUDA library is not
built or no GPU is present: there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

from . import build as _build

HEADER = os.path.join(os.path.dirname(_build.PKG), "include", "liggghts_gb300.h")

STATUS = {0: "DEM_OK", 1: "DEM_ERR_BAD_ARG", 2: "DEM_ERR_CUDA", 3: "DEM_ERR_NEIGH_OVERFLOW",
          4: "DEM_ERR_NAN", 5: "DEM_ERR_TIMEOUT", 6: "DEM_ERR_BOX", 7: "DEM_ERR_UNSUPPORTED",
          8: "DEM_ERR_NO_DEVICE", 9: "DEM_ERR_CAPACITY"}


def mesh_topology(nodes):
    """Edge/corner activity flags of a triangle mesh (host-only C++ of the library)."""
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    ea = np.zeros((len(nodes), 3), np.uint8)
    ca = np.zeros((len(nodes), 3), np.uint8)
    rc = load().dem_mesh_topology(len(nodes), _p(nodes), _p(ea), _p(ca))
    if rc != 0:
        raise DemError("dem_mesh_topology: %s" % STATUS.get(rc, rc))
    return ea, ca


class DemConfig(ctypes.Structure):
    _fields_ = [("boxlo", ctypes.c_double * 3), ("boxhi", ctypes.c_double * 3),
                ("periodic", ctypes.c_int * 3), ("dt", ctypes.c_double),
                ("skin", ctypes.c_double), ("contact_distance_factor", ctypes.c_double),
                ("neigh_every", ctypes.c_int), ("neigh_delay", ctypes.c_int),
                ("neigh_check", ctypes.c_int), ("normal_model", ctypes.c_int),
                ("rolling_model", ctypes.c_int), ("cohesion_model", ctypes.c_int),
                ("tangential_damping", ctypes.c_int), ("limit_force", ctypes.c_int),
                ("gravity_on", ctypes.c_int), ("gravity", ctypes.c_double * 3)]


# on/off settings of cohesion bond/nonlinear, dem_bond_settings order
BOND_FLAGS = ("stressBreak", "tensionStress", "compressionStress", "shearStress",
              "normalTorqueStress", "shearTorqueStress", "createBondAlways", "dampingBond",
              "dampingBondSmooth", "ratioTCBond")


class DemBondSettings(ctypes.Structure):
    _fields_ = [("tsCreate", ctypes.c_double)] + [(k, ctypes.c_int) for k in BOND_FLAGS]


class DemStats(ctypes.Structure):
    _fields_ = [("ntimestep", ctypes.c_longlong), ("nrebuilds", ctypes.c_longlong),
                ("npairs", ctypes.c_longlong), ("nlost", ctypes.c_longlong),
                ("natoms", ctypes.c_longlong), ("device", ctypes.c_int),
                ("pair_capacity", ctypes.c_int), ("last_step_ms", ctypes.c_double),
                ("host_direct", ctypes.c_int), ("mesh_slot_capacity", ctypes.c_int),
                ("ens_inplace_builds", ctypes.c_int), ("ens_relayout_builds", ctypes.c_int)]


class DemKernelTimes(ctypes.Structure):
    _fields_ = [("pair_ms", ctypes.c_double), ("pair_launches", ctypes.c_longlong),
                ("particle_ms", ctypes.c_double), ("particle_launches", ctypes.c_longlong),
                ("neigh_ms", ctypes.c_double), ("neigh_stages", ctypes.c_longlong),
                ("kernel_launches", ctypes.c_longlong), ("wall_ms", ctypes.c_double),
                ("wall_launches", ctypes.c_longlong)]


class DemDiagnostics(ctypes.Structure):
    _fields_ = [("ke_translational", ctypes.c_double), ("ke_rotational", ctypes.c_double),
                ("ncontacts", ctypes.c_longlong), ("solid_volume", ctypes.c_double),
                ("packing_fraction", ctypes.c_double), ("nwalls", ctypes.c_int),
                ("wall_force", (ctypes.c_double * 3) * 16)]


_lib = None
P = ctypes.c_void_p


def load(build=True):
    """Loads libdemgpu.so (building it first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    L = ctypes.CDLL(path)
    I = ctypes.c_int
    L.dem_create.argtypes = [ctypes.POINTER(DemConfig), ctypes.POINTER(P)]
    L.dem_destroy.argtypes = [P]
    L.dem_set_pair_params.argtypes = [P, I] + [P] * 6 + [ctypes.c_double]
    L.dem_set_bond_params.argtypes = [P, P, ctypes.POINTER(DemBondSettings)]
    L.dem_derive_hertz_tables.argtypes = [I] + [P] * 7
    L.dem_add_plane.argtypes = [P, I, ctypes.c_double, I, I, P]
    L.dem_add_cylinder.argtypes = [P, I, ctypes.c_double, ctypes.c_double, ctypes.c_double, I, I, P]
    L.dem_add_plane_per_type.argtypes = [P, I, P, I, P]
    L.dem_set_tuning.argtypes = [P, I, ctypes.c_double]
    L.dem_set_particle_threads.argtypes = [P, I]
    L.dem_set_ensemble.argtypes = [P, I]
    L.dem_ensemble_rebuilds.argtypes = [P, P]
    L.dem_upload_atoms.argtypes = [P, I] + [P] * 7
    L.dem_add_mesh.argtypes = [P, I, P, I, I, P, P, P]
    L.dem_mesh_topology.argtypes = [I, P, P, P]
    L.dem_mesh_ncontacts.argtypes = [P, I, P]
    L.dem_set_mesh_motion.argtypes = [P, I, P]
    L.dem_set_mesh_rotation.argtypes = [P, I, P, P, ctypes.c_double]
    L.dem_download_mesh_nodes.argtypes = [P, I, P]
    L.dem_download_mesh_contacts.argtypes = [P, I, P, P, P, P]
    L.dem_upload_contact_history.argtypes = [P, I, P, P, P]
    L.dem_upload_wall_history.argtypes = [P, I, P]
    L.dem_setup.argtypes = [P]
    L.dem_step.argtypes = [P, I]
    L.dem_natoms.argtypes = [P, P]
    L.dem_download_atoms.argtypes = [P] + [P] * 9
    L.dem_npairs.argtypes = [P, P, P]
    L.dem_download_contacts.argtypes = [P] + [P] * 5
    L.dem_download_wall_history.argtypes = [P, I, P]
    L.dem_get_stats.argtypes = [P, ctypes.POINTER(DemStats)]
    L.dem_last_error.argtypes = [P]
    L.dem_last_error.restype = ctypes.c_char_p
    L.dem_version.restype = ctypes.c_char_p
    L.dem_profile.argtypes = [P, I]
    L.dem_get_kernel_times.argtypes = [P, ctypes.POINTER(DemKernelTimes)]
    L.dem_measure_fp64_peak.argtypes = [ctypes.POINTER(ctypes.c_double)]
    L.dem_get_diagnostics.argtypes = [P, P, P, ctypes.POINTER(DemDiagnostics)]
    L.dem_set_capacity.argtypes = [P, I, ctypes.c_double, ctypes.c_double]
    L.dem_insert_atoms.argtypes = [P, I] + [P] * 7
    _lib = L
    return L


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    v = ctypes.c_double()
    rc = load().dem_measure_fp64_peak(ctypes.byref(v))
    if rc != 0:
        raise DemError("dem_measure_fp64_peak: %s" % STATUS.get(rc, rc))
    return v.value


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


class DemError(RuntimeError):
    pass


class DemSystem:
    """One resident granular system on the GPU (one C-ABI handle)."""

    def __init__(self, case):
        L = load()
        c = DemConfig()
        c.boxlo[:] = case["boxlo"]
        c.boxhi[:] = case["boxhi"]
        c.periodic[:] = case["periodic"]
        c.dt = case["dt"]
        c.skin = case["skin"]
        c.contact_distance_factor = case.get("cdf", 1.0)
        c.neigh_every, c.neigh_delay, c.neigh_check = case.get("neigh", (1, 0, 1))
        c.normal_model = case.get("normal_model", 0)
        c.rolling_model = case.get("rolling_model", 0)
        c.cohesion_model = case.get("cohesion_model", 0)
        c.tangential_damping = 1
        c.limit_force = 0
        g = case.get("gravity")
        c.gravity_on = 1 if g is not None else 0
        c.gravity[:] = g if g is not None else (0.0, 0.0, 0.0)
        h = P()
        rc = L.dem_create(ctypes.byref(c), ctypes.byref(h))
        if rc != 0:
            raise DemError("dem_create: %s" % STATUS.get(rc, rc))
        self.h = h
        nt = int(case["ntypes"])
        tabs = [np.ascontiguousarray(case[k], dtype=np.float64).reshape(nt + 1, nt + 1)
                for k in ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRollFrict", "coeffRestLog")]
        self._check(L.dem_set_pair_params(self.h, nt, *[_p(a) for a in tabs],
                                          float(case.get("charVel", 0.0))))
        if c.cohesion_model == 1:
            b = case["bond"]
            bt = np.ascontiguousarray(b["tables"], dtype=np.float64)
            assert bt.shape == (23, nt + 1, nt + 1)
            st = DemBondSettings()
            st.tsCreate = float(b["settings"]["tsCreate"])
            for k in BOND_FLAGS:
                setattr(st, k, int(b["settings"][k]))
            self._check(L.dem_set_bond_params(self.h, _p(bt), ctypes.byref(st)))
        for (axis, pos, wtype, roll) in case.get("planes", []):
            self._check(L.dem_add_plane(self.h, int(axis), float(pos), int(wtype), int(roll), None))
        for (axis, rad, c1, c2, wtype, roll) in case.get("cylinders", []):
            self._check(L.dem_add_cylinder(self.h, int(axis), float(rad), float(c1), float(c2), int(wtype),
                                           int(roll), None))
        for (axis, pos_t, roll) in case.get("planes_per_type", []):
            pt = np.ascontiguousarray(pos_t, dtype=np.float64)
            self._check(L.dem_add_plane_per_type(self.h, int(axis), _p(pt), int(roll), None))
        if case.get("tuning") is not None:
            bps, cs = case["tuning"][0], case["tuning"][1]
            self._check(L.dem_set_tuning(self.h, int(bps), float(cs)))
            if len(case["tuning"]) > 2 and case["tuning"][2] is not None:
                self._check(L.dem_set_particle_threads(self.h, int(case["tuning"][2])))
        if case.get("ensemble"):
            self._check(L.dem_set_ensemble(self.h, int(case["ensemble"])))
        self._meshkeep = []
        self._nodes_shape = []
        for m in case.get("meshes", []):
            nodes = np.ascontiguousarray(m["nodes"], dtype=np.float64)
            ea, ca = m.get("edge_active"), m.get("corner_active")
            ea = np.ascontiguousarray(ea, dtype=np.uint8) if ea is not None else None
            ca = np.ascontiguousarray(ca, dtype=np.uint8) if ca is not None else None
            self._meshkeep += [nodes, ea, ca]
            self._check(L.dem_add_mesh(self.h, len(nodes), _p(nodes), int(m["wall_type"]),
                                       int(m.get("rolling", 0)), _p(ea), _p(ca), None))
            if m.get("vel") is not None:
                vel = np.ascontiguousarray(m["vel"], dtype=np.float64)
                self._check(L.dem_set_mesh_motion(self.h, len(self._meshkeep) // 3 - 1, _p(vel)))
            if m.get("rotate") is not None:
                ro = m["rotate"]
                org = np.ascontiguousarray(ro["origin"], dtype=np.float64)
                axv = np.ascontiguousarray(ro["axis"], dtype=np.float64)
                self._check(L.dem_set_mesh_rotation(self.h, len(self._meshkeep) // 3 - 1, _p(org), _p(axv),
                                                    float(ro["period"])))
            self._nodes_shape.append(nodes.shape)
        if case.get("capacity") is not None:  # (natoms_max, rmin, rmax) for later insertions
            nmax_, rmin_, rmax_ = case["capacity"]
            self._check(L.dem_set_capacity(self.h, int(nmax_), float(rmin_), float(rmax_)))
        if "atoms" in case:
            self.upload(case["atoms"])

    def _check(self, rc):
        if rc != 0:
            msg = load().dem_last_error(self.h).decode() if getattr(self, "h", None) else ""
            raise DemError("%s: %s" % (STATUS.get(rc, rc), msg))

    def upload(self, a):
        n = len(a["tag"])
        arrs = [np.ascontiguousarray(a[k], dtype=t) for k, t in
                (("tag", np.int32), ("type", np.int32), ("x", np.float64), ("v", np.float64),
                 ("omega", np.float64), ("radius", np.float64), ("rmass", np.float64))]
        self._check(load().dem_upload_atoms(self.h, n, *[_p(x) for x in arrs]))

    def insert(self, a):
        """dem_insert_atoms: atoms (dict as in the case's "atoms") that join
        at the next step after its initial integration."""
        arrs = [np.ascontiguousarray(a[k], dtype=t) for k, t in
                (("tag", np.int32), ("type", np.int32), ("x", np.float64), ("v", np.float64),
                 ("omega", np.float64), ("radius", np.float64), ("rmass", np.float64))]
        self._check(load().dem_insert_atoms(self.h, len(arrs[0]), *[_p(x) for x in arrs]))

    def set_restart(self, tag_owner, tag_partner, hist, wall_hist=()):
        """Restart contact/wall history (between upload and setup)."""
        to = np.ascontiguousarray(tag_owner, dtype=np.int32)
        tp = np.ascontiguousarray(tag_partner, dtype=np.int32)
        h = np.ascontiguousarray(hist, dtype=np.float64)
        self._check(load().dem_upload_contact_history(self.h, len(to), _p(to), _p(tp), _p(h)))
        for w, wh in enumerate(wall_hist):
            wh = np.ascontiguousarray(wh, dtype=np.float64)
            self._check(load().dem_upload_wall_history(self.h, w, _p(wh)))

    def setup(self):
        self._check(load().dem_setup(self.h))

    def step(self, n):
        self._check(load().dem_step(self.h, int(n)))

    run = step

    def natoms(self):
        n = ctypes.c_int()
        self._check(load().dem_natoms(self.h, ctypes.byref(n)))
        return n.value

    @staticmethod
    def atom_buffers(n):
        """Host arrays for atoms(out=...): the caller's own per-atom arrays,
        kept across calls as the reference keeps atom->x, atom->v, ..."""
        out = dict(tag=np.empty(n, np.int32), type=np.empty(n, np.int32),
                   x=np.empty((n, 3)), v=np.empty((n, 3)), omega=np.empty((n, 3)),
                   f=np.empty((n, 3)), torque=np.empty((n, 3)), radius=np.empty(n),
                   rmass=np.empty(n))
        for a in out.values():  # written once, so the pages exist (np.zeros maps them lazily)
            a.fill(0)
        return out

    def atoms(self, out=None):
        """dem_download_atoms into `out` (atom_buffers of at least natoms()
        rows; new arrays when None or too small); returns the first natoms()
        rows of each array, in the device's order."""
        n = self.natoms()
        if out is None or len(out["tag"]) < n:
            out = self.atom_buffers(n)
        keys = ("tag", "type", "x", "v", "omega", "f", "torque", "radius", "rmass")
        for k in keys:
            a = out[k]
            assert a.flags.c_contiguous and a.dtype == (np.int32 if k in ("tag", "type") else np.float64)
        self._check(load().dem_download_atoms(self.h, *[_p(out[k]) for k in keys]))
        return {k: out[k][:n] for k in keys}

    def pairs(self):
        L = load()
        n, d = ctypes.c_int(), ctypes.c_int()
        self._check(L.dem_npairs(self.h, ctypes.byref(n), ctypes.byref(d)))
        n, d = n.value, d.value
        out = dict(tag_i=np.zeros(n, np.int32), tag_j=np.zeros(n, np.int32),
                   shift=np.zeros((n, 3), np.int32), flag=np.zeros(n, np.int32),
                   hist=np.zeros((n, d)))
        self._check(L.dem_download_contacts(self.h, *[_p(out[k]) for k in
                                                      ("tag_i", "tag_j", "shift", "flag", "hist")]))
        return out

    def mesh_nodes(self, k):
        nodes = np.zeros(self._nodes_shape[k])
        self._check(load().dem_download_mesh_nodes(self.h, int(k), _p(nodes)))
        return nodes

    def mesh_contacts(self, k):
        L = load()
        n = ctypes.c_int()
        self._check(L.dem_mesh_ncontacts(self.h, int(k), ctypes.byref(n)))
        n = n.value
        out = dict(tag=np.zeros(n, np.int32), tri=np.zeros(n, np.int32), slot=np.zeros(n, np.int32),
                   hist=np.zeros((n, 3)))
        self._check(L.dem_download_mesh_contacts(self.h, int(k), *[_p(out[q]) for q in
                                                                  ("tag", "tri", "slot", "hist")]))
        return out

    def wall_history(self, w):
        h = np.zeros((self.natoms(), 3))
        self._check(load().dem_download_wall_history(self.h, int(w), _p(h)))
        return h

    def diagnostics(self, region=None):
        """dem_get_diagnostics: kinetic energies, contact count, solid volume
        and packing fraction of the atoms centred in region=(lo, hi) (None:
        the box), per-wall total forces of the last force pass."""
        d = DemDiagnostics()
        lo = hi = None
        if region is not None:
            lo = np.ascontiguousarray(region[0], dtype=np.float64)
            hi = np.ascontiguousarray(region[1], dtype=np.float64)
        self._check(load().dem_get_diagnostics(self.h, _p(lo), _p(hi), ctypes.byref(d)))
        wf = np.array([[d.wall_force[w][k] for k in range(3)] for w in range(d.nwalls)]).reshape(-1, 3)
        return dict(ke_translational=d.ke_translational, ke_rotational=d.ke_rotational,
                    ncontacts=int(d.ncontacts), solid_volume=d.solid_volume,
                    packing_fraction=d.packing_fraction, wall_force=wf)

    def stats(self):
        s = DemStats()
        self._check(load().dem_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in DemStats._fields_}

    def profile(self, enable=True):
        self._check(load().dem_profile(self.h, 1 if enable else 0))

    def kernel_times(self):
        t = DemKernelTimes()
        self._check(load().dem_get_kernel_times(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in DemKernelTimes._fields_}

    @property
    def nrebuilds(self):
        return self.stats()["nrebuilds"]

    def close(self):
        if getattr(self, "h", None):
            load().dem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
