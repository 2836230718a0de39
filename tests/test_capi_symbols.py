"""CPU checks of the drop-in boundary: the C-ABI library builds/loads and
exports every entry point include/liggghts_gb300.h declares; without a GPU
it fails loudly (no CPU fallback)."""
import ctypes
import os
import re

from gb300dem import api, workloads

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    out = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            out += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(dem_\w+)\s*\(", txt, re.M)
    return sorted(set(out))


def test_library_exports_every_declared_symbol():
    L = api.load()
    syms = declared_symbols()
    assert "dem_step" in syms and "dem_create" in syms
    for s in syms:
        assert hasattr(L, s), s


def test_no_device_is_an_error_not_a_fallback():
    try:
        import torch
        if torch.cuda.is_available():
            return
    except Exception:
        pass
    L = api.load()
    h = api.P()
    c = api.DemConfig()
    c.dt, c.skin, c.contact_distance_factor, c.neigh_every = 1e-6, 5e-4, 1.0, 1
    rc = L.dem_create(ctypes.byref(c), ctypes.byref(h))
    assert rc == 8  # DEM_ERR_NO_DEVICE


def test_library_mesh_topology_matches_reference_flags():
    """Edge/corner activity derived by the library's host code (used when a
    caller uploads a bare mesh) equals the reference's own flags."""
    import numpy as np
    from golden_io import load_golden
    for name in ("hopper_mesh", "hopper_mesh_cdt"):
        case, snaps = load_golden(name)
        ea, ca = api.mesh_topology(case["meshes"][0]["nodes"])
        assert np.array_equal(ea, snaps[0]["mesh0_edge_active"]), name
        assert np.array_equal(ca, snaps[0]["mesh0_corner_active"]), name


def test_host_table_derivation_matches_reference_formulas():
    L = api.load()
    E = [5e6, 1e7]
    nu = [0.45, 0.3]
    e = [[0.9, 0.7], [0.7, 0.5]]
    ref = workloads.derive_tables(E, nu, e, [[0.5, 0.4], [0.4, 0.6]])
    import numpy as np
    Y, G, B, R = (np.zeros((3, 3)) for _ in range(4))
    Ea, nua, ea = (np.ascontiguousarray(a, dtype=np.float64) for a in (E, nu, e))
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    assert L.dem_derive_hertz_tables(2, p(Ea), p(nua), p(ea), p(Y), p(G), p(B), p(R)) == 0
    assert np.array_equal(Y, ref["Yeff"]) and np.array_equal(G, ref["Geff"])
    assert np.array_equal(B, ref["betaeff"]) and np.array_equal(R, ref["coeffRestLog"])
