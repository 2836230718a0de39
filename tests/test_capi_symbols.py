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


def test_ctypes_structures_match_the_header_layout(tmp_path):
    """Every struct of include/liggghts_gb300.h that the ctypes binding
    mirrors has the header's size and field offsets: a C program built with
    gcc from the header prints them, field names taken from the binding."""
    import shutil
    import subprocess
    from gb300dem import adjoint
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        import pytest
        pytest.skip("no C compiler")
    mirrors = {"dem_config": api.DemConfig, "dem_bond_settings": api.DemBondSettings,
               "dem_stats": api.DemStats, "dem_kernel_times": api.DemKernelTimes,
               "dem_diagnostics": api.DemDiagnostics, "dem_adjoint_config": adjoint.DemAdjointConfig,
               "dem_adjoint_loss": adjoint.DemAdjointLoss}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "liggghts_gb300.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('  printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('  printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                        check=True).stdout.splitlines())
    for cname, py in mirrors.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got["%s.%s" % (cname, fname)]) == getattr(py, fname).offset, (cname, fname)
