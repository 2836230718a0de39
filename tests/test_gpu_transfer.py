"""Atom transfer through the C ABI (dem_upload_atoms, dem_download_atoms).

The caller's per-atom arrays (the reference's atom->x[i][d] layout) go to the
device unchanged; one kernel transposes them into the device's SoA state,
forms FixNVESphere's per-atom factors and checks every atom; download is the
mirror image.  Where the GPU reaches pageable host memory through the host
page tables the kernels read and write the caller's arrays in place, else the
arrays pass through device staging copies (LIGGGHTS_GB300_STAGED_COPIES=1
forces those).  Both paths must give the same bits, and bad input must come
back as a status, never as a fault or a silent fallback.
"""
import numpy as np
import pytest

from golden_io import load_golden

pytestmark = pytest.mark.gpu


def _sys(case, staged, monkeypatch):
    from gb300dem.api import DemSystem
    if staged:
        monkeypatch.setenv("LIGGGHTS_GB300_STAGED_COPIES", "1")
    else:
        monkeypatch.delenv("LIGGGHTS_GB300_STAGED_COPIES", raising=False)
    g = DemSystem(case)
    monkeypatch.delenv("LIGGGHTS_GB300_STAGED_COPIES", raising=False)
    return g


@pytest.mark.parametrize("staged", [False, True])
def test_upload_download_round_trip(staged, monkeypatch):
    """Before any rebuild the device holds the atoms in upload order: the
    download returns the uploaded arrays bit for bit, forces zero."""
    case, _ = load_golden("poly_cdt")
    g = _sys(case, staged, monkeypatch)
    if staged:
        assert g.stats()["host_direct"] == 0
    a = case["atoms"]
    out = g.atoms()
    for k in ("tag", "type", "x", "v", "omega", "radius", "rmass"):
        assert np.array_equal(out[k], a[k]), k
    assert not np.any(out["f"]) and not np.any(out["torque"])
    g.close()


def test_direct_and_staged_transfers_give_identical_runs(monkeypatch):
    case, _ = load_golden("hopper_mesh_cdt")
    res = []
    for staged in (False, True):
        g = _sys(case, staged, monkeypatch)
        g.setup()
        g.step(37)
        buf = g.atom_buffers(len(case["atoms"]["tag"]) + 5)
        res.append({k: v.copy() for k, v in g.atoms(buf).items()})
        g.close()
    for k in res[0]:
        assert np.array_equal(res[0][k], res[1][k]), k


def _bad(case, field, idx, value):
    c = dict(case)
    c["atoms"] = {k: v.copy() for k, v in case["atoms"].items()}
    c["atoms"][field][idx] = value
    return c


@pytest.mark.parametrize("staged", [False, True])
@pytest.mark.parametrize("field,idx,value,status", [
    ("x", (17, 1), np.nan, "DEM_ERR_NAN"),
    ("v", (3, 2), np.inf, "DEM_ERR_NAN"),
    ("omega", (40, 0), -np.inf, "DEM_ERR_NAN"),
    ("type", 9, 0, "DEM_ERR_BAD_ARG"),
    ("type", 9, 3, "DEM_ERR_BAD_ARG"),
    ("radius", 11, 0.0, "DEM_ERR_BAD_ARG"),
    ("rmass", 12, np.nan, "DEM_ERR_BAD_ARG"),
])
def test_upload_rejects_bad_atoms(field, idx, value, status, staged, monkeypatch):
    """A non-finite position, velocity or angular velocity is DEM_ERR_NAN; a
    type outside 1..ntypes or a radius/mass that is not finite and positive
    is DEM_ERR_BAD_ARG; the handle stays usable (a good upload follows)."""
    from gb300dem.api import DemError
    case, _ = load_golden("poly_cdt")
    g = _sys(case, staged, monkeypatch)
    with pytest.raises(DemError, match=status):
        g.upload(_bad(case, field, idx, value)["atoms"])
    with pytest.raises(DemError, match="DEM_ERR_BAD_ARG"):
        g.setup()
    g.upload(case["atoms"])
    g.setup()
    g.step(5)
    assert np.all(np.isfinite(g.atoms()["x"]))
    g.close()


def test_download_of_some_arrays_over_several_tiles():
    """The download kernel writes each 3-vector through a shared-memory tile
    of 256 atoms.  A caller may pass null for arrays it does not want: those
    are left alone and the others come back as in the full download (700
    atoms after 25 steps with rebuilds: three tiles, the last one partial)."""
    import ctypes
    from gb300dem import api, workloads
    case = workloads.lattice_case(seed=3, nx=10, ny=10, nz=7, spacing=1.97e-3, radius=(0.9e-3, 1.05e-3),
                                  z0=1.0e-3, jitter=3e-5, vmax=1.0, wmax=80.0)
    g = api.DemSystem(case)
    g.setup()
    g.step(25)
    full = {k: v.copy() for k, v in g.atoms().items()}
    n = g.natoms()
    assert n == 700
    keys = ("tag", "type", "x", "v", "omega", "f", "torque", "radius", "rmass")
    L = api.load()
    for sel in (("x", "f"), ("v", "torque", "radius"), ("omega", "tag", "rmass", "type"), ()):
        out = {k: np.full_like(full[k], -7) for k in keys}
        ptrs = [out[k].ctypes.data_as(ctypes.c_void_p) if k in sel else None for k in keys]
        assert L.dem_download_atoms(g.h, *ptrs) == 0
        for k in keys:
            if k in sel:
                assert np.array_equal(out[k], full[k]), (sel, k)
            else:
                assert np.all(out[k] == -7), (sel, k)
    g.close()
