"""The adjoint's per-pair laws against finite differences, on the CPU.

tests/adjoint_vjp_check.cpp compiles the device headers of the adjoint
(adjoint_law.cuh: Hertz + tangential history, with and without CDT rolling,
for pairs, walls and bonded pairs; adjoint_bond.cuh: cohesion bond/nonlinear) for the host and
compares each vector-Jacobian product with a fourth-order central difference
of the forward law along random directions of all inputs (positions,
velocities, spins, history, radii, masses, material parameters).  Cases
whose branch decisions change within the difference stencil are skipped
(the law has no derivative there) and counted.
"""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "liggghts-inl_gb300", "csrc")
CUDA_INC = "/usr/local/cuda/include"

VJP_RTOL = 1e-6  # directional derivative vs fourth-order central difference

# kBond* bits (liggghts-inl_gb300/csrc/dem_device.cuh)
STRESS, TENSION, COMPRESSION, SHEAR, TWIST, BEND, CREATE_ALWAYS, DAMP, SMOOTH = (1 << k for k in range(9))
ALL_LAWS = TENSION | COMPRESSION | SHEAR | TWIST | BEND


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    if shutil.which("g++") is None or not os.path.isfile(os.path.join(CUDA_INC, "vector_types.h")):
        pytest.skip("g++ or the CUDA headers not available")
    out = str(tmp_path_factory.mktemp("vjp") / "libvjpcheck.so")
    cmd = ["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-D__device__=", "-D__forceinline__=inline",
           "-I" + CSRC, "-I" + CUDA_INC, os.path.join(ROOT, "tests", "adjoint_vjp_check.cpp"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = ctypes.CDLL(out)
    L.check_law.restype = ctypes.c_double
    L.check_law.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.POINTER(ctypes.c_int)]
    L.check_bond.restype = ctypes.c_double
    L.check_bond.argtypes = [ctypes.c_uint64, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_int)]
    return L


@pytest.mark.parametrize("kind", [0, 1, 2], ids=["pair", "wall", "bonded_pair"])
@pytest.mark.parametrize("upd", [0, 1], ids=["setup_pass", "history_update"])
@pytest.mark.parametrize("rolling", [0, 1], ids=["no_rolling", "cdt_rolling"])
def test_contact_law_vjp(lib, kind, upd, rolling):
    c = (ctypes.c_int * 3)()
    n = 2000
    err = lib.check_law(11, n, kind, upd, rolling, c)
    assert c[0] > n // 10 and c[1] > n // 10, "both sticking and sliding contacts must be covered"
    assert c[2] < n // 50
    assert err < VJP_RTOL, err


BOND_SETS = {
    "all_laws": ALL_LAWS,
    "sign_damping": ALL_LAWS | DAMP,
    "smooth_damping": ALL_LAWS | DAMP | SMOOTH,
    "stress_breakage": ALL_LAWS | STRESS,
    "normal_only": TENSION | COMPRESSION,
}


@pytest.mark.parametrize("name", sorted(BOND_SETS))
@pytest.mark.parametrize("mode", ["existing_setup_pass", "existing", "created"])
def test_bond_vjp(lib, name, mode):
    flags = BOND_SETS[name]
    create = 1 if mode == "created" else 0
    upd = 0 if mode == "existing_setup_pass" else 1
    b = (ctypes.c_int * 12)()
    n = 3000
    err = lib.check_bond(7, n, flags, create, upd, b)
    assert b[11] < n // 50, "too many cases at a branch switch"
    assert err < VJP_RTOL, err
    if not create:
        # the piecewise normal law: every reachable branch (the first one,
        # disp below the running minimum, cannot occur once the minimum has
        # been updated with disp)
        assert all(b[k] > 0 for k in range(1, 6)), list(b)
        if flags & (TWIST | BEND):
            assert all(b[k] > 0 for k in range(6, 10)), list(b)
        if flags & STRESS and upd:
            assert n // 10 < b[10] < n - n // 10, list(b)
