"""dem_contact_forces_noalloc: the contact-force entry point that allocates
nothing on the device, for callers that cannot call cudaMalloc while they run
(their GPU memory belongs to another allocator or pool, or their loop must not
allocate after start-up).

The test owns every device buffer (allocated here through torch, standing in
for the caller's own allocator), calls the entry point through the C ABI twice
in a row, and checks both results against the forces of the existing resident
path (dem_setup on the same state, no gravity, no walls) within the force
tolerance the parity tests use.  The second call also checks that the shared
scratch array left by the first call does not leak into the next result.
"""
import ctypes

import numpy as np
import pytest

from golden_io import FORCE_RTOL, max_rel

pytestmark = pytest.mark.gpu


def _case():
    from gb300dem import workloads
    case = workloads.lattice_case(seed=17, nx=16, ny=16, nz=8, spacing=1.97e-3,
                                  radius=(0.9e-3, 1.05e-3), z0=1.0e-3, jitter=3e-5, vmax=1.5,
                                  wmax=100.0, rolling_model=1, rollfrict=((0.3,),),
                                  gravity=None, plane_z=None)
    return case


def test_noalloc_matches_resident_setup_forces_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gb300dem import api
    case = _case()
    g = api.DemSystem(case)
    g.setup()                      # forces of the setup pass: pair contacts only here
    a = g.atoms()                  # device order, with tags
    pr = g.pairs()                 # list order (owner-sorted), tags
    n, npairs = len(a["tag"]), len(pr["tag_i"])
    assert 0 < npairs <= 131072 and n <= 32768
    idx = {int(t): k for k, t in enumerate(a["tag"])}
    pi = np.array([idx[int(t)] for t in pr["tag_i"]], np.int32)
    pj = np.array([idx[int(t)] for t in pr["tag_j"]], np.int32)
    assert np.all(np.diff(pi) >= 0)

    dev = torch.device("cuda:0")
    T = lambda arr, dt: torch.as_tensor(np.ascontiguousarray(arr), dtype=dt, device=dev)  # noqa: E731
    bufs = dict(x=T(a["x"], torch.float64), v=T(a["v"], torch.float64),
                omega=T(a["omega"], torch.float64), radius=T(a["radius"], torch.float64),
                rmass=T(a["rmass"], torch.float64), type=T(a["type"], torch.int32),
                pi=T(pi, torch.int32), pj=T(pj, torch.int32), shift=T(pr["shift"], torch.int32),
                hist=T(pr["hist"], torch.float64))
    f = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    t = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()

    L = api.load()
    P = ctypes.c_void_p
    L.dem_contact_forces_noalloc.argtypes = ([ctypes.c_int] + [P] * 6 + [ctypes.c_int] + [P] * 4
                                             + [ctypes.POINTER(api.DemConfig), ctypes.c_int]
                                             + [P] * 6 + [ctypes.c_double, P, P, P])
    cfg = api.DemConfig()
    cfg.boxlo[:] = case["boxlo"]
    cfg.boxhi[:] = case["boxhi"]
    cfg.periodic[:] = case["periodic"]
    cfg.dt, cfg.skin, cfg.contact_distance_factor = case["dt"], case["skin"], 1.0
    cfg.neigh_every, cfg.neigh_delay, cfg.neigh_check = 1, 0, 1
    cfg.normal_model, cfg.rolling_model = case["normal_model"], case["rolling_model"]
    cfg.tangential_damping, cfg.limit_force = 1, 0
    nt = case["ntypes"]
    tabs = [np.ascontiguousarray(case[k], dtype=np.float64).reshape(nt + 1, nt + 1)
            for k in ("Yeff", "Geff", "betaeff", "coeffFrict", "coeffRollFrict", "coeffRestLog")]
    dp = lambda k: P(bufs[k].data_ptr())  # noqa: E731
    hp = lambda arr: arr.ctypes.data_as(P)  # noqa: E731

    def call():
        f.fill_(np.nan)
        t.fill_(np.nan)
        torch.cuda.synchronize()
        rc = L.dem_contact_forces_noalloc(
            n, dp("x"), dp("v"), dp("omega"), dp("radius"), dp("rmass"), dp("type"), npairs,
            dp("pi"), dp("pj"), dp("shift"), dp("hist"), ctypes.byref(cfg), nt,
            *[hp(tb) for tb in tabs], float(case.get("charVel", 0.0)),
            P(f.data_ptr()), P(t.data_ptr()), None)
        assert rc == 0, api.STATUS.get(rc, rc)
        return f.cpu().numpy().copy(), t.cpu().numpy().copy()

    for _ in range(2):
        fo, to = call()
        assert np.all(np.isfinite(fo)) and np.all(np.isfinite(to))
        assert max_rel(fo, a["f"]) < FORCE_RTOL
        assert max_rel(to, a["torque"]) < FORCE_RTOL
    g.close()
