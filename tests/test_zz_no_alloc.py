"""dem_contact_forces_noalloc: the contact-force entry point that allocates
nothing on the device, for callers that cannot call cudaMalloc while they run
(their GPU memory belongs to another allocator or pool, or their loop must not
allocate after start-up).

The state carries real tangential history: a lattice is run for 60 steps on
the resident path, and its atoms and contact histories become restart data.
The test owns every device buffer (allocated here through torch, standing in
for the caller's own allocator), calls the entry point through the C ABI twice
in a row, and checks both results within the force tolerance of the parity
tests against
  * the existing resident path (dem_setup from the same restart data: the
    setup force pass, history read and not updated, no gravity, no walls),
  * the oracle's setup pass from the same restart data,
for Hertz with CDT rolling and for Hooke.  The second call also checks that
the shared scratch array left by the first call does not leak into the next
result, and that it takes no device memory (the first call loaded the module
that holds the array).
"""
import ctypes

import numpy as np
import pytest

from golden_io import FORCE_RTOL, max_rel, sort_by_tag

pytestmark = pytest.mark.gpu


def _case(model):
    from gb300dem import workloads
    kw = dict(rolling_model=1, rollfrict=((0.3,),)) if model == "hertz" else dict(normal_model=1, charVel=0.5)
    return workloads.lattice_case(seed=17, nx=16, ny=16, nz=8, spacing=1.97e-3,
                                  radius=(0.9e-3, 1.05e-3), z0=1.0e-3, jitter=3e-5, vmax=1.5,
                                  wmax=100.0, gravity=None, plane_z=None, **kw)


@pytest.mark.parametrize("model", ["hertz", "hooke"])
def test_noalloc_matches_resident_and_oracle_twice(model):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from gb300dem import api, workloads
    from oracle.binding import Oracle
    case = _case(model)
    g0 = api.DemSystem(case)
    g0.setup()
    g0.step(60)                    # contacts build up tangential history
    ck, to, tp, hh, walls = workloads.restart_state(g0, case)
    g0.close()
    g = api.DemSystem(ck)
    g.set_restart(to, tp, hh, walls)
    g.setup()                      # setup pass on the restart state: pair contacts only here
    o = Oracle(ck)
    o.set_restart(to, tp, hh, walls)
    o.setup()
    a = g.atoms()                  # device order, with tags
    pr = g.pairs()                 # list order (owner-sorted), tags
    n, npairs = len(a["tag"]), len(pr["tag_i"])
    assert 0 < npairs <= 131072 and n <= 32768
    assert pr["hist"].shape[1] == 3 and np.count_nonzero(np.any(pr["hist"] != 0, axis=1)) > 100
    idx = {int(t): k for k, t in enumerate(a["tag"])}
    pi = np.array([idx[int(t)] for t in pr["tag_i"]], np.int32)
    pj = np.array([idx[int(t)] for t in pr["tag_j"]], np.int32)
    assert np.all(np.diff(pi) >= 0)
    ob = sort_by_tag(o.atoms())
    order = np.argsort(a["tag"], kind="stable")
    assert np.array_equal(a["tag"][order], ob["tag"])

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
    cfg.boxlo[:] = ck["boxlo"]
    cfg.boxhi[:] = ck["boxhi"]
    cfg.periodic[:] = ck["periodic"]
    cfg.dt, cfg.skin, cfg.contact_distance_factor = ck["dt"], ck["skin"], 1.0
    cfg.neigh_every, cfg.neigh_delay, cfg.neigh_check = 1, 0, 1
    cfg.normal_model, cfg.rolling_model = ck["normal_model"], ck["rolling_model"]
    cfg.tangential_damping, cfg.limit_force = 1, 0
    nt = ck["ntypes"]
    tabs = [np.ascontiguousarray(ck[k], dtype=np.float64).reshape(nt + 1, nt + 1)
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
            *[hp(tb) for tb in tabs], float(ck.get("charVel", 0.0)),
            P(f.data_ptr()), P(t.data_ptr()), None)
        assert rc == 0, api.STATUS.get(rc, rc)
        return f.cpu().numpy().copy(), t.cpu().numpy().copy()

    for k in range(2):
        free0 = torch.cuda.mem_get_info()[0]
        fo, to_ = call()
        if k == 1:  # after the first call loaded the array: no device memory taken
            assert torch.cuda.mem_get_info()[0] == free0
        assert np.all(np.isfinite(fo)) and np.all(np.isfinite(to_))
        assert max_rel(fo, a["f"]) < FORCE_RTOL
        assert max_rel(to_, a["torque"]) < FORCE_RTOL
        assert max_rel(fo[order], ob["f"]) < FORCE_RTOL
        assert max_rel(to_[order], ob["torque"]) < FORCE_RTOL
    g.close()
