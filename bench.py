"""Benchmark of the GB300 sphere-DEM timestep (particle-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload column1m|...]

One bench step = one DEM timestep (Verlet iteration) of the whole system.
value: device-timed throughput with the state resident in HBM (CUDA events
on the library's stream around dem_step(K)).  e2e: the same metric through
the C ABI with host buffers: upload + setup + K steps + download, host
copies inside the timed region.  --impl reference times the reference
binary built from the unmodified reference sources (oracle/_ref/lmp_ref) on
the same workload, one process per host core.  N>1: independent replicas,
one per rank (the path has no exchange step), "scaling": "weak".
"""
import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "liggghts-inl_gb300", "python"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s (1M Hertz/history spheres)"
REF_MAX_STEPS = 100  # timed steps per reference process (--impl reference)
METRICS = {"fibres200k": "particle-steps/s (200k bonded fibre spheres)"}

# Per-unit figures of the two step kernels (the roofline multiplies them by
# the run's own atoms n, list entries E and touching entries C):
#   k_pair_pf   bytes: 100 per atom (x, v, omega, r as doubles, type, the
#               FP32 position copy), 10 per list entry (i, j, image code,
#               active flag), 152 per touching entry (reff, c0, c1; history
#               read and written; flag read and written; F, Ti, Tj written);
#               FP64: flop per touching entry (DADD + DMUL + 2 DFMA, ncu);
#   k_particle  bytes: 273 per atom (x, v, omega, f, torque read and
#               written, dtfm, dtir, holds, rows, the FP32 copy), 5 per list
#               entry (active flag, reverse index), 96 per touching entry (F
#               read by both atoms, Ti and Tj by one each);
#               FP64: flop per atom (gravity, two half-kicks, drift, wall
#               sums) plus 12 per touching entry (two sides of six adds).
KERNEL_UNITS = {
    "pair": {"bytes_atom": 100, "bytes_entry": 10, "bytes_contact": 152, "flop_contact": 204.0},
    "particle": {"bytes_atom": 273, "bytes_entry": 5, "bytes_contact": 96, "flop_atom": 34.0,
                 "flop_contact": 12.0},
}
# DRAM bytes (read + write) per atom of one launch, from the ncu capture of
# the workload (hopper1m at 500k atoms: k_pair_pf 131.0 MB read + 19.7 MB
# written, k_particle 106.8 + 13.3 MB)
DRAM_PER_ATOM = {"hopper1m": {"pair": 301.3, "particle": 240.2}}


# ----------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------

def workload(name, scale=1.0, seed=2024):
    from gb300dem import workloads
    if name == "hopper1m":
        # conical hopper discharge (half-angle 30 deg, top radius 0.25 m,
        # outlet radius 0.03 m, 256 x 64 quads = 32,768 triangles), outlet open,
        # radii U[0.8, 1.2] mm, rho 1500, E 1e7, e 0.5, mu 0.6, CDT rolling 0.3
        # on pairs and wall, dt 5e-7; the lowest 1M sites of a jittered lattice
        case = workloads.hopper_case(
            seed=seed, r_out=0.03, r_top=0.25, half_angle_deg=30.0, n_az=256, n_ax=64,
            spacing=2.2e-3, radius=(0.8e-3, 1.2e-3), density=1500.0, jitter=1e-4, E=(1e7,),
            nu=(0.45,), rest=((0.5,),), frict=((0.6,),), rollfrict=((0.3,),), rolling_model=1,
            dt=5e-7, skin=5e-4, max_atoms=max(1000, int(round(1_000_000 * scale))),
            clearance=-1e-4, z_below=-0.02)
        desc = dict(workload="hopper1m", atoms=int(len(case["atoms"]["tag"])), triangles=32768,
                    description="1M-sphere conical hopper discharge: triangle-mesh cone "
                                "(32,768 triangles), outlet open, polydisperse Hertz/history + CDT "
                                "rolling (pair and wall), jittered lattice (2.2 mm) filling the "
                                "cone from the outlet up, dt 5e-7",
                    l2="state + neighbour list > L2 (129 MB); no flush needed")
        return case, desc
    if name == "column1m":
        # the hopper's materials (r U[0.8,1.2] mm, rho 1500, E 1e7, e 0.5, mu 0.6,
        # CDT 0.3), dense jittered lattice in a periodic column with a floor.
        nx = max(4, int(round(100 * scale ** (1 / 3))))
        case = workloads.lattice_case(
            seed=seed, nx=nx, ny=nx, nz=nx, spacing=2.2e-3, radius=(0.8e-3, 1.2e-3),
            density=1500.0, z0=1.2e-3, jitter=5e-5, vmax=0.2, wmax=20.0, E=(1e7,), nu=(0.3,),
            rest=((0.5,),), frict=((0.6,),), rollfrict=((0.3,),), rolling_model=1, dt=5e-7,
            skin=5e-4)
        desc = dict(workload="column1m", atoms=int(len(case["atoms"]["tag"])),
                    description="polydisperse Hertz/history + CDT rolling spheres, dense jittered "
                                "lattice (2.2 mm, r 0.8-1.2 mm) in a periodic x/y column with a "
                                "floor plane; the hopper's materials, dt 5e-7",
                    l2="state + neighbour list > L2 (129 MB); no flush needed")
        return case, desc
    if name == "dense1m":
        # the dense regime: 1M spheres of the hopper's materials (r U[0.97,
        # 1.03] mm, rho 1500, E 1e7, e 0.5, mu 0.6, CDT 0.3 on pairs and
        # floor) collapsed from an FCC lattice (nearest neighbours 2.04 mm)
        # onto a floor in a periodic x/y column, settled on the GPU for
        # 16,000 steps at dt 5e-6, then restarted from that state (atoms,
        # contact and wall histories through the restart-data path) and timed
        # at the hopper's dt 5e-7: about five touching contacts per sphere
        nx = max(4, int(round(100 * scale ** 0.5)))
        case = workloads.packed_bed_case(
            seed, nx, nx, 25, dnn=2.04e-3, radius=(0.97e-3, 1.03e-3), density=1500.0, dt=5e-6,
            E=(1e7,), nu=(0.45,), rest=((0.5,),), frict=((0.6,),), rollfrict=((0.3,),), rolling_model=1,
            skin=5e-4)
        desc = dict(workload="dense1m", atoms=int(len(case["atoms"]["tag"])), settle_steps=16000,
                    settle_dt=5e-6, dt=5e-7,
                    description="1M polydisperse Hertz/history + CDT spheres settled into a dense bed "
                                "(FCC start, 16,000 steps at dt 5e-6 on the GPU, restarted with its "
                                "contact history), periodic x/y column on a floor, timed at dt 5e-7",
                    l2="state + neighbour list > L2 (129 MB); no flush needed")
        return case, desc
    if name == "fibres200k":
        # bonded-fibre compression: 20,000 fibres x 10 spheres (200k), r 0.5 mm,
        # cohesion bond/nonlinear for an elastoplastic bond material (elastic
        # 1e9 Pa, yield strain 0.01, hardening ratio 0.1; the tables from
        # workloads.elastoplastic_bond_params), bond radius ratio 0.5,
        # tsCreate 1 and createDistance just above 2r, so intra-fibre touching
        # pairs bond at step 1; Hertz between fibres; a two-triangle lid moving
        # down at 0.05 m/s; dt 1e-7.  A 40 mm cube cannot hold 200k spheres of
        # r 0.5 mm (1.6x its volume), so the fibres lie in plywood layers
        # (workloads.fibre_bed_case) in a closed 40.8 x 40.8 mm box.
        r = 0.5e-3
        bp = workloads.elastoplastic_bond_params(
            2, [1], E=1e9, yield_strain=0.01, hardening=0.1, radius=r, lam=0.5, nu=0.3, tsCreate=1.0,
            damp_fn=0.05, damp_ft=0.05, damp_tn=0.05, damp_tt=0.05, maxDistance=2 * r * 1.0035,
            maxSigma=6e6, maxTau=6e6, ratioTC=0.5, createDistance=2 * r * 1.002)
        case = workloads.fibre_bed_case(seed, max(100, int(round(200_000 * scale)) // 10 * 10), radius=r,
                                        bond=bp, dt=1e-7, skin=2e-4, vmax=0.05, plate_vel=(0.0, 0.0, -0.05),
                                        plate_gap=0.0)
        desc = dict(workload="fibres200k", atoms=int(len(case["atoms"]["tag"])), fibres=case["nfibres"],
                    description="200k bonded fibre spheres: 10-sphere fibres (r 0.5 mm) in plywood "
                                "layers, Hertz/history between fibres, cohesion bond/nonlinear within "
                                "(elastoplastic bond: 1e9 Pa, yield strain 0.01, hardening 0.1; bonds "
                                "created at step 1), closed box with a lid pressing down at 0.05 m/s, "
                                "dt 1e-7",
                    l2="state + neighbour list + 28-value bond histories > L2 (129 MB); no flush needed")
        return case, desc
    raise SystemExit("unknown workload %s" % name)


# ----------------------------------------------------------------------------
# helpers
# ----------------------------------------------------------------------------

class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.p = None
        # the samples of the timed region; BENCH_CLOCKS_CSV keeps them in a
        # file of the caller's choice, else a temporary file is used
        self.path = os.environ.get("BENCH_CLOCKS_CSV") or os.path.join(
            tempfile.gettempdir(), "gb300dem_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            if os.path.dirname(self.path):
                os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            c = [t.strip() for t in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                mx = max(mx, float(c[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if c[5 + k].lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


class NvmlClocks:
    """SM clock and clock-event reasons sampled through NVML (libnvidia-ml,
    read-only queries) by a thread that polls every half millisecond while
    the timed region runs, so that even a few-millisecond region has
    samples.  The region's dem_step is a ctypes call, which releases the
    GIL.  Falls back to the nvidia-smi sampler (Clocks) where NVML cannot be
    loaded."""
    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self):
        import ctypes
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        idx = 0
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
        if vis.isdigit():
            idx = int(vis)
        cnt = ctypes.c_uint(0)
        self.lib.nvmlDeviceGetCount_v2(ctypes.byref(cnt))
        if idx >= cnt.value:
            idx = 0
        self.h = ctypes.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(idx), ctypes.byref(self.h)) != 0:
            raise RuntimeError("nvmlDeviceGetHandleByIndex failed")
        self.get_reasons = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.samples, self.reasons = [], set()
        self.thread, self.stop_flag = None, False

    def _sample(self):
        ct = self.ct
        clk, rs = ct.c_uint(0), ct.c_ulonglong(0)
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(clk)) == 0:  # NVML_CLOCK_SM
            self.samples.append(float(clk.value))
        if self.get_reasons(self.h, ct.byref(rs)) == 0:
            for bit, name in self.REASONS.items():
                if rs.value & bit:
                    self.reasons.add(name)

    def _run(self):
        while not self.stop_flag:
            self._sample()
            time.sleep(0.0005)

    def start(self):
        import threading
        self._sample()
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def stop(self):
        self.stop_flag = True
        self.thread.join(timeout=5)
        self._sample()
        mx = self.ct.c_uint(0)
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, self.ct.byref(mx))
        if not self.samples:
            return None
        return {"sm_mhz": statistics.median(self.samples), "sm_max_mhz": float(mx.value),
                "reasons": sorted(self.reasons), "samples": len(self.samples), "source": "nvml"}


def clock_sampler():
    try:
        return NvmlClocks()
    except Exception:
        return Clocks()


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def _oracle_sample_worker(args):
    name, scale, seed, warm, steps = args
    sys.path.insert(0, os.path.join(ROOT, "liggghts-inl_gb300", "python"))
    sys.path.insert(0, ROOT)
    from oracle.binding import Oracle
    case, _ = workload(name, scale=scale, seed=seed)
    o = Oracle(case)
    o.setup()
    o.run(warm)
    t0 = time.perf_counter()
    o.run(steps)
    dt = time.perf_counter() - t0
    return len(case["atoms"]["tag"]), steps, dt


def cpu_sample(name, cores, steps, warm=2, scale=0.01):
    """Times the oracle port (the C restatement) on `cores` independent
    replicas of the workload at the given scale, one per process."""
    from oracle import binding
    binding.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_oracle_sample_worker, [(name, scale, 2024 + k, warm, steps) for k in range(cores)])
    tot = sum(n * s for n, s, _ in res)
    tmax = max(dt for _, _, dt in res)
    return tot / tmax, res


def ref_binary():
    """The reference binary oracle/ref/Makefile builds from the unmodified
    reference sources (serial, its own MPI stubs, -O3, the GPU path's contact
    models compiled in through the reference's whitelist), or None."""
    p = os.path.join(ROOT, "oracle", "_ref", "lmp_ref")
    return p if os.path.isfile(p) and os.access(p, os.X_OK) else None


def lmp_sample(name, nproc, steps, warm, seed=2024, case=None):
    """Times the reference binary on the full workload: one input script
    (seeded data file, STL mesh, the reference's own commands), `nproc`
    independent processes (one per host core), each "run warm" then "run
    steps"; the timed figure is the reference's "Loop time" of the second
    run (output off inside it).  Returns (particle-steps/s of all processes
    over the slowest one's loop time, [(atoms, steps, loop s)])."""
    import shutil
    from oracle.lmp_input import write_inputs
    exe = ref_binary()
    if case is None:
        case, _ = workload(name, seed=seed)
    n0 = len(case["atoms"]["tag"])
    top = tempfile.mkdtemp(prefix="lmp_ref_")
    try:
        # the reference's own spatial sort on (its default, "sort 1000 0"):
        # its fastest setting; the parity runs keep the atoms' order instead
        write_inputs(case, top, 0, runs=[warm, steps], atom_sort="1000 0")
        files = [f for f in os.listdir(top) if os.path.isfile(os.path.join(top, f))]
        procs = []
        for k in range(nproc):
            d = os.path.join(top, "p%d" % k)
            os.makedirs(d)
            for f in files:
                os.symlink(os.path.join(top, f), os.path.join(d, f))
            procs.append(subprocess.Popen([exe, "-in", "in.case", "-log", "log.case", "-screen", "screen.case"],
                                          cwd=d, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
        res = []
        for k, p in enumerate(procs):
            rc = p.wait()
            log = open(os.path.join(top, "p%d" % k, "log.case")).read()
            loops = [ln.split() for ln in log.splitlines() if ln.startswith("Loop time of")]
            if rc != 0 or len(loops) < 2:
                raise RuntimeError("reference run failed (rc %d): %s" % (rc, log[-1500:]))
            res.append((n0, int(loops[-1][8]), float(loops[-1][3])))
    finally:
        shutil.rmtree(top, ignore_errors=True)
    tot = sum(n * s for n, s, _ in res)
    return tot / max(t for _, _, t in res), res


# ----------------------------------------------------------------------------
# replicas (N > 1): independent systems, one per rank, no data-path exchange
# ----------------------------------------------------------------------------

def replica_throughput(dev_ms, atoms, steps, dist=None, device=None):
    """Whole-job particle-steps/s of N replicas: every rank ran `atoms`
    atoms for `steps` steps in `dev_ms` ms (its device time); the job's time
    is the slowest rank's (max over ranks).  Returns (value, max_ms)."""
    world = 1
    if dist is not None and dist.is_initialized():
        import torch
        world = dist.get_world_size()
        t = torch.tensor([float(dev_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dev_ms = float(t.item())
    return world * atoms * steps / (dev_ms * 1e-3), dev_ms


# ----------------------------------------------------------------------------
# arms
# ----------------------------------------------------------------------------

def run_reference(args):
    """The reference's own CPU implementation of the path on the host cores:
    the reference binary (oracle/_ref/lmp_ref) on the full workload, one
    serial process per core (no MPI library on the machine: the build is the
    reference's serial one against its MPI stubs), beside the C port on one
    core for the port-to-binary ratio.  Without the binary (no reference
    sources staged), the port on all cores stands in, kind "port"."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    # a bounded sample: at most REF_MAX_STEPS timed steps of the full
    # workload per process (the metric is a rate), so that a long K still
    # ends within a few minutes
    steps = max(1, min(args.steps, REF_MAX_STEPS))
    warm = max(1, min(args.warmup, 5))
    t0 = time.perf_counter()
    exe = ref_binary()
    if exe:
        val, res = lmp_sample(args.workload, cores, steps, warm)
        pv, pres = cpu_sample(args.workload, 1, steps, warm=1, scale=1.0)
        kind = "reference"
        sample = ("reference binary (oracle/_ref/lmp_ref: unmodified reference sources, serial, -O3, "
                  "whitelisted contact models, atom_modify sort 1000 0) on the full %d-atom %s, %d "
                  "independent processes (one per core), 'run %d' then the timed 'run %d' (its Loop time)"
                  % (res[0][0], args.workload, cores, warm, steps))
        per_proc = statistics.mean(n * s / t for n, s, t in res)
        port = {"value": pv, "cores": 1, "per_process_binary": per_proc, "port_over_binary": pv / per_proc,
                "sample": "oracle port (oracle/dem_oracle.c) on the same full workload, 1 thread, "
                          "%d steps after 1" % steps}
        config = {"workload": args.workload, "atoms": res[0][0], "processes": cores}
        ms = 1e3 * max(t for _, _, t in res) / steps
    else:
        val, res = cpu_sample(args.workload, cores, steps, warm=warm)
        kind = "port"
        sample = ("%d independent replicas (one per core) of a %d-atom slice of %s, %d timed steps each "
                  "(the reference binary is not built here)" % (cores, res[0][0], args.workload, steps))
        port = None
        config = {"workload": args.workload, "sample_atoms": res[0][0], "replicas": cores}
        ms = 1e3 * max(r[2] for r in res) / steps
    wall = time.perf_counter() - t0
    line = {"metric": METRICS.get(args.workload, METRIC), "value": val, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "timed_steps_per_process": steps,
            "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "impl": "reference", "config": config,
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": cores, "kind": kind,
                             "sample": sample},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": wall}
    if port:
        line["port"] = port
    print(json.dumps(line))


def settle_bed(case, desc):
    """The dense workload's preparation (outside every timed region): the
    bed settles on the GPU at desc["settle_dt"], then its state becomes the
    restart data of the timed run at desc["dt"]."""
    from gb300dem import api, workloads
    g = api.DemSystem(dict(case, dt=desc["settle_dt"]))
    g.setup()
    g.step(desc["settle_steps"])
    ck, to, tp, hh, walls = workloads.restart_state(g, case)
    g.close()
    ck["dt"] = desc["dt"]
    return ck, (to, tp, hh, walls)


def run_gb300(args):
    from gb300dem import api
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    case, desc = workload(args.workload, scale=args.scale, seed=2024 + rank)
    restart = None
    if desc.get("settle_steps"):
        case, restart = settle_bed(case, desc)
    n = len(case["atoms"]["tag"])
    g = api.DemSystem(case)
    if restart:
        g.set_restart(*restart)
    g.setup()
    g.step(args.warmup)
    # ---- headline: device-timed K steps, state resident
    if dist:
        dist.barrier()
    clocks = clock_sampler()
    clocks.start()
    g.profile(False)
    t0 = time.perf_counter()
    g.step(args.steps)
    wall = time.perf_counter() - t0
    cl = clocks.stop()
    st = g.stats()
    kt = g.kernel_times()
    value, dev_ms = replica_throughput(st["last_step_ms"], n, args.steps, dist, device="cuda")
    # ---- per-kernel times (separate profiled run of the same length)
    g.profile(True)
    g.step(args.steps)
    kp = g.kernel_times()
    g.profile(False)
    # ---- e2e through the C ABI with host buffers
    # (the caller's host arrays exist before the run, as the reference's
    # atom->x, atom->v, ... do; the device reads and fills them)
    # The caller's arrays are in pinned (page-locked) host memory, allocated
    # and filled before the timed region.  Pageable arrays go through the
    # same calls (the kernels reach them through the host page tables), but
    # their transfer time depends on the pages' history: 1 to 16 ms for the
    # 144 MB of a download, against the pinned arrays' steady rate.
    import torch
    pinned = []

    def _pinned(shape, dtype):
        tt = {np.dtype(np.float64): torch.float64, np.dtype(np.int32): torch.int32}[np.dtype(dtype)]
        t = torch.empty(shape, dtype=tt, pin_memory=True)
        pinned.append(t)
        return t.numpy()

    a = case["atoms"]
    host = {}
    for k, v in a.items():
        host[k] = _pinned(v.shape, v.dtype)
        host[k][...] = v
    g2 = api.DemSystem({k: v for k, v in case.items() if k != "atoms"})
    hout = {}
    for k, v in g2.atom_buffers(n).items():
        hout[k] = _pinned(v.shape, v.dtype)
        hout[k].fill(0)
    t0 = time.perf_counter()
    g2.upload(host)
    if restart:
        g2.set_restart(*restart)
    t1 = time.perf_counter()
    g2.setup()
    t2 = time.perf_counter()
    g2.step(args.steps)
    t3 = time.perf_counter()
    out = g2.atoms(hout)
    t4 = time.perf_counter()
    e2e_s = t4 - t0
    h2d = n * (3 * 3 * 8 + 2 * 8 + 2 * 4)
    d2h = n * (5 * 3 * 8 + 2 * 8 + 2 * 4)
    assert out["x"].shape[1] == 3 and len(out["x"]) <= n
    phases = {"upload_ms": 1e3 * (t1 - t0), "setup_ms": 1e3 * (t2 - t1), "steps_ms": 1e3 * (t3 - t2),
              "download_ms": 1e3 * (t4 - t3), "host_direct": g2.stats()["host_direct"]}
    e2e, _ = replica_throughput(e2e_s * 1e3, n, args.steps, dist, device="cuda")  # slowest rank
    g2.close()
    # ---- roofline of the dominant kernel
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    npairs = st["npairs"]
    pair_ms = kp["pair_ms"] / max(1, kp["pair_launches"])
    wall_ms = kp["wall_ms"] / max(1, kp["wall_launches"]) if kp.get("wall_launches") else 0.0
    part_ms = kp["particle_ms"] / max(1, kp["particle_launches"])
    neigh_ms = kp["neigh_ms"] / max(1, kp["neigh_stages"])
    tot_ms = pair_ms + part_ms + neigh_ms + wall_ms
    # ---- roofline of the dominant kernel from this run's own counts: atoms
    # n, list entries E, touching entries C (dem_get_diagnostics after the
    # timed steps), times the per-unit figures of KERNEL_UNITS
    try:
        fp64_peak = api.fp64_peak_tflops()
    except Exception:
        fp64_peak = None
    ncontact = int(g.diagnostics()["ncontacts"])
    E, C = int(npairs), ncontact
    ku = KERNEL_UNITS
    pair_bytes = n * ku["pair"]["bytes_atom"] + E * ku["pair"]["bytes_entry"] + C * ku["pair"]["bytes_contact"]
    part_bytes = (n * ku["particle"]["bytes_atom"] + E * ku["particle"]["bytes_entry"]
                  + C * ku["particle"]["bytes_contact"])
    pair_flop = C * ku["pair"]["flop_contact"]
    part_flop = n * ku["particle"]["flop_atom"] + C * ku["particle"]["flop_contact"]
    dom = "pair" if pair_ms >= part_ms else "particle"
    # the pair kernel that runs: k_pair_pf (contact distance factor 1, no
    # cohesion) or k_pair (bonds, or a larger contact distance)
    bonded = bool(case.get("bond")) or float(case.get("cdf", 1.0)) != 1.0
    pair_kernel = "k_pair" if bonded else "k_pair_pf"
    dom_bytes = pair_bytes if dom == "pair" else part_bytes
    dom_flop = pair_flop if dom == "pair" else part_flop
    dom_ms = pair_ms if dom == "pair" else part_ms
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = DRAM_PER_ATOM.get(args.workload, {}).get(dom)
    hbm_roof = {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": traffic * n if traffic else None,
                "algorithmic_bytes_per_launch": dom_bytes,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks.get("hbm_gbs")
                else "6800 GB/s (of fallback: no MEASURED_PEAKS.json)"}
    if fp64_peak:
        ach_tf = dom_flop / (dom_ms * 1e-3) / 1e12
        roof = {"kernel": pair_kernel if dom == "pair" else "k_particle", "bound": "fp64",
                "achieved": ach_tf, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach_tf / fp64_peak,
                "traffic": hbm_roof["traffic"],
                "peak_source": "FP64 FMA peak measured live on this GPU (dem_measure_fp64_peak), "
                               "of measured",
                "fp64_flop_per_launch": dom_flop, "hbm": hbm_roof,
                "note": "flop counts DADD/DMUL + 2*DFMA per unit (ncu) times this run's units; the "
                        "FP64 pipe also issues compares, conversions and the idle lanes of partly "
                        "active warps, so its active fraction exceeds achieved/peak"
                        + ("; k_pair: the contact law's flops only, not the bond law's"
                           if bonded and dom == "pair" else "")}
    else:
        roof = dict(hbm_roof, kernel=pair_kernel if dom == "pair" else "k_particle", bound="hbm")
    roof.update({"avg_launch_ms": dom_ms,
                 "units": {"atoms": n, "list_entries": E, "touching_entries": C,
                           "touching_per_atom": C / max(1, n)},
                 "shares": {"pair": pair_ms / tot_ms, "particle": part_ms / tot_ms,
                            "wall": wall_ms / tot_ms, "neigh": neigh_ms / tot_ms},
                 "shares_note": "host-queued profiled run (kernels serialised, rebuild stage as "
                                "no-op launches); the timed graph runs the wall kernel beside "
                                "the pair kernel and skips the rebuild stage unless needed"})
    if fp64_peak:
        roof["fp64_peak_tflops_measured"] = fp64_peak
    # ---- CPU baseline (oracle port, bounded sample, rank 0, N=1 only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        if ref_binary() and args.scale == 1.0:
            v, res = lmp_sample(args.workload, 1, args.cpu_steps, 1, case=case if restart else None)
            cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "reference",
                   "sample": "reference binary (oracle/_ref/lmp_ref, serial, -O3, sort 1000 0) on the full "
                             "%d-atom %s%s, "
                             "'run 1' then the timed 'run %d' (its Loop time), 1 process"
                             % (res[0][0], args.workload,
                                " (the settled positions, read_data without contact history)" if restart else "",
                                args.cpu_steps)}
        else:
            v, res = cpu_sample(args.workload, 1, steps=args.cpu_steps, warm=1)
            cpu = {"value": v, "unit": "particle-steps/s", "cores": 1, "kind": "port",
                   "sample": "oracle (CPU restatement, pinned to the reference binary) on a %d-atom slice "
                             "of %s, %d steps, 1 thread" % (res[0][0], args.workload, args.cpu_steps)}
    if rank == 0:
        line = {"metric": METRICS.get(args.workload, METRIC), "value": value, "unit": "particle-steps/s",
                "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded)", "impl": "gb300",
                "config": dict(desc, parallelism="replicas" if world > 1 else "single",
                               pairs=npairs, rebuilds_total=st["nrebuilds"]),
                "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d / args.steps,
                        "d2h_bytes_per_step": d2h / args.steps,
                        "note": "upload+setup+K steps+download through the C ABI, pinned host buffers",
                        "phases": phases},
                "gpu_launches": kt["kernel_launches"],
                "roofline": roof, "cpu_baseline": cpu, "clocks": cl, "wall_s": wall,
                "kernel_ms_per_step": {"pair": pair_ms, "particle": part_ms, "wall": wall_ms,
                                       "neigh": neigh_ms}}
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_ensemble(args):
    """Batched ensemble (256 settling columns, N_k ~ U[2000, 20000]): the
    packed ensemble against the same systems run one at a time through the
    plain path (one handle per system, same library, same step count)."""
    from gb300dem import api, ensemble
    nsys = max(2, int(round(256 * args.scale)))
    systems = ensemble.settling_systems(2024, nsys)
    ntot = sum(len(s["atoms"]["tag"]) for s in systems)
    # launch shape, cell size and skin, timed over enough steps to include
    # the rebuilds a skin implies; the tuned skin is used by both the
    # ensemble and the one-at-a-time runs below
    s0 = float(systems[0]["skin"])
    best, table = ensemble.autotune(systems[: max(2, nsys // 4)], steps=200, warm=20,
                                    blocks_per_sm=(4, 8, 16), cell_scale=(1.0, 1.25),
                                    skins=(0.6 * s0, s0, 1.5 * s0), particle_threads=(128, 256))
    skin = best[2]
    systems = [dict(sy, skin=skin) for sy in systems]
    e = ensemble.Ensemble(systems, tuning=(best[0], best[1], best[3]))
    e.setup()
    e.step(args.warmup)
    clocks = clock_sampler()
    clocks.start()
    e.step(args.steps)
    cl = clocks.stop()
    st = e.stats()
    ens_ms = st["last_step_ms"]
    value = ntot * args.steps / (ens_ms * 1e-3)
    e.close()
    # plain path: each system alone, the same number of steps
    plain_ms, plain_ps = 0.0, 0
    for s in systems:
        g = api.DemSystem(s)
        g.setup()
        g.step(args.warmup)
        g.step(args.steps)
        plain_ms += g.stats()["last_step_ms"]
        plain_ps += len(s["atoms"]["tag"]) * args.steps
        g.close()
    plain = plain_ps / (plain_ms * 1e-3)
    line = {"metric": "particle-steps/s (batched ensemble, %d settling columns)" % nsys, "value": value,
            "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ens_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "gb300",
            "config": {"workload": "ensemble%d" % nsys, "systems": nsys, "atoms": ntot,
                       "description": "settling columns, N_k ~ U[2000, 20000], r U[0.9, 1.1] mm, "
                                      "E log-U[1e6, 1e8] Pa, e U[0.3, 0.95], mu U[0.1, 0.9], box "
                                      "0.05 x 0.05 x 0.3 m periodic x/y, floor, Hertz + history, dt 1e-6",
                       "tuning": {"blocks_per_sm": best[0], "cell_scale": best[1], "skin": skin,
                                  "particle_threads": best[3]},
                       "rebuilds_total": st["nrebuilds"]},
            "plain_one_at_a_time": {"value": plain, "unit": "particle-steps/s",
                                    "note": "the same systems, one handle each, run in turn"},
            "ensemble_over_plain": value / plain,
            "autotune": [{"blocks_per_sm": t[0][0], "cell_scale": t[0][1], "skin": t[0][2],
                          "particle_threads": t[0][3], "ms_per_step": t[1]} for t in table],
            "clocks": cl}
    print(json.dumps(line))


def adjoint_case(seed=2024, n=20000):
    """Adjoint case: n spheres as the settling columns (r U[0.9, 1.1]
    mm, jittered 2.2 mm lattice above a floor, 0.05 x 0.05 x 0.3 m box
    periodic in x/y), one parameter set (E 1e7, e 0.6, mu 0.5), dt 1e-6"""
    from gb300dem import workloads
    spacing = 2.2e-3
    nx = ny = int(0.05 / spacing)
    nz = (n + nx * ny - 1) // (nx * ny)
    c = workloads.lattice_case(seed=seed, nx=nx, ny=ny, nz=nz, spacing=spacing, radius=(0.9e-3, 1.1e-3),
                               density=2500.0, z0=1.2 * 1.1e-3, jitter=0.05 * spacing, E=(1e7,), nu=(0.3,),
                               rest=((0.6,),), frict=((0.5,),), dt=1e-6, skin=5e-4, zhi=0.3,
                               pad=(0.05 - nx * spacing, 0.05 - ny * spacing))
    keep = np.arange(len(c["atoms"]["tag"])) < n
    c["atoms"] = {k: v[keep] for k, v in c["atoms"].items()}
    return c


def run_adjoint(args):
    """Cost of one adjoint gradient (forward with checkpoints + backward with
    replay) of the kinetic energy after `steps` steps, against the plain
    path's forward run of the same system and steps."""
    from gb300dem import api
    from gb300dem.adjoint import DemAdjoint, make_loss
    n = max(1000, int(round(20000 * args.scale)))
    steps = args.steps
    seg = max(1, int(round(steps ** 0.5)))
    case = adjoint_case(n=n)
    g = api.DemSystem(case)
    g.setup()
    g.step(args.warmup)
    g.step(steps)
    plain_ms = g.stats()["last_step_ms"]
    g.close()
    eng = DemAdjoint(case)
    spec = make_loss(w_ke=1.0)
    modes = {}
    for mode, name in ((0, "checkpoint_replay"), (1, "recorded")):
        eng.set_tape(mode)
        for _ in range(2):  # the first run sizes the arena
            val, grad = eng.gradient(1e7, 0.6, 0.5, nsteps=steps, segment=seg, loss=spec)
        tm = eng.times()
        modes[name] = {"forward_ms": tm["forward_ms"], "backward_ms": tm["backward_ms"],
                       "total_over_plain_forward": (tm["forward_ms"] + tm["backward_ms"]) / plain_ms,
                       "backward_over_forward": tm["backward_ms"] / tm["forward_ms"]}
    eng.close()
    t = {"forward_ms": modes["recorded"]["forward_ms"], "backward_ms": modes["recorded"]["backward_ms"],
         "segments": tm["segments"], "max_pairs": tm["max_pairs"]}
    total = t["forward_ms"] + t["backward_ms"]
    line = {"metric": "adjoint gradient time / plain forward time", "value": total / plain_ms, "unit": "x",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup, "higher_is_better": False,
            "dtype": "f64", "data": "synthetic (seeded)", "impl": "gb300",
            "config": {"workload": "adjoint%dk" % (n // 1000), "atoms": n, "segment": seg,
                       "description": "20k settling-column spheres, one parameter set, "
                                      "kinetic-energy loss, gradients w.r.t. E, e, mu and every radius"},
            "plain_forward_ms": plain_ms, "adjoint_forward_ms": t["forward_ms"],
            "adjoint_backward_ms": t["backward_ms"], "backward_over_forward": t["backward_ms"] / t["forward_ms"],
            "segments": t["segments"], "max_pairs": t["max_pairs"], "loss": val, "tape_modes": modes,
            "note": "value: the record taken in the forward pass (tape mode 1); checkpoint_replay: the "
                    "sqrt(N) checkpoints with the replay of each segment (tape mode 0)",
            "grad": {"E": grad["E"], "restitution": grad["restitution"], "friction": grad["friction"]}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="hopper1m",
                    choices=["hopper1m", "column1m", "dense1m", "fibres200k", "ensemble256", "adjoint20k"])
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="fraction of the workload's atoms (small cases for ncu captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "ensemble256":
        run_ensemble(args)
    elif args.workload == "adjoint20k":
        run_adjoint(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
