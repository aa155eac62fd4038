#!/usr/bin/env python
"""Throughput of the per-step particle update on one GB300 (and N independent replicas on N GPUs).

Headline workload: the (20,10,10) ellipsoid meshed as a level-7 icosphere (163,842 vertices,
327,680 faces), 1,048,576 particles at area packing 0.5 (radius from packing, r_max = 2.4 R),
eta = 0.3, dt = 0.01, FP32 state. Synthetic, seeded placement (no dataset exists).

One bench step = one simulation step of the whole system (4 kernels). The K timed steps run back
to back, launched as the library launches them, between CUDA events on the handle's stream; no L2
flush inside the timed region, because each step touches more than the 126 MB L2 (state, its
sorted copy, cell tables, face records). value = particle-steps/s over all ranks (max time over
ranks). The same steps with a 256 MB L2 flush before each step are reported beside it
(flushed_per_step). e2e = the same metric through the C-ABI with host buffers: set_state (H2D) +
step + get_state (D2H) per step, from/to pinned host memory, enqueued with the pipelined calls so
that the upload of step k+1 overlaps the download of step k (the synchronous-call figure is
reported beside it).

The same line carries the rest of the metric (particle-steps/s forward and forward+adjoint,
batched vs plain), each on its own workload with its step count stated:
  ensemble         4,096 replicas on the (4,2,2) ellipsoid (level-4 icosphere), particle counts
                   log-uniform in [64, 8192], eta U[0, 2 pi], v0 U[0.5, 1.5]: batched in one handle
                   vs the same replicas (a seeded sample) launched one by one with plain handles;
  adjoint          10,000 particles on the (6,3,3) ellipsoid, 2,000 steps, checkpoint every 50:
                   forward+adjoint time over forward time;
  adjoint_batched  512 replicas on the bumpy sphere (level-6 icosphere), 1,000-20,000 particles
                   each, per-replica v0/k/tau/eta, 500 steps: forward+adjoint over forward.

--impl reference times the CPU restatement of the path (oracle, FP64, all host threads) on the same
workload; it loads only the oracle's library (the mesh arrays come from the workload file that
build() writes); under torchrun only rank 0 runs it.
"""
import argparse
import hashlib
import importlib
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (forward step, 1M-particle plain system)"
UNIT = "particle-steps/s"
ALG_BYTES_PARTICLE = 68  # FP32: read uv 8 + theta 4 + face 4 + r3d 12; write those + vel_uv 8 + count 4
ALG_BYTES_FACE = 60      # 3 UV corners x 8 + 3 3D corners x 12
ALG_BYTES_REPLICA = 4    # order parameter
N_1M = 1 << 20
# the headline workload's mesh and chart arrays, written by build() with the product's mesh code so
# that the reference arm can read them without loading the product library
WORKLOAD_MESH = os.path.join(ROOT, "oracle", "_build", "workload_ellipsoid_l7_20_10_10.npz")


def save_workload_mesh(tg, path=WORKLOAD_MESH):
    mesh = tg.Mesh.ellipsoid(7, (20.0, 10.0, 10.0))
    a = mesh.arrays()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp%d.npz" % os.getpid()
    np.savez(tmp, area=np.float64(mesh.area), **a)
    os.replace(tmp, path)
    return mesh


def load_workload_mesh():
    """The headline mesh's arrays without the product library (written by build(); made by a
    separate process when missing)."""
    if not os.path.exists(WORKLOAD_MESH):
        subprocess.run([sys.executable, os.path.abspath(__file__), "--write-workload-mesh"], check=True)
    z = np.load(WORKLOAD_MESH)
    return {k: z[k] for k in ("v3", "f3", "uv", "fuv", "uv2v")}, float(z["area"])


def mesh_sha16(a):
    h = hashlib.sha256()
    for k in ("v3", "f3", "uv", "fuv"):
        h.update(np.ascontiguousarray(a[k]).tobytes())
    return h.hexdigest()[:16]


def workload_params(area):
    """Radius from area packing 0.5 of N_1M particles, r_max = 2.4 R, eta 0.3, dt 0.01; the other
    parameters are the 100-particle system's (k 10, k_adh 0.75, v0 1, mu 1, tau 1, align 0.5)."""
    radius = float(np.sqrt(0.5 * area / (np.pi * N_1M)))
    return dict(radius=radius, k_rep=10.0, k_adh=0.75, r_max=2.4 * radius, v0=1.0, mu=1.0, tau=1.0, align=0.5,
                eta=0.3, dt=0.01)


def oracle_params(prm):
    return dict(R=prm["radius"], k=prm["k_rep"], k_adh=prm["k_adh"], r_max=prm["r_max"], v0=prm["v0"], mu=prm["mu"],
                tau=prm["tau"], align=prm["align"], eta=prm["eta"], dt=prm["dt"])


def workload_config(faces, prm, sha):
    """The workload, identical in both arms (how each arm runs it is reported outside config)."""
    return {"workload": "plain step, (20,10,10) ellipsoid L7 icosphere, 1,048,576 particles, packing 0.5",
            "faces": int(faces), "particles": N_1M, "radius": round(prm["radius"], 6), "r_max": round(prm["r_max"], 6),
            "eta": prm["eta"], "dt": prm["dt"], "seeded": True, "mesh_sha16": sha}


def workload_1m(tg):
    mesh = tg.Mesh.ellipsoid(7, (20.0, 10.0, 10.0))
    prm = workload_params(mesh.area)
    return mesh, tg.Params(**prm), N_1M, prm


def measured_peak():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(name, n_particles):
    """DRAM bytes per k_step launch from a committed ncu summary (per particle, scaled)."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("dram_bytes_per_particle:"):
                return float(line.split(":")[1]) * n_particles
    except OSError:
        pass
    return None


class _Nvml:
    """Read-only NVML queries through ctypes (SM clock, max SM clock, clock-event reasons)."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index):
        import ctypes as C
        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h)) != 0:
            raise OSError("no NVML device %d" % index)
        reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = reasons_fn or self.lib.nvmlDeviceGetCurrentClocksThrottleReasons

    def sample(self):
        C = self.C
        mhz, r = C.c_uint(0), C.c_ulonglong(0)
        ok = self.lib.nvmlDeviceGetClockInfo(self.h, C.c_int(1), C.byref(mhz)) == 0  # NVML_CLOCK_SM
        self.reasons_fn(self.h, C.byref(r))
        return (float(mhz.value) if ok else None), int(r.value)

    def max_sm(self):
        C = self.C
        mhz = C.c_uint(0)
        return float(mhz.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, C.c_int(1), C.byref(mhz)) == 0 else None


class Clocks:
    """SM clocks and clock-event reasons during the timed region: an NVML poller every 5 ms (the
    timed region can be shorter than nvidia-smi's sampling period) and nvidia-smi at 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        import threading
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        self.nv_samples, self.nv_max = [], None
        self.done = threading.Event()
        self.t = None
        try:
            self.nv = _Nvml(index)
            self.nv_max = self.nv.max_sm()
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
        except (OSError, AttributeError):
            self.nv = None

    def _poll(self):
        while not self.done.is_set():
            self.nv_samples.append(self.nv.sample())
            self.done.wait(0.005)

    def stop(self):
        self.done.set()
        if self.t is not None:
            self.t.join()
        rows = []
        if self.p is not None:
            self.p.terminate()
            self.p.wait()
            self.f.seek(0)
            rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        nv_sm = [s for s, _ in self.nv_samples if s is not None]
        for _, bits in self.nv_samples:
            for b, nm in _Nvml.REASONS.items():
                if bits & b:
                    reasons.add(nm)
        if nv_sm:
            return {"sm_mhz": float(np.median(nv_sm)), "sm_max_mhz": self.nv_max or (max(mx) if mx else None),
                    "reasons": sorted(reasons), "samples": len(nv_sm), "source": "NVML every 5 ms",
                    "nvidia_smi_samples": len(rows)}
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows), "source": "nvidia-smi every 200 ms"}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl != "reference" else "gloo")
    return world, rank, local


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def oracle_cpu_rate(arrays, prm, state, n, budget_s=20.0, threads=0):
    """FP64 oracle steps over the full state; returns (particle-steps/s, sample, cores, one-core record)."""
    import oracle
    om = oracle.Mesh(arrays["v3"], arrays["f3"], arrays["uv"], arrays["fuv"])
    cen = arrays["v3"].mean(0)
    op = oracle_params(prm)
    st = dict(uv=state["uv"], theta=state["theta"], face=state["face"], r3d=state["r3d"],
              ids=np.arange(n, dtype=np.int32))
    cores = threads or os.cpu_count()
    t0 = time.perf_counter()
    oracle.model_step(om, op, st, 0, 0, centroid=cen, threads=cores)
    t1 = time.perf_counter() - t0
    steps = max(1, min(10, int(budget_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    for k in range(steps):
        out = oracle.model_step(om, op, st, k + 1, 0, centroid=cen, threads=cores)
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=st["ids"])
    dt = time.perf_counter() - t0
    # one core (the reference is single-threaded): a seeded subset updated from the full state
    sub = np.sort(np.random.default_rng(2).choice(n, min(n, 65536), replace=False)).astype(np.int32)
    t0 = time.perf_counter()
    k1 = 0
    while k1 < 10 and time.perf_counter() - t0 < 5.0:
        oracle.model_step(om, op, st, steps + 1 + k1, 0, centroid=cen, subset=sub, threads=1)
        k1 += 1
    one = {"value": len(sub) * k1 / (time.perf_counter() - t0), "cores": 1,
           "sample": "%d steps updating a seeded %d-particle subset of the full state" % (k1, len(sub))}
    return (n * steps / dt, "%d full steps of the %d-particle state (FP64 oracle, %d threads)" % (steps, n, cores),
            cores, one)


def seeded_state(arrays, n, seed):
    """Area-weighted seeded placement in numpy (host only), for the CPU reference arm."""
    v3, f3, uv, fuv = arrays["v3"], arrays["f3"], arrays["uv"], arrays["fuv"]
    rng = np.random.default_rng(seed)
    A, B, C = v3[f3[:, 0]], v3[f3[:, 1]], v3[f3[:, 2]]
    ar = 0.5 * np.linalg.norm(np.cross(B - A, C - A), axis=1)
    cdf = np.cumsum(ar) / ar.sum()
    f = np.minimum(np.searchsorted(cdf, rng.random(n)), len(cdf) - 1)
    s, t = np.sqrt(rng.random(n)), rng.random(n)
    w = np.stack([1 - s, s * (1 - t), s * t], 1)
    p = w[:, 0, None] * uv[fuv[f, 0]] + w[:, 1, None] * uv[fuv[f, 1]] + w[:, 2, None] * uv[fuv[f, 2]]
    r3 = w[:, 0, None] * A[f] + w[:, 1, None] * B[f] + w[:, 2, None] * C[f]
    th = rng.random(n) * 2 * np.pi - np.pi
    return dict(uv=p, theta=th, face=f.astype(np.int32), r3d=r3)


def run_reference(args):
    """The CPU path on the host cores: the FP64 oracle's model step (all host threads) on the
    headline workload. Only the oracle's library is loaded; the mesh comes from the workload file."""
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return
    import oracle
    arrays, area = load_workload_mesh()
    prm = workload_params(area)
    op = oracle_params(prm)
    n = N_1M
    state = seeded_state(arrays, n, 0)
    om = oracle.Mesh(arrays["v3"], arrays["f3"], arrays["uv"], arrays["fuv"])
    cen = arrays["v3"].mean(0)
    cores = os.cpu_count()
    st = dict(state, ids=np.arange(n, dtype=np.int32))
    t0 = time.perf_counter()
    for k in range(max(args.warmup, 1)):
        out = oracle.model_step(om, op, st, k, 0, centroid=cen, threads=cores)
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=st["ids"])
    t_full = (time.perf_counter() - t0) / max(args.warmup, 1)
    # bounded sample: full steps of the whole state (the CPU's best throughput), at most as many as
    # fit in ~60 s when the requested K steps would take longer
    n_steps = max(1, min(args.steps, int(60.0 / max(t_full, 1e-6))))
    t0 = time.perf_counter()
    for k in range(n_steps):
        out = oracle.model_step(om, op, st, args.warmup + k, 0, centroid=cen, threads=cores)
        st = dict(uv=out["uv"], theta=out["theta"], face=out["face"], r3d=out["r3d"], ids=st["ids"])
    dt = time.perf_counter() - t0
    value = n * n_steps / dt
    sample = ("%d full steps of the %d-particle state (of %d requested; FP64 oracle, %d threads)"
              % (n_steps, n, args.steps, cores))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3 / n_steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded placement)",
            "config": workload_config(len(arrays["f3"]), prm, mesh_sha16(arrays)),
            "state": "fp64 host arrays (oracle)", "l2": "n/a (CPU)",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _event_ms(torch, stream, fn):
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(stream)
    fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def ensemble_leg(tg, steps=50, sample=64, autotune=False, replicas=4096):
    """Batched ragged ensemble (4096 replicas on the (4,2,2) ellipsoid, level-4 icosphere, particle
    counts log-uniform in [64, 8192], eta in [0, 2 pi], v0 in [0.5, 1.5], dt 0.02) in one handle,
    against a seeded sample of the same replicas each in its own plain handle. Working set > L2."""
    import torch
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    mesh = tg.Mesh.ellipsoid(4, (4.0, 2.0, 2.0))
    n, eta, v0 = ens.ragged_replicas(seed=0, n_replicas=replicas)
    ns = [int(x) for x in n]
    total = int(n.sum())
    ps = [tg.Params(radius=0.05, r_max=0.12, v0=float(v), eta=float(e), dt=0.02) for e, v in zip(eta, v0)]
    tuning, tune_rate = None, None
    if autotune:
        tuning, tune_rate = tg.autotune(mesh, ps, ns, seed=0, precision=32, trial_steps=64)
    sim = tg.Simulation(mesh, ps, ns, seed=0, precision=32, tuning=tuning)
    sim.start()
    stream = torch.cuda.ExternalStream(sim.stream())
    sim.step(3)
    ms = _event_ms(torch, stream, lambda: sim.step_async(steps))
    assert sim.status() == 0
    batched = total * steps / (ms * 1e-3)
    # per-kernel events over directly launched steps: the step kernel's duration for the roofline
    sim.kernel_timing(True)
    sim.step_async(10)
    torch.cuda.synchronize()
    kt = sim.kernel_times()
    sim.kernel_timing(False)
    k_ms = kt["step"][0] / max(kt["step"][1], 1)
    summed_ms = sum(v[0] for v in kt.values()) / 10
    alg = ALG_BYTES_PARTICLE * total + ALG_BYTES_FACE * mesh.F + ALG_BYTES_REPLICA * len(ns)
    peak, peak_kind = measured_peak()
    phi, _ = sim.order_parameter()
    sim_tuning = sim.tuning()
    sim.close()
    # one by one: a seeded sample of replicas, each its own plain handle, each replica's steps
    # launched as the library launches a plain system's steps (one loop-graph launch), one replica
    # after the other (each run waited for before the next replica starts)
    pick = np.sort(np.random.default_rng(1).choice(len(ns), min(sample, len(ns)), replace=False))
    sims = [tg.Simulation(mesh, ps[i], ns[i], seed=int(i), precision=32) for i in pick]
    for s_ in sims:
        s_.start()
        s_.step(16)
    torch.cuda.synchronize()
    steps1 = max(16, steps // 16 * 16)
    t0 = time.perf_counter()
    for s_ in sims:
        s_.step(steps1)
    one_by_one = int(n[pick].sum()) * steps1 / (time.perf_counter() - t0)
    # the same handles' runs enqueued on their own streams without waiting (they may overlap)
    t0 = time.perf_counter()
    for s_ in sims:
        s_.step_async(steps1)
    torch.cuda.synchronize()
    concurrent = int(n[pick].sum()) * steps1 / (time.perf_counter() - t0)
    # the same handles interleaved step by step (one direct launch sequence per replica per step)
    t0 = time.perf_counter()
    for _ in range(8):
        for s_ in sims:
            s_.step_async(1)
    torch.cuda.synchronize()
    interleaved = int(n[pick].sum()) * 8 / (time.perf_counter() - t0)
    for s_ in sims:
        assert s_.status() == 0
        s_.close()
    return {"metric": "particle-steps/s (ragged ensemble, %d replicas)" % len(ns), "value": batched, "unit": UNIT,
            "steps": steps, "ms_per_step": ms / steps,
            "config": {"workload": "ensemble, (4,2,2) ellipsoid L4, N log-uniform [64,8192], eta U[0,2pi], "
                                   "v0 U[0.5,1.5], R 0.05, dt 0.02", "replicas": len(ns), "particles": total,
                       "faces": mesh.F},
            "one_by_one": {"value": one_by_one, "replicas_sampled": len(pick), "steps": steps1,
                           "path": "each sampled replica in its own plain handle, its steps launched as a plain "
                                   "system's (one loop-graph launch), one replica after the other, each run "
                                   "waited for"},
            "concurrent_streams": {"value": concurrent,
                                   "path": "the same handles' runs enqueued on their own streams without waiting"},
            "interleaved_one_by_one": {"value": interleaved, "steps": 8,
                                       "path": "the same handles, one step of each replica in turn"},
            "batched_over_one_by_one": batched / one_by_one,
            "batched_over_concurrent_streams": batched / concurrent,
            "roofline": {"bound": "hbm", "achieved": alg / (k_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                         "frac": alg / (k_ms * 1e-3) / 1e9 / peak,
                         "traffic": profiled_traffic("k_step_ensemble_4096_replicas.md", total),
                         "peak_source": peak_kind,
                         "kernel": "k_step", "kernel_ms": k_ms, "algorithmic_bytes": alg},
            "step_ms_graph_launched": ms / steps, "step_ms_kernels_summed": summed_ms,
            "tuning": sim_tuning, "autotuned": bool(autotune),
            "order_parameter_series": {"steps": int(phi.shape[0]), "replicas": int(phi.shape[1])}}


def _adjoint_common(tg, torch, mesh, target_params, params, ns, seed, T, stride, window):
    """Target run, then the forward (tds_step) and forward+adjoint timings from the same state."""
    ref = tg.Simulation(mesh, target_params, ns, seed=seed, precision=32)
    ref.start()
    s0 = ref.get_state()
    ref.step(T)
    r_star = ref.get_state()["r3d"]
    phi_star = ref.order_parameter()[0][-T:].copy()
    ref.close()
    sim = tg.Simulation(mesh, params, ns, seed=seed, precision=32)

    def reset():
        sim.set_state(s0["uv"], s0["theta"], s0["face"])
        torch.cuda.synchronize()

    reset()
    sim.step(16)  # warm-up (graph capture)
    reset()
    t0 = time.perf_counter()
    sim.step(T)
    fwd_s = time.perf_counter() - t0
    kw = dict(r3d_target=r_star, w_pos=1.0, phi_target=phi_star, w_phi=1.0, checkpoint_stride=stride)
    reset()
    sim.adjoint(T, **kw)  # warm-up: the handle keeps the adjoint's work memory between calls
    reset()
    t0 = time.perf_counter()
    res = sim.adjoint(T, **kw)
    adj_s = time.perf_counter() - t0
    reset()
    win = sim.adjoint(T, window=window, **kw)
    sim.close()
    return fwd_s, adj_s, res, win


def adjoint_leg(tg, T=2000, window=25):
    """Forward+adjoint vs forward (the differentiable-step workload): N = 10,000 particles on the
    (6,3,3) ellipsoid (level-4 icosphere), R = 0.05, FP32, Philox noise fixed by the seed; loss =
    mean |r_T - r*|^2 + sum_t (phi_t - phi*_t)^2 against a target run with (v0 1, k 10, tau 1,
    align 0.5); the differentiated run has v0 1.1, k 9, tau 1.2, align 0.4; T steps with a
    checkpoint every 50."""
    import torch
    mesh = tg.Mesh.ellipsoid(4, (6.0, 3.0, 3.0))
    n = 10000
    fwd_s, adj_s, res, win = _adjoint_common(tg, torch, mesh, tg.Params(v0=1.0, k_rep=10.0, tau=1.0, align=0.5),
                                             tg.Params(v0=1.1, k_rep=9.0, tau=1.2, align=0.4), n, 0, T, 50, window)
    g = res["d_params"]
    return {"metric": "particle-steps/s (forward+adjoint, 10,000-particle differentiable step)",
            "value": n * T / adj_s, "unit": UNIT, "steps": T,
            "config": {"workload": "differentiable step, (6,3,3) ellipsoid L4, 10,000 particles, R 0.05, "
                                   "checkpoint every 50 steps", "particles": n, "steps": T},
            "forward": {"value": n * T / fwd_s, "unit": UNIT, "path": "tds_step (CUDA graphs)"},
            "adjoint_over_forward": adj_s / fwd_s, "loss": res["loss"],
            "finite_gradients": bool(np.isfinite(g).all()),
            "windowed": {"window": window, "finite_gradients": bool(np.isfinite(win["d_params"]).all()),
                         "grad_params": dict(zip(tg.GRAD_PARAMS, [float(x) for x in win["d_params"][0]]))},
            "note": "the exact gradient of the whole run grows ~8x per contact step at these parameters "
                    "(2 dt mu k / 2R = 4) and overflows FP32 after ~40 steps; the windowed (truncated) "
                    "gradient covers the last `window` steps"}


def adjoint_batched_leg(tg, T=500, window=25):
    """Batched adjoint for parameter inference: 512 replicas on the bumpy sphere
    r = 1 + 0.2 Re Y_4^2 scaled x5 (level-6 icosphere), particle counts uniform in [1000, 20000],
    per-replica v0 U[0.5,1.5], k U[5,20], tau U[0.5,2], eta U[0.1,1]; R 0.05, dt 0.02, FP32, T
    steps, checkpoint stride chosen to fit device memory. Target: the same replicas run with v0 1,
    k 10, tau 1, eta 0.5."""
    import torch
    mesh = tg.Mesh.bumpy_sphere(6, 0.2, 5.0)
    rng = np.random.default_rng(5)
    R = 512
    ns = [int(x) for x in rng.integers(1000, 20001, size=R)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(R)]
    fwd_s, adj_s, res, win = _adjoint_common(tg, torch, mesh, [tg.Params(v0=1.0, k_rep=10.0, tau=1.0, eta=0.5)] * R,
                                             ps, ns, 1, T, 0, window)
    total = int(sum(ns))
    g, gw = res["d_params"], win["d_params"]
    return {"metric": "particle-steps/s (forward+adjoint, batched ragged ensemble, 512 replicas)",
            "value": total * T / adj_s, "unit": UNIT, "steps": T,
            "config": {"workload": "batched adjoint, bumpy sphere 1+0.2 Re Y_4^2 x5, L6 icosphere, 512 replicas, "
                                   "N U[1000,20000], per-replica v0/k/tau/eta", "replicas": R, "particles": total,
                       "steps": T, "checkpoint_stride": res["checkpoint_stride"]},
            "forward": {"value": total * T / fwd_s, "unit": UNIT, "path": "tds_step (CUDA graphs)"},
            "adjoint_over_forward": adj_s / fwd_s, "loss": res["loss"],
            "replicas_with_finite_gradients": int(np.isfinite(g).all(1).sum()),
            "windowed": {"window": window, "replicas_with_finite_gradients": int(np.isfinite(gw).all(1).sum())}}


def run_gpu(args):
    import torch
    world, rank, local = dist_setup(args)
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    tg = importlib.import_module("2dtissue_gb300")
    mesh, p, n, prm = workload_1m(tg)
    arrays = mesh.arrays()
    sha = mesh_sha16(arrays)
    if rank == 0 and not os.path.exists(WORKLOAD_MESH):
        save_workload_mesh(tg)
    sim = tg.Simulation(mesh, p, n, seed=rank, precision=32)
    sim.start()
    stream = torch.cuda.ExternalStream(sim.stream())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def flush_l2(k):
        with torch.cuda.stream(stream):
            flush.fill_(k & 255)

    # clocks are sampled from the start of the warm-up (the same steps back to back) to the end of
    # the timed region, so that a short timed region still has samples under the same load
    clk = Clocks(local)
    for k in range(args.warmup):
        sim.step_async(16)
    torch.cuda.synchronize()
    assert sim.status() == 0, "device status set during warm-up"

    # ---- timed region: K steps back to back, launched as the library launches them; the per-step
    # working set (state, its sorted copy, cell tables, cell descriptors, face records: ~220 MB) is
    # larger than the 126 MB L2, so no flush ----
    ga, gb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    ga.record(stream)
    sim.step_async(args.steps)
    gb.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = clk.stop()
    total_ms = ga.elapsed_time(gb)
    status = sim.status()
    if status:
        raise SystemExit("device status 0x%x in the timed region" % status)
    total_ms = allreduce_max(total_ms, world)
    value = world * n * args.steps / (total_ms * 1e-3)

    # ---- per-kernel events over the same K steps launched one by one (no graphs): the dominant
    # kernel's duration for the roofline, and each kernel's share of the step ----
    sim.kernel_timing(True)
    sim.step_async(args.steps)
    torch.cuda.synchronize()
    kt = sim.kernel_times()
    sim.kernel_timing(False)
    step_ms, step_n = kt["step"]
    avg_s = step_ms * 1e-3 / max(step_n, 1)
    alg = ALG_BYTES_PARTICLE * n + ALG_BYTES_FACE * mesh.F + ALG_BYTES_REPLICA
    peak, peak_kind = measured_peak()
    achieved = alg / avg_s / 1e9
    traffic = profiled_traffic("k_step_1m_particles.md", n)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": peak_kind, "kernel": "k_step",
                "kernel_ms": avg_s * 1e3, "algorithmic_bytes": alg}
    step_frac = alg / (total_ms * 1e-3 / args.steps) / 1e9 / peak
    shares = {k: v[0] / max(1e-12, sum(x[0] for x in kt.values())) for k, v in kt.items()}

    # ---- each step after a 256 MB L2 flush, event-timed per step (informational) ----
    fl_steps = min(args.steps, 50)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(fl_steps)]
    for k in range(fl_steps):
        flush_l2(k + 7)
        ev[k][0].record(stream)
        sim.step_async(1)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    flushed_ms = allreduce_max(sum(a.elapsed_time(b) for a, b in ev), world)
    flushed_rate = world * n * fl_steps / (flushed_ms * 1e-3)

    # ---- end to end through the C-ABI with pinned host buffers ----
    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    # the step's input state: chart position, polarity angle and face (the 3D position is the
    # face's chart map of the chart position; tds_set_state derives it on the device when r3d is
    # NULL, bit for bit as the step computes it)
    hin = sim.get_state()
    e2e_steps = 100  # the loop's own sample: long enough that host-side jitter averages out

    def end_to_end(fdt):
        """Per step: state upload, one step, state download, through the state views of float
        type fdt (torch.float32: tds_*_state_f32*, the FP32 state as it is; torch.float64: the
        double views). Returns (pipelined s, synchronous s, H2D bytes, D2H bytes)."""
        pin_in = dict(uv=pinned((n, 2), fdt), theta=pinned((n,), fdt), face=pinned((n,), torch.int32))
        for k in pin_in:
            pin_in[k][...] = hin[k]  # FP32 state values: exact in either type
        out_types = dict(uv=((n, 2), fdt), theta=((n,), fdt), face=((n,), torch.int32), r3d=((n, 3), fdt),
                         vel_uv=((n, 2), fdt), nbr=((n,), torch.int32))
        pin_out = {k: pinned(*v) for k, v in out_types.items()}
        pin_out2 = {k: pinned(*v) for k, v in out_types.items()}
        h2d = int(sum(v.nbytes for v in pin_in.values()))
        d2h = int(sum(v.nbytes for v in pin_out.values()))
        # synchronous: each call returns when its transfer is done
        sim.set_state(**pin_in)
        sim.step(1)
        sim.get_state(pin_out)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.set_state(**pin_in)
            sim.step(1)
            sim.get_state(pin_out)
        sync_s = allreduce_max(time.perf_counter() - t0, world)
        # pipelined: the same calls enqueued; step k+1's upload overlaps step k's download
        # (host outputs double-buffered, as a caller consuming the results would)
        sim.set_state_async(**pin_in)
        sim.step_async(1)
        sim.get_state_async(pin_out)
        sim.sync()
        barrier(world)
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            sim.set_state_async(**pin_in)
            sim.step_async(1)
            sim.get_state_async(pin_out if k % 2 == 0 else pin_out2)
        sim.sync()
        return allreduce_max(time.perf_counter() - t0, world), sync_s, h2d, d2h

    e2e_s, sync_s, h2d_bytes, d2h_bytes = end_to_end(torch.float32)
    d_s, d_sync_s, d_h2d, d_d2h = end_to_end(torch.float64)
    e2e = {"value": world * n * e2e_steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes, "steps": e2e_steps,
           "path": "per step: tds_set_state_f32_async of uv, theta, face (pinned H2D, upload stream; r3d derived "
                   "on the device) + tds_step_async + tds_get_state_f32_async of uv, theta, face, r3d, vel_uv, nbr "
                   "(pinned D2H, download stream); tds_sync after the last step. The FP32 views carry the FP32 "
                   "state exactly (the double views return the same values widened)",
           "synchronous": {"value": world * n * e2e_steps / sync_s, "unit": UNIT,
                           "path": "tds_set_state_f32 + tds_step + tds_get_state_f32, each waiting"},
           "double_views": {"value": world * n * e2e_steps / d_s, "unit": UNIT, "h2d_bytes_per_step": d_h2d,
                            "d2h_bytes_per_step": d_d2h, "synchronous": world * n * e2e_steps / d_sync_s,
                            "path": "the same loop through tds_set_state_async / tds_get_state_async (double "
                                    "arrays, the reference's type)"}}
    # the step kernels, plus the loop graph's own: k_loop_set and k_loop_arm once per run, k_loop_ctl
    # once per pass of each WHILE loop (blocks of 16 steps, then single steps)
    launches = sim.kernels_per_step() * args.steps
    if args.steps >= 2 and sim.tuning()["graph_steps"] == 0:
        launches += 2 + args.steps // 16 + args.steps % 16
    final = sim.get_state()
    sim.close()

    # ---- the rest of the metric: batched vs plain, forward+adjoint (rank 0, one GPU) ----
    extra = {}
    if rank == 0 and world == 1 and not args.plain_only:
        extra["ensemble"] = ensemble_leg(tg)
        extra["adjoint"] = adjoint_leg(tg)
        extra["adjoint_batched"] = adjoint_batched_leg(tg)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        rate, sample, cores, one = oracle_cpu_rate(arrays, prm, final, n)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample, "one_core": one}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded placement)",
                "config": workload_config(mesh.F, prm, sha), "state": "fp32 SoA on the device",
                "l2": "inputs larger than L2: ~220 MB touched per step vs 126 MB L2; steps back to back, no flush",
                "roofline": roofline, "step_hbm_frac": step_frac, "kernel_share": shares,
                "flushed_per_step": {"value": flushed_rate, "unit": UNIT, "steps": fl_steps,
                                     "note": "each step after a 256 MB L2 flush, event-timed per step"},
                "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clocks,
                "parallelism": "replicas only (one independent 1M-particle system per GPU)"}
        line.update(extra)
        print(json.dumps(line), flush=True)


def _print_leg(leg, args):
    line = dict(leg)
    line.update({"n_gpus": 1, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
                 "data": "synthetic (seeded)"})
    print(json.dumps(line), flush=True)


def run_ref(args):
    """Reference-semantics step (tds_ref_*: the reference's own algorithm, FP64) on the (2,1,1)
    ellipsoid (level-4 icosphere): 100 particles with the 100-particle system's values (R 0.05,
    k 10, v0 1, dt 0.02) and 2,000 particles with the reference's constructor defaults, `steps`
    steps each (default 50), against the oracle's ref-form step on one host core (the reference is
    single-threaded) over a bounded sample of steps."""
    import torch
    tg = importlib.import_module("2dtissue_gb300")
    import oracle
    mesh = tg.Mesh.ellipsoid(4, (2.0, 1.0, 1.0))
    a = mesh.arrays()
    D = tg.ref_vertex_distances(mesh)
    T = args.steps
    cases = [("100 particles, R 0.05, k 10, v0 1, dt 0.02", 100,
              dict(v0=1.0, k=10.0, sigma=0.05, r_adh=0.12, k_adh=0.75, step_size=0.02)),
             ("2,000 particles, reference ctor defaults", 2000,
              dict(v0=0.1, k=1.0, sigma=0.41667, r_adh=1.0, k_adh=0.75, step_size=0.001))]
    out = []
    for name, n, prm in cases:
        sim = tg.RefSimulation(mesh, tg.RefParams(**prm), n, seed=0, vertex_dist=D)
        sim.start()
        sim.step(max(args.warmup, 3))
        s0 = sim.get_state()
        stream = torch.cuda.ExternalStream(sim.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.step(T)
        e1.record(stream)
        torch.cuda.synchronize()
        gpu_rate = n * T / (e0.elapsed_time(e1) * 1e-3)
        sim.close()
        st = dict(uv=s0["uv"], n_deg=s0["n_deg"], nearest=s0["nearest"])
        k, t0 = 0, time.perf_counter()
        while k < T and time.perf_counter() - t0 < 15.0:
            o = oracle.ref_step(a, D, prm, st["uv"], st["n_deg"], st["nearest"])
            st = dict(uv=o["uv"], n_deg=o["n_deg"], nearest=o["nearest"])
            k += 1
        cpu_rate = n * k / (time.perf_counter() - t0)
        out.append({"case": name, "particles": n, "steps": T, "value": gpu_rate, "unit": UNIT,
                    "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": 1, "kind": "port",
                                     "sample": "%d steps of the ref-form oracle step (orc_ref_step)" % k},
                    "gpu_over_cpu": gpu_rate / cpu_rate})
    line = {"metric": "particle-steps/s (reference-semantics step, FP64)", "value": out[0]["value"], "unit": UNIT,
            "n_gpus": 1, "steps": T, "warmup": args.warmup, "higher_is_better": True, "dtype": "f64",
            "data": "synthetic (seeded centroid placement)",
            "config": {"workload": "reference-semantics step, (2,1,1) ellipsoid L4 (Vuv %d, F %d)" % (mesh.Vuv, mesh.F)},
            "cases": out}
    print(json.dumps(line), flush=True)


def run_profile_adjoint(args):
    """Minimal driver for ncu: the 512-replica bumpy-sphere ensemble of the batched-adjoint workload,
    placed, then one adjoint run of `steps` steps (one stored segment); no timing."""
    import torch
    tg = importlib.import_module("2dtissue_gb300")
    mesh = tg.Mesh.bumpy_sphere(6, 0.2, 5.0)
    rng = np.random.default_rng(5)
    R = 512
    ns = [int(x) for x in rng.integers(1000, 20001, size=R)]
    ps = [tg.Params(v0=float(rng.uniform(0.5, 1.5)), k_rep=float(rng.uniform(5, 20)), tau=float(rng.uniform(0.5, 2)),
                    eta=float(rng.uniform(0.1, 1.0))) for _ in range(R)]
    sim = tg.Simulation(mesh, ps, ns, seed=1, precision=32, tuning=PROFILE_TUNING)
    sim.start()
    s0 = sim.get_state()
    T = args.steps
    sim.adjoint(T, r3d_target=s0["r3d"], w_pos=1.0, phi_target=np.full((T, R), 0.05), w_phi=1.0)
    torch.cuda.synchronize()
    sim.close()


# ncu cannot profile the kernel nodes of a graph that holds conditional nodes (the loop graph), so
# the profiling drivers launch the steps as graphs of 16 steps (the same kernels)
PROFILE_TUNING = dict(cells_per_particle=4.0, step_block=128, graph_steps=16, lanes_per_particle=1)


def run_profile(args):
    """Minimal driver for ncu: the 1M-particle system, `warmup` steps, then `steps` steps (graphs of
    16 steps; `--lanes` lanes per particle); no timing."""
    import torch
    tg = importlib.import_module("2dtissue_gb300")
    mesh, p, n, _ = workload_1m(tg)
    sim = tg.Simulation(mesh, p, n, seed=0, precision=32, tuning=dict(PROFILE_TUNING, lanes_per_particle=args.lanes))
    sim.start()
    sim.step(args.warmup)
    sim.step_async(args.steps)
    torch.cuda.synchronize()
    assert sim.status() == 0
    sim.close()


def run_profile_ensemble(args):
    """Minimal driver for ncu: the 4,096-replica ensemble of the ensemble leg, placed, `warmup` steps,
    then `steps` steps (graphs of 16 steps); no timing."""
    import torch
    tg = importlib.import_module("2dtissue_gb300")
    ens = importlib.import_module("2dtissue_gb300.ensemble")
    mesh = tg.Mesh.ellipsoid(4, (4.0, 2.0, 2.0))
    n, eta, v0 = ens.ragged_replicas(seed=0, n_replicas=4096)
    ps = [tg.Params(radius=0.05, r_max=0.12, v0=float(v), eta=float(e), dt=0.02) for e, v in zip(eta, v0)]
    sim = tg.Simulation(mesh, ps, [int(x) for x in n], seed=0, precision=32, tuning=PROFILE_TUNING)
    sim.start()
    sim.step(args.warmup)
    sim.step_async(args.steps)
    torch.cuda.synchronize()
    assert sim.status() == 0
    sim.close()


def run_profile_e2e(args):
    """Minimal driver for ncu: the 1M-particle system, then `steps` iterations of the end-to-end loop
    (pinned FP32-view upload of uv, theta, face; one step; pinned FP32-view download); no timing."""
    import torch
    tg = importlib.import_module("2dtissue_gb300")
    mesh, p, n, _ = workload_1m(tg)
    sim = tg.Simulation(mesh, p, n, seed=0, precision=32, tuning=PROFILE_TUNING)
    sim.start()
    sim.step(args.warmup)
    hin = sim.get_state(dtype=np.float32)

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
        return t.numpy()
    pin_in = {k: pinned(hin[k]) for k in ("uv", "theta", "face")}
    for k in pin_in:
        pin_in[k][...] = hin[k]
    outs = [{k: pinned(v) for k, v in hin.items()} for _ in range(2)]
    for k in range(args.steps):
        sim.set_state_async(**pin_in)
        sim.step_async(1)
        sim.get_state_async(outs[k % 2])
    sim.sync()
    sim.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: plain 500, ensemble 50, adjoint 2000, adjoint_batched 500, ref 50)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--plain-only", action="store_true", help="only the headline plain-step leg")
    ap.add_argument("--lanes", type=int, default=1, choices=[1, 2, 4],
                    help="with --profile (plain workload): lanes per particle of the step kernel")
    ap.add_argument("--profile", action="store_true", help="only run warmup + steps (for ncu)")
    ap.add_argument("--e2e", action="store_true", help="with --profile: steps iterations of the end-to-end loop")
    ap.add_argument("--workload", default="plain", choices=["plain", "ensemble", "adjoint", "adjoint_batched", "ref"])
    ap.add_argument("--replicas", type=int, default=4096, help="ensemble workload: replicas")
    ap.add_argument("--sample", type=int, default=64, help="ensemble workload: replicas run one by one")
    ap.add_argument("--autotune", action="store_true", help="ensemble workload: time the autotuner's choice")
    ap.add_argument("--write-workload-mesh", action="store_true", help="write the headline mesh's arrays and exit")
    args = ap.parse_args()
    if args.write_workload_mesh:
        save_workload_mesh(importlib.import_module("2dtissue_gb300"))
        return
    if args.steps is None:
        args.steps = {"plain": 500, "ensemble": 50, "adjoint": 2000, "adjoint_batched": 500, "ref": 50}[args.workload]
    if args.profile:
        if args.e2e:
            return run_profile_e2e(args)
        if args.workload == "ensemble":
            return run_profile_ensemble(args)
        return run_profile_adjoint(args) if args.workload == "adjoint_batched" else run_profile(args)
    if args.impl != "reference":
        tg = None
        if args.workload != "plain":
            tg = importlib.import_module("2dtissue_gb300")
        if args.workload == "ensemble":
            return _print_leg(ensemble_leg(tg, args.steps, args.sample, args.autotune, args.replicas), args)
        if args.workload == "adjoint":
            return _print_leg(adjoint_leg(tg, args.steps), args)
        if args.workload == "adjoint_batched":
            return _print_leg(adjoint_batched_leg(tg, args.steps), args)
        if args.workload == "ref":
            return run_ref(args)
    if args.warmup < 3 and args.impl != "reference":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
