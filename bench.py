#!/usr/bin/env python
"""Benchmark of the CGFD3D time-stepping hot path on GB300.

Metric: grid-point RK-stage updates per second (N_phys * 4 * steps / time).
Default workload: the curvilinear-topography isotropic model (400 x 400 x
200 physical points, CFS-PML 12 layers on five faces, traction-image free
surface, a double-couple source and 400 surface receivers), synthetic and
seeded.  --workload vti / visco run the same topography at 300 x 300 x 150
with a VTI or a GMB visco-elastic (3 Maxwell bodies) medium; --workload flat
the 100 x 100 x 60 flat model.

One "step" is one RK4 time step (four stage kernels, the CFS-PML face
kernels, the surface and receiver kernels) of the whole model, with every
input resident in HBM (several GB, far larger than the 129 MB L2, so no
flush is needed between steps).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload topo|vti|visco|flat]

Multi-GPU runs (torchrun, one rank per GPU) are independent replicas of the
whole model: the single-domain path keeps the domain on one GPU, so ranks
share nothing but the barrier and the max-over-ranks timing.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "grid-pt RK-stage updates/s"
UNIT = "pt-stage/s"
# algorithmic HBM bytes per point-stage, RK-stage average: wavefield
# components (stage 0: pre r, tmp w, end w; stages 1-2: cur, pre, end r, tmp,
# end w; stage 3: cur, end r, end w) plus the per-point coefficients (9
# metrics + media), float32.  iso 36+12, vti 36+15, visco 108+18 floats.
BYTES_PER_PT_STAGE = {"topo": 192, "flat": 192, "vti": 204, "visco": 504, "aniso": 268}
WORKLOADS = {"topo": dict(ni=400, nj=400, nk=200),
             "slices": dict(ni=400, nj=400, nk=200),
             "locate": dict(ni=400, nj=400, nk=200),
             "media": dict(ni=400, nj=400, nk=200),
             "media_bin": dict(ni=400, nj=400, nk=200),
             "batch": dict(ni=400, nj=400, nk=200),
             "vti": dict(ni=300, nj=300, nk=150),
             "aniso": dict(ni=300, nj=300, nk=150),
             "visco": dict(ni=300, nj=300, nk=150),
             "flat": dict(ni=100, nj=100, nk=60),
             "surrogate": dict(ni=256, nj=256, nk=128),
             "surrogate_net": dict(ni=256, nj=256, nk=128)}
SAMPLE_NK = 24                 # CPU sample: same model, 24 planes deep
CPU_SAMPLE_S = 24.0            # target seconds of CPU work per baseline sample


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--media-method", default="har", choices=["loc", "har", "ari"],
                    help="equivalent-medium method of --workload media")
    ap.add_argument("--workload", default="topo", choices=sorted(WORKLOADS))
    ap.add_argument("--nshot", type=int, default=64,
                    help="batch workload: shots per GPU")
    ap.add_argument("--sg-train", type=int, default=448,
                    help="surrogate workload: training shots")
    ap.add_argument("--sg-test", type=int, default=64,
                    help="surrogate workload: held-out shots")
    ap.add_argument("--sg-iters", type=int, default=3000,
                    help="surrogate workload: training steps (batch 256)")
    ap.add_argument("--ni", type=int, default=None)
    ap.add_argument("--nj", type=int, default=None)
    ap.add_argument("--nk", type=int, default=None)
    a = ap.parse_args()
    for k in ("ni", "nj", "nk"):
        if getattr(a, k) is None:
            setattr(a, k, WORKLOADS[a.workload][k])
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peak_hbm():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_ratio(workload):
    """DRAM traffic over algorithmic bytes of the stage kernel, from the
    committed ncu capture of a smaller case of the same kernel
    (profiles/k_stage_<workload>_traffic.json), or None."""
    name = "topo" if workload in ("topo", "flat") else workload
    path = os.path.join(REPO, "profiles", "k_stage_%s_traffic.json" % name)
    try:
        with open(path) as f:
            return float(json.load(f)["measured_over_algorithmic"])
    except (OSError, KeyError, ValueError):
        return None


# CFS-PML auxiliaries per face point per RK stage, stage average: stage 0
# reads cur and writes tmp, end (27 floats), stages 1-2 read cur, pre, end
# and write tmp, end (45), stage 3 reads cur, end and writes end (27)
PML_AUX_BYTES = 144


def face_points(p):
    n = 0
    for row in p.pml:
        for f in row:
            if f is not None:
                b = f["box"]
                n += int((b[1] - b[0] + 1) * (b[3] - b[2] + 1) * (b[5] - b[4] + 1))
    return n


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def build_model(args, steps, nk=None):
    from cgfd3d_gb300 import models
    nk = nk or args.nk
    if args.workload == "flat":
        return models.flat_model(ni=args.ni, nj=args.nj, nk=nk, steps=steps)
    if args.workload in ("vti", "visco", "aniso"):
        return models.topo_media_model(args.workload, ni=args.ni, nj=args.nj,
                                       nk=nk, steps=steps, dt=0.005, nrecv=400)
    return models.topo_model(ni=args.ni, nj=args.nj, nk=nk, steps=steps,
                             dt=0.01, nrecv=400)


def workload_name(args):
    return {"topo": "topography iso %dx%dx%d, CFS-PML 12 on 5 faces, timg free "
                    "surface, DC point source, 400 receivers",
            "vti": "topography VTI %dx%dx%d (Thomsen eps,delta,gamma, 5%% GRF), "
                   "CFS-PML 12, timg free surface, DC source, 400 receivers",
            "visco": "topography visco-elastic GMB 3 bodies %dx%dx%d (Qp 200, Qs "
                     "100), CFS-PML 12, timg free surface, DC source, 400 receivers",
            "aniso": "topography tilted TI %dx%dx%d (21 constants; VTI of the vti "
                     "workload tilted 30+-10 deg), CFS-PML 12, timg free surface, DC "
                     "source, 400 receivers",
            "flat": "flat iso %dx%dx%d, CFS-PML 10, timg free surface, explosive "
                    "source, 20 receivers"}[
                "topo" if args.workload == "slices" else args.workload] % (
                args.ni, args.nj, args.nk)


def host_link_gbs(nbytes=1 << 30):
    """Copy-engine rate of the host link (pinned host memory <-> HBM, GB/s),
    the floor under the end-to-end number's transfers."""
    import torch
    h = torch.empty(nbytes // 4, dtype=torch.float32, pin_memory=True)
    d = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
    h.fill_(1.0)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    out = {}
    for name, dst, src in (("h2d", d, h), ("d2h", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(3):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        out[name] = 3 * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
    del h, d
    return out


def pin_problem(p):
    """Move the large host arrays of a problem into pinned memory."""
    import numpy as np
    import torch

    holders = []

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
        holders.append(t)           # the tensor owns the pinned pages
        out = t.numpy()
        out[:] = a.ravel()
        return out

    for k in list(p.metric):
        p.metric[k] = pinned(p.metric[k])
    for k in list(p.media):
        p.media[k] = pinned(p.media[k])
    p.Ylam = [pinned(a) for a in p.Ylam]
    p.Ymu = [pinned(a) for a in p.Ymu]
    p.wav = pinned(p.wav)
    for row in p.pml:
        for f in row:
            if f is not None:
                f["aux"] = pinned(f["aux"])
    return holders


def cpu_rate(args, steps, threads):
    """Oracle (CPU port of the reference path) on a bounded sample: `steps`
    RK4 steps of the workload's model cut to SAMPLE_NK planes."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    oracle.build()
    p = build_model(args, steps - 1, nk=min(SAMPLE_NK, args.nk))
    t0 = time.perf_counter()
    oracle.allstep(p, oracle.TIMG_ZERO, threads)
    t = time.perf_counter() - t0
    n = p.ni * p.nj * p.nk * 4 * p.nt_total
    return n / t, t, p


def cpu_sample(args, threads):
    """CPU baseline sized to about CPU_SAMPLE_S seconds: one step to gauge
    the rate, then as many steps as fit.  Returns (rate, seconds, steps)."""
    r1, t1, _ = cpu_rate(args, 1, threads)
    steps = max(1, min(400, int(math.ceil(CPU_SAMPLE_S / max(t1, 1e-3)))))
    r, t, _ = cpu_rate(args, steps, threads)
    return r, t, steps


def run_reference_batch(args):
    """CPU reference arm of the batch workload: RK4 steps of one window shot
    with the C port on all host threads, converted to shots/s at 1000 steps
    per shot."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from cgfd3d_gb300 import models
    threads = os.cpu_count() or 1
    base = models._topo_base(args.ni, args.nj, args.nk, 2024)
    p = models.window_shots(1, base=(args.ni, args.nj, args.nk), steps=1,
                            base_model=base, seed=3000)[0]
    del base
    oracle.allstep(p.copy(), oracle.TIMG_ZERO, threads)      # warm-up
    ts = []
    for _ in range(max(args.steps, 1)):
        q = p.copy()
        t0 = time.perf_counter()
        oracle.allstep(q, oracle.TIMG_ZERO, threads)
        ts.append((time.perf_counter() - t0) / q.nt_total)
    step_s = sum(ts) / len(ts)
    rate = 1.0 / (step_s * 1000.0)
    sample = ("%d RK4 steps of one %dx%dx%d window shot per timed step, C oracle "
              "port, %d threads" % (p.nt_total, p.ni, p.nj, p.nk, threads))
    line = {"impl": "reference", "metric": "shots/s (1000 RK4 steps per shot)",
            "value": rate, "unit": "shots/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step_s,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded window shots)",
            "config": {"workload": "batched shots (CPU: one window at a time)"},
            "cpu_baseline": {"value": rate, "unit": "shots/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": "shots/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    if args.workload == "batch":
        return run_reference_batch(args)
    if args.workload == "locate":
        return run_locate(args, reference=True)
    if args.workload == "media":
        return run_media(args, reference=True)
    if args.workload == "media_bin":
        return run_media_bin(args, reference=True)
    threads = os.cpu_count() or 1
    # warm-up sample, then the timed samples (one RK4 step each)
    cpu_rate(args, 1, threads)
    rates, tot = [], 0.0
    for _ in range(max(args.warmup, 0)):
        cpu_rate(args, 1, threads)
    for _ in range(args.steps):
        r, t, p = cpu_rate(args, 1, threads)
        rates.append(r)
        tot += t
    rate = args.steps / sum(1.0 / r for r in rates)
    # the reference itself is single-threaded: the same sample on one thread
    r1, t1, _ = cpu_rate(args, 1, 1)
    nk_cut = min(SAMPLE_NK, args.nk)
    sample = ("one RK4 step per timed step of the %s model (same generator, "
              "nk cut to %d), C oracle port, %d threads" %
              (args.workload, nk_cut, threads))
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": workload_name(args) + (
            " -- CPU arm: the C port of the reference path (bit-identical to the "
            "reference build), %d threads, on the model cut to nk=%d (rate per "
            "point-stage; the reference sources are not on the GPU machine)"
            % (threads, nk_cut)),
            "same_config": False},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": sample,
                         "single_thread": {"value": r1, "unit": UNIT, "cores": 1,
                                           "seconds": t1}},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cgfd3d_gb300 import solver

    K, W = args.steps, max(args.warmup, 0)
    p = build_model(args, K + W)
    n_phys = p.ni * p.nj * p.nk

    # ---- device-resident timing ------------------------------------------
    s = solver.Solver(p)
    s.run(W)
    s.set_timing(True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.6)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    s.run(K)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    (t_stage, t_total, _), (n_stage, n_all, _) = s.kernel_times()
    s.check_finite()
    s.close()
    t = t_total * 1e-3
    if world > 1:
        tt = torch.tensor([t], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    value = world * n_phys * 4 * K / t

    # ---- roofline of the stage kernel -----------------------------------
    peak, peak_kind = measured_peak_hbm()
    avg_launch = t_stage * 1e-3 / n_stage
    bpps = BYTES_PER_PT_STAGE[args.workload]
    alg_bytes = n_phys * bpps
    achieved = alg_bytes / avg_launch / 1e9
    nface = face_points(p)
    alg_aux = alg_bytes + nface * PML_AUX_BYTES
    ratio = traffic_ratio(args.workload)

    # ---- end to end through the C ABI with host (pinned) buffers ---------
    q = build_model(args, K - 1)
    pinned_owner = pin_problem(q)
    # one small call first so that module loading is not timed
    from cgfd3d_gb300 import models
    solver.drv_rk_curv_col_allstep(models.topo_model(ni=48, nj=48, nk=40, steps=1,
                                                     dt=0.01, nrecv=4))
    if world > 1:
        torch.distributed.barrier()
    # three end-to-end runs of the same problem (each from host buffers to
    # host buffers), the median reported: host-side copies vary from run to run
    reps, phases = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        se = solver.Solver(q)
        t1 = time.perf_counter()
        se.run(q.nt_total)
        t2 = time.perf_counter()
        se.fetch()
        t3 = time.perf_counter()
        h2d, d2h = se.transfer_bytes()
        se.close()
        t4 = time.perf_counter()
        reps.append(t4 - t0)
        phases.append({"create": t1 - t0, "run": t2 - t1, "fetch": t3 - t2, "close": t4 - t3})
    t_e2e = sorted(reps)[1]
    mid = phases[reps.index(t_e2e)]
    link = host_link_gbs()
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())
    e2e = world * n_phys * 4 * q.nt_total / t_e2e

    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": 1e3 * t / K,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": workload_name(args),
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs (%.1f GB resident) larger than L2, no flush"
                         % (solver.device_bytes(p) / 1e9)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": None if ratio is None else ratio * alg_aux,
                     "traffic_basis": "DRAM/algorithmic ratio of the committed "
                                      "ncu capture (256x256x96 case) times this "
                                      "launch's algorithmic bytes incl. PML aux",
                     "alg_bytes_per_launch": alg_bytes,
                     "alg_bytes_per_launch_incl_pml_aux": alg_aux,
                     "achieved_incl_pml_aux": alg_aux / avg_launch / 1e9,
                     "pml_face_points": nface,
                     "avg_launch_ms": avg_launch * 1e3,
                     "kernel": "k_stage3 (stage kernel with fused CFS-PML)",
                     "whole_step_frac": value / world * bpps / 1e9 / peak},
        "e2e": {"value": e2e, "unit": UNIT,
                "h2d_bytes_per_step": h2d / q.nt_total,
                "d2h_bytes_per_step": d2h / q.nt_total,
                "steps": q.nt_total, "runs_ms": [1e3 * t for t in reps],
                "reported": "median of 3 runs",
                "phases_ms": {k: 1e3 * v for k, v in mid.items()},
                "host_link_gbs": link,
                "transfer_floor_ms": 1e3 * (h2d / (link["h2d"] * 1e9) +
                                            d2h / (link["d2h"] * 1e9))},
        "gpu_launches": n_all,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        r, tcpu, nst = cpu_sample(args, threads)
        line["cpu_baseline"] = {
            "value": r, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%d RK4 steps of the same model cut to nk=%d, C oracle "
                      "port, %d threads, %.1f s" % (nst, min(SAMPLE_NK, args.nk),
                                                    threads, tcpu)}
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_batch(args):
    """Batched shots (config 3): `nshot` shots per GPU on windows of the
    topography model, 1000 RK4 steps per shot by definition of the metric;
    K timed steps of the whole batch against the same shots run one at a
    time.  Ranks shard shots (disjoint seeds), no collective until the end."""
    import torch
    from cgfd3d_gb300 import _lib, models, solver
    import ctypes as C
    rank, world, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    K, W = args.steps, max(args.warmup, 0)
    base = models._topo_base(args.ni, args.nj, args.nk, 2024)
    probs = models.window_shots(args.nshot, base=(args.ni, args.nj, args.nk),
                                steps=max(W + K, 8), base_model=base,
                                seed=3000 + 1009 * rank)
    pts = sum(p.ni * p.nj * p.nk for p in probs)
    b = solver.Batch(probs)
    cache = os.path.join(REPO, "cgfd3d_gb300", "_build", "batch_tune.json")
    key = "iso:%d:%d" % (args.nshot, pts)
    tune = b.autotune(candidates=(16, 24, 32, 48, 64, 96, 160), steps=2, cache=cache,
                     key=key)
    b.run(W)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.4)
    if world > 1:
        torch.distributed.barrier()
    b.run(K)
    ms, launches = b.times()
    clocks = sampler.stop()
    # the same shots one at a time (each shot's own solver, same kernels)
    b.reset()
    L = _lib.lib()
    t_seq = 0.0
    for k in range(len(probs)):
        h = L.cgfd_batch_shot(b._h, k)
        _lib.check(L.cgfd_solver_run(h, W))
        _lib.check(L.cgfd_solver_run(h, K))
        t = (C.c_float * 3)()
        n = (C.c_int * 3)()
        _lib.check(L.cgfd_solver_kernel_times(h, t, n))
        t_seq += t[1]
    b.close()
    del probs
    t = ms * 1e-3
    if world > 1:
        tt = torch.tensor([t, t_seq * 1e-3], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t, tseq = float(tt[0]), float(tt[1])
    else:
        tseq = t_seq * 1e-3
    step_s = t / K
    shots_per_s = world * args.nshot / (step_s * 1000.0)
    seq_shots_per_s = world * args.nshot / (tseq / K * 1000.0)
    # end to end: upload + K steps + fetch of every shot, host buffers
    q = models.window_shots(args.nshot, base=(args.ni, args.nj, args.nk), steps=K,
                            base_model=base, seed=3000 + 1009 * rank)
    t0 = time.perf_counter()
    be = solver.Batch(q, kchunk=tune["kchunk"])
    be.set_schedule(tune.get("persistent", 0))
    be.run(K)
    be.fetch()
    be.close()
    t_e2e = time.perf_counter() - t0
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())
    h2d = sum(4 * (p.ncmp + 13) * p.vol for p in q)
    d2h = sum(4 * (p.ncmp * p.vol + p.recv["n"] * p.recv["ncmp"] * p.recv["max_nt"]) for p in q)
    if rank != 0:
        return 0
    peak, peak_kind = measured_peak_hbm()
    alg = pts * 4 * BYTES_PER_PT_STAGE["topo"] / step_s / 1e9   # per GPU
    line = {
        "metric": "shots/s (1000 RK4 steps per shot)", "value": shots_per_s,
        "unit": "shots/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * step_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded window shots of the topography model)",
        "config": {"workload": "batched shots: %d iso windows per GPU (128-256 x "
                   "128-256 x 96-160) of the %dx%dx%d topography model, random DC "
                   "moment tensors, Ricker 2 Hz, 64 receivers each"
                   % (args.nshot, args.ni, args.nj, args.nk),
                   "points_per_gpu": pts, "kchunk": tune["kchunk"],
                   "schedule": "persistent CTAs, items largest first"
                               if tune.get("persistent", 0) else "one CTA per item",
                   "autotune_ms": tune["ms"],
                   "autotune_ms_persistent": tune.get("ms_persistent"),
                   "parallelism": "shots sharded" if world > 1 else "single",
                   "l2": "inputs far larger than L2, no flush"},
        "sequential": {"value": seq_shots_per_s, "unit": "shots/s",
                       "how": "the same shots one at a time, same kernels"},
        "batched_over_sequential": shots_per_s / seq_shots_per_s,
        "pt_stage_per_s": world * pts * 4 / step_s,
        "roofline": {"bound": "hbm", "achieved": alg, "peak": peak, "unit": "GB/s",
                     "frac": alg / peak, "peak_kind": peak_kind, "traffic": None,
                     "basis": "whole step: 192 B per point-stage of every shot"},
        "e2e": {"value": args.nshot * world / (t_e2e * 1000.0 / K), "unit": "shots/s",
                "h2d_bytes_per_step": h2d / K, "d2h_bytes_per_step": d2h / K,
                "how": "create (upload) + K steps + fetch, charged to K steps"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_slices(args):
    """Time loop with slice output every step, as a run with slices in its
    parameter file does: three slices (x and y through the middle, z at the
    free surface) of the 9 components copied to a host state buffer after
    every step, packed on the device and handed out while the device runs
    the next step: as arrays in the writers' order (the headline), scattered
    into a host state buffer (what the drop-in hands the reference's
    writers); against the scatter without overlap, against copying the whole
    state, and against stepping with no output."""
    import numpy as np
    import torch
    rank, world, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from cgfd3d_gb300 import output, solver
    K, W = args.steps, max(args.warmup, 0)
    p = build_model(args, 5 * (K + W))
    n_phys = p.ni * p.nj * p.nk
    boxes = output.slice_boxes(p, x=[(p.ni1 + p.ni2) // 2], y=[(p.nj1 + p.nj2) // 2],
                               z=[p.nk2])
    nfl = sum((b.c2 - b.c1 + 1) * b.ni * b.nj * b.nk for b in boxes)
    w = np.zeros((p.ncmp, p.nz, p.ny, p.nx), np.float32)
    s = solver.Solver(p)

    def loop(mode, n):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if mode.startswith("overlap"):   # step n+1 runs while step n is handed out
            dst = w if mode == "overlap_scatter" else None
            slot = 0
            for it in range(n):
                s.run_async(1)
                s.pack_boxes_async(boxes, slot)
                if it > 0:
                    s.collect_boxes(slot ^ 1, dst)
                slot ^= 1
            if n > 0:
                s.collect_boxes(slot ^ 1, dst)
            s.run(0)
        for _ in range(0 if mode.startswith("overlap") else n):
            s.run(1)
            if mode == "packed":
                s.fetch_boxes(boxes, w)
            elif mode == "whole":
                s.fetch_state(w)
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    sampler = ClockSampler(local)
    res = {}
    for mode in ("overlap_arrays", "overlap_scatter", "packed", "whole", "none"):
        loop(mode, W)
        if mode == "overlap_arrays":
            sampler.start()
            time.sleep(0.6)
        res[mode] = loop(mode, K) / K
        if mode == "overlap_arrays":
            clocks = sampler.stop()
    s.check_finite()
    h2d, d2h = s.transfer_bytes()
    s.close()
    value = n_phys * 4 / res["overlap_arrays"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": K,
        "warmup": W, "ms_per_step": 1e3 * res["overlap_arrays"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded generator, no dataset)",
        "config": {"workload": workload_name(args) + "; 3 slices (x, y, z) of 9 "
                   "components to the host every step",
                   "parallelism": "single",
                   "l2": "inputs larger than L2, no flush"},
        "output": {"floats_per_step": nfl,
                   "ms_per_step_overlapped_arrays": 1e3 * res["overlap_arrays"],
                   "ms_per_step_overlapped_scatter": 1e3 * res["overlap_scatter"],
                   "ms_per_step_blocking_scatter": 1e3 * res["packed"],
                   "ms_per_step_whole_state": 1e3 * res["whole"],
                   "ms_per_step_no_output": 1e3 * res["none"],
                   "whole_state_bytes": 4 * p.ncmp * p.nx * p.ny * p.nz},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 4 * nfl},
        "gpu_launches": None,
        "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


def locate_points(X, Y, Z, nsta=400, nsrc=64, seed=9):
    """Stations on a regular 20 x 20 surface grid given by depth 0 and
    sources at depth 1-8 km given by depth, over the physical area."""
    import numpy as np
    rng = np.random.default_rng(seed)
    xs, ys = X[3, 3:-3, 3:-3], Y[3, 3:-3, 3:-3]
    x0, x1, y0, y1 = float(xs.min()), float(xs.max()), float(ys.min()), float(ys.max())
    m = int(round(nsta ** 0.5))
    gx, gy = np.meshgrid(np.linspace(x0, x1, m + 2)[1:-1], np.linspace(y0, y1, m + 2)[1:-1])
    sta = np.stack([gx.ravel(), gy.ravel(), np.zeros(m * m)], 1)
    src = np.stack([rng.uniform(x0, x1, nsrc), rng.uniform(y0, y1, nsrc),
                    rng.uniform(1000.0, 8000.0, nsrc)], 1)
    pts = np.concatenate([sta, src]).astype(np.float32)
    return pts, np.ones(len(pts), np.int32)


def run_locate(args, reference=False):
    """Set-up of stations and sources given by coordinates: 400 stations and
    64 sources located on the topography grid (depth converted to z, cell
    search, shift sampling), points per second."""
    import numpy as np
    from types import SimpleNamespace
    from cgfd3d_gb300 import models
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    X, Y, Z = [a.reshape(args.nk + 6, args.nj + 6, args.ni + 6) for a in
               models._coords_of(SimpleNamespace(ni=args.ni, nj=args.nj, nk=args.nk), 2024)]
    pts, dep = locate_points(X, Y, Z)
    name = ("point location: %d stations (depth 0) + %d sources (depth 1-8 km) on the "
            "topography grid %dx%dx%d" % (400, len(pts) - 400, args.ni, args.nj, args.nk))
    sample_n = 6
    line = {"metric": "points located/s", "unit": "points/s", "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": name, "parallelism": "single"}}
    if reference or not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        sub = np.linspace(0, len(pts) - 1, sample_n).astype(int)
        t0 = time.perf_counter()
        oracle.locate(X, Y, Z, pts[:0], dep[:0])          # grid bounds only
        t1 = time.perf_counter()
        oracle.locate(X, Y, Z, pts[sub], dep[sub])
        t2 = time.perf_counter()
        t_cpu = max((t2 - t1) - (t1 - t0), 1e-9)
        cpu = {"value": sample_n / t_cpu, "unit": "points/s", "cores": 1, "kind": "port",
               "sample": "%d of the points, C oracle port, 1 thread, %.2f s after the "
                         "grid bounds (%.2f s, once per grid)" % (sample_n, t_cpu, t1 - t0)}
    if reference:
        line.update({"impl": "reference", "value": cpu["value"], "steps": 1, "warmup": 0,
                     "ms_per_step": 1e3 * sample_n / cpu["value"], "cpu_baseline": cpu,
                     "e2e": {"value": cpu["value"], "unit": "points/s",
                             "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        print(json.dumps(line), flush=True)
        return 0
    import torch
    torch.cuda.set_device(local)
    from cgfd3d_gb300 import locate
    K, W = args.steps, max(args.warmup, 0)
    t0 = time.perf_counter()
    L = locate.Locator(X, Y, Z)
    t_setup = time.perf_counter() - t0
    for _ in range(W):
        L.locate(pts, dep)
    times = []
    for _ in range(K):
        t0 = time.perf_counter()
        L.locate(pts, dep)
        times.append(time.perf_counter() - t0)
    L.close()
    t = sum(times) / len(times)
    line.update({"value": len(pts) / t, "steps": K, "warmup": W, "ms_per_step": 1e3 * t,
                 "setup_ms": 1e3 * t_setup,
                 "e2e": {"value": len(pts) / (t + t_setup / K), "unit": "points/s",
                         "h2d_bytes_per_step": int(3 * X.size * 4 / K + pts.nbytes),
                         "d2h_bytes_per_step": int(len(pts) * 32)},
                 "gpu_launches": None})
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def layered_model(X, Y, nlayer=4, seed=13):
    """A layered elastic isotropic model over the grid's area: undulating
    interfaces from 3 km above sea level down to -15 km, velocities and
    densities increasing with depth, perturbed by 2 % per mesh point; linear
    vp and rho gradients, as the reference's example layered models have
    (example/prep_medium/gen_eliso_lay.m: powers 1, no vs gradient)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    NX, NY = 81, 81
    minx, miny = float(X.min()) - 100.0, float(Y.min()) - 100.0
    dx = (float(X.max()) + 100.0 - minx) / (NX - 1)
    dy = (float(Y.max()) + 100.0 - miny) / (NY - 1)
    xs, ys = minx + dx * np.arange(NX), miny + dy * np.arange(NY)
    XX, YY = np.meshgrid(xs, ys)
    tops = [3000.0, -3000.0, -9000.0, -15000.0][:nlayer]
    recs = []
    for n, t in enumerate(tops):
        e = t + 300.0 * np.sin(XX / 7000.0 + n) * np.cos(YY / 5000.0)
        rho, vp, vs = 2300 + 200 * n, 4000 + 800 * n, 2300 + 450 * n
        r = lambda a: a * (1 + 0.02 * rng.uniform(-1, 1, XX.shape))
        recs.append(np.stack([e, r(rho), np.full_like(XX, 0.02), np.full_like(XX, 1.0),
                              r(vp), np.full_like(XX, 0.05), np.full_like(XX, 1.0),
                              r(vs), np.full_like(XX, 0.0), np.full_like(XX, 1.0)], -1))
    return dict(NI=len(tops), NX=NX, NY=NY, MINX=minx, MINY=miny, DX=dx, DY=dy,
                rec=np.stack(recs).astype(np.float32))


def run_media(args, reference=False):
    """Media discretisation: a 4-interface layered elastic isotropic model
    onto the topography grid with the equivalent-medium method
    --media-method, grid points per second (host coordinates in, host
    lambda/mu/rho out)."""
    import numpy as np
    from types import SimpleNamespace
    from cgfd3d_gb300 import models
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    shp = (args.nk + 6, args.nj + 6, args.ni + 6)
    X, Y, Z = [a.reshape(shp) for a in
               models._coords_of(SimpleNamespace(ni=args.ni, nj=args.nj, nk=args.nk), 2024)]
    m = layered_model(X, Y)
    npts = X.size
    line = {"metric": "grid points discretised/s", "unit": "points/s", "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "layered elastic isotropic model (4 interfaces, "
                       "81x81 mesh) onto the topography grid %dx%dx%d (padded), "
                       "method %s" % (args.ni, args.nj, args.nk, args.media_method),
                       "parallelism": "single"}}
    if reference or not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        cw = 96                                # a block of 96 x 96 full-depth columns
        sx, sy, sz = [np.ascontiguousarray(a[:, :cw, :cw]) for a in (X, Y, Z)]
        t0 = time.perf_counter()
        oracle.layer_el_iso(m, sx, sy, sz, args.media_method)
        tc = time.perf_counter() - t0
        cpu = {"value": sx.size / tc, "unit": "points/s", "cores": 1, "kind": "port",
               "sample": "%dx%d full-depth columns (%d points), C oracle port, 1 thread, "
                         "%.2f s" % (cw, cw, sx.size, tc)}
    if reference:
        line.update({"impl": "reference", "value": cpu["value"], "steps": 1, "warmup": 0,
                     "ms_per_step": 1e3 * npts / cpu["value"], "cpu_baseline": cpu,
                     "e2e": {"value": cpu["value"], "unit": "points/s",
                             "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        print(json.dumps(line), flush=True)
        return 0
    import torch
    torch.cuda.set_device(local)
    from cgfd3d_gb300 import media
    K, W = args.steps, max(args.warmup, 0)
    for _ in range(W):
        media.layer_el_iso(m, X, Y, Z, args.media_method)
    ts = []
    for _ in range(K):
        t0 = time.perf_counter()
        media.layer_el_iso(m, X, Y, Z, args.media_method)
        ts.append(time.perf_counter() - t0)
    t = sorted(ts)[len(ts) // 2]
    line.update({"value": npts / t, "steps": K, "warmup": W, "ms_per_step": 1e3 * t,
                 "e2e": {"value": npts / t, "unit": "points/s",
                         "h2d_bytes_per_step": 3 * npts * 4 + m["rec"].nbytes,
                         "d2h_bytes_per_step": 3 * npts * 4,
                         "how": "host coordinates to host media, median of K calls"},
                 "gpu_launches": K * (1 if args.media_method == "loc" else 4)})
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def run_media_bin(args, reference=False):
    """A model given as binary volumes (rho, vp, vs; 161 x 161 x 80 samples,
    stored z fastest, z decreasing) interpolated onto the topography grid,
    grid points per second (host coordinates and volumes in, host rho,
    lambda, mu out)."""
    import numpy as np
    from types import SimpleNamespace
    from cgfd3d_gb300 import models
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    shp = (args.nk + 6, args.nj + 6, args.ni + 6)
    X, Y, Z = [a.reshape(shp) for a in
               models._coords_of(SimpleNamespace(ni=args.ni, nj=args.nj, nk=args.nk), 2024)]
    npts = X.size
    ext = (float(X.min()), float(X.max()), float(Y.min()), float(Y.max()))
    nxb, nyb, nzb = 161, 161, 80
    dx = (ext[1] - ext[0] + 400.0) / (nxb - 1)
    dy = (ext[3] - ext[2] + 400.0) / (nyb - 1)
    z0, dz = float(Z.max()) + 100.0, -(float(Z.max()) - float(Z.min()) + 200.0) / (nzb - 1)
    order, size = (2, 0, 1), (nzb, nxb, nyb)
    spacing, origin = (dz, dx, dy), (z0, ext[0] - 200.0, ext[2] - 200.0)
    rng = np.random.default_rng(31)
    depth = np.clip(-(z0 + dz * np.arange(nzb)), 0, None)[None, None, :]
    base = np.ones((nyb, nxb, 1), np.float32)
    vols = [(b + g * depth + a * rng.standard_normal((nyb, nxb, nzb))).astype(np.float32)
            * base for b, g, a in ((2200.0, 0.05, 20.0), (3600.0, 0.12, 60.0),
                                   (2000.0, 0.07, 30.0))]
    line = {"metric": "grid points discretised/s", "unit": "points/s", "n_gpus": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": "binary-volume model 161x161x80 (rho, vp, vs) onto the "
                       "topography grid %dx%dx%d (padded), trilinear"
                       % (args.ni, args.nj, args.nk), "parallelism": "single"}}
    if reference or not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(REPO, "oracle"))
        import oracle
        m = dict(order=np.array(order, np.int32), size=np.array(size, np.int32),
                 spacing=np.array(spacing, np.float32), origin=np.array(origin, np.float32),
                 ext=np.array(ext, np.float32), rho_vol=vols[0], vp_vol=vols[1], vs_vol=vols[2])
        kk = 16                                 # a slab of 16 k-planes
        t0 = time.perf_counter()
        oracle.bin_model(m, X[:kk], Y[:kk], Z[:kk])
        tc = time.perf_counter() - t0
        cpu = {"value": X[:kk].size / tc, "unit": "points/s", "cores": 1, "kind": "port",
               "sample": "%d k-planes (%d points), C oracle port, 1 thread, %.2f s"
                         % (kk, X[:kk].size, tc)}
    if reference:
        line.update({"impl": "reference", "value": cpu["value"], "steps": 1, "warmup": 0,
                     "ms_per_step": 1e3 * npts / cpu["value"], "cpu_baseline": cpu,
                     "e2e": {"value": cpu["value"], "unit": "points/s",
                             "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        print(json.dumps(line), flush=True)
        return 0
    import torch
    torch.cuda.set_device(local)
    from cgfd3d_gb300 import media
    lay = media.BinModel.of(order, size, spacing, origin)
    for _ in range(max(args.warmup, 0)):
        media.bin_model(lay, ext, vols, X, Y, Z)
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        media.bin_model(lay, ext, vols, X, Y, Z)
        ts.append(time.perf_counter() - t0)
    t = sorted(ts)[len(ts) // 2]
    line.update({"value": npts / t, "steps": args.steps, "warmup": args.warmup,
                 "ms_per_step": 1e3 * t,
                 "e2e": {"value": npts / t, "unit": "points/s",
                         "h2d_bytes_per_step": 3 * npts * 4 + 3 * vols[0].nbytes,
                         "d2h_bytes_per_step": 3 * npts * 4,
                         "how": "host coordinates and volumes to host media, median of K calls"},
                 "gpu_launches": args.steps})
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def measured_peak_bf16():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, KeyError, ValueError):
        return 1900.0, "fallback"


def run_surrogate_net(args):
    """The surrogate network's device work alone (no solver shots): K training
    steps at batch 256 on seeded synthetic targets, then K inference batches,
    and the dominant product (the last decoder layer, 262,144 x 1152 x 640)
    timed alone.  value = training steps/s; small enough to profile."""
    import numpy as np
    import torch
    from cgfd3d_gb300 import surrogate as SG
    torch.cuda.set_device(0)
    B, K, W = 256, max(args.steps, 1), max(args.warmup, 0)
    rng = np.random.default_rng(3)
    net = SG.Surrogate(nrec=64, nt=1000, seed=1, scale=1.0)
    pos = torch.from_numpy(rng.uniform(-1, 1, (B, 3)).astype(np.float32)).cuda()
    M = torch.from_numpy(rng.standard_normal((B, 6)).astype(np.float32)).cuda()
    U = torch.from_numpy(rng.standard_normal((B, 1000, 192)).astype(np.float32)).cuda()
    norm = (U.double() ** 2).reshape(B, -1).sum(1).float()
    for _ in range(W):
        net.gradients(pos, M, U, norm)
        net.apply()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = net.launches
    e0.record()
    for _ in range(K):
        net.gradients(pos, M, U, norm)
        net.apply()
    e1.record()
    torch.cuda.synchronize()
    train_ms = e0.elapsed_time(e1) / K
    train_launches = (net.launches - n0) // K
    for _ in range(W):
        net.predict(pos, M)
    e0.record()
    for _ in range(K):
        net.predict(pos, M)
    e1.record()
    torch.cuda.synchronize()
    inf_ms = e0.elapsed_time(e1) / K
    # the same inference through the C object: host descriptors in, host
    # seismograms out (cgfd_sg_net_predict)
    cnet = SG.Net.of(net)
    pos_h, M_h = pos.cpu().numpy(), M.cpu().numpy()
    # the seismograms come back into pinned host memory (a pageable
    # destination is bound by the host-side copy, ~20 GB/s)
    u_pin = torch.empty((B, 1000, 192), dtype=torch.float32, pin_memory=True).numpy()
    cnet.predict(pos_h, M_h, out=u_pin)
    t0 = time.perf_counter()
    for _ in range(K):
        cnet.predict(pos_h, M_h, out=u_pin)
    c_s = (time.perf_counter() - t0) / K
    cnet.close()
    lay = net.lay
    d = net._buffers(B, False)
    o, k = lay.dec[-1]
    rows = B * lay.T
    last = len(lay.dec) - 1
    args_g = (d["a_d%d" % last], k, net.W(len(lay.layers) - 1), k, d["h_d%d" % last], o,
              rows, o, k)
    bias_g = net.bias(len(lay.layers) - 1)     # as the forward pass calls it
    for _ in range(2):
        net._gemm(*args_g, bias=bias_g)
    e0.record()
    for _ in range(10):
        net._gemm(*args_g, bias=bias_g)
    e1.record()
    torch.cuda.synchronize()
    g_ms = e0.elapsed_time(e1) / 10
    achieved = 2.0 * rows * o * k / (g_ms * 1e-3) / 1e12
    peak, peak_kind = measured_peak_bf16()
    line = {
        "metric": "surrogate training steps/s (batch 256)", "value": 1e3 / train_ms,
        "unit": "steps/s", "n_gpus": 1, "steps": K, "warmup": W, "ms_per_step": train_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 (fp32 accumulation)", "data": "synthetic targets (seeded)",
        "config": {"workload": "surrogate network alone: 5.5 M parameters, 64 receivers x 3 "
                   "components x 1000 samples, batch 256", "parallelism": "single"},
        "inference": {"ms_per_batch": inf_ms, "shots_per_s": B / (inf_ms * 1e-3),
                      "host_to_host_c_object": {
                          "ms_per_batch": 1e3 * c_s, "shots_per_s": B / c_s,
                          "h2d_bytes": B * 9 * 4, "d2h_bytes": B * 1000 * 192 * 4}},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                     "kernel": "k_gemm_tn_p (persistent form, 128 x 256 tiles; last decoder "
                               "layer, %d x %d x %d)" % (rows, o, k),
                     "ms": g_ms},
        "gpu_launches": train_launches,
        "device_error": net.device_error(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_surrogate(args):
    """Learned surrogate (config 4).  Shots of the batched solver on the fixed
    256 x 256 x 128 crop of the topography model (sources uniform in the
    volume 1-8 km deep, random unit moment tensors, Ricker 2 Hz, 64 surface
    receivers x 3 components x 1000 samples) train the network; held-out
    shots score it by relative L2 misfit.  value = surrogate inference
    shots/s at batch 256 (timed alone, CUDA events); beside it the batched
    solver's shots/s on the same shots, the held-out misfits, the k-nearest
    least-squares baseline without the network, and the throughput of the
    fallback rule (2 solver check shots per 64-shot request, the solver for
    the whole request when a check misfit exceeds 5 %)."""
    import numpy as np
    import torch
    from cgfd3d_gb300 import models, surrogate as SG
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(0)
    crop = (args.ni, args.nj, args.nk)
    t_setup = time.perf_counter()
    base = models._topo_base(400, 400, 200, 2024)
    model = SG.crop_model(base, crop)
    del base
    ntr, nte = args.sg_train, args.sg_test
    ijd_tr, M_tr = SG.draw_sources(ntr, crop, seed=41)
    ijd_te, M_te = SG.draw_sources(nte, crop, seed=43)
    t_setup = time.perf_counter() - t_setup
    sampler = ClockSampler(0)
    sampler.start()
    U_tr, s_tr = SG.solve_shots(model, ijd_tr, M_tr, steps=1000, batch=64)
    U_te, s_te = SG.solve_shots(model, ijd_te, M_te, steps=1000, batch=64)
    solver_rate = (ntr + nte) / (s_tr + s_te)
    scale = float(np.sqrt((U_tr.astype(np.float64) ** 2).mean()))
    pos_tr, pos_te = SG.normalise_positions(ijd_tr, crop), SG.normalise_positions(ijd_te, crop)
    net = SG.Surrogate(nrec=64, nt=1000, seed=1, scale=scale, lr=1e-3, wd=1e-4)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    tp, tM, tU = dev(pos_tr), dev(M_tr), dev(U_tr)
    tnorm = (tU.double() ** 2).reshape(ntr, -1).sum(1).float()
    B = min(256, ntr)
    g = torch.Generator(device="cuda").manual_seed(5)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    hist = []
    for it in range(args.sg_iters):
        idx = torch.randperm(ntr, generator=g, device="cuda")[:B]
        lr = 1e-5 + 0.5 * (1e-3 - 1e-5) * (1.0 + math.cos(math.pi * it / args.sg_iters))
        loss_b = net.gradients(tp[idx].contiguous(), tM[idx].contiguous(),
                               tU[idx].contiguous(), tnorm[idx].contiguous())
        net.apply(lr)
        if it % 100 == 0 or it == args.sg_iters - 1:
            hist.append((it, float(torch.sqrt((loss_b / tnorm[idx]).mean()).item())))
    e1.record()
    torch.cuda.synchronize()
    train_s = e0.elapsed_time(e1) * 1e-3
    # held-out scoring
    pred = np.concatenate([net.predict(dev(pos_te[a:a + 256]), dev(M_te[a:a + 256])).cpu().numpy()
                           for a in range(0, nte, 256)])
    mis = SG.misfit(pred, U_te)
    mis_tr = SG.misfit(net.predict(dev(pos_tr[:256]), dev(M_tr[:256])).cpu().numpy(),
                       U_tr[:256])
    knn = SG.misfit(SG.knn_green(pos_tr, M_tr, U_tr, pos_te, M_te, k=12), U_te)
    # inference throughput at batch 256, inputs resident
    pb = dev(np.resize(pos_te, (256, 3)))
    mb = dev(np.resize(M_te, (256, 6)))
    for _ in range(3):
        net.predict(pb, mb)
    torch.cuda.synchronize()
    n0 = net.launches
    e0.record()
    reps = max(args.steps, 1)
    for _ in range(reps):
        net.predict(pb, mb)
    e1.record()
    torch.cuda.synchronize()
    inf_s = e0.elapsed_time(e1) * 1e-3 / reps
    launches = (net.launches - n0) // reps
    rate = 256.0 / inf_s
    # end to end: host positions and moment tensors in, host seismograms out
    ph = torch.from_numpy(np.resize(pos_te, (256, 3))).pin_memory()
    mh = torch.from_numpy(np.resize(M_te, (256, 6))).pin_memory()
    t0 = time.perf_counter()
    for _ in range(reps):
        out = net.predict(ph.cuda(non_blocking=True), mh.cuda(non_blocking=True)).cpu()
    e2e_s = (time.perf_counter() - t0) / reps
    # the dominant kernel alone: the last decoder layer's product
    lay = net.lay
    d = net._buffers(256, False)
    o, k = lay.dec[-1]
    rows = 256 * lay.T
    bias_g = net.bias(len(lay.layers) - 1)     # as the forward pass calls it
    for _ in range(2):
        net._gemm(d["a_d%d" % (len(lay.dec) - 1)], k, net.W(len(lay.layers) - 1), k,
                  d["h_d%d" % (len(lay.dec) - 1)], o, rows, o, k, bias=bias_g)
    e0.record()
    for _ in range(10):
        net._gemm(d["a_d%d" % (len(lay.dec) - 1)], k, net.W(len(lay.layers) - 1), k,
                  d["h_d%d" % (len(lay.dec) - 1)], o, rows, o, k, bias=bias_g)
    e1.record()
    torch.cuda.synchronize()
    g_ms = e0.elapsed_time(e1) / 10
    flops = 2.0 * rows * o * k
    achieved = flops / (g_ms * 1e-3) / 1e12
    clocks = sampler.stop()
    peak, peak_kind = measured_peak_bf16()
    # fallback rule over the held-out shots, 64-shot requests
    rng = np.random.default_rng(9)
    per_shot_solver = 1.0 / solver_rate
    t_rule, n_fb, n_req = 0.0, 0, 0
    for a in range(0, nte, 64):
        req = np.arange(a, min(a + 64, nte))
        chk = rng.choice(req, size=min(2, len(req)), replace=False)
        t_rule += len(req) / rate + len(chk) * per_shot_solver
        n_req += 1
        if mis[chk].max() > 0.05:
            t_rule += (len(req) - len(chk)) * per_shot_solver
            n_fb += 1
    line = {
        "metric": "surrogate shots/s (batch 256 inference)", "value": rate,
        "unit": "shots/s", "n_gpus": 1, "steps": reps, "warmup": 3,
        "ms_per_step": 1e3 * inf_s, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (fp32 accumulation)",
        "data": "synthetic: shots of the batched solver on the seeded topography model",
        "config": {"workload": "learned surrogate on the %dx%dx%d crop of the topography "
                   "model: %d training + %d held-out solver shots, 64 receivers x 3 "
                   "components x 1000 samples, %d training steps at batch %d"
                   % (crop + (ntr, nte, args.sg_iters, B)),
                   "parameters": lay.nparam, "parallelism": "single"},
        "solver": {"value": solver_rate, "unit": "shots/s",
                   "how": "batched solver, 64 shots per launch, 1000 steps each",
                   "seconds": s_tr + s_te},
        "surrogate_over_solver": rate / solver_rate,
        "heldout_misfit": {"median": float(np.median(mis)), "mean": float(mis.mean()),
                           "p90": float(np.percentile(mis, 90)),
                           "within_5pct": float((mis <= 0.05).mean())},
        "train_misfit_median": float(np.median(mis_tr)),
        "knn_baseline_misfit": {"median": float(np.median(knn)), "mean": float(knn.mean()),
                                "within_5pct": float((knn <= 0.05).mean()),
                                "how": "12 nearest training shots, least-squares Green's "
                                       "functions, no network"},
        "fallback_rule": {"shots_per_s": nte / t_rule, "requests": n_req,
                          "fell_back": n_fb,
                          "how": "2 solver check shots per 64-shot request; the solver "
                                 "for the request when a check misfit exceeds 5 %"},
        "training": {"seconds": train_s, "steps": args.sg_iters,
                     "misfit_history": hist},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": None, "kernel": "k_gemm_tn_p (persistent form, 128 x 256 "
                     "tiles; last decoder layer, %d x %d x %d)" % (rows, o, k), "ms": g_ms},
        "e2e": {"value": 256.0 / e2e_s, "unit": "shots/s",
                "h2d_bytes_per_step": 256 * 9 * 4, "d2h_bytes_per_step": int(out.numel()) * 4},
        "gpu_launches": launches,
        "clocks": clocks,
        "setup_s": t_setup,
        "device_error": net.device_error(),
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "slices":
        return run_slices(args)
    if args.workload == "locate":
        return run_locate(args)
    if args.workload == "media":
        return run_media(args)
    if args.workload == "media_bin":
        return run_media_bin(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.workload == "surrogate_net":
        return run_surrogate_net(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
