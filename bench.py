"""Benchmark of the batched EOB waveform + likelihood path on GB300.

Default workload: the ragged-batching configuration -- 1024 aligned-spin
binaries, M ~ U[20, 200] Msun, q ~ U[1, 8], chi ~ U[-0.9, 0.9],
f0 ~ U[10, 20] Hz, (2,2) mode, dt = 1/2048 s, N = 2^17 samples, white-noise
data with one injection at SNR 30, FP64 throughout.  A step is one pass of the
whole path (parameters -> lnL) over the batch.

    python bench.py [--gpus N] [--steps K] [--warmup W]
                    [--impl native|reference|plain|refloop] [--config 1|2|3|4|5]

The default line also carries, on one GPU, the plain FP64 GPU method on the
same batch (`plain`, `vs_plain`) and the serving workload (`serving`: a
2000-request Poisson trace of walker batches through the continuous-batching
server in mixed precision, its capacity, request latency p50/p99 at 70 % load,
and the plain method serving the same requests one at a time).

Under torchrun (N > 1) every rank runs its own batch (replicas: the path has
no exchange step); value = all binaries of all ranks / max-over-ranks time.
`--impl reference` times the CPU restatement of the reference path (the
oracle) on the host cores; `--impl plain` the plain FP64 GPU method alone;
`--impl refloop` the reference's own launch structure (a host loop of
per-stage launches) on the GPU.  Prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from eobgpu_gb300 import workload  # noqa: E402

METRIC = "waveform+lnL evals/s"
# FP64 floating-point operations of one right-hand-side evaluation of the
# integrator, frozen: the hardware census of the one-lane kernel (ncu DADD +
# DMUL + 2 DFMA thread instructions divided by the lane-RHS count,
# profiles/k_integrate_fp64_census.md).  It stays fixed when later kernels
# need fewer instructions per right-hand side, so that roofline fractions
# compare across versions.
F_RHS = 1533.0
# FP64 warp instructions per warp of a four-warp group per right-hand side
# (profiles/k_integrate_quad_census.md): the work on the longest binary's chain
QUAD_FP64_PER_WARP = 104.0

TRAFFIC = os.path.join(ROOT, "profiles", "k_integrate_traffic_config2.md")


def _traffic_bytes():
    """DRAM bytes (read + write) of one integrator launch on the default
    workload, from the committed ncu capture (profiles/)."""
    try:
        with open(TRAFFIC) as f:
            for line in f:
                if line.startswith("TRAFFIC_BYTES_PER_LAUNCH"):
                    return int(line.split("=")[1].strip())
    except OSError:
        pass
    return None


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("EOB_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), f"eob_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        try:
            self.f.close()
        except Exception:
            pass

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) >= 9:
                        rows.append(p)
            os.remove(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([float(r[1]) for r in rows])
        mx = float(rows[0][2])
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].lower() == "active"})
        busy = sm[sm > 0.5 * np.max(sm)] if len(sm) else sm
        return {"sm_mhz": float(np.median(busy)), "sm_max_mhz": mx, "reasons": reasons, "samples": len(rows)}


def make_inputs(cfg, stream_seed, device, max_steps):
    """Seeded parameters of the configuration and data built from the injection."""
    import torch
    from eobgpu_gb300.pipeline import WaveformLikelihood
    params = workload.draw_params(cfg, stream=stream_seed)
    inj = workload.injection_params(cfg)
    wl = WaveformLikelihood(1, max_steps, list(cfg.modes), cfg.n_samples, device=device)
    h, st = wl.strain(torch.tensor(inj[None, :], device=device), cfg.dt, cfg.n_samples)
    torch.cuda.synchronize()
    data, amp = workload.make_data(h[0].real.cpu().numpy(), cfg.n_samples, cfg.index)
    del wl
    return params, data, amp


_POOL_DATA = None


def _pool_init(data):
    """Worker initialiser: the data vector is sent to each worker once."""
    global _POOL_DATA
    _POOL_DATA = data


def _oracle_worker(args):
    p, dt, N, modes, amp, max_step = args
    from oracle.oracle import Oracle
    o = Oracle()
    return o.lnl_one(p, dt, N, modes, _POOL_DATA, amp, max_step=max_step)["lnl"]


def cpu_time(params, cfg, data, amp, max_step, cores):
    """Wall time of the oracle (CPU restatement of the reference path) over params on `cores` processes."""
    import multiprocessing as mp
    jobs = [(p, cfg.dt, cfg.n_samples, list(cfg.modes), amp, max_step) for p in params]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_pool_init, initargs=(data,)) as pool:
        pool.map(_oracle_worker, jobs[:cores])  # start-up and first-call costs outside the timing
        t0 = time.perf_counter()
        out = pool.map(_oracle_worker, jobs, chunksize=1)
        t1 = time.perf_counter()
    return t1 - t0, np.array(out)


def _oracle_detail_worker(args):
    """Free-running oracle, and the oracle replayed on the GPU's knots."""
    p, dt, N, modes, amp, max_step, knots = args
    from oracle.oracle import Oracle
    o = Oracle()
    r = o.lnl_one(p, dt, N, modes, _POOL_DATA, amp, max_step=max_step, want_detail=True)
    rr = o.lnl_one(p, dt, N, modes, _POOL_DATA, amp, max_step=max_step, want_detail=True, replay_t=knots)
    return (r["lnl"], r["status"], r["h"], r["npts"]), (rr["lnl"], rr["status"], rr["h"], rr["npts"], rr["y"])


def accuracy_vs_oracle(params, cfg, data, amp, max_steps, precision, device, sample, cores):
    """Waveform and lnL error of the GPU path against the FP64 oracle on an
    evenly spread sample of the batch (outside any timed region), two ways:

    replay -- the oracle carried over the GPU's own accepted knots (one
      DOPR853 step per pair of trajectory rows): identical sampling, so the
      differences are the arithmetic's alone (rows, strain, lnL);
    free-running -- each side chooses its own steps: phase and relative
      amplitude at the oracle's amplitude peak, mismatch 1 - Re<a, c> /
      (|a| |c|) over the N samples, |dlnL| and |dlnL| / |lnL|.  The adaptive
      controller turns rounding-level differences into other knots; binaries
      whose template ends on another sample than the oracle's (the last
      sample, at the merger, carries h^2 ~ 25-50 of lnL) are counted apart."""
    import multiprocessing as mp
    import torch
    from eobgpu_gb300 import _lib
    from eobgpu_gb300.pipeline import WaveformLikelihood
    idx = np.unique(np.linspace(0, len(params) - 1, min(sample, len(params))).astype(int))
    P = np.ascontiguousarray(params[idx])
    N = int(len(data))
    o = _lib.default_options()
    o.precision = precision
    wl = WaveformLikelihood(len(P), max_steps, list(cfg.modes), N, device=device, options=o)
    Pd = torch.tensor(P, device=device)
    lnl, st = wl.run(Pd, torch.tensor(data, device=device), cfg.dt, amp)
    hs, _ = wl.synth_strain(len(P), cfg.dt, N)
    lnl, st, hs = lnl.cpu().numpy(), st.cpu().numpy(), hs.cpu().numpy()
    nsteps, npts, _, trajs = wl.trajectories()
    del wl, Pd
    torch.cuda.empty_cache()
    jobs = [(p, cfg.dt, N, list(cfg.modes), amp, max_steps, trajs[b][0]) for b, p in enumerate(P)]
    with mp.get_context("spawn").Pool(cores, initializer=_pool_init, initargs=(data,)) as pool:
        res = pool.map(_oracle_detail_worker, jobs, chunksize=1)
    m = {True: [], False: []}  # same end sample as the oracle: metrics
    rep = []
    skipped = 0
    for b, ((ol, ost, a, onp), (rl, rst, ra, rnp, ry)) in enumerate(res):
        if ost != 0 or st[b] != 0 or rst != 0:
            skipped += 1
            continue
        c = hs[b]
        k = int(np.argmax(np.abs(a)))
        ov = np.real(np.vdot(a, c)) / np.sqrt(np.real(np.vdot(a, a)) * np.real(np.vdot(c, c)))
        m[int(npts[b]) == int(onp)].append((
            abs((np.angle(c[k]) - np.angle(a[k]) + np.pi) % (2 * np.pi) - np.pi), abs(abs(c[k]) / abs(a[k]) - 1),
            1 - ov, abs(lnl[b] - ol), abs(lnl[b] - ol) / abs(ol)))
        y = trajs[b][1]
        kr = int(np.argmax(np.abs(ra)))
        rep.append((float(np.max(np.abs(y - ry) / np.max(np.abs(y), axis=0))),
                    float(np.max(np.abs(c - ra)) / abs(ra[kr])),
                    abs((np.angle(c[kr]) - np.angle(ra[kr]) + np.pi) % (2 * np.pi) - np.pi),
                    abs(lnl[b] / rl - 1), int(rnp != npts[b])))
    same = np.array(m[True]).reshape(-1, 5)
    flip = np.array(m[False]).reshape(-1, 5)
    rep = np.array(rep).reshape(-1, 5)
    out = {"vs": "FP64 oracle (CPU restatement, pinned to the reference's own code)",
           "precision": "mixed" if precision else "f64", "sample": len(P), "skipped_status": skipped}
    if len(rep):
        out["replay"] = {"how": "oracle integrated on the GPU's accepted knots (identical sampling)",
                         "max_rel_row_error": float(rep[:, 0].max()),
                         "max_strain_error_of_peak": float(rep[:, 1].max()),
                         "max_dphi_at_peak_rad": float(rep[:, 2].max()),
                         "max_rel_dlnl": float(rep[:, 3].max()), "median_rel_dlnl": float(np.median(rep[:, 3])),
                         "frac_rel_dlnl_le_1e-9": float(np.mean(rep[:, 3] <= 1e-9)),
                         "sample_count_differs": int(rep[:, 4].sum())}
    free = {"how": "each side chooses its own steps", "same_end_sample": len(same),
            "end_sample_differs": len(flip)}
    if len(same):
        free.update({"max_dphi_at_peak_rad": float(same[:, 0].max()), "max_rel_amp_at_peak": float(same[:, 1].max()),
                     "max_mismatch": float(same[:, 2].max()), "max_abs_dlnl": float(same[:, 3].max()),
                     "max_rel_dlnl": float(same[:, 4].max()), "median_rel_dlnl": float(np.median(same[:, 4])),
                     "frac_rel_dlnl_le_1e-9": float(np.mean(same[:, 4] <= 1e-9))})
    if len(flip):
        free["end_sample_differs_worst"] = {"max_mismatch": float(flip[:, 2].max()),
                                            "max_abs_dlnl": float(flip[:, 3].max())}
    out["free_running"] = free
    return out


def cpu_sample(params, n):
    """Deterministic bounded sample: every k-th binary."""
    step = max(1, len(params) // n)
    return params[::step][:n]


def run_reference(args, cfg, ws, rank):
    """The reference arm: CPU restatement of the reference path on all host cores."""
    if rank != 0:
        return None
    from oracle import oracle as orc
    orc.build()
    cores = os.cpu_count() or 1
    params = workload.draw_params(cfg, stream=0)
    # data from the oracle's own injection (the reference arm runs without a GPU)
    inj = orc.Oracle().lnl_one(workload.injection_params(cfg), cfg.dt, cfg.n_samples, list(cfg.modes),
                               np.zeros(cfg.n_samples), 1.0, max_step=args.max_steps, want_detail=True)
    data, amp = workload.make_data(inj["h"].real, cfg.n_samples, cfg.index)
    n = args.cpu_sample
    sample = cpu_sample(params, n)
    for _ in range(max(0, min(args.warmup, 1))):
        cpu_time(sample[:cores], cfg, data, amp, args.max_steps, cores)
    times = []
    for _ in range(args.steps):
        t, _ = cpu_time(sample, cfg, data, amp, args.max_steps, cores)
        times.append(t)
    tt = float(np.sum(times))
    value = len(sample) * args.steps / tt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded parameters, white noise + one injection at SNR 30",
            "config": config_block(cfg, args),
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": cores, "kind": "port",
                             "sample": f"{len(sample)} of {cfg.batch} binaries (every {max(1, cfg.batch // n)}th), "
                                       f"per step; the oracle (CPU restatement of the reference path, pinned to "
                                       f"the reference's own code), one process per core"},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def longest_on_four_warps(args, B, nsm):
    """Whether the launch puts the batch's longest binary on a four-warp group
    (the automatic choice of the integrator's launcher, mirrored: lane groups
    up to 32 while B * 2G <= nsm * 256, warp pairs up to B * 64 <= nsm * 512,
    and with warp pairs a head of min(B / 64, 16) four-warp groups)."""
    if args.lanes == 128:
        return True
    if args.head_quads == 0:
        return False
    G = args.lanes
    if G not in (1, 2, 4, 8, 16, 32, 64):
        target = nsm * 4 * 32 * 2
        G = 1
        while G < 32 and B * G * 2 <= target:
            G *= 2
        if G == 32 and B * 64 <= 2 * target:
            G = 64
    if args.head_quads > 0:
        return G == 64 or 8 <= G <= 32
    return G == 64 and B >= 64


def config_block(cfg, args, extra=None):
    """The workload (the same for every arm)."""
    d = {"workload": f"config {cfg.index}: {cfg.name}", "batch": args.batch or cfg.batch,
         "total_mass_msun": list(cfg.total_mass), "mass_ratio": list(cfg.mass_ratio), "chi": list(cfg.chi),
         "f0_hz": list(cfg.f0), "modes": [list(m) for m in cfg.modes], "dt_s": cfg.dt, "n_samples": cfg.n_samples,
         "max_steps": args.max_steps, "rtol": 1e-12, "atol": 1e-12,
         "l2": "flushed between timed steps (256 MiB write)"}
    if extra:
        d.update(extra)
    return d


def impl_block(args, extra=None):
    """How the native arm ran the workload."""
    d = {"queue": "longest first", "lanes_per_binary": getattr(args, "lanes", 0) or "auto",
         "head_quads": "auto" if getattr(args, "head_quads", -1) < 0 else args.head_quads,
         "integrator_block": getattr(args, "block", 0) or "default",
         "integrator_grid": getattr(args, "grid", 0) or "auto"}
    if extra:
        d.update(extra)
    return d


def census(args):
    """Every lane integrates the same binary, so the launch's lane-RHS count is
    exact; run under ncu with -k regex:k_integrate -s 3 -c 1 and divide the
    FP64 instruction census by rhs_all_lanes.  One lane per binary unless
    --lanes is given."""
    import torch
    from eobgpu_gb300.pipeline import WaveformLikelihood
    cfg = workload.CONFIGS[1]
    p = workload.draw_params(cfg, batch=1, stream=0)
    P = torch.tensor(np.repeat(p, 128, axis=0), device="cuda")
    from eobgpu_gb300 import _lib
    opt = _lib.default_options()
    opt.lanes_per_binary = args.lanes or 1
    wl = WaveformLikelihood(128, 4000, [(2, 2)], cfg.n_samples, options=opt)
    for _ in range(4):
        wl.prepare(P, cfg.dt, stages=3)
    torch.cuda.synchronize()
    print(json.dumps({"census": wl.counters()}))


def run_refloop(args, cfg, local):
    """The reference's own launch structure on the GPU: a host loop issuing the
    DOPR853 stages, error norm and controller as separate launches per step
    (eob/new_Dormand_horiz.py:424-778, src/DOPR853.cu:357-762) on top of the
    reference-shaped RHS kernels, run through the drop-in eob/ mirror on the
    same batch.  Only setup, initial conditions and the two trajectory passes
    are timed (everything after the trajectory costs under 1 % of the fused
    path), so its evals/s is an upper bound for that structure."""
    import torch
    from eobgpu_gb300.eob.seobnrv4phm import SEOBNRv4PHM
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    params = workload.draw_params(cfg)
    P = torch.tensor(params, device=device)
    mt = P[:, 0] + P[:, 1]
    omega0 = P[:, 4] * (mt * 4.925491025543576e-06 * np.pi)

    def once():
        gen = SEOBNRv4PHM(max_step=args.max_steps)
        gen.setup_class(P[:, 0] / mt, P[:, 1] / mt, P[:, 2], P[:, 3], omega0)
        r0, pphi0, pr0 = gen.get_initial_conditions(P[:, 0], P[:, 1], P[:, 2], P[:, 3], fs=P[:, 4])
        t, traj, num_steps = gen.run_trajectory(r0, pphi0, pr0, P[:, 0], P[:, 1], P[:, 2], P[:, 3], fs=P[:, 4])
        torch.cuda.synchronize()
        return num_steps

    for _ in range(max(1, min(args.warmup, 1))):
        once()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        ns = once()
        times.append(time.perf_counter() - t0)
    tt = float(np.sum(times))
    B = len(params)
    print(json.dumps({"impl": "refloop", "metric": METRIC, "value": B * args.steps / tt, "unit": "evals/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": 1e3 * tt / args.steps,
                      "higher_is_better": True, "dtype": "f64", "config": config_block(cfg, args),
                      "impl_config": {"timed": "setup + IC + two trajectory passes",
                                      "rows_max": int(ns.max().item())}}))


PLAIN_METHOD = ("plain FP64 GPU method: one warp (32 lanes) per binary, every binary on its own warp from the "
                "start (grid = B / 4 blocks of 4 warps, queue in input order, no head of four-warp groups), "
                "fused DOPR853 integrator + FP64 multipoles, splines, synthesis and lnL, eager launches, no "
                "CUDA graph, no autotuning, one batch at a time")


def plain_options(B):
    """eob_options of the plain FP64 GPU method for a batch of B binaries."""
    from eobgpu_gb300 import _lib
    o = _lib.default_options()
    o.lanes_per_binary = 32
    o.head_quads = 0
    o.precision = 0
    o.block = 128
    o.grid = max(1, -(-int(B) // 4))
    return o


def time_plain(P, D, cfg, amp, max_steps, device, steps, warmup, flush):
    """The plain method on one batch: ms per step (CUDA events, L2 flushed
    between steps) and the last lnL/status."""
    import torch
    from eobgpu_gb300.pipeline import WaveformLikelihood
    B = int(P.shape[0])
    wl = WaveformLikelihood(B, max_steps, list(cfg.modes), int(D.shape[0]), device=device, options=plain_options(B))
    ident = torch.arange(B, dtype=torch.int32, device=device)
    for _ in range(warmup):
        wl.run(P, D, cfg.dt, amp, order=ident)
    torch.cuda.synchronize()
    ms = []
    for i in range(steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lnl, st = wl.run(P, D, cfg.dt, amp, order=ident)
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    out = (ms, lnl.cpu().numpy(), st.cpu().numpy())
    del wl
    torch.cuda.empty_cache()
    return out


def run_plain(args, cfg, local):
    """--impl plain: the plain FP64 GPU method alone on the workload's batch."""
    import torch
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    params, data, amp = make_inputs(cfg, 0, device, args.max_steps)
    P = torch.tensor(params, device=device)
    D = torch.tensor(data, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    ms, _, st = time_plain(P, D, cfg, amp, args.max_steps, device, args.steps, args.warmup, flush)
    t = float(np.sum(ms))
    print(json.dumps({"impl": "plain", "metric": METRIC, "value": len(params) * args.steps / (t / 1e3),
                      "unit": "evals/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": t / args.steps, "higher_is_better": True, "dtype": "f64",
                      "config": config_block(cfg, args), "method": PLAIN_METHOD,
                      "status_ok": int(np.sum(st == 0))}))


OP_CENSUS = os.path.join(ROOT, "profiles", "tdinterp_fdlnl_fp64_census.md")


def _op_flops(key):
    """FP64 FLOP per output of a reference-shaped kernel, from the committed census."""
    try:
        with open(OP_CENSUS) as f:
            for line in f:
                if line.startswith(key):
                    return float(line.split("=")[1].strip())
    except OSError:
        pass
    return None


def fp64_peak_tflops(lib, device):
    """The device's FP64 issue peak, measured live (eob_fp64_probe: independent
    DFMA chains on every lane), best of three."""
    import torch
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    pk_out = torch.empty(nsm * 8 * 256, dtype=torch.float64, device=device)
    iters = 4096
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        lib.eob_fp64_probe(pk_out.data_ptr(), nsm * 8, 256, iters, torch.cuda.current_stream().cuda_stream)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * 8 * iters * nsm * 8 * 256 / (best / 1e3) / 1e12


def run_op(args, local):
    """Reference-shaped kernels outside the fused path, timed alone on
    synthetic inputs of the benchmark's shapes (B = 1024 binaries, N = 2^17
    samples or 2^16 + 1 frequency bins): --op tdinterp2 (mode synthesis on the
    uniform grid, TD2) or --op fd_lnl (frequency-domain likelihood partials,
    three detectors).  Reports the kernel time, algorithmic bytes and the
    fraction of the measured HBM bandwidth; both kernels evaluate one FP64
    sincos per output (per mode for TD2), so they are FP64-issue bound."""
    import torch
    from eobgpu_gb300.eob import pytdinterp
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    g = torch.Generator(device="cpu").manual_seed(7)
    B = args.batch or 1024
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    if args.op == "tdinterp2":
        K = len(workload.CONFIGS[3].modes) if args.config == 3 else 1
        N, L = 131072, 4096
        dt = 1.0 / 2048
        ts = (torch.arange(L, dtype=torch.float64) * (N * dt / (L - 1))).repeat(B).to(device)
        nsubs = 2 * K + 1
        arrs = [torch.randn(B * nsubs * L, generator=g, dtype=torch.float64).to(device) for _ in range(4)]
        tgrid = torch.arange(N, dtype=torch.float64, device=device) * dt
        lengths = torch.full((B,), N, dtype=torch.int32, device=device)
        inds = torch.clamp(torch.searchsorted(ts[:L].contiguous(), tgrid, right=True) - 1, 0, L - 1).to(torch.int32)
        inds = inds.repeat(B)
        old = torch.full((B,), L, dtype=torch.int32, device=device)
        ms = torch.tensor([2, 1, 3, 4, 5][:K], dtype=torch.int32, device=device)
        out = torch.empty(B * N, dtype=torch.complex128, device=device)

        def once():
            pytdinterp.TDInterp_wrap2(out, tgrid, ts, *arrs, L, old, N, B, K, ms, ms, inds, lengths, N)
        units = B * N
        byts = units * (16 + 4 + 8) + B * nsubs * L * 32 + B * L * 8
        flops = _op_flops("FLOP_PER_OUTPUT_TDINTERP2_K5" if K == 5 else "FLOP_PER_OUTPUT_TDINTERP2_K1")
        work = f"{B} binaries x {N} samples, {K} mode(s): write 16 B, read index 4 B and time 8 B per sample, " \
               f"spline tables once; {flops} FP64 FLOP per sample (census)"
    elif args.op == "fd_split":
        # the fused frequency-domain likelihood of BBHWaveformTD.get_ll: one
        # complex FFT per binary of N = 2^17 samples (h~_+ and h~_x recovered
        # from it), three detectors, N/2 + 1 bins
        from eobgpu_gb300 import fd as fdmod
        nch, N = 3, 131072
        Nf = N // 2 + 1
        H = torch.randn((B, N), dtype=torch.complex128, generator=g).to(device)
        data = torch.randn((nch, Nf), dtype=torch.complex128, generator=g).to(device)
        psd = (torch.rand((nch, Nf), dtype=torch.float64, generator=g) + 0.5).to(device)
        Fp, Fx = [torch.rand(nch * B, dtype=torch.float64, generator=g).to(device) for _ in range(2)]
        tau = (0.02 * torch.rand(nch * B, dtype=torch.float64, generator=g) - 0.01).to(device)
        scratch = torch.empty(int(fdmod._lib.load().eob_fd_lnl_scratch_bytes(B, N)), dtype=torch.uint8, device=device)

        def once():
            fdmod.fd_lnl_from_fft(H, data, psd, Fp, Fx, tau, 1.0 / 64.0, 0, scratch)
        units = B * Nf * nch
        byts = B * N * 16 + nch * Nf * 24 + B * 8
        flops = _op_flops("FLOP_PER_OUTPUT_FD_SPLIT")
        work = f"{B} binaries x {Nf} bins x {nch} detectors: the complex FFT (16 B per sample) read once, " \
               f"data and 1/PSD per detector; {flops} FP64 FLOP per (binary, bin, detector) (census)"
    else:
        nch, N = 3, 65537
        hp = torch.randn(B * N, dtype=torch.complex128, generator=g).to(device)
        hc = torch.randn(B * N, dtype=torch.complex128, generator=g).to(device)
        data = torch.randn(nch * N, dtype=torch.complex128, generator=g).to(device)
        psd = (torch.rand(nch * N, dtype=torch.float64, generator=g) + 0.5).to(device)
        F = [torch.rand(nch * B, dtype=torch.float64, generator=g).to(device) for _ in range(3)]
        temp = torch.empty(((N + 1023) // 1024) * B * nch, dtype=torch.complex128, device=device)

        def once():
            pytdinterp.all_in_one_likelihood(temp, hp, hc, data, psd, F[0], F[1], F[2] * 0.01, 0.125, B, nch, N)
        units = B * N * nch
        byts = B * N * 32 + nch * N * 24 + temp.numel() * 16
        flops = _op_flops("FLOP_PER_OUTPUT_FD_LNL")
        work = f"{B} binaries x {N} bins x {nch} detectors: templates 32 B per (binary, bin) read once, " \
               f"data and PSD per detector; {flops} FP64 FLOP per (binary, bin, detector) (census)"
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    for _ in range(args.warmup):
        once()
    torch.cuda.synchronize()
    ms_l = []
    for i in range(args.steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        once()
        e1.record()
        torch.cuda.synchronize()
        ms_l.append(e0.elapsed_time(e1))
    t = float(np.median(ms_l))
    gbs = byts / (t / 1e3) / 1e9
    from eobgpu_gb300 import _lib
    pk = fp64_peak_tflops(_lib.load(), device)
    roof = {"bound": "fp64", "achieved": None, "peak": pk, "unit": "TFLOP/s", "frac": None, "traffic": None,
            "work": work, "peak_source": "measured live: FP64 DFMA probe (eob_fp64_probe), burst",
            "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}}
    if flops:
        roof["achieved"] = flops * units / (t / 1e3) / 1e12
        roof["frac"] = roof["achieved"] / pk
    print(json.dumps({"op": args.op, "metric": "outputs/s", "value": units / (t / 1e3), "unit": "outputs/s",
                      "ms": t, "steps": args.steps, "warmup": args.warmup, "dtype": "f64", "roofline": roof,
                      "l2": "flushed between timed launches (256 MiB write)"}))


def serving_measure(args, device, rank, ws, n_requests, precision=1, plain_sample=64, clocks=True):
    """Configuration 4 on one GPU: a seeded Poisson trace of n_requests walker
    requests (1..512 binaries each, 80 % from a ball around the injection,
    20 % from the configuration-1 prior, dt = 1/1024 s, N = 8192) through
    LikelihoodServer (continuous batching over concurrent slots, mixed
    precision by default).

    capacity -- the server saturated: the first min(n, 400) requests all
      queued at t = 0; evals/s;
    replay -- the whole trace replayed in wall-clock time at 70 % of that
      capacity: request latency (completion minus arrival) p50/p99;
    plain -- the plain FP64 GPU method serving the same requests one at a
      time (each request one batch; host parameters in, lnL out, synchronous),
      on every k-th request of the trace (plain_sample of them): evals/s."""
    import torch
    from eobgpu_gb300.pipeline import WaveformLikelihood
    from eobgpu_gb300.serving import LikelihoodServer
    cfg = workload.CONFIGS[1]
    max_steps = 4000
    _, data, amp = make_inputs(cfg, rank, device, max_steps)
    lanes = getattr(args, "lanes", 0) or 8
    # slot classes by trajectory capacity: four concurrent batches of up to
    # 2048 short binaries and one of 1024 long ones (a sweep of batch sizes
    # 1024..4096, 2..8 slots and 4..16 lanes per binary on the saturated
    # trace put the capacity's plateau here)
    classes = [(1500, 2048, 4), (max_steps, 1024, 1)]
    server = LikelihoodServer(data, cfg.dt, amp, classes=classes, lanes_per_binary=lanes, precision=precision,
                              head_quads=getattr(args, "head_quads", -1), device=device)
    trace = workload.serving_trace(n_requests, 1.0, stream=rank)
    for _ in range(2):
        server.evaluate(trace.params[0])
    npre = min(n_requests, 400)
    sat = server.run_trace(np.zeros(npre), trace.params[:npre])
    capacity = sat["binaries"] / sat["wall_s"]
    sizes = np.array([len(np.atleast_2d(p)) for p in trace.params])
    rate = 0.7 * capacity / float(np.mean(sizes))  # requests/s for 70 % of capacity
    barrier(ws)
    if clocks:
        with ClockSampler(device.index if device.index is not None else 0) as clk:
            res = server.run_trace(trace.arrivals, trace.params, time_scale=1.0 / rate)
        clk_summary = clk.summary()
    else:
        res = server.run_trace(trace.arrivals, trace.params, time_scale=1.0 / rate)
        clk_summary = None
    ok = all(np.all(st == 0) for st in res["status"])
    sts = np.concatenate([np.asarray(st) for st in res["status"]])
    status_other = {str(int(v)): int(c) for v, c in zip(*np.unique(sts[sts != 0], return_counts=True))}
    del server
    torch.cuda.empty_cache()
    # the plain FP64 GPU method on the same requests, one at a time
    Dd = torch.tensor(data, device=device)
    wl = WaveformLikelihood(512, max_steps, list(cfg.modes), cfg.n_samples, device=device, options=plain_options(512))
    ident = torch.arange(512, dtype=torch.int32, device=device)
    step = max(1, n_requests // plain_sample)
    pick = list(range(0, n_requests, step))[:plain_sample]
    host = [torch.from_numpy(np.ascontiguousarray(trace.params[i])).pin_memory() for i in pick]
    out_h = torch.empty(512, dtype=torch.float64).pin_memory()
    wl.options.grid = plain_options(len(host[0])).grid
    wl.run(host[0].to(device), Dd, cfg.dt, amp, order=ident[:len(host[0])])
    torch.cuda.synchronize()
    t_plain = 0.0
    n_plain = 0
    for hp in host:
        n = int(hp.shape[0])
        wl.options.grid = plain_options(n).grid
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        l_d, _ = wl.run(hp.to(device, non_blocking=True), Dd, cfg.dt, amp, order=ident[:n])
        out_h[:n].copy_(l_d, non_blocking=True)
        torch.cuda.synchronize()
        t_plain += time.perf_counter() - t0
        n_plain += n
    del wl
    torch.cuda.empty_cache()
    plain = n_plain / t_plain
    out = {"workload": "config 4: serving, continuous batching over concurrent slots",
           "requests": n_requests, "request_size": [1, 512], "binaries": int(res["binaries"]),
           "precision": "mixed (f64 integrator, phase and spline solve; f32 amplitude, sincos, residual)"
                        if precision else "f64",
           "capacity": {"value": capacity, "unit": "evals/s",
                        "how": f"first {npre} requests all queued at t = 0 (saturated server)",
                        "slot_busy_fraction": sat["slot_busy_fraction"]},
           "replay": {"rate_hz": rate, "offered_load": "70 % of the measured capacity",
                      "throughput": res["binaries"] / res["wall_s"], "wall_s": res["wall_s"],
                      "latency_ms": {"p50": res["p50_ms"], "p99": res["p99_ms"]},
                      "slot_busy_fraction": res["slot_busy_fraction"], "batches": res["batches"],
                      "requeued": res["requeued"], "status_ok": bool(ok), "status_other": status_other},
           "plain": {"value": plain, "unit": "evals/s", "method": PLAIN_METHOD,
                     "sample": f"{len(pick)} requests (every {step}th), {n_plain} binaries, one request at a time, "
                               f"host parameters in and lnL out per request"},
           "served_vs_plain": capacity / plain, "target_served_vs_plain": 5.0,
           "classes_max_steps_batch_slots": classes, "lanes_per_binary": lanes,
           "admission": "by estimated trajectory rows (chirp-time fit x3), re-run on overflow",
           "dt_s": cfg.dt, "n_samples": cfg.n_samples}
    if clk_summary is not None:
        out["clocks"] = clk_summary
    return out, res, sat


def run_serving(args, ws, rank, local):
    """--config 4: the serving workload alone, one JSON line (every rank
    replays its own trace)."""
    import torch
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    sv, res, sat = serving_measure(args, device, rank, ws, args.requests, precision=0 if args.fp64 else 1)
    wall = max_over_ranks(float(res["wall_s"]), ws, device)
    nbin = res["binaries"] * ws
    if rank == 0:
        value = nbin / wall
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": 1,
                "warmup": args.warmup, "ms_per_step": 1e3 * wall, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64" if args.fp64 else "f64 integrator; f64 phase + f32 amplitude/sincos/residual synthesis",
                "data": "synthetic: seeded Poisson trace of walker requests, white noise + one injection at SNR 30",
                "config": {"workload": sv["workload"], "requests": args.requests, "request_size": [1, 512],
                           "dt_s": sv["dt_s"], "n_samples": sv["n_samples"],
                           "l2": "inputs of each batch are new; no flush (latency run)"},
                "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": int(nbin / ws * 40),
                        "d2h_bytes_per_step": int(nbin / ws * 12)},
                "latency_ms": sv["replay"]["latency_ms"], "serving": sv,
                "gpu_launches": int(8 * res["batches"]), "roofline": None, "cpu_baseline": None,
                "clocks": sv.get("clocks"), "status_ok": sv["replay"]["status_ok"]}
        if args.accuracy_sample > 0:
            cfg = workload.CONFIGS[1]
            _, data, amp = make_inputs(cfg, rank, device, 4000)
            trace = workload.serving_trace(args.requests, 1.0, stream=rank)
            allp = np.concatenate([np.atleast_2d(p) for p in trace.params])
            line["accuracy"] = accuracy_vs_oracle(allp, cfg, data, amp, 4000, 0 if args.fp64 else 1, device,
                                                  args.accuracy_sample, os.cpu_count() or 1)
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference", "plain", "refloop"])
    ap.add_argument("--config", type=int, default=2, choices=[1, 2, 3, 4, 5])
    ap.add_argument("--fp64", action="store_true", help="configuration 3 in FP64 instead of mixed precision")
    ap.add_argument("--requests", type=int, default=2000, help="configuration 4: requests in the trace")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the serving block (configuration 4 trace) of the default line")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 GPU method on the same batch in the default line")
    ap.add_argument("--plain-steps", type=int, default=3, help="timed steps of the plain method in the default line")
    ap.add_argument("--head", type=int, default=0,
                    help="configuration 5: longest binaries run concurrently on their own workspace (-1: B/50)")
    ap.add_argument("--slots", type=int, default=1, help="configuration 5: concurrent chunk workspaces")
    ap.add_argument("--hbm-frac", type=float, default=0.9, help="configuration 5: HBM budget, fraction of free memory")
    ap.add_argument("--head-lanes", type=int, default=8, help="configuration 5: lanes per binary of the head")
    ap.add_argument("--no-graph", action="store_true", help="launch the path eagerly instead of replaying a CUDA graph")
    ap.add_argument("--autotune", action="store_true", help="pick lanes per binary, block and spline tile by timing")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--max-steps", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=96)
    ap.add_argument("--accuracy-sample", type=int, default=-1,
                    help="binaries compared with the FP64 oracle after the timing (-1: 64, or 256 for "
                         "configuration 5; 0: none)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lanes", type=int, default=0, help="integrator lanes per binary (0: chosen from the batch size)")
    ap.add_argument("--head-quads", type=int, default=-1,
                    help="longest binaries on four warps each beside groups of 8..64 lanes (-1: the library's choice)")
    ap.add_argument("--block", type=int, default=0, help="integrator threads per block (0: default)")
    ap.add_argument("--grid", type=int, default=0, help="integrator blocks (0: one wave of resident blocks)")
    ap.add_argument("--op", default=None, choices=["tdinterp2", "fd_lnl", "fd_split"],
                    help="time one kernel alone: mode synthesis TD2, FD likelihood partials, or the fused split-FFT FD likelihood")
    ap.add_argument("--imr", action="store_true",
                    help="attach NQC corrections and ringdowns (eob_options.imr, the drop-in class's default): "
                         "the full inspiral-merger-ringdown template instead of the inspiral")
    ap.add_argument("--census", action="store_true",
                    help="FP64 census run: 128 copies of one binary through setup + integrator, 3 warm-up + 1 launch")
    args = ap.parse_args()
    cfg = workload.CONFIGS[1 if args.config == 4 else args.config]
    if args.batch:
        cfg = workload.Config(**{**cfg.__dict__, "batch": args.batch})
    if not args.max_steps:
        args.max_steps = {1: 4000, 2: 6000, 3: 4000, 4: 4000, 5: 16000}[args.config]
    args.warmup = max(3, args.warmup)
    if args.accuracy_sample < 0:
        args.accuracy_sample = 256 if args.config == 5 else 64
    if args.census:
        census(args)
        return
    if args.imr:
        # the oracle's likelihood (the accuracy sample, the CPU arms) is the
        # inspiral template's; the completion's parity is checked against the
        # oracle's own IMR restatement by tests/test_gpu_imr.py
        args.accuracy_sample = 0
        args.no_cpu_baseline = True
        args.no_plain = True
        args.no_serving = True
        if args.impl != "native" or args.config not in (1, 2):
            print(json.dumps({"impl": args.impl, "unavailable": "--imr is a native measurement on "
                              "configurations 1 and 2 (the CPU arms time the inspiral template)"}))
            return
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        line = run_reference(args, cfg, int(os.environ.get("WORLD_SIZE", "1")), rank)
        if line is not None:
            print(json.dumps(line))
        return
    ws, rank, local = dist_init()
    if args.impl == "plain":
        run_plain(args, cfg, local)
        return
    if args.impl == "refloop":
        run_refloop(args, cfg, local)
        return
    if args.op:
        run_op(args, local)
        return
    if args.config == 4:
        run_serving(args, ws, rank, local)
        return

    import torch
    from eobgpu_gb300.pipeline import WaveformLikelihood, longest_first, chirp_duration_M
    device = torch.device(f"cuda:{local}")
    torch.cuda.set_device(device)
    params, data, amp = make_inputs(cfg, rank, device, args.max_steps)
    B = params.shape[0]
    K = len(cfg.modes)
    from eobgpu_gb300 import _lib
    opt = _lib.default_options()
    opt.lanes_per_binary = args.lanes
    opt.head_quads = args.head_quads
    opt.block = args.block
    opt.grid = args.grid
    mixed = args.config in (3, 5) and not args.fp64
    opt.precision = 1 if mixed else 0
    opt.imr = 1 if args.imr else 0
    P = torch.tensor(params, device=device)
    D = torch.tensor(data, device=device)
    order = longest_first(P)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    chunked = None
    tuned = None
    if args.config == 5:
        from eobgpu_gb300.pipeline import ChunkedLikelihood
        head = args.head if args.head >= 0 else B // 50
        free, _ = torch.cuda.mem_get_info(device)
        chunked = ChunkedLikelihood(B, cfg.n_samples, list(cfg.modes), args.max_steps, slots=args.slots, options=opt,
                                    head=head, head_lanes=args.head_lanes, device=device,
                                    hbm_budget_bytes=int(args.hbm_frac * free))
        wl = chunked.engines[0]

        def run_any(Pd, Od):
            return chunked.run(Pd, D, cfg.dt, amp)
    else:
        tuned = None
        if args.autotune:
            from eobgpu_gb300 import autotune
            tuned = autotune.tune(P, D, cfg.dt, amp, list(cfg.modes), args.max_steps, base=opt)
            opt = tuned.options(opt)
        wl = WaveformLikelihood(B, args.max_steps, list(cfg.modes), cfg.n_samples, device=device, options=opt)
        if args.no_graph:
            def run_any(Pd, Od):
                return wl.run(Pd, D, cfg.dt, amp, order=Od)
        else:
            # the whole path as one CUDA graph; a step copies its parameters
            # into the captured input and replays
            Pg = P.clone()
            graph = wl.capture(Pg, D, cfg.dt, amp)

            def run_any(Pd, Od):
                if Pd is not Pg:
                    Pg.copy_(Pd, non_blocking=True)
                return graph.replay()

    def step():
        return run_any(P, order)

    for _ in range(args.warmup):
        lnl, st = step()
    torch.cuda.synchronize()

    # ---- device-resident timing (value)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for i in range(args.steps):
            flush.fill_(float(i))
            ev[i][0].record()
            lnl, st = step()
            ev[i][1].record()
        torch.cuda.synchronize()
        barrier(ws)
        step_ms = [a.elapsed_time(b) for a, b in ev]
        # ---- end to end through the public API with host buffers
        params_h = torch.tensor(params).pin_memory()
        order_h = order.cpu().pin_memory()
        lnl_h = torch.empty(B, dtype=torch.float64).pin_memory()
        st_h = torch.empty(B, dtype=torch.int32).pin_memory()
        ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))
            ev2[i][0].record()
            if chunked is None and not args.no_graph:
                Pg.copy_(params_h, non_blocking=True)
                l_d, s_d = graph.replay()
            else:
                Pd = params_h.to(device, non_blocking=True)
                Od = order_h.to(device, non_blocking=True)
                l_d, s_d = run_any(Pd, Od)
            lnl_h.copy_(l_d, non_blocking=True)
            st_h.copy_(s_d, non_blocking=True)
            ev2[i][1].record()
        torch.cuda.synchronize()
        e2e_ms = [a.elapsed_time(b) for a, b in ev2]
    clocks = clk.summary()
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    t_dev = max_over_ranks(float(np.sum(step_ms)), ws, device)
    t_e2e = max_over_ranks(float(np.sum(e2e_ms)), ws, device)
    value = B * ws * args.steps / (t_dev / 1e3)
    e2e_value = B * ws * args.steps / (t_e2e / 1e3)
    status = st.cpu().numpy()

    # ---- stage timing and roofline of the integrator (one more untimed step)
    # (chunked runs: on the first chunk, the longest binaries)
    if chunked is None:
        Pst, ordst = P, order
    else:
        Pst = P[order[:wl.max_batch].long()].contiguous()
        ordst = None
    Bst = int(Pst.shape[0])
    s_ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)]
    flush.fill_(1.0)
    s_ev[0].record()
    wl.prepare(Pst, cfg.dt, order=ordst, stages=1)
    s_ev[1].record()
    wl.prepare(Pst, cfg.dt, order=ordst, stages=2)
    s_ev[2].record()
    wl.prepare(Pst, cfg.dt, order=ordst, stages=4)
    s_ev[3].record()
    wl.synth_lnl(Bst, D, cfg.dt, amp)
    s_ev[4].record()
    torch.cuda.synchronize()
    stage_ms = {"setup_ic": s_ev[0].elapsed_time(s_ev[1]), "integrate": s_ev[1].elapsed_time(s_ev[2]),
                "modes_splines": s_ev[2].elapsed_time(s_ev[3]), "synth_lnl": s_ev[3].elapsed_time(s_ev[4])}
    cnt = wl.counters()
    # the integrator's critical path: the binary with the most right-hand sides
    rhs_b = wl.rhs_counts()
    crit = int(rhs_b.max()) if len(rhs_b) else 0
    us_rhs = 1e3 * stage_ms["integrate"] / max(1, crit)
    critical = {"binary_rhs_max": crit, "binary_rhs_median": float(np.median(rhs_b)) if len(rhs_b) else 0.0,
                "rhs_total": int(rhs_b.sum()),
                "integrate_us_per_rhs_on_path": us_rhs,
                # the chain's length in FP64 issue slots of one SM sub-partition
                # (one FP64 warp instruction per 64 cycles at the sampled clock)
                "fp64_slots_per_rhs_on_path": us_rhs * sm_mhz / 64.0}
    if longest_on_four_warps(args, B, torch.cuda.get_device_properties(device).multi_processor_count) \
            and chunked is None:
        # the chain's own roofline: the FP64 instructions a warp of a four-warp
        # group issues per right-hand side (ncu census of the four-warp kernel)
        # against the slots the chain takes
        critical["fp64_issue_frac_of_chain"] = QUAD_FP64_PER_WARP / critical["fp64_slots_per_rhs_on_path"]
        critical["fp64_per_warp_per_rhs"] = QUAD_FP64_PER_WARP
    # FP64 peak of this device, measured
    fp64_peak = fp64_peak_tflops(wl.lib, device)
    roof = None
    if F_RHS:
        achieved = F_RHS * cnt["rhs_binaries"] / (stage_ms["integrate"] / 1e3) / 1e12
        default_workload = args.config == 2 and not args.batch and not args.lanes
        roof = {"kernel": "k_integrate", "bound": "fp64", "achieved": achieved, "peak": fp64_peak,
                "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                "traffic": _traffic_bytes() if default_workload else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, "
                                  "profiles/k_integrate_traffic_config2.md" if default_workload else None,
                "peak_source": "measured live: FP64 DFMA probe (eob_fp64_probe), burst",
                "work": f"{F_RHS:.0f} FP64 FLOP per RHS x {cnt['rhs_binaries']} RHS evaluations",
                "lane_occupancy": cnt["rhs_binaries"] / max(1, cnt["rhs_all_lanes"])}

    # ---- the plain FP64 GPU method on the same batch, and the serving
    # workload (configuration 4 trace), one GPU only
    plain_block = None
    if ws == 1 and chunked is None and not args.no_plain:
        pms, plnl, pst = time_plain(P, D, cfg, amp, args.max_steps, device, max(1, args.plain_steps), 1, flush)
        pt = float(np.sum(pms))
        plain_block = {"value": B * len(pms) / (pt / 1e3), "unit": "evals/s", "ms_per_step": pt / len(pms),
                       "steps": len(pms), "warmup": 1, "method": PLAIN_METHOD,
                       "status_ok": int(np.sum(pst == 0)),
                       "max_rel_dlnl_vs_this_run": float(np.max(np.abs(plnl / lnl.cpu().numpy() - 1)))}
    serving = None
    if ws == 1 and args.config == 2 and not args.batch and not args.no_serving:
        serving, _, _ = serving_measure(args, device, rank, ws, args.requests)

    graphed = chunked is None and not args.no_graph
    extra_cfg = {"cuda_graph": graphed,
                 "template": "inspiral-merger-ringdown (NQC + ringdown attached on the GPU)" if args.imr
                 else "inspiral (to the trajectory's last row)"}
    if chunked is not None:
        extra_cfg["chunks"] = chunked.info(B)
    if chunked is None and tuned is not None:
        extra_cfg["autotune"] = {"lanes_per_binary": tuned.lanes_per_binary, "block": tuned.block,
                                 "spline_series_per_block": tuned.spline_series_per_block,
                                 "head_quads": tuned.head_quads, "table": tuned.table}
    line = None
    if rank == 0:
        accuracy = None
        if args.accuracy_sample > 0:
            if chunked is not None:
                del chunked, wl, run_any
            torch.cuda.empty_cache()
            accuracy = accuracy_vs_oracle(params, cfg, data, amp, args.max_steps, 1 if mixed else 0, device,
                                          args.accuracy_sample, os.cpu_count() or 1)
        cpu_base = None
        if not args.no_cpu_baseline:
            cores = os.cpu_count() or 1
            sample = cpu_sample(params, args.cpu_sample)
            t, _ = cpu_time(sample, cfg, data, amp, args.max_steps, cores)
            cpu_base = {"value": len(sample) / t, "unit": "evals/s", "cores": cores, "kind": "port",
                        "sample": f"{len(sample)} of {B} binaries (every {max(1, B // args.cpu_sample)}th)"}
        launches_per_step = 8  # setup, integrate, scan_rows, modes, spline, scan_chunks, synth, finalize
        line = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_dev / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f64 integrator; f64 phase + f32 amplitude/sincos/residual synthesis" if mixed else "f64",
                "data": "synthetic: seeded parameters, white noise + one injection at SNR 30",
                "config": config_block(cfg, args), "impl_config": impl_block(args, extra=extra_cfg),
                "e2e": {"value": e2e_value, "unit": "evals/s",
                        "h2d_bytes_per_step": int(B * 5 * 8 + (0 if graphed else B * 4)),
                        "d2h_bytes_per_step": int(B * 8 + B * 4)},
                "roofline": roof, "cpu_baseline": cpu_base, "clocks": clocks,
                "gpu_launches": launches_per_step * args.steps,
                "latency_ms": (dict(serving["replay"]["latency_ms"], source="request latency of the serving "
                               "block (2000-request Poisson trace at 70 % load)") if serving else
                               {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99)),
                                "source": "timed steps of this batch"}),
                "step_latency_ms": {"p50": float(np.percentile(step_ms, 50)),
                                    "p99": float(np.percentile(step_ms, 99))},
                "plain": plain_block, "vs_plain": (value / plain_block["value"]) if plain_block else None,
                "serving": serving,
                "stages_ms": stage_ms, "stages_batch": Bst, "critical_path": critical,
                "fp64_peak_tflops": fp64_peak,
                "status_ok": int(np.sum(status == 0)),
                "status_other": {str(int(v)): int(c) for v, c in zip(*np.unique(status[status != 0],
                                                                                  return_counts=True))},
                "rows": cnt["rows"], "accuracy": accuracy}
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
