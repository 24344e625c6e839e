"""Throughput of the batched through-transport solve on GB300.

Workload: 16 volumes of 256^3 (blurred Gaussian noise, sigma 2, porosity U[0.35, 0.70]), solved
together by the drop-in ``Solver`` (red-black SOR, float32 sweeps, float64 layer reductions) to
the reference's convergence rule. One step = one complete solve of the batch from the initial
field. Inputs (1.07 GB of field) exceed L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's own CPU Solver (installed under baseline/_ref) on the
host cores, on a bounded sample of the same workload; without the installed reference, the
oracle's float32 restatement in numpy. Under torchrun every rank solves its own batch (weak
scaling, no data-path collective).
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-updates/s & solves/s at D_eff within 1e-4 of FP64 oracle; adjoint/forward time"
UNIT = "voxel-updates/s"
N_VOL, SIDE, SIGMA = 16, 256, 2.0
CONV_CRIT = 1e-4
CPU_SAMPLE_HALF_SWEEPS = 10
# DRAM bytes per voxel moved by one launch of the fused sweep (16x128 tile, 4 half-sweeps):
# dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture on 4 x 256^3 blurred-noise
# volumes (645–647 MB for 67.1 M voxels); traffic grows in proportion to the voxels processed.
TRAFFIC_BYTES_PER_VOXEL_LAUNCH = 645.2e6 / (4 * 256 ** 3)


def workload_config(extra=None):
    cfg = {"workload": f"Solver batch {N_VOL}x{SIDE}^3 blurred noise sigma={SIGMA} porosity U[0.35,0.70]",
           "batch": N_VOL, "shape": [SIDE] * 3, "conv_crit": CONV_CRIT, "bc": [-0.5, 0.5],
           "l2": "inputs larger than L2 (1.07 GB field per batch)"}
    if extra:
        cfg.update(extra)
    return cfg


# ----------------------------------------------------------------------------- CPU baseline
def _cpu_worker(args):
    """Advance the oracle on one volume by n half-sweeps; returns the half-sweep wall time."""
    i, n = args
    sys.path.insert(0, ROOT)
    from oracle.sor import OracleSolve
    from taufactor_gb300.synthetic import blurred_noise

    por = np.random.default_rng(999).uniform(0.35, 0.70, N_VOL)[i]
    o = OracleSolve(blurred_noise((SIDE,) * 3, SIGMA, por, 1000 + i), kind="binary")
    t0 = time.perf_counter()
    o.half_sweep(n)
    return time.perf_counter() - t0


def cpu_baseline(pool, workers):
    """Voxel-updates/s of the reference arithmetic on the host cores (one process per volume).

    Each worker builds its volume and times only its half-sweeps; volumes run in waves of
    `workers` processes, so the batch's sweep wall time is (slowest volume) x (waves).
    """
    times = pool.map(_cpu_worker, [(i, CPU_SAMPLE_HALF_SWEEPS) for i in range(N_VOL)])
    sweep_wall = max(times) * math.ceil(N_VOL / workers)
    vu = N_VOL * CPU_SAMPLE_HALF_SWEEPS * SIDE ** 3 / 2
    return vu / sweep_wall, {"sample": f"{CPU_SAMPLE_HALF_SWEEPS} half-sweeps on each of the {N_VOL} volumes "
                                       f"({workers} processes, numpy float32 restatement)",
                             "cores": workers}


# ----------------------------------------------------------------------------- the reference itself
REF_HALF_SWEEPS = 100  # one sample: 100 half-sweeps, i.e. one convergence check of the reference


def reference_module():
    """The reference package installed under baseline/_ref (its plotting imports stubbed), or None."""
    from oracle.ref_shim import import_reference

    return import_reference(os.path.join(ROOT, "baseline", "_ref"))


def workload_volume(i: int) -> np.ndarray:
    """Volume i of the 16 x 256^3 workload, alone (the same draws as synthetic.batch_256)."""
    from taufactor_gb300.synthetic import blurred_noise

    por = np.random.default_rng(999).uniform(0.35, 0.70, i + 1)[i]
    return blurred_noise((SIDE,) * 3, SIGMA, por, 1000 + i)


def reference_cpu_sample(tau, i: int, half_sweeps: int = REF_HALF_SWEEPS):
    """The reference's own Solver(device='cpu') on volume i (taufactor.py:380-385, :156-191):
    set-up, then solve(iter_limit=half_sweeps). Returns (solve s, set-up s, half-sweeps done)."""
    import contextlib
    import io

    vol = workload_volume(i)
    with contextlib.redirect_stdout(io.StringIO()):  # its "not converged" notice
        t0 = time.perf_counter()
        s = tau.Solver(vol, device="cpu")
        t1 = time.perf_counter()
        s.solve(iter_limit=half_sweeps, verbose=False, conv_crit=CONV_CRIT)
        t2 = time.perf_counter()
    return t2 - t1, t1 - t0, int(s.iter)


def reference_cuda_rate(tau, half_sweeps: int = 200):
    """The reference's own torch-eager GPU path (device='cuda') on the whole 16 x 256^3 batch:
    voxel-updates/s of solve(iter_limit=half_sweeps) after a 100-half-sweep warm-up solve."""
    import contextlib
    import io

    import torch

    from taufactor_gb300.synthetic import batch_256

    vols = batch_256(N_VOL, SIDE, SIGMA)
    with contextlib.redirect_stdout(io.StringIO()):
        s = tau.Solver(vols, device="cuda")
        s.solve(iter_limit=100, verbose=False, conv_crit=CONV_CRIT)
        s = tau.Solver(vols, device="cuda")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(iter_limit=half_sweeps, verbose=False, conv_crit=CONV_CRIT)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    rate = s.iter * vols.size / 2 / dt
    del s
    torch.cuda.empty_cache()
    return {"value": rate, "unit": UNIT, "half_sweeps": half_sweeps,
            "what": "the reference's Solver(device='cuda') (torch eager) on the same 16 x 256^3 batch, "
                    "solve(iter_limit=200) after a warm-up solve; informational"}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------- arms
def run_reference(args):
    """The reference arm: the reference's own CPU Solver on the host cores (baseline/_ref), each
    step one bounded sample of the workload (volume step % 16, set-up excluded, 100 half-sweeps
    with the reference's convergence check); without an installed reference, the oracle's numpy
    restatement of its op sequence (kind "port"). Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    tau = reference_module()
    if tau is None:
        return run_reference_port(args)
    import torch

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    V = SIDE ** 3
    for w in range(args.warmup):
        reference_cpu_sample(tau, w % N_VOL, 10)
    rates, setups = [], []
    for j in range(args.steps):
        dt, ts, n = reference_cpu_sample(tau, j % N_VOL)
        rates.append(n * V / 2 / dt)
        setups.append(ts)
    v = float(np.median(rates))
    sample = (f"taufactor {getattr(tau, '__version__', '1.2.1')} Solver(device='cpu'), torch {torch.__version__} "
              f"with {cores} threads: per step one 256^3 volume of the workload (volume step % {N_VOL}), "
              f"solve(iter_limit={REF_HALF_SWEEPS}) timed after set-up (set-up median "
              f"{float(np.median(setups)):.2f} s)")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "reference", "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if torch.cuda.is_available() and not getattr(args, "no_reference_cuda", False):
        try:
            out["reference_torch_cuda"] = reference_cuda_rate(tau)
        except Exception as e:  # informational only
            out["reference_torch_cuda"] = {"unavailable": f"{type(e).__name__}: {e}"}
    print(json.dumps(out), flush=True)


def run_reference_port(args):
    """Reference arm without an installed reference: the oracle's float32 restatement."""
    workers = min(N_VOL, os.cpu_count() or 1)
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        for _ in range(args.warmup):
            pool.map(_cpu_worker, [(i, 1) for i in range(N_VOL)])
        rates = []
        for _ in range(args.steps):
            times = pool.map(_cpu_worker, [(i, CPU_SAMPLE_HALF_SWEEPS) for i in range(N_VOL)])
            sweep_wall = max(times) * math.ceil(N_VOL / workers)
            rates.append(N_VOL * CPU_SAMPLE_HALF_SWEEPS * SIDE ** 3 / 2 / sweep_wall)
    v = float(np.median(rates))
    sample = (f"{CPU_SAMPLE_HALF_SWEEPS} half-sweeps on each of the {N_VOL} volumes, {workers} processes "
              "(numpy float32 restatement of the reference's op sequence)")
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": workers, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def rank_volumes(rank: int, n: int = N_VOL) -> range:
    """Indices in the seeded volume sequence that rank `rank` solves: its own n consecutive
    volumes, so rank 0's batch is the single-GPU workload and no two ranks share a volume."""
    return range(rank * n, rank * n + n)


def _rank_entry(local: int, world: int, port: int, target, targs):
    """One process of a self-launched multi-GPU run: the environment torchrun would give it."""
    os.environ.update(RANK=str(local), LOCAL_RANK=str(local), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    target(*targs)


def spawn_ranks(world: int, target, *targs):
    """Run target(*targs) in `world` processes with RANK / LOCAL_RANK / WORLD_SIZE / MASTER_*
    set as torchrun sets them (rendezvous on 127.0.0.1, a free port)."""
    import socket

    import torch.multiprocessing as tmp

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    tmp.spawn(_rank_entry, args=(world, port, target, targs), nprocs=world, join=True)


def check_world(gpus: int, env=None) -> bool:
    """True when this process must launch the ranks itself (--gpus N > 1 without torchrun);
    a WORLD_SIZE that disagrees with --gpus is an error."""
    env = os.environ if env is None else env
    ws = env.get("WORLD_SIZE")
    if ws is not None and int(ws) != gpus:
        raise SystemExit(f"bench.py: WORLD_SIZE={ws} but --gpus {gpus}; launch exactly one rank per GPU")
    return ws is None and gpus > 1


def combine_ranks(ms: float, units: float, world: int, device=None):
    """(max over the ranks of the timed region in ms, sum over the ranks of the units they
    processed); the values themselves at N = 1. Every rank must call it."""
    if world == 1:
        return ms, units
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def run_ours(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pool = None
    workers = min(N_VOL, os.cpu_count() or 1)
    ref_tau = reference_module() if (rank == 0 and world == 1 and not args.no_cpu_baseline) else None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and ref_tau is None:
        # the oracle port instead; started before any CUDA call (spawned workers never touch the GPU)
        pool = mp.get_context("spawn").Pool(workers)
    import torch

    import taufactor_gb300 as tg
    from taufactor_gb300 import _capi
    from taufactor_gb300.synthetic import batch_256

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    vols = batch_256(N_VOL, SIDE, SIGMA, first=rank_volumes(rank).start)  # each rank its own volumes
    V = vols.size  # voxels in this rank's batch

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    s = tg.Solver(vols, device=dev)
    if args.tile is not None:  # fixed kernel configuration (e.g. to repeat a run under a profiler)
        from taufactor_gb300.autotune import apply
        apply(s, args.tile, args.kmax)
        tuning = {}
    else:
        tuning = {f"tile{t}_k{k}": round(ms, 5) for (t, k), ms in s.tune().items()}
    for _ in range(args.warmup):
        s.reset()
        s.solve(verbose=False, conv_crit=CONV_CRIT)
    lib = _capi.load()
    s.event_log = []
    iters, d_eff = [], None
    n0 = lib.tf_launch_count()
    barrier()
    with ClockSampler(local) as clk:
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            s.reset()
            s.solve(verbose=False, conv_crit=CONV_CRIT)
            iters.append(s.iter)
        e1.record()
        barrier()
    launches = lib.tf_launch_count() - n0
    half_sweeps = sum(iters)
    ms, vu_total = combine_ranks(e0.elapsed_time(e1), half_sweeps * V / 2, world, dev)
    value = vu_total / (ms / 1e3)
    solves_per_s = N_VOL * args.steps * world / (ms / 1e3)
    d_eff = s.D_eff.copy()
    # dominant kernel: the fused multi-half-sweep launches, timed by events around tf_advance
    adv_ms = sum(a.elapsed_time(b) for a, b, _ in s.event_log)
    adv_half = sum(n for _, _, n in s.event_log)
    kmax = s._op.k_max or 4
    n_tiled = sum(math.ceil(n / kmax) for _, _, n in s.event_log)
    s.event_log = None
    peak, peak_kind = measured_peak_hbm()
    achieved = adv_half * V / 2 * 8 / (adv_ms / 1e3) / 1e9  # GB/s of algorithmic bytes (8 B per update)
    algo_gb_launch = kmax * V / 2 * 8 / 1e9
    traffic_gb_launch = TRAFFIC_BYTES_PER_VOXEL_LAUNCH * V / 1e9 if (kmax == 4 and s._op.tile == 1) else None
    dram_min = n_tiled * V * 8 / (adv_ms / 1e3) / 1e9  # read + write of the field once per launch
    # accuracy: the timed result against the FP64 solution of the same operator (float64 defect
    # correction on the device to a relative residual of 1e-10)
    # (multigrid-PCG inner solves; the same correction with SOR inner solves timed beside it)
    # untimed warm-up of both refinement paths on a 64^3 crop: the first use of each kernel in a
    # process (module loading, library pages read from disk on a fresh machine) took up to 3 s,
    # which the timed refinement below must not include
    warm = tg.Solver(np.ascontiguousarray(vols[:2, :64, :64, :64]), device=dev)
    warm.solve(verbose=False, conv_crit=CONV_CRIT)
    for inner in ("mg", "sor"):
        warm.refine(tol=1e-10, inner=inner)
    del warm
    ref = tg.Solver(vols, device=dev)
    ref.solve(verbose=False, conv_crit=CONV_CRIT)
    cur0 = ref._cur.clone()
    refine_s = {}
    for inner in ("mg", "sor"):
        ref._cur.copy_(cur0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hist = ref.refine(tol=1e-10, inner=inner)
        torch.cuda.synchronize()
        refine_s[inner] = {"seconds": time.perf_counter() - t0, "outer_steps": len(hist) - 1,
                           "final_relative_residual": hist[-1]}
        if inner == "mg":
            d_mg = ref.D_eff.copy()
    rel_err = float(np.max(np.abs(d_eff - ref.D_eff) / np.abs(ref.D_eff)))
    mg_vs_sor = float(np.max(np.abs(d_mg - ref.D_eff) / np.abs(ref.D_eff)))
    fp64_resid = hist[-1]
    del ref, cur0
    # end to end through the public API from host buffers: the labels in pinned host memory (a
    # NumPy view of a page-locked buffer, which the Solver's upload copies by DMA), copied into
    # HBM by every step
    vols_host = torch.empty(vols.shape, dtype=torch.uint8, pin_memory=True).numpy()
    vols_host[...] = vols
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 2))
    h2d = d2h = 0
    for _ in range(e2e_steps):
        s2 = tg.Solver(vols_host, device=dev)
        s2.solve(verbose=False, conv_crit=CONV_CRIT)
        _ = float(s2.D_eff[0])
        h2d += vols.nbytes + 4 * SIDE
        d2h += (s2.iter // 100) * (8 * N_VOL * (2 * SIDE - 1) + 4)
        e2e_iters = s2.iter
        del s2
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = e2e_steps * e2e_iters * V / 2 / e2e_s
    secondary = None
    if rank == 0 and world == 1 and not args.no_secondary:
        secondary = secondary_metrics(dev)
    cpu = None
    if pool is not None:
        rate, info = cpu_baseline(pool, workers)
        pool.close()
        cpu = {"value": rate, "unit": UNIT, "cores": info["cores"], "kind": "port", "sample": info["sample"]}
    elif ref_tau is not None:
        cores = os.cpu_count() or 1
        torch.set_num_threads(cores)
        reference_cpu_sample(ref_tau, 0, 10)  # warm-up
        samples = [reference_cpu_sample(ref_tau, i) for i in range(2)]
        rate = float(np.median([n * SIDE ** 3 / 2 / dt for dt, _, n in samples]))
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "reference",
               "sample": f"the reference's Solver(device='cpu') on volumes 0 and 1 of the workload, "
                         f"solve(iter_limit={REF_HALF_SWEEPS}) after set-up, torch with {cores} threads"}
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config({"parallelism": f"{world} independent batches" if world > 1 else "1 GPU",
                                   "half_sweeps_per_solve": int(np.mean(iters))}),
        "solves_per_s": solves_per_s,
        "accuracy": {"max_rel_D_eff_vs_fp64": rel_err, "fp64_relative_residual": fp64_resid,
                     "fp64_reference": "float64 defect correction of the same operator on the device",
                     "fp64_refine_to_1e-10": {"multigrid_pcg": refine_s["mg"], "sor": refine_s["sor"],
                                              "speedup": refine_s["sor"]["seconds"] / refine_s["mg"]["seconds"],
                                              "max_rel_D_eff_multigrid_vs_sor": mg_vs_sor}},
        "kernel_config": {"tile": int(s._op.tile), "half_sweeps_per_launch": int(kmax), "autotune_ms_per_half_sweep": tuning},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind, "traffic": traffic_gb_launch, "traffic_unit": "GB per launch (ncu)",
                     "algorithmic_GB_per_launch": algo_gb_launch,
                     "per_unit": "8 B per voxel-update (read + write of float32 c)",
                     "dram_min_GBps": dram_min, "kernel": f"k_stream ({kmax} half-sweeps per launch)",
                     "avg_launch_ms": adv_ms / max(n_tiled, 1)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d // e2e_steps,
                "d2h_bytes_per_step": d2h // e2e_steps},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    if cpu:
        out["cpu_baseline"] = cpu
    if secondary:
        out.update(secondary)
    print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def secondary_metrics(dev):
    """The metric's other parts, on the same GPU after the main measurement: converged solves/s of
    the 64-volume uneven batch against the per-volume loop (FP32, and FP32 + FP64 correction to a
    relative residual of 1e-4), and the adjoint/forward time with a central-difference check of
    the gradient on 8 voxels of the 320^3 per-voxel conductivity field; and the design loop cut
    to 384^3 and 3 steps (per-step time, gradient checks)."""
    u = uneven_batch(dev, repeat=1, refine_tols=(1e-4,), reference_tol=1e-10)
    r4 = u["refined"]["0.0001"]
    a = adjoint_cost(dev, side=320, fd_voxels=8, phases=False)
    # untimed warm-up on 64^3: the first optimizer step and warm start of a process took seconds
    # on a fresh machine (kernel modules loaded on first use), which the timed steps must not hold
    design_loop(dev, side=64, steps=2)
    dl = design_loop(dev, side=384, steps=3)
    return {
        "design_loop_384_3steps": {"workload": dl["workload"] + " (the 768^3 loop cut to 384^3 and 3 steps)",
                                   "method": dl["method"], "mean_step_s": dl["mean_step_s"], "first_step_s": dl["first"]["forward_s"] +
                                   dl["first"]["adjoint_s"], "last_step_s": dl["last"]["forward_s"] +
                                   dl["last"]["adjoint_s"], "max_euler_rel_err": dl["max_euler_rel_err"],
                                   "direction_fd_rel_err": dl["direction_fd_rel_err"],
                                   "last_fp64_residual": dl["last"]["fp64_residual"],
                                   "last_adjoint_residual": dl["last"]["adjoint_residual"]},
        "uneven_batch": {"workload": u["workload"], "batched_solves_per_s": u["batched_solves_per_s"],
                         "per_volume_loop_solves_per_s": u["per_volume_loop_solves_per_s"],
                         "speedup_vs_loop": u["speedup"], "refined_1e-4_solves_per_s": r4["solves_per_s"],
                         "refined_1e-4_speedup_vs_loop": r4["speedup_vs_loop"],
                         "max_rel_D_eff_vs_fp64": u["max_rel_D_eff_loop_vs_fp64"],
                         "refined_1e-4_max_rel_D_eff_vs_fp64": r4["max_rel_D_eff_vs_fp64"],
                         "max_rel_D_eff_batched_vs_loop": u["max_rel_D_eff_batched_vs_loop"]},
        "adjoint": {"workload": a["workload"], "inner_solve": a["inner_solve"], "forward_s": a["forward_s"],
                    "adjoint_s": a["adjoint_s"], "adjoint_over_forward": a["adjoint_over_forward"],
                    "forward_multigrid_only_s": a["forward_multigrid_only_s"],
                    "sor_inner_forward_s": a["sor_inner"]["forward_s"], "sor_inner_adjoint_s": a["sor_inner"]["adjoint_s"],
                    "fd_voxels": a["fd_voxels"],
                    "fd_h": a["fd_h"], "fd_max_rel_err": a["fd_max_rel_err"],
                    "fd_direction_rel_err": a["fd_direction_rel_err"], "euler_rel_err": a["euler_rel_err"]},
    }


def uneven_batch(dev, conv_crit=CONV_CRIT, repeat=2, refine_tols=(1e-4, 1e-6, 1e-8), reference_tol=1e-10):
    """64 volumes with sides from {64..256} (half PeriodicSolver): batched solve (one graph per
    200 half-sweeps, device-side convergence) vs the plain per-volume loop of drop-in solvers.
    Both reach the same per-volume results; reported as converged solves/s."""
    import torch

    import taufactor_gb300 as tg
    from taufactor_gb300.synthetic import uneven_volumes

    vols = uneven_volumes(64)
    periodic = [i % 2 == 1 for i in range(len(vols))]
    voxels = sum(v.size for v in vols)
    b = tg.BatchSolve(vols, periodic=periodic, device=dev)
    b.solve(conv_crit=conv_crit)  # warm-up (graph capture)
    t_batch = []
    for _ in range(repeat):
        b = tg.BatchSolve(vols, periodic=periodic, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = b.solve(conv_crit=conv_crit)
        torch.cuda.synchronize()
        t_batch.append(time.perf_counter() - t0)
    iters = [r.iter for r in res]
    d_batch = np.array([r.D_eff[0] for r in res])
    t_ref = {}
    d_ref = {}
    # FP64 reference D_eff: the batch refined to a relative residual of reference_tol
    rr = tg.BatchSolve(vols, periodic=periodic, device=dev).solve(conv_crit=conv_crit,
                                                                  refine={"tol": reference_tol, "max_outer": 60})
    d_fp64 = np.array([r.D_eff[0] for r in rr])
    for tol in refine_tols:
        b = tg.BatchSolve(vols, periodic=periodic, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rr = b.solve(conv_crit=conv_crit, refine={"tol": tol})
        torch.cuda.synchronize()
        t_ref[tol] = time.perf_counter() - t0
        d_ref[tol] = (np.array([r.D_eff[0] for r in rr]), max(r.residual_history[-1] for r in rr))
    solvers = [(tg.PeriodicSolver if p else tg.Solver)(v, device=dev) for v, p in zip(vols, periodic)]
    for s in solvers[:4]:
        s.solve(verbose=False, conv_crit=conv_crit)  # warm-up
    solvers = [(tg.PeriodicSolver if p else tg.Solver)(v, device=dev) for v, p in zip(vols, periodic)]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    d_loop = []
    for s in solvers:
        s.solve(verbose=False, conv_crit=conv_crit)
        d_loop.append(s.D_eff[0])
    torch.cuda.synchronize()
    t_loop = time.perf_counter() - t0
    tb = min(t_batch)
    vu = sum(it * v.size / 2 for it, v in zip(iters, vols))
    return {"workload": "64 volumes, sides from {64,96,128,192,256}, blurred noise sigma=2, porosity U[0.35,0.70], "
                        "half PeriodicSolver", "voxels": int(voxels), "conv_crit": conv_crit,
            "batched_solves_per_s": 64 / tb, "per_volume_loop_solves_per_s": 64 / t_loop,
            "speedup": t_loop / tb, "batched_voxel_updates_per_s": vu / tb,
            "max_rel_D_eff_batched_vs_loop": float(np.max(np.abs(d_batch - np.array(d_loop)) /
                                                          np.abs(np.array(d_loop)))),
            "max_rel_D_eff_loop_vs_fp64": float(np.max(np.abs(np.array(d_loop) - d_fp64) / np.abs(d_fp64))),
            "fp64_reference": f"the batch refined to a relative residual of {reference_tol:g}",
            "refined": {f"{tol:g}": {"solves_per_s": 64 / t_ref[tol], "speedup_vs_loop": t_loop / t_ref[tol],
                                     "max_fp64_residual": d_ref[tol][1],
                                     "max_rel_D_eff_vs_fp64": float(np.max(np.abs(d_ref[tol][0] - d_fp64)
                                                                           / np.abs(d_fp64)))}
                        for tol in refine_tols},
            "timing": "wall clock excl. input generation and solver construction"}


def design_loop(dev, side=768, steps=50, lr=0.05, lam=0.5, tol=1e-8, conv_crit=1e-3, method="mg"):
    """Gradient-driven design loop on one side^3 volume: kappa = sigmoid(logits), logits =
    blur_sigma4(N(0,1)) from default_rng(5000); Adam on the logits maximising
    D_eff - lam * mean(kappa). Every step: forward solve warm-started from the previous step's
    field to an FP64 relative residual of tol, adjoint solve warm-started from the previous
    adjoint field. method "mg": FP64 correction with multigrid conjugate-gradient inner solves
    from the warm start (no float32 loop), adjoint likewise; "sor": the float32 loop to conv_crit
    and SOR inner solves. Reports per-step times, the solve and adjoint residuals, Euler's
    identity sum(kappa dD/dkappa) = D_eff per step and, at the last step, a directional central
    difference along the update direction."""
    inner = "mg" if method == "mg" else "sor"
    import torch
    from scipy.ndimage import gaussian_filter

    import taufactor_gb300 as tg

    logits0 = gaussian_filter(np.random.default_rng(5000).standard_normal((side,) * 3, dtype=np.float32), 4.0)
    logits = torch.from_numpy(logits0.astype(np.float32)).to(dev).requires_grad_(True)
    opt = torch.optim.Adam([logits], lr=lr, maximize=True)
    prev = None
    rows = []
    t_all = time.perf_counter()
    for k in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.no_grad():
            kap = torch.sigmoid(logits).float().contiguous()
        s = tg.KappaSolver(kap, device=dev)
        if prev is not None:
            s.warm_start(prev)
        s.solve(conv_crit=conv_crit, refine={"tol": tol, "max_outer": 40, "inner": inner}, method=method)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = s.gradient(tol=tol, max_outer=40, lam0=prev.lam if prev is not None else None, inner=inner)[0]
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        d = float(s.D_eff[0])
        euler = abs(float((s.kappa[0].double() * g).sum()) - d) / d
        with torch.no_grad():
            kk = kap.double()
            logits.grad = ((g - lam / kap.numel()) * kk * (1.0 - kk)).float()
        opt.step()
        rows.append({"step": k, "forward_s": t1 - t0, "adjoint_s": t2 - t1, "half_sweeps": s.iter, "D_eff": d,
                     "mean_kappa": float(kap.double().mean()), "objective": d - lam * float(kap.double().mean()),
                     "fp64_residual": s.residual_history[-1], "adjoint_residual": s.adjoint_history[-1],
                     "euler_rel_err": euler})
        if prev is not None:
            del prev
        prev = s
    total = time.perf_counter() - t_all
    # directional central difference of D_eff along the last gradient direction at the last kappa
    with torch.no_grad():
        kap = prev.kappa[0]
        direc = torch.sign(g).float()
        h = 1e-3

        def deff(kk):
            t = tg.KappaSolver(kk.contiguous(), device=dev)
            t.warm_start(prev)
            t.solve(conv_crit=conv_crit, refine={"tol": 1e-13, "max_outer": 40, "inner": inner}, method=method)
            return float(t.D_eff[0])

        kp = (kap + h * direc).float()
        km = (kap - h * direc).float()
        fd = (deff(kp) - deff(km)) / 2.0
        step = ((kp.double() - km.double()) / 2.0)
        ad = float((g * step).sum())
    return {"workload": f"design loop {side}^3, kappa = sigmoid(logits), logits = blur_sigma4(N(0,1)) rng 5000, "
                        f"Adam lr {lr} on D_eff - {lam} mean(kappa)", "method": method, "steps": steps, "total_s": total,
            "mean_step_s": total / steps, "first": rows[0], "last": rows[-1],
            "max_euler_rel_err": max(r["euler_rel_err"] for r in rows),
            "direction_fd_rel_err": abs(fd - ad) / abs(fd), "fd_h": h, "per_step": rows}


def electrode_throughput(dev, batch=4, side=256, conv_crit=1e-3, cpu_half_sweeps=10):
    """ElectrodeSolver on batch x side^3 three-label volumes (argmax of three blurred noise fields,
    sigma 2, default_rng(4000 + i); 1 = pore (conductive), 0 = active material (reactive),
    2 = inert): one solve to the reference's rule, voxel-updates/s of the whole solve, the
    fused kernel's effective bandwidth, and the oracle port's sweeps on the host cores."""
    import torch
    from scipy.ndimage import gaussian_filter

    import taufactor_gb300 as tg
    from oracle.sor import OracleSolve

    rngs = [np.random.default_rng(4000 + i) for i in range(batch)]
    vols = np.stack([np.argmax(np.stack([gaussian_filter(r.standard_normal((side,) * 3, dtype=np.float32), 2.0)
                                         for _ in range(3)]), axis=0).astype(np.uint8) for r in rngs])
    s = tg.ElectrodeSolver(vols, device=dev)
    s.solve(verbose=False, conv_crit=conv_crit, iter_limit=200)  # warm-up
    s = tg.ElectrodeSolver(vols, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.solve(verbose=False, conv_crit=conv_crit)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    vu = s.iter * vols.size / 2
    o = OracleSolve(vols[:1, : side // 4], kind="electrode")  # a quarter of one volume on the host
    t1 = time.perf_counter()
    o.half_sweep(cpu_half_sweeps)
    tc = time.perf_counter() - t1
    return {"workload": f"ElectrodeSolver {batch}x{side}^3, labels argmax of 3 blurred fields sigma 2 (rng 4000+i)",
            "conv_crit": conv_crit, "half_sweeps": int(s.iter), "converged": bool(s.converged),
            "tau": [float(v) for v in s.tau], "solve_s": t, "voxel_updates_per_s": vu / t,
            "effective_GBps_8B_per_update": vu / t * 8 / 1e9,
            "cpu_oracle_voxel_updates_per_s": cpu_half_sweeps * o.factor.size / 2 / tc,
            "cpu_sample": f"oracle port, 1 process, {cpu_half_sweeps} half-sweeps on 1x{side // 4}x{side}x{side}"}


def impedance_volume(side, seed, porosity=0.45, sigma=2.0):
    """Pore (1) / active material (0) from a blurred noise field thresholded at its `porosity`
    quantile; pore clusters that do not reach the inlet plane x = 0 become inert (2)."""
    from scipy.ndimage import gaussian_filter, label

    f = gaussian_filter(np.random.default_rng(seed).standard_normal((side,) * 3, dtype=np.float32), sigma)
    vol = (f > np.quantile(f, 1 - porosity)).astype(np.uint8)
    lab, _ = label(vol)
    keep = np.unique(lab[0][lab[0] > 0])
    vol[(vol == 1) & ~np.isin(lab, keep)] = 2
    return vol


def impedance_throughput(dev, side=256, nyq_side=64, cpu_half_sweeps=4):
    """ImpedanceSolver (complex128) on a side^3 pore volume (impedance_volume, seed 5000): the
    drop-in tau_e solve (two frequencies in sequence, the reference's rule), the sweep kernel
    alone timed with CUDA events (22 double operations per voxel-update), the oracle's
    half-sweeps on a quarter of the volume on the host; and the 26-frequency Nyquist sweep of a
    nyq_side^3 volume, sequential (the reference's loop) against solve_frequencies."""
    import contextlib
    import io

    import torch

    import taufactor_gb300 as tg
    from oracle import impedance as oi

    vol = impedance_volume(side, 5000)
    quiet = contextlib.redirect_stdout(io.StringIO())
    with quiet:
        w = tg.ImpedanceSolver(vol, device=dev)
        w.solve(verbose=False, iter_limit=200)  # warm-up
    s = tg.ImpedanceSolver(vol, device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with contextlib.redirect_stdout(io.StringIO()):
        s.solve(verbose=False)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    vu = s.sum_iter * vol.size / 2
    # kernel only: 200 half-sweeps of the converged field
    st = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = 200
    s.iter = 0
    e0.record(st)
    s._advance(n)
    e1.record(st)
    torch.cuda.synchronize()
    k_ms = e0.elapsed_time(e1) / n
    k_rate = vol.size / 2 / (k_ms * 1e-3)
    # host: the oracle's numpy half-sweep on a quarter of the volume
    stq = oi.setup(vol[: side // 4])
    fq = oi.init_field(stq, float(stq["frequency"][0]))
    code = (stq["nn"] + 8 * stq["nr"]).astype(np.int64)
    code[stq["mask"] == 0] = 0
    fac = oi.factor_table(float(stq["frequency"][0]))[code]
    cb = oi.chequerboard(stq["shape"], s.omega)
    t1 = time.perf_counter()
    for i in range(cpu_half_sweeps):
        oi.half_sweep(fq, fac, cb[i % 2], False)
    tc = time.perf_counter() - t1
    # Nyquist: 26 frequencies in sequence (reference loop) and side by side
    nv = impedance_volume(nyq_side, 5001)
    with contextlib.redirect_stdout(io.StringIO()):
        a = tg.ImpedanceSolver(nv, device=dev, mode="nyquist")
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        a.solve(verbose=False)
        torch.cuda.synchronize()
        t_seq = time.perf_counter() - t2
    b = tg.ImpedanceSolver(nv, device=dev, mode="nyquist")
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    r = b.solve_frequencies()
    torch.cuda.synchronize()
    t_bat = time.perf_counter() - t3
    # Red-black SOR with the reference's omega is unstable on this complex operator at the high
    # end of the sweep: fields grow to ~1e278 while the relative-error test still passes, so an
    # "impedance" of ~1e-278 is returned, and the sequential loop carries that field into every
    # lower frequency (it re-initialises only after a NaN). Physically meaningful results: the
    # converged, finite impedances of sane magnitude. The sequential loop is therefore run again
    # from the first frequency that solve_frequencies solved sanely, and the two are compared there.
    imp_b = np.asarray(r["impedance"])
    sane_b = np.asarray(r["converged"], dtype=bool) & np.isfinite(imp_b) & (np.abs(imp_b) > 1e-12) & \
        (np.abs(imp_b) < 1e12)
    agree, k0, a2 = [], None, None
    if sane_b.any():
        k0 = int(np.flatnonzero(sane_b)[0])
        with contextlib.redirect_stdout(io.StringIO()):
            a2 = tg.ImpedanceSolver(nv, device=dev, mode="nyquist")
            a2.frequency = a2.frequency[k0:]
            a2.solve(verbose=False)
        imp_a = np.array([complex(z) for z in a2.impedance])
        sane_a = np.array(a2.converged_freq, dtype=bool) & np.isfinite(imp_a) & (np.abs(imp_a) > 1e-12) & \
            (np.abs(imp_a) < 1e12)
        both = sane_a & sane_b[k0:]
        agree = [abs(imp_a[k] - imp_b[k0 + k]) / abs(imp_b[k0 + k]) for k in np.flatnonzero(both)]
    return {"workload": f"ImpedanceSolver {side}^3 pore volume (porosity 0.45, sigma 2, rng 5000; isolated pores inert)",
            "dtype": "complex128", "half_sweeps": int(s.sum_iter), "converged_freq": s.converged_freq,
            "taus": [float(np.asarray(v)[0]) for v in s.taus], "solve_s": t, "voxel_updates_per_s": vu / t,
            "kernel_ms_per_half_sweep": k_ms, "kernel_voxel_updates_per_s": k_rate,
            "kernel_fp64_Gops": 22 * k_rate / 1e9,
            "cpu_oracle_voxel_updates_per_s": cpu_half_sweeps * vol[: side // 4].size / 2 / tc,
            "cpu_sample": f"oracle port (numpy), 1 process, {cpu_half_sweeps} half-sweeps on {side // 4}x{side}x{side}",
            "nyquist": {"volume": f"{nyq_side}^3 (rng 5001)", "frequencies": int(len(a.frequency)),
                        "sequential_s": t_seq, "sequential_half_sweeps": int(a.sum_iter),
                        "sequential_converged": int(sum(a.converged_freq)),
                        "side_by_side_s": t_bat, "side_by_side_half_sweeps": [int(v) for v in r["iters"]],
                        "side_by_side_converged": int(r["converged"].sum()),
                        "side_by_side_sane": int(sane_b.sum()),
                        "blown_up_frequencies": int(np.sum(np.isfinite(imp_b) & (np.abs(imp_b) <= 1e-12))),
                        "sequential_from_first_sane": k0,
                        "compared_frequencies": len(agree),
                        "max_rel_diff_converged": float(max(agree)) if agree else None,
                        "note": "the sequential loop warm-starts each frequency from the previous one; "
                                "both stop at the reference's conv_crit 1e-3"}}


def adjoint_cost(dev, side=320, fd_voxels=0, tol=1e-12, fd_tol=1e-14, phases=True):
    """Per-voxel conductivity kappa = sigmoid(blur_2(2 N(0,1))) on side^3 (default_rng(3003)):
    forward solve + FP64 refinement, then the adjoint gradient; times and, with fd_voxels > 0,
    central finite differences (h = 1e-3) on random voxels (default_rng(3004))."""
    import torch
    from scipy.ndimage import gaussian_filter

    import taufactor_gb300 as tg

    warm = tg.KappaSolver(np.full((32, 32, 32), 0.5, dtype=np.float32), device=dev)  # first-call costs
    warm.solve(conv_crit=1e-3, refine={"tol": tol})
    warm.gradient(tol=tol)
    logits = gaussian_filter(2.0 * np.random.default_rng(3003).standard_normal((side,) * 3, dtype=np.float32), 2.0)
    kap = (1.0 / (1.0 + np.exp(-logits))).astype(np.float32)
    def timed(inner, method="sor"):
        s = tg.KappaSolver(kap, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.solve(conv_crit=1e-3, refine={"tol": tol, "inner": inner}, method=method)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        g = s.gradient(tol=tol, inner=inner)
        torch.cuda.synchronize()
        return s, g, t_fwd, time.perf_counter() - t0

    # the default: the reference's float32 loop to conv_crit, then FP64 correction and adjoint
    # with multigrid conjugate-gradient inner solves
    s, g, t_fwd, t_adj = timed("mg")
    s_sor, _, f_sor, a_sor = timed("sor")
    s_mg, _, f_mg, _ = timed("mg", method="mg")
    out = {"workload": f"kappa field {side}^3 = sigmoid(blur_sigma2(2 N(0,1)))", "inner_solve": "multigrid PCG",
           "forward_s": t_fwd, "adjoint_s": t_adj, "adjoint_over_forward": t_adj / t_fwd,
           "half_sweeps_forward": s.iter, "pcg_iterations": [int(i) for i, _ in s.multigrid().history],
           "fp64_residual": s.residual_history[-1], "adjoint_residual": s.adjoint_history[-1],
           "D_eff": float(s.D_eff[0]),
           # D_eff is homogeneous of degree 1 in kappa, so sum(kappa * dD_eff/dkappa) = D_eff
           "euler_rel_err": abs(float((s.kappa.double() * g).sum()) - float(s.D_eff[0])) / float(s.D_eff[0]),
           "forward_multigrid_only_s": f_mg, "forward_multigrid_only_D_eff_rel_diff":
               abs(float(s_mg.D_eff[0]) / float(s.D_eff[0]) - 1.0),
           "sor_inner": {"forward_s": f_sor, "adjoint_s": a_sor, "outer_steps": len(s_sor.residual_history) - 1,
                         "adjoint_outer_steps": len(s_sor.adjoint_history) - 1,
                         "D_eff_rel_diff": abs(float(s_sor.D_eff[0]) / float(s.D_eff[0]) - 1.0)}}
    del s_sor, s_mg
    # per-phase gradients of MultiPhaseSolver on the three-label volume (labels = argmax of three
    # blurred fields, default_rng(3000..3002), D = {0: 0, 1: 1, 2: 0.1}) against central
    # differences in D_1 and D_2 of the operator they differentiate: kappa = D[label] with float64
    # faces (the float32 faces of MultiPhaseSolver's own refined D_eff move in rounding steps that
    # dominate a difference of step 1e-3). D_0 = 0 is a one-sided point: a phase of zero
    # conductivity is not part of the system, so no central difference exists there.
    if not phases:
        return _adjoint_fd(out, s, g, kap, side, fd_voxels, fd_tol, dev) if fd_voxels else out
    from taufactor_gb300.synthetic import three_phase

    lab = three_phase(side)
    ds = {0: 0.0, 1: 1.0, 2: 0.1}
    m = tg.MultiPhaseSolver(lab, dict(ds), device=dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m.solve(verbose=False, conv_crit=1e-3, refine={"tol": tol})
    torch.cuda.synchronize()
    t_mf = time.perf_counter() - t0
    t0 = time.perf_counter()
    pg = m.phase_gradients(conv_crit=1e-3, tol=tol)
    torch.cuda.synchronize()
    t_pg = time.perf_counter() - t0
    phase = {"forward_s": t_mf, "phase_gradients_s": t_pg, "D_eff": float(m.D_eff[0]),
             "gradients": {str(p): float(v[0]) for p, v in pg.items()}}
    for p in (1, 2):
        h = 1e-3
        dd = []
        for sgn in (1, -1):
            dsp = dict(ds)
            dsp[p] = ds[p] + sgn * h
            kp = np.asarray([dsp[0], dsp[1], dsp[2]], dtype=np.float32)[lab]
            t = tg.KappaSolver(kp, device=dev)
            t.warm_start(m.kappa_solver)
            t.solve(conv_crit=1e-3, refine={"tol": fd_tol, "max_outer": 40})
            dd.append(float(t.D_eff[0]))
        hp = float(np.float32(ds[p] + h)) - float(np.float32(ds[p] - h))
        fd = (dd[0] - dd[1]) / hp
        phase[f"fd_rel_err_phase{p}"] = abs(fd - float(pg[p][0])) / abs(fd)
    out["multiphase_320"] = phase
    return _adjoint_fd(out, s, g, kap, side, fd_voxels, fd_tol, dev) if fd_voxels else out


def _adjoint_fd(out, s, g, kap, side, fd_voxels, fd_tol, dev):
    """Central differences (h = 1e-3) of D_eff on random voxels and along a random direction,
    against the adjoint gradient g of solver s."""
    import taufactor_gb300 as tg

    if fd_voxels:
        def deff(kk):
            t = tg.KappaSolver(kk, device=dev)
            t.warm_start(s)
            t.solve(conv_crit=1e-3, refine={"tol": fd_tol})
            return t.D_eff[0]

        rng = np.random.default_rng(3004)
        gn = g[0].cpu().numpy()
        errs = []
        for _ in range(fd_voxels):
            i = tuple(int(rng.integers(0, side)) for _ in range(3))
            kp, km = kap.copy(), kap.copy()
            kp[i] += np.float32(1e-3)
            km[i] -= np.float32(1e-3)
            fd = (deff(kp) - deff(km)) / (float(kp[i]) - float(km[i]))
            errs.append(abs(fd - gn[i]) / abs(fd))
        out["fd_h"] = 1e-3
        out["fd_voxels"] = fd_voxels
        out["fd_max_rel_err"] = float(max(errs))
        out["fd_median_rel_err"] = float(np.median(errs))
        # directional derivative along a random +-1 pattern over all voxels (strong signal)
        v = np.where(rng.random(kap.shape) < 0.5, -1.0, 1.0).astype(np.float32)
        kp = (kap + np.float32(1e-3) * v).astype(np.float32)
        km = (kap - np.float32(1e-3) * v).astype(np.float32)
        fd = (deff(kp) - deff(km)) / 2.0
        step = (kp.astype(np.float64) - km.astype(np.float64)) / 2.0
        out["fd_direction_rel_err"] = float(abs(fd - float((gn * step).sum())) / abs(fd))
    return out


def run_profile(args):
    """Small fixed workload for profiler captures: `--half-sweeps` half-sweeps of a
    `--batch` x `--side`^3 batch after 8 warm-up half-sweeps. Prints nothing to measure."""
    import torch

    import taufactor_gb300 as tg
    from taufactor_gb300.synthetic import batch_256

    if args.uneven:  # one batched solve of the 64 uneven volumes (half periodic)
        from taufactor_gb300.synthetic import uneven_volumes

        vols = uneven_volumes(64)
        b = tg.BatchSolve(vols, periodic=[i % 2 == 1 for i in range(len(vols))], device="cuda")
        b.solve(conv_crit=CONV_CRIT)
        torch.cuda.synchronize()
        print(f"profile workload done: uneven batch of {len(vols)} volumes, {max(r.iter for r in b.results)} "
              "half-sweeps for the slowest")
        return
    if args.impedance:  # ImpedanceSolver on one --side^3 pore volume (impedance_volume, seed 5000)
        s = tg.ImpedanceSolver(impedance_volume(args.side, 5000), device="cuda")
        s.frc = s.frequency[0]
        s.field = s.init_field_internal()
        s._set_factor(s.frc)
        s._advance(8)
        torch.cuda.synchronize()
        s._advance(args.half_sweeps)
        s._reduce()
        torch.cuda.synchronize()
        print(f"profile workload done: impedance {args.side}^3, {args.half_sweeps} half-sweeps")
        return
    if args.electrode:  # ElectrodeSolver on --batch three-label --side^3 volumes (electrode_throughput's)
        from scipy.ndimage import gaussian_filter

        rngs = [np.random.default_rng(4000 + i) for i in range(args.batch)]
        vols = np.stack([np.argmax(np.stack([gaussian_filter(r.standard_normal((args.side,) * 3, dtype=np.float32), 2.0)
                                             for _ in range(3)]), axis=0).astype(np.uint8) for r in rngs])
        s = tg.ElectrodeSolver(vols, device="cuda")
        s._advance(8)
        torch.cuda.synchronize()
        s._advance(args.half_sweeps)
        torch.cuda.synchronize()
        print(f"profile workload done: electrode {args.batch}x{args.side}^3, {args.half_sweeps} half-sweeps")
        return
    if args.anisotropic:  # AnisotropicSolver, spacing (1, 1.3, 0.7), on --batch volumes of the main workload
        s = tg.AnisotropicSolver(batch_256(args.batch, args.side, SIGMA), (1.0, 1.3, 0.7), device="cuda")
        s._advance(8)
        torch.cuda.synchronize()
        s._advance(args.half_sweeps)
        torch.cuda.synchronize()
        print(f"profile workload done: anisotropic {args.batch}x{args.side}^3, {args.half_sweeps} half-sweeps")
        return
    if args.multiphase:  # MultiPhaseSolver on the three-label --side^3 volume, --half-sweeps half-sweeps
        from taufactor_gb300.synthetic import three_phase

        s = tg.MultiPhaseSolver(three_phase(args.side), {0: 0.0, 1: 1.0, 2: 0.1}, device="cuda")
        s._advance(8)
        torch.cuda.synchronize()
        s._advance(args.half_sweeps)
        s._layer_means()
        torch.cuda.synchronize()
        print(f"profile workload done: multiphase {args.side}^3, {args.half_sweeps} half-sweeps")
        return
    if args.multigrid:  # KappaSolver --side^3 (C4 generator, rng 3003): one FP64 correction, multigrid PCG
        from scipy.ndimage import gaussian_filter

        lg = gaussian_filter(2.0 * np.random.default_rng(3003).standard_normal((args.side,) * 3, dtype=np.float32), 2.0)
        kap = (1.0 / (1.0 + np.exp(-lg))).astype(np.float32)
        s = tg.KappaSolver(kap, device="cuda")
        s.multigrid()
        torch.cuda.synchronize()
        s.solve(method="mg", refine={"tol": 1e-8})
        torch.cuda.synchronize()
        print(f"profile workload done: multigrid correction {args.side}^3, PCG iterations "
              f"{[i for i, _ in s.multigrid().history]}")
        return
    vols = batch_256(args.batch, args.side, SIGMA)
    cls = tg.PeriodicSolver if args.periodic else tg.Solver
    s = cls(vols, device="cuda")
    if args.tile is not None:
        from taufactor_gb300.autotune import apply
        apply(s, args.tile, args.kmax)
    s._advance(8)
    torch.cuda.synchronize()
    s._advance(args.half_sweeps)
    s._layer_means()
    torch.cuda.synchronize()
    print(f"profile workload done: {args.batch}x{args.side}^3, {args.half_sweeps} half-sweeps")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the uneven-batch and adjoint measurements")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="--impl reference: skip the reference's own GPU path")
    ap.add_argument("--tile", type=int, default=None, help="fixed tile shape instead of autotuning (0..3)")
    ap.add_argument("--kmax", type=int, default=4, help="with --tile: half-sweeps per launch (1..4)")
    ap.add_argument("--profile", action="store_true", help="run the small profiler workload only")
    ap.add_argument("--batch", type=int, default=4, help="--profile: volumes")
    ap.add_argument("--side", type=int, default=256, help="--profile: volume side")
    ap.add_argument("--half-sweeps", type=int, default=40, help="--profile: half-sweeps")
    ap.add_argument("--periodic", action="store_true", help="--profile: PeriodicSolver")
    ap.add_argument("--multiphase", action="store_true",
                    help="--profile: MultiPhaseSolver on the three-label --side^3 volume")
    ap.add_argument("--multigrid", action="store_true",
                    help="--profile: one multigrid-PCG FP64 correction of a --side^3 kappa field")
    ap.add_argument("--impedance", action="store_true", help="--profile: ImpedanceSolver on one volume")
    ap.add_argument("--anisotropic", action="store_true",
                    help="--profile: AnisotropicSolver (spacing 1, 1.3, 0.7) on --batch volumes of the workload")
    ap.add_argument("--electrode", action="store_true",
                    help="--profile: ElectrodeSolver on --batch three-label --side^3 volumes")
    ap.add_argument("--uneven", action="store_true", help="--profile: one batched solve of the uneven batch")
    ap.add_argument("--workload", choices=["uneven", "adjoint", "design", "electrode", "impedance"], default=None,
                    help="print the secondary measurement of this workload only")
    ap.add_argument("--fd-voxels", type=int, default=0, help="--workload adjoint: finite-difference check")
    ap.add_argument("--adj-side", dest="adj_side", type=int, default=320, help="--workload adjoint: volume side")
    ap.add_argument("--design-side", type=int, default=768, help="--workload design: volume side")
    ap.add_argument("--design-steps", type=int, default=50, help="--workload design: Adam steps")
    ap.add_argument("--design-method", choices=["mg", "sor"], default="mg",
                    help="--workload design: multigrid inner solves (mg) or the float32 loop + SOR (sor)")
    args = ap.parse_args()
    if args.workload:
        import torch

        dev = torch.device("cuda", 0)
        if args.workload == "uneven":
            print(json.dumps(uneven_batch(dev)), flush=True)
        elif args.workload == "electrode":
            print(json.dumps(electrode_throughput(dev)), flush=True)
        elif args.workload == "impedance":
            print(json.dumps(impedance_throughput(dev)), flush=True)
        elif args.workload == "design":
            print(json.dumps(design_loop(dev, args.design_side, args.design_steps, method=args.design_method)),
                  flush=True)
        else:
            print(json.dumps(adjoint_cost(dev, args.adj_side, args.fd_voxels)), flush=True)
    elif args.profile:
        run_profile(args)
    elif check_world(args.gpus):
        spawn_ranks(args.gpus, run_reference if args.impl == "reference" else run_ours, args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
