#!/usr/bin/env python
"""Benchmark of the labelling hot path (one JSON line on rank 0).

Workload (one step): cc3d-style connected components of a 512^3 uint32
Voronoi volume (4096 seeds, labels in [1, 2^20], one-voxel membrane, 2 % salt),
26-connectivity: provisional-label estimate, labelling, numbering and the
write of the uint32 output.  Inputs are synthetic and seeded.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl gb300 (default)
    value  GVoxels/s with the input resident in HBM (CUDA tensor through the
           public API, output allocated on the device).  The 512 MiB input is
           larger than L2 (129 MB), so no flush is needed between steps.
    e2e    the same metric through the C ABI with pinned host buffers: the
           host->device copy of the input and the device->host copy of the
           labels are inside the timed region.  Two host threads take
           alternate volumes (the library keeps a workspace and stream per
           thread); each of a volume's two stages (copy-in + tile pass,
           then numbering + write + copy-out) is held by one thread at a
           time, so one volume's copy-out overlaps the next one's copy-in
           and tile pass; the single-thread figure is reported beside it.
           Median of five K-step runs, every run listed.
--impl reference
    The reference's CPU implementation of the path on this machine's host
    cores: the compiled reference where it was built here (oracle/_ref), else
    the oracle's C restatement.  It is single-threaded, so each step labels
    one copy of the volume per core in parallel processes.

Multi-GPU (torchrun): every rank labels its own volume (replicas; the
path has no data exchange), value = all voxels / max over ranks of the time.
"""
from __future__ import annotations

import argparse
import concurrent.futures
import contextlib
import ctypes
import json
import os
import statistics as pystats
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "connected-components-3d_gb300"))

import numpy as np  # noqa: E402

METRIC = "GVoxels/s 512^3 uint32 26-conn labelling (bit-exact)"
SHAPE = (512, 512, 512)  # --size changes it for profiling captures only
N_SEEDS = 4096
LABEL_MAX = 1 << 20
CONN = 26
HBM_SPEC_GBS = 7900.0  # GB300 HBM3e nominal bandwidth; the roofline's peak is the measured copy rate


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    self.samples.append((time.perf_counter(), parts))
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()
        # the timed region starts once samples are flowing
        t0 = time.perf_counter()
        while not self.samples and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def window(self, t0: float, t1: float):
        """Summarise only the samples taken in [t0, t1] (the last earlier one if none)."""
        self.span = (t0, t1)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        samples = list(self.samples)
        if getattr(self, "span", None):
            t0, t1 = self.span
            inside = [x for x in samples if t0 <= x[0] <= t1]
            samples = inside or [x for x in samples if x[0] <= t1][-1:]
        rows = [r for _, r in samples]
        sm = [float(s[1]) for s in rows if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in rows if s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in rows:
            for name, v in zip(names, s[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": pystats.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if os.environ.get("CC3D_BENCH_BACKEND") != "gloo" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_volume(rank: int) -> np.ndarray:
    from cc3d_gb300 import synth
    return synth.voronoi_volume(SHAPE, N_SEEDS, LABEL_MAX, seed=1 + rank, dtype=np.uint32)


def host_cpu_model() -> str:
    """The host CPU's model name (lscpu), else the machine type."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_reference(vol: np.ndarray, budget_s: float = 20.0):
    """Time the reference's CPU path (compiled reference if present, else the
    oracle's C port) on the full workload volume, best of up to 3 runs."""
    import oracle
    oracle.build()
    kind = "reference" if oracle.have_reference() else "port"
    times = []
    t_start = time.perf_counter()
    N = None
    while len(times) < 3 and (time.perf_counter() - t_start) < budget_s:
        t0 = time.perf_counter()
        _, N = oracle.connected_components(vol, connectivity=CONN, return_N=True, backend=kind)
        times.append(time.perf_counter() - t0)
    best = min(times)
    return {"value": vol.size / best / 1e9, "unit": "GVoxels/s", "cores": 1, "cpu_model": host_cpu_model(),
            "kind": kind,
            "sample": f"full 512^3 uint32 volume, 26-conn, best of {len(times)} runs "
                      f"({best:.3f} s per volume, N={N})"}


_REF_VOLUME = None


def _ref_worker_init(path: str) -> None:
    global _REF_VOLUME
    _REF_VOLUME = np.load(path, mmap_mode="r")


def _ref_worker_label(_: int):
    """One labelling of the workload volume by the reference's CPU path (the
    compiled reference where present, else the oracle port); returns seconds."""
    import oracle
    kind = "reference" if oracle.have_reference() else "port"
    vol = np.ascontiguousarray(_REF_VOLUME)
    t0 = time.perf_counter()
    _, n = oracle.connected_components(vol, connectivity=CONN, return_N=True, backend=kind)
    return time.perf_counter() - t0, int(n)


def run_reference(args, world, rank):
    """The reference's CPU implementation on all host cores: the reference is
    single-threaded, so every step labels one copy of the workload volume per
    core, in parallel processes (spawned before any GPU use).  value = voxels
    labelled by all cores / wall time of the step."""
    if rank != 0:
        return
    import multiprocessing as mp
    import tempfile
    import oracle
    oracle.build()
    kind = "reference" if oracle.have_reference() else "port"
    vol = make_volume(0)
    cores = max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))
    # every process holds its copy of the input, the output and the union-find:
    # take no more processes than host memory allows (about 3 x the volume each)
    try:
        with open("/proc/meminfo") as f:
            avail = int(next(l for l in f if l.startswith("MemAvailable")).split()[1]) * 1024
        cores = max(1, min(cores, int(avail * 0.6 // (3 * vol.nbytes))))
    except (OSError, StopIteration, ValueError):
        pass
    shm = "/dev/shm" if os.path.isdir("/dev/shm") else None
    with tempfile.TemporaryDirectory(dir=shm) as tmp:
        path = os.path.join(tmp, "volume.npy")
        np.save(path, vol)
        ctx = mp.get_context("spawn")
        with ctx.Pool(cores, initializer=_ref_worker_init, initargs=(path,)) as pool:
            times = []
            for i in range(args.warmup + args.steps):
                t0 = time.perf_counter()
                res = pool.map(_ref_worker_label, range(cores), chunksize=1)
                dt = time.perf_counter() - t0
                if i >= args.warmup:
                    times.append(dt)
    ms = 1000.0 * sum(times) / len(times)
    value = cores * vol.size / (ms / 1000.0) / 1e9
    per_volume_s = float(np.median([r[0] for r in res]))
    line = {
        "metric": METRIC, "value": value, "unit": "GVoxels/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded Voronoi)",
        "config": {"workload": "512^3 uint32 Voronoi(4096 seeds, labels in [1,2^20])+membrane+2% salt, "
                               "connectivity 26, output uint32",
                   "volumes_per_step": cores, "l2": "input larger than L2"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "GVoxels/s", "cores": cores, "cpu_model": host_cpu_model(),
                         "kind": kind,
                         "sample": f"{cores} copies of the full 512^3 volume per step, one per core in "
                                   f"parallel processes ({per_volume_s:.3f} s per volume, N={res[0][1]})"},
        "e2e": {"value": value, "unit": "GVoxels/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


E2E_THREADS = 2  # host threads of the end-to-end leg
E2E_REPS = 5     # timed K-step runs of the end-to-end leg (median reported)


def run_gpu(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import cc3d_gb300 as cc3d
    cc3d.build()
    nat = cc3d._native
    lib = nat.load()
    cc3d.set_tile_pass(args.tile_pass)

    vol = make_volume(rank)
    voxels = vol.size
    dev = torch.from_numpy(vol).cuda()
    # the expected N for this volume, from one labelled warm-up
    out, N = cc3d.connected_components(dev, connectivity=CONN, return_N=True)
    torch.cuda.synchronize()
    out_dtype = out.dtype

    # ---------------- device-resident value
    for _ in range(args.warmup):
        cc3d.connected_components(dev, connectivity=CONN, return_N=True)
    torch.cuda.synchronize()
    nat.profile_enable(True)
    nat.profile_read()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_host0 = time.perf_counter()
    ev0.record()
    for _ in range(args.steps):
        _, n = cc3d.connected_components(dev, connectivity=CONN, return_N=True)
        assert n == N
    ev1.record()
    torch.cuda.synchronize()
    t_host1 = time.perf_counter()
    t_host = t_host1 - t_host0
    barrier(world)
    sampler.window(t_host0, t_host1)
    clocks = sampler.stop()
    stage = nat.profile_read()
    nat.profile_enable(False)
    ms_total = ev0.elapsed_time(ev1)
    ms_total = max_over_ranks(world, ms_total)
    ms_per_step = ms_total / args.steps
    value = world * voxels * args.steps / (ms_total / 1000.0) / 1e9

    info = nat.Prepared()
    sx, sy, sz = SHAPE[2], SHAPE[1], SHAPE[0]
    nat.check(lib.cc3d_gpu_label_prepare(dev.data_ptr(), nat.U32, sx, sy, sz, CONN, 0, 0,
                                         nat.IN_DEVICE | nat.OUT_DEVICE,
                                         ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                         ctypes.byref(info)))
    edges = int(info.edges)

    # ---------------- end to end through the C ABI with pinned host buffers
    pin_in = torch.from_numpy(vol).pin_memory()
    host_in = pin_in.numpy()
    osz = {torch.uint16: 2, torch.uint32: 4, torch.uint64: 8}[out_dtype]
    ocode = {2: nat.U16, 4: nat.U32, 8: nat.U64}[osz]
    pin_outs = [torch.empty(voxels * osz, dtype=torch.uint8).pin_memory() for _ in range(E2E_THREADS)]

    # With several threads, each of the two stages of a volume is held by one
    # thread at a time: the copy-in stage (prepare: input copy overlapped with
    # the tile pass) and the copy-out stage (finish: merge, numbering, write
    # overlapped with the label copy).  The threads then stay one stage apart,
    # so a volume's copy-out always runs beside the next volume's copy-in
    # (opposite directions of the host link) instead of the threads falling
    # into step and contending for the same direction.
    stage_in, stage_out = threading.Lock(), threading.Lock()

    def e2e_step(pin_out, staged=False):
        # prepare (input staged once; the estimate comes from the same pass),
        # then write the labels into the pinned host buffer
        info = nat.Prepared()
        with (stage_in if staged else contextlib.nullcontext()):
            nat.check(lib.cc3d_gpu_label_prepare(host_in.ctypes.data, nat.U32, sx, sy, sz, CONN, 0, 0, 0,
                                                 None, ctypes.byref(info)))
        n = ctypes.c_uint64(0)
        with (stage_out if staged else contextlib.nullcontext()):
            nat.check(lib.cc3d_gpu_label_finish(info.token, int(min(info.epl, voxels)), pin_out.data_ptr(),
                                                ocode, ctypes.byref(n), 0, None))
        return n.value

    # persistent host threads: the library keeps one device workspace per
    # thread, so the same threads serve the warm-up and the timed steps
    pool = concurrent.futures.ThreadPoolExecutor(E2E_THREADS)
    gate = threading.Barrier(E2E_THREADS, timeout=120)  # a thread that fails cannot hang the others

    def e2e_run(nsteps, nthreads):
        # nthreads > 1: volumes alternate between the pool's threads; each
        # labels its share one volume at a time through the C ABI (its own
        # workspace and stream), so one volume's label copy-out overlaps the
        # next one's copy-in and tile pass.  nthreads == 1: the calling thread.
        def worker(t):
            torch.cuda.set_device(local)
            gate.wait()  # every pool thread takes one share
            return [e2e_step(pin_outs[t], staged=True) for _ in range(t, nsteps, nthreads)]
        t0 = time.perf_counter()
        if nthreads == 1:
            ns = [e2e_step(pin_outs[0]) for _ in range(nsteps)]
        else:
            futs = [pool.submit(worker, t) for t in range(nthreads)]
            ns = [n for f in futs for n in f.result()]
        dt = time.perf_counter() - t0
        assert all(n == N for n in ns), "e2e N differs from the device path"
        return dt

    e2e_value = e2e_single = None
    e2e_stages = None
    reps_multi, reps_single = [], []
    if not args.skip_e2e:
        # every thread's workspace allocated and warm before timing
        e2e_run(max(args.warmup, 1) * E2E_THREADS, E2E_THREADS)
        e2e_run(max(args.warmup, 1), 1)
        # The host side of these copies is shared with other tenants of the
        # machine, so the K-step run is repeated (alternating with the
        # single-thread run) and the median reported, every repetition listed.
        reps_multi, reps_single = [], []
        for _ in range(E2E_REPS):
            barrier(world)
            t_e2e = max_over_ranks(world, e2e_run(args.steps, E2E_THREADS))
            reps_multi.append(world * voxels * args.steps / t_e2e / 1e9)
            barrier(world)
            t_one = max_over_ranks(world, e2e_run(args.steps, 1))
            reps_single.append(world * voxels * args.steps / t_one / 1e9)
        e2e_value = pystats.median(reps_multi)
        e2e_single = pystats.median(reps_single)
        expect = out.cpu().numpy().reshape(-1).view(np.uint8)
        for t in range(min(E2E_THREADS, args.steps)):
            assert np.array_equal(pin_outs[t].numpy(), expect), "e2e labels differ from the device path"
        pool.shutdown()
        # one more (untimed) step with the stage timer: where the end-to-end time goes
        nat.profile_enable(True)
        nat.profile_read()
        e2e_step(pin_outs[0])
        e2e_stages = {k: v[0] for k, v in nat.profile_read().items() if v[1]}
        nat.profile_enable(False)

    # ---------------- roofline of the dominant kernel
    peak, peak_kind = load_peaks()
    isz, osz_b = vol.itemsize, osz
    kern_bytes = {
        # algorithmic bytes per launch: the share of the job's (input + output)
        # traffic the kernel is responsible for
        "tile_local": voxels * isz,
        "write": voxels * osz_b,
    }
    per_launch = {k: (stage[k][0] / stage[k][1] if stage[k][1] else 0.0) for k in stage}
    dom = max(("tile_local", "write"), key=lambda k: per_launch[k])
    dom_ms = per_launch[dom]
    achieved = kern_bytes[dom] / (dom_ms / 1000.0) / 1e9 if dom_ms else 0.0
    job_bytes = voxels * (isz + osz_b)
    pipeline_gbs = job_bytes / (ms_per_step / 1000.0) / 1e9
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            traffic = json.load(f).get(dom)

    # the CPU baseline is one process's figure: timed at N = 1 only
    cpu = None
    if world == 1 and not args.skip_cpu:
        cpu = cpu_reference(vol)

    # the mixed-size stream: batched vs the plain per-volume path, and the
    # shipped cost model's regret on a held-out stream
    batch = None
    if world == 1 and not args.skip_batch:
        batch = measure_batch(batch_stream(BATCH_VOLUMES), max(3, min(args.steps, 10)), 3)
        batch["costmodel"] = costmodel_regret()

    launches_per_step = 6  # tile pass, edge merge, 3 numbering-scan kernels, label writer
    line = {
        "metric": METRIC, "value": value, "unit": "GVoxels/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (seeded Voronoi; the reference publishes no number for this config)",
        "config": {"workload": "512^3 uint32 Voronoi(4096 seeds, labels in [1,2^20])+membrane+2% salt, "
                               "connectivity 26, output uint32",
                   "volumes_per_step_per_gpu": 1, "N": N, "boundary_edges": edges,
                   "l2": "input (512 MiB) larger than L2, no flush"},
        "e2e": {"value": e2e_value, "unit": "GVoxels/s",
                "h2d_bytes_per_step": voxels * isz, "d2h_bytes_per_step": voxels * osz_b,
                "path": f"C ABI (cc3d_gpu_label_prepare + cc3d_gpu_label_finish) per volume, pinned host "
                        f"buffers, {E2E_THREADS} host threads taking alternate volumes (each with its own "
                        "workspace and stream; the prepare stage and the finish stage are each held by one "
                        "thread at a time, so one volume's label copy-out overlaps the next one's "
                        "copy-in and tile pass); within a call input and labels cross in 8 chunks "
                        "overlapped with the tile pass and the writer",
                "repetitions": {"runs": E2E_REPS, "steps_each": args.steps,
                                "values": reps_multi if e2e_value is not None else None,
                                "single_thread_values": reps_single if e2e_value is not None else None},
                "single_thread_value": e2e_single,
                "stage_ms": e2e_stages},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                     "algorithmic_bytes_per_launch": kern_bytes[dom], "avg_launch_ms": dom_ms,
                     "frac_of_spec": achieved / HBM_SPEC_GBS},
        "pipeline_roofline": {"algorithmic_bytes_per_step": job_bytes, "achieved_gbs": pipeline_gbs,
                              "frac": pipeline_gbs / peak, "frac_of_spec": pipeline_gbs / HBM_SPEC_GBS,
                              "stage_ms_per_step": {k: v[0] / args.steps for k, v in stage.items() if v[1]}},
        "cpu_baseline": cpu,
        "batch": batch,
        "clocks": clocks,
        "gpu_launches": launches_per_step * args.steps,
        "host_wall_s": t_host,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ------------------------------------------------------------ all workloads
def _workloads():
    """The benchmarked workloads: (name, volume factory, labelling kwargs)."""
    from cc3d_gb300 import synth
    vor512 = lambda: synth.voronoi_volume((512, 512, 512), 4096, 1 << 20, seed=1, dtype=np.uint32)  # noqa: E731
    out = [("voronoi512_u32_c%d" % c, vor512, dict(connectivity=c)) for c in (26, 18, 6)]
    out.append(("voronoi768_u64_c26", lambda: synth.voronoi_volume((768, 768, 768), 4096, 1 << 48, seed=2,
                                                                   dtype=np.uint64),
                dict(connectivity=26, out_dtype=np.uint64)))
    for p in (0.2, 0.3116, 0.5):
        f = (lambda p=p: synth.bernoulli_volume((512, 512, 512), p, seed=int(p * 1e4)))
        for c in (6, 18, 26):
            out.append((f"bernoulli{p}_512_u8_c{c}_binary", f, dict(connectivity=c, binary_image=True)))
        out.append((f"bernoulli{p}_512_u8_c6_binary_periodic", f,
                    dict(connectivity=6, binary_image=True, periodic_boundary=True)))
    img = lambda: synth.bernoulli_volume((8192, 8192), 0.5, seed=8192)  # noqa: E731
    for c in (8, 4):
        for b in (True, False):
            out.append((f"bernoulli0.5_8192x8192_u8_c{c}_{'binary' if b else 'multilabel'}", img,
                        dict(connectivity=c, binary_image=b)))
    return out


def run_all_configs(args):
    """One JSON line per workload: device-resident GVoxels/s of each tile-pass
    variant and of the autotuned choice (CUDA events, input larger than L2)."""
    import torch
    import cc3d_gb300 as cc3d
    cc3d.build()
    cache = {}
    for name, make, kw in _workloads():
        key = make
        if key not in cache:
            cache.clear()
            cache[key] = torch.from_numpy(make()).cuda()
        dev = cache[key]
        res = {}
        from cc3d_gb300.tuning import CONFIGS
        for variant in CONFIGS + ("auto",):
            if variant == "auto":
                cc3d.set_tile_pass("auto")
                tuned = cc3d.autotune(dev, connectivity=kw["connectivity"],
                                      binary_image=kw.get("binary_image", False))
            else:
                cc3d.set_tile_pass(variant)
            for _ in range(args.warmup):
                cc3d.connected_components(dev, **kw)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(args.steps):
                _, n = cc3d.connected_components(dev, return_N=True, **kw)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            res[variant] = {"ms": ms, "GVoxels/s": dev.numel() / ms / 1e6}
        cc3d.set_tile_pass("auto")
        print(json.dumps({"workload": name, "N": n, "voxels": dev.numel(), "tuned": tuned["best"],
                          "variants": res}), flush=True)


# ------------------------------------------------------------ connectivity graphs
def run_graphs(args):
    """Device-resident voxel_connectivity_graph (a stencil: one read of the
    labels, one write of the bitfield) and color_connectivity_graph on the
    headline volume; one JSON line per function."""
    import torch
    import cc3d_gb300 as cc3d
    cc3d.build()
    peak, peak_kind = load_peaks()
    vol = make_volume(0)
    dev = torch.from_numpy(vol).cuda()
    voxels = vol.size

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(args.steps):
            r = fn()
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / args.steps, r

    ms, vcg = timed(lambda: cc3d.voxel_connectivity_graph(dev, connectivity=26))
    nbytes = voxels * (vol.itemsize + 4)
    print(json.dumps({"metric": "GVoxels/s voxel_connectivity_graph 512^3 uint32, 26-connected (uint32 bits)",
                      "value": voxels / ms / 1e6, "unit": "GVoxels/s", "ms_per_step": ms,
                      "steps": args.steps, "warmup": args.warmup,
                      "roofline": {"bound": "hbm", "achieved": nbytes / ms / 1e6, "peak": peak, "unit": "GB/s",
                                   "frac": nbytes / ms / 1e6 / peak, "peak_source": peak_kind,
                                   "algorithmic_bytes_per_step": nbytes}}), flush=True)
    ms, res = timed(lambda: cc3d.color_connectivity_graph(vcg, connectivity=26, return_N=True))
    print(json.dumps({"metric": "GVoxels/s color_connectivity_graph 512^3 (uint32 graph of the volume), 26",
                      "value": voxels / ms / 1e6, "unit": "GVoxels/s", "ms_per_step": ms,
                      "steps": args.steps, "warmup": args.warmup, "N": int(res[1])}), flush=True)


# ------------------------------------------------------------ statistics
def run_statistics(args):
    """Device-resident statistics (voxel counts, bounding boxes, centroids; no
    slice conversion) of the labels of the headline volume, one JSON line.
    Algorithmic bytes: one read of the labels plus the three tables,
    sizeof(label) * voxels + (N + 1) * (4 + 6 * sizeof(bbox) + 24).  The
    result is checked against the oracle's, which is timed beside it on one
    host core."""
    import torch
    import cc3d_gb300 as cc3d
    cc3d.build()
    peak, peak_kind = load_peaks()
    vol = make_volume(0)
    labels, N = cc3d.connected_components(torch.from_numpy(vol).cuda(), connectivity=CONN, return_N=True)
    voxels = labels.numel()

    def stats():
        return cc3d.statistics(labels, no_slice_conversion=True)

    for _ in range(args.warmup):
        stats()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.steps):
        got = stats()
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    bbox_bytes = got["bounding_boxes"].element_size()
    nbytes = voxels * labels.element_size() + (N + 1) * (4 + 6 * bbox_bytes + 24)
    host = labels.cpu().numpy()
    import oracle
    times, t_start = [], time.perf_counter()
    while len(times) < 3 and time.perf_counter() - t_start < 20.0:
        t0 = time.perf_counter()
        exp = oracle.statistics(host, no_slice_conversion=True)
        times.append(time.perf_counter() - t0)
    exact = all(np.array_equal(got[k].cpu().numpy(), exp[k], equal_nan=(k == "centroids"))
                for k in ("voxel_counts", "bounding_boxes", "centroids"))
    assert exact, "statistics differ from the oracle"
    best = min(times)
    print(json.dumps({
        "metric": f"GVoxels/s statistics of the {SHAPE[0]}^3 uint32 labels (counts, boxes, centroids; exact)",
        "value": voxels / ms / 1e6, "unit": "GVoxels/s", "ms_per_step": ms, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "N": int(N), "exact_vs_oracle": exact,
        "roofline": {"bound": "hbm", "achieved": nbytes / ms / 1e6, "peak": peak, "unit": "GB/s",
                     "frac": nbytes / ms / 1e6 / peak, "peak_source": peak_kind,
                     "algorithmic_bytes_per_step": nbytes},
        "cpu_baseline": {"value": voxels / best / 1e9, "unit": "GVoxels/s", "cores": 1,
                         "cpu_model": host_cpu_model(), "kind": "port",
                         "sample": f"the same labels, oracle's numpy restatement, best of {len(times)} "
                                   f"({best:.3f} s)"},
        "config": {"workload": f"labels of the {SHAPE[0]}^3 uint32 Voronoi volume at connectivity 26 "
                               "(device tensors in and out)", "l2": "labels larger than L2"},
    }), flush=True)


# ------------------------------------------------------------ batched stream
_STREAM = None


def _stream_worker_init(path: str) -> None:
    global _STREAM
    _STREAM = np.load(path, mmap_mode="r")


def _stream_worker_label(task):
    """One volume of the mixed-size stream by the reference's CPU path (the
    compiled reference where present, else the oracle port); returns voxels."""
    import oracle
    off, shape, kind = task
    n = int(np.prod(shape))
    vol = np.ascontiguousarray(_STREAM[off:off + n]).reshape(shape)
    oracle.connected_components(vol, connectivity=26, backend=kind)
    return n


def cpu_stream_all_cores(vols, kind: str, reps: int = 3):
    """The whole mixed-size stream on every host core: one spawned process per
    core takes volumes largest first (the reference is single-threaded, so
    this is its upper CPU rate on the stream).  Median wall time of `reps`
    passes after one untimed pass."""
    import multiprocessing as mp
    import tempfile
    cores = max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1))
    offs = np.cumsum([0] + [v.size for v in vols])
    tasks = sorted(((int(offs[i]), v.shape, kind) for i, v in enumerate(vols)),
                   key=lambda t: -int(np.prod(t[1])))
    shm = "/dev/shm" if os.path.isdir("/dev/shm") else None
    with tempfile.TemporaryDirectory(dir=shm) as tmp:
        path = os.path.join(tmp, "stream.npy")
        np.save(path, np.concatenate([v.reshape(-1) for v in vols]))
        with mp.get_context("spawn").Pool(cores, initializer=_stream_worker_init, initargs=(path,)) as pool:
            pool.map(_stream_worker_label, tasks, chunksize=1)
            times = []
            for _ in range(reps):
                t0 = time.perf_counter()
                done = sum(pool.map(_stream_worker_label, tasks, chunksize=1))
                times.append(time.perf_counter() - t0)
    t = pystats.median(times)
    return {"value": done / t / 1e9, "unit": "GVoxels/s", "cores": cores, "cpu_model": host_cpu_model(),
            "kind": kind,
            "sample": f"all {len(vols)} volumes of the stream ({done} voxels) spread over {cores} spawned "
                      f"processes, largest first; median of {reps} passes ({t:.3f} s per pass)"}


BATCH_VOLUMES = 1024  # the mixed-size stream of the default line


def batch_stream(n: int):
    """The mixed-size stream: n uint16 Voronoi+membrane volumes, every edge
    log-uniform in [16, 256], one seed per 4096 voxels, labels in [1, 65535]."""
    from cc3d_gb300 import synth
    shapes = synth.batch_shapes(n, 16, 256, seed=12)
    return [synth.voronoi_volume(s, max(1, int(np.prod(s)) // 4096), 65535, seed=100 + i, dtype=np.uint16,
                                 salt=0.0) for i, s in enumerate(shapes)]


def measure_batch(vols, steps: int, warmup: int) -> dict:
    """The batched path against the plain per-volume path on the same stream,
    26-connectivity, device-resident inputs, both through the C ABI with
    outputs allocated beforehand.

    batched   cc3d_gpu_label_batch in the persistent mode (one cooperative
              kernel launch per batch, replayed from a CUDA graph); every
              timed step labels the stream in a fresh random order, so each
              step is a new batch layout.
    staged    the same calls in the staged mode (one launch per stage, the
              tuned tile pass; its graph is captured per layout, inside the
              timed region).
    api       cc3d.connected_components_batch (persistent), which also builds
              the descriptors and the per-volume output tensors in Python.
    per volume  one cc3d_gpu_label_prepare + cc3d_gpu_label_finish per volume
              (ctypes, device buffers), one tile-pass configuration
              (list/8x8) for all.
    Every volume's batched labels, N and dtype are checked against its
    per-volume result."""
    import torch
    import cc3d_gb300 as cc3d
    from cc3d_gb300 import batch as cbatch
    nat = cc3d._native
    lib = nat.load()
    voxels = int(sum(v.size for v in vols))
    dev = [torch.from_numpy(v).cuda() for v in vols]
    n = len(dev)
    tuned = cc3d.autotune_batch(dev, connectivity=26)
    rng = np.random.default_rng(5)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    # one output pool, 4 bytes per voxel, 256-byte aligned slices
    sizes = [((d.numel() * 4 + 255) // 256) * 256 for d in dev]
    pool = torch.empty((sum(sizes),), dtype=torch.uint8, device="cuda")
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    shapes = np.array([d.shape for d in dev], np.int64)
    ins = np.array([d.data_ptr() for d in dev], np.uint64)
    res = np.zeros(n, cbatch._RESULT_DTYPE)

    def abi_batch(order):
        desc = np.empty(n, cbatch._VOLUME_DTYPE)
        desc["in"] = ins[order]
        desc["out"] = pool.data_ptr() + offs[order]
        desc["sx"], desc["sy"], desc["sz"] = shapes[order, 2], shapes[order, 1], shapes[order, 0]
        nat.check(lib.cc3d_gpu_label_batch(desc.ctypes.data, n, nat.U16, 26, res.ctypes.data, stream))

    def batched():
        abi_batch(rng.permutation(n))

    def api():
        order = rng.permutation(n)
        return cc3d.connected_components_batch([dev[i] for i in order], connectivity=26, return_N=True)

    def timed(fn, k):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3) / k

    prev_mode = cc3d.set_batch_mode("persistent")
    try:
        ms_batch = timed(batched, steps)
        ms_api = timed(api, steps)
        cc3d.set_batch_mode("staged")
        ms_staged = timed(batched, steps)
    finally:
        cc3d.set_batch_mode(prev_mode)
    # the plain path: per-volume C ABI calls, preallocated uint32 outputs
    outs = [torch.empty(d.shape, dtype=torch.uint32, device="cuda") for d in dev]
    flags = nat.IN_DEVICE | nat.OUT_DEVICE
    prev = cc3d.set_tile_pass("list/8x8")

    def plain():
        out = []
        for d, o in zip(dev, outs):
            sz, sy, sx = d.shape
            info = nat.Prepared()
            nat.check(lib.cc3d_gpu_label_prepare(d.data_ptr(), nat.U16, sx, sy, sz, 26, 0, 0, flags, stream,
                                                 ctypes.byref(info)))
            nn = ctypes.c_uint64(0)
            code = nat.U16 if min(info.epl, d.numel()) < 65535 else nat.U32
            nat.check(lib.cc3d_gpu_label_finish(info.token, int(min(info.epl, d.numel())), o.data_ptr(), code,
                                                ctypes.byref(nn), flags, stream))
            out.append((nn.value, code))
        return out

    try:
        ms_plain = timed(plain, max(1, steps // 2))
        plain_res = plain()
    finally:
        cc3d.set_tile_pass(prev)
    # the persistent batch in stream order, checked volume by volume
    prev_mode = cc3d.set_batch_mode("persistent")
    try:
        abi_batch(np.arange(n))
        torch.cuda.synchronize()
    finally:
        cc3d.set_batch_mode(prev_mode)
    mismatches = 0
    out_bytes = 0
    for i, ((pn, pcode), o, d) in enumerate(zip(plain_res, outs, dev)):
        code, N = int(res["out_dtype"][i]), int(res["N"][i])
        w = 2 if code == nat.U16 else 4
        out_bytes += w * d.numel()
        got = pool[offs[i]:offs[i] + w * d.numel()]
        ref = o.reshape(-1).view(torch.uint8)[:w * d.numel()]  # (a uint16 result fills the first half)
        mismatches += int(pn != N or code != pcode or not torch.equal(got, ref))
    peak, peak_kind = load_peaks()
    alg_bytes = voxels * 2 + out_bytes
    gbs = alg_bytes / (ms_batch / 1e3) / 1e9
    return {"value": voxels / ms_batch / 1e6, "unit": "GVoxels/s", "ms_per_step": ms_batch,
            "path": "cc3d_gpu_label_batch, persistent mode: one cooperative kernel launch per batch, "
                    "replayed from a CUDA graph (C ABI, device buffers, outputs allocated beforehand)",
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                         "peak_source": peak_kind, "algorithmic_bytes_per_step": alg_bytes},
            "per_volume": {"value": voxels / ms_plain / 1e6, "unit": "GVoxels/s", "ms_per_step": ms_plain,
                           "path": "cc3d_gpu_label_prepare + cc3d_gpu_label_finish per volume (C ABI, "
                                   "device buffers), tile pass list/8x8 for every volume"},
            "ratio_batched_vs_per_volume": ms_plain / ms_batch,
            "staged": {"value": voxels / ms_staged / 1e6, "unit": "GVoxels/s", "ms_per_step": ms_staged,
                       "path": "cc3d_gpu_label_batch, staged mode: one launch per stage, the stage graph "
                               "captured per layout (tuned tile pass)"},
            "api": {"value": voxels / ms_api / 1e6, "unit": "GVoxels/s", "ms_per_step": ms_api,
                    "path": "cc3d.connected_components_batch (persistent), descriptors and output tensors "
                            "built in Python every step"},
            "mismatched_volumes": mismatches, "tuned": tuned,
            "workload": f"{len(vols)} uint16 Voronoi+membrane volumes, edges log-uniform in [16, 256], one seed "
                        "per 4096 voxels, connectivity 26, device-resident; each timed batched step in a "
                        "fresh volume order (a new layout)",
            "voxels": voxels}


def run_batch(args):
    """The mixed-size stream as its own line: the batched and per-volume GPU
    paths (measure_batch), the reference's CPU path on one core (a bounded
    sample) and on every host core (the whole stream)."""
    import cc3d_gb300 as cc3d
    cc3d.build()
    t0 = time.perf_counter()
    vols = batch_stream(args.batch)
    t_gen = time.perf_counter() - t0
    res = measure_batch(vols, args.steps, args.warmup)
    cpu = cpu_all = None
    if not args.skip_cpu:
        import oracle
        oracle.build()
        kind = "reference" if oracle.have_reference() else "port"
        done, t_cpu, t0 = 0, 0.0, time.perf_counter()
        k = 0
        while k < len(vols) and time.perf_counter() - t0 < 20.0:
            t1 = time.perf_counter()
            oracle.connected_components(vols[k], connectivity=26, backend=kind)
            t_cpu += time.perf_counter() - t1
            done += vols[k].size
            k += 1
        cpu = {"value": done / t_cpu / 1e9, "unit": "GVoxels/s", "cores": 1, "cpu_model": host_cpu_model(),
               "kind": kind,
               "sample": f"the first {k} volumes of the stream ({done} voxels), one after another"}
        cpu_all = cpu_stream_all_cores(vols, kind)
    line = {"metric": "GVoxels/s mixed-size stream, batched vs per-volume (bit-exact)"}
    line.update(res)
    line.update({"cpu_baseline": cpu, "cpu_all_cores": cpu_all, "generation_s": t_gen})
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------ cost model
COSTMODEL_HELD_OUT = 40  # volumes of the held-out stream timed by the default run


def costmodel_regret() -> dict:
    """The shipped cost model (cc3d_gb300/costmodel_params.npy) judged on a
    held-out-seed stream of COSTMODEL_HELD_OUT generated volumes (edges 64-256,
    the training generators): every configuration timed by the exhaustive
    autotuner, the model's pick compared with the best and with the plain
    single configuration (list/8x8)."""
    import cc3d_gb300 as cc3d
    cm = cc3d.costmodel
    if not cm.load():
        return {"unavailable": "no shipped parameters"}
    t0 = time.perf_counter()
    Xt, Yt, _ = cm.collect(COSTMODEL_HELD_OUT, seed=7, lo=64, hi=256, repeats=2)
    reg = cm.regret(Yt, cm.predict(Xt))
    reg.update({"volumes": int(Xt.shape[0]), "timings": int(np.isfinite(Yt).sum()), "held_out_seed": 7,
                "plain_config": "list/8x8", "seconds": time.perf_counter() - t0})
    return reg


def run_costmodel(args):
    """Train the cost model on autotuner timings of `args.costmodel` generated
    volumes (Voronoi with 1 to ~1e6 seeds, Bernoulli p 0.05-0.95, multilabel
    Bernoulli K 2-1000; uint8/16/32/64; edges 64-768; connectivity 26/18/6)
    and evaluate it on a held-out-seed stream by its regret against the
    exhaustive autotuner.  One JSON line; the parameters are saved where
    --save-params says (and loaded by set_tile_pass("model") when shipped in
    the package)."""
    import torch
    import cc3d_gb300 as cc3d
    cm = cc3d.costmodel
    cc3d.build()
    t0 = time.perf_counter()
    X, Y, _ = cm.collect(args.costmodel, seed=1, lo=64, hi=768, repeats=2)
    t_collect = time.perf_counter() - t0
    loss = cm.train(X, Y, epochs=300, batch=256, lr=1e-3, seed=0)
    t_train = time.perf_counter() - t0 - t_collect
    n_test = max(50, args.costmodel // 5)
    Xt, Yt, desc = cm.collect(n_test, seed=2, lo=64, hi=768, repeats=2)
    P = cm.predict(Xt)
    reg = cm.regret(Yt, P)
    low_conf = reg["fallback_fraction"]
    if args.save_params:
        os.makedirs(os.path.dirname(os.path.abspath(args.save_params)), exist_ok=True)
        cm.save(args.save_params)
    print(json.dumps({
        "metric": "cost-model regret vs exhaustive autotuner (held-out seeds)",
        "value": reg["mean_regret"], "unit": "fraction slower than the best configuration",
        "higher_is_better": False, "regret": reg, "low_confidence_fraction": low_conf,
        "train": {"volumes": int(X.shape[0]), "timings": int(np.isfinite(Y).sum()), "final_loss": loss,
                  "collect_s": t_collect, "train_s": t_train},
        "test": {"volumes": int(Xt.shape[0]), "timings": int(np.isfinite(Yt).sum())},
        "model": "FP32 MLP 16-64-64-12 (ReLU), Adam, trained by the library's CUDA kernels; outputs: "
                 "log-ms of list/runs x 8x8/4x16/16x4 x TMA/plain-load box",
        "plain_config": "list/8x8 (the default single configuration)",
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-batch", action="store_true", help="leave the mixed-size stream out of the line")
    ap.add_argument("--size", type=int, default=512, help="cube edge (profiling captures only)")
    ap.add_argument("--all-configs", action="store_true",
                    help="one line per benchmarked workload and tile-pass variant instead of the headline")
    ap.add_argument("--batch", type=int, default=0,
                    help="the mixed-size stream of this many volumes instead of the headline")
    ap.add_argument("--graphs", action="store_true",
                    help="voxel and colour connectivity graphs of the headline volume instead of the headline")
    ap.add_argument("--statistics", action="store_true",
                    help="statistics of the headline volume's labels instead of the headline")
    ap.add_argument("--costmodel", type=int, default=0,
                    help="train and evaluate the cost model on this many generated volumes instead of the headline")
    ap.add_argument("--save-params", default="", help="where --costmodel saves the trained parameters")
    ap.add_argument("--tile-pass", default="auto",
                    help="tile-pass configuration of the headline run: auto, list, runs or "
                         "<variant>/<shape> (profiling captures)")
    args = ap.parse_args()
    global SHAPE, N_SEEDS
    if args.size != 512:
        SHAPE = (args.size,) * 3
        N_SEEDS = max(1, 4096 * args.size ** 3 // 512 ** 3)
    if args.warmup < 3:
        args.warmup = 3
    if args.all_configs:
        run_all_configs(args)
        return
    if args.batch:
        run_batch(args)
        return
    if args.graphs:
        run_graphs(args)
        return
    if args.statistics:
        run_statistics(args)
        return
    if args.costmodel:
        run_costmodel(args)
        return
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
