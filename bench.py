"""Benchmark of the full space-charge kick (deposit + solve + interpolate).

Workload (one "step" = one full kick): a Lorentz-boosted anisotropic Gaussian
bunch of 1,000,000 macro-particles, sigma_x = sigma_y = 1 mm, sigma_z = 0.1 mm
(lab frame, draws beyond 5 sigma resampled, seed 42), gamma = 10, 1 nC in
equal weights, FP64 SoA positions and charges, on a 64 x 64 x 128 mesh
spanning +-5 sigma.  The mixed-precision kick (FP32 deposit/FFT/gather, FP64
IGF and origin offsets) is timed with the Green function rebuilt on every
kick (the reference rebuilds it in every solve!), inputs resident in HBM and
L2 flushed (256 MB write) between kicks.  The plain FP64 path (the
reference's algorithm with cuFFT Z2Z) is timed on the same inputs and the
mixed fields are compared with it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank runs the same kick on its own GPU
(replicas; the kick has no data-parallel exchange), the timed region is
bracketed by barriers and the max over ranks is reported.

--impl reference times the CPU restatement of the reference (oracle/, FP64
NumPy/SciPy, all host cores for the FFTs) on the same workload; rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "spacecharge.jl_gb300", "python"))

METRIC = "full kick ms (deposit+solve+interp), mixed vs FP64 at rel-err<=1e-5; grad ms"
GRID = (64, 64, 128)
NP = 1_000_000
SIGMA = (1e-3, 1e-3, 1e-4)
GAMMA = 10.0
QTOT = 1e-9
SEED = 42
BOUNDS = tuple((-5 * s for s in SIGMA)), tuple((5 * s for s in SIGMA))
WORKLOAD = "boosted Gaussian 1M particles, 64x64x128 mesh, gamma=10, +-5 sigma, FP64 particles"


def make_bunch(n=NP, seed=SEED, sigma=SIGMA):
    rng = np.random.default_rng(seed)
    out = []
    for s in sigma:
        v = rng.standard_normal(n)
        bad = np.abs(v) > 5.0
        while bad.any():
            v[bad] = rng.standard_normal(int(bad.sum()))
            bad = np.abs(v) > 5.0
        out.append(v * s)
    out.append(np.full(n, QTOT / n))
    return out


def algorithmic_bytes(np_, n, s_g, s_out=8):
    """Compulsory bytes of one kick: particles read by deposit (x,y,z,q) and
    gather (x,y,z) and written by the gather (Ex,Ey,Ez), rho written and read,
    E written and read (FFT intermediates and the Green spectrum excluded)."""
    return np_ * (32 + 24 + 3 * s_out) + n * 8 * s_g


# ----------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ distributed
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


# ------------------------------------------------------ batched bunches
BATCH_GRIDS = [(32, 32, 32), (64, 64, 64), (64, 64, 128), (128, 128, 128)]


def make_batch(nb=64, seed=7):
    """64 independent Gaussian bunches: particle counts log-uniform in
    [1e4, 2e6], sigma uniform in [0.2, 2] mm per axis, gamma uniform in
    [1, 50], charge uniform in [10 pC, 1 nC], grid drawn from BATCH_GRIDS."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nb):
        n = int(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        sig = rng.uniform(0.2e-3, 2e-3, 3)
        gamma = float(rng.uniform(1.0, 50.0))
        qtot = float(rng.uniform(10e-12, 1e-9))
        grid = BATCH_GRIDS[int(rng.integers(0, len(BATCH_GRIDS)))]
        v = rng.standard_normal((3, n)) * sig[:, None]
        out.append((grid, gamma, v[0].copy(), v[1].copy(), v[2].copy(), np.full(n, qtot / n)))
    return out


def bench_batch(sc, L, C, torch, flush, stream, ws, rank, steps, warmup):
    """Batched graph kick of this rank's shard of 64 bunches against the same
    bunches kicked one by one (mixed) and with the plain FP64 path."""
    from spacecharge_gb300.shard import shard_bunches

    spec_all = make_batch()
    mine = shard_bunches([len(s[2]) for s in spec_all], ws, rank)
    spec = [spec_all[i] for i in mine]
    dev = [[torch.from_numpy(a).cuda() for a in s[2:]] for s in spec]
    meshes = [sc.Mesh3D(g, d[0], d[1], d[2], precision="mixed", gamma=gm) for (g, gm, *_), d in zip(spec, dev)]
    batch = sc.Batch(meshes)
    xs, ys, zs, qs = zip(*dev)

    def ev_time(fn, reps):
        times = []
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        return float(np.mean(times))

    # the batch's own autotuner picks the group budget and the forward form
    # (untimed, like the warm-up)
    tuned_bytes, tuned_fused = batch.autotune(xs, ys, zs, qs)
    for _ in range(max(2, warmup)):
        batch.kick(xs, ys, zs, qs)  # first call eager + capture, then replays
    torch.cuda.synchronize()
    ms_batch = max_over_ranks(ev_time(lambda: batch.kick(xs, ys, zs, qs), steps), ws)
    nodes = batch.graph_nodes
    staged, staged_launches = batch.staged
    # the batch's fields, kept for the comparison with the plain FP64 kicks below
    bout = [[t.double().cpu() for t in o] for o in batch.kick(xs, ys, zs, qs)]
    bmesh = [m.efield.double().cpu() for m in meshes]
    # the same batch with every bunch's whole kick on 8 internal streams
    batch.set_staged(False)
    for _ in range(max(2, warmup)):
        batch.kick(xs, ys, zs, qs)
    torch.cuda.synchronize()
    ms_streams = max_over_ranks(ev_time(lambda: batch.kick(xs, ys, zs, qs), max(2, steps // 2)), ws)
    nodes_streams = batch.graph_nodes
    batch.set_staged(True)

    outs = [[torch.empty_like(d[0]) for _ in range(3)] for d in dev]

    def seq_mixed():
        for m, d, o in zip(meshes, dev, outs):
            L.call("sc_kick", m.ptr, *[C.c_void_p(t.data_ptr()) for t in d], d[0].numel(), L.SC_F64, 0,
                   *[C.c_void_p(t.data_ptr()) for t in o], C.c_void_p(stream.cuda_stream))

    seq_mixed()
    ms_seq = max_over_ranks(ev_time(seq_mixed, max(2, steps // 4)), ws)
    # plain FP64 path, one bunch at a time (meshes created and freed outside the timed region)
    ms_plain = 0.0
    err = {"mesh": [0.0, 0.0], "particles": [0.0, 0.0]}  # worst bunch: [max rel, RMS rel]

    def worse(key, a, r):
        e = (a - r).abs()
        err[key][0] = max(err[key][0], float(e.max() / r.abs().max()))
        err[key][1] = max(err[key][1], float(e.norm() / r.norm()))

    for (g, gm, *_), d, o, bo, bm in zip(spec, dev, outs, bout, bmesh):
        mp = sc.Mesh3D(g, d[0], d[1], d[2], precision="plain64", gamma=gm)
        k = lambda: L.call("sc_kick", mp.ptr, *[C.c_void_p(t.data_ptr()) for t in d], d[0].numel(), L.SC_F64, 0,
                           *[C.c_void_p(t.data_ptr()) for t in o], C.c_void_p(stream.cuda_stream))
        k()
        ms_plain += ev_time(k, 1)
        worse("mesh", bm, mp.efield.double().cpu())
        worse("particles", torch.stack(bo), torch.stack([t.cpu() for t in o]))
        del mp
    ms_plain = max_over_ranks(ms_plain, ws)
    npart = sum(len(s[2]) for s in spec)
    del batch
    return {"bunches": len(spec), "bunches_total": len(spec_all), "particles": npart,
            "grids": sorted({str(s[0]) for s in spec}), "ms_batched_graph": round(ms_batch, 3),
            "ms_sequential_mixed": round(ms_seq, 3), "ms_sequential_fp64_plain": round(ms_plain, 3),
            "speedup_vs_fp64_plain": round(ms_plain / ms_batch, 2), "graph_nodes": nodes,
            "staged_bunches": staged, "staged_launches": staged_launches,
            "autotuned": {"group_bytes": tuned_bytes if tuned_bytes < 2**62 else "unbounded",
                          "fused_forward": tuned_fused},
            "ms_batched_streams": round(ms_streams, 3), "graph_nodes_streams": nodes_streams,
            "max_rel_err_vs_fp64": {k: v[0] for k, v in err.items()},
            "rms_rel_err_vs_fp64": {k: v[1] for k, v in err.items()},
            "green": "cached per bunch (fixed geometry)", "l2": "flushed between calls"}


def bench_batch_graph(sc, torch, flush, stream, steps, warmup):
    """The 64-bunch batch graph alone, one group per grid class and two-pass
    forward transforms (no autotuning, no comparison kicks)."""
    spec = make_batch()
    dev = [[torch.from_numpy(a).cuda() for a in s[2:]] for s in spec]
    meshes = [sc.Mesh3D(g, d[0], d[1], d[2], precision="mixed", gamma=gm) for (g, gm, *_), d in zip(spec, dev)]
    batch = sc.Batch(meshes)
    batch.set_group_bytes(1 << 62)
    batch.set_fused_forward(False)
    xs, ys, zs, qs = zip(*dev)
    for _ in range(max(2, warmup)):
        batch.kick(xs, ys, zs, qs)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        batch.kick(xs, ys, zs, qs)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return {"bunches": len(spec), "ms_batched_graph": round(float(np.mean(times)), 3),
            "graph_nodes": batch.graph_nodes, "group_bytes": "unbounded", "fused_forward": False}


def bench_potential(sc, torch, dev, flush, stream, steps, warmup):
    """Scalar potential of the headline bunch's charge (sc_solve_potential),
    mixed and FP64 meshes (FP64 mode and double-FP32 mode), the potential
    Green function rebuilt every solve."""
    res = {"workload": WORKLOAD + ", scalar potential of the deposited charge", "green": "rebuilt every solve"}
    for prec in ("mixed", "fp64", "fp64_df32", "plain64"):
        m = sc.Mesh3D(GRID, *BOUNDS, precision="fp64" if prec == "fp64_df32" else prec, gamma=GAMMA,
                      total_charge=QTOT)
        if prec == "fp64_df32":
            m.set_fp64_arithmetic("df32")
        sc.deposit(m, *dev)
        m.set_green_cache(False)
        for _ in range(warmup):
            sc.solve_potential(m)
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps if prec != "plain64" else max(2, steps // 4)):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sc.solve_potential(m)
            b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        res["ms_" + prec] = round(float(np.mean(ts)), 4)
        del m
    return res


def flat_top_cylinder(n, seed=3):
    """Uniform cylinder of radius 1 mm and length 2 mm with a 0.05 mm Gaussian
    edge per transverse axis, z in [0.1, 2.1] mm above the cathode plane."""
    rng = np.random.default_rng(seed)
    r = 1e-3 * np.sqrt(rng.uniform(0, 1, n))
    th = rng.uniform(0, 2 * np.pi, n)
    x = r * np.cos(th) + rng.normal(0, 0.05e-3, n)
    y = r * np.sin(th) + rng.normal(0, 0.05e-3, n)
    z = rng.uniform(0.1e-3, 2.1e-3, n)
    return x, y, z


def bench_cathode(sc, L, C, torch, flush, stream, ws, steps, warmup):
    """4M particles, 100 pC, gamma 1.01, 128^3 mesh from the particles, cathode
    image on: mixed kick (Green rebuilt every kick) against the plain FP64
    path, and their field difference."""
    n = 4_000_000
    dev = [torch.from_numpy(v).cuda() for v in flat_top_cylinder(n)]
    dev.append(torch.full((n,), 100e-12 / n, dtype=torch.float64, device="cuda"))
    outs = [torch.empty_like(dev[0]) for _ in range(3)]

    def ev_time(fn, reps):
        for _ in range(warmup):
            fn()
        times = []
        for _ in range(reps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        return float(np.mean(times))

    res = {}
    fields = {}
    for prec in ("mixed", "plain64"):
        m = sc.Mesh3D((128, 128, 128), dev[0], dev[1], dev[2], precision=prec, gamma=1.01, total_charge=100e-12)
        m.set_green_cache(False)
        k = lambda: L.call("sc_kick", m.ptr, *[C.c_void_p(t.data_ptr()) for t in dev], n, L.SC_F64, 1,
                           *[C.c_void_p(t.data_ptr()) for t in outs], C.c_void_p(stream.cuda_stream))
        res[prec] = max_over_ranks(ev_time(k, steps if prec == "mixed" else 3), ws)
        fields[prec] = [t.cpu().numpy() for t in outs]
        del m
        torch.cuda.empty_cache()
    err = max(float(np.abs(a - b).max() / np.abs(b).max()) for a, b in zip(fields["mixed"], fields["plain64"]))
    return {"workload": "flat-top cylinder 4M particles on the cathode, 128^3, gamma=1.01, image on",
            "ms_mixed": round(res["mixed"], 4), "ms_fp64_plain": round(res["plain64"], 3),
            "speedup_vs_fp64_plain": round(res["plain64"] / res["mixed"], 2),
            "max_rel_err_vs_fp64_particles": err, "green": "rebuilt every kick", "l2": "flushed between kicks"}


# ---------------------------------------------------------- CPU reference
def cpu_kick_time(steps, warmup, bunch, max_seconds=None):
    """Time the oracle (FP64 NumPy/SciPy restatement of the reference) on the
    full workload; returns (ms per kick, kicks timed)."""
    import oracle as O

    x, y, z, q = bunch
    times = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        m = O.mesh_manual(GRID, *BOUNDS, gamma=GAMMA, total_charge=QTOT)
        O.kick(m, x, y, z, q)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
        if max_seconds is not None and sum(times) > max_seconds and times:
            break
    return 1e3 * float(np.mean(times)), len(times)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    bunch = make_bunch()
    ms, k = cpu_kick_time(args.steps, args.warmup, bunch)
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": round(ms, 3), "unit": "ms", "n_gpus": args.gpus,
        "steps": k, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Gaussian bunch)",
        "config": {"workload": WORKLOAD, "grid": list(GRID), "particles": NP, "gamma": GAMMA},
        "cpu_baseline": {"value": round(ms, 3), "unit": "ms", "cores": cores, "kind": "port",
                         "sample": f"{k} full kicks of the workload (FP64 oracle: serial deposit, "
                                   f"scipy.fft workers={cores})"},
        "e2e": {"value": round(ms, 3), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# -------------------------------------------------------------- GPU arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-cathode", action="store_true")
    ap.add_argument("--cathode-only", action="store_true",
                    help="time only the 4M-particle cathode workload (128^3, image on) and print its JSON object")
    ap.add_argument("--batch-only", action="store_true",
                    help="time only the 64-bunch batch workload and print its JSON object")
    ap.add_argument("--potential-only", action="store_true",
                    help="time only the scalar potential of the headline bunch and print its JSON object")
    ap.add_argument("--batch-graph-only", action="store_true",
                    help="replay only the 64-bunch batch graph in the configuration its autotuner usually "
                         "picks (one group per grid class, two-pass forward), W warm-up and K timed calls; "
                         "for launch lists")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # N ranks requested without a launcher: start them under torchrun,
        # one process per GPU, and pass its exit status on
        import socket
        import subprocess

        sock = socket.socket()
        sock.bind(("127.0.0.1", 0))
        port = sock.getsockname()[1]
        sock.close()
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", f"--master-port={port}", os.path.abspath(__file__)] + sys.argv[1:]
        return subprocess.call(cmd)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    ws, rank, local = dist_env()
    if local >= torch.cuda.device_count():
        raise SystemExit(f"rank {rank} needs GPU {local}, but only {torch.cuda.device_count()} are visible")
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__ as g

    g.build()
    import spacecharge_gb300 as sc
    from spacecharge_gb300 import _lib as L
    import ctypes as C

    bunch = make_bunch()
    dev = [torch.from_numpy(v).cuda() for v in bunch]
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    if args.cathode_only:
        res = bench_cathode(sc, L, C, torch, flush, stream, ws, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    if args.potential_only:
        res = bench_potential(sc, torch, dev, flush, stream, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    if args.batch_graph_only:
        res = bench_batch_graph(sc, torch, flush, stream, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    if args.batch_only:
        res = bench_batch(sc, L, C, torch, flush, stream, ws, rank, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0

    def timed(fn, steps, warmup, per_step_flush=True):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        barrier(ws)
        torch.cuda.synchronize()
        for a, b in evs:
            if per_step_flush:
                flush.zero_()
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
        return float(np.mean([a.elapsed_time(b) for a, b in evs]))

    ex, ey, ez = (torch.empty_like(dev[0]) for _ in range(3))

    def kick(m):
        return lambda: L.call("sc_kick", m.ptr, *[C.c_void_p(t.data_ptr()) for t in dev[:4]], NP, L.SC_F64, 0,
                              C.c_void_p(ex.data_ptr()), C.c_void_p(ey.data_ptr()), C.c_void_p(ez.data_ptr()),
                              C.c_void_p(stream.cuda_stream))

    # ---- mixed kick, Green function rebuilt each kick (headline value)
    mm = sc.Mesh3D(GRID, *BOUNDS, precision="mixed", gamma=GAMMA, total_charge=QTOT)
    mm.set_green_cache(False)
    kick(mm)()
    l0 = C.c_int64()
    L.call("sc_mesh_launch_count", mm.ptr, C.byref(l0))
    sampler = ClockSampler(local)
    sampler.start()
    ms_mixed = timed(kick(mm), args.steps, args.warmup)
    l1 = C.c_int64()
    L.call("sc_mesh_launch_count", mm.ptr, C.byref(l1))
    launches_per_kick = (l1.value - l0.value) / (args.steps + args.warmup)
    mixed_e = [t.double().cpu().numpy() for t in (ex, ey, ez)]
    mixed_grid = mm.efield.double().cpu().numpy()
    ms_mixed = max_over_ranks(ms_mixed, ws)

    # ---- stage times: the same kicks again with the per-stage CUDA events on
    #      (the Green build runs on a side stream, overlapping the deposit)
    L.call("sc_mesh_set_profiling", mm.ptr, 1)
    L.call("sc_mesh_stage_times", mm.ptr, None, None, C.c_void_p(stream.cuda_stream))  # reset
    timed(kick(mm), args.steps, 0)
    stage_ms = (C.c_double * L.SC_NUM_STAGES)()
    stage_n = (C.c_int64 * L.SC_NUM_STAGES)()
    L.call("sc_mesh_stage_times", mm.ptr, stage_ms, stage_n, C.c_void_p(stream.cuda_stream))
    L.call("sc_mesh_set_profiling", mm.ptr, 0)

    # ---- mixed kick with the Green spectrum reused (same geometry)
    mm.set_green_cache(True)
    ms_cached = max_over_ranks(timed(kick(mm), args.steps, args.warmup), ws)

    # ---- the hand-written FP64 pipeline (the Julia host's T=Float64), Green
    #      function rebuilt every kick and cached
    m64 = sc.Mesh3D(GRID, *BOUNDS, precision="fp64", gamma=GAMMA, total_charge=QTOT)
    m64.set_green_cache(False)
    ms_fp64 = max_over_ranks(timed(kick(m64), max(3, args.steps // 2), 3), ws)
    m64.set_green_cache(True)
    ms_fp64_cached = max_over_ranks(timed(kick(m64), max(3, args.steps // 2), 3), ws)
    fp64_grid = m64.efield.double().cpu().numpy()
    fp64_part = [t.double().cpu().numpy() for t in (ex, ey, ez)]
    # the same in double-FP32 mode (opt-in: the z pass, the inverse passes and
    # the interpolation with 48-bit significands)
    m64.set_fp64_arithmetic("df32")
    m64.set_green_cache(False)
    ms_fp64_df32 = max_over_ranks(timed(kick(m64), max(3, args.steps // 2), 3), ws)
    df32_err = {"mesh": float(np.abs(m64.efield.double().cpu().numpy() - fp64_grid).max() / np.abs(fp64_grid).max()),
                "particles": max(float(np.abs(t.double().cpu().numpy() - r).max() / np.abs(r).max())
                                 for t, r in zip((ex, ey, ez), fp64_part))}
    del m64

    # ---- plain FP64 path (reference algorithm, cuFFT Z2Z)
    mp = sc.Mesh3D(GRID, *BOUNDS, precision="plain64", gamma=GAMMA, total_charge=QTOT)
    ms_plain = max_over_ranks(timed(kick(mp), max(3, args.steps // 4), 3), ws)
    plain_e = [t.double().cpu().numpy() for t in (ex, ey, ez)]
    plain_grid = mp.efield.double().cpu().numpy()

    def rel(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max()), float(np.linalg.norm(a - b) / np.linalg.norm(b))

    err_grid = rel(mixed_grid, plain_grid)
    errs_p = [rel(a, b) for a, b in zip(mixed_e, plain_e)]
    err_part = (max(e[0] for e in errs_p), max(e[1] for e in errs_p))

    # ---- end to end through the public API with host buffers: sc_kick_host
    #      copies the page-locked particles in, kicks, copies the field out
    host_in = [torch.from_numpy(v).pin_memory() for v in bunch]
    host_out = [torch.empty(NP, dtype=torch.float64).pin_memory() for _ in range(3)]
    mm.set_green_cache(False)

    def e2e_step():
        L.call("sc_kick_host", mm.ptr, *[C.c_void_p(t.data_ptr()) for t in host_in], NP, L.SC_F64, 0,
               *[C.c_void_p(t.data_ptr()) for t in host_out], C.c_void_p(stream.cuda_stream))

    ms_e2e = max_over_ranks(timed(e2e_step, args.steps, args.warmup), ws)

    # ---- gradient: hand-written adjoint of the kick for the loss
    #      L = sum_i q_i Ez(x_i)^2 + eps0/2 sum_n |E_n|^2 dV
    #      (upstream dL/dEz_i = 2 q_i Ez_i, dL/dE_n = eps0 dV E_n)
    kick(mm)()
    eps0 = 8.8541878128e-12
    dV = float(np.prod([(BOUNDS[1][d] - BOUNDS[0][d]) / (GRID[d] - 1) for d in range(3)]))
    gez = (2.0 * dev[3] * ez).contiguous()
    gg = torch.zeros((GRID[2], GRID[1], GRID[0], 4), dtype=torch.float32, device="cuda")
    gg[..., :3] = (eps0 * dV) * mm.efield.permute(2, 1, 0, 3)
    dxyzq = [torch.empty_like(dev[0]) for _ in range(4)]

    def grad_step():
        L.call("sc_kick_adjoint", mm.ptr, *[C.c_void_p(t.data_ptr()) for t in dev[:4]], NP, L.SC_F64, 0, None,
               None, C.c_void_p(gez.data_ptr()), C.c_void_p(gg.data_ptr()),
               *[C.c_void_p(t.data_ptr()) for t in dxyzq], C.c_void_p(stream.cuda_stream))

    ms_grad = max_over_ranks(timed(grad_step, args.steps, args.warmup), ws)
    clocks = sampler.stop()

    # ---- tracking (the kick's caller): per step a kick, B from E and a
    #      relativistic Boris push of the device-resident bunch (sc_track),
    #      with the bounds refitted to the bunch every step (one extrema
    #      reduction and host read per step) or held; Green rebuilt as needed
    nstep = 10
    state = [t.clone() for t in dev[:3]] + [torch.zeros_like(dev[0]) for _ in range(3)]
    mt = sc.Mesh3D(GRID, dev[0], dev[1], dev[2], precision="mixed", gamma=GAMMA, total_charge=QTOT)

    def track(refit):
        return lambda: sc.track(mt, *state, dev[3], dt=1e-13, qm=-1.75882001076e11, steps=nstep, refit=refit)

    track_res = {"steps_per_call": nstep, "workload": WORKLOAD + ", bunch at rest, dt = 0.1 ps",
                 "ms_per_step_refit": round(max_over_ranks(timed(track(True), 3, 1), ws) / nstep, 4),
                 "ms_per_step_fixed_bounds": round(max_over_ranks(timed(track(False), 3, 1), ws) / nstep, 4)}
    del mt, state

    # ---- deposit alone in each mode (same particles, mixed mesh)
    dep_ms = {}
    for name, mode in (("atomic", L.SC_DEPOSIT_ATOMIC), ("sorted", L.SC_DEPOSIT_SORTED),
                       ("deterministic", L.SC_DEPOSIT_DETERMINISTIC), ("tiled", L.SC_DEPOSIT_TILED),
                       ("vector", L.SC_DEPOSIT_VECTOR)):
        dep = lambda: L.call("sc_deposit", mm.ptr, *[C.c_void_p(t.data_ptr()) for t in dev[:4]], NP, L.SC_F64, 1,
                             mode, C.c_void_p(stream.cuda_stream))
        dep_ms[name] = round(max_over_ranks(timed(dep, max(3, args.steps // 2), args.warmup), ws), 4)

    # ---- scalar potential of the same charge (mixed, FP64, plain FP64)
    pot_res = bench_potential(sc, torch, dev, flush, stream, max(3, args.steps // 2), args.warmup)

    # ---- cathode workload: 4M-particle flat-top cylinder on the cathode, 128^3
    cath_res = None
    if not args.no_cathode:
        del mp
        torch.cuda.empty_cache()
        cath_res = bench_cathode(sc, L, C, torch, flush, stream, ws, max(3, args.steps // 4), args.warmup)
        mp = None

    # ---- batched bunches (64 uneven bunches in one graph-replayed call)
    batch_res = None
    if not args.no_batch:
        mp = None
        torch.cuda.empty_cache()
        batch_res = bench_batch(sc, L, C, torch, flush, stream, ws, rank, max(3, args.steps // 2), args.warmup)

    # ---- roofline of the dominant stage: the longest stage on the caller's
    #      stream (CUDA events around it on that stream), multi-kernel stages
    #      included.  The Green build runs on a side stream beside the deposit
    #      and the forward passes and is not on the caller's stream.
    names = L.STAGES
    per = {names[k]: stage_ms[k] / max(1, stage_n[k]) for k in range(L.SC_NUM_STAGES) if stage_n[k]}
    nx, ny, nz = GRID
    N = nx * ny * nz
    Hx, Ly, Lz = 65, 128, 256
    # kernels and algorithmic bytes per launch of each stage on the caller's stream
    stages = {
        "deposit": ("memset + deposit_vector<double> + k_corner_sum", NP * 32 + N * 4),
        "zpass": ("k2_zpass<256, true>", Hx * Ly * nz * 8 + 3 * Hx * Ly * nz * 8),
        "gather": ("gather_packed<double,float>", NP * (24 + 24) + N * 16),
        "fwd_x": ("k2_fwd_x<128>", N * 4 + Hx * ny * nz * 8),
        "fwd_y": ("k2_col<128,fwd>", Hx * ny * nz * 8 + Hx * Ly * nz * 8),
        # inverse y and x run as one kernel (the stage timer files it under inv_y)
        "inv_y": ("k2_inv_yx<128>", 3 * Hx * Ly * nz * 8 + N * 16),
    }
    # DRAM bytes read + written per launch from one `ncu --set full` capture of
    # this workload (cold caches; written lines are still in L2 when a kernel
    # ends, so writes read ~0); the deposit stage: deposit_vector + k_corner_sum
    # (the corner memset writes 16.8 MB of zero sectors into L2)
    ncu_traffic = {"deposit": 51.9e6, "zpass": 15.10e6, "gather": 26.80e6, "fwd_x": 2.12e6, "fwd_y": 4.28e6,
                   "inv_y": 25.60e6}
    dom = max((k for k in stages if k in per), key=lambda k: per[k])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]), "measured"
    kname, abytes = stages[dom]
    ach = abytes / (per[dom] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": kname, "stage": dom, "achieved": round(ach, 1), "peak": peak,
                "unit": "GB/s", "frac": round(ach / peak, 4), "peak_source": peak_src,
                "traffic": ncu_traffic.get(dom), "algorithmic_bytes": abytes, "ms_per_launch": round(per[dom], 5),
                "note": "longest stage on the caller's stream, measured while the Green build runs beside it; "
                        "L2-resident working set: latency/issue-bound, not HBM-bound"}
    # the same for every stage, for reading the whole kick
    roofline["stages"] = {k: {"ms": round(per[k], 5), "GBps": round(stages[k][1] / (per[k] * 1e-3) / 1e9, 1)}
                          for k in stages if k in per}

    # ---- CPU baseline: the oracle on a bounded sample (rank 0, N = 1)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu_ms, k = cpu_kick_time(2, 0, bunch, max_seconds=30)
        cpu = {"value": round(cpu_ms, 2), "unit": "ms", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{k} full kicks of the same workload with the FP64 oracle (serial deposit, "
                         f"scipy.fft workers={os.cpu_count()})"}

    kick_bytes = algorithmic_bytes(NP, N, 4)
    line = {
        "metric": METRIC, "value": round(ms_mixed, 4), "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_mixed, 4), "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 IGF, offsets)",
        "data": "synthetic (seeded Gaussian bunch)",
        "config": {"workload": WORKLOAD, "grid": list(GRID), "particles": NP, "gamma": GAMMA,
                   "precision": "mixed", "green": "rebuilt every kick", "l2": "flushed (256 MB) between kicks",
                   "parallelism": f"replicas x{ws}"},
        "ms_fp64_plain": round(ms_plain, 4),
        "ms_fp64_native": round(ms_fp64, 4),
        "ms_fp64_native_green_cached": round(ms_fp64_cached, 4),
        "ms_fp64_native_df32": round(ms_fp64_df32, 4),
        "fp64_df32_max_rel_diff_vs_fp64": df32_err,
        "speedup_vs_fp64_plain": round(ms_plain / ms_mixed, 3),
        "ms_green_cached": round(ms_cached, 4),
        "max_rel_err_vs_fp64": {"mesh": err_grid[0], "particles": err_part[0]},
        "rms_rel_err_vs_fp64": {"mesh": err_grid[1], "particles": err_part[1]},
        "grad_ms": round(ms_grad, 4),
        "grad_over_forward": round(ms_grad / ms_mixed, 3),
        "grad_loss": "sum_i q_i Ez_i^2 + eps0/2 sum |E|^2 dV (adjoint recomputes deposit+solve)",
        "particles_per_s": round(ws * NP / (ms_mixed * 1e-3), 1),
        "kick_algorithmic_bytes": kick_bytes,
        "kick_GBps": round(kick_bytes / (ms_mixed * 1e-3) / 1e9, 1),
        "stage_ms": {k: round(v, 5) for k, v in per.items()},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": round(ms_e2e, 4), "unit": "ms", "h2d_bytes_per_step": 4 * NP * 8,
                "d2h_bytes_per_step": 3 * NP * 8},
        "deposit_modes_ms": dep_ms,
        "track": track_res,
        "potential": pot_res,
        "cathode_128": cath_res,
        "batch": batch_res,
        "gpu_launches": int(round(launches_per_kick * args.steps)),
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
