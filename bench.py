#!/usr/bin/env python
"""Benchmark of the GB300 3D backpropagation.

Metric: backprop voxel-angle updates/s (A * Nx * Ny * Nx per reconstruction)
on one GB300, FP32 GPU arithmetic against the FP64 oracle, with the rel-L2
error stated.

Workload (one step = one full reconstruction): ``backpropagate_3d`` with
A=200 angles uniform in [0, 2 pi), a 256x256 complex64 sinogram of a seeded
random-ellipsoid phantom (3-12 ellipsoids, semi-axes 8-60 px, n in
[1.335, 1.36], nm=1.333, res=3 px/wavelength, Rytov data a + i*phi),
padfac 1.75 (512x512 padded FFTs), intp_order=2, output 256^3 complex64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--config NAME]

--config selects another workload (one JSON line each, same keys):
  c1     the same reconstruction at A=60, 64x64 (the CPU-runnable case)
  c3     backpropagate_3d_tilted, A=220, 200x200, axis 0.2 rad from y
  c4     forward + vector-Jacobian product through the autograd wrapper
  c5     the learned wedge filter against the plain one
  rytov  sinogram_as_rytov of the headline sinogram's field
  apple  apple.correct of the headline reconstruction
  ri     odt_to_ri of a 256^3 volume (opt_to_ri beside it)
  bpp2d  backpropagate_2d, A=400 x 512
  mlp    the learned-gain network alone (tcgen05 and mma.sync kernels)

value   device-resident throughput (sinogram already in HBM; the prepared
        plan's kernels timed with CUDA events on their stream, L2 flushed
        between steps by a 256 MiB write outside the timed events)
e2e     the same metric through the public API ``backpropagate_3d`` with a
        pinned host sinogram in and a host volume out (H2D + D2H inside)
roofline  stage (b), the propagator + inverse 2D FFT (its two kernels,
        the largest share of the step), timed live with CUDA events around
        each launch: algorithmic bytes (spectra read + slabs written) over
        the two kernels' summed time, against MEASURED_PEAKS.json's HBM
        bandwidth, and their FP32 rate against the nominal FP32 peak
roofline_rotate  stage (c), resampling + accumulation, against HBM
roofline_step  every stage's algorithmic bytes over the whole step
accuracy  rel-L2 and max error of the timed volume against the FP64 oracle
        run over the whole workload (all angles)
cpu_baseline  that FP64 oracle run (the port of the reference's CPU path)
        on this host's cores
c3, c4, c5  (default run) the tilted, differentiation and learned-filter
        configurations measured in the same run after the headline (c3 with
        its own full-size oracle check, c5 over 200 held-out phantoms);
        --headline-only skips them
With --gpus N > 1 (torchrun), every rank runs an independent replica of the
workload (the path has no exchange step); value sums the ranks' updates
over the slowest rank's time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = ("backprop voxel-angle updates/s on 1 GB300, FP32 vs FP64 plain, "
          "at stated rel-L2")
UNIT = "voxel-angle updates/s"
WORKLOADS = {
    # the headline configuration (one GPU)
    "c2": dict(A=200, n=256, padfac=1.75, intp_order=2, res=3.0, nm=1.333,
               lD=0.0, seed=2024, count_range=(3, 12), semi_range=(8, 60),
               axis=None,
               name="backpropagate_3d: A=200 x 256x256 complex64 sinogram "
                    "(ellipsoid phantom) -> 256^3 complex64, padfac 1.75 "
                    "(512^2 FFTs), intp_order 2"),
    # tilted axis, 0.2 rad from y toward z
    "c3": dict(A=220, n=200, padfac=1.75, intp_order=2, res=3.0, nm=1.333,
               lD=0.0, seed=2025, count_range=(3, 12), semi_range=(8, 50),
               axis=(0.0, float(np.cos(0.2)), float(np.sin(0.2))),
               name="backpropagate_3d_tilted: A=220 x 200x200 complex64 "
                    "sinogram, axis 0.2 rad toward z -> 200^3 complex64, "
                    "padfac 1.75 (512^2 FFTs), intp_order 2"),
    # the reference's own CPU-sized case
    "c1": dict(A=60, n=64, padfac=1.75, intp_order=2, res=3.0, nm=1.333,
               lD=0.0, seed=2023, count_range=(1, 5), semi_range=(5, 20),
               axis=None,
               name="backpropagate_3d: A=60 x 64x64 -> 64^3, padfac 1.75 "
                    "(128^2 FFTs), intp_order 2"),
}
# differentiation and learned-filter configurations (single GPU; no
# counterpart in the reference)
WORKLOADS["c4"] = dict(
    A=90, n=128, res=3.0, nm=1.333, seed=5, count_range=(2, 6),
    semi_range=(6, 30), axis=None, padfac=1.75, intp_order=2, lD=0.0,
    name="differentiation: forward + vector-Jacobian product (sinogram and "
         "256x256 filter gain) through the autograd wrapper, A=90 x 128x128 "
         "-> 128^3, intp_order 2")
WORKLOADS["c5"] = dict(
    A=40, n=128, res=3.0, nm=1.333, seed=0, axis=None, padfac=1.75,
    intp_order=2, lD=0.0,
    name="learned wedge filter: A=40 uniform over 120 deg, 128x128 -> 128^3, "
         "shipped network (trained on 2000 phantoms); rel-L2 to the plain "
         "A=400 full-circle reconstruction on held-out phantoms")
# the learned-gain network alone on the wedge configuration's points
WORKLOADS["mlp"] = dict(
    A=40, n=128, res=3.0, nm=1.333, padfac=1.75,
    name="learned-gain MLP 4-64-64-64-2 (SiLU, BF16 operands, FP32 "
         "accumulation) on the 40-angle wedge configuration's filter support "
         "of the 256x256 padded grid: inference and backward")
# sinogram preparation of the headline sinogram (the step before the
# reconstruction; the reference's sinogram_as_rytov)
WORKLOADS["rytov"] = dict(
    A=200, n=256, res=3.0, nm=1.333, seed=2024, count_range=(3, 12),
    semi_range=(8, 60), axis=None,
    name="sinogram_as_rytov: A=200 x 256x256 complex64 field exp(a + i*phi) "
         "of the ellipsoid phantom -> Rytov sinogram, reliability-sorted 2D "
         "unwrap per frame + align_unwrapped")
# missing-apple-core correction of the headline reconstruction (the step
# after the reconstruction; the reference's apple.correct)
WORKLOADS["apple"] = dict(
    A=200, n=256, padfac=1.75, intp_order=2, res=3.0, nm=1.333, lD=0.0,
    seed=2024, count_range=(3, 12), semi_range=(8, 60), axis=None,
    name="apple.correct: 256^3 complex64 reconstruction of the headline "
         "sinogram, method nn, enforce_envelope 0.95, max_iter 100, "
         "min_diff 0.01 (single-precision 3D FFTs)")
# object function -> refractive index of the headline volume size (the
# reference's odt_to_ri; opt_to_ri timed beside it)
WORKLOADS["ri"] = dict(
    n=256, res=3.0, nm=1.333, seed=2024,
    name="odt_to_ri: 256^3 complex64 object function -> refractive index "
         "nm*sqrt(f/km^2+1) (principal root, real part made non-negative)")
# the 2D reconstruction: the central plane of the headline phantom, 400
# angles over the full circle, 512 detector pixels
WORKLOADS["bpp2d"] = dict(
    A=400, n=512, res=3.0, nm=1.333, lD=0.0, seed=2024,
    count_range=(3, 12), semi_range=(16, 120),
    name="backpropagate_2d: A=400 x 512 complex64 Rytov sinogram (central "
         "plane of an ellipsoid phantom) -> 512^2 complex64 image, padding "
         "to 2048 (2.1x rule, linear ramp to 0), cubic-spline rotation")
WORKLOAD = WORKLOADS["c2"]
WORKLOAD_NAME = WORKLOAD["name"]
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU oracle sample (and the rel-L2 check)")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--headline-only", action="store_true",
                    help="default configuration only: skip the tilted, "
                    "differentiation and learned-filter sub-results")
    ap.add_argument("--config", choices=sorted(WORKLOADS), default="c2",
                    help="workload (default c2, the headline configuration)")
    ap.add_argument("--ncu-rotate-case", action="store_true",
                    help="16 angles in one batch (one resampling launch) "
                    "for ncu captures of the resampling kernel")
    ap.add_argument("--ncu-n", type=int, default=128,
                    help="volume edge of the apple profiling case")
    ap.add_argument("--ncu-case", action="store_true",
                    help="profiling case: the workload's plane and volume "
                         "size with 8 angles and the save_memory workspace, "
                         "two executions, nothing else")
    return ap.parse_args()


def make_workload(w=None):
    from sino_gen import ellipsoid_phantom_sinogram
    w = WORKLOAD if w is None else w
    sino, angles = ellipsoid_phantom_sinogram(
        w["n"], w["A"], seed=w["seed"], count_range=w["count_range"],
        semi_range=w["semi_range"], res=w["res"], nm=w["nm"],
        axis=w["axis"] or (0, 1, 0))
    return sino.astype(np.complex64), angles


def updates(A, n):
    return float(A) * n * n * n


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu),
                 "--query-gpu=" + self.FIELDS, "--format=csv,noheader",
                 "-lms", "200", "-f", self.path],
                stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None

        def num(s):
            try:
                return float(s.split()[0])
            except (ValueError, IndexError):
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap")
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def stage_flops(rec, A):
    """Algorithmic FP32 flops of the two FFT stages of one reconstruction:
    5 N log2 N per complex N-point transform, 6 per complex multiply.
    Column stage: the forward y transform of every nonzero spectrum column
    once per angle, then per plane the propagator multiply and the backward
    y transform of those columns; row stage: per plane the backward x
    transform of every cropped row."""
    import math
    g = rec.padding_geometry
    lNy, lNx = g["lNy"], g["lNx"]
    _A, ny, nx = rec.shape
    nz = nx
    cols = np.unique(rec.filter_support() % lNx).size

    def f(n):
        return 5.0 * n * math.log2(n)
    planes = A * nz
    return {"columns_propagate": planes * cols * (f(lNy) + 6 * lNy)
            + A * cols * f(lNy),
            "rows_inverse": planes * ny * f(lNx)}


def profile_traffic(stage, units_per_launch):
    """DRAM bytes of one launch of `stage` from the committed ncu summary
    (profiles/dram_traffic.md), scaled from the captured launch to a launch
    of `units_per_launch` units; None if absent."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.md")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            parts = [p.strip() for p in line.strip().strip("|").split("|")]
            if len(parts) >= 3 and parts[0] == stage:
                try:
                    return float(parts[1]) / float(parts[2]) * units_per_launch
                except ValueError:
                    return None
    return None


# --------------------------------------------------------------- CPU side
def oracle_full(sino, angles, w):
    """The FP64 oracle over the whole workload (every angle), with all host
    threads; returns (seconds, volume, cores).  The propagator table of the
    reference's default path is built inside the timed call, as the
    reference builds it inside its own."""
    from oracle import odt_oracle
    cores = os.cpu_count() or 1
    s = sino.astype(np.complex128)
    kw = dict(lD=w["lD"], padfac=w["padfac"], intp_order=w["intp_order"],
              nthreads=cores, fft_workers=cores)
    t0 = time.perf_counter()
    if w["axis"] is None:
        vol = odt_oracle.backpropagate_3d(s, angles, w["res"], w["nm"], **kw)
    else:
        vol = odt_oracle.backpropagate_3d_tilted(
            s, angles, w["res"], w["nm"], tilted_axis=w["axis"], **kw)
    return time.perf_counter() - t0, vol, cores


def rel_errors(got, ref):
    """rel-L2 and max |error| / max |ref| of a GPU volume against the FP64
    oracle's."""
    got = np.asarray(got)
    return (float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
            float(np.abs(got - ref).max() / np.abs(ref).max()))


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation (the
    FP64 oracle port; the reference is pure Python) on this host's cores.
    One step = one angle of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import odt_oracle
    sino, angles = make_workload()
    w = WORKLOAD
    cores = os.cpu_count() or 1
    s = sino.astype(np.complex128)
    times = []
    # the propagator table is per-call setup in the reference, amortised
    # over its 200 angles; it is built in the first warm-up step here
    cache = {}
    for it in range(args.warmup + args.steps):
        a = it % w["A"]
        t0 = time.perf_counter()
        if w["axis"] is None:
            odt_oracle.backpropagate_3d(s, angles, w["res"], w["nm"],
                                        lD=w["lD"], padfac=w["padfac"],
                                        intp_order=w["intp_order"],
                                        nthreads=cores, fft_workers=cores,
                                        angle_subset=[a], cache=cache)
        else:
            odt_oracle.backpropagate_3d_tilted(
                s, angles, w["res"], w["nm"], lD=w["lD"],
                tilted_axis=w["axis"], padfac=w["padfac"],
                intp_order=w["intp_order"], nthreads=cores,
                fft_workers=cores, angle_subset=[a], cache=cache)
        dt = time.perf_counter() - t0
        if it >= args.warmup:
            times.append(dt)
    step = statistics.mean(times)
    value = updates(1, w["n"]) / step
    sample = ("one angle of the workload per step (256^3 updates), FP64, "
              "scipy.fft + OpenMP spline resampling")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "sample": "1 angle per step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _reference_line(args, metric, unit, value, step_s, workload, sample,
                    cores):
    return {
        "impl": "reference", "metric": metric, "value": value, "unit": unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic", "config": {"workload": workload,
                                        "sample": sample},
        "cpu_baseline": {"value": value, "unit": unit, "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}


def run_reference_rytov(args):
    """--impl reference for the sinogram preparation: the oracle port of
    the reference's sinogram_as_rytov (Kruskal unwrapping per frame, NumPy
    alignment) on a bounded sample of two frames per step."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import unwrap_oracle
    from sino_gen import ellipsoid_phantom_sinogram
    w = WORKLOAD
    ryt, _ = ellipsoid_phantom_sinogram(
        w["n"], w["A"], seed=w["seed"], count_range=w["count_range"],
        semi_range=w["semi_range"], res=w["res"], nm=w["nm"])
    field = np.exp(ryt)
    times = []
    k = 2
    for it in range(args.warmup + args.steps):
        a0 = (it * k) % (w["A"] - k)
        t0 = time.perf_counter()
        unwrap_oracle.sinogram_as_rytov(field[a0:a0 + k], align=True)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    step = statistics.mean(times)
    samples = k * field[0].size
    print(json.dumps(_reference_line(
        args, "sinogram_as_rytov samples/s on 1 GB300 (3D frames, FP32)",
        "sinogram samples/s", samples / step, step, w["name"],
        "2 of the 200 frames per step (oracle port of the reference: "
        "Kruskal unwrapping, NumPy alignment), FP64", 1)), flush=True)


def run_reference_apple(args):
    """--impl reference for the apple-core correction: the oracle port of
    the reference's apple.correct (NumPy + scipy.fft, single precision like
    pyFFTW) on a 256^3 volume, two iterations per step (setup and envelope
    included in the first)."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import apple_oracle
    w = WORKLOAD
    n = w["n"]
    g = np.arange(n) - n / 2
    z, y, x = np.meshgrid(g, g, g, indexing="ij", sparse=True)
    vol = (np.exp(-(x * x + y * y + z * z) / (0.1 * n * n))
           + 0.3 * np.exp(-((x - 0.2 * n) ** 2 + y * y + z * z) / 60.0))
    k = 2
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        apple_oracle.correct(vol, w["res"], w["nm"], max_iter=k,
                             min_diff=0.0)
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    step = statistics.mean(times)
    print(json.dumps(_reference_line(
        args, "apple.correct voxel-iterations/s on 1 GB300 (FP32 FFTs)",
        "voxel-iterations/s", float(n) ** 3 * k / step, step, w["name"],
        "2 iterations of a %d^3 correction per step (oracle port of the "
        "reference: NumPy + scipy.fft), setup and envelope included" % n,
        1)), flush=True)


def replica_throughput(units_per_rank, local_ms, world, device=None):
    """Whole-job throughput of `world` independent replicas, each having
    processed `units_per_rank` units in `local_ms`: the job takes as long
    as its slowest rank (max over ranks, one all-reduce), and the units of
    all ranks count.  Returns (units/s, job ms)."""
    t = float(local_ms)
    if world > 1:
        import torch
        import torch.distributed as dist
        x = torch.tensor([t], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return units_per_rank * world / (t / 1e3), t


# --------------------------------------------------------------- GPU side
def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    from odtbrain_gb300._alg3d import Backprop3D

    w = WORKLOAD
    sino, angles = make_workload()
    A, n = w["A"], w["n"]
    U = updates(A, n)
    host = torch.from_numpy(sino).pin_memory()
    dsino = host.to(dev)
    rec = Backprop3D(tuple(sino.shape), angles, w["res"], w["nm"], lD=w["lD"],
                     tilted_axis=w["axis"], padfac=w["padfac"],
                     intp_order=w["intp_order"], input_dtype="complex64",
                     device=dev)
    vol = torch.empty(rec.volume_shape(), device=dev, dtype=torch.complex64)
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    for _ in range(max(args.warmup, 1)):
        rec(dsino, out=vol)
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    stream = torch.cuda.current_stream(dev)
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        rec(dsino, out=vol, check=False)
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    rec.check()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    _, total_ms = replica_throughput(U * args.steps, sum(step_ms), world, dev)
    ms_per_step = total_ms / args.steps
    value = U * world / (ms_per_step / 1e3)

    # save_memory path (smaller angle batches), same result
    rec_sm = Backprop3D(tuple(sino.shape), angles, w["res"], w["nm"],
                        lD=w["lD"], tilted_axis=w["axis"], padfac=w["padfac"],
                        intp_order=w["intp_order"], save_memory=True,
                        input_dtype="complex64", device=dev)
    vol_sm = rec_sm(dsino)
    torch.cuda.synchronize()
    sm_ev = (torch.cuda.Event(enable_timing=True),
             torch.cuda.Event(enable_timing=True))
    flush.zero_()
    sm_ev[0].record(stream)
    rec_sm(dsino, out=vol_sm, check=False)
    sm_ev[1].record(stream)
    torch.cuda.synchronize()
    sm_ms = sm_ev[0].elapsed_time(sm_ev[1])
    sm_diff = float((vol_sm - vol).abs().max() / vol.abs().max())
    del rec_sm, vol_sm

    # per-stage live timing (event pair around every launch, the stages
    # serialised on one stream)
    flush.zero_()
    stages = rec.timed(dsino, out=vol)
    peak, peak_kind = measured_peaks()
    peak_source = ("measured (MEASURED_PEAKS.json hbm_gbs)"
                   if peak_kind == "measured" else "fallback 6.8 TB/s")
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    roofline, roofline_rotate, fp32, whole = stage_rooflines(
        rec, stages, A, n, w, peak, peak_source, sm_mhz, ms_per_step)
    stage_summary = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                         "share": round(v["ms"] / sum(x["ms"] for x in
                                                      stages.values()), 4),
                         "GB_per_s": (v["bytes"] / (v["ms"] / 1e3) / 1e9
                                      if v["ms"] > 0 else None)}
                     for k, v in stages.items()}

    # end to end through the public API, host buffers
    e2e = public_e2e(w, host, angles, U, args, world, dev, barrier)
    got_vol = vol.cpu().numpy() if rank == 0 else None

    line = None
    if rank == 0:
        extras = {}
        if not args.headline_only and args.config == "c2":
            # the other configurations, measured in this run after the
            # headline's timed region
            extras["c3"] = measure_recon_config(WORKLOADS["c3"], args, dev,
                                                flush, stream)
            extras["c4"] = measure_diff(args, dev)
            extras["c5"] = measure_learned(args, dev, n_eval=200)
        cpu = None
        accuracy = None
        if not args.no_cpu_baseline:
            t_cpu, ref, cores = oracle_full(sino, angles, w)
            cpu = {"value": U / t_cpu, "unit": UNIT, "cores": cores,
                   "kind": "port",
                   "sample": "the whole workload (all %d angles, %d x %d^3 "
                             "updates), FP64 oracle port (scipy.fft + OpenMP "
                             "C spline resampling), %.1f s"
                             % (A, A, n, t_cpu)}
            rel, mx = rel_errors(got_vol, ref)
            accuracy = {"rel_l2": rel, "max_abs_rel": mx,
                        "vs": "FP64 oracle, full A=%d (the measured "
                              "configuration)" % A}
            del ref
            if "c3" in extras:
                c3 = extras["c3"]
                t3, ref3, _ = oracle_full(c3.pop("_sino"), c3.pop("_angles"),
                                          WORKLOADS["c3"])
                rel3, mx3 = rel_errors(c3.pop("_volume"), ref3)
                c3["accuracy"] = {"rel_l2": rel3, "max_abs_rel": mx3,
                                  "vs": "FP64 oracle, full A=%d"
                                  % WORKLOADS["c3"]["A"]}
                c3["cpu_oracle_s"] = t3
                del ref3
        for v in extras.values():
            for k in [k for k in v if k.startswith("_")]:
                v.pop(k)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (complex64)", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "A": A, "n": n,
                       "padded_fft": rec.padding_geometry["lNx"], "intp_order": w["intp_order"],
                       "save_memory": False,
                       "l2": "flushed between steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "1 GPU"},
            "e2e": e2e,
            "gpu_launches": rec.launches_per_call * args.steps,
            "roofline": roofline,
            "roofline_rotate": roofline_rotate,
            "roofline_step": whole,
            "fp32_stages": fp32,
            "stages": stage_summary,
            "save_memory_ms_per_step": sm_ms,
            "save_memory_max_rel_diff": sm_diff,
            "accuracy": accuracy,
            "cpu_baseline": cpu,
            "clocks": clk,
            "step_ms": [round(x, 3) for x in step_ms],
        }
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def stage_rooflines(rec, stages, A, n, w, peak, peak_source, sm_mhz,
                    ms_per_step):
    """Rooflines from the per-stage CUDA-event times of one serialised
    execution.

    roofline: stage (b), the propagator + inverse FFT (k_columns_propagate
      + k_rows_inverse), the largest share of the step.  Algorithmic bytes
      (per reconstruction): the filtered spectra read, A*lNy*lNx*8, plus the
      cropped slabs written, A*nz*ny*nx*8; achieved = those bytes over the
      two kernels' summed time; also their FP32 rate (5 N log2 N flops per
      transform, 6 per propagator multiply) against the nominal FP32 peak.
    roofline_rotate: stage (c), slab read + volume traffic over the
      resampling time.
    whole: every stage's algorithmic bytes over the pipelined step time."""
    g = rec.padding_geometry
    lNy, lNx = g["lNy"], g["lNx"]
    _A, ny, nx = rec.shape
    nz = nx
    U = float(A) * nz * ny * nx
    col, row = stages["columns_propagate"], stages["rows_inverse"]
    b_bytes = float(A) * lNy * lNx * 8 + U * 8
    b_ms = col["ms"] + row["ms"]
    b_launches = col["launches"] + row["launches"]
    planes = A * nz
    tc = profile_traffic("columns_propagate", planes)
    tr = profile_traffic("rows_inverse", planes)
    b_traffic = (tc + tr) if tc is not None and tr is not None else None
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    fl = stage_flops(rec, A)
    fp32 = {k: {"tflops": fl[k] / (stages[k]["ms"] / 1e3) / 1e12,
                "frac": fl[k] / (stages[k]["ms"] / 1e3) / 1e12 / fp32_peak,
                "algorithmic_gflop": fl[k] / 1e9}
            for k in fl if stages.get(k, {}).get("ms")}
    b_flops = sum(fl.values())
    achieved = b_bytes / (b_ms / 1e3) / 1e9
    roofline = {
        "bound": "hbm", "kernel": "stage (b): k_columns_propagate + "
        "k_rows_inverse (propagator, inverse 2D FFT, crop)",
        "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": achieved / peak, "peak_source": peak_source,
        "traffic": b_traffic,
        "traffic_note": "DRAM bytes of both kernels per reconstruction, "
                        "scaled by planes from one ncu capture each "
                        "(profiles/dram_traffic.md); includes the chunk "
                        "buffer between them",
        "algorithmic_bytes": b_bytes, "ms": b_ms, "launches": b_launches,
        "fp32": {"tflops": b_flops / (b_ms / 1e3) / 1e12,
                 "frac": b_flops / (b_ms / 1e3) / 1e12 / fp32_peak,
                 "algorithmic_gflop": b_flops / 1e9,
                 "peak_tflops": fp32_peak,
                 "peak_source": "nominal at %.0f MHz" % sm_mhz}}
    rs = stages["rotate"]
    rot_achieved = rs["bytes"] / (rs["ms"] / 1e3) / 1e9
    rot_key = "rotate" if w["axis"] is None else "rotate_tilted"
    roofline_rotate = {"bound": "hbm", "kernel": "stage (c): resampling and "
                       "accumulation", "achieved": rot_achieved,
                       "peak": peak, "unit": "GB/s",
                       "frac": rot_achieved / peak,
                       "peak_source": peak_source,
                       "traffic": profile_traffic(rot_key, U),
                       "algorithmic_bytes": rs["bytes"], "ms": rs["ms"],
                       "launches": rs["launches"],
                       "algorithmic_bytes_per_launch":
                           rs["bytes"] / rs["launches"],
                       "launch_ms": rs["ms"] / rs["launches"]}
    a_bytes = stages["rows_forward"]["bytes"]
    step_bytes = a_bytes + b_bytes + rs["bytes"]
    whole = {"algorithmic_bytes": step_bytes, "ms": ms_per_step,
             "achieved": step_bytes / (ms_per_step / 1e3) / 1e9,
             "peak": peak, "unit": "GB/s",
             "frac": step_bytes / (ms_per_step / 1e3) / 1e9 / peak,
             "note": "stages (a)+(b)+(c) algorithmic bytes over the "
                     "pipelined step time"}
    return roofline, roofline_rotate, fp32, whole


def public_e2e(w, host, angles, U, args, world, dev, barrier):
    """The metric through the public API with host buffers: pinned host
    sinogram in, NumPy volume out, copies inside the timed region."""
    import torch
    import odtbrain_gb300 as odt
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 5))
    kw = dict(lD=w["lD"], padfac=w["padfac"], intp_order=w["intp_order"],
              dtype=np.float32)
    if w["axis"] is None:
        api = odt.backpropagate_3d
    else:
        api = odt.backpropagate_3d_tilted
        kw["tilted_axis"] = w["axis"]
    host_np = host.numpy()
    # the same warm-up as the device timing: the returned volumes live in
    # pinned host blocks of torch's caching allocator, and the first calls
    # allocate the blocks the later ones reuse (a result is still alive
    # while the next call runs)
    for _ in range(max(args.warmup, 3)):
        out = api(host_np, angles, w["res"], w["nm"], **kw)
    e2e_t = []
    barrier()
    for _ in range(e2e_steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = api(host_np, angles, w["res"], w["nm"], **kw)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value, e2e_ms = replica_throughput(U, statistics.mean(e2e_t) * 1e3,
                                           world, dev)
    return {"value": e2e_value, "unit": UNIT,
            "h2d_bytes_per_step": int(host.numel() * host.element_size()),
            "d2h_bytes_per_step": int(out.nbytes),
            "ms_per_step": e2e_ms}


def measure_recon_config(w, args, dev, flush, stream):
    """Device-resident and end-to-end timing of another reconstruction
    workload (one GPU), with its volume kept for the accuracy check."""
    import torch
    from odtbrain_gb300._alg3d import Backprop3D
    sino, angles = make_workload(w)
    A, n = w["A"], w["n"]
    U = updates(A, n)
    host = torch.from_numpy(sino).pin_memory()
    dsino = host.to(dev)
    rec = Backprop3D(tuple(sino.shape), angles, w["res"], w["nm"], lD=w["lD"],
                     tilted_axis=w["axis"], padfac=w["padfac"],
                     intp_order=w["intp_order"], input_dtype="complex64",
                     device=dev)
    vol = torch.empty(rec.volume_shape(), device=dev, dtype=torch.complex64)
    ms, step_ms = _timed(lambda: rec(dsino, out=vol, check=False),
                         args.steps, args.warmup, flush, stream)
    rec.check()
    flush.zero_()
    stages = rec.timed(dsino, out=vol)
    got = vol.cpu().numpy()
    e2e = public_e2e(w, host, angles, U, args, 1, dev, lambda: None)
    out = {"workload": w["name"], "ms_per_step": ms, "value": U / (ms / 1e3),
           "unit": UNIT, "steps": args.steps,
           "stages_ms": {k: round(v["ms"], 3) for k, v in stages.items()},
           "e2e": e2e, "gpu_launches_per_step": rec.launches_per_call,
           "_sino": sino, "_angles": angles, "_volume": got}
    del rec, vol, dsino
    torch.cuda.empty_cache()
    return out


def _timed(fn, steps, warmup, flush, stream):
    """Mean CUDA-event time (ms) of fn over `steps` calls after `warmup`,
    L2 flushed before each call outside the events."""
    import torch
    for _ in range(max(warmup, 1)):
        fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        flush.zero_()
        a, b = (torch.cuda.Event(enable_timing=True),
                torch.cuda.Event(enable_timing=True))
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    return statistics.mean(ms), ms


def _base_line(args, w, value, ms, extra):
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic",
            "config": {"workload": w["name"],
                       "l2": "256 MiB flush before every timed step"}}
    line.update(extra)
    return line


def run_diff(args):
    """Forward + vector-Jacobian product of the y-axis reconstruction (the
    differentiation configuration): one step = forward through the autograd
    wrapper, then backward of a linear loss for the sinogram and the filter
    gain."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    if args.ncu_case:
        measure_diff(args, dev)
        return
    r = measure_diff(args, dev)
    w = WORKLOADS["c4"]
    U = updates(w["A"], w["n"])
    ms = r.pop("ms_per_step")
    line = _base_line(args, w, U / (ms / 1e3), ms, r)
    print(json.dumps(line), flush=True)


def measure_diff(args, dev):
    """The differentiation workload (A=90, 128^2 -> 128^3): forward + VJP
    time, forward time and peak device memory; a dict of results."""
    import torch
    from odtbrain_gb300._alg3d import Backprop3D
    from odtbrain_gb300.autograd import backpropagate_3d_autograd
    from sino_gen import ellipsoid_phantom_sinogram
    w = WORKLOADS["c4"]
    sino, angles = ellipsoid_phantom_sinogram(
        w["n"], w["A"], seed=w["seed"], count_range=w["count_range"],
        semi_range=w["semi_range"])
    A, n = w["A"], w["n"]
    U = updates(A, n)
    rec = Backprop3D(sino.shape, angles, w["res"], w["nm"],
                     input_dtype="complex64", device=dev)
    host = torch.from_numpy(sino.astype(np.complex64)).pin_memory()
    dsino = host.to(dev)
    rng = np.random.default_rng(1)
    gain = torch.tensor(rng.uniform(0.8, 1.2, rec.gain_shape())
                        .astype(np.float32), device=dev)
    cot = torch.tensor((rng.normal(size=rec.volume_shape()) + 1j *
                        rng.normal(size=rec.volume_shape()))
                       .astype(np.complex64), device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    stream = torch.cuda.current_stream(dev)
    grads = {}

    def step(src=None):
        s = (dsino if src is None else src).clone().requires_grad_(True)
        g = gain.clone().requires_grad_(True)
        vol = backpropagate_3d_autograd(s, angles, w["res"], w["nm"], gain=g,
                                        plan=rec)
        loss = torch.vdot(cot.flatten(), vol.flatten()).real
        loss.backward()
        grads["s"], grads["g"] = s.grad, g.grad

    def forward():
        rec.forward_gain(dsino, gain, check=False)

    if args.ncu_case:  # profiling case: two forward + VJP steps
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        print("ncu case done")
        return None

    clocks = ClockSampler(0)
    clocks.start()
    ms, step_ms = _timed(step, args.steps, args.warmup, flush, stream)
    clk = clocks.stop()
    fwd_ms, _ = _timed(forward, args.steps, args.warmup, flush, stream)
    torch.cuda.reset_peak_memory_stats(dev)
    base = torch.cuda.memory_allocated(dev)
    step()
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated(dev)
    # end to end: pinned host sinogram in, sinogram gradient out
    out_host = torch.empty(sino.shape, dtype=torch.complex64).pin_memory()

    def e2e():
        step(host.to(dev, non_blocking=True))
        out_host.copy_(grads["s"], non_blocking=True)
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 5)), 1, flush, stream)
    return {
        "workload": w["name"], "ms_per_step": ms, "value": U / (ms / 1e3),
        "unit": UNIT,
        "step": "forward + VJP (sinogram and gain), slabs recomputed",
        "forward_ms": fwd_ms, "backward_ms": ms - fwd_ms,
        "peak_device_mib": (peak - base) / 2**20,
        "peak_device_mib_incl_inputs": peak / 2**20,
        "clocks": clk, "gpu_launches_forward": rec.launches_per_call,
        "step_ms": step_ms,
        "e2e": {"value": U / (e2e_ms / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(host.numel() * 8),
                "d2h_bytes_per_step": int(host.numel() * 8),
                "ms_per_step": e2e_ms},
        "cpu_baseline": None,
        "accuracy": {"checked_by": "tests/test_gpu_adjoint.py: central "
                     "differences h=1e-3 over 64 directions and autograd "
                     "through the dense FP64 model"}}


def run_learned(args):
    """Learned wedge filter: GPU time of the learned reconstruction against
    the plain one, and the error cut of the shipped network on the 200
    held-out phantoms."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    r = measure_learned(args, dev, n_eval=200)
    w = WORKLOADS["c5"]
    ms = r.pop("ms_per_step")
    line = _base_line(args, w, r["value"], ms, r)
    print(json.dumps(line), flush=True)


def run_mlp(args):
    """The learned-gain network on the wedge configuration's point set
    (40 angles x the filter support of the 256^2 padded grid): inference and
    backward (data part + weight gradients) on the tcgen05 kernels, and the
    same network on the warp-level mma.sync kernels beside it (selected with
    odt_mlp_select_kernels), timed with CUDA events in the same run."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    from odtbrain_gb300 import _native
    from odtbrain_gb300._alg3d import Backprop3D
    from odtbrain_gb300.learned import (WEDGE_CONFIG, load_learned_filter,
                                        wedge_angles)
    c = dict(WEDGE_CONFIG)
    A, n = c["num_angles"], c["n"]
    rec = Backprop3D((A, n, n), wedge_angles(A, c["span"]), c["res"], c["nm"],
                     device=dev)
    lf = load_learned_filter(rec)
    g = lf.gains()
    rng = np.random.default_rng(3)
    dg = torch.tensor((rng.normal(size=tuple(g.shape)) + 1j *
                       rng.normal(size=tuple(g.shape))).astype(np.complex64),
                      device=dev)
    points = int(A * lf.positions.numel())
    L = _native.lib()
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    stream = torch.cuda.current_stream(dev)

    def forward():
        lf.mlp.gains(lf.feat, *rec.gain_shape(), out=g,
                     positions=lf.positions)

    def backward():
        lf.mlp.grads(lf.feat, dg, positions=lf.positions)

    times = {}
    try:
        for family, tc in (("tcgen05", 1), ("mma_sync", 0)):
            _native.check(L.odt_mlp_select_kernels(tc))
            for name, fn in (("forward", forward), ("backward", backward)):
                ms, _ = _timed(fn, args.steps, args.warmup, flush, stream)
                times["%s_%s_ms" % (family, name)] = ms
            lf.mlp.check()
    finally:
        _native.check(L.odt_mlp_select_kernels(1))
    # 2 * (4*64 + 64*64 + 64*64 + 64*2) FLOP per point through the network
    flop = 2.0 * (4 * 64 + 64 * 64 + 64 * 64 + 64 * 2)
    ms = times["tcgen05_forward_ms"]
    w = WORKLOADS["mlp"]
    line = _base_line(args, w, points / (ms / 1e3), ms, {})
    line.update({
        "metric": "learned-gain MLP inference points/s on 1 GB300 "
                  "(tcgen05, BF16 operands, FP32 accumulation)",
        "unit": "points/s", "dtype": "bf16 (fp32 accumulation)",
        "points": points, "tflops_inference": points * flop / (ms / 1e3) / 1e12,
        "kernels": times,
        "gpu_launches": args.steps,  # one inference launch per timed step
        "cpu_baseline": None})
    print(json.dumps(line), flush=True)


def measure_learned(args, dev, n_eval):
    """The learned wedge filter (A=40 over 120 deg, 128^2 -> 128^3): GPU
    time learned vs plain, and mean rel-L2 to the plain dense A=400
    reconstruction over `n_eval` held-out phantoms (seeds 2,000,000 on,
    disjoint from training and validation); a dict of results."""
    import torch
    from odtbrain_gb300._alg3d import Backprop3D
    from odtbrain_gb300.learned import (WEDGE_CONFIG, evaluate,
                                        load_learned_filter, make_pairs,
                                        wedge_angles)
    w = WORKLOADS["c5"]
    c = dict(WEDGE_CONFIG)
    A, n = c["num_angles"], c["n"]
    U = updates(A, n)
    sp = wedge_angles(A, c["span"])
    de = np.linspace(0, 2 * np.pi, c["dense_angles"], endpoint=False)
    rec = Backprop3D((A, n, n), sp, c["res"], c["nm"], device=dev)
    rec_d = Backprop3D((c["dense_angles"], n, n), de, c["res"], c["nm"],
                       device=dev)
    seeds = 2_000_000 + np.arange(n_eval)  # the held-out seed range
    learned_s, plain_s = [], []
    lf = load_learned_filter(rec)
    sinos = None
    for k in range(0, n_eval, 50):  # pairs in batches of 50 phantoms
        sinos, targets = make_pairs(c, seeds[k:k + 50], rec, rec_d, sp, de,
                                    dev)
        l_, p_ = evaluate(lf, sinos, targets)
        learned_s.append(l_ * len(targets))
        plain_s.append(p_ * len(targets))
        del targets
    learned = float(sum(learned_s) / n_eval)
    plain = float(sum(plain_s) / n_eval)
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    stream = torch.cuda.current_stream(dev)
    vol = torch.empty(rec.volume_shape(), dtype=torch.complex64, device=dev)
    s0 = sinos[0]
    gain = lf.gains()
    clocks = ClockSampler(0)
    clocks.start()
    ms_l, step_ms = _timed(lambda: rec.forward_gain(s0, angle_gain=gain,
                                                    out=vol, check=False),
                           args.steps, args.warmup, flush, stream)
    clk = clocks.stop()
    ms_p, _ = _timed(lambda: rec(s0, out=vol, check=False), args.steps,
                     args.warmup, flush, stream)

    def with_inference():
        lf.mlp.gains(lf.feat, *rec.gain_shape(), out=gain,
                     positions=lf.positions)
        rec.forward_gain(s0, angle_gain=gain, out=vol, check=False)
    ms_i, _ = _timed(with_inference, args.steps, args.warmup, flush, stream)
    host = sinos[0].cpu().pin_memory()
    out_host = torch.empty(rec.volume_shape(),
                           dtype=torch.complex64).pin_memory()

    def e2e():
        lf(host.to(dev, non_blocking=True), out=vol)
        out_host.copy_(vol, non_blocking=True)
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 5)), 1, flush, stream)
    return {
        "workload": w["name"], "ms_per_step": ms_l,
        "value": U / (ms_l / 1e3), "unit": UNIT,
        "step": "learned-gain reconstruction, gains cached per angle set",
        "plain_ms": ms_p, "time_ratio_cached": ms_l / ms_p,
        "learned_with_inference_ms": ms_i,
        "time_ratio_with_inference": ms_i / ms_p,
        "eval_phantoms": n_eval, "rel_l2_learned": learned,
        "rel_l2_plain": plain, "reduction": 1.0 - learned / plain,
        "clocks": clk, "gpu_launches": rec.launches_per_call,
        "step_ms": step_ms,
        "e2e": {"value": U / (e2e_ms / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": int(host.numel() * 8),
                "d2h_bytes_per_step": int(out_host.numel() * 8),
                "ms_per_step": e2e_ms},
        "cpu_baseline": None}


def run_rytov(args):
    """sinogram_as_rytov on the headline sinogram's field: one step = one
    conversion of all 200 frames (phase, log-amplitude, per-frame unwrap,
    alignment, composition)."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    import odtbrain_gb300 as odt
    from odtbrain_gb300._prepare_sino import SinogramPrep
    from sino_gen import ellipsoid_phantom_sinogram
    w = WORKLOAD
    ryt, _angles = ellipsoid_phantom_sinogram(
        w["n"], w["A"], seed=w["seed"], count_range=w["count_range"],
        semi_range=w["semi_range"], res=w["res"], nm=w["nm"])
    field = np.exp(ryt).astype(np.complex64)
    samples = field.size
    metric = "sinogram_as_rytov samples/s on 1 GB300 (3D frames, FP32)"
    unit = "sinogram samples/s"
    prep = SinogramPrep(field.shape, "rytov", align=True, single=True,
                        device=dev)
    host = torch.from_numpy(field).pin_memory()
    dfield = host.to(dev)
    out = torch.empty(field.shape, dtype=torch.complex64, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    stream = torch.cuda.current_stream(dev)
    if args.ncu_case:
        for _ in range(2):
            prep(dfield, out=out)
        torch.cuda.synchronize()
        print("ncu case done")
        return
    clocks = ClockSampler(0)
    clocks.start()
    ms, step_ms = _timed(lambda: prep(dfield, out=out, check=False),
                         args.steps, args.warmup, flush, stream)
    clk = clocks.stop()
    prep(dfield, out=out, check=True)
    host_np = host.numpy()  # pinned

    def e2e():
        # the public call: host field in, host Rytov sinogram out
        odt.sinogram_as_rytov(uSin=host_np, align=True)
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 5)), 1, flush, stream)
    # parity on a bounded sample: two frames against the oracle (FP64
    # restatement of the reference, same anchor rule)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import unwrap_oracle
        k = 2
        t0 = time.perf_counter()
        ref = unwrap_oracle.sinogram_as_rytov(field[:k].astype(np.complex128),
                                              align=False,
                                              anchor="first_edge")
        cpu_s = time.perf_counter() - t0
        sub = SinogramPrep((k,) + field.shape[1:], "rytov", align=False,
                           single=True, device=dev)(dfield[:k].contiguous())
        err = float(np.abs(sub.cpu().numpy() - ref).max())
        cpu = {"value": k * field[0].size / cpu_s, "unit": unit, "cores": 1,
               "kind": "port",
               "sample": "%d of %d frames (oracle, FP64, align off)"
                         % (k, field.shape[0]),
               "max_abs_diff_vs_gpu": err}
    algo = samples * 16  # complex64 field in, complex64 Rytov sinogram out
    peak, peak_kind = measured_peaks()
    achieved = algo / (ms / 1e3) / 1e9
    line = {"metric": metric, "value": samples / (ms / 1e3), "unit": unit,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32 (reliabilities fp64)",
            "data": "synthetic",
            "config": {"workload": w["name"],
                       "l2": "256 MiB flush before every timed step"},
            "roofline": {"bound": "hbm", "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None,
                         "note": "whole conversion against 16 B/sample "
                                 "(field in, sinogram out); the spanning-"
                                 "tree rounds re-read their state"},
            "clocks": clk, "gpu_launches": prep.launches_per_call,
            "step_ms": step_ms,
            "e2e": {"value": samples / (e2e_ms / 1e3), "unit": unit,
                    "h2d_bytes_per_step": int(field.nbytes),
                    "d2h_bytes_per_step": int(field.nbytes),
                    "ms_per_step": e2e_ms},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_apple(args):
    """apple.correct on the 256^3 reconstruction of the headline sinogram:
    one step = one correction (iterations until the reference's stopping
    test); the unit counts voxels times iterations."""
    import ctypes
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    from odtbrain_gb300 import _native
    from odtbrain_gb300 import apple as gapple
    from odtbrain_gb300._alg3d import Backprop3D
    w = WORKLOAD
    if args.ncu_case:
        # profiling case: an n^3 volume of smooth blobs (no reconstruction
        # before it; n = --ncu-n, 128 by default), three iterations
        nn = args.ncu_n
        g = torch.arange(nn, device=dev, dtype=torch.float32) - nn / 2
        z, y, x = torch.meshgrid(g, g, g, indexing="ij")
        vol = (torch.exp(-(x * x + y * y + z * z) / 800.0)
               + 0.3 * torch.exp(-((x - 20) ** 2 + y * y + z * z) / 60.0)
               ).to(torch.complex64)
    else:
        sino, angles = make_workload()
        rec = Backprop3D(tuple(sino.shape), angles, w["res"], w["nm"],
                         lD=w["lD"], padfac=w["padfac"],
                         intp_order=w["intp_order"], input_dtype="complex64",
                         device=dev)
        vol = rec(torch.from_numpy(sino).to(dev))
    shape = tuple(vol.shape)
    N = int(np.prod(shape))
    fr = vol.real.contiguous()
    d = gapple._desc(shape, w["res"], w["nm"])
    L = _native.lib()
    nb = ctypes.c_uint64()
    _native.check(L.odt_apple_workspace_size(ctypes.byref(d),
                                             ctypes.byref(nb)))
    ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
    out = torch.empty(shape, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    its = ctypes.c_int32()

    def step():
        _native.check(L.odt_apple_correct(
            ctypes.byref(d), ctypes.c_void_p(fr.data_ptr()), None,
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
            nb.value, ctypes.byref(its), ctypes.c_void_p(stream.cuda_stream)))
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    if args.ncu_case:
        d.max_iter = 3
        step()
        torch.cuda.synchronize()
        print("ncu case done")
        return
    clocks = ClockSampler(0)
    clocks.start()
    ms, step_ms = _timed(step, args.steps, args.warmup, flush, stream)
    clk = clocks.stop()
    iters = its.value
    unit = "voxel-iterations/s"
    value = N * iters / (ms / 1e3)
    # the public call on a pinned host copy of the reconstruction
    host_t = torch.empty(shape, dtype=torch.complex64, pin_memory=True)
    host_t.copy_(vol)
    host = host_t.numpy()

    def e2e():
        gapple.correct(host, w["res"], w["nm"])
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 3)), 1, flush, stream)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import apple_oracle
        k = 2
        t0 = time.perf_counter()
        apple_oracle.correct(host, w["res"], w["nm"], max_iter=k,
                             min_diff=0.0)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": N * k / cpu_s, "unit": unit, "cores": 1,
               "kind": "port",
               "sample": "%d iterations (oracle, NumPy + scipy.fft, setup "
                         "and envelope included)" % k}
    # algorithmic bytes per voxel and iteration: the complex64 volume read
    # and written once, the original spectrum (8 B) and envelope (4 B) read
    algo = 28.0 * N * iters
    peak, peak_kind = measured_peaks()
    achieved = algo / (ms / 1e3) / 1e9
    line = {"metric": "apple.correct voxel-iterations/s on 1 GB300 (FP32 "
                      "FFTs)",
            "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic",
            "config": {"workload": w["name"], "iterations": iters,
                       "l2": "256 MiB flush before every timed step"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": profile_traffic("apple_iteration",
                                                    N * iters),
                         "note": "28 B per voxel-iteration (volume read + "
                                 "write, original spectrum and envelope "
                                 "read); traffic: DRAM bytes of the "
                                 "iterations' launches (ncu, 256^3), "
                                 "71.6 B per voxel-iteration"},
            "clocks": clk, "gpu_launches_per_iteration": 5,
            "step_ms": step_ms,
            "e2e": {"value": N * iters / (e2e_ms / 1e3), "unit": unit,
                    "h2d_bytes_per_step": int(host.nbytes),
                    "d2h_bytes_per_step": int(N * 8), "ms_per_step": e2e_ms},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def _ri_volume(w):
    """Object function of a blob phantom, f = km^2 ((n/nm)^2 - 1) with n in
    [nm, nm + 0.03] and a small absorbing imaginary part (complex128)."""
    n = w["n"]
    rng = np.random.default_rng(w["seed"])
    g = np.arange(n) - n / 2
    z, y, x = np.meshgrid(g, g, g, indexing="ij", sparse=True)
    ri = w["nm"] + 0.03 * np.exp(-(x * x + y * y + z * z) / (0.08 * n * n))
    km = 2 * np.pi * w["nm"] / w["res"]
    f = km * km * ((ri / w["nm"]) ** 2 - 1)
    return f + 1j * rng.normal(0, 1e-3 * km * km, f.shape)


def run_ri(args):
    """odt_to_ri on a 256^3 complex64 volume through the C ABI: one step =
    one conversion of the whole volume (8 B read + 8 B written per voxel,
    the algorithmic bytes)."""
    import ctypes
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    import odtbrain_gb300 as odt
    from odtbrain_gb300 import _native
    w = WORKLOAD
    f = _ri_volume(w).astype(np.complex64)
    N = f.size
    host = torch.from_numpy(f).pin_memory()
    df = host.to(dev)
    out = torch.empty_like(df)
    stream = torch.cuda.current_stream(dev)
    L = _native.lib()

    def conv(name, dst):
        _native.check(getattr(L, name)(
            ctypes.c_void_p(df.data_ptr()), ctypes.c_void_p(dst.data_ptr()),
            N, _native.ODT_DATA_C64, w["res"], w["nm"],
            ctypes.c_void_p(stream.cuda_stream)))
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    if args.ncu_case:
        for _ in range(2):
            conv("odt_odt_to_ri", out)
        torch.cuda.synchronize()
        print("ncu case done")
        return
    clocks = ClockSampler(0)
    clocks.start()
    ms, step_ms = _timed(lambda: conv("odt_odt_to_ri", out), args.steps,
                         args.warmup, flush, stream)
    clk = clocks.stop()
    opt_ms, _ = _timed(lambda: conv("odt_opt_to_ri", out), args.steps, 1,
                       flush, stream)
    conv("odt_odt_to_ri", out)
    got = out.cpu().numpy()
    unit = "voxels/s"

    host_np = host.numpy()  # pinned

    def e2e():
        odt.odt_to_ri(host_np, w["res"], w["nm"])
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 5)), 1, flush, stream)
    cpu = None
    if not args.no_cpu_baseline:
        from oracle import odt_oracle
        f64 = f.astype(np.complex128)
        t0 = time.perf_counter()
        ref = odt_oracle.odt_to_ri(f64, w["res"], w["nm"])
        cpu_s = time.perf_counter() - t0
        cpu = {"value": N / cpu_s, "unit": unit, "cores": 1, "kind": "port",
               "sample": "the whole %d^3 volume (oracle, NumPy FP64)" % w["n"],
               "max_abs_rel_diff_vs_gpu":
                   float(np.abs(got - ref).max() / np.abs(ref).max())}
    algo = 16.0 * N
    peak, peak_kind = measured_peaks()
    achieved = algo / (ms / 1e3) / 1e9
    line = {"metric": "odt_to_ri voxels/s on 1 GB300 (complex64)",
            "value": N / (ms / 1e3), "unit": unit, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (complex64)", "data": "synthetic",
            "config": {"workload": w["name"],
                       "l2": "256 MiB flush before every timed step"},
            "roofline": {"bound": "hbm", "kernel": "k_odt_to_ri_complex",
                         "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": profile_traffic("odt_to_ri", N),
                         "algorithmic_bytes_per_launch": algo,
                         "launch_ms": ms},
            "opt_to_ri": {"ms": opt_ms,
                          "GB_per_s": algo / (opt_ms / 1e3) / 1e9},
            "clocks": clk, "gpu_launches": 1, "step_ms": step_ms,
            "e2e": {"value": N / (e2e_ms / 1e3), "unit": unit,
                    "h2d_bytes_per_step": int(f.nbytes),
                    "d2h_bytes_per_step": int(f.nbytes),
                    "ms_per_step": e2e_ms},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def _bpp2d_workload(w):
    from sino_gen import ellipsoid_phantom_sinogram
    sino, angles = ellipsoid_phantom_sinogram(
        w["n"], w["A"], seed=w["seed"], count_range=w["count_range"],
        semi_range=w["semi_range"], res=w["res"], nm=w["nm"], ny=1)
    return sino[:, 0, :].astype(np.complex64), angles


def run_bpp2d(args):
    """backpropagate_2d: one step = one 512^2 reconstruction from 400
    angles; the unit counts pixels times angles."""
    import torch
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    from odtbrain_gb300 import build as native_build
    native_build.build()
    import odtbrain_gb300 as odt
    from odtbrain_gb300._alg2d import Backprop2D
    w = WORKLOAD
    sino, angles = _bpp2d_workload(w)
    A, n = sino.shape
    U = float(A) * n * n
    unit = "pixel-angle updates/s"
    rec = Backprop2D(sino.shape, angles, w["res"], w["nm"], lD=w["lD"],
                     device=dev)
    host = torch.from_numpy(sino).pin_memory()
    ds = host.to(dev)
    out = torch.empty((n, n), dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(L2_FLUSH_BYTES, device=dev, dtype=torch.uint8)
    if args.ncu_case:
        for _ in range(2):
            rec(ds, out=out)
        torch.cuda.synchronize()
        print("ncu case done")
        return
    clocks = ClockSampler(0)
    clocks.start()
    ms, step_ms = _timed(lambda: rec(ds, out=out, check=False), args.steps,
                         args.warmup, flush, stream)
    clk = clocks.stop()
    rec(ds, out=out, check=True)
    flush.zero_()
    stages = rec.timed(ds, out=out)
    stage_summary = {k: {"ms": round(v["ms"], 3), "launches": v["launches"],
                         "GB_per_s": (v["bytes"] / (v["ms"] / 1e3) / 1e9
                                      if v["ms"] > 0 else None)}
                     for k, v in stages.items()}
    dom = max(stages, key=lambda k: stages[k]["ms"])
    ds_ = stages[dom]
    peak, peak_kind = measured_peaks()
    achieved = ds_["bytes"] / (ds_["ms"] / 1e3) / 1e9
    # DRAM bytes of the dominant launch from the committed ncu summary,
    # scaled by its units (planes for the fused row stage, updates for the
    # resampling)
    nl = max(1, ds_["launches"])
    traffic = {"rows_inverse": lambda: profile_traffic("rows_line_2d",
                                                       A * n / nl),
               "rotate": lambda: profile_traffic("rotate_plane", U / nl)
               }.get(dom, lambda: None)()

    host_np = host.numpy()  # pinned

    def e2e():
        odt.backpropagate_2d(host_np, angles, w["res"], w["nm"], lD=w["lD"])
    e2e_ms, _ = _timed(e2e, max(3, min(args.steps, 5)), 1, flush, stream)
    cpu = None
    if not args.no_cpu_baseline:
        # parity and CPU time on a bounded sample: 8 of the angles as an
        # 8-angle problem
        from oracle import odt_oracle
        k = 8
        idx = np.arange(0, A, A // k)[:k]
        sub = sino[idx].astype(np.complex128)
        t0 = time.perf_counter()
        ref = odt_oracle.backpropagate_2d(sub, angles[idx], w["res"],
                                          w["nm"], lD=w["lD"])
        cpu_s = time.perf_counter() - t0
        got = Backprop2D(sub.shape, angles[idx], w["res"], w["nm"],
                         lD=w["lD"], device=dev)(
                             torch.from_numpy(sub.astype(np.complex64))
                             .to(dev)).cpu().numpy()
        cpu = {"value": k * n * n / cpu_s, "unit": unit, "cores": 1,
               "kind": "port",
               "sample": "%d of the %d angles as a %d-angle problem "
                         "(oracle, NumPy/scipy FP64)" % (k, A, k),
               "rel_l2_vs_gpu": float(np.linalg.norm(got - ref)
                                      / np.linalg.norm(ref))}
    line = {"metric": "backpropagate_2d pixel-angle updates/s on 1 GB300 "
                      "(FP32)",
            "value": U / (ms / 1e3), "unit": unit, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 (complex64)", "data": "synthetic",
            "config": {"workload": w["name"], "A": A, "n": n,
                       "padded_fft": rec.padding_geometry["lN"],
                       "l2": "256 MiB flush before every timed step"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved,
                         "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "algorithmic_bytes_per_launch":
                             ds_["bytes"] / max(1, ds_["launches"]),
                         "launch_ms": ds_["ms"] / max(1, ds_["launches"])},
            "stages": stage_summary,
            "clocks": clk, "gpu_launches": rec.launches_per_call,
            "step_ms": step_ms,
            "e2e": {"value": U / (e2e_ms / 1e3), "unit": unit,
                    "h2d_bytes_per_step": int(sino.nbytes),
                    "d2h_bytes_per_step": int(n * n * 8),
                    "ms_per_step": e2e_ms},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def run_reference_ri(args):
    """--impl reference for odt_to_ri: the oracle port of the reference
    (NumPy FP64, as the reference computes) on the whole volume per step."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import odt_oracle
    w = WORKLOAD
    f = _ri_volume(w)
    times = []
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        odt_oracle.odt_to_ri(f, w["res"], w["nm"])
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    step = statistics.mean(times)
    print(json.dumps(_reference_line(
        args, "odt_to_ri voxels/s on 1 GB300 (complex64)", "voxels/s",
        f.size / step, step, w["name"],
        "the whole %d^3 volume per step (oracle port of the reference, "
        "NumPy FP64)" % w["n"], 1)), flush=True)


def run_reference_bpp2d(args):
    """--impl reference for backpropagate_2d: the oracle port of the
    reference (NumPy FFTs + scipy.ndimage.rotate, FP64) on a bounded
    sample of 4 angles per step."""
    if int(os.environ.get("RANK", "0")) != 0:
        return
    from oracle import odt_oracle
    w = WORKLOAD
    sino, angles = _bpp2d_workload(w)
    A, n = sino.shape
    s = sino.astype(np.complex128)
    k = 4
    times = []
    for it in range(args.warmup + args.steps):
        a0 = (it * k) % (A - k)
        t0 = time.perf_counter()
        odt_oracle.backpropagate_2d(s[a0:a0 + k], angles[a0:a0 + k],
                                    w["res"], w["nm"], lD=w["lD"])
        if it >= args.warmup:
            times.append(time.perf_counter() - t0)
    step = statistics.mean(times)
    print(json.dumps(_reference_line(
        args, "backpropagate_2d pixel-angle updates/s on 1 GB300 (FP32)",
        "pixel-angle updates/s", k * n * n / step, step, w["name"],
        "4 of the 400 angles per step as a 4-angle problem (oracle port of "
        "the reference: NumPy FFTs, scipy.ndimage.rotate), FP64", 1)),
        flush=True)


def run_ncu_case(rotate_case=False):
    """Small case for ncu captures: the workload's plane and volume sizes
    with 8 angles and the save_memory workspace, or (``rotate_case``) 16
    angles in one batch, so that one resampling launch covers 16 angles as
    in the full run."""
    import torch
    from odtbrain_gb300 import build as native_build
    native_build.build()
    from odtbrain_gb300._alg3d import Backprop3D
    w = WORKLOAD
    sino, angles = make_workload()
    k = 16 if rotate_case else 8
    sino, angles = sino[:k].copy(), angles[:k].copy()
    dev = torch.device("cuda", 0)
    rec = Backprop3D(tuple(sino.shape), angles, w["res"], w["nm"],
                     lD=w["lD"], tilted_axis=w["axis"], padfac=w["padfac"],
                     intp_order=w["intp_order"],
                     save_memory=not rotate_case,
                     input_dtype="complex64", device=dev)
    d = torch.from_numpy(sino).to(dev)
    for _ in range(2):
        vol = rec(d)
    torch.cuda.synchronize()
    print("ncu case done: %d launches per execution, volume %s" %
          (rec.launches_per_call, tuple(vol.shape)))


def main():
    global WORKLOAD, WORKLOAD_NAME
    args = parse_args()
    WORKLOAD = WORKLOADS[args.config]
    WORKLOAD_NAME = WORKLOAD["name"]
    if args.config == "apple":
        if args.impl == "reference":
            run_reference_apple(args)
        else:
            run_apple(args)
    elif args.config == "rytov":
        if args.impl == "reference":
            run_reference_rytov(args)
        else:
            run_rytov(args)
    elif args.config == "ri":
        if args.impl == "reference":
            run_reference_ri(args)
        else:
            run_ri(args)
    elif args.config == "bpp2d":
        if args.impl == "reference":
            run_reference_bpp2d(args)
        else:
            run_bpp2d(args)
    elif args.config == "mlp":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "no counterpart in the reference (it has a "
                              "fixed filter)"}))
        else:
            run_mlp(args)
    elif args.config in ("c4", "c5"):
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable":
                              "no counterpart in the reference (it has no "
                              "derivatives and a fixed filter)"}))
        elif args.config == "c4":
            run_diff(args)
        else:
            run_learned(args)
    elif args.ncu_case or args.ncu_rotate_case:
        run_ncu_case(rotate_case=args.ncu_rotate_case)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
