"""Benchmark: fwd+adj NUFFT throughput at 128^3 (8 coils) on one GB300.

Workload (the single-GPU configuration the headline metric is quoted on):
N = 128^3 image, u = 2 (K = 256^3), Kaiser-Bessel J = 6 radial kernel,
3-D golden-angle koosh ball with 256 samples/spoke x 32768 spokes
(M = 8,388,608 samples), 8 coils (modified Shepp-Logan phantom with phase
times Gaussian coil maps), complex64.

One step = fNUFT of all coils + aNUFT of all coils.
  value   -- M*nc/t in Msample/s, inputs resident in HBM, device pointers
             through the C ABI (nufft3d_forward / nufft3d_adjoint);
  e2e     -- the same through the host-pointer entry points
             (nufft3d_forward_host / nufft3d_adjoint_host) from pinned host
             memory, every copy inside the timed region; four host threads
             each run whole steps on their own handle of the plan, the
             handles moving the buffers with copy-engine transfers, so the
             calls' host-link transfers overlap the other calls' compute.
The grid (1.07 GB) and the samples (0.54 GB) are far larger than L2, so no
flush is needed between steps.

--impl reference times the CPU restatement of the reference's sparse path
(oracle/, FP64, all host threads): each step is fNUFT + aNUFT of one of the
8 coils over the full trajectory, measured, not extrapolated.  The
cpu_baseline leg of the GPU run times two such steps and, being the one place
this script runs the oracle, also compares the GPU results of the timed
workload with FP64 per coil ("accuracy").
Multi-GPU: replicas only (one independent workload per rank, no collective on
the data path; value = all ranks' samples / max time).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+adj NUFFT Msample/s at 128^3"
E2E_THREADS = 4      # concurrent host-pointer callers in the e2e leg, one handle each
E2E_HOST_COPY = 1    # how the host-pointer calls move pinned buffers (nufft3d_plan_set_host_copy):
                     # copy engines (measured 7869 Msample/s with 4 threads at 128^3 x 8, against
                     # 6228 with 2 threads and kernels reading the buffers in place)
E2E_FREE_SMS = {0: 16, 1: 0}  # multiprocessors the handles' interpolation kernels leave free, per mode
WORKLOAD = "koosh ball 256x32768 (M=8388608) at N=128^3, u=2 (K=256^3), J=6 radial KB, 8 coils, complex64"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        rows = []
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[3:7]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def stage_bytes(obj, nc):
    """Algorithmic bytes per launch of each stage (reads + writes of its
    inputs/outputs).  Interpolation stages count the grid, the samples and
    12 bytes of coordinates per sample (per coil 8 K^3 + 8 M + 12 M/nc);
    the stored H and H' that the 8-coil gather and spread read instead of
    evaluating weights are reported beside them (`stored_h_bytes`,
    `stored_h_t_bytes`), not counted."""
    N1, N2, N3 = (int(v) for v in obj.N)
    K1, K2, K3 = (int(v) for v in obj.K)
    M, nnz = obj.M, obj.nnz
    c = 8 * nc
    img, u = N1 * N2 * N3, N1 * N2 * N3 * 4
    b1, b2, g = K1 * N2 * N3, K1 * K2 * N3, K1 * K2 * K3
    coords = nnz * 12
    return {
        "fft_x_fwd": img * c + u + b1 * c,
        "fft_y_fwd": b1 * c + b2 * c,
        "fft_z_fwd": b2 * c + g * c,
        "gather": g * c + coords + nnz * c,
        "permute_out": nnz * c + M * 4 + M * c,
        "permute_in": M * c + M * 4 + nnz * c,
        "grid_zero": g * c,
        "spread": nnz * c + coords + g * c,
        "fft_z_adj": g * c + b2 * c,
        "fft_y_adj": b2 * c + b1 * c,
        "fft_x_adj": b1 * c + u + img * c,
    }


def ncu_figures():
    p = os.path.join(ROOT, "profiles", "interp_traffic_N128.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f)


def ncu_traffic(kernel):
    """DRAM bytes per launch of `kernel` at this workload from the committed ncu summary."""
    return ncu_figures().get(kernel)


def ncu_sm_side(kernel):
    """Issue and shared-memory utilisation of `kernel` from the committed ncu summary."""
    return ncu_figures().get("sm_side", {}).get(kernel)


def dist_init(backend="nccl"):
    """One process per GPU under torchrun (RANK/LOCAL_RANK/WORLD_SIZE/MASTER_*);
    replicas: ranks share nothing but the barrier and the max-over-ranks time."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    if backend == "nccl":
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local


def max_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, seconds, ws):
    """Whole-job rate of independent replicas: all ranks' units over the slowest
    rank's time (weak scaling: per-rank work fixed)."""
    t = max_over_ranks(seconds, ws)
    return units_per_rank * ws / t, t


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def build_inputs(N, n_read, n_spokes, nc):
    from nufft_3d_gb300 import synth
    om = synth.koosh_ball(N, n_read, n_spokes)
    im = synth.phantom_with_phase(N)[..., None] * synth.coil_maps(N, nc)
    return om, im.astype(np.complex64)


def rotated(om, seed):
    """The same trajectory shape under a seeded random rotation (a new trajectory)."""
    rng = np.random.default_rng(seed)
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                  [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                  [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])
    return R @ om


def uneven_volumes(n_vol=48, seed=3):
    """Batched uneven sizes: N in {64, 96, 128, 160}, radial / stack-of-spirals /
    uniform-random trajectories (0.5-1.5 N^3 samples), 4-16 coils each."""
    from nufft_3d_gb300 import synth
    rng = np.random.default_rng(seed)
    vols = []
    for v in range(n_vol):
        N = int(rng.choice([64, 96, 128, 160]))
        kind = ["radial", "spiral", "random"][v % 3]
        nc = int(rng.integers(4, 17))
        count = int(rng.uniform(0.5, 1.5) * N ** 3)
        if kind == "radial":
            om = rotated(synth.koosh_ball(N, N, max(1, count // N)), seed + v)
        elif kind == "spiral":
            parts = min(64, N)
            om = synth.stack_of_spirals(N, n_interleaves=16, n_samples=max(64, count // (16 * parts)),
                                        n_partitions=parts)
        else:
            om = synth.random_uniform(N, count, seed=seed + v)
        vols.append((om, N, nc, kind))
    return vols


def bench_batched(maxit=20, damp=1e-3):
    """48 uneven volumes reconstructed by the batched CG (one launch per
    stage for all volumes) against the same volumes one after another."""
    import torch
    from nufft_3d_gb300 import NufftBatch, nufft_3d
    vols = uneven_volumes()
    # the batched kernels read each volume's stored H but not its H' (the
    # batched spread evaluates the kernel): plans made for a batch skip H'
    objs = [nufft_3d(om, N, "J", 6, density_iters=20, spread_table=0) for om, N, _, _ in vols]
    ncs = [nc for _, _, nc, _ in vols]
    g = torch.Generator(device="cuda").manual_seed(0)
    raws = [torch.randn((nc, o.M), dtype=torch.complex64, device="cuda", generator=g) for o, nc in zip(objs, ncs)]
    batch = NufftBatch(objs, ncs)
    batch.inverse(raws, 2, damp)            # warm-up (graph, buffers)
    for o, r in zip(objs, raws):
        o.iNUFT(r, 2, damp, solver="cg", tol=0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xb = batch.inverse(raws, maxit, damp)
    torch.cuda.synchronize()
    t_b = time.perf_counter() - t0
    t0 = time.perf_counter()
    xs = [o.iNUFT(r, maxit, damp, solver="cg", tol=0) for o, r in zip(objs, raws)]
    torch.cuda.synchronize()
    t_s = time.perf_counter() - t0
    err = max(float((a - b).abs().norm() / b.abs().norm()) for a, b in zip(xb, xs))
    samples = sum(o.M * nc for o, nc in zip(objs, ncs))
    batch.close()
    for o in objs:
        o.close()
    return {"workload": "48 uneven volumes, N in {64,96,128,160}, radial/spiral/random, 4-16 coils, "
                        "%d CG iterations, damp %g" % (maxit, damp),
            "coil_samples": samples, "batched_volumes_per_s": round(len(vols) / t_b, 3),
            "sequential_volumes_per_s": round(len(vols) / t_s, 3), "speedup": round(t_s / t_b, 3),
            "batched_s": round(t_b, 3), "sequential_s": round(t_s, 3),
            "max_rel_l2_batched_vs_single": err}


def bench_large_cg(maxit=50, damp=1e-3):
    """Large CG: N=192^3 (K=384^3), koosh ball 384 x 60000 (M = 23,040,000), 16
    coils, density from the plan (20 iterations), 50 CG iterations with FP64
    scalars, one CUDA graph per iteration.  Check at this size: coils are
    independent systems, so coils 0-1 solved alone equal the same coils of the
    16-coil solve (rel L2 after 5 iterations)."""
    import torch
    from nufft_3d_gb300 import nufft_3d, synth
    N, nr, ns, nc = 192, 384, 60000, 16
    om = synth.koosh_ball(N, nr, ns)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    obj = nufft_3d(om, N, "J", 6, "u", 2)
    torch.cuda.synchronize()
    t_plan = time.perf_counter() - t0
    g = torch.Generator(device="cuda").manual_seed(4)
    raw = torch.randn((nc, obj.M), dtype=torch.complex64, device="cuda", generator=g)
    obj.iNUFT(raw[:2], 1, damp, solver="cg", tol=0)       # warm-up: buffers, graph
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    im, its = obj.iNUFT(raw, maxit, damp, solver="cg", tol=0, return_iters=True)
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t0
    # coil independence after 5 iterations (over 50 the CG iterates of an
    # ill-conditioned system amplify rounding differences: the spread's
    # fixed-point scale is chosen per block from the coils in the pass)
    im5 = obj.iNUFT(raw, 5, damp, solver="cg", tol=0)
    im2 = obj.iNUFT(raw[:2].contiguous(), 5, damp, solver="cg", tol=0)
    err = float((im5[:2] - im2).abs().norm() / im2.abs().norm())
    out = {"workload": "large CG: N=192^3 (K=384^3), koosh 384x60000 (M=23040000), 16 coils, density 20 it, "
                       "%d CG iterations, FP64 scalars, one graph per iteration" % maxit,
           "plan_s": round(t_plan, 3), "solve_s": round(t_solve, 3), "iterations": int(max(its)),
           "ms_per_iteration": round(1e3 * t_solve / maxit, 2),
           "msample_per_s_fwd_adj": round(obj.M * nc * maxit / t_solve / 1e6, 1),
           "rel_l2_coils01_alone_vs_in_16_after_5_it": err}
    obj.close()
    del im, im2, im5, raw
    torch.cuda.empty_cache()
    return out


SERVING_MIX = [(64, 64, 2048, 4), (96, 96, 4096, 6), (128, 128, 8192, 8), (64, 64, 4096, 8)]
SERVING_128x8 = [(128, 128, 8192, 8)]


def serving_requests(n_req=40, rate=20.0, seed=5, shapes=SERVING_MIX):
    """Serving stream: Poisson arrivals at `rate` per second (rate None: all
    at t=0, a backlog that measures capacity); 60% reuse one of 8 resident
    trajectories, 40% new ones; koosh balls (N, samples/spoke, spokes, coils)
    drawn from `shapes`; 20 CG iterations each."""
    from nufft_3d_gb300 import synth
    from nufft_3d_gb300.serving import Request
    rng = np.random.default_rng(seed)
    resident = []
    for i in range(8):
        N, nr, ns, nc = shapes[i % len(shapes)]
        resident.append((rotated(synth.koosh_ball(N, nr, ns), 100 + i), N, nc))
    reqs = []
    t = 0.0
    for i in range(n_req):
        t += rng.exponential(1.0 / rate) if rate else 0.0
        if rng.random() < 0.6:
            om, N, nc = resident[int(rng.integers(0, 8))]
        else:
            N, nr, ns, nc = shapes[int(rng.integers(0, len(shapes)))]
            om = rotated(synth.koosh_ball(N, nr, ns), 1000 + i)
        raw = (rng.standard_normal((om.shape[1], nc)) + 1j * rng.standard_normal((om.shape[1], nc))).astype(np.complex64)
        reqs.append(Request(om=om, N=N, raw=raw, maxit=20, damp=1e-3, arrival=t))
    return reqs


def serve_pair(reqs, slots):
    """The same requests through the server and through the plain path."""
    from nufft_3d_gb300.serving import Request, run_plain, run_served, summarize
    copy = [Request(om=r.om, N=r.N, raw=r.raw, maxit=r.maxit, damp=r.damp, arrival=r.arrival, key=r.key)
            for r in reqs]
    served, wall_s = run_served(reqs, slots=slots)
    plain, wall_p = run_plain(copy)
    err = max(float(np.linalg.norm(a.result - b.result) / np.linalg.norm(b.result))
              for a, b in zip(sorted(served, key=lambda r: r.arrival), sorted(plain, key=lambda r: r.arrival)))
    s = summarize(served, wall_s)
    p = summarize(plain, wall_p)
    return {"served": s, "plain": p, "throughput_speedup": round(s["volumes_per_s"] / p["volumes_per_s"], 3),
            "p50_speedup": round(p["p50_ms"] / s["p50_ms"], 3), "max_rel_l2_served_vs_plain": err}


def bench_serving(slots=4):
    """Latency runs (Poisson 20 req/s: throughput there is the offered load)
    and capacity runs (all requests queued at t=0), for the mixed shapes and
    for 128^3 x 8-coil requests."""
    out = {"slots": slots, "iterations": 20,
           "mixed_shapes": "N in {64,96,128}, 4-8 coils, koosh balls of 131K-1M samples",
           "shapes_128x8": "N=128, 8 coils, koosh 128 x 8192 (M = 1,048,576)"}
    out["mixed_latency"] = dict(serve_pair(serving_requests(40, 20.0, 5, SERVING_MIX), slots),
                                arrivals="Poisson 20 req/s, 40 requests")
    out["mixed_capacity"] = dict(serve_pair(serving_requests(40, None, 5, SERVING_MIX), slots),
                                 arrivals="40 requests queued at t=0")
    out["128x8_latency"] = dict(serve_pair(serving_requests(24, 20.0, 6, SERVING_128x8), slots),
                                arrivals="Poisson 20 req/s, 24 requests")
    out["128x8_capacity"] = dict(serve_pair(serving_requests(24, None, 6, SERVING_128x8), slots),
                                 arrivals="24 requests queued at t=0")
    return out


def bench_cufft(N, K, nc, ours, reps=10):
    """Comparator only: cuFFT (through torch.fft) on the same transform sizes
    -- zero-pad the nc x N^3 image into nc x K^3 and run a 3-D FFT (forward),
    inverse 3-D FFT and crop (adjoint) -- beside this library's pruned pass
    chains (x, y, z passes with pad/crop, shift and deapodization fused)."""
    import torch
    pad = (K - N) // 2
    x = torch.randn((nc, N, N, N), dtype=torch.complex64, device="cuda")
    g = torch.zeros((nc, K, K, K), dtype=torch.complex64, device="cuda")
    g2 = torch.empty_like(g)
    xo = torch.empty_like(x)

    def fwd():
        g.zero_()
        g[:, pad:pad + N, pad:pad + N, pad:pad + N] = x
        torch.fft.fftn(g, dim=(1, 2, 3), out=g2)

    def adj():
        torch.fft.ifftn(g2, dim=(1, 2, 3), out=g)
        xo.copy_(g[:, pad:pad + N, pad:pad + N, pad:pad + N])

    out = {}
    for name, fn in (("fwd", fwd), ("adj", adj)):
        for _ in range(3):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out["cufft_%s_ms" % name] = round(e0.elapsed_time(e1) / reps, 4)
    del x, g, g2, xo
    torch.cuda.empty_cache()
    out.update({"ours_fwd_ms": round(ours["fwd"], 4), "ours_adj_ms": round(ours["adj"], 4),
                "what": "cuFFT via torch.fft: pad + fftn over nc x K^3 (fwd), ifftn + crop (adj); ours: "
                        "pruned x/y/z pass chains with pad/crop, shift and deap fused (stage times of the "
                        "timed steps); comparator only"})
    return out


def cpu_baseline(om, N, im, k_gpu, a_gpu, steps=2):
    """The oracle timed on two one-coil steps of the workload, and the GPU
    results (k_gpu = fNUFT(im), a_gpu = aNUFT(k_gpu)) against it per coil."""
    from oracle import cpu_bench
    r, ref, _ = cpu_bench.run(om, N, steps)
    acc = cpu_bench.accuracy(ref, im, k_gpu, a_gpu)
    return r, acc


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    om, _ = build_inputs(args.N, args.n_read, args.n_spokes, args.nc)
    from oracle import cpu_bench
    ref = cpu_bench.make_ref(om, args.N)
    cpu_bench.time_steps(ref, args.warmup)
    t0 = time.perf_counter()
    cpu_bench.time_steps(ref, args.steps)
    t = time.perf_counter() - t0
    v = ref.M * args.steps / t / 1e6      # coil-samples processed / time
    sample = cpu_bench.sample_text(ref)
    line = {"metric": METRIC, "value": v, "unit": "Msample/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "step": "1 of the 8 coils, full trajectory",
                       "l2": "inputs larger than L2"},
            "cpu_baseline": {"value": v, "unit": "Msample/s", "cores": cpu_bench.cores(), "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "Msample/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--N", type=int, default=128)
    ap.add_argument("--n-read", dest="n_read", type=int, default=256)
    ap.add_argument("--n-spokes", dest="n_spokes", type=int, default=32768)
    ap.add_argument("--nc", type=int, default=8)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched, serving and large-CG runs")
    ap.add_argument("--tile", type=str, default=None)
    ap.add_argument("--coils-per-pass", type=int, default=0)
    ap.add_argument("--samples-per-block", type=int, default=0)
    ap.add_argument("--no-tune", action="store_true", help="skip the plan-time autotuner")
    ap.add_argument("--tap-table", dest="tap_table", type=int, default=-1, choices=[-1, 0, 1],
                    help="stored H: -1 auto (library default), 0 evaluate taps on the fly, 1 always")
    ap.add_argument("--host-copy", dest="host_copy", type=int, default=None, choices=[0, 1],
                    help="e2e leg: 0 kernels use the pinned buffers in place, 1 copy-engine transfers")
    ap.add_argument("--e2e-threads", dest="e2e_threads", type=int, default=None,
                    help="e2e leg: host threads, each on its own handle")
    ap.add_argument("--e2e-free-sms", dest="e2e_free_sms", type=int, default=None,
                    help="e2e leg: multiprocessors the handles' interpolation kernels leave free")
    ap.add_argument("--spread-table", dest="spread_table", type=int, default=-1, choices=[-1, 0, 1],
                    help="stored H' for the 8-coil spread: -1 auto (library default), 0 on the fly, 1 always")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    from nufft_3d_gb300 import _lib, nufft_3d

    rank, ws, local = dist_init()
    torch.cuda.set_device(local)
    om, im = build_inputs(args.N, args.n_read, args.n_spokes, args.nc)
    tile = tuple(int(t) for t in args.tile.split(",")) if args.tile else None
    obj = nufft_3d(om, args.N, "J", 6, "u", 2, device=local, tile=tile, coils_per_pass=args.coils_per_pass,
                   samples_per_block=args.samples_per_block, tap_table=args.tap_table,
                   spread_table=args.spread_table)
    L, plan = obj._L, obj.plan
    nc, M = args.nc, obj.M
    # the plan-time autotuner picks the piece size and coils per pass
    tune = None
    if not args.no_tune and not (args.coils_per_pass or args.samples_per_block):
        tune = obj.tune(nc)
    x = torch.from_numpy(np.ascontiguousarray(im.transpose(3, 2, 1, 0))).cuda()
    k = torch.empty((nc, M), dtype=torch.complex64, device="cuda")
    x2 = torch.empty_like(x)
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        _lib.check(L.nufft3d_forward(plan, x.data_ptr(), k.data_ptr(), nc, sp))
        _lib.check(L.nufft3d_adjoint(plan, k.data_ptr(), x2.data_ptr(), nc, sp))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    _lib.check(L.nufft3d_profile(plan, 1))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    buf = ctypes.create_string_buffer(8192)
    _lib.check(L.nufft3d_profile_read(plan, buf, 8192))
    _lib.check(L.nufft3d_profile(plan, 0))
    prof = json.loads(buf.value.decode())
    barrier(ws)
    rate, t_max = replica_throughput(M * nc * args.steps, ms / 1e3, ws)
    ms_max = t_max * 1e3
    value = rate / 1e6

    # e2e: host-pointer entry points, pinned host buffers, copies inside the
    # timed region.  Two host threads, each with its own handle on the
    # trajectory (nufft3d_plan_share: own work buffers and stream), run whole
    # steps concurrently, so one call's host-link transfers overlap the other
    # call's compute: either kernels reading and writing the pinned buffers in
    # place (host copy mode 0; the handles' persistent interpolation kernels
    # then leave some multiprocessors free for them, nufft3d_plan_set_sms) or
    # copy-engine transfers through device staging buffers (mode 1).
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    host_copy = E2E_HOST_COPY if args.host_copy is None else args.host_copy
    free_sms = E2E_FREE_SMS[host_copy] if args.e2e_free_sms is None else args.e2e_free_sms
    nthreads = E2E_THREADS if args.e2e_threads is None else args.e2e_threads
    hs = [obj.share() for _ in range(nthreads)]
    hbufs = []
    for h in hs:
        _lib.check(L.nufft3d_plan_set_sms(h.plan, max(1, nsm - free_sms)))
        _lib.check(L.nufft3d_plan_set_host_copy(h.plan, host_copy))
        xh = torch.from_numpy(np.ascontiguousarray(im.transpose(3, 2, 1, 0))).pin_memory()
        kh = torch.empty((nc, M), dtype=torch.complex64).pin_memory()
        x2h = torch.empty_like(xh).pin_memory()
        hbufs.append((xh, kh, x2h))

    def step_host(i):
        xh, kh, x2h = hbufs[i]
        _lib.check(L.nufft3d_forward_host(hs[i].plan, xh.data_ptr(), kh.data_ptr(), nc))
        _lib.check(L.nufft3d_adjoint_host(hs[i].plan, kh.data_ptr(), x2h.data_ptr(), nc))

    def host_steps(n):
        errs = []

        def worker(i):
            try:
                for _ in range(n):
                    step_host(i)
            except Exception as e:  # re-raised on the main thread
                errs.append(e)
        th = [threading.Thread(target=worker, args=(i,)) for i in range(len(hs))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        if errs:
            raise errs[0]

    host_steps(args.warmup)
    torch.cuda.synchronize()
    barrier(ws)
    e_steps = max(5, args.steps)   # per thread
    t0 = time.perf_counter()
    host_steps(e_steps)
    torch.cuda.synchronize()
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e, ws)
    e2e = M * nc * e_steps * len(hs) * ws / t_e2e / 1e6
    for h in hs:
        h.close()
    del hbufs
    h2d = (x.numel() + k.numel()) * 8
    d2h = (k.numel() + x.numel()) * 8

    # roofline of the dominant stage
    hbm, src = peaks()
    sb = stage_bytes(obj, nc)
    stages = {}
    for name, r in prof.items():
        if r["launches"] == 0:
            stages[name] = {"ms_per_step": r["ms"] / args.steps, "launches": 0, "note": "cudaMemsetAsync"}
            continue
        per_launch_ms = r["ms"] / r["launches"]
        gbs = sb[name] / (per_launch_ms / 1e3) / 1e9 / (r["launches"] / r["calls"])
        stages[name] = {"ms_per_step": r["ms"] / args.steps, "launches": r["launches"],
                        "algo_bytes_per_launch": sb[name] // max(1, r["launches"] // r["calls"]),
                        "achieved_gbs": round(gbs, 1), "frac_of_%s_hbm" % src: round(gbs / hbm, 4)}
    dom = max((n for n in stages if stages[n]["launches"]), key=lambda n: stages[n]["ms_per_step"])
    d = stages[dom]
    roof = {"bound": "hbm", "kernel": dom, "achieved": d["achieved_gbs"], "peak": hbm, "unit": "GB/s",
            "frac": round(d["achieved_gbs"] / hbm, 4), "peak_source": src,
            "traffic": ncu_traffic(dom), "algo_bytes_per_launch": d["algo_bytes_per_launch"],
            "sm_side": ncu_sm_side(dom)}
    if "gather" in stages and obj.tap_table_bytes and nc >= 8:
        # the stored H read by the 8-coil gather passes, beside its algorithmic bytes
        hb = obj.tap_table_bytes * (nc // 8)
        g = stages["gather"]
        g["stored_h_bytes"] = hb
        g["achieved_gbs_with_stored_h"] = round((g["algo_bytes_per_launch"] + hb) /
                                                (g["ms_per_step"] / 1e3 / max(1, g["launches"] // args.steps)) / 1e9, 1)
    if "spread" in stages and obj.spread_table_bytes and nc >= 8:
        # the stored H' read by the 8-coil spread passes, beside its algorithmic bytes
        hb = obj.spread_table_bytes * (nc // 8)
        g = stages["spread"]
        g["stored_h_t_bytes"] = hb
        g["achieved_gbs_with_stored_h_t"] = round((g["algo_bytes_per_launch"] + hb) /
                                                  (g["ms_per_step"] / 1e3 / max(1, g["launches"] // args.steps)) / 1e9, 1)
    launches = sum(r["launches"] for r in prof.values())
    ours_fft = {"fwd": sum(stages[n]["ms_per_step"] for n in ("fft_x_fwd", "fft_y_fwd", "fft_z_fwd") if n in stages),
                "adj": sum(stages[n]["ms_per_step"] for n in ("fft_x_adj", "fft_y_adj", "fft_z_adj") if n in stages)}
    # results of the timed workload, for the per-coil accuracy check
    want_acc = not args.no_cpu_baseline and ws == 1
    k_host = k.cpu().numpy().T.copy() if want_acc else None
    a_host = x2.cpu().numpy().transpose(3, 2, 1, 0).copy() if want_acc else None

    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": round(value, 2), "unit": "Msample/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64 (fp32)",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "N": args.N, "M": M, "nnz": obj.nnz, "nc": nc,
                       "taps_per_sample": round(obj.taps_per_sample, 2), "tile": list(obj.tile),
                       "stored_h_bytes": obj.tap_table_bytes, "stored_h_t_bytes": obj.spread_table_bytes,
                       "blocks": obj.info()["n_blocks"], "l2": "inputs larger than L2 (grid 1.07 GB), no flush",
                       "parallelism": "replicas" if ws > 1 else "single GPU"},
            "e2e": {"value": round(e2e, 2), "unit": "Msample/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "steps": e_steps * nthreads,
                    "api": "nufft3d_forward_host + nufft3d_adjoint_host from %d host threads, each on its own "
                           "nufft3d_plan_share handle capped at %d SMs (nufft3d_plan_set_sms); pinned buffers %s"
                           % (nthreads, nsm - free_sms,
                              "moved by copy-engine transfers (nufft3d_plan_set_host_copy 1)" if host_copy else
                              "read/written in place by the kernels")},
            "gpu_launches": launches,
            "autotune": tune,
            "roofline": roof,
            "stages": stages,
            "clocks": clk.summary()}
    if not args.no_extras and ws == 1:
        line["fft_comparator"] = bench_cufft(args.N, int(obj.K[0]), nc, ours_fft)
        obj.close()
        del x, k, x2
        torch.cuda.empty_cache()
        line["batched"] = bench_batched()
        line["serving"] = bench_serving()
        line["large_cg"] = bench_large_cg()
    if want_acc:
        line["cpu_baseline"], line["accuracy"] = cpu_baseline(om, args.N, im, k_host, a_host)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
