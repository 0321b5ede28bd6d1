"""Times the oracle (the FP64 CPU restatement of the reference's sparse path)
on the benchmark workload, and measures the GPU results' per-coil accuracy
against it.  TEST INFRASTRUCTURE: used only by bench.py's cpu_baseline leg and
its --impl reference arm.

One step = fNUFT + aNUFT of ONE coil over the FULL trajectory: deapodization,
pad and FFT on the whole oversampled grid (scipy.fft, all host threads), the
interpolation through the matrix-free FP64 H and H' (interp_ref.c, OpenMP on
all host threads).  Nothing is extrapolated: the rate is the coil-samples
actually processed (M per step) over the measured time.  The literal scipy
CSR form of H is not used at this size: H has 0.95 G nonzeros, and building
it and H' takes far longer than a benchmark run (about 23 GB of CSR arrays);
the matrix-free form applies the same weights (rounded to single,
nufft_3d.m:160) and was checked against the CSR form at small sizes
(tests/test_oracle.py).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from oracle.nufft_ref import NufftRef


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def make_ref(om, N, J=6, u=2):
    """Oracle object on the whole trajectory (matrix-free H, all host threads)."""
    return NufftRef(om, N, J=J, u=u, matrix=False, density_iters=0, workers=cores())


def time_steps(ref, steps, seed=0):
    """Seconds of each fNUFT+aNUFT step of one coil over the full trajectory."""
    rng = np.random.default_rng(seed)
    N = ref.N
    x = rng.standard_normal((N[0], N[1], N[2], 1)) + 1j * rng.standard_normal((N[0], N[1], N[2], 1))
    y = rng.standard_normal((ref.M, 1)) + 1j * rng.standard_normal((ref.M, 1))
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ref.fNUFT(x)
        ref.aNUFT(y)
        times.append(time.perf_counter() - t0)
    return times


def sample_text(ref):
    return ("fNUFT+aNUFT of 1 coil per step over the full trajectory (M=%d), FP64 oracle: deap+pad+FFT+crop "
            "on the full %d^3 grid (scipy.fft, %d threads), matrix-free H and H' (C, OpenMP, %d threads); "
            "rate = coil-samples/s measured, nothing extrapolated" % (ref.M, ref.K[0], cores(), cores()))


def run(om, N, steps, warmup=0):
    """CPU baseline: median over `steps` timed steps after `warmup` untimed ones."""
    ref = make_ref(om, N)
    if warmup:
        time_steps(ref, warmup)
    times = time_steps(ref, steps)
    t = float(np.median(times))
    return {"value": ref.M / t / 1e6, "unit": "Msample/s", "cores": cores(), "kind": "port",
            "sec_per_coil_step": t, "steps": steps, "sample": sample_text(ref)}, ref, times


def forward_per_coil(ref, x):
    """fNUFT of an (N1,N2,N3,nc) image: fft3_pad coil by coil (bounded host
    memory), one matrix-free H product for all coils."""
    nc = x.shape[3]
    G = np.empty((int(np.prod(ref.K)), nc), dtype=np.complex128)
    for c in range(nc):
        k = np.asarray(x[..., c:c + 1], dtype=np.complex128) * ref.U[..., None]
        G[:, c] = ref.fft3_pad(k).reshape(-1, order="F")
    return ref.spmv(G) / math.sqrt(ref.nnz)


def adjoint_per_coil(ref, y):
    K = ref.K
    nc = y.shape[1]
    G = ref.spmv_t(np.asarray(y, dtype=np.complex128))
    out = np.empty(tuple(ref.N) + (nc,), dtype=np.complex128)
    for c in range(nc):
        g = G[:, c].reshape(K[0], K[1], K[2], 1, order="F")
        out[..., c] = (ref.ifft3_crop(g) * ref.U[..., None])[..., 0] / math.sqrt(ref.nnz)
    return out


def accuracy(ref, x, k_gpu, a_gpu):
    """Per-coil relative L2 errors of the GPU results against FP64.

    x: (N1,N2,N3,nc) image given to fNUFT; k_gpu: (M, nc) its GPU forward;
    a_gpu: (N1,N2,N3,nc) the GPU adjoint of k_gpu (the same complex64 data is
    given to the oracle's adjoint)."""
    kr = forward_per_coil(ref, x)
    fwd = [float(np.linalg.norm(k_gpu[:, c] - kr[:, c]) / np.linalg.norm(kr[:, c])) for c in range(kr.shape[1])]
    del kr
    ar = adjoint_per_coil(ref, np.asarray(k_gpu, dtype=np.complex64))
    adj = [float(np.linalg.norm(a_gpu[..., c] - ar[..., c]) / np.linalg.norm(ar[..., c]))
           for c in range(ar.shape[3])]
    return {"fwd_rel_l2_per_coil": fwd, "adj_rel_l2_per_coil": adj, "max": max(fwd + adj), "tolerance": 1e-5,
            "against": "FP64 oracle (matrix-free H, H'; FP64 FFTs), same inputs",
            "adj_input": "the GPU forward output (complex64)"}
