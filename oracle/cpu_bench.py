"""Times the oracle (the FP64 CPU restatement of the reference's sparse path)
on a bounded sample of a fwd+adj workload.  TEST INFRASTRUCTURE: used only by
bench.py's cpu_baseline leg and its --impl reference arm.

One step = fNUFT + aNUFT of one coil through the restatement: the
deapodization and pad/FFT/crop run on the full oversampled grid, the
interpolation (matrix-free H and H', OpenMP) on a subset of the spokes; the
interpolation time is scaled to the full sample count, so the reported rate
is for the whole trajectory (samples/s per coil == coil-samples/s).
"""
from __future__ import annotations

import math
import os
import time

import numpy as np

from oracle.interp_ref import interp_adjoint, interp_forward
from oracle.nufft_ref import NufftRef


def cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1


def make_sample(om_full, N, n_read, spoke_stride, J=6, u=2, workers=None):
    """Oracle object on every spoke_stride-th spoke of a koosh-ball trajectory."""
    n_spokes = om_full.shape[1] // n_read
    om = om_full.reshape(3, n_read, n_spokes, order="F")[:, :, ::spoke_stride].reshape(3, -1, order="F")
    ref = NufftRef(om, N, J=J, u=u, matrix=False, density_iters=0, workers=workers or cores())
    return ref, om.shape[1]


def time_step(ref, x, y, M_full):
    """Seconds for one full-trajectory fwd+adj of one coil (interp scaled)."""
    t0 = time.perf_counter()
    k = ref.fNUFT(x)
    ref.aNUFT(y)
    t_all = time.perf_counter() - t0
    G = int(np.prod(ref.K))
    g = np.zeros((G, 1), dtype=np.complex128)
    t0 = time.perf_counter()
    interp_forward(ref, g)
    interp_adjoint(ref, y)
    t_interp = time.perf_counter() - t0
    scale = M_full / ref.M
    return t_all + t_interp * (scale - 1), k


def run(om_full, N, n_read, nc, steps, spoke_stride=32, seed=0):
    rng = np.random.default_rng(seed)
    ref, m_sub = make_sample(om_full, N, n_read, spoke_stride)
    M = om_full.shape[1]
    x = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    y = rng.standard_normal((m_sub, 1)) + 1j * rng.standard_normal((m_sub, 1))
    times = []
    for _ in range(steps):
        t, _ = time_step(ref, x, y, M)
        times.append(t)
    t = float(np.median(times))
    return {"value": M / t / 1e6, "unit": "Msample/s", "cores": cores(), "kind": "port",
            "sec_per_coil_step": t, "steps": steps,
            "sample": "1 coil per step; deap+pad+FFT+crop on the full %d^3 grid (scipy.fft, %d threads); "
                      "interpolation (matrix-free FP64 H, H', OpenMP) on 1/%d of the spokes (%d of %d samples), "
                      "time scaled to all samples; rate = samples/s per coil" % (ref.K[0], cores(), spoke_stride,
                                                                                 m_sub, M)}
