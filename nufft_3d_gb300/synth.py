"""Seeded synthetic inputs with the shapes of the reference's demo and the benchmark workloads.

Nothing here is part of the transform; these build test and benchmark inputs:

* ``koosh_ball``     center-out radial spokes on a golden-angle sphere, the
                      rotation scheme of test_nufft3d.m:17-45 with uniform
                      radial spacing (om in cycles/FOV, spoke end N/2-1 as
                      test_nufft3d.m:11 scales it so no sample is dropped).
* ``stack_of_spirals`` 2-D Archimedean spiral interleaves stacked in kz.
* ``random_uniform``  uniform samples in the [-N/2, N/2-1] box.
* ``phantom3d``       sum of ellipsoids with the modified Shepp-Logan table
                      (Toft's published values); meshgrid x/y order as the
                      reference's phantom3d.m:81-84 uses.
* ``coil_maps``       smooth Gaussian sensitivities on a ring, random phase.
* ``add_noise``       complex Gaussian noise at a given SNR (dB).

Arrays follow the MATLAB column-major convention of the reference: an image
is (N1, N2, N3[, nc]) read with ``order='F'``; om is (3, M).
"""
from __future__ import annotations

import math

import numpy as np


def koosh_ball(N, n_read, n_spokes, dtype=np.float64):
    """om [3, n_read*n_spokes]: spoke s, readout r at index r + n_read*s."""
    t = np.linspace(0.0, N / 2 - 1, n_read)
    k = np.arange(n_spokes, dtype=np.float64)
    dH = 1 - 2 * k / max(n_spokes - 1, 1)
    polar = np.arccos(np.clip(dH, -1.0, 1.0))
    azim = k * math.pi * (3 - math.sqrt(5))
    # third column of the demo's rotation matrix applied to [0; 0; t]
    d = np.stack([np.cos(azim) * np.sin(polar), np.sin(azim) * np.sin(polar), np.cos(polar)])
    om = d[:, None, :] * t[None, :, None]          # (3, n_read, n_spokes)
    return om.reshape(3, -1, order="F").astype(dtype)


def stack_of_spirals(N, n_interleaves=16, n_samples=2048, n_partitions=64, turns=None, dtype=np.float64):
    kmax = N / 2 - 1
    turns = turns if turns is not None else max(1.0, N / (2 * n_interleaves))
    t = np.linspace(0.0, 1.0, n_samples)
    r = kmax * t
    theta = 2 * math.pi * turns * t
    kz = np.linspace(-N / 2, N / 2 - 1, n_partitions)
    pts = []
    for p in range(n_partitions):
        for i in range(n_interleaves):
            ph = theta + 2 * math.pi * i / n_interleaves
            pts.append(np.stack([r * np.cos(ph), r * np.sin(ph), np.full(n_samples, kz[p])]))
    return np.concatenate(pts, axis=1).astype(dtype)


def random_uniform(N, M, seed=0, dtype=np.float64):
    rng = np.random.default_rng(seed)
    return rng.uniform(-N / 2, N / 2 - 1, size=(3, M)).astype(dtype)


# Modified Shepp-Logan (Toft 1996): A, a, b, c, x0, y0, z0, phi, theta, psi
_MSL = np.array([
    [1.0, .6900, .920, .810, 0, 0, 0, 0, 0, 0],
    [-.8, .6624, .874, .780, 0, -.0184, 0, 0, 0, 0],
    [-.2, .1100, .310, .220, .22, 0, 0, -18, 0, 10],
    [-.2, .1600, .410, .280, -.22, 0, 0, 18, 0, 10],
    [.1, .2100, .250, .410, 0, .35, -.15, 0, 0, 0],
    [.1, .0460, .046, .050, 0, .1, .25, 0, 0, 0],
    [.1, .0460, .046, .050, 0, -.1, .25, 0, 0, 0],
    [.1, .0460, .023, .050, -.08, -.605, 0, 0, 0, 0],
    [.1, .0230, .023, .020, 0, -.606, 0, 0, 0, 0],
    [.1, .0230, .046, .020, .06, -.605, 0, 0, 0, 0],
])


def phantom3d(n):
    """Modified Shepp-Logan head phantom on an n^3 grid (real, float64)."""
    rng = (np.arange(n) - (n - 1) / 2) / ((n - 1) / 2)
    # meshgrid: x varies along dim 2, y along dim 1
    y, x, z = np.meshgrid(rng, rng, rng, indexing="ij")
    coord = np.stack([x.ravel(order="F"), y.ravel(order="F"), z.ravel(order="F")])
    p = np.zeros(coord.shape[1])
    for A, a, b, c, x0, y0, z0, ph, th, ps in _MSL:
        ph, th, ps = np.deg2rad([ph, th, ps])
        cph, sph, cth, sth, cps, sps = np.cos(ph), np.sin(ph), np.cos(th), np.sin(th), np.cos(ps), np.sin(ps)
        R = np.array([[cps * cph - cth * sph * sps, cps * sph + cth * cph * sps, sps * sth],
                      [-sps * cph - cth * sph * cps, -sps * sph + cth * cph * cps, cps * sth],
                      [sth * sph, -sth * cph, cth]])
        cp = R @ coord
        dist = (cp[0] - x0) ** 2 / a ** 2 + (cp[1] - y0) ** 2 / b ** 2 + (cp[2] - z0) ** 2 / c ** 2
        p[dist <= 1] += A
    return p.reshape(n, n, n, order="F")


def phantom_with_phase(n):
    """The demo's test object: phantom with im(im==1) = i (test_nufft3d.m:5-7)."""
    im = phantom3d(n).astype(np.complex128)
    im[im == 1] = 1j
    return im


def coil_maps(N, nc, seed=0, sigma=0.5):
    """Gaussian sensitivities exp(-|r-c|^2/(2 sigma^2)) (r in FOV units), centres
    on a ring of radius 0.5 in the x-y plane, each with a random phase."""
    rng = np.random.default_rng(seed)
    g = (np.arange(N) - N / 2) / N
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    maps = np.empty((N, N, N, nc), dtype=np.complex128)
    for c in range(nc):
        ang = 2 * math.pi * c / nc
        cx, cy = 0.5 * math.cos(ang), 0.5 * math.sin(ang)
        r2 = (X - cx) ** 2 + (Y - cy) ** 2 + Z ** 2
        maps[..., c] = np.exp(-r2 / (2 * sigma ** 2)) * np.exp(1j * rng.uniform(0, 2 * math.pi))
    return maps


def add_noise(data, snr_db, seed=0):
    rng = np.random.default_rng(seed)
    data = np.asarray(data)
    noise = rng.standard_normal(data.shape) + 1j * rng.standard_normal(data.shape)
    scale = np.linalg.norm(data) / np.linalg.norm(noise) * 10 ** (-snr_db / 20)
    return data + scale * noise, scale / math.sqrt(2)
