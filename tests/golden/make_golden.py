"""Generates the golden fixtures in this folder from the FP64 oracle.

The reference (MATLAB) cannot run on either machine and ships no golden
vectors, so these fixtures are the oracle's outputs on small seeded inputs;
the oracle itself is pinned by the known-answer tests in tests/test_oracle.py.
Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from nufft_3d_gb300 import synth  # noqa: E402
from oracle.nufft_ref import NufftRef  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (om builder, N, opts, nc)
    "radial_j6_koosh": (lambda: synth.koosh_ball(16, 16, 96), 16, dict(J=6, u=2, radial=True), 2),
    "radial_j4_random": (lambda: synth.random_uniform(12, 1500, seed=3), 12, dict(J=4, u=2, radial=True), 1),
    "separable_j5_u1p5": (lambda: synth.random_uniform(16, 1200, seed=4), 16, dict(J=5, u=1.5, radial=False), 3),
    "outofbounds_j6": (lambda: np.random.default_rng(5).uniform(-10, 10, (3, 900)), 16, dict(J=6, u=2, radial=True), 1),
}


def make(name, build, N, opts, nc, seed=0):
    rng = np.random.default_rng(seed)
    om = build()
    ref = NufftRef(om, N, **opts)
    Nv = tuple(int(v) for v in ref.N)
    x = (rng.standard_normal(Nv + (nc,)) + 1j * rng.standard_normal(Nv + (nc,)))
    y = (rng.standard_normal((ref.M, nc)) + 1j * rng.standard_normal((ref.M, nc)))
    k = ref.fNUFT(x)
    a = ref.aNUFT(y)
    raw = k + 0.01 * y
    im_mr = ref.iNUFT(raw, maxit=8, damp=1e-2, solver="minres", tol=0)
    im_cg = ref.iNUFT(raw, maxit=8, damp=1e-2, solver="cg", tol=0)
    im_gr = ref.iNUFT(raw, maxit=0)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), om=om, N=np.array(N), J=opts["J"], u=opts["u"],
                        radial=int(opts["radial"]), alpha=ref.alpha, nnz=ref.nnz, x=x.astype(np.complex64),
                        y=y.astype(np.complex64), k=k.astype(np.complex64), a=a.astype(np.complex64), U=ref.U.astype(np.float32),
                        d=ref.d.astype(np.float32), raw=raw.astype(np.complex64),
                        im_minres=im_mr.astype(np.complex64), im_cg=im_cg.astype(np.complex64),
                        im_regrid=im_gr.astype(np.complex64), damp=1e-2, maxit=8)


if __name__ == "__main__":
    for name, (b, N, o, nc) in CASES.items():
        make(name, b, N, o, nc)
        print("wrote", name)
