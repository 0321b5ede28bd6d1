"""GPU test of nufft3d_forward_noalloc, the forward transform that allocates
no device memory per call (for callers that must not trigger cudaMalloc).

It is compared with the regular nufft3d_forward through the C ABI on two
calls in a row (the second call reuses the shared fixed scratch left by the
first), within the forward tolerance used by the parity tests.  This file is
collected last so a run that stops at the first failure has run everything
else first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL_OP = 1e-5


def _traj(N, two_d):
    from nufft_3d_gb300 import synth
    if not two_d:
        return synth.koosh_ball(N, N, 600)
    rng = np.random.default_rng(9)
    return np.vstack([rng.uniform(-N / 2, N / 2 - 1, (2, 3000)), np.zeros((1, 3000))])


@pytest.mark.parametrize("N,nc,two_d", [
    (24, 3, False),   # coil passes of 2 and 1: the kernel-evaluating gather
    (24, 8, False),   # one 8-coil pass: the stored-H gather, bulk tile copies on the carved grid
    (48, 8, True),    # 2-D: the grid aliases the y-pass buffer
])
def test_forward_noalloc_matches_forward_twice(cuda, N, nc, two_d):
    torch = cuda
    from nufft_3d_gb300 import _lib, nufft_3d

    L = _lib.load()
    om = _traj(N, two_d)
    obj = nufft_3d(om, N, "J", 6, density_iters=0, tap_table=1)
    if nc == 8:
        assert obj.tap_table_bytes > 0
    if two_d:
        assert list(obj.N) == [N, N, 1]
    shape = (nc,) + tuple(int(v) for v in obj.N[::-1])
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    g = torch.Generator(device="cuda").manual_seed(0)
    outs = []
    for call in range(2):
        x = torch.randn(shape, dtype=torch.complex64, device="cuda", generator=g)
        ref = torch.empty((nc, obj.M), dtype=torch.complex64, device="cuda")
        out = torch.full((nc, obj.M), float("nan"), dtype=torch.complex64, device="cuda")
        _lib.check(L.nufft3d_forward(obj.plan, x.data_ptr(), ref.data_ptr(), nc, sp))
        _lib.check(L.nufft3d_forward_noalloc(obj.plan, x.data_ptr(), out.data_ptr(), nc, sp))
        _lib.check(L.nufft3d_check_status(obj.plan, sp))  # no bounded wait expired
        err = float((out - ref).abs().norm() / ref.abs().norm())
        assert err < TOL_OP, (call, err)
        outs.append(out)
    assert not torch.equal(outs[0], outs[1])  # two different inputs, two results


def test_forward_noalloc_rejects_oversize(cuda):
    from nufft_3d_gb300 import _lib, nufft_3d, synth

    L = _lib.load()
    cap = L.nufft3d_forward_noalloc_scratch_bytes()
    assert cap == 32 << 20
    N = 64  # grid 128^3 x 8 B x nc: needs more than the fixed scratch at nc=2
    obj = nufft_3d(synth.koosh_ball(N, 32, 64), N, "J", 6, density_iters=0)
    torch = cuda
    x = torch.zeros((2, N, N, N), dtype=torch.complex64, device="cuda")
    k = torch.zeros((2, obj.M), dtype=torch.complex64, device="cuda")
    st = L.nufft3d_forward_noalloc(obj.plan, x.data_ptr(), k.data_ptr(), 2, None)
    assert st == _lib.ERR_SIZE
    assert "fixed scratch" in _lib.last_error()
