"""GPU tests of concurrent host-pointer calls on shared handles.

Two host threads each call nufft3d_forward_host / nufft3d_adjoint_host on its
own handle of one trajectory (nufft3d_plan_share), with the persistent
interpolation kernels capped below the device's SM count
(nufft3d_plan_set_sms) so that one call's host-link stages run beside the
other's compute.  Results equal those of one handle called alone: the cap
changes only how many blocks take the tile pieces (rel L2 <= 1e-6; the grid's
float atomics may add halos in another order).
"""
import ctypes
import threading

import numpy as np
import pytest

from nufft_3d_gb300 import _lib, nufft_3d, synth

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def test_two_handles_on_two_threads_match_one(cuda):
    torch = cuda
    N, nc = 48, 8
    om = synth.koosh_ball(N, 48, 3000)
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    L = obj._L
    rng = np.random.default_rng(3)
    xs = [(rng.standard_normal((nc, N, N, N)) + 1j * rng.standard_normal((nc, N, N, N))).astype(np.complex64)
          for _ in range(2)]
    # one handle, sequential
    ref_k, ref_a = [], []
    for x in xs:
        k = np.empty((nc, obj.M), np.complex64)
        a = np.empty_like(x)
        _lib.check(L.nufft3d_forward_host(obj.plan, x.ctypes.data, k.ctypes.data, nc))
        _lib.check(L.nufft3d_adjoint_host(obj.plan, k.ctypes.data, a.ctypes.data, nc))
        ref_k.append(k)
        ref_a.append(a)
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    hs = [obj.share(), obj.share()]
    for h in hs:
        _lib.check(L.nufft3d_plan_set_sms(h.plan, nsm - 16))
    bufs = [(torch.from_numpy(x).pin_memory(), torch.empty((nc, obj.M), dtype=torch.complex64).pin_memory(),
             torch.empty(x.shape, dtype=torch.complex64).pin_memory()) for x in xs]
    errs = []

    def worker(i):
        try:
            xh, kh, ah = bufs[i]
            for _ in range(3):
                _lib.check(L.nufft3d_forward_host(hs[i].plan, xh.data_ptr(), kh.data_ptr(), nc))
                _lib.check(L.nufft3d_adjoint_host(hs[i].plan, kh.data_ptr(), ah.data_ptr(), nc))
        except Exception as e:
            errs.append(e)

    th = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs
    for i in range(2):
        assert rel(bufs[i][1].numpy(), ref_k[i]) < 1e-6
        assert rel(bufs[i][2].numpy(), ref_a[i]) < 1e-6
    for h in hs:
        h.close()


def test_sm_cap_rejects_negative(cuda):
    obj = nufft_3d(synth.koosh_ball(16, 16, 100), 16, "J", 6, density_iters=0)
    assert obj._L.nufft3d_plan_set_sms(obj.plan, -1) == _lib.ERR_ARG
    assert obj._L.nufft3d_plan_set_sms(obj.plan, 1) == _lib.SUCCESS
    x = np.ones((16, 16, 16), np.complex64)
    k1 = obj.fNUFT(x)                       # one block takes every piece
    _lib.check(obj._L.nufft3d_plan_set_sms(obj.plan, 0))
    assert rel(k1, obj.fNUFT(x)) < 1e-6


def test_host_copy_modes_match(cuda):
    """nufft3d_plan_set_host_copy: page-locked buffers used in place by the
    kernels (mode 0) or moved by copy-engine transfers through device staging
    buffers (mode 1) give the same results; pageable buffers are staged in
    either mode."""
    torch = cuda
    N, nc = 32, 8
    om = synth.koosh_ball(N, 32, 1500)
    obj = nufft_3d(om, N, "J", 6, density_iters=0)
    L = obj._L
    rng = np.random.default_rng(4)
    x = (rng.standard_normal((nc, N, N, N)) + 1j * rng.standard_normal((nc, N, N, N))).astype(np.complex64)
    out = {}
    for mode in (0, 1):
        _lib.check(L.nufft3d_plan_set_host_copy(obj.plan, mode))
        for pinned in (True, False):
            xh = torch.from_numpy(x.copy())
            kh = torch.empty((nc, obj.M), dtype=torch.complex64)
            ah = torch.empty(x.shape, dtype=torch.complex64)
            if pinned:
                xh, kh, ah = xh.pin_memory(), kh.pin_memory(), ah.pin_memory()
            _lib.check(L.nufft3d_forward_host(obj.plan, xh.data_ptr(), kh.data_ptr(), nc))
            _lib.check(L.nufft3d_adjoint_host(obj.plan, kh.data_ptr(), ah.data_ptr(), nc))
            out[(mode, pinned)] = (kh.numpy().copy(), ah.numpy().copy())
    k0, a0 = out[(0, True)]
    for key, (k, a) in out.items():
        assert np.array_equal(k, k0), key          # the gather is deterministic
        assert rel(a, a0) < 1e-6, key              # the grid's float atomics may add in another order
    assert L.nufft3d_plan_set_host_copy(obj.plan, 2) == _lib.ERR_ARG
