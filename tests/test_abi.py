"""CPU tests of the C ABI: the library loads, exports every declared entry
point, and rejects the reference's invalid arguments before touching a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from nufft_3d_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nufft3d.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nufft3d_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_opts_struct_layout_matches_defaults():
    L = _lib.load()
    o = _lib.Opts()
    assert L.nufft3d_opts_default(ctypes.byref(o)) == 0
    assert (o.J, o.u, o.alpha, o.radial, o.gpu, o.density_iters) == (4.0, 2.0, 0.0, 1, 1, 20)
    assert o.tap_table == -1  # the stored H is built when it fits
    assert o.wait_polls == 1 << 22
    assert o.spread_table == -1  # last field: the layout matches the header


def test_header_struct_fields_match_ctypes():
    """Every field of nufft3d_opts / nufft3d_info in include/nufft3d.h is mirrored, in order."""
    import os, re
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "nufft3d.h")).read()
    for cname, cls in (("nufft3d_opts", _lib.Opts), ("nufft3d_info", _lib.Info),
                       ("nufft3d_tune_result", _lib.TuneResult)):
        body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (cname, cname), hdr, re.S).group(1)
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        names = []
        for decl in body.split(";"):
            if not decl.strip():
                continue
            parts = decl.split(",")  # "double J, u, alpha"
            for i, part in enumerate(parts):
                word = part.split()[-1] if i == 0 else part.strip()
                names.append(re.sub(r"\[.*\]", "", word.lstrip("*")))
        assert names == [f[0] for f in cls._fields_], (cname, names)


def _create(om, N, **kw):
    L = _lib.load()
    o = _lib.Opts()
    L.nufft3d_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    om = np.ascontiguousarray(np.asarray(om, dtype=np.float64).T)
    Nc = (ctypes.c_int32 * 3)(*np.resize(np.asarray(N, dtype=np.int32), 3))
    plan = ctypes.c_void_p()
    st = L.nufft3d_plan_create(om.ctypes.data, om.shape[0], ctypes.cast(Nc, ctypes.c_void_p), np.size(N),
                               ctypes.byref(o), ctypes.byref(plan))
    return st, _lib.last_error()


@pytest.mark.parametrize("kw,N,code,msg", [
    (dict(u=0.5), 16, _lib.ERR_ARG, "value of u"),          # nufft_3d.m:82-83
    (dict(u=7.0), 16, _lib.ERR_ARG, "value of u"),
    ({}, 15, _lib.ERR_ARG, "even integer"),                 # nufft_3d.m:101-102
    ({}, [16, 15, 16], _lib.ERR_ARG, "even integer"),
    (dict(gpu=0), 16, _lib.ERR_UNSUPPORTED, "CPU"),         # no CPU fallback
    (dict(J=9.0), 16, _lib.ERR_UNSUPPORTED, "J"),
    (dict(wait_polls=-1), 16, _lib.ERR_ARG, "wait_polls"),
])
def test_invalid_arguments_rejected(kw, N, code, msg):
    om = np.random.default_rng(0).uniform(-4, 4, (3, 50))
    st, err = _create(om, N, **kw)
    assert st == code and msg in err


def test_too_large_grid_rejected():
    # nufft_3d.m:111: prod(K) >= intmax('int32')
    om = np.random.default_rng(0).uniform(-4, 4, (3, 50))
    st, err = _create(om, 1024, u=2.0)
    assert st == _lib.ERR_SIZE and "too large" in err


def test_empty_trajectory_rejected():
    st, err = _create(np.zeros((3, 0)), 16)
    assert st == _lib.ERR_ARG and "om must be" in err


def test_python_class_argument_checks():
    from nufft_3d_gb300 import nufft_3d
    with pytest.raises(ValueError, match="leading dimension of 3"):
        nufft_3d(np.zeros((2, 4)), 16)
    with pytest.raises(ValueError, match="string/value pairs"):
        nufft_3d(np.ones((3, 4)), 16, "J")
    with pytest.raises(ValueError, match="unknown property"):
        nufft_3d(np.ones((3, 4)), 16, "K", 3)
    with pytest.raises(_lib.NufftError, match="value of u"):
        nufft_3d(np.ones((3, 4)), 16, "u", 9)


def test_solver_entry_points_check_arguments_without_a_device():
    """The warm-start and phase-constrained entry points validate their
    arguments before touching a device (NULL plan, negative lambda)."""
    L = _lib.load()
    buf = (ctypes.c_float * 8)()
    its = (ctypes.c_int * 1)()
    for fn in (L.nufft3d_inverse_x0, L.nufft3d_inverse):
        assert fn(None, buf, buf, 1, 5, 0.1, None, _lib.SOLVER_CG, 0.0, its, None) == _lib.ERR_ARG
    for fn in (L.nufft3d_inverse_x0_host, L.nufft3d_inverse_host):
        assert fn(None, buf, buf, 1, 5, 0.1, None, _lib.SOLVER_MINRES, 0.0, its) == _lib.ERR_ARG
    assert L.nufft3d_inverse_phase(None, buf, buf, 1, 5, 0.1, 0.5, None, 0.0, its, None) == _lib.ERR_ARG
    assert L.nufft3d_inverse_phase_host(None, buf, buf, 1, 5, 0.1, -1.0, None, 0.0, its) == _lib.ERR_ARG
    assert "lambda" in _lib.last_error()


def test_check_status_rejects_null_plan():
    L = _lib.load()
    assert L.nufft3d_check_status(None, None) == _lib.ERR_ARG


def test_set_sms_rejects_null_plan():
    L = _lib.load()
    assert L.nufft3d_plan_set_sms(None, 4) == _lib.ERR_ARG
    assert L.nufft3d_plan_set_host_copy(None, 1) == _lib.ERR_ARG


def test_tune_rejects_bad_arguments():
    L = _lib.load()
    r = _lib.TuneResult()
    assert L.nufft3d_plan_tune(None, 8, 0, ctypes.byref(r)) == _lib.ERR_ARG


def test_kernel_eval_checks_arguments():
    L = _lib.load()
    assert L.nufft3d_kernel_eval(None, None, None, 4, None) == _lib.ERR_ARG
