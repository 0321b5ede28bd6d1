"""The MATLAB gateway (nufft_3d_gb300/matlab/nufft3d_mex.c) compiles with
strict warnings against include/nufft3d.h and a declaration-only mex.h (no
MATLAB here, so it is type-checked, not linked or run), and the class folder
exposes the reference's method files."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MATLAB = os.path.join(ROOT, "nufft_3d_gb300", "matlab")


def test_gateway_type_checks():
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    r = subprocess.run([cc, "-std=c99", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "tests", "stubs"), "-I", os.path.join(ROOT, "include"),
                        os.path.join(MATLAB, "nufft3d_mex.c")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_class_folder_has_reference_methods():
    cls = os.path.join(MATLAB, "@nufft_3d")
    for f in ("nufft_3d.m", "fNUFT.m", "aNUFT.m", "iNUFT.m"):
        assert os.path.exists(os.path.join(cls, f)), f
    src = open(os.path.join(cls, "nufft_3d.m")).read()
    for prop in ("J(1,1)", "u(1,1)", "N(1,3)", "alpha(1,1)", "radial(1,1)", "K(1,3)", "nnz(1,1)"):
        assert prop in src, prop
    # every gateway command the class uses is implemented by the gateway
    gw = open(os.path.join(MATLAB, "nufft3d_mex.c")).read()
    for cmd in ("create", "info", "deap", "getd", "destroy", "forward", "adjoint", "inverse"):
        assert '"%s"' % cmd in gw, cmd
