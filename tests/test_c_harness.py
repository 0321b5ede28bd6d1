"""The plain C host (nufft_3d_gb300/c_harness/nufft3d_harness.c) builds against
include/nufft3d.h with strict C99 warnings, and on a GPU passes its adjoint
identity and iNUFT objective checks through the host-pointer entry points."""
import os
import subprocess

import pytest

from nufft_3d_gb300 import build as nb


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if not os.path.exists(nb.LIB):
        pytest.skip("libnufft3d.so not built")
    out = str(tmp_path_factory.mktemp("harness") / "nufft3d_harness")
    return nb.build_harness(out)


def test_harness_builds_and_reports_missing_device(harness):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present: covered by the gpu test")
    r = subprocess.run([harness], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2, r.stdout + r.stderr
    assert "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_harness_passes_on_gpu(harness):
    r = subprocess.run([harness], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "PASS" in r.stdout
    r = subprocess.run([harness, "48", "900"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
