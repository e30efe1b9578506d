"""The reference-side shims (mray_gb300/shim/) compile against the reference's own headers: the drop-in seams
type-check.  Runs only where the reference sources were staged (oracle/stage_reference.py)."""
import os
import shutil
import subprocess

import pytest

from stage_reference import reference_src

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = reference_src()


@pytest.mark.skipif(REF is None, reason="reference sources not staged")
@pytest.mark.parametrize("shim", ["moment_raymarcher_gb300.cpp", "moment_image_io_gb300.cpp"])
def test_shim_compiles_against_reference_headers(tmp_path, shim):
    cuda_inc = "/usr/local/cuda/include"
    if not shutil.which("g++") or not os.path.isdir(cuda_inc):
        pytest.skip("g++ or CUDA headers missing")
    cmd = ["g++", "-std=c++14", "-fsyntax-only", "-DCUDA_SUPPORT", "-include", "algorithm", "-include", "cstring",
           "-include", "numeric", "-I", REF, "-I", os.path.join(ROOT, "include"), "-I", cuda_inc, "-w",
           os.path.join(ROOT, "mray_gb300", "shim", shim)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
