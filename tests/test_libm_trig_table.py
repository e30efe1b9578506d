"""CPU check of the sinf / cosf exception table (mray_gb300/csrc/libm_trig_core.h): the core evaluated on the
host plus the table's corrections equal the host C library's cosf / sinf for every float of [-pi, pi].  The device
evaluates the same core with the same roundings (tests/test_gpu_libm_trig.py checks the device itself)."""
import os
import subprocess

from mray_gb300 import build as B


def test_table_matches_c_library_everywhere():
    if not (os.path.exists(B.TRIG_TABLE) and os.path.exists(B.TRIG_GEN)):
        os.makedirs(B.BUILD_DIR, exist_ok=True)
        B._trig_table()
    r = subprocess.run([B.TRIG_GEN, "--verify", B.TRIG_TABLE], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "0 mismatches" in r.stdout
