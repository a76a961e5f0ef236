"""Device status word to C ABI error code, on the host (no GPU).

A kernel whose bounded wait runs out writes a non-zero word into its
context's device status; the host reads it back after the call and the C ABI
returns BCG_ERR_DEVICE_TIMEOUT with a message (the reference turns every CUDA
failure into an exception the same way, native-smoke/solve.cu:46-49).  The
C++ program in tests/native/status_map.cpp runs that mapping with the
library's own code; tests/test_gpu_timeout.py makes a wait run out on a GPU.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "fherma-bytecrt_gb300")
CSRC = os.path.join(PKG, "csrc")


def _nvcc():
    for root in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if root and os.path.exists(os.path.join(root, "bin", "nvcc")):
            return os.path.join(root, "bin", "nvcc")
    return shutil.which("nvcc")


def test_device_status_maps_to_timeout_code(tmp_path):
    # The library's headers carry device code, so nvcc compiles the host program.
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not available")
    if not os.path.exists(os.path.join(PKG, "libbytecrt_gb300.so")):
        pytest.skip("native library not built")
    exe = tmp_path / "status_map"
    subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", CSRC, "-I", os.path.join(REPO, "include"),
                    os.path.join(HERE, "native", "status_map.cpp"), "-o", str(exe),
                    "-L", PKG, "-lbytecrt_gb300", f"-Xlinker=-rpath,{PKG}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "ok"
