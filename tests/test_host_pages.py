"""The host-buffer page arithmetic on the host (no GPU).

Registering an unaligned range locks the whole pages around it and so takes
in neighbouring buffers' bytes; copies that start in a registered page must
stay in its registration.  csrc/host_pages.hpp keeps registrations to whole
pages inside each buffer and cuts every group's copy accordingly;
tests/native/host_pages.cpp checks those rules on 200,000 random buffer
placements, group sizes and page sizes (4 KiB and 64 KiB).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(REPO, "fherma-bytecrt_gb300", "csrc")


def test_page_arithmetic(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path / "host_pages"
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", CSRC, os.path.join(HERE, "native", "host_pages.cpp"),
                    "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok ")
