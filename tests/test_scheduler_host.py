"""Serving-loop policy on the host: scheduler.hpp against a mock executor.

The C++ program in tests/native/sched_mock.cpp drives the real admission and
batch-formation code in virtual time (Poisson arrivals of three request
sizes, 1 to 5 slots) and checks, at every step, that the memory budget is
never exceeded, that the oldest waiting request leads every batch, that a
batch holds one point and one resident operand in arrival order within its
limit, and that every request completes exactly once (large requests are not
starved by a stream of small ones).
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "fherma-bytecrt_gb300", "csrc")


@pytest.fixture(scope="module")
def mock_binary(tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("sched") / "sched_mock"
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", CSRC,
                    os.path.join(HERE, "native", "sched_mock.cpp"), "-o", str(out)], check=True)
    return str(out)


@pytest.mark.parametrize("seed,slots", [(1, 3), (2, 1), (3, 5), (4, 2)])
def test_policy_invariants(mock_binary, seed, slots):
    r = subprocess.run([mock_binary, str(seed), str(slots)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    assert r.stdout.startswith("ok requests=4000")
