"""The drop-in boundary as the challenge's harness sees it: the `solution`
binary (same wire format as native-smoke/main.cpp) over libfherma_gb300.so,
and the batched variant over libfherma_gb300_batched.so (the plugin ABI of
native-smoke/fherma.h:46-48 and native-batched/fherma.h:47-49)."""
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import package, gpu_available
from oracle import oracle as O

PKG_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "fherma-bytecrt_gb300")


def binary(name):
    path = os.path.join(PKG_DIR, name)
    if not os.path.exists(path):
        pytest.skip(f"{name} not built")
    return path


def write_point(root, N, W, q, cases, B=None, truncate=()):
    L = len(q)
    man = {"N": N, "W": W, "L": L, "cases": len(cases)}
    if B is not None:
        man["B"] = B
    os.makedirs(os.path.join(root, "point"))
    with open(os.path.join(root, "manifest.json"), "w") as f:
        json.dump(man, f)
    q.astype("<u4").tofile(os.path.join(root, "point", "q.bin"))
    for i, (a, b) in enumerate(cases):
        d = os.path.join(root, "cases", f"{i:06d}")
        os.makedirs(d)
        a.astype("<u4").tofile(os.path.join(d, "a.bin"))
        raw = b.astype("<u4").tobytes()
        with open(os.path.join(d, "b.bin"), "wb") as f:
            f.write(raw[:-4] if i in truncate else raw)


@pytest.mark.parametrize("lib", ["libfherma_gb300.so", "libfherma_gb300_batched.so"])
def test_shim_exports_the_plugin_abi(lib):
    if not shutil.which("nm"):
        pytest.skip("nm not available")
    out = subprocess.run(["nm", "-DC", "--defined-only", binary(lib)], capture_output=True, text=True).stdout
    for sym in ("fherma_init(fherma::Point const&)", "fherma_run(void*, fherma::Inputs const&)",
                "fherma_free(void*)"):
        assert sym in out, sym


def test_harness_usage_error():
    r = subprocess.run([binary("solution")], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_harness_init_failure_is_loud(tmp_path):
    pkg = package()
    q = pkg.inputs.modulus(200, 1)
    a = pkg.inputs.uniform(q, 64, 1)
    write_point(str(tmp_path), 64, 200, q, [(a, a)])
    r = subprocess.run([binary("solution"), str(tmp_path)], capture_output=True, text=True)
    # As in the reference harness, an exception from fherma_init ends the run.
    assert r.returncode != 0
    assert "CUDA" in r.stderr or "cuda" in r.stderr


@pytest.mark.gpu
def test_harness_runs_cases_bit_exact(tmp_path):
    pkg = package()
    N, W = 1024, 200
    q = pkg.inputs.modulus(W, 3)
    cases = [(pkg.inputs.uniform(q, N, 2 * i), pkg.inputs.uniform(q, N, 2 * i + 1)) for i in range(3)]
    write_point(str(tmp_path), N, W, q, cases, truncate=(1,))
    r = subprocess.run([binary("solution"), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    res = json.load(open(tmp_path / "out" / "results.json"))
    assert res["init_s"] > 0
    assert [c["status"] for c in res["cases"]] == ["ok", "crashed", "ok"]
    assert "reading the case" in res["cases"][1]["note"]
    o = O.Oracle(N, W, q)
    for i in (0, 2):
        got = np.fromfile(tmp_path / "out" / f"{i:06d}" / "c.bin", dtype="<u4").reshape(N, len(q))
        assert np.array_equal(got, o.multiply(*cases[i]))
        assert res["cases"][i]["seconds"] > 0


@pytest.mark.gpu
def test_batched_harness_bit_exact(tmp_path):
    pkg = package()
    N, W, B = 2048, 434, 3
    q = pkg.inputs.modulus(W, 4)
    cases = []
    for i in range(2):
        a = np.stack([pkg.inputs.uniform(q, N, 10 * i + k) for k in range(B)])
        b = np.stack([pkg.inputs.uniform(q, N, 10 * i + k + 5) for k in range(B)])
        cases.append((a, b))
    write_point(str(tmp_path), N, W, q, cases, B=B)
    r = subprocess.run([binary("solution_batched"), str(tmp_path)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    res = json.load(open(tmp_path / "out" / "results.json"))
    assert [c["status"] for c in res["cases"]] == ["ok", "ok"]
    o = O.Oracle(N, W, q)
    for i, (a, b) in enumerate(cases):
        got = np.fromfile(tmp_path / "out" / f"{i:06d}" / "c.bin", dtype="<u4").reshape(B, N, len(q))
        for k in range(B):
            assert np.array_equal(got[k], o.multiply(a[k], b[k]))


@pytest.mark.gpu
def test_batched_harness_large_output_bit_exact(tmp_path):
    """A batched case whose owned output is above 128 MiB takes the shim's
    destination path (the vector grows run by run and each group is copied
    straight into it): every product equals the device-resident one, and two
    of them the oracle."""
    pkg = package()
    N, W, B = 65536, 1747, 10
    q = pkg.inputs.modulus(W, 5)
    a = np.stack([pkg.inputs.uniform(q, N, 40 + k) for k in range(B)])
    b = np.stack([pkg.inputs.uniform(q, N, 60 + k) for k in range(B)])
    assert a.nbytes >= 128 << 20
    write_point(str(tmp_path), N, W, q, [(a, b)], B=B)
    r = subprocess.run([binary("solution_batched"), str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    res = json.load(open(tmp_path / "out" / "results.json"))
    assert [c["status"] for c in res["cases"]] == ["ok"]
    got = np.fromfile(tmp_path / "out" / "000000" / "c.bin", dtype="<u4").reshape(B, N, len(q))
    m = pkg.Multiplier(N, W, q)
    assert np.array_equal(got, m.multiply(a, b))
    m.close()
    o = O.Oracle(N, W, q)
    for k in (0, B - 1):
        assert np.array_equal(got[k], o.multiply(a[k], b[k])), k
