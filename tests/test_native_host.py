"""Host-side checks of the native library that need no GPU: it loads, it
exports every function include/bytecrt_gb300.h declares, its plan equals the
oracle's (which is pinned to the reference), and bad points are rejected."""
import ctypes

import numpy as np
import pytest

from conftest import package, gpu_available
from oracle import oracle as O


def test_library_exports_every_header_function():
    pkg = package()
    names = pkg.header_functions()
    assert len(names) >= 15
    L = pkg.lib()
    for n in names:
        assert hasattr(L, n), n


@pytest.mark.parametrize("N,W,seed", [(16, 40, 1), (64, 100, 2), (256, 434, 3), (1024, 868, 4),
                                      (16384, 434, 5), (32768, 868, 6), (65536, 1747, 7), (4096, 2016, 8)])
def test_native_plan_equals_oracle(N, W, seed):
    pkg = package()
    q = pkg.inputs.modulus(W, seed)
    p = pkg.Plan(N, W, q)
    o = O.Oracle(N, W, q)
    primes, psi, cinv = p.primes()
    assert p.P == o.P
    assert np.array_equal(primes, o.primes)
    assert np.array_equal(psi, o.psi)
    assert np.array_equal(cinv, o.crt_inverse)
    assert np.array_equal(p.weights(), o.weights)
    assert p.info.kpad == o.kpad


def test_reference_geometries_shapes():
    pkg = package()
    for N, W, P, kpad in ((65536, 1747, 114, 480), (32768, 868, 57, 256), (16384, 434, 29, 128)):
        q = pkg.inputs.modulus(W, 1)
        info = pkg.Plan(N, W, q).info
        assert (info.P, info.kpad) == (P, kpad)
        assert info.crt_k == 4 * (P + 1)
        assert info.enc_cols % 64 in (0, 16, 32, 48)


@pytest.mark.parametrize("N,W,mutate,msg", [
    (1000, 434, None, "power of two"),
    (8, 434, None, "power of two"),
    (16384, 434, "even", "odd"),
    (16384, 434, "short", "W bits"),
    (16384, 2100, None, "2016"),
])
def test_invalid_points_rejected(N, W, mutate, msg):
    pkg = package()
    Wq = min(W, 2016) if W <= 2016 else W
    L = (W + 31) // 32
    q = pkg.inputs.modulus(Wq, 3) if W <= 2016 else np.full(L, 0xFFFFFFFF, np.uint32)
    if mutate == "even":
        q = q.copy(); q[0] &= ~np.uint32(1)
    if mutate == "short":
        q = q.copy(); q[-1] = 0
    with pytest.raises(pkg.BcgError) as e:
        pkg.Plan(N, W, q)
    assert e.value.code == pkg.BCG_ERR_INVALID
    assert msg in str(e.value)


def test_gap_form_and_generic_moduli_accepted():
    pkg = package()
    for q in (pkg.inputs.gap_modulus(1747, 1), pkg.inputs.gap_modulus(868, 65535),
              pkg.inputs.modulus(1747, 99)):
        W = 32 * (len(q) - 1) + int(q[-1]).bit_length()
        assert pkg.Plan(65536 if W == 1747 else 32768, W, q).P in (57, 114)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_context_without_gpu_fails_loudly():
    pkg = package()
    q = pkg.inputs.modulus(434, 1)
    with pytest.raises(pkg.BcgError) as e:
        pkg.Multiplier(16384, 434, q)
    assert e.value.code in (pkg.BCG_ERR_CUDA, pkg.BCG_ERR_NOMEM)


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU error path")
def test_batch_and_server_without_gpu_fail_loudly():
    pkg = package()
    with pytest.raises(pkg.BcgError) as e:
        pkg.Batch(0)
    assert e.value.code == pkg.BCG_ERR_CUDA
    with pytest.raises(pkg.BcgError) as e:
        pkg.Server(0)
    assert e.value.code == pkg.BCG_ERR_CUDA


def test_batch_and_server_reject_null_handles():
    L = package().lib()
    assert L.bcg_batch_run(None, None) == 1
    assert L.bcg_batch_add(None, 16, 64, 2, None, None, None, None, 1) == 1
    assert L.bcg_server_submit(None, 1, None, 0, None, None, None) == 1
    assert L.bcg_server_wait(None, 1, 0, None) == 1
    assert L.bcg_server_drain(None) == 1


def test_plugin_rejects_bad_points_before_touching_the_gpu():
    pkg = package()
    q = pkg.inputs.modulus(434, 1)
    with pytest.raises(RuntimeError):
        pkg.fherma_init(pkg.Point(N=16384, W=434, L=15, q=q))
    with pytest.raises(RuntimeError):
        pkg.fherma_init(pkg.Point(N=16384, W=434, L=14, q=q[:13]))
