"""Bounded device waits run out on purpose, and the context stays usable.

Every kernel wait on another warp role's arrival (a tile built, an MMA
committed, a copy landed for the consumer) is bounded by the context's wait
limit.  With the limit set to 1 ns (finer than the device clock resolves)
such a wait gives up at its first poll that finds the arrival missing, which
every launch meets: the kernel records the timeout in the context's status word, skips its
remaining work, waits for its own copies and MMAs and frees its TMEM.  The
call reports BCG_ERR_DEVICE_TIMEOUT, and the next call on the same context,
with the default limit, is bit-exact against the oracle.  No kernel is broken
and nothing faults: only the limit is short.  (The reference has no bounded
device waits; its error convention is an exception per CUDA failure,
native-smoke/solve.cu:46-49.)
"""
import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

N, W = 4096, 868


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


@pytest.fixture(scope="module")
def case():
    pkg = package()
    q = pkg.inputs.modulus(W, 31)
    count = 3
    a = np.stack([pkg.inputs.uniform(q, N, 300 + i) for i in range(count)])
    b = np.stack([pkg.inputs.uniform(q, N, 310 + i) for i in range(count)])
    o = O.Oracle(N, W, q)
    want = np.stack([o.multiply(a[i], b[i]) for i in range(count)])
    return pkg, q, a, b, want


def _expect_timeout(pkg, m):
    with pytest.raises(pkg.BcgError) as e:
        m.synchronize()
    assert e.value.code == pkg.BCG_ERR_DEVICE_TIMEOUT, str(e.value)
    assert "bounded wait" in str(e.value)


def test_whole_product_wait_runs_out_then_exact(case):
    pkg, q, a, b, want = case
    count = a.shape[0]
    m = pkg.Multiplier(N, W, q)
    da, db = _dev(a), _dev(b)
    dc = torch.zeros_like(da)
    m.set_tuning("wait_limit_ns", 1)
    assert m.get_tuning("wait_limit_ns") == 1
    m.multiply_device(da, db, dc, count)
    _expect_timeout(pkg, m)
    m.set_tuning("wait_limit_ns", 0)
    assert m.get_tuning("wait_limit_ns") == 2_000_000_000
    for _ in range(2):
        dc.fill_(-1)
        m.multiply_device(da, db, dc, count)
        m.synchronize()
        assert np.array_equal(dc.cpu().numpy().view(np.uint32), want)
    m.close()


def test_encode_wait_runs_out_then_exact(case):
    pkg, q, a, b, want = case
    m = pkg.Multiplier(N, W, q)
    pw = m.plane_words
    da, db = _dev(a[:1]), _dev(b[:1])
    pa = torch.zeros(pw, dtype=torch.int32, device="cuda")
    pb = torch.zeros(pw, dtype=torch.int32, device="cuda")
    dc = torch.zeros_like(da)
    m.set_tuning("wait_limit_ns", 1)
    m.encode_device(da, db, pa, pb, pw, 1)
    _expect_timeout(pkg, m)
    m.set_tuning("wait_limit_ns", 0)
    m.encode_device(da, db, pa, pb, pw, 1)
    m.negacyclic_device(pa, pb, pw, 1)
    m.crt_device(pa, pw, dc, 1)
    m.synchronize()
    assert np.array_equal(dc.cpu().numpy().view(np.uint32)[0], want[0])
    m.close()


@pytest.mark.parametrize("persistent,tiles", [(1, 2), (0, 1), (0, 2)])
def test_crt_wait_runs_out_then_exact(case, persistent, tiles):
    pkg, q, a, b, want = case
    m = pkg.Multiplier(N, W, q)
    m.set_tuning("crt_persistent", persistent)
    m.set_tuning("crt_tiles", tiles)
    pw = m.plane_words
    da, db = _dev(a[:1]), _dev(b[:1])
    pa = torch.zeros(pw, dtype=torch.int32, device="cuda")
    pb = torch.zeros(pw, dtype=torch.int32, device="cuda")
    dc = torch.zeros_like(da)
    m.encode_device(da, db, pa, pb, pw, 1)
    m.negacyclic_device(pa, pb, pw, 1)
    m.synchronize()
    # Only the CRT runs with the short limit; the terms it reads stay intact.
    m.set_tuning("wait_limit_ns", 1)
    m.crt_device(pa, pw, dc, 1)
    _expect_timeout(pkg, m)
    m.set_tuning("wait_limit_ns", 0)
    dc.fill_(-1)
    m.crt_device(pa, pw, dc, 1)
    m.synchronize()
    assert np.array_equal(dc.cpu().numpy().view(np.uint32)[0], want[0])
    m.close()
