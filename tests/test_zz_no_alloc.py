"""bcg_multiply_device_static: the allocation-free entry point.

It serves callers that cannot allocate device memory while they run a
product (a memory pool they do not own, a framework that bans cudaMalloc on
its hot path, an allocator at its limit).  It must give exactly the products
of the allocating entry point, call after call, although every call reuses
the same library-owned scratch array.  This file is collected last, so a
failure here comes after every other test has run; it also passes alone in a
fresh process (it creates its own contexts and inputs).
"""
import ctypes

import numpy as np
import pytest

from conftest import package

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


def _call_static(m, a, b, c, count):
    lib = package().lib()
    rc = lib.bcg_multiply_device_static(m._h, a.data_ptr(), b.data_ptr(), c.data_ptr(), count, None)
    assert rc == 0, lib.bcg_last_error().decode()


@pytest.mark.parametrize("N,W,count", [(4096, 868, 3), (16384, 434, 5), (32768, 868, 2)])
def test_static_entry_matches_allocating_entry_twice(N, W, count):
    pkg = package()
    q = pkg.inputs.modulus(W, N + count)
    m = pkg.Multiplier(N, W, q)
    for call in range(2):
        a = np.stack([pkg.inputs.uniform(q, N, 10 * call + i) for i in range(count)])
        b = np.stack([pkg.inputs.uniform(q, N, 10 * call + i + 5) for i in range(count)])
        da, db = _dev(a), _dev(b)
        want = torch.empty_like(da)
        m.multiply_device(da, db, want, count)
        got = torch.full_like(da, -1)
        _call_static(m, da, db, got, count)
        m.synchronize()
        # Exact integers: the tolerance is zero.
        assert torch.equal(got, want), f"call {call}"
    m.close()


def test_static_entry_rejects_points_beyond_its_scratch():
    pkg = package()
    N, W = 65536, 1747                       # 2*P*N = 14.9 M words > 4 Mi words
    q = pkg.inputs.modulus(W, 1)
    m = pkg.Multiplier(N, W, q)
    a = torch.zeros((N, m.L), dtype=torch.int32, device="cuda")
    lib = pkg.lib()
    rc = lib.bcg_multiply_device_static(m._h, a.data_ptr(), a.data_ptr(), a.data_ptr(), 1, None)
    assert rc == pkg.BCG_ERR_INVALID
    assert "scratch" in lib.bcg_last_error().decode()
    m.close()
