"""bcg_multiply_device_static: the allocation-free entry point.

It serves callers that cannot allocate device memory while they run a
product (a memory pool they do not own, a framework that bans cudaMalloc on
its hot path, an allocator at its limit).  It must give exactly the products
of the allocating entry point, call after call, although every call reuses
the same library-owned scratch array, and after its first call on a device
(which looks up the array's address) a call must leave the device's free
memory unchanged.  This file is collected last, so a failure here comes after
every other test has run; it also passes alone in a fresh process (it creates
its own contexts and inputs).
"""
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


def _operands(pkg, q, N, count, seed):
    L = len(q)
    a = pkg.inputs.uniform(q, N * count, seed).reshape(count, N, L)
    b = pkg.inputs.uniform(q, N * count, seed + 1).reshape(count, N, L)
    return a, b


# (4096, 868): several products per launch chain; (16384, 434) and (32768, 868):
# mid-size points; (32768, 980): P = 64, so one product fills the 4 Mi-word
# scratch exactly and every chain holds one product; (16, 40): 3 primes, so the
# scratch would hold 43,690 products at once, more than a grid dimension allows
# for the column pass (2 x products on grid.z): the chains must stay at the
# context's own length.
@pytest.mark.parametrize("N,W,count", [(4096, 868, 3), (16384, 434, 5), (32768, 868, 2), (32768, 980, 2),
                                       (16, 40, 70000)])
def test_static_entry_matches_allocating_entry_twice(N, W, count):
    pkg = package()
    q = pkg.inputs.modulus(W, N + count)
    m = pkg.Multiplier(N, W, q)
    for call in range(2):
        a, b = _operands(pkg, q, N, count, 10 * call + 1)
        da, db = _dev(a), _dev(b)
        want = torch.empty_like(da)
        m.multiply_device(da, db, want, count)
        got = torch.full_like(da, -1)
        _call_static(m, da, db, got, count)
        m.synchronize()
        # Exact integers: the tolerance is zero.
        assert torch.equal(got, want), f"call {call}"
    m.close()


def test_static_entry_allocates_nothing_after_its_first_call():
    pkg = package()
    N, W, count = 16384, 434, 4
    q = pkg.inputs.modulus(W, 5)
    m = pkg.Multiplier(N, W, q)
    a, b = _operands(pkg, q, N, count, 40)
    da, db = _dev(a), _dev(b)
    got = torch.full_like(da, -1)
    want = torch.empty_like(da)
    m.multiply_device(da, db, want, count)       # the allocating path's workspace exists from here on
    _call_static(m, da, db, got, count)          # set-up: the scratch address is looked up once
    m.synchronize()
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _call_static(m, da, db, got, count)
    m.synchronize()
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert torch.equal(got, want)
    m.close()


@pytest.mark.parametrize("N,W", [(65536, 1747), (32768, 984)])
def test_static_entry_rejects_points_beyond_its_scratch(N, W):
    pkg = package()
    q = pkg.inputs.modulus(W, 1)
    m = pkg.Multiplier(N, W, q)
    assert 2 * m.P * N > (4 << 20)              # 2*P*N words do not fit 4 Mi words
    a = torch.zeros((N, m.L), dtype=torch.int32, device="cuda")
    lib = pkg.lib()
    rc = lib.bcg_multiply_device_static(m._h, a.data_ptr(), a.data_ptr(), a.data_ptr(), 1, None)
    assert rc == pkg.BCG_ERR_INVALID
    assert "scratch" in lib.bcg_last_error().decode()
    m.close()
