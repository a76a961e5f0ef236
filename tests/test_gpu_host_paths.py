"""Host-buffer paths through the C ABI at sizes that take several staging
groups: pageable buffers (bcg_multiply: direct DMA of the inputs where the
GPU reads host page tables, staged output pieces), pinned buffers (direct DMA
both ways), and the sink entry point the plugin uses (bcg_multiply_sink: the
product in order, in pieces).  Every product equals the device-resident path,
and a few are checked against the oracle."""
import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def operands(pkg, q, N, count, seed):
    a = np.stack([pkg.inputs.uniform(q, N, seed + i) for i in range(count)])
    b = np.stack([pkg.inputs.uniform(q, N, seed + 500 + i) for i in range(count)])
    return a, b


def device_products(m, a, b):
    da = torch.from_numpy(a.view(np.int32)).cuda()
    db = torch.from_numpy(b.view(np.int32)).cuda()
    dc = torch.empty_like(da)
    m.multiply_device(da, db, dc, a.shape[0])
    m.synchronize()
    return dc.cpu().numpy().view(np.uint32)


# (N, W, count): one host group, two (still a small call: no page locking), and
# three or more (the staging groups hold about 128 MiB of operands: 4 products
# at N=65536, 32 at N=16384).
CASES = [(4096, 868, 5), (65536, 1747, 6), (65536, 1747, 9), (16384, 434, 150)]


@pytest.mark.parametrize("N,W,count", CASES)
def test_pageable_host_buffers(N, W, count):
    pkg = package()
    q = pkg.inputs.modulus(W, 31)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 100)
    got = m.multiply(a, b)
    assert np.array_equal(got, device_products(m, a, b))
    o = O.Oracle(N, W, q)
    for i in (0, count - 1):
        assert np.array_equal(got[i], o.multiply(a[i], b[i])), i
    m.close()


@pytest.mark.parametrize("N,W,count", CASES)
def test_pinned_host_buffers(N, W, count):
    pkg = package()
    q = pkg.inputs.modulus(W, 32)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 200)
    ta = torch.from_numpy(a.view(np.int32)).pin_memory()
    tb = torch.from_numpy(b.view(np.int32)).pin_memory()
    tc = torch.zeros_like(ta).pin_memory()
    m.multiply_into(ta, tb, tc, count)
    assert np.array_equal(tc.numpy().view(np.uint32), device_products(m, a, b))
    m.close()


@pytest.mark.parametrize("N,W,count", CASES)
def test_sink_pieces_arrive_in_order(N, W, count):
    pkg = package()
    q = pkg.inputs.gap_modulus(W, 12345) if W > 70 else pkg.inputs.modulus(W, 33)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 300)
    calls, pieces = [], []

    def sink(words, n):
        calls.append((words is None, n))
        if words is not None:
            assert words.shape == (n,)
            pieces.append(words.copy())

    m.multiply_sink(a, b, sink)
    # Each group's words are announced by a preparation call (words=None, n =
    # the group's words), then arrive in pieces that add up to exactly n.
    assert calls[0][0]
    left = 0
    for prep, n in calls:
        if prep:
            assert left == 0 and n > 0
            left = n
        else:
            left -= n
            assert left >= 0
    assert left == 0
    assert sum(n for prep, n in calls if prep) == a.size
    got = np.concatenate(pieces).reshape(a.shape)
    assert np.array_equal(got, device_products(m, a, b))
    m.close()


def test_sink_exception_is_reraised():
    pkg = package()
    N, W = 1024, 200
    q = pkg.inputs.modulus(W, 34)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, 2, 400)

    def sink(words, n):
        if words is not None:
            raise RuntimeError("caller-side failure")

    with pytest.raises(RuntimeError, match="caller-side failure"):
        m.multiply_sink(a, b, sink)
    # The context stays usable.
    assert np.array_equal(m.multiply(a, b), device_products(m, a, b))
    m.close()


@pytest.mark.parametrize("N,W,count", CASES)
def test_dest_runs_fill_one_buffer(N, W, count):
    """bcg_multiply_dest as the plugin drives it: consecutive runs of one
    pageable buffer (neighbouring runs share pages), named in order."""
    pkg = package()
    q = pkg.inputs.modulus(W, 35)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 500)
    out = np.zeros(a.size + 7, dtype=np.uint32)[3:3 + a.size]     # not page-aligned
    sizes = []

    def dest(n):
        at = sum(sizes)
        sizes.append(n)
        return out.ctypes.data + 4 * at

    m.multiply_dest(a, b, dest)
    assert sum(sizes) == a.size and all(n > 0 for n in sizes)
    assert np.array_equal(out.reshape(a.shape), device_products(m, a, b))
    m.close()


@pytest.mark.parametrize("count", [1, 10])
@pytest.mark.parametrize("layout", ["separate", "reversed", "pinned"])
def test_dest_layouts(layout, count):
    """Runs in separate buffers, runs placed back to front in one buffer, and
    runs in pinned memory, in a small call (one group: written by the SMs where
    the GPU uses the host page tables) and a larger one (three groups: whole
    pages locked run by run, partial pages through staging): the same products
    as the device path."""
    pkg = package()
    N, W = 65536, 1747
    q = pkg.inputs.modulus(W, 36)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 600)
    words = a.size
    keep, runs = [], []
    whole = (torch.zeros(words, dtype=torch.int32).pin_memory() if layout == "pinned"
             else np.zeros(words + 5, dtype=np.uint32)[1:1 + words])
    base = whole.data_ptr() if layout == "pinned" else whole.ctypes.data
    placed = [0]

    def dest(n):
        if layout == "separate":
            buf = np.zeros(n + 3, dtype=np.uint32)[2:2 + n]
            keep.append(buf)
            runs.append(buf)
            return buf.ctypes.data
        placed[0] += n
        start = words - placed[0] if layout == "reversed" else placed[0] - n
        runs.append((start, n))
        return base + 4 * start

    m.multiply_dest(a, b, dest)
    if layout == "separate":
        got = np.concatenate(runs)
    else:
        flat = whole.numpy().view(np.uint32) if layout == "pinned" else whole
        got = np.concatenate([flat[s:s + n] for s, n in runs])
    assert np.array_equal(got.reshape(a.shape), device_products(m, a, b))
    m.close()


def test_dest_refusal_fails_the_call_and_keeps_the_context():
    pkg = package()
    N, W, count = 65536, 1747, 9
    q = pkg.inputs.modulus(W, 37)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 700)
    out = np.zeros(a.size, dtype=np.uint32)
    named = []

    def dest(n):
        named.append(n)
        return 0 if len(named) == 2 else out.ctypes.data + 4 * sum(named[:-1])

    with pytest.raises(pkg.BcgError):
        m.multiply_dest(a, b, dest)
    assert len(named) == 2
    assert np.array_equal(m.multiply(a, b), device_products(m, a, b))
    m.close()


def test_host_alloc_buffers():
    """Pinned buffers from bcg_host_alloc take the direct copy path and give the device path's products."""
    import ctypes
    pkg = package()
    N, W, count = 16384, 434, 80
    q = pkg.inputs.modulus(W, 38)
    m = pkg.Multiplier(N, W, q)
    a, b = operands(pkg, q, N, count, 800)
    nbytes = a.nbytes
    pa, pb, pc = (pkg.native.host_alloc(nbytes) for _ in range(3))
    try:
        ctypes.memmove(pa, a.ctypes.data, nbytes)
        ctypes.memmove(pb, b.ctypes.data, nbytes)
        m.multiply_into(pa, pb, pc, count)
        got = np.ctypeslib.as_array((ctypes.c_uint32 * a.size).from_address(pc)).reshape(a.shape).copy()
    finally:
        for p in (pa, pb, pc):
            pkg.native.host_free(p)
    assert np.array_equal(got, device_products(m, a, b))
    m.close()


@pytest.mark.parametrize("N,W,count", [(4096, 868, 5), (65536, 1747, 6)])
def test_small_calls_without_host_page_tables(N, W, count):
    """host_direct = 0: small calls pack pageable operands into pinned staging
    and take outputs back in 4 MiB pieces, the path of systems whose GPU does
    not use the host page tables; pageable output, sink and named destination
    all give the device path's products."""
    pkg = package()
    q = pkg.inputs.modulus(W, 39)
    m = pkg.Multiplier(N, W, q)
    m.set_tuning("host_direct", 0)
    assert m.get_tuning("host_direct") == 0
    a, b = operands(pkg, q, N, count, 900)
    want = device_products(m, a, b)
    assert np.array_equal(m.multiply(a, b), want)
    pieces = []
    m.multiply_sink(a, b, lambda words, n: pieces.append(words.copy()) if words is not None else None)
    assert np.array_equal(np.concatenate(pieces).reshape(a.shape), want)
    out = np.zeros(a.size + 3, dtype=np.uint32)[1:1 + a.size]
    sizes = []

    def dest(n):
        at = sum(sizes)
        sizes.append(n)
        return out.ctypes.data + 4 * at

    m.multiply_dest(a, b, dest)
    assert np.array_equal(out.reshape(a.shape), want)
    m.set_tuning("host_direct", 1)
    m.close()


@pytest.mark.parametrize("host_group", [1, 2, 3, 8])
def test_host_group_knob(host_group):
    """Any number of products per host-path group gives the device path's products (pageable and pinned)."""
    pkg = package()
    N, W, count = 65536, 1747, 9
    q = pkg.inputs.modulus(W, 40)
    m = pkg.Multiplier(N, W, q)
    m.set_tuning("host_group", host_group)
    assert m.get_tuning("host_group") == host_group
    a, b = operands(pkg, q, N, count, 1000)
    want = device_products(m, a, b)
    assert np.array_equal(m.multiply(a, b), want)
    ta = torch.from_numpy(a.view(np.int32)).pin_memory()
    tb = torch.from_numpy(b.view(np.int32)).pin_memory()
    tc = torch.zeros_like(ta).pin_memory()
    m.multiply_into(ta, tb, tc, count)
    assert np.array_equal(tc.numpy().view(np.uint32), want)
    m.close()
