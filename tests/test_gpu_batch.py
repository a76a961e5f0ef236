"""Batched form through the C ABI (bcg_batch_*): products of uneven points
grouped by (geometry, q) in one CUDA graph.  Every product is bit-exact
against the single-product path and the oracle; B=1 and B=128 agree."""
import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(x: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


def single(pkg, N, W, q, a, b):
    m = pkg.Multiplier(N, W, q)
    out = torch.empty_like(a)
    m.multiply_device(a, b, out, a.shape[0])
    m.synchronize()
    m.close()
    return out


def operands(pkg, q, N, count, seed):
    a = np.stack([pkg.inputs.uniform(q, N, seed + 2 * i) for i in range(count)])
    b = np.stack([pkg.inputs.uniform(q, N, seed + 2 * i + 1) for i in range(count)])
    return dev(a), dev(b)


def test_uneven_batch_matches_single_products_twice():
    pkg = package()
    points = [(4096, 868, 1, 3), (4096, 868, 2, 2), (1024, 434, 3, 5), (16384, 434, 4, 2), (512, 1747, 5, 1)]
    batch = pkg.Batch()
    cases = []
    for N, W, seed, count in points:
        q = pkg.inputs.modulus(W, seed)
        a, b = operands(pkg, q, N, count, 100 * seed)
        c = torch.full_like(a, -1)
        batch.add(N, W, q, a, b, c, count)
        cases.append((N, W, q, a, b, c))
    info = batch.info()
    assert info["groups"] == len(points) and info["products"] == sum(p[3] for p in points)
    # Several groups: two graph branches by default; then one, then two again, explicitly.
    for run, lanes in enumerate((0, 0, 1, 2)):
        if lanes:
            batch.set_lanes(lanes)
        for case in cases:
            case[5].fill_(-1)
        batch.run()
        batch.synchronize()
        for N, W, q, a, b, c in cases:
            assert torch.equal(c, single(pkg, N, W, q, a, b)), (N, W, run, lanes)
    batch.close()


def test_b1_and_b128_bit_exact_at_full_size():
    pkg = package()
    N, W, B, distinct = 65536, 1747, 128, 16
    q = pkg.inputs.modulus(W, 2025)
    a16, b16 = operands(pkg, q, N, distinct, 7)
    a, b = a16.repeat(B // distinct, 1, 1).contiguous(), b16.repeat(B // distinct, 1, 1).contiguous()
    c = torch.empty_like(a)
    big = pkg.Batch()
    big.add(N, W, q, a, b, c, B)
    big.run()
    big.synchronize()
    one = pkg.Batch()
    c1 = torch.empty_like(a16[:1])
    for i in (0, 5, 15):
        one.close()
        one = pkg.Batch()
        one.add(N, W, q, a16[i:i + 1].contiguous(), b16[i:i + 1].contiguous(), c1, 1)
        one.run()
        one.synchronize()
        for k in range(B // distinct):
            assert torch.equal(c[i + distinct * k], c1[0]), (i, k)
    want = O.Oracle(N, W, q).multiply(a16[0].cpu().numpy().view(np.uint32), b16[0].cpu().numpy().view(np.uint32))
    assert np.array_equal(c[0].cpu().numpy().view(np.uint32), want)
    big.close()
    one.close()


def test_config4_shape_uneven_full_size():
    """60% N=32768/W=868 and 40% N=65536/W=1747, three moduli per geometry
    (a tenth of the 96-product workload)."""
    pkg = package()
    batch = pkg.Batch()
    cases = []
    for (N, W), counts in (((32768, 868), (2, 2, 2)), ((65536, 1747), (2, 1, 1))):
        for k, count in enumerate(counts):
            q = pkg.inputs.modulus(W, 300 + k)
            a, b = operands(pkg, q, N, count, 1000 * k + N)
            c = torch.empty_like(a)
            batch.add(N, W, q, a, b, c, count)
            cases.append((N, W, q, a, b, c))
    assert batch.info()["groups"] == 6
    batch.run()
    batch.synchronize()
    for N, W, q, a, b, c in cases:
        assert torch.equal(c, single(pkg, N, W, q, a, b))
    batch.close()


def test_profile_inside_graph():
    pkg = package()
    N, W = 16384, 434
    q = pkg.inputs.modulus(W, 9)
    a, b = operands(pkg, q, N, 40, 3)
    c = torch.empty_like(a)
    batch = pkg.Batch()
    batch.add(N, W, q, a, b, c, 40)
    batch.profile(every=1)
    batch.run()
    batch.synchronize()
    p = batch.read_profile()
    info = batch.info()
    assert p["chains"] == info["chains"] >= 2
    assert sum(p["launches"].values()) == info["launches"]
    for stage in ("encode", "column", "row", "column_inverse", "crt"):
        assert p["timed"][stage] == p["launches"][stage] > 0
        assert p["ms"][stage] > 0
    assert torch.equal(c, single(pkg, N, W, q, a, b))
    batch.close()
