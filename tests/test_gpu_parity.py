"""GPU parity: every stage and the whole product, through the C ABI, bit-exact
against the CPU oracle (oracle/oracle.c, pinned to the reference)."""
import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(x: np.ndarray):
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int32)).cuda()


def host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def empty(words: int):
    return torch.zeros(words, dtype=torch.int32, device="cuda")


_cache = {}


def setup(N, W, seed):
    key = (N, W, seed)
    if key not in _cache:
        pkg = package()
        q = pkg.inputs.modulus(W, seed)
        _cache[key] = (pkg.Multiplier(N, W, q), O.Oracle(N, W, q), q)
    return _cache[key]


SMALL = [(16, 40), (64, 100), (256, 434), (512, 868), (2048, 300), (4096, 1747)]
FULL = [(16384, 434), (32768, 868), (65536, 1747)]


@pytest.mark.parametrize("N,W", SMALL + FULL)
def test_encode_matches_oracle(N, W):
    pkg = package()
    m, o, q = setup(N, W, 1)
    a = pkg.inputs.uniform(q, N, 11)
    b = pkg.inputs.fixture(q, N, "minus_one")
    pw = m.plane_words
    pa, pb = empty(pw), empty(pw)
    m.encode_device(dev(a), dev(b), pa, pb, pw, 1)
    m.synchronize()
    p = o.primes.astype(np.uint64)[:, None]
    for x, planes in ((a, pa), (b, pb)):
        got = host(planes).reshape(o.P, N).astype(np.uint64)
        assert (got < 2 * p).all()
        assert np.array_equal(got % p, o.encode(x).astype(np.uint64))


SCALAR = [(16, 40), (64, 100), (256, 434), (2048, 300), (1024, 1020), (16384, 434), (32768, 868)]


@pytest.mark.parametrize("N,W", SCALAR)
def test_encode_scalar_matches_oracle(N, W):
    """The CUDA-core encoder (L <= 32) leaves canonical residues equal to the
    oracle's, for canonical operands and for limbs at their 32-bit maximum, and
    whole products through it stay bit-exact."""
    pkg = package()
    q = pkg.inputs.modulus(W, 41)
    m, o = pkg.Multiplier(N, W, q), O.Oracle(N, W, q)
    m.set_tuning("encode_scalar", 1)
    assert m.get_tuning("encode_scalar") == 1
    L = len(q)
    ones = np.full((N, L), 0xFFFFFFFF, dtype=np.uint32)
    cases = [pkg.inputs.uniform(q, N, 12), pkg.inputs.fixture(q, N, "minus_one"), ones]
    pw = m.plane_words
    for x, y in ((cases[0], cases[1]), (cases[2], cases[0])):
        pa, pb = empty(pw), empty(pw)
        m.encode_device(dev(x), dev(y), pa, pb, pw, 1)
        m.synchronize()
        for z, planes in ((x, pa), (y, pb)):
            assert np.array_equal(host(planes).reshape(o.P, N), o.encode(z))
    # Three products per chain: the grid walks products and operands.
    a = np.stack([pkg.inputs.uniform(q, N, 90 + i) for i in range(3)])
    b = np.stack([pkg.inputs.fixture(q, N, "half_high"), pkg.inputs.uniform(q, N, 95),
                  pkg.inputs.fixture(q, N, "minus_one")])
    out = torch.zeros((3, N, L), dtype=torch.int32, device="cuda")
    m.multiply_device(dev(a), dev(b), out, 3)
    m.synchronize()
    for i in range(3):
        assert np.array_equal(host(out[i]), o.multiply(a[i], b[i])), i
    m.set_tuning("encode_scalar", 0)
    m.close()


def test_encode_scalar_rejects_wide_points():
    pkg = package()
    m, _, _ = setup(65536, 1747, 1)
    with pytest.raises(Exception, match="L <= 32"):
        m.set_tuning("encode_scalar", 1)
    assert m.get_tuning("encode_scalar") == 0


@pytest.mark.parametrize("N,W", SMALL + FULL)
def test_negacyclic_terms_match_oracle(N, W):
    pkg = package()
    m, o, q = setup(N, W, 2)
    a = pkg.inputs.uniform(q, N, 21)
    b = pkg.inputs.uniform(q, N, 22)
    ra, rb = o.encode(a), o.encode(b)
    pw = m.plane_words
    pa, pb = dev(ra.reshape(-1)), dev(rb.reshape(-1))
    m.negacyclic_device(pa, pb, pw, 1)
    m.synchronize()
    got = host(pa).reshape(o.P, N)
    primes, cinv = o.primes, o.crt_inverse
    for j in ([0, 1, o.P // 2, o.P - 1] if N >= 16384 else range(o.P)):
        want = o.prime_product(j, ra[j], rb[j]).astype(np.uint64) * int(cinv[j]) % int(primes[j])
        assert np.array_equal(got[j].astype(np.uint64), want), f"prime {j}"


@pytest.mark.parametrize("N,W", SMALL + FULL)
def test_crt_matches_oracle(N, W):
    pkg = package()
    m, o, q = setup(N, W, 3)
    a = pkg.inputs.uniform(q, N, 31)
    b = pkg.inputs.uniform(q, N, 32)
    ra, rb = o.encode(a), o.encode(b)
    prods = np.stack([o.prime_product(j, ra[j], rb[j]) for j in range(o.P)])
    terms = (prods.astype(np.uint64) * o.crt_inverse.astype(np.uint64)[:, None]
             % o.primes.astype(np.uint64)[:, None]).astype(np.uint32)
    c = empty(N * m.L)
    m.crt_device(dev(terms.reshape(-1)), m.plane_words, c, 1)
    m.synchronize()
    assert np.array_equal(host(c).reshape(N, m.L), o.crt(prods))


@pytest.mark.parametrize("N,W", SMALL + FULL)
def test_multiply_device_matches_oracle(N, W):
    pkg = package()
    m, o, q = setup(N, W, 4)
    a = pkg.inputs.uniform(q, N, 41)
    b = pkg.inputs.uniform(q, N, 42)
    c = empty(N * m.L)
    m.multiply_device(dev(a), dev(b), c, 1)
    m.synchronize()
    assert np.array_equal(host(c).reshape(N, m.L), o.multiply(a, b))


@pytest.mark.parametrize("kind_a,kind_b", [("zero", "random"), ("one", "random"), ("minus_one", "minus_one"),
                                           ("half_low", "half_high"), ("half_high", "half_high"),
                                           ("minus_one", "one")])
@pytest.mark.parametrize("N,W", [(1024, 868), (32768, 868), (65536, 1747)])
def test_edge_fixtures(N, W, kind_a, kind_b):
    pkg = package()
    m, o, q = setup(N, W, 5)
    pick = lambda kind, s: pkg.inputs.uniform(q, N, s) if kind == "random" else pkg.inputs.fixture(q, N, kind)
    a, b = pick(kind_a, 51), pick(kind_b, 52)
    got = m.multiply(a, b)
    assert np.array_equal(got, o.multiply(a, b))


@pytest.mark.parametrize("seed", [101, 102, 103])
def test_full_size_three_moduli(seed):
    """N=65536, W=1747 (L=55, P=114) with three seeded 1747-bit moduli."""
    pkg = package()
    N, W = 65536, 1747
    q = pkg.inputs.modulus(W, seed)
    m = pkg.Multiplier(N, W, q)
    o = O.Oracle(N, W, q)
    a, b = pkg.inputs.uniform(q, N, seed * 3), pkg.inputs.uniform(q, N, seed * 3 + 1)
    assert np.array_equal(m.multiply(a, b), o.multiply(a, b))
    m.close()


@pytest.mark.parametrize("gap", [1, 2 * 65536 - 1, (1 << 32) - 1])
def test_gap_form_moduli(gap):
    """The reference's own modulus form q = 2^W - gap at its main geometry."""
    pkg = package()
    N, W = 65536, 1747
    q = pkg.inputs.gap_modulus(W, gap)
    m = pkg.Multiplier(N, W, q)
    o = O.Oracle(N, W, q)
    a, b = pkg.inputs.uniform(q, N, gap % 1000), pkg.inputs.fixture(q, N, "minus_one")
    assert np.array_equal(m.multiply(a, b), o.multiply(a, b))
    m.close()


def test_batch_equals_single_products():
    pkg = package()
    N, W, B = 16384, 434, 7
    m, o, q = setup(N, W, 6)
    a = np.stack([pkg.inputs.uniform(q, N, 600 + i) for i in range(B)])
    b = np.stack([pkg.inputs.uniform(q, N, 700 + i) for i in range(B)])
    batched = m.multiply(a, b)
    for i in (0, 3, B - 1):
        assert np.array_equal(batched[i], m.multiply(a[i], b[i]))
        assert np.array_equal(batched[i], o.multiply(a[i], b[i]))


def test_repeated_calls_are_deterministic():
    pkg = package()
    N, W = 32768, 868
    m, o, q = setup(N, W, 7)
    a, b = pkg.inputs.uniform(q, N, 1), pkg.inputs.uniform(q, N, 2)
    first = m.multiply(a, b)
    for _ in range(3):
        assert np.array_equal(m.multiply(a, b), first)


def test_plugin_abi_roundtrip():
    pkg = package()
    N, W = 16384, 434
    q = pkg.inputs.modulus(W, 8)
    st = pkg.fherma_init(pkg.Point(N=N, W=W, L=14, q=q))
    a, b = pkg.inputs.uniform(q, N, 1), pkg.inputs.uniform(q, N, 2)
    out = pkg.fherma_run(st, pkg.Inputs(a=a, b=b))
    assert out.c.shape == (N, 14)
    assert np.array_equal(out.c, O.Oracle(N, W, q).multiply(a, b))
    with pytest.raises(RuntimeError):
        pkg.fherma_run(st, pkg.Inputs(a=a[:-1], b=b))
    pkg.fherma_free(st)


@pytest.mark.parametrize("N,W", [(16, 40), (64, 100), (2048, 300), (16384, 434), (32768, 868), (65536, 1747)])
def test_tuning_knobs_stay_bit_exact(N, W):
    """Every CRT kernel and tile shape and every row-pass kernel and CTA shape gives the oracle's product."""
    pkg = package()
    m, o, q = setup(N, W, 1)
    a = np.stack([pkg.inputs.uniform(q, N, 70 + i) for i in range(3)])
    b = np.stack([pkg.inputs.uniform(q, N, 80 + i) for i in range(3)])
    want = [o.multiply(a[i], b[i]) for i in range(3)]
    da, db = dev(a), dev(b)
    for persistent, tiles, rows, local, rpass in ((0, 1, 0, 3, 0), (0, 2, 8, 0, 1), (0, 1, 64, 3, 1),
                                                  (1, 2, 0, 0, 0), (1, 2, 64, 0, 1), (1, 2, 128, 3, 0),
                                                  (1, 2, 0, 3, 1), (1, 2, 16, 0, 1), (1, 2, 0, 0, 1)):
        m.set_tuning("crt_persistent", persistent)
        m.set_tuning("crt_tiles", tiles)
        m.set_tuning("row_rows", rows)
        m.set_tuning("row_local", local)
        m.set_tuning("row_pass", rpass)
        for rep in range(2):
            out = torch.zeros_like(da)
            m.multiply_device(da, db, out, 3)
            m.synchronize()
            for i in range(3):
                assert np.array_equal(host(out[i]), want[i]), (persistent, tiles, rows, local, rpass, rep, i)
    # One product per chain through the sliced row pass.
    m.set_tuning("row_pass", 1)
    out = torch.zeros_like(da[:1])
    m.multiply_device(da[:1], db[:1], out, 1)
    m.synchronize()
    assert np.array_equal(host(out[0]), want[0])
    m.set_tuning("crt_persistent", 1)
    m.set_tuning("crt_tiles", 2)
    m.set_tuning("row_rows", 0)
    m.set_tuning("row_local", 0)
    m.set_tuning("row_pass", 0)


@pytest.mark.parametrize("N,W", [(1024, 200), (4096, 868), (32768, 868)])
def test_radix_splits_stay_bit_exact(N, W):
    """Every valid split N = C * 2^row_bits gives the oracle's product."""
    pkg = package()
    q = pkg.inputs.modulus(W, 21)
    o = O.Oracle(N, W, q)
    a, b = pkg.inputs.uniform(q, N, 1), pkg.inputs.uniform(q, N, 2)
    want = o.multiply(a, b)
    m = pkg.Multiplier(N, W, q)
    n_bits = N.bit_length() - 1
    tried = 0
    for rb in range(max(4, n_bits - 8), min(8, n_bits) + 1):
        if N >> rb > 1 and rb < 5:
            continue
        m.set_tuning("row_bits", rb)
        assert m.get_tuning("row_bits") == rb
        for rpass in (0, 1):                     # both row passes
            m.set_tuning("row_pass", rpass)
            out = torch.zeros((1, N, len(q)), dtype=torch.int32, device="cuda")
            m.multiply_device(dev(a[None]), dev(b[None]), out, 1)
            m.synchronize()
            assert np.array_equal(host(out[0]), want), (rb, rpass)
        tried += 1
    assert tried >= 2
    m.close()


def test_autotune_applies_and_is_remembered():
    pkg = package()
    N, W = 16384, 434
    q = pkg.inputs.modulus(W, 31)
    m = pkg.Multiplier(N, W, q)
    r = m.autotune(max_group=8)
    assert r["candidates"] >= 5
    assert 0 < r["us_per_product_tuned"] <= r["us_per_product_default"] * 1.05
    assert r["crt_tiles"] in (1, 2) and 1 <= r["group"] <= 8
    for knob in ("group", "crt_tiles", "crt_persistent", "row_rows", "row_local", "row_bits", "row_pass",
                 "encode_scalar"):
        assert m.get_tuning(knob) == r[knob], knob
    a, b = pkg.inputs.uniform(q, N, 3), pkg.inputs.uniform(q, N, 4)
    assert np.array_equal(m.multiply(a, b), O.Oracle(N, W, q).multiply(a, b))
    # Another context of the same geometry (another q) starts from the tuned shapes.
    q2 = pkg.inputs.modulus(W, 32)
    m2 = pkg.Multiplier(N, W, q2)
    for knob in ("group", "crt_tiles", "crt_persistent", "row_rows", "row_local", "row_bits", "row_pass",
                 "encode_scalar"):
        assert m2.get_tuning(knob) == r[knob], knob
    a2, b2 = pkg.inputs.uniform(q2, N, 5), pkg.inputs.uniform(q2, N, 6)
    assert np.array_equal(m2.multiply(a2, b2), O.Oracle(N, W, q2).multiply(a2, b2))
    m.close()
    m2.close()


@pytest.mark.parametrize("N,W,gap", [(1024, 71, 1), (1024, 96, 5), (2048, 128, (1 << 32) - 1), (4096, 868, 65537),
                                     (16384, 434, 3), (65536, 1747, 1)])
def test_gap_form_fold_matches_generic_and_oracle(N, W, gap):
    """q = 2^W - gap reduces by two folds (the reference's form); the generic
    reduction gives the same bits, and both equal the oracle, on random and
    edge operands."""
    pkg = package()
    q = pkg.inputs.gap_modulus(W, gap)
    m = pkg.Multiplier(N, W, q)
    assert m.get_tuning("gap") == gap
    o = O.Oracle(N, W, q)
    cases = [(pkg.inputs.uniform(q, N, 1), pkg.inputs.uniform(q, N, 2)),
             (pkg.inputs.fixture(q, N, "minus_one"), pkg.inputs.fixture(q, N, "minus_one")),
             (pkg.inputs.fixture(q, N, "half_high"), pkg.inputs.fixture(q, N, "minus_one")),
             (pkg.inputs.fixture(q, N, "one"), pkg.inputs.uniform(q, N, 3))]
    a = np.stack([c[0] for c in cases])
    b = np.stack([c[1] for c in cases])
    want = [o.multiply(a[i], b[i]) for i in range(len(cases))]
    for fold in (1, 0):
        m.set_tuning("crt_gap_fold", fold)
        out = torch.zeros((len(cases), N, len(q)), dtype=torch.int32, device="cuda")
        m.multiply_device(dev(a), dev(b), out, len(cases))
        m.synchronize()
        for i in range(len(cases)):
            assert np.array_equal(host(out[i]), want[i]), (fold, i)
    m.close()


def test_generic_modulus_has_no_gap():
    pkg = package()
    q = pkg.inputs.modulus(868, 7)
    m = pkg.Multiplier(4096, 868, q)
    assert m.get_tuning("gap") == 0
    m.close()
