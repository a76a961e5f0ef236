"""Seeded randomized parity: random points (N, W), generic and gap-form
moduli, random kernel shapes, and operands mixing uniform values with edge
patterns.  Every product is compared bit for bit with the oracle."""
import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CASES = 40


def _point(rng):
    n_bits = int(rng.integers(4, 15))                  # N = 16 .. 16384 (oracle-friendly sizes)
    N = 1 << n_bits
    W = int(rng.integers(20, 1200))
    return N, W


def _modulus(pkg, rng, W):
    if W > 70 and rng.random() < 0.4:
        gap = int(rng.integers(1, 1 << 32)) | 1
        return pkg.inputs.gap_modulus(W, gap)
    return pkg.inputs.modulus(W, int(rng.integers(1, 1 << 30)))


def _operand(pkg, rng, q, N):
    kind = rng.random()
    if kind < 0.6:
        return pkg.inputs.uniform(q, N, int(rng.integers(1, 1 << 30)))
    if kind < 0.8:
        return pkg.inputs.fixture(q, N, ["zero", "one", "minus_one", "half_low", "half_high"][int(rng.integers(5))])
    # Mix: random rows replaced by edge values.
    x = pkg.inputs.uniform(q, N, int(rng.integers(1, 1 << 30)))
    e = pkg.inputs.fixture(q, N, ["minus_one", "half_high"][int(rng.integers(2))])
    rows = rng.random(N) < 0.3
    x[rows] = e[rows]
    return x


@pytest.mark.parametrize("case", range(CASES))
def test_random_points_bit_exact(case):
    pkg = package()
    rng = np.random.default_rng(1000 + case)
    N, W = _point(rng)
    q = _modulus(pkg, rng, W)
    m = pkg.Multiplier(N, W, q)
    n_bits = N.bit_length() - 1
    knobs = {"crt_persistent": int(rng.integers(2)), "crt_tiles": int(rng.integers(1, 3)),
             "row_rows": int(rng.choice([0, 8, 64])), "crt_gap_fold": int(rng.integers(2)),
             "row_local": int(rng.choice([0, 3])), "row_pass": int(rng.integers(2)),
             "encode_scalar": int(rng.integers(2)) if len(q) <= 32 else 0}
    splits = [rb for rb in range(max(4, n_bits - 8), min(8, n_bits) + 1) if not (N >> rb > 1 and rb < 5)]
    knobs["row_bits"] = int(rng.choice(splits))
    for k, v in knobs.items():
        m.set_tuning(k, v)
    count = int(rng.integers(1, 4))
    a = np.stack([_operand(pkg, rng, q, N) for _ in range(count)])
    b = np.stack([_operand(pkg, rng, q, N) for _ in range(count)])
    o = O.Oracle(N, W, q)
    out = torch.zeros((count, N, len(q)), dtype=torch.int32, device="cuda")
    m.multiply_device(torch.from_numpy(a.view(np.int32)).cuda(), torch.from_numpy(b.view(np.int32)).cuda(), out, count)
    m.synchronize()
    got = out.cpu().numpy().view(np.uint32)
    for i in range(count):
        assert np.array_equal(got[i], o.multiply(a[i], b[i])), (N, W, knobs, i)
    m.close()
