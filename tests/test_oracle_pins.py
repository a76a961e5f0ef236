"""Pins the CPU oracle (oracle/oracle.c) to the reference's own artefacts.

Every fixture here was produced from the reference checkout by
tests/golden/make_golden.py: the reference's compiled host plan
(native-smoke/rns-plan.hpp), its Python model (reference.py) and its
G1 golden files (native-smoke/fixtures/g1-*.bin).
"""
import hashlib

import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O


def _q(words):
    return np.array(words, dtype=np.uint32)


@pytest.mark.parametrize("case", golden("ref_plans.json"), ids=lambda c: f"N{c['N']}-gap{c['gap']}")
def test_plan_matches_reference_compiled_plan(case):
    o = O.Oracle(case["N"], case["W"], _q(case["q"]))
    assert o.P == case["P"] and o.kpad == case["kpad"]
    assert o.primes.tolist() == case["primes"]
    assert o.psi.tolist() == case["psi"]
    assert o.crt_inverse.tolist() == case["crt_inverse"]
    b4 = o.b4().tobytes()
    assert len(b4) == case["b4_len"]
    assert hashlib.sha256(b4).hexdigest() == case["b4_sha256"]


@pytest.mark.parametrize("case", golden("pyref_plans.json"), ids=lambda c: f"N{c['N']}-W{c['W']}")
def test_plan_matches_reference_python_plan_generic_q(case):
    o = O.Oracle(case["N"], case["W"], _q(case["q"]))
    assert o.primes.tolist() == case["primes"]
    assert o.crt_inverse.tolist() == case["crt_inverse"]
    assert o.product_bits == case["product_bits"]
    w = o.weights
    assert hashlib.sha256(w.tobytes()).hexdigest() == case["weights_sha256"]
    assert w[0].tolist() == case["weights_first"]
    assert w[-1].tolist() == case["weights_alpha"]


def test_known_geometries():
    # native-smoke/README.md table and reference-result.json: P and CRT inner axis.
    for N, W, P, K in ((65536, 1747, 114, 480), (32768, 868, 57, 256), (16384, 434, 29, 128)):
        q = np.zeros((W + 31) // 32, dtype=np.uint32)
        q[0] = 1
        q[-1] = 1 << ((W - 1) % 32)
        o = O.Oracle(N, W, q)
        assert (o.P, o.kpad) == (P, K)


_CRT = golden("crt_fixtures.json")
_plans = {}


def _plan(N, W, q):
    key = (N, W, tuple(q))
    if key not in _plans:
        _plans[key] = O.Oracle(N, W, _q(q))
    return _plans[key]


@pytest.mark.parametrize("i", range(len(_CRT)))
def test_crt_matches_reference_py_fixtures(i):
    case = _CRT[i]
    o = _plan(case["N"], case["W"], case["q"])
    alpha, wide, reduced = o.crt_terms(case["terms"])
    assert alpha == case["alpha"]
    assert wide.tolist() == case["wide"]
    assert reduced.tolist() == case["reduced"]


@pytest.mark.parametrize("case", golden("g1_vectors.json"), ids=lambda c: f"N{c['N']}-gap{c['gap']}")
def test_crt_matches_reference_g1_golden_files(case):
    o = _plan(case["N"], case["W"], case["q"])
    assert o.P == case["P"] and o.kpad == case["kpad"]
    for row in case["rows"]:
        _, _, reduced = o.crt_terms(row["terms"])
        assert reduced.tolist() == row["golden"]


def _dense_input(n, p, operand):
    """native-smoke/ntt-smoke.cu:65-84 restated (splitmix finaliser per index)."""
    M = (1 << 64) - 1

    def mix(x):
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & M
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & M
        return x ^ (x >> 31)
    a = []
    for i in range(n):
        seed = ((p << 32) ^ n ^ ((0x9E3779B97F4A7C15 * (i + 1 + operand * n)) & M)) & M
        a.append(mix(seed) % p)
    a[0] = p - 1 if operand else 0
    a[1] = 1 if operand else p - 1
    a[n // 2] = p // 2
    a[n - 1] = p - 1 if operand else 1
    return a


def test_prime_product_matches_schoolbook_ntt_smoke_inputs():
    # ntt-smoke.cu:131-147: the CPU NTT product is pinned by an N=16 schoolbook
    # for the first two primes of the plan.
    n = 16
    q = np.zeros(2, dtype=np.uint32)
    q[0] = 1
    q[1] = 1 << 7          # W = 40
    o = O.Oracle(n, 40, q)
    for j in range(2):
        p = int(o.primes[j])
        a, b = _dense_input(n, p, 0), _dense_input(n, p, 1)
        school = [0] * n
        for x in range(n):
            for y in range(n):
                k = (x + y) % n
                v = a[x] * b[y] % p
                school[k] = (school[k] + (v if x + y < n else p - v)) % p
        got = o.prime_product(j, np.array(a, np.uint32), np.array(b, np.uint32))
        assert got.tolist() == school


def test_mont_mul_word():
    # native-smoke/rns-encode.cuh:15-22: a*b*2^-32 mod p.
    p = 2147352577
    n_dash = (-pow(p, -1, 1 << 32)) % (1 << 32)
    for a, b in ((0, 5), (1, 1), (p - 1, p - 1), (0xFFFFFFFF, p - 2), (123456789, 987654321)):
        want = a * b * pow(1 << 32, -1, p) % p
        assert O.lib().orc_mont_mul_word(a, b, p, n_dash) == want


def test_encode_matches_bigint_mod():
    from conftest import package
    inp = package().inputs
    for N, W in ((16, 40), (64, 868)):
        q = inp.modulus(W, 3)
        o = O.Oracle(N, W, q)
        x = inp.uniform(q, N, 5)
        res = o.encode(x)
        vals = O.coeffs_to_ints(x)
        for j, p in enumerate(o.primes.tolist()):
            assert res[j].tolist() == [v % p for v in vals]


@pytest.mark.parametrize("N,W", [(16, 40), (64, 100), (256, 434), (512, 868)])
def test_oracle_product_matches_schoolbook(N, W):
    from conftest import package
    inp = package().inputs
    q = inp.modulus(W, N + W)
    a, b = inp.uniform(q, N, 1), inp.uniform(q, N, 2)
    o = O.Oracle(N, W, q)
    assert np.array_equal(o.multiply(a, b), O.schoolbook(a, b, inp.q_int(q)))


@pytest.mark.parametrize("kind", ["zero", "one", "minus_one", "half_low", "half_high"])
def test_oracle_edge_fixtures_match_kronecker(kind):
    from conftest import package
    inp = package().inputs
    if O.gmp() is None:
        pytest.skip("libgmp not present")
    N, W = 1024, 868
    q = inp.modulus(W, 9)
    a = inp.fixture(q, N, kind)
    b = inp.fixture(q, N, "minus_one") if kind != "zero" else inp.uniform(q, N, 4)
    o = O.Oracle(N, W, q)
    assert np.array_equal(o.multiply(a, b), O.kronecker(a, b, inp.q_int(q)))


@pytest.mark.slow
def test_oracle_full_size_matches_kronecker():
    from conftest import package
    inp = package().inputs
    if O.gmp() is None:
        pytest.skip("libgmp not present")
    N, W = 32768, 868
    q = inp.modulus(W, 21)
    a, b = inp.uniform(q, N, 1), inp.uniform(q, N, 2)
    o = O.Oracle(N, W, q)
    assert np.array_equal(o.multiply(a, b), O.kronecker(a, b, inp.q_int(q)))
