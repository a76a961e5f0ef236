"""Served form through the C ABI (bcg_server_*): continuous batching of
products of different points, resident operands with cached forward-NTT
residues, admission by a device-memory budget.  Every response is bit-exact
and identical to the same product run alone."""
import threading

import numpy as np
import pytest

from conftest import package
from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

POINTS = [(16384, 434, 11), (4096, 868, 12), (1024, 200, 13)]


def alone(pkg, N, W, q, a, b):
    m = pkg.Multiplier(N, W, q)
    out = m.multiply(a, b)
    m.close()
    return out


def test_mixed_requests_identical_alone_and_in_the_mix():
    pkg = package()
    rng = np.random.default_rng(5)
    srv = pkg.Server(slots=3)
    pts = []
    for N, W, seed in POINTS:
        q = pkg.inputs.modulus(W, seed)
        pid = srv.add_point(N, W, q)
        a_res = pkg.inputs.uniform(q, N, seed * 7)
        oid = srv.add_operand(pid, a_res)
        pts.append((N, W, q, pid, a_res, oid))
    reqs = []
    for i in range(72):
        N, W, q, pid, a_res, oid = pts[rng.integers(len(pts))]
        resident = bool(rng.integers(2))
        a = a_res if resident else pkg.inputs.uniform(q, N, 1000 + i)
        b = pkg.inputs.uniform(q, N, 5000 + i)
        c = np.zeros_like(b)
        reqs.append(dict(N=N, W=W, q=q, pid=pid, a=a, b=b, c=c, oid=oid if resident else 0))
    # Two submitting threads, so arrivals interleave with running batches.
    ids = [None] * len(reqs)

    def submit(part):
        for i in part:
            r = reqs[i]
            ids[i] = srv.submit(r["pid"], r["b"], r["c"], a=None if r["oid"] else r["a"], operand=r["oid"])

    threads = [threading.Thread(target=submit, args=(range(k, len(reqs), 2),)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    lat = [srv.wait(i) for i in ids]
    assert all(x > 0 for x in lat)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batched_products"] == len(reqs) and 1 <= st["batches"] <= len(reqs)
    assert st["memory_peak"] <= st["memory_budget"]
    for r in reqs:
        assert np.array_equal(r["c"], alone(pkg, r["N"], r["W"], r["q"], r["a"], r["b"]))
    # The small point against the oracle as well.
    r = next(r for r in reqs if r["N"] == 1024)
    assert np.array_equal(r["c"], O.Oracle(r["N"], r["W"], r["q"]).multiply(r["a"], r["b"]))
    srv.close()


def test_budget_refuses_a_product_that_cannot_fit():
    pkg = package()
    srv = pkg.Server(memory_bytes=1 << 20)
    q = pkg.inputs.modulus(434, 1)
    pid = srv.add_point(16384, 434, q)
    b = pkg.inputs.uniform(q, 16384, 2)
    with pytest.raises(pkg.BcgError) as e:
        srv.submit(pid, b, np.zeros_like(b), a=b)
    assert e.value.code == pkg.BCG_ERR_BUSY
    assert srv.stats()["rejected"] == 1
    srv.close()


def test_operand_lifecycle_and_errors():
    pkg = package()
    srv = pkg.Server()
    N, W = 2048, 300
    q = pkg.inputs.modulus(W, 3)
    pid = srv.add_point(N, W, q)
    a = pkg.inputs.uniform(q, N, 1)
    b = pkg.inputs.uniform(q, N, 2)
    oid = srv.add_operand(pid, a)
    c = np.zeros_like(b)
    srv.wait(srv.submit(pid, b, c, operand=oid))
    assert np.array_equal(c, alone(pkg, N, W, q, a, b))
    assert srv.stats()["operands"] == 1
    srv.remove_operand(oid)
    assert srv.stats()["operands"] == 0
    with pytest.raises(pkg.BcgError) as e:
        srv.submit(pid, b, c, operand=oid)
    assert e.value.code == pkg.BCG_ERR_INVALID
    with pytest.raises(pkg.BcgError):
        srv.submit(pid + 5, b, c, a=a)
    with pytest.raises(pkg.BcgError):
        srv.wait(123456)
    srv.close()


def test_close_finishes_pending_requests():
    pkg = package()
    srv = pkg.Server(slots=1)
    N, W = 16384, 868
    q = pkg.inputs.modulus(W, 4)
    pid = srv.add_point(N, W, q)
    a = pkg.inputs.uniform(q, N, 1)
    b = pkg.inputs.uniform(q, N, 2)
    outs = [np.zeros_like(b) for _ in range(6)]
    for c in outs:
        srv.submit(pid, b, c, a=a)
    srv.close()   # drains: every submitted product completes
    want = alone(pkg, N, W, q, a, b)
    for c in outs:
        assert np.array_equal(c, want)


def test_config5_geometries_identical_alone_and_in_the_mix():
    """The served workload's three points (N=16384/W=434, 32768/868,
    65536/1747), about 30 mixed requests from two threads, half of them with a
    resident left operand: every response equals the same product run alone,
    and one response per geometry equals the oracle's product."""
    pkg = package()
    rng = np.random.default_rng(55)
    srv = pkg.Server(slots=3)
    pts = []
    for k, (N, W) in enumerate(((16384, 434), (32768, 868), (65536, 1747))):
        q = pkg.inputs.modulus(W, 60 + k)
        pid = srv.add_point(N, W, q)
        a_res = pkg.inputs.uniform(q, N, 600 + k)
        oid = srv.add_operand(pid, a_res)
        pts.append(dict(N=N, W=W, q=q, pid=pid, a_res=a_res, oid=oid, m=pkg.Multiplier(N, W, q)))
    reqs = []
    for i in range(30):
        p = pts[i % 3] if i < 3 else pts[int(rng.integers(3))]
        resident = bool(i % 2)
        a = p["a_res"] if resident else pkg.inputs.uniform(p["q"], p["N"], 7000 + i)
        b = pkg.inputs.uniform(p["q"], p["N"], 8000 + i)
        reqs.append(dict(p=p, a=a, b=b, c=np.zeros_like(b), oid=p["oid"] if resident else 0))
    ids = [None] * len(reqs)

    def submit(part):
        for i in part:
            r = reqs[i]
            ids[i] = srv.submit(r["p"]["pid"], r["b"], r["c"], a=None if r["oid"] else r["a"], operand=r["oid"])

    threads = [threading.Thread(target=submit, args=(range(k, len(reqs), 2),)) for k in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i in ids:
        srv.wait(i)
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    for r in reqs:
        assert np.array_equal(r["c"], r["p"]["m"].multiply(r["a"], r["b"])), (r["p"]["N"], bool(r["oid"]))
    for p in pts:
        r = next(r for r in reqs if r["p"] is p)
        assert np.array_equal(r["c"], O.Oracle(p["N"], p["W"], p["q"]).multiply(r["a"], r["b"])), p["N"]
        p["m"].close()
    srv.close()
