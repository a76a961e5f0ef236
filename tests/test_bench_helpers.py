"""CPU checks of the arithmetic behind bench.py's JSON line: the host-link
bound that `e2e.link_frac` is measured against, and the per-stage
algorithmic bytes and rates the rooflines are computed from."""
import os
import sys
from types import SimpleNamespace

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

IN_BYTES = 2 * 65536 * 55 * 4      # two operands per product at N=65536, L=55
OUT_BYTES = 65536 * 55 * 4


def link(h2d, d2h, both):
    return {"h2d_gbs": h2d, "d2h_gbs": d2h, "both_gbs": both, "method": "test"}


def test_link_bound_is_the_slowest_capacity():
    l = link(211.7, 193.6, 343.4)
    t = max(IN_BYTES / 211.7e9, OUT_BYTES / 193.6e9, (IN_BYTES + OUT_BYTES) / 343.4e9)
    assert bench.link_bound(l, IN_BYTES, OUT_BYTES) == pytest.approx(1.0 / t)
    assert bench.link_bound(l, IN_BYTES, OUT_BYTES) == pytest.approx(7341.6, rel=1e-3)   # H2D alone binds
    # A slow two-way rate binds instead.
    assert bench.link_bound(link(211.7, 193.6, 250.0), IN_BYTES, OUT_BYTES) == \
        pytest.approx(250.0e9 / (IN_BYTES + OUT_BYTES))


def test_link_bound_is_an_upper_bound_of_the_even_split_model():
    for h2d, d2h, both in ((211.7, 193.6, 343.4), (108.0, 100.0, 150.0), (50.0, 400.0, 420.0), (200.0, 100.0, 300.0)):
        l = link(h2d, d2h, both)
        for nin, nout in ((IN_BYTES, OUT_BYTES), (1_000_000, 2_000_000)):
            bound = bench.link_bound(l, nin, nout)
            assert bound <= h2d * 1e9 / nin * (1 + 1e-12)
            assert bound <= d2h * 1e9 / nout * (1 + 1e-12)
            assert bound <= both * 1e9 / (nin + nout) * (1 + 1e-12)
            if both / 2 <= min(h2d, d2h):       # the model's shared phase is within both one-way rates
                assert bench.link_model_even_split(l, nin, nout) <= bound * (1 + 1e-12)


def test_even_split_model():
    l = link(211.7, 193.6, 343.4)
    t = OUT_BYTES / (343.4e9 / 2) + (IN_BYTES - OUT_BYTES) / 211.7e9
    assert bench.link_model_even_split(l, IN_BYTES, OUT_BYTES) == pytest.approx(1.0 / t)
    assert bench.link_model_even_split(l, IN_BYTES, OUT_BYTES) == pytest.approx(6575.6, rel=1e-3)
    # More bytes out than in: the remainder runs at the D2H rate.
    l2 = link(200.0, 100.0, 300.0)
    assert bench.link_model_even_split(l2, 1_000_000, 2_000_000) == pytest.approx(1.0 / (1e6 / 150e9 + 1e6 / 100e9))


def test_best_link_takes_the_higher_rate_per_direction():
    a = link(200.0, 195.0, 330.0)
    b = link(211.0, 180.0, 343.0)
    best = bench.best_link(a, b)
    assert (best["h2d_gbs"], best["d2h_gbs"], best["both_gbs"]) == (211.0, 195.0, 343.0)
    assert bench.link_bound(best, IN_BYTES, OUT_BYTES) >= max(bench.link_bound(a, IN_BYTES, OUT_BYTES),
                                                               bench.link_bound(b, IN_BYTES, OUT_BYTES))
    assert "before" in best["method"] and "after" in best["method"]


def test_algorithmic_bytes_per_stage():
    info = SimpleNamespace(P=114, L=55)
    alg = bench.algorithmic(info)
    plane, io = 4 * 114 * bench.N, 4 * bench.N * 55
    assert alg == {"encode": 2 * io + 2 * plane, "column": 4 * plane, "row": 3 * plane,
                   "column_inverse": 2 * plane, "crt": plane + io}
    # The whole chain moves about 402 MB per product at N=65536, W=1747.
    assert sum(alg.values()) / 1e6 == pytest.approx(402.0, abs=1.0)


def test_rooflines_fractions_follow_from_stage_times(monkeypatch):
    info = SimpleNamespace(P=114, L=55, enc_k=224, enc_cols=456, crt_k=480, crt_n=224)
    monkeypatch.setattr(bench, "load_peaks", lambda: (6787.2, "measured"))
    monkeypatch.setattr(bench, "load_tensor_peak", lambda: (1715.7, "measured (sustained)"))
    monkeypatch.setattr(bench, "load_traffic", lambda: {"warp_instructions_per_product": {"row": 33.3e6}})
    stage_us = {"encode": 30.6, "column": 25.8, "row": 39.4, "column_inverse": 14.6, "crt": 18.4}
    r = bench.rooflines(info, stage_us, 152, 2070.0)
    alg = bench.algorithmic(info)
    row = r["stages"]["row"]
    assert row["hbm_gbs"] == pytest.approx(alg["row"] / 39.4e-6 / 1e9)
    assert row["hbm_frac"] == pytest.approx(row["hbm_gbs"] / 6787.2)
    assert row["issue_frac"] == pytest.approx(33.3e6 * 32 / 39.4e-6 / (152 * 4 * 32 * 2070e6))
    assert "issue_frac" not in r["stages"]["column"]      # no instruction count given for it
    enc = r["stages"]["encode"]
    assert enc["tensor_tflops"] == pytest.approx(2.0 * 2 * bench.N * 224 * 456 / 30.6e-6 / 1e12)
    assert r["whole_chain"]["us_per_product"] == pytest.approx(sum(stage_us.values()))
