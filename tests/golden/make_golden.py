#!/usr/bin/env python3
"""Regenerate the committed golden vectors from the reference checkout.

Runs only in a container that has the reference checkout, named by the
REFERENCE_ROOT environment variable.  It reads the reference's own artefacts and
writes compact fixtures under tests/golden/, which the tests then use on any
machine (the reference itself does not travel):

* ref_plans.json     — bytecrt::make_rns_plan (native-smoke/rns-plan.hpp:174-324)
                       compiled here by oracle/build_ref.sh and run for
                       q = 2^W - gap at both reference geometries.
* pyref_plans.json   — reference.py plan() (reference.py:39-54) for generic odd
                       q at several (N, W), including N=16384/W=434.
* crt_fixtures.json  — reference.py's signed CRT fixtures {0, 1, -1, +-N(q-1)^2,
                       seeded random} (reference.py:98-123): terms t_j, alpha,
                       the B4 wide value (byte_matrices + epilogue, computed
                       here with reference.py's own functions on B4 columns),
                       and x mod q.
* g1_vectors.json    — the terms (A rows) and golden x mod q of the six
                       native-smoke/fixtures/g1-*.bin files (format of
                       native-smoke/make_g1_fixtures.py:5-6).
"""
from __future__ import annotations

import hashlib
import json
import os
import random
import struct
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("REFERENCE_ROOT", "")
if not os.path.isdir(REF):
    sys.exit("set REFERENCE_ROOT to the reference checkout")


def words(v: int, n: int):
    return [(v >> (32 * i)) & 0xFFFFFFFF for i in range(n)]


def sha(data: bytes) -> str:
    return hashlib.sha256(data).hexdigest()


def ref_plans():
    exe = subprocess.run(["sh", os.path.join(REPO, "oracle", "build_ref.sh")],
                         check=True, capture_output=True, text=True).stdout.strip()
    out = []
    for n, w in ((65536, 1747), (32768, 868)):
        for gap in (1, 2 * n - 1, 2 * n * 124 - 1, (1 << 32) - 1):
            d = json.loads(subprocess.run([exe, str(n), str(w), str(gap)], check=True,
                                          capture_output=True, text=True).stdout)
            b4 = bytes(d.pop("b4"))
            d["b4_sha256"] = sha(b4)
            d["b4_len"] = len(b4)
            out.append(d)
    return out


def seeded_q(w: int, seed: int) -> int:
    rng = random.Random(seed)
    return rng.getrandbits(w) | (1 << (w - 1)) | 1


def pyref_plans(reference):
    out = []
    for n, w, seed in ((16, 40, 1), (64, 100, 2), (256, 434, 3), (1024, 868, 4),
                       (16384, 434, 5), (32768, 868, 6), (65536, 1747, 7)):
        q = seeded_q(w, seed)
        product, primes, bases, inverses, weights = reference.plan(n, w, q)
        limbs = (w + 31) // 32
        wbytes = b"".join(struct.pack(f"<{limbs}I", *words(x, limbs)) for x in weights)
        out.append(dict(N=n, W=w, L=limbs, q=words(q, limbs), primes=primes,
                        crt_inverse=inverses, product_bits=product.bit_length(),
                        weights_sha256=sha(wbytes), weights_first=words(weights[0], limbs),
                        weights_alpha=words(weights[-1], limbs)))
    return out


def b4_columns(weights, limbs, q):
    """B4 columns W[j,a] = (256^a * weight_j) mod q (native-smoke/README.md, four-column CRT)."""
    cols = []
    for l in range(limbs):
        for d in range(4):
            col = []
            for wj in weights:
                for a in range(4):
                    word = ((wj * pow(256, a, q)) % q) >> (32 * l) & 0xFFFFFFFF
                    col.append(word >> (8 * d) & 255)
            cols.append(col)
    return cols


def crt_fixtures(reference):
    out = []
    cases = [(65536, 1747, "gap", g) for g in (1, 2 * 65536 - 1, 2 * 65536 * 124 - 1)]
    cases += [(32768, 868, "gap", g) for g in (1, 2 * 32768 - 1, 2 * 32768 * 124 - 1)]
    cases += [(16384, 434, "seed", 11), (32768, 868, "seed", 12), (65536, 1747, "seed", 13)]
    for n, w, kind, arg in cases:
        q = (1 << w) - arg if kind == "gap" else seeded_q(w, arg)
        limbs = (w + 31) // 32
        product, primes, bases, inverses, weights = reference.plan(n, w, q)
        bound = n * (q - 1) ** 2
        rng = random.Random(n + w + arg)
        cols = b4_columns(weights, limbs, q)
        for x in (0, 1, -1, bound, -bound, rng.randrange(-bound, bound + 1)):
            terms = [x % p * inv % p for p, inv in zip(primes, inverses)]
            approx = 0.0
            for t, p in zip(terms, primes):
                approx += float(t) * (1.0 / float(p))
            alpha = int(approx + 0.5)
            assert sum(t * b for t, b in zip(terms, bases)) - alpha * product == x
            a = [v >> (8 * d) & 255 for v in terms + [alpha] for d in range(4)]
            c = [sum(u * v for u, v in zip(a, col)) for col in cols]
            # reference.py's epilogue over 7-digit groups; B4 has 4 digits per limb,
            # so restate its carry on groups of four (g1-crt.cuh:304-318).
            value, carry = 0, 0
            for l in range(limbs):
                lo = sum(c[4 * l + d] << (8 * d) for d in range(4))
                total = carry + lo
                value |= (total & 0xFFFFFFFF) << (32 * l)
                carry = total >> 32
            wide = value | carry << (32 * limbs)
            assert wide % q == x % q
            out.append(dict(N=n, W=w, L=limbs, q=words(q, limbs), x_sign=(x > 0) - (x < 0),
                            terms=terms, alpha=alpha, wide=words(wide, limbs + 2),
                            reduced=words(x % q, limbs)))
    return out


def g1_vectors():
    out = []
    for n, w, gap in ((65536, 1747, 1), (65536, 1747, 131071), (65536, 1747, (1 << 32) - 1),
                      (32768, 868, 1), (32768, 868, 65535), (32768, 868, (1 << 32) - 1)):
        path = os.path.join(REF, "native-smoke", "fixtures", f"g1-n{n}-w{w}-g{gap}.bin")
        blob = open(path, "rb").read()
        assert blob[:8] == b"BCRT01\0\0"
        fn, fw, limbs, p, kpad, m, nc, fgap = struct.unpack("<8I", blob[8:40])
        assert (fn, fw, fgap) == (n, w, gap)
        off = 40
        q = list(struct.unpack(f"<{limbs}I", blob[off:off + 4 * limbs])); off += 4 * limbs
        off += 8 * p                      # fp64 1/p_j
        off += kpad * nc                  # B7 columns (the fixture path's matrix)
        a = blob[off:off + m * kpad]; off += m * kpad
        golden = list(struct.unpack(f"<{m * limbs}I", blob[off:off + 4 * m * limbs]))
        rows = []
        for r in range(m):
            row = a[r * kpad:(r + 1) * kpad]
            terms = list(struct.unpack(f"<{p}I", row[:4 * p]))
            rows.append(dict(terms=terms, golden=golden[r * limbs:(r + 1) * limbs]))
        out.append(dict(N=n, W=w, L=limbs, gap=gap, P=p, kpad=kpad, q=q, rows=rows))
    return out


def main():
    sys.path.insert(0, REF)
    import reference  # noqa: E402  (the reference's CPU model, reference.py)
    fixtures = {
        "ref_plans.json": ref_plans(),
        "pyref_plans.json": pyref_plans(reference),
        "crt_fixtures.json": crt_fixtures(reference),
        "g1_vectors.json": g1_vectors(),
    }
    for name, data in fixtures.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(data, f, separators=(",", ":"))
        print(name, os.path.getsize(os.path.join(HERE, name)), "bytes")


if __name__ == "__main__":
    main()
