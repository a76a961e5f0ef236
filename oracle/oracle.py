"""ORACLE — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module, and only as the checker; the product never does.

Three independent CPU references for c = a*b mod (X^N+1) mod q:

* ``Oracle``: ctypes binding of oracle/oracle.c, the C restatement of the
  reference's RNS pipeline (plan native-smoke/rns-plan.hpp:174-324, byte-power
  encode native-smoke/rns-encode-mma.cuh:15-52, per-prime NTT product
  native-smoke/ntt-smoke.cu:86-129, FP32-alpha B4 CRT native-smoke/g1-crt.cuh:
  201-335 with a generic mod-q).  Multithreaded with OpenMP.
* ``schoolbook``: Python big integers, O(N^2) — small N only.
* ``kronecker``: Kronecker substitution with libgmp's mpz_mul through ctypes
  (where libgmp.so.10 exists), fully independent of RNS/NTT.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_u32p = ctypes.POINTER(ctypes.c_uint32)


def build(force: bool = False) -> str:
    """Compile oracle/oracle.c into oracle/liboracle.so with gcc."""
    src = os.path.join(HERE, "oracle.c")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
           "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_plan_create.restype = ctypes.c_void_p
        L.orc_plan_create.argtypes = [ctypes.c_uint32] * 3 + [_u32p]
        L.orc_plan_free.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        for name in ("orc_plan_pcount", "orc_plan_kpad", "orc_plan_product_bits"):
            getattr(L, name).restype = ctypes.c_uint32
            getattr(L, name).argtypes = [ctypes.c_void_p]
        for name in ("orc_plan_primes", "orc_plan_psi", "orc_plan_crt_inverse",
                     "orc_plan_weights"):
            getattr(L, name).argtypes = [ctypes.c_void_p, _u32p]
        L.orc_plan_b4.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8)]
        L.orc_encode.argtypes = [ctypes.c_void_p, _u32p, _u32p, ctypes.c_int]
        L.orc_prime_product.argtypes = [ctypes.c_void_p, ctypes.c_uint32, _u32p, _u32p, _u32p]
        L.orc_crt.argtypes = [ctypes.c_void_p, _u32p, _u32p, ctypes.c_int]
        L.orc_crt_terms.argtypes = [ctypes.c_void_p, _u32p, _u32p, _u32p, _u32p]
        L.orc_multiply.argtypes = [ctypes.c_void_p, _u32p, _u32p, _u32p, ctypes.c_int]
        L.orc_multiply.restype = ctypes.c_int
        L.orc_mont_mul_word.restype = ctypes.c_uint32
        L.orc_mont_mul_word.argtypes = [ctypes.c_uint32] * 4
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_u32p)


def words_to_int(words) -> int:
    v = 0
    for w in reversed([int(x) for x in words]):
        v = (v << 32) | w
    return v


def int_to_words(v: int, n: int) -> np.ndarray:
    return np.array([(v >> (32 * i)) & 0xFFFFFFFF for i in range(n)], dtype=np.uint32)


class Oracle:
    """One plan (N, W, q) of the C restatement."""

    def __init__(self, N: int, W: int, q_words):
        self.N, self.W = int(N), int(W)
        self.L = (self.W + 31) // 32
        self.q_words = np.ascontiguousarray(q_words, dtype=np.uint32)
        self._h = lib().orc_plan_create(self.N, self.W, self.L, _p(self.q_words))
        if not self._h:
            raise ValueError(lib().orc_last_error().decode())
        self.P = lib().orc_plan_pcount(self._h)
        self.kpad = lib().orc_plan_kpad(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().orc_plan_free(h)
            self._h = None

    def _arr(self, name, n):
        out = np.zeros(n, dtype=np.uint32)
        getattr(lib(), name)(self._h, _p(out))
        return out

    @property
    def primes(self):
        return self._arr("orc_plan_primes", self.P)

    @property
    def psi(self):
        return self._arr("orc_plan_psi", self.P)

    @property
    def crt_inverse(self):
        return self._arr("orc_plan_crt_inverse", self.P)

    @property
    def weights(self):
        return self._arr("orc_plan_weights", (self.P + 1) * self.L).reshape(self.P + 1, self.L)

    @property
    def product_bits(self):
        return lib().orc_plan_product_bits(self._h)

    def b4(self):
        out = np.zeros(4 * self.L * self.kpad, dtype=np.uint8)
        lib().orc_plan_b4(self._h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        return out.reshape(4 * self.L, self.kpad)

    def encode(self, x: np.ndarray, threads: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.uint32).reshape(self.N, self.L)
        out = np.zeros((self.P, self.N), dtype=np.uint32)
        lib().orc_encode(self._h, _p(x), _p(out), threads or lib().orc_max_threads())
        return out

    def prime_product(self, j: int, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.uint32)
        y = np.ascontiguousarray(y, dtype=np.uint32)
        out = np.zeros(self.N, dtype=np.uint32)
        lib().orc_prime_product(self._h, j, _p(x), _p(y), _p(out))
        return out

    def crt(self, res: np.ndarray, threads: int = 0) -> np.ndarray:
        res = np.ascontiguousarray(res, dtype=np.uint32).reshape(self.P, self.N)
        out = np.zeros((self.N, self.L), dtype=np.uint32)
        lib().orc_crt(self._h, _p(res), _p(out), threads or lib().orc_max_threads())
        return out

    def crt_terms(self, terms):
        """One coefficient: (alpha, wide L+2 words, reduced L words)."""
        t = np.ascontiguousarray(terms, dtype=np.uint32)
        alpha = np.zeros(1, dtype=np.uint32)
        wide = np.zeros(self.L + 2, dtype=np.uint32)
        out = np.zeros(self.L, dtype=np.uint32)
        lib().orc_crt_terms(self._h, _p(t), _p(alpha), _p(wide), _p(out))
        return int(alpha[0]), wide, out

    def multiply(self, a: np.ndarray, b: np.ndarray, threads: int = 0) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint32).reshape(self.N, self.L)
        b = np.ascontiguousarray(b, dtype=np.uint32).reshape(self.N, self.L)
        c = np.zeros((self.N, self.L), dtype=np.uint32)
        rc = lib().orc_multiply(self._h, _p(a), _p(b), _p(c), threads or lib().orc_max_threads())
        if rc != 0:
            raise MemoryError("oracle multiply allocation failed")
        return c


def max_threads() -> int:
    return lib().orc_max_threads()


# ---------------- independent big-integer references ----------------

def coeffs_to_ints(x: np.ndarray):
    x = np.asarray(x, dtype=np.uint32)
    return [words_to_int(row) for row in x]


def ints_to_coeffs(vals, L: int) -> np.ndarray:
    return np.stack([int_to_words(v, L) for v in vals]) if vals else np.zeros((0, L), np.uint32)


def schoolbook(a: np.ndarray, b: np.ndarray, q: int) -> np.ndarray:
    """O(N^2) negacyclic product with Python integers (small N only)."""
    N, L = a.shape
    A, B = coeffs_to_ints(a), coeffs_to_ints(b)
    out = [0] * N
    for i in range(N):
        ai = A[i]
        if ai == 0:
            continue
        for j in range(N):
            k = i + j
            if k < N:
                out[k] += ai * B[j]
            else:
                out[k - N] -= ai * B[j]
    return ints_to_coeffs([v % q for v in out], L)


_gmp = None


def gmp():
    """libgmp through ctypes (no headers needed), or None when absent."""
    global _gmp
    if _gmp is None:
        name = ctypes.util.find_library("gmp") or "libgmp.so.10"
        try:
            g = ctypes.CDLL(name)
        except OSError:
            _gmp = False
            return None
        _gmp = g
    return _gmp or None


class _Mpz(ctypes.Structure):
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


def _mpz_from_bytes(g, data: bytes):
    z = _Mpz()
    g.__gmpz_init(ctypes.byref(z))
    # mpz_import(rop, count, order=-1 (LSW first), size=1, endian=0, nails=0, op)
    g.__gmpz_import(ctypes.byref(z), ctypes.c_size_t(len(data)), ctypes.c_int(-1),
                    ctypes.c_size_t(1), ctypes.c_int(0), ctypes.c_size_t(0), data)
    return z


def _mpz_to_bytes(g, z, nbytes: int) -> bytes:
    buf = ctypes.create_string_buffer(nbytes + 16)
    count = ctypes.c_size_t(0)
    g.__gmpz_export(buf, ctypes.byref(count), ctypes.c_int(-1), ctypes.c_size_t(1),
                    ctypes.c_int(0), ctypes.c_size_t(0), ctypes.byref(z))
    return buf.raw[:nbytes]


def kronecker(a: np.ndarray, b: np.ndarray, q: int) -> np.ndarray:
    """Kronecker substitution with libgmp: pack each operand into one integer
    with slot width S bits (S > 2W + log2 N + 1), multiply once, unpack the
    2N-1 slots, fold negacyclically (c_k = C_k - C_{k+N}) and reduce mod q."""
    g = gmp()
    if g is None:
        raise RuntimeError("libgmp not available")
    N, L = a.shape
    W = q.bit_length()
    S = (2 * W + N.bit_length() + 2 + 31) // 32 * 32   # slot width in bits, whole words
    sw = S // 32
    packed = []
    for x in (a, b):
        buf = np.zeros((N, sw), dtype=np.uint32)
        buf[:, :L] = x
        packed.append(_mpz_from_bytes(g, buf.tobytes()))
    prod = _Mpz()
    g.__gmpz_init(ctypes.byref(prod))
    g.__gmpz_mul(ctypes.byref(prod), ctypes.byref(packed[0]), ctypes.byref(packed[1]))
    raw = _mpz_to_bytes(g, prod, 2 * N * sw * 4)
    for z in packed + [prod]:
        g.__gmpz_clear(ctypes.byref(z))
    slots = np.frombuffer(raw, dtype=np.uint32).reshape(2 * N, sw)
    lo = [words_to_int(r) for r in slots[:N]]
    hi = [words_to_int(r) for r in slots[N:]]
    return ints_to_coeffs([(lo[k] - hi[k]) % q for k in range(N)], L)
