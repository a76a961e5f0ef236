"""ORACLE — test and measurement infrastructure only (never imported by the product).

Runs the reference's own encode and CRT kernels on the GPU, for comparison with
this library's kernels on the same GB300:

* ``encode_mma32<L, P, Kpad, true>`` (native-smoke/rns-encode-mma.cuh:148-252),
  launched as ``launch_encode_mma32_transposed`` does (:302-315): grid
  (N/32, 2 operands), 224 threads; input ``[2][N][L]`` u32, byte-power matrix
  from ``make_encode_b`` (:15-36), ``mu = floor(2^64 / p)`` (:43-52), output
  ``[2][P][256][N/256]`` u32;
* ``g1_crt32<W, L, P, Kpad, true>`` (native-smoke/g1-crt.cuh:201-335), launched
  as ``launch_g1_crt32_transposed`` does (:375-387): N/32 CTAs of 224 threads;
  terms ``A_t[256][Kpad/4][N/256]`` (coefficient id + 256*i, word j = t_j,
  alpha and padding words zero), the plan's B4 bytes, fp32 1/p_j, q = 2^W - gap,
  output ``[N][L]``.

The kernels come unmodified from the reference checkout, compiled by
oracle/build_ref.sh into ``oracle/_ref/ref_kernels.cubin`` (sm_103a, device code
only), and are loaded here through the CUDA driver API.  Only the geometries the
reference supports exist: N=65536/W=1747 and N=32768/W=868, gap-form q only.

Each run checks the launch against the oracle (every encode residue plane as a
multiset, a sample of CRT coefficients exactly) before it reports times.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")

# (N, W) -> (L, P, encode Kpad, CRT Kpad)
GEOMETRIES = {(65536, 1747): (55, 114, 224, 480), (32768, 868): (28, 57, 128, 256)}


def available() -> bool:
    return os.path.exists(CUBIN)


class _Driver:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.cu.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        self.cu.cuModuleGetFunctionCount.argtypes = [ctypes.POINTER(ctypes.c_uint), ctypes.c_void_p]
        self.cu.cuModuleEnumerateFunctions.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_uint,
                                                       ctypes.c_void_p]
        self.cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p]
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [
            ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        self.cu.cuModuleUnload.argtypes = [ctypes.c_void_p]

    def check(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUDA driver error {rc}")


class RefKernels:
    """The reference's encode and CRT kernels, loaded from the cubin."""

    def __init__(self):
        import torch
        if not available():
            raise FileNotFoundError(f"{CUBIN} not built (oracle/build_ref.sh needs the reference checkout)")
        torch.zeros(1, device="cuda")          # make the primary context current on this thread
        self.d = _Driver()
        self.mod = ctypes.c_void_p()
        self.d.check(self.d.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        count = ctypes.c_uint()
        self.d.check(self.d.cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * count.value)()
        self.d.check(self.d.cu.cuModuleEnumerateFunctions(funcs, count.value, self.mod), "cuModuleEnumerateFunctions")
        self.funcs = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self.d.check(self.d.cu.cuFuncGetName(ctypes.byref(name), f), "cuFuncGetName")
            self.funcs[name.value.decode()] = f

    def _find(self, *parts):
        hits = [f for n, f in self.funcs.items() if all(p in n for p in parts)]
        if len(hits) != 1:
            raise KeyError(f"kernel {parts} not found in {sorted(self.funcs)}")
        return hits[0]

    def _launch(self, f, grid, block, args, stream):
        holders, ptrs = [], []
        for kind, v in args:
            h = ctypes.c_uint(v) if kind == "u32" else ctypes.c_void_p(v)
            holders.append(h)
            ptrs.append(ctypes.cast(ctypes.byref(h), ctypes.c_void_p))
        arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
        self.d.check(self.d.cu.cuLaunchKernel(f, grid[0], grid[1], 1, block, 1, 1, 0, ctypes.c_void_p(stream), arr,
                                              None), "cuLaunchKernel")

    def encode_kernel(self, N, W):
        L, P, kenc, _ = GEOMETRIES[(N, W)]
        return self._find("encode_mma32", f"ILj{L}ELj{P}ELj{kenc}ELb1E")

    def crt_kernel(self, N, W):
        L, P, _, kcrt = GEOMETRIES[(N, W)]
        return self._find("g1_crt32", f"ILj{W}ELj{L}ELj{P}ELj{kcrt}ELb1E")

    def encode(self, N, W, inputs, b, primes, mu, out, stream):
        self._launch(self.encode_kernel(N, W), (N // 32, 2), 224,
                     [("u32", N), ("ptr", inputs), ("ptr", b), ("ptr", primes), ("ptr", mu), ("ptr", out),
                      ("u32", 0)], stream)

    def crt(self, N, W, a_t, b4, invp, q, gap, out, stream):
        self._launch(self.crt_kernel(N, W), (N // 32, 1), 224,
                     [("ptr", a_t), ("ptr", b4), ("ptr", invp), ("ptr", q), ("u32", gap), ("ptr", out),
                      ("u32", 0)], stream)


def make_encode_b(L: int, P: int, primes) -> np.ndarray:
    """Byte-power matrix as make_encode_b builds it (rns-encode-mma.cuh:15-36):
    column 4j+d, input byte k holds byte_d(2^(8k) mod p_j); 4P columns of K bytes."""
    K = (4 * L + 31) // 32 * 32
    b = np.zeros((4 * P, K), dtype=np.uint8)
    p = np.asarray(primes, dtype=np.uint64)
    power = np.ones(P, dtype=np.uint64)
    for k in range(4 * L):
        for d in range(4):
            b[4 * np.arange(P) + d, k] = ((power >> np.uint64(8 * d)) & np.uint64(255)).astype(np.uint8)
        power = power * np.uint64(256) % p
    return b


def gap_modulus(W: int, gap: int) -> np.ndarray:
    L = (W + 31) // 32
    q = (1 << W) - gap
    return np.array([(q >> (32 * i)) & 0xFFFFFFFF for i in range(L)], dtype=np.uint32)


def run(N: int, W: int, gap: int = 0x9E3779B1, reps: int = 10, copies: int = 4, seed: int = 7) -> dict:
    """Checks and times both reference kernels at (N, W); microseconds per product."""
    import torch
    from oracle import oracle
    L, P, _, kcrt = GEOMETRIES[(N, W)]
    rk = RefKernels()
    q = gap_modulus(W, gap)
    o = oracle.Oracle(N, W, q)
    assert o.P == P and o.kpad == kcrt, (o.P, o.kpad)
    primes = o.primes
    rng = np.random.default_rng(seed)
    dev = torch.device("cuda")
    st = torch.cuda.current_stream().cuda_stream

    # ---- encode: uniform operands in [0, q) (top limb masked below q's top word)
    x = rng.integers(0, 1 << 32, size=(2, N, L), dtype=np.uint64).astype(np.uint32)
    x[:, :, L - 1] &= np.uint32((1 << (W - 32 * (L - 1))) - 1) >> np.uint32(1)
    b = torch.from_numpy(make_encode_b(L, P, primes)).to(dev)
    p_d = torch.from_numpy(primes.astype(np.uint32).view(np.int32)).to(dev)
    mu = torch.from_numpy((np.uint64(0xFFFFFFFFFFFFFFFF) // primes.astype(np.uint64)).view(np.int64)).to(dev)
    ins = [torch.from_numpy(x.view(np.int32)).to(dev) for _ in range(copies)]
    outs = [torch.zeros((2, P, N), dtype=torch.int32, device=dev) for _ in range(copies)]
    rk.encode(N, W, ins[0].data_ptr(), b.data_ptr(), p_d.data_ptr(), mu.data_ptr(), outs[0].data_ptr(), st)
    torch.cuda.synchronize()
    got = outs[0].cpu().numpy().view(np.uint32)
    for op in range(2):
        want = o.encode(x[op])
        for j in range(P):
            if not np.array_equal(np.sort(got[op, j]), np.sort(want[j])):
                raise AssertionError(f"reference encode launch disagrees with the oracle (operand {op}, prime {j})")
    enc_us = _time(lambda i: rk.encode(N, W, ins[i % copies].data_ptr(), b.data_ptr(), p_d.data_ptr(),
                                       mu.data_ptr(), outs[i % copies].data_ptr(), st), reps)

    # ---- CRT: terms t_j uniform in [0, p_j), transposed A_t words
    terms = (rng.random((P, N)) * primes[:, None].astype(np.float64)).astype(np.uint64).astype(np.uint32)
    rw, nt = kcrt // 4, N // 256
    a_t = np.zeros((256, rw, nt), dtype=np.uint32)
    # coefficient n = id + 256*i  ->  A_t[id][j][i]
    a_t[:, :P, :] = terms.reshape(P, nt, 256).transpose(2, 0, 1)
    b4 = torch.from_numpy(np.ascontiguousarray(o.b4())).to(dev)
    invp = torch.from_numpy((1.0 / primes.astype(np.float64)).astype(np.float32)).to(dev)
    q_d = torch.from_numpy(q.view(np.int32)).to(dev)
    a_ts = [torch.from_numpy(a_t.view(np.int32)).to(dev) for _ in range(copies)]
    couts = [torch.zeros((N, L), dtype=torch.int32, device=dev) for _ in range(copies)]
    rk.crt(N, W, a_ts[0].data_ptr(), b4.data_ptr(), invp.data_ptr(), q_d.data_ptr(), gap, couts[0].data_ptr(), st)
    torch.cuda.synchronize()
    cgot = couts[0].cpu().numpy().view(np.uint32)
    for n in rng.choice(N, size=256, replace=False):
        _, _, want = o.crt_terms(terms[:, n])
        if not np.array_equal(cgot[n], want):
            raise AssertionError(f"reference CRT launch disagrees with the oracle at coefficient {n}")
    crt_us = _time(lambda i: rk.crt(N, W, a_ts[i % copies].data_ptr(), b4.data_ptr(), invp.data_ptr(),
                                    q_d.data_ptr(), gap, couts[i % copies].data_ptr(), st), reps)
    return {"N": N, "W": W, "q": f"2^{W} - {gap}", "encode_mma32_us": round(enc_us, 2),
            "g1_crt32_us": round(crt_us, 2), "checked": True}


def _time(launch, reps: int) -> float:
    import torch
    for i in range(3):
        launch(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for i in range(reps):
        launch(i)
    e1.record()
    e1.synchronize()
    return 1000.0 * e0.elapsed_time(e1) / reps
