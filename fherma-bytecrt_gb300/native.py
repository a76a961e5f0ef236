"""ctypes binding of libbytecrt_gb300.so (include/bytecrt_gb300.h).

The product path is native only: if the shared library is missing this module
raises, it never falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libbytecrt_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "bytecrt_gb300.h")

BCG_OK = 0
BCG_ERR_INVALID = 1
BCG_ERR_CUDA = 2
BCG_ERR_NOMEM = 3
BCG_ERR_DEVICE_TIMEOUT = 4
BCG_ERR_BUSY = 5
BCG_ERR_TIMEOUT = 6

_u32p = ctypes.POINTER(ctypes.c_uint32)
SINK = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), ctypes.c_size_t)
DEST = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t)


class BcgError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"bcg error {code}: {message}")
        self.code = code


class bcg_info(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in
                ("N", "W", "L", "P", "kpad", "enc_k", "enc_cols", "crt_k", "crt_n",
                 "product_bits", "group", "reserved")] + [("workspace_bytes_per_product", ctypes.c_uint64)]


class bcg_profile(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_double * 8), ("launches", ctypes.c_uint64 * 8), ("timed", ctypes.c_uint64 * 8),
                ("chains", ctypes.c_uint64)]


class bcg_autotune_report(ctypes.Structure):
    _fields_ = [("group", ctypes.c_uint32), ("crt_tiles", ctypes.c_uint32), ("row_rows", ctypes.c_uint32),
                ("row_bits", ctypes.c_uint32), ("candidates", ctypes.c_uint32), ("crt_persistent", ctypes.c_uint32),
                ("row_local", ctypes.c_uint32), ("row_pass", ctypes.c_uint32),
                ("encode_scalar", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("us_per_product_default", ctypes.c_double), ("us_per_product_tuned", ctypes.c_double)]


class bcg_batch_info(ctypes.Structure):
    _fields_ = [("groups", ctypes.c_uint32), ("reserved", ctypes.c_uint32), ("products", ctypes.c_uint64),
                ("chains", ctypes.c_uint64), ("launches", ctypes.c_uint64)]


class bcg_server_options(ctypes.Structure):
    _fields_ = [("memory_bytes", ctypes.c_uint64), ("slots", ctypes.c_uint32), ("max_batch", ctypes.c_uint32),
                ("max_queue", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class bcg_server_stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in
                ("submitted", "completed", "failed", "rejected", "batches", "batched_products", "operands",
                 "memory_budget", "memory_used", "memory_peak")]


STAGES = ("encode", "column", "row", "column_inverse", "crt")

_lib = None


def header_functions() -> list[str]:
    """Names of every function declared in include/bytecrt_gb300.h."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(bcg_[a-z_0-9]+)\s*\(", text, re.M)))


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"native library missing: {LIB_PATH} (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        L.bcg_last_error.restype = ctypes.c_char_p
        vp = ctypes.c_void_p
        L.bcg_plan_create.argtypes = [ctypes.c_uint32] * 3 + [_u32p, ctypes.POINTER(vp)]
        L.bcg_plan_destroy.argtypes = [vp]
        L.bcg_plan_destroy.restype = None
        L.bcg_plan_info.argtypes = [vp, ctypes.POINTER(bcg_info)]
        L.bcg_plan_primes.argtypes = [vp, _u32p, _u32p, _u32p]
        L.bcg_plan_weights.argtypes = [vp, _u32p]
        L.bcg_context_create.argtypes = [ctypes.c_uint32] * 3 + [_u32p, ctypes.c_int, ctypes.POINTER(vp)]
        L.bcg_context_destroy.argtypes = [vp]
        L.bcg_context_destroy.restype = None
        L.bcg_context_info.argtypes = [vp, ctypes.POINTER(bcg_info)]
        L.bcg_context_set_group.argtypes = [vp, ctypes.c_uint32]
        L.bcg_context_set_tuning.argtypes = [vp, ctypes.c_char_p, ctypes.c_int64]
        L.bcg_context_get_tuning.argtypes = [vp, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]
        L.bcg_multiply.argtypes = [vp, _u32p, _u32p, _u32p, ctypes.c_uint32]
        L.bcg_host_alloc.argtypes = [ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(vp)]
        L.bcg_host_free.argtypes = [vp]
        L.bcg_multiply_sink.argtypes = [vp, _u32p, _u32p, ctypes.c_uint32, SINK, vp]
        L.bcg_multiply_dest.argtypes = [vp, _u32p, _u32p, ctypes.c_uint32, DEST, vp]
        L.bcg_context_autotune.argtypes = [vp, ctypes.c_uint32, ctypes.POINTER(bcg_autotune_report)]
        L.bcg_multiply_device.argtypes = [vp, vp, vp, vp, ctypes.c_uint32, vp]
        L.bcg_multiply_device_static.argtypes = [vp, vp, vp, vp, ctypes.c_uint32, vp]
        L.bcg_encode_device.argtypes = [vp, vp, vp, vp, vp, ctypes.c_size_t, ctypes.c_uint32, vp]
        L.bcg_negacyclic_device.argtypes = [vp, vp, vp, ctypes.c_size_t, ctypes.c_uint32, vp]
        L.bcg_crt_device.argtypes = [vp, vp, ctypes.c_size_t, vp, ctypes.c_uint32, vp]
        L.bcg_synchronize.argtypes = [vp]
        L.bcg_profile_enable.argtypes = [vp, ctypes.c_int]
        L.bcg_profile_read.argtypes = [vp, ctypes.POINTER(bcg_profile), ctypes.c_int]
        u32, u64 = ctypes.c_uint32, ctypes.c_uint64
        L.bcg_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(vp)]
        L.bcg_batch_destroy.argtypes = [vp]
        L.bcg_batch_destroy.restype = None
        L.bcg_batch_add.argtypes = [vp, u32, u32, u32, _u32p, vp, vp, vp, u32]
        L.bcg_batch_run.argtypes = [vp, vp]
        L.bcg_batch_synchronize.argtypes = [vp, vp]
        L.bcg_batch_get_info.argtypes = [vp, ctypes.POINTER(bcg_batch_info)]
        L.bcg_batch_profile_enable.argtypes = [vp, ctypes.c_int]
        L.bcg_batch_set_lanes.argtypes = [vp, u32]
        L.bcg_batch_profile_read.argtypes = [vp, ctypes.POINTER(bcg_profile)]
        L.bcg_server_create.argtypes = [ctypes.c_int, ctypes.POINTER(bcg_server_options), ctypes.POINTER(vp)]
        L.bcg_server_destroy.argtypes = [vp]
        L.bcg_server_destroy.restype = None
        L.bcg_server_add_point.argtypes = [vp, u32, u32, u32, _u32p, ctypes.POINTER(u32)]
        L.bcg_server_add_operand.argtypes = [vp, u32, vp, ctypes.POINTER(u64)]
        L.bcg_server_remove_operand.argtypes = [vp, u64]
        L.bcg_server_submit.argtypes = [vp, u32, vp, u64, vp, vp, ctypes.POINTER(u64)]
        L.bcg_server_wait.argtypes = [vp, u64, u32, ctypes.POINTER(ctypes.c_double)]
        L.bcg_server_drain.argtypes = [vp]
        L.bcg_server_get_stats.argtypes = [vp, ctypes.POINTER(bcg_server_stats)]
        _lib = L
    return _lib


def _check(rc: int):
    if rc != BCG_OK:
        raise BcgError(rc, lib().bcg_last_error().decode())


def _p(a: np.ndarray):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_u32p)


def _ptr(x) -> int | None:
    """Device pointer of a torch tensor (or an int address)."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def limbs(W: int) -> int:
    return (W + 31) // 32


class Plan:
    """Host-only plan (no GPU needed)."""

    def __init__(self, N: int, W: int, q):
        self.N, self.W, self.L = int(N), int(W), limbs(W)
        q = np.ascontiguousarray(q, dtype=np.uint32)
        h = ctypes.c_void_p()
        _check(lib().bcg_plan_create(self.N, self.W, self.L, _p(q), ctypes.byref(h)))
        self._h = h
        info = bcg_info()
        _check(lib().bcg_plan_info(self._h, ctypes.byref(info)))
        self.info = info
        self.P = info.P

    def __del__(self):
        if getattr(self, "_h", None):
            lib().bcg_plan_destroy(self._h)
            self._h = None

    def primes(self):
        p, s, c = (np.zeros(self.P, np.uint32) for _ in range(3))
        _check(lib().bcg_plan_primes(self._h, _p(p), _p(s), _p(c)))
        return p, s, c

    def weights(self):
        w = np.zeros((self.P + 1) * self.L, np.uint32)
        _check(lib().bcg_plan_weights(self._h, _p(w)))
        return w.reshape(self.P + 1, self.L)


def host_alloc(nbytes: int, device: int = 0) -> int:
    """Pinned host memory (bcg_host_alloc): the address of nbytes; free with host_free."""
    p = ctypes.c_void_p()
    _check(lib().bcg_host_alloc(nbytes, device, ctypes.byref(p)))
    return p.value


def host_free(address: int) -> None:
    _check(lib().bcg_host_free(address))


class Multiplier:
    """One point (N, W, q) on one GPU: the native context behind fherma_init."""

    def __init__(self, N: int, W: int, q, device: int = 0):
        self.N, self.W, self.L = int(N), int(W), limbs(W)
        self.q = np.ascontiguousarray(q, dtype=np.uint32)
        h = ctypes.c_void_p()
        _check(lib().bcg_context_create(self.N, self.W, self.L, _p(self.q), int(device), ctypes.byref(h)))
        self._h = h
        info = bcg_info()
        _check(lib().bcg_context_info(self._h, ctypes.byref(info)))
        self.info = info
        self.P = info.P

    def close(self):
        if getattr(self, "_h", None):
            lib().bcg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def plane_words(self) -> int:
        return self.P * self.N

    def set_group(self, group: int):
        _check(lib().bcg_context_set_group(self._h, int(group)))
        info = bcg_info()
        _check(lib().bcg_context_info(self._h, ctypes.byref(info)))
        self.info = info

    def set_tuning(self, knob: str, value: int):
        _check(lib().bcg_context_set_tuning(self._h, knob.encode(), int(value)))
        info = bcg_info()
        _check(lib().bcg_context_info(self._h, ctypes.byref(info)))
        self.info = info

    def get_tuning(self, knob: str) -> int:
        v = ctypes.c_int64()
        _check(lib().bcg_context_get_tuning(self._h, knob.encode(), ctypes.byref(v)))
        return int(v.value)

    # ---- host buffers
    def autotune(self, max_group: int = 16) -> dict:
        """Times candidate kernel shapes for this geometry and keeps the fastest."""
        r = bcg_autotune_report()
        _check(lib().bcg_context_autotune(self._h, max_group, ctypes.byref(r)))
        return {n: getattr(r, n) for n, _ in bcg_autotune_report._fields_ if n != "reserved"}

    def multiply(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint32)
        b = np.ascontiguousarray(b, dtype=np.uint32)
        if a.shape != b.shape or a.size % (self.N * self.L):
            raise ValueError("operands must be [count][N][L] uint32 of equal shape")
        count = a.size // (self.N * self.L)
        c = np.zeros_like(a)
        _check(lib().bcg_multiply(self._h, _p(a), _p(b), _p(c), count))
        return c

    def multiply_sink(self, a: np.ndarray, b: np.ndarray, sink) -> None:
        """c = a*b from host buffers, handed over in order as sink(words) calls
        (a read-only numpy view valid during the call; words=None, first, with
        the number of words that arrive first, as a chance to prepare)."""
        a = np.ascontiguousarray(a, dtype=np.uint32)
        b = np.ascontiguousarray(b, dtype=np.uint32)
        if a.shape != b.shape or a.size % (self.N * self.L):
            raise ValueError("operands must be [count][N][L] uint32 of equal shape")
        count = a.size // (self.N * self.L)
        errors = []

        def call(user, words, n):
            try:
                if not words:
                    sink(None, int(n))
                else:
                    sink(np.ctypeslib.as_array(words, shape=(int(n),)), int(n))
            except BaseException as e:   # never raise through the C ABI
                errors.append(e)

        cb = SINK(call)
        _check(lib().bcg_multiply_sink(self._h, _p(a), _p(b), count, cb, None))
        if errors:
            raise errors[0]

    def multiply_dest(self, a: np.ndarray, b: np.ndarray, dest) -> None:
        """c = a*b from host buffers into memory the caller names run by run:
        dest(n) returns the host address (an int) where the next n words go,
        or 0 to refuse (BcgError).  The memory must stay valid and untouched
        until the call returns."""
        a = np.ascontiguousarray(a, dtype=np.uint32)
        b = np.ascontiguousarray(b, dtype=np.uint32)
        if a.shape != b.shape or a.size % (self.N * self.L):
            raise ValueError("operands must be [count][N][L] uint32 of equal shape")
        count = a.size // (self.N * self.L)
        errors = []

        def call(user, n):
            try:
                return int(dest(int(n)) or 0) or None
            except BaseException as e:   # never raise through the C ABI
                errors.append(e)
                return None

        cb = DEST(call)
        try:
            _check(lib().bcg_multiply_dest(self._h, _p(a), _p(b), count, cb, None))
        finally:
            if errors:
                raise errors[0]

    def multiply_into(self, a, b, c, count: int):
        """Host buffers given as addresses (e.g. pinned torch tensors): c = a*b, synchronous."""
        vp = ctypes.c_void_p
        _check(lib().bcg_multiply(self._h, ctypes.cast(vp(_ptr(a)), _u32p), ctypes.cast(vp(_ptr(b)), _u32p),
                                  ctypes.cast(vp(_ptr(c)), _u32p), count))

    # ---- device buffers (torch tensors or raw addresses)
    def multiply_device(self, a, b, c, count: int, stream=None):
        _check(lib().bcg_multiply_device(self._h, _ptr(a), _ptr(b), _ptr(c), count, _ptr(stream)))

    def multiply_device_static(self, a, b, c, count: int, stream=None):
        """Like multiply_device, but allocates nothing (library-owned 16 MiB scratch)."""
        _check(lib().bcg_multiply_device_static(self._h, _ptr(a), _ptr(b), _ptr(c), count, _ptr(stream)))

    def encode_device(self, a, b, planes_a, planes_b, plane_stride: int, count: int, stream=None):
        _check(lib().bcg_encode_device(self._h, _ptr(a), _ptr(b), _ptr(planes_a), _ptr(planes_b),
                                       plane_stride, count, _ptr(stream)))

    def negacyclic_device(self, planes_a, planes_b, plane_stride: int, count: int, stream=None):
        _check(lib().bcg_negacyclic_device(self._h, _ptr(planes_a), _ptr(planes_b), plane_stride, count,
                                           _ptr(stream)))

    def crt_device(self, terms, plane_stride: int, c, count: int, stream=None):
        _check(lib().bcg_crt_device(self._h, _ptr(terms), plane_stride, _ptr(c), count, _ptr(stream)))

    def synchronize(self):
        _check(lib().bcg_synchronize(self._h))

    # ---- measurement
    def profile(self, enable: bool = True, every: int = 1):
        """Time the stages of every `every`-th launch chain with CUDA events (off: enable=False)."""
        _check(lib().bcg_profile_enable(self._h, int(every) if enable else 0))

    def read_profile(self, reset: bool = True) -> dict:
        p = bcg_profile()
        _check(lib().bcg_profile_read(self._h, ctypes.byref(p), 1 if reset else 0))
        return _profile_dict(p)


def _hptr(x) -> int:
    """Host address of a numpy array or a (pinned) CPU torch tensor."""
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        assert x.flags.c_contiguous
        return x.ctypes.data
    return x.data_ptr()


def _profile_dict(p: "bcg_profile") -> dict:
    return {"ms": {s: p.ms[i] for i, s in enumerate(STAGES)},
            "launches": {s: int(p.launches[i]) for i, s in enumerate(STAGES)},
            "timed": {s: int(p.timed[i]) for i, s in enumerate(STAGES)},
            "chains": int(p.chains)}


class Batch:
    """Products of uneven points in one CUDA graph (bcg_batch_*)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        _check(lib().bcg_batch_create(int(device), ctypes.byref(h)))
        self._h = h
        self._keep = []   # moduli and buffers referenced by the graph

    def add(self, N: int, W: int, q, a, b, c, count: int):
        q = np.ascontiguousarray(q, dtype=np.uint32)
        self._keep.append((q, a, b, c))
        _check(lib().bcg_batch_add(self._h, N, W, limbs(W), _p(q), _ptr(a), _ptr(b), _ptr(c), count))

    def run(self, stream=None):
        _check(lib().bcg_batch_run(self._h, _ptr(stream)))

    def synchronize(self, stream=None):
        _check(lib().bcg_batch_synchronize(self._h, _ptr(stream)))

    def info(self) -> dict:
        i = bcg_batch_info()
        _check(lib().bcg_batch_get_info(self._h, ctypes.byref(i)))
        return {"groups": i.groups, "products": i.products, "chains": i.chains, "launches": i.launches}

    def profile(self, every: int = 1):
        _check(lib().bcg_batch_profile_enable(self._h, int(every)))

    def set_lanes(self, lanes: int):
        """Alternate the launch chains over 1 or 2 parallel graph branches."""
        _check(lib().bcg_batch_set_lanes(self._h, int(lanes)))

    def read_profile(self) -> dict:
        p = bcg_profile()
        _check(lib().bcg_batch_profile_read(self._h, ctypes.byref(p)))
        return _profile_dict(p)

    def close(self):
        if getattr(self, "_h", None):
            lib().bcg_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Server:
    """Request loop with continuous batching on one GPU (bcg_server_*)."""

    def __init__(self, device: int = 0, memory_bytes: int = 0, slots: int = 0, max_batch: int = 0,
                 max_queue: int = 0):
        o = bcg_server_options(memory_bytes, slots, max_batch, max_queue, 0)
        h = ctypes.c_void_p()
        _check(lib().bcg_server_create(int(device), ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    def add_point(self, N: int, W: int, q) -> int:
        q = np.ascontiguousarray(q, dtype=np.uint32)
        out = ctypes.c_uint32()
        _check(lib().bcg_server_add_point(self._h, N, W, limbs(W), _p(q), ctypes.byref(out)))
        return out.value

    def add_operand(self, point: int, a) -> int:
        out = ctypes.c_uint64()
        _check(lib().bcg_server_add_operand(self._h, point, _hptr(a), ctypes.byref(out)))
        return out.value

    def remove_operand(self, operand: int):
        _check(lib().bcg_server_remove_operand(self._h, operand))

    def submit(self, point: int, b, c, a=None, operand: int = 0) -> int:
        out = ctypes.c_uint64()
        _check(lib().bcg_server_submit(self._h, point, None if a is None else _hptr(a), operand, _hptr(b),
                                       _hptr(c), ctypes.byref(out)))
        return out.value

    def wait(self, request: int, timeout_ms: int = 0) -> float:
        """Latency in ms; raises BcgError with the request's own status on failure."""
        lat = ctypes.c_double()
        _check(lib().bcg_server_wait(self._h, request, timeout_ms, ctypes.byref(lat)))
        return lat.value

    def drain(self):
        _check(lib().bcg_server_drain(self._h))

    def stats(self) -> dict:
        s = bcg_server_stats()
        _check(lib().bcg_server_get_stats(self._h, ctypes.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in bcg_server_stats._fields_}

    def close(self):
        if getattr(self, "_h", None):
            lib().bcg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()
