"""Build recipe for the in-tree native libraries (sm_103a only).

    python -c "import importlib; importlib.import_module('fherma-bytecrt_gb300.build').build()"

Compiles csrc/*.cu with nvcc for sm_103a, in parallel, into
libbytecrt_gb300.so (the C ABI of include/bytecrt_gb300.h) and
libfherma_gb300.so (the reference's C++ plugin ABI on top of it), plus the
`solution` harness binary.  Objects go to _build/ (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(REPO, "_build")
LIB = os.path.join(HERE, "libbytecrt_gb300.so")
SHIM = os.path.join(HERE, "libfherma_gb300.so")
HARNESS = os.path.join(HERE, "solution")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CORE_SOURCES = ["plan.cu", "encode.cu", "encode_scalar.cu", "host_copy.cu", "ntt.cu", "crt.cu", "crt_persistent.cu", "engine.cu", "capi.cu", "static_scratch.cu", "autotune.cu",
                "batch.cu", "server.cu", "capi_serve.cu"]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return path


def _flags():
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC,-O3,-fopenmp",
            "-I", os.path.join(REPO, "include")]


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".cuh", ".h"))] + \
        [os.path.join(REPO, "include", f) for f in os.listdir(os.path.join(REPO, "include"))]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if _stale(obj, [src, *_headers(), __file__]):
        cmd = [nvcc(), *_flags(), "-c", src, "-o", obj + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    sources = [os.path.join(CSRC, s) for s in CORE_SOURCES]
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, sources))
    if _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fopenmp", "-lgomp"],
                       check=True)
        os.replace(tmp, LIB)
    # The plugin ABI twice: single product and batched (Point carries B).
    inc = ["-I", os.path.join(REPO, "include")]
    shim_src = os.path.join(CSRC, "fherma_shim.cpp")
    harness_src = os.path.join(CSRC, "harness.cpp")
    for suffix, defs in (("", []), ("_batched", ["-DFHERMA_BATCHED"])):
        shim = os.path.join(HERE, f"libfherma_gb300{suffix}.so")
        if _stale(shim, [shim_src, LIB, os.path.abspath(__file__), *_headers()]):
            tmp = shim + f".tmp{os.getpid()}"
            # The shim's own references (the owned vector's growth and copies, which the wraps
            # below make parallel) bind to its own definitions: a host executable's instantiation
            # of the same std::vector members, built without the wraps, must not replace them.
            subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-fvisibility-inlines-hidden",
                            "-Wl,-Bsymbolic-functions", "-Wl,--wrap=memcpy", "-Wl,--wrap=memmove",
                            "-Wl,--wrap=memset", *defs, *inc, "-o", tmp, shim_src,
                            "-L", HERE, "-lbytecrt_gb300", "-Wl,-rpath,$ORIGIN"], check=True)
            os.replace(tmp, shim)
        harness = os.path.join(HERE, f"solution{suffix}")
        if _stale(harness, [harness_src, shim, *_headers()]):
            tmp = harness + f".tmp{os.getpid()}"
            subprocess.run(["g++", "-std=c++17", "-O2", *defs, *inc, "-o", tmp, harness_src, "-L", HERE,
                            f"-lfherma_gb300{suffix}", "-lbytecrt_gb300", "-Wl,-rpath,$ORIGIN"], check=True)
            os.replace(tmp, harness)
    return LIB


if __name__ == "__main__":
    print(build())
