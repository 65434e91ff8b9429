"""Build libtdic_gb300.so: hand-written CUDA for sm_103a plus the C ABI.

nvcc compiles each translation unit in parallel (one -gencode, sm_103a) and links a shared
library into _build/ next to this file.  hotpath.cu holds the single-pair first-order ZNSSD
kernels, batch.cu the batched propagation (once per precision), heap_order.cu the host rounds of
the heap order.  variants.cu is compiled once per solver route other than
first-order ZNSSD (-DTDIC_ROUTE=1 SSD, 2 second order, 3 second-order SSD, 4 masked first-order
ZNSSD), so the routes' kernels build side by side.  No torch types cross the ABI, so the library is built with plain nvcc, not
torch.utils.cpp_extension.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libtdic_gb300.so")
# (source, object, extra nvcc flags)
UNITS = [("api.cu", "api.o", []), ("prefilter.cu", "prefilter.o", []), ("hotpath.cu", "hotpath.o", []),
         ("heap_order.cu", "heap_order.o", []),
         ("batch.cu", "batch_f32.o", ["-DTDIC_BATCH_FP64=0", "-DTDIC_BATCH_VAR=0"]),
         ("batch.cu", "batch_f64.o", ["-DTDIC_BATCH_FP64=1", "-DTDIC_BATCH_VAR=0"]),
         ("batch.cu", "batch_f32_masked.o", ["-DTDIC_BATCH_FP64=0", "-DTDIC_BATCH_VAR=4"]),
         ("batch.cu", "batch_f64_masked.o", ["-DTDIC_BATCH_FP64=1", "-DTDIC_BATCH_VAR=4"]),
         ("results.cpp", "results.o", []),
         ("seed.cu", "seed.o", []), ("strain.cu", "strain.o", []),
         ("variants.cu", "route1.o", ["-DTDIC_ROUTE=1"]), ("variants.cu", "route2.o", ["-DTDIC_ROUTE=2"]),
         ("variants.cu", "route3.o", ["-DTDIC_ROUTE=3"]), ("variants.cu", "route4.o", ["-DTDIC_ROUTE=4"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
         "-Xcompiler", "-Wall", "-I", os.path.join(HERE, "..", "include")]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src, os.path.join(HERE, "..", "include", "tdic_gb300.h")]
    deps += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    return any(os.path.getmtime(d) > os.path.getmtime(obj) for d in deps)


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    extra = extra or []

    def compile_one(unit) -> str:
        name, oname, defs = unit
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, oname)
        if _stale(obj, src) or extra:
            cmd = [nvcc, *ARCH, *FLAGS, *defs, *extra, "-c", src, "-o", obj]
            if verbose:
                print(" ".join(cmd))
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {oname}:\n{r.stdout}\n{r.stderr}")
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
