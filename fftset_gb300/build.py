"""Builds libfftset_gb300.so in-tree (fftset_gb300/_lib/) for sm_103a.

nvcc compiles the CUDA kernels, gcc the C host layer; translation units are
compiled in parallel and only when their sources changed."""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libfftset_gb300.so")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["fgk_resident.cu", "fgk_static.cu", "fgk_static_1536.cu", "fgk_static_4096.cu", "fgk_static_1024.cu", "fgk_static_complex.cu", "fgk_fourstep.cu", "fgk_tasks.cu", "fgk_tasks_fc.cu", "fgk_tasks_ff.cu", "fgk_tasks_ic.cu", "fgk_tasks_if.cu", "fgk_tasks_fcw.cu", "fgk_tasks_ffw.cu", "fgk_tasks_icw.cu", "fgk_tasks_ifw.cu", "fgk_tasks_fcs.cu", "fgk_tasks_ffs.cu", "fgk_tasks_ics.cu", "fgk_tasks_ifs.cu", "fgk_fixed_scratch.cu", "fgk_adjoint.cu", "fgk_ola.cu"]
C_SOURCES = ["fftset_alloc.c", "fftset_host.c", "fftset_layout.c", "fgk_plan.c", "fftset_ragged.c", "fftset_adjoint.c", "fftset_ola.c", "fftset_tuning.c"]
HEADERS = ["fgk.h", "fgk_codelets.cuh", "fftset_layout.h", "fgk_static.cuh", "fftset_internal.h", "fgk_pingpong.cuh", "fgk_tasks.cuh", "fgk_serve.cuh"]


def _digest(paths, flags):
    h = hashlib.sha256(" ".join(flags).encode())
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def _compile(src: str, extra_dbg: bool) -> str:
    path = os.path.join(CSRC, src)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "fftset.h")]
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    if src.endswith(".cu"):
        flags = [NVCC, *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", *inc]
        if extra_dbg:
            flags += ["-Xptxas", "-v"]
    else:
        flags = ["gcc", "-O2", "-std=gnu11", "-fPIC", "-Wall", "-Wextra", *inc, "-I", os.path.join(CUDA, "include")]
    obj = os.path.join(OUT, f"{src}.{_digest([path] + hdrs, flags)}.o")
    if not os.path.exists(obj):
        r = subprocess.run(flags + ["-c", path, "-o", obj + ".tmp"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compiling {src} failed:\n{r.stdout}\n{r.stderr}")
        if extra_dbg:
            sys.stderr.write(r.stderr)
        os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), CU_SOURCES + C_SOURCES))
    stamp = os.path.join(OUT, "link.stamp")
    key = ",".join(sorted(objs))
    if not (os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == key):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart", "-lpthread", "-lm", "-ldl",
               "-Xlinker", "-rpath=" + os.path.join(CUDA, "lib64")]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"linking failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
        with open(stamp, "w") as f:
            f.write(key)
        # drop stale objects
        keep = set(objs)
        for fn in os.listdir(OUT):
            p = os.path.join(OUT, fn)
            if fn.endswith(".o") and p not in keep:
                os.remove(p)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
