"""In-tree build of the native library ``libtqec_gb300.so`` (sm_103a).

Each translation unit under ``csrc/`` is compiled by nvcc in parallel into
``_build/`` and the objects are linked into the shared library next to this
file.  Only a CUDA toolkit with sm_103a support is needed (no torch, no
cmake); the same recipe runs on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtqec_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
         "--expt-relaxed-constexpr"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtqec_gb300.so")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                  if f.endswith((".cu", ".cpp")))


def build(verbose: bool = False, extra_flags=None) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "tqec_gb300.h"))
    newest_header = max(os.path.getmtime(h) for h in headers if os.path.exists(h))
    extra = list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        if (os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(src)
                and os.path.getmtime(obj) >= newest_header and not extra):
            return obj
        cmd = [nvcc, *ARCH, *FLAGS, *extra, "-I", CSRC, "-c", src, "-o", obj]
        if src.endswith(".cpp"):
            cmd[len([nvcc, *ARCH, *FLAGS, *extra]):len([nvcc, *ARCH, *FLAGS, *extra])] = ["-x", "cu"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if (not os.path.exists(LIB) or extra
            or max(os.path.getmtime(o) for o in objs) > os.path.getmtime(LIB)):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, extra_flags=sys.argv[1:]))
