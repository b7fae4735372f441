"""Builds libfnum.so (the C ABI of include/fnum.h) in-tree with nvcc for sm_103a."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libfnum.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["fnum_kernels.cu", "fnum_host.cpp", "fnum_diag.cu", "fnum_noalloc.cu", "fnum_post.cu", "fnum_dft_tc.cu",
           "fnum_sa_tc.cu"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfnum.so")


def _newest_source_mtime() -> float:
    paths = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "fnum.h")]
    return max(os.path.getmtime(p) for p in paths)


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_source_mtime():
        return LIB
    cc = nvcc()
    common = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include")]
    with tempfile.TemporaryDirectory() as tmp:
        objs = []
        cmds = []
        for src in SOURCES:
            obj = os.path.join(tmp, src + ".o")
            objs.append(obj)
            cmds.append([cc] + common + ["-c", os.path.join(CSRC, src), "-o", obj])

        def run(cmd):
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
            if verbose:
                sys.stdout.write(r.stdout + r.stderr)

        with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
            list(ex.map(run, cmds))
        tmp_lib = os.path.join(tmp, "libfnum.so")
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(cc))), "lib64")
        run([cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp_lib] + objs +
            ["-Xlinker", "-rpath", "-Xlinker", cuda_lib])
        shutil.move(tmp_lib, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
