"""Builds the oracle's native parts.

TEST INFRASTRUCTURE ONLY.
* oracle/liboracle.so: the C restatement (gcc + OpenMP; portable C, builds on
  x86_64 and aarch64).
* oracle/_ref/ref_kernels.fatbin: the reference's own CUDA kernels compiled
  from their sources in the reference checkout's +cuda directory (device code
  for sm_103a only; built where the reference is mounted, then shipped with the
  tree).  The checkout is $FNUM_REFERENCE_ROOT, or ``--reference DIR``, by
  default /root/reference.
* oracle/_ref/libref_harness.so: the project-written host driver that runs
  those kernels with the MEX host sequence (nvcc; built wherever the fatbin
  and a CUDA toolkit are present).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "fnum_oracle.c")
REF_DIR = os.path.join(HERE, "_ref")
FATBIN = os.path.join(REF_DIR, "ref_kernels.fatbin")
HARNESS = os.path.join(REF_DIR, "libref_harness.so")
REFERENCE_ROOT = os.environ.get("FNUM_REFERENCE_ROOT", "/root/reference")
REFERENCE_CUDA = os.path.join(REFERENCE_ROOT, "+cuda")
TU = os.path.join(HERE, "ref_harness", "ref_kernels_tu.cu")
DRIVER = os.path.join(HERE, "ref_harness", "ref_driver.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, *srcs):
    return not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs)


def _nvcc():
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    return None


def build_c(force=False):
    if force or _stale(LIB, SRC):
        _run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", SRC, "-o", LIB, "-lm"])
    return LIB


def build_ref(force=False, reference_cuda=None):
    """Reference kernels (only where the reference sources are mounted) and the
    harness driver (wherever the fatbin exists).  Returns the harness path or None."""
    nv = _nvcc()
    if nv is None:
        return None
    ref_cuda = reference_cuda or REFERENCE_CUDA
    os.makedirs(REF_DIR, exist_ok=True)
    if os.path.isdir(ref_cuda) and (force or _stale(FATBIN, TU)):
        _run([nv, "-fatbin"] + ARCH + ["-I", ref_cuda, TU, "-o", FATBIN])
    if not os.path.exists(FATBIN):
        return None
    if force or _stale(HARNESS, DRIVER):
        _run([nv, "-O2", "-std=c++17", "-shared", "-Xcompiler", "-fPIC"] + ARCH +
             [DRIVER, "-o", HARNESS, "-lcuda", "-lcufft", "-lcublas"])
    return HARNESS


def build(force=False, reference_root=None):
    build_c(force)
    try:
        build_ref(force, os.path.join(reference_root, "+cuda") if reference_root else None)
    except RuntimeError as e:  # the checker's optional half: report, do not stop the product build
        sys.stderr.write("reference harness not built: %s\n" % e)
    return LIB


if __name__ == "__main__":
    root = None
    if "--reference" in sys.argv:
        root = sys.argv[sys.argv.index("--reference") + 1]
    print(build(force="--force" in sys.argv, reference_root=root))
