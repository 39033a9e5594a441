"""Build recipe for the GB300 GROUP BY library and the CPU oracle.

``build_lib()`` compiles every CUDA/C++ source under ``slothdb_gb300/csrc``
for sm_103a with nvcc (translation units compiled in parallel) and links
``slothdb_gb300/_build/libslothdb_gb300.so`` in-tree.  ``build_oracle()``
compiles the oracle C sources with gcc into ``oracle/_build/liboracle.so``.
Both are idempotent: a target newer than all its sources is not rebuilt.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "slothdb_gb300")
CSRC = os.path.join(PKG, "csrc")
OPDIR = os.path.join(PKG, "operator")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libslothdb_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_BUILD, "liboracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit")


def _sources(exts):
    out = []
    for d in (CSRC, OPDIR):
        for name in sorted(os.listdir(d)):
            if os.path.splitext(name)[1] in exts:
                out.append(os.path.join(d, name))
    return out


def _headers():
    hs = [os.path.join(ROOT, "include", n) for n in os.listdir(os.path.join(ROOT, "include"))]
    for d in (CSRC, OPDIR):
        hs += [os.path.join(d, n) for n in os.listdir(d) if n.endswith((".h", ".cuh", ".hpp"))]
    return hs


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    return p


def build_lib(verbose: bool = False, force: bool = False) -> str:
    srcs = _sources({".cu", ".cpp"})
    deps = srcs + _headers() + [os.path.abspath(__file__)]
    if not force and _newer(LIB, deps):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + inc + ["-c", src, "-o", obj]
        if src.startswith(OPDIR):  # host-only C++ over the C ABI
            cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC"] + inc + ["-c", src, "-o", obj]
        elif src.endswith(".cpp"):
            cmd = [nvcc, "-x", "cu"] + ARCH + NVCC_FLAGS + inc + ["-c", src, "-o", obj]
        _run(cmd)
        if verbose:
            print("compiled", os.path.basename(src), file=sys.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(srcs)))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    _run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static", "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    return LIB


OPERATOR_TEST = os.path.join(BUILD, "test_gpu_operator")


def build_operator_test(force: bool = False) -> str:
    """The C++ test program of the operator mirror (tests/cpp), linked
    against the library."""
    src = os.path.join(ROOT, "tests", "cpp", "test_gpu_operator.cpp")
    lib = build_lib()
    deps = [src, lib, os.path.join(OPDIR, "gpu_operator.hpp")]
    if not force and _newer(OPERATOR_TEST, deps):
        return OPERATOR_TEST
    tmp = OPERATOR_TEST + ".tmp"
    _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), "-I", OPDIR, src,
          "-o", tmp, "-L", BUILD, "-lslothdb_gb300", "-Wl,-rpath," + BUILD, "-lpthread"])
    os.replace(tmp, OPERATOR_TEST)
    return OPERATOR_TEST


def build_oracle(force: bool = False) -> str:
    srcs = [os.path.join(ORACLE_DIR, n) for n in sorted(os.listdir(ORACLE_DIR)) if n.endswith(".c")]
    if not force and _newer(ORACLE_LIB, srcs + [os.path.abspath(__file__)]):
        return ORACLE_LIB
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    tmp = ORACLE_LIB + ".tmp"
    _run([cc, "-O2", "-std=c11", "-fPIC", "-shared", "-pthread", "-o", tmp] + srcs + ["-lm"])
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_lib(verbose=True, force="--force" in sys.argv))
    print(build_oracle(force="--force" in sys.argv))
