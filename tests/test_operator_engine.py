"""The C++ operator compiled against SlothDB's own headers and linked with
the engine built from the reference's sources (oracle/ref.mk): the program
feeds PhysicalGpuHashAggregate engine DataChunks and compares its result
with the engine's own GROUP BY of the same rows (tests/cpp/
engine_operator_check.cpp).  Runs where the reference's sources are; without
a CUDA device the operator reports the missing device after the engine's
query ran, which still proves it builds and links against the engine."""
import os
import subprocess

import pytest

from oracle import reference

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "slothdb_gb300", "_build")


def test_operator_against_engine_headers(tmp_path):
    src = reference.reference_source()
    if src is None:
        pytest.skip("the reference's sources are not here")
    reference.build()
    lib = os.path.join(reference.REF_DIR, "libslothdb_ref.a")
    from slothdb_gb300 import build as gbuild
    gbuild.build_lib()
    objs = sorted(os.path.join(BUILD, n) for n in os.listdir(BUILD)
                  if n.endswith(".o") and not n.startswith("gpu_operator"))
    cxx = os.environ.get("CXX", "g++")
    flags = ["-std=c++20", "-O1", "-DSLOTHDB_GB300_ENGINE_HEADERS", "-I", os.path.join(src, "include"),
             "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "slothdb_gb300", "operator")]
    op_o, drv_o, exe = str(tmp_path / "op.o"), str(tmp_path / "drv.o"), str(tmp_path / "check")
    for s, o in ((os.path.join(ROOT, "slothdb_gb300", "operator", "gpu_operator.cpp"), op_o),
                 (os.path.join(ROOT, "tests", "cpp", "engine_operator_check.cpp"), drv_o)):
        p = subprocess.run([cxx] + flags + ["-c", s, "-o", o], capture_output=True, text=True)
        assert p.returncode == 0, p.stderr[-3000:]
    cuda_lib = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "lib64")
    p = subprocess.run([cxx, "-o", exe, drv_o, op_o] + objs + [lib, "-L", cuda_lib, "-lcudart_static", "-lpthread",
                                                               "-ldl", "-lrt"], capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-3000:]
    p = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    lines = p.stdout.splitlines()
    assert lines[0].startswith("engine: 3 groups over 10000 rows"), p.stdout
    assert all(("equal: 3 groups" in ln) or ln.startswith("no device") for ln in lines[1::2]), p.stdout
    assert len(lines) == 4, p.stdout
