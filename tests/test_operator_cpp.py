"""The C++ operator mirror (PhysicalGpuHashAggregate over the C ABI): the
test program builds here (no GPU needed) and passes on the GPU."""
import subprocess

import pytest

from slothdb_gb300 import build


def test_operator_test_program_builds():
    exe = build.build_operator_test()
    assert exe.endswith("test_gpu_operator")


@pytest.mark.gpu
def test_operator_test_program_passes():
    exe = build.build_operator_test()
    p = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "all operator tests passed" in p.stdout
