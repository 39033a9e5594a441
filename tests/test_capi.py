"""The C-ABI library loads (no GPU needed) and exports every symbol that
include/*.h declares; the ctypes binding covers the same set."""
import glob
import os
import re
import subprocess

import pytest

from conftest import ROOT


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*(?:[\w\s\*]+?)\b(gb_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols(gblib):
    from slothdb_gb300 import capi
    decl = _declared()
    assert len(decl) >= 15
    out = subprocess.run(["nm", "-D", "--defined-only", capi.lib_path()], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = decl - exported
    assert not missing, "declared but not exported: %s" % sorted(missing)
    for name in decl:
        assert getattr(gblib, name) is not None


def test_binding_covers_header(gblib):
    from slothdb_gb300 import capi
    decl = _declared()
    unbound = decl - set(capi.declared_symbols())
    assert not unbound, "declared but not bound in capi: %s" % sorted(unbound)


def test_abi_version(gblib):
    assert gblib.gb_abi_version() == 1


def test_invalid_spec_rejected_without_gpu_work(gblib):
    """Spec validation happens on the host before any CUDA call."""
    import ctypes as C
    from slothdb_gb300 import capi
    h = C.c_void_p()
    assert gblib.gb_agg_create(None, C.byref(h)) == 1  # GB_ERR_INVALID
    assert b"null spec" in gblib.gb_last_error()


def test_estimate_bytes_host_only(gblib):
    """gb_agg_estimate_bytes compiles the plan only (no GPU needed)."""
    from slothdb_gb300 import capi
    comp = ([capi.INTEGER, capi.SMALLINT, capi.BIGINT, capi.INTEGER], [0, 1], [("count_star", -1), ("sum", 2)])
    a = capi.estimate_bytes(*comp, nrows=10_000, est_groups=1000)
    b = capi.estimate_bytes(*comp, nrows=10_000_000, est_groups=1_000_000)
    c = capi.estimate_bytes(*comp, nrows=500, est_groups=1_000_000)   # groups bounded by rows
    assert 0 < c <= a < b
    s = capi.estimate_bytes([capi.VARCHAR, capi.BIGINT], [0], [("count_star", -1)], nrows=10_000, est_groups=1000)
    assert s > capi.estimate_bytes([capi.BIGINT, capi.BIGINT], [0], [("count_star", -1)], nrows=10_000,
                                   est_groups=1000)
    with pytest.raises(capi.GbError):
        capi.estimate_bytes([capi.VARCHAR, capi.BIGINT], [0], [("sum", 0)], nrows=10)   # SUM over VARCHAR


def test_count_distinct_plan_host_only(gblib):
    """COUNT(DISTINCT) plans compile on the host: pair sets add to the
    estimate (twice for a nullable BIGINT key); DOUBLE input and a third
    distinct column are refused."""
    from slothdb_gb300 import capi
    base = capi.estimate_bytes([capi.INTEGER, capi.BIGINT], [0], [("count_star", -1)], nrows=100_000,
                               est_groups=1000)
    d = capi.estimate_bytes([capi.INTEGER, capi.BIGINT], [0], [("count_distinct", 1)], nrows=100_000,
                            est_groups=1000)
    assert d >= base + 2 * 100_000 * 16
    dn = capi.estimate_bytes([capi.BIGINT, capi.BIGINT], [0], [("count_distinct", 1)], nrows=100_000,
                             est_groups=1000, nullable=[0])
    assert dn >= d + 2 * 100_000 * 16
    with pytest.raises(capi.GbError):
        capi.estimate_bytes([capi.INTEGER, capi.DOUBLE], [0], [("count_distinct", 1)], nrows=10)
    with pytest.raises(capi.GbError):
        capi.estimate_bytes([capi.INTEGER, capi.BIGINT, capi.BIGINT, capi.BIGINT], [0],
                            [("count_distinct", 1), ("count_distinct", 2), ("count_distinct", 3)], nrows=10)
