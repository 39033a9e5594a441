"""The C-ABI library loads (no GPU needed) and exports every symbol that
include/*.h declares; the ctypes binding covers the same set."""
import glob
import os
import re
import subprocess

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
