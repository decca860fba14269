"""CPU tests of the C ABI library: it builds for sm_103a, loads, and exports
every function include/fkg.h declares. No compute calls (no GPU here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(fkg\w*)\s*\(", src)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(fkg_lib):
    from fk_mc_gb300 import _lib
    names = declared_functions()
    assert "fkg_eigh_logz" in names and "fkg_propose_accept" in names
    for nm in names:
        assert hasattr(fkg_lib, nm), f"{nm} declared in include/ but not exported"
        assert nm in _lib.SIGNATURES, f"{nm} has no ctypes binding"


def test_library_is_sm103a_only(fkg_lib):
    from fk_mc_gb300 import buildlib
    assert buildlib.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_null_context_is_rejected(fkg_lib):
    # argument checks run on the host before any CUDA call
    assert fkg_lib.fkg_set_precision(None, 0) == -1
    assert fkg_lib.fkg_last_error(None) == b"null context"
    assert fkg_lib.fkg_eigh_logz(None, 1, None, None, None, None, None, None, None, None) == -1
