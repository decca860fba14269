"""CPU tests of the C ABI libraries: they build (sm_103a for the CUDA one),
load, and export every function the headers in include/ declare. No compute
calls (no GPU here)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"typedef struct \w+ \{.*?\}\s*\w+;", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b((?:fkg|fkh)\w*)\s*\(", src)))


def test_headers_are_covered():
    assert sorted(os.listdir(os.path.join(ROOT, "include"))) == ["fk_mc_host.h", "fkg.h"]


def test_fkg_exports_every_declared_symbol(fkg_lib):
    from fk_mc_gb300 import _lib
    names = declared_functions("fkg.h")
    assert "fkg_eigh_logz" in names and "fkg_propose_accept" in names
    for nm in names:
        assert hasattr(fkg_lib, nm), f"{nm} declared in include/fkg.h but not exported"
        assert nm in _lib.SIGNATURES, f"{nm} has no ctypes binding"


def test_host_adapter_exports_every_declared_symbol(fkg_lib):
    from fk_mc_gb300 import host_lib, stats
    h = host_lib.load()
    names = declared_functions("fk_mc_host.h")
    assert names == ["fkh_binning", "fkh_estimate_bin", "fkh_graph_lattice_csr", "fkh_jackknife",
                     "fkh_measure_eigen", "fkh_run_batched", "fkh_run_chain", "fkh_run_chain_graph",
                     "fkh_save_stats"]
    for nm in names:
        assert hasattr(h, nm) and (nm in host_lib.SIGNATURES or nm in stats.SIGNATURES), nm


def test_library_is_sm103a_only(fkg_lib):
    from fk_mc_gb300 import buildlib
    assert buildlib.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_null_context_is_rejected(fkg_lib):
    # argument checks run on the host before any CUDA call
    assert fkg_lib.fkg_set_precision(None, 0) == -1
    assert fkg_lib.fkg_last_error(None) == b"null context"
    assert fkg_lib.fkg_eigh_logz(None, 1, None, None, None, None, None, None, None, None) == -1
