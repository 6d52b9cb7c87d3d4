"""The C-ABI library loads, exports every entry point include/*.h declares,
and reports errors as status codes (no compute calls: these run without a GPU)."""
import ctypes
import os

import pytest


def test_library_exports_every_declared_symbol(axbc):
    L = axbc.lib()
    names = axbc.exported_symbols()
    assert "axbc_run_batch" in names and "scan_col_csc_cuda_mono" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_in_tree(axbc):
    assert os.path.dirname(axbc.LIB_PATH) == os.path.dirname(os.path.abspath(axbc.__file__))
    assert os.path.exists(axbc.LIB_PATH)


def test_status_strings(axbc):
    L = axbc.lib()
    assert L.axbc_status_str(0) == b"ok"
    assert L.axbc_status_str(4) == b"device wait timed out"
    assert axbc.version().startswith("axbc_gb300")


def test_null_arguments_return_invalid(axbc):
    L = axbc.lib()
    assert L.axbc_graph_info(None, None, None, None, None) == 1
    assert b"null" in L.axbc_last_error()
    assert L.axbc_run_pivot(None, 0, 1.0, 0, None) == 1
    assert L.axbc_ctx_destroy(None) == 0


def test_headers_compile_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "axbc.h"\n#include "axbc_compat.h"\nint main(void){return AXBC_OK;}\n')
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    import subprocess
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", inc, str(src), "-o",
                        str(tmp_path / "t")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
