"""CPU-side checks of the drop-in boundary: the C-ABI library builds, loads
and exports every entry point include/adeco_deposit.h declares (no compute
calls without a GPU), and the C++ shim header compiles against it."""
import ctypes
import os
import subprocess

import pytest

from adeco_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from adeco_gb300 import build
    build.build()
    return L.load()


def test_header_declares_entry_points():
    names = L.declared_symbols()
    for expected in ("adeco_deposit_tets", "adeco_deposit_tets_ex", "adeco_session_create",
                     "adeco_session_build_octree", "adeco_session_deposit_leaves", "adeco_session_submit"):
        assert expected in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in L.declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_bindings_cover_every_declared_symbol():
    assert set(L.declared_symbols()) <= set(L._SIGS), set(L.declared_symbols()) - set(L._SIGS)


def test_abi_version(lib):
    assert lib.adeco_abi_version() == 1


def test_last_error_is_empty_string_initially(lib):
    assert isinstance(lib.adeco_last_error(), bytes)


def test_cpp_wrapper_header_compiles(tmp_path):
    src = tmp_path / "use_wrapper.cpp"
    src.write_text('#include "adeco_deposit_wrapper.hpp"\n'
                   'int main(){ float d[8]={0}; const float bb[6]={0,1,0,1,0,1};\n'
                   '  try { AdaptiveMassDeposit::DepositWrapper::deposit_tets(false,0,0,0,nullptr,0,7,bb,2,d); }\n'
                   '  catch (const AdaptiveMassDeposit::AdRuntimeException&) { return 1; }\n'
                   '  return 0; }\n')
    r = subprocess.run(["g++", "-std=c++11", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
