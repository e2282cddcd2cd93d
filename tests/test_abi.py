"""The C ABI library loads and exports every entry point include/svgpu.h
declares (no GPU needed: nothing here launches a kernel)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "svgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sv_[a-zA-Z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from pyscaledvecchia_gb300 import _build, _lib
    _build.build()
    return _lib.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 20
    for nm in names:
        assert hasattr(lib, nm), nm


def test_binding_table_covers_the_header():
    from pyscaledvecchia_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_status_strings(lib):
    assert lib.sv_abi_version() == 1
    assert lib.sv_status_string(0) == b"ok"
    assert b"Cholesky" in lib.sv_status_string(2)


def test_library_is_sm103a_only():
    from pyscaledvecchia_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
