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


def declared_arities():
    """name -> number of parameters, from the prototypes in the header."""
    src = open(os.path.join(ROOT, "include", "svgpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"\b(sv_[a-zA-Z0-9_]+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_binding_argument_counts_match_the_prototypes():
    from pyscaledvecchia_gb300 import _lib
    ar = declared_arities()
    assert set(ar) == set(_lib.SIGNATURES)
    for name, (_, argtypes) in _lib.SIGNATURES.items():
        assert len(argtypes) == ar[name], (name, len(argtypes), ar[name])


def test_status_strings(lib):
    assert lib.sv_abi_version() == 1
    assert lib.sv_status_string(0) == b"ok"
    assert b"Cholesky" in lib.sv_status_string(2)


def test_library_is_sm103a_only():
    from pyscaledvecchia_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
