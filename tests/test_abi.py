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
    from pyscaledvecchia_gb300 import _lib
    assert lib.sv_abi_version() == _lib.ABI_VERSION
    assert lib.sv_status_string(0) == b"ok"
    assert b"Cholesky" in lib.sv_status_string(2)


def test_library_is_sm103a_only():
    from pyscaledvecchia_gb300 import _build
    assert _build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_side_stream_and_host_memory_flag_are_per_device(monkeypatch):
    """The library's side stream and the host-memory answer are kept per
    device (stand-ins for torch and the library: no CUDA call)."""
    import ctypes
    from pyscaledvecchia_gb300 import _lib

    class FakeStream:
        def __init__(self, device=None):
            self.device = device

    class Cuda:
        dev = 0
        Stream = FakeStream

        def current_device(self):
            return self.dev

    class Torch:
        cuda = Cuda()

    class Lib:
        answers = {0: 1, 1: 0}
        calls = []

        def sv_device_reads_host_memory(self, ref):
            Lib.calls.append(Torch.cuda.dev)
            ref._obj.value = Lib.answers[Torch.cuda.dev]
            return _lib.SV_OK

    monkeypatch.setattr(_lib, "_SIDE", {})
    monkeypatch.setattr(_lib, "_HOST_READABLE", None)
    monkeypatch.setattr(_lib, "_HOST_READABLE_DEV", {})
    monkeypatch.setattr(_lib, "_torch", lambda: Torch)
    t, lib = Torch(), Lib()
    s0 = _lib.side_stream(t)
    assert s0.device == 0 and _lib.side_stream(t) is s0
    assert _lib.device_reads_host_memory(lib) is True
    assert _lib.device_reads_host_memory(lib) is True
    Torch.cuda.dev = 1
    s1 = _lib.side_stream(t)
    assert s1 is not s0 and s1.device == 1
    assert _lib.device_reads_host_memory(lib) is False
    assert Lib.calls == [0, 1]
    monkeypatch.setattr(_lib, "_HOST_READABLE", True)  # fixed answer: no query
    assert _lib.device_reads_host_memory(lib) is True
    assert Lib.calls == [0, 1]
    Torch.cuda.dev = 0


def test_structure_layouts_match_the_header(tmp_path):
    """Every ctypes mirror in _lib has the size and field offsets that a C
    compiler gives the header's structure."""
    import ctypes
    import shutil
    import subprocess

    from pyscaledvecchia_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"sv_loglik_desc": _lib.LoglikDesc, "sv_prob_desc": _lib.ProbDesc,
             "sv_batch_desc": _lib.BatchDesc, "sv_reorder_prob": _lib.ReorderProb,
             "sv_pack_group": _lib.PackGroup, "sv_chunk_group": _lib.ChunkGroup,
             "sv_reorder_desc": _lib.ReorderDesc, "sv_pred_desc": _lib.PredDesc}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "svgpu.h"', "int main(void) {"]
    expect = []
    for cname, py in pairs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(ctypes.sizeof(py))
        for fname, _ in py._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {fname}));')
            expect.append(getattr(py, fname).offset)
    lines += ["  printf(\"%d\\n\", SV_ABI_VERSION);", "  return 0;", "}"]
    expect.append(_lib.ABI_VERSION)
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got == expect
