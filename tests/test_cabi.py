"""The C-ABI library builds for sm_103a, loads on a CPU-only host and exports every symbol
that include/osd_gb300.h declares.  No compute calls are made here."""
import ctypes
import os
import re

from opensubdiv_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "osd_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(GB300[A-Za-z0-9]+)\s*\(", text)))


def test_header_and_python_bindings_agree():
    assert sorted(_lib.exported_symbols()) == declared_functions()


def test_library_loads_and_exports_every_declared_symbol():
    lib = _lib.load(build=True)
    for name in declared_functions():
        assert hasattr(lib, name), name
    raw = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared_functions():
        assert getattr(raw, name) is not None


def test_version_and_error_string_without_gpu():
    lib = _lib.load()
    assert lib.GB300GetVersion() >= 100
    assert isinstance(lib.GB300GetLastErrorString(), bytes)


def test_stencil_table_create_rejects_entries_outside_the_arrays():
    """Entry ranges are validated on the host before any device work: a stencil whose
    [offset, offset + size) leaves [0, nnz) is rejected with GB300_ERR_INVALID_ARGUMENT."""
    import numpy as np
    lib = _lib.load()
    sizes = np.array([2, 3], np.int32)
    idx = np.zeros(4, np.int32)
    w = np.ones(4, np.float32)
    p = lambda a: a.ctypes.data  # noqa: E731
    for offsets in (np.array([0, 2], np.int32), np.array([-1, 0], np.int32)):
        h = lib.GB300StencilTableCreate(2, 4, p(sizes), p(offsets), p(idx), p(w), None, None,
                                        None, None, None, None)
        assert not h
        assert b"outside" in lib.GB300GetLastErrorString()
