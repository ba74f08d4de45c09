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
    return sorted(set(re.findall(r"\b(GB300[A-Za-z]+)\s*\(", text)))


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
