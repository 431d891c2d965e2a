"""The C-ABI library loads and exports every symbol include/gbns.h declares (no compute)."""
import ctypes
import os
import re

import pytest

from tests.conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "gbns.h")).read()
    return sorted(set(re.findall(r"^(?:int|const char \*)\s*(gbns_\w+)\(", src, re.M)))


@pytest.fixture(scope="module")
def lib():
    from jaxns_gb300.build import build_library
    build_library()
    from jaxns_gb300 import _ffi
    return _ffi.load()


def test_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_binding_lists_declared_symbols():
    from jaxns_gb300 import _ffi
    assert set(_ffi.EXPORTED) == set(_declared())


def test_abi_struct_sizes(lib):
    from jaxns_gb300 import _ffi
    out = (ctypes.c_longlong * 6)()
    assert lib.gbns_abi_sizes(out, 6) == 0
    assert list(out) == [ctypes.sizeof(c) for c in (_ffi.TermCond, _ffi.EvCalc, _ffi.RunDesc, _ffi.RunState,
                                                    _ffi.Batch, _ffi.ResultsBufs)]


def test_version_and_errors(lib):
    assert lib.gbns_version() == 1
    assert lib.gbns_batch_iterate(None, 1, None) == -1
    assert b"NULL" in lib.gbns_last_error()
