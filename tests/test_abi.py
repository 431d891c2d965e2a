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


def _prototypes():
    """{name: [C parameter types]} of every int-returning entry point in include/gbns.h."""
    src = open(os.path.join(ROOT, "include", "gbns.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    out = {}
    for name, params in re.findall(r"^int\s+(gbns_\w+)\(([^)]*)\);", src, re.M):
        ps = [p.strip() for p in params.replace("\n", " ").split(",") if p.strip() and p.strip() != "void"]
        out[name] = [re.sub(r"\s*\b\w+$", "", p) if "*" not in p.split()[-1] else p for p in ps]
    return out


def _null_args(types):
    args = []
    for t in types:
        if "*" in t:
            args.append(ctypes.c_void_p(None))
        elif "double" in t:
            args.append(ctypes.c_double(0.0))
        elif "long long" in t:
            args.append(ctypes.c_longlong(0))
        else:
            args.append(ctypes.c_int(0))
    return args


NO_ARGUMENT_CHECK = {"gbns_version", "gbns_abi_sizes"}


@pytest.mark.parametrize("name", sorted(set(_prototypes()) - NO_ARGUMENT_CHECK))
def test_null_arguments_are_rejected_before_any_cuda_call(lib, name):
    """NULL pointers and zero sizes give -1 and a message naming the argument problem; the
    checks run on the host before any CUDA call, so no device is needed."""
    rc = getattr(lib, name)(*_null_args(_prototypes()[name]))
    msg = lib.gbns_last_error().decode()
    assert rc == -1, (name, rc, msg)
    assert msg and "CUDA" not in msg and "cuda" not in msg, (name, msg)


def test_batch_field_checks(lib):
    from jaxns_gb300 import _ffi
    runs = (_ffi.RunDesc * 1)()
    state = (_ffi.RunState * 1)()
    ncoef = (ctypes.c_double * 8)()
    b = _ffi.Batch()
    b.num_runs = 0
    assert lib.gbns_batch_iterate(ctypes.byref(b), 1, None) == -1
    assert b"no runs" in lib.gbns_last_error()
    b.num_runs, b.runs, b.state, b.ncoef = 1, ctypes.cast(runs, ctypes.c_void_p), ctypes.cast(state, ctypes.c_void_p), \
        ctypes.cast(ncoef, ctypes.c_void_p)
    b.nmax, b.ncoef_n, b.chains_per_item = 8, 8, 48
    assert lib.gbns_batch_iterate(ctypes.byref(b), 1, None) == -1
    assert b"multiple of 32" in lib.gbns_last_error()
    b.chains_per_item, b.nmax = 64, 5000
    assert lib.gbns_batch_iterate(ctypes.byref(b), 1, None) == -1
    assert b"nmax" in lib.gbns_last_error()
    b.nmax, b.ncoef_n = 8, 4
    assert lib.gbns_batch_iterate(ctypes.byref(b), 1, None) == -1
    assert b"ncoef" in lib.gbns_last_error()
    b.ncoef_n = 8
    assert lib.gbns_batch_iterate(ctypes.byref(b), -1, None) == -1
    assert b"negative" in lib.gbns_last_error()
    lg = _ffi.LGBufs()
    assert lib.gbns_lg_steps(ctypes.byref(b), ctypes.byref(lg), 1, None) == -1
    assert b"pmax" in lib.gbns_last_error()


def test_size_limits(lib):
    k = (ctypes.c_uint32 * 2)()
    out = (ctypes.c_uint32 * 2)()
    for fn in ("gbns_threefry_split", "gbns_random_bits64", "gbns_uniform", "gbns_normal"):
        assert getattr(lib, fn)(k, out, ctypes.c_longlong(1 << 32), None) == -1, fn
        assert getattr(lib, fn)(k, out, ctypes.c_longlong(-1), None) == -1, fn
    assert lib.gbns_count_crossed_edges_static(None, None, ctypes.c_longlong(262144), out, out, None) == -1
    assert b"262143" in lib.gbns_last_error()


def test_binding_matches_header():
    """jaxns_gb300.binding declares every symbol of the header with the header's argument
    kinds (pointer / int / long long / double)."""
    from jaxns_gb300.binding import ARGTYPES
    protos = dict(_prototypes(), gbns_last_error=[])
    assert set(ARGTYPES) == set(protos) == set(_declared())

    def kind(t):
        if "*" in t:
            return ctypes.c_void_p
        return {"double": ctypes.c_double, "long long": ctypes.c_longlong,
                "int": ctypes.c_int}[t.replace("const ", "").strip()]

    for name, types in protos.items():
        assert ARGTYPES[name] == [kind(t) for t in types], name


def test_binding_runs(lib):
    """The binding loads the built library and its error paths answer through it."""
    from jaxns_gb300.binding import bind
    b = bind(lib._name)
    assert b.gbns_version() == 1
    assert b.gbns_batch_iterate(None, 1, None) == -1
    assert b"NULL" in b.gbns_last_error()
    assert b.gbns_evidence_adjoint_tc(None, None, 0, 0, None, None, 0, 0.0, 0.0, None, None, None, None,
                                      None, None, None) == -1


def test_header_and_library_from_plain_c(lib, tmp_path):
    """include/gbns.h compiles as C (gcc -std=c99) and the C program links and runs against the
    built library: sizes seen by a C compiler equal the library's own."""
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    libdir = os.path.dirname(lib._name)
    exe = str(tmp_path / "abi_from_c")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_from_c.c"), "-L", libdir, "-lgbns",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True, capture_output=True, text=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, (out.returncode, out.stderr)
    assert out.stdout.startswith("ok 1 ")
