"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every
symbol that include/parament.h declares, and its host-only functions agree
with the reference's (order tables, norm bound, error strings)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "parament.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"PARAMENT_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)))


def test_header_declares_reference_abi():
    names = declared_symbols()
    for ref in ["Parament_create", "Parament_destroy", "Parament_setHamiltonian", "Parament_equiprop",
                "Parament_selectIterationCycles_fp32", "Parament_setIterationCyclesManually",
                "Parament_automaticIterationCycles", "Parament_peekAtLastError", "Parament_errorMessage",
                "Parament_create_fp64", "Parament_destroy_fp64", "Parament_setHamiltonian_fp64",
                "Parament_equiprop_fp64", "Parament_setIterationCyclesManually_fp64",
                "Parament_automaticIterationCycles_fp64", "Parament_peekAtLastError_fp64",
                "Parament_selectIterationCycles_fp64", "OneNorm", "OneNorm_fp64", "device_info"]:
        assert ref in names


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_order_tables(built_lib, ref_host):
    lib = ctypes.CDLL(built_lib)
    for n in ("Parament_selectIterationCycles_fp32", "Parament_selectIterationCycles_fp64"):
        getattr(lib, n).argtypes = [ctypes.c_double, ctypes.c_double]
    for x, m32, m64 in ref_host["cycles"]:
        assert lib.Parament_selectIterationCycles_fp32(x, 1.0) == m32
        assert lib.Parament_selectIterationCycles_fp64(x, 1.0) == m64


def test_error_messages(built_lib, ref_host):
    lib = ctypes.CDLL(built_lib)
    lib.Parament_errorMessage.argtypes = [ctypes.c_int]
    lib.Parament_errorMessage.restype = ctypes.c_char_p
    for code, msg in ref_host["messages"].items():
        assert lib.Parament_errorMessage(int(code)).decode() == msg


def test_onenorm(built_lib, ref_host):
    lib = ctypes.CDLL(built_lib)
    lib.OneNorm.argtypes = [np.ctypeslib.ndpointer(np.complex64), ctypes.c_uint]
    lib.OneNorm.restype = ctypes.c_double
    lib.OneNorm_fp64.argtypes = [np.ctypeslib.ndpointer(np.complex128), ctypes.c_uint]
    lib.OneNorm_fp64.restype = ctypes.c_double
    for n in ref_host["norms"]:
        d = n["d"]
        m = (np.array(n["re"]) + 1j * np.array(n["im"])).reshape(d, d)
        assert lib.OneNorm_fp64(np.ascontiguousarray(m.ravel()), d) == pytest.approx(n["onenorm_fp64"], rel=1e-15)
        m32 = np.ascontiguousarray(m.astype(np.complex64).ravel())
        assert lib.OneNorm(m32, d) == pytest.approx(n["onenorm_fp32"], rel=1e-6)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device path")
def test_create_without_device_reports_init_failure(built_lib):
    import parament_gb300 as parament
    with pytest.raises(RuntimeError, match="Error code 30"):
        parament.Parament()
    with pytest.raises(RuntimeError, match="Error code 30"):
        parament.Parament("fp64")


def test_wrapper_rejects_bad_precision(built_lib):
    import parament_gb300 as parament
    with pytest.raises(ValueError, match="precision must be either"):
        parament.Parament("fp16")


def test_sample_packing_passes_contiguous_rows_through():
    """equiprop's sample packing: rows of one C-contiguous array of the
    context's type go through without a copy; anything else is copied and
    converted, with the same values."""
    from parament_gb300.parament import _pack_samples
    rng = np.random.default_rng(3)
    base = np.ascontiguousarray((rng.standard_normal((3, 50)) + 1j * rng.standard_normal((3, 50))).astype(np.complex64))
    packed = _pack_samples(tuple(base), np.complex64, 3, 50)
    assert np.shares_memory(packed, base) and np.array_equal(packed, base.ravel())
    # another type, a subset of rows, reordered rows, separate arrays: copies
    for carr in (tuple(base[:2]), (base[1], base[0], base[2]), tuple(np.array(r) for r in base)):
        for ctype in (np.complex64, np.complex128):
            out = _pack_samples(carr, ctype, len(carr), 50)
            assert out.dtype == ctype and out.flags.c_contiguous and not np.shares_memory(out, base)
            assert np.array_equal(out, np.concatenate([np.asarray(c, ctype) for c in carr]))
    out = _pack_samples(tuple(base), np.complex128, 3, 50)
    assert not np.shares_memory(out, base) and np.array_equal(out, base.ravel().astype(np.complex128))
