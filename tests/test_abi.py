"""The C ABI: the in-tree library loads and exports every function include/nce_gb300.h declares (no GPU work)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "nce_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(?:int|void)\s+\**(nce_\w+)\s*\(", src)))


def test_header_declares_the_boundary():
    names = declared()
    for n in ("nce_ce_create", "nce_ce_energy", "nce_ce_delta", "nce_ce_run_chunk", "nce_ce_run_batch", "nce_ce_run_chunk_host",
              "nce_nce_create", "nce_nce_full_cache", "nce_nce_run_chunk", "nce_last_error", "nce_philox4x32"):
        assert n in names


def test_library_exports_every_declared_symbol():
    import ctypes
    lib_path = os.path.join(ROOT, "neuralce_gb300", "libnce_gb300.so")
    if not os.path.exists(lib_path):
        from neuralce_gb300.build import build
        build()
    lib = ctypes.CDLL(lib_path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.nce_version() >= 10000


def test_binding_signatures_cover_the_header():
    from neuralce_gb300 import _lib
    names = set(declared()) - {"nce_ce_energy_noalloc"}
    assert names <= set(_lib.SIGNATURES), names - set(_lib.SIGNATURES)


def test_device_error_flags_are_named():
    """Host decoding of a model's device error word: every set flag is named in the NceError, a clear word
    raises nothing (the C entry point is replaced by a fake that writes the word)."""
    import ctypes as C
    from neuralce_gb300 import _lib

    def fake(word):
        def fn(handle, ptr):
            C.cast(ptr, C.POINTER(C.c_int32))[0] = word
            return 0
        return fn
    _lib.raise_device_errors(fake(0), None, _lib.NCE_ERROR_FLAGS, "NeuralCE kernels")
    with pytest.raises(_lib.NceError) as e:
        _lib.raise_device_errors(fake(1 | 32), None, _lib.NCE_ERROR_FLAGS, "NeuralCE kernels")
    assert "0x21" in str(e.value) and "out of range" in str(e.value) and "tensor-core" in str(e.value)
    with pytest.raises(_lib.NceError, match="delta query"):
        _lib.raise_device_errors(fake(2), None, _lib.CE_ERROR_FLAGS, "CE kernels")
