"""The C ABI library: loads on any host, exports every symbol the header
declares, and refuses to run without a device instead of falling back."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "mfem_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*|void)\s*\*?\s*(mfem_\w+)\s*\(", hdr,
                                 flags=re.M)))


def test_every_declared_symbol_is_exported():
    from minifem import _native
    lib = ctypes.CDLL(_native.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    # and the Python binding covers all of them
    assert set(names) <= set(_native.exported_symbols())


def test_abi_version():
    from minifem import _native
    assert _native.lib.mfem_abi_version() == 1


def test_no_device_means_error_not_fallback():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    import minifem
    with pytest.raises(minifem.MfemError):
        minifem.Assembler(0)


def test_null_context_is_rejected():
    from minifem import _native
    assert _native.lib.mfem_assemble(None, 0, 0, 0) == -1
    assert _native.lib.mfem_destroy(None) == -1
