"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every symbol that
include/pibronic_gb300.h declares (no compute calls here)."""
import ctypes
import os
import re

from conftest import REPO


def declared_symbols():
    text = open(os.path.join(REPO, "include", "pibronic_gb300.h")).read()
    return sorted(set(re.findall(r"^(?:int|int32_t|int64_t|const char\*)\s+(pbr_\w+)\(", text, re.M)))


def test_header_declares_the_binding_list():
    from pibronic_gb300 import _native
    assert declared_symbols() == sorted(_native.EXPORTED)


def test_library_builds_and_exports_all_symbols():
    from pibronic_gb300 import build, _native
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    lib = _native.load(path)
    assert b"sm_103a" in lib.pbr_version()


def test_product_path_fails_loudly_without_cuda():
    import torch
    from pibronic_gb300 import _native
    if torch.cuda.is_available():
        return
    try:
        _native.require_cuda()
    except RuntimeError as err:
        assert "no CPU fallback" in str(err)
    else:
        raise AssertionError("require_cuda must raise without a device")


def test_calls_with_a_wrong_argument_count_are_rejected():
    """ctypes would pass a surplus argument on silently; the loaded library refuses it before
    anything reaches the native code."""
    import pytest
    from pibronic_gb300 import build, _native
    lib = _native.load(build.build())
    assert lib.pbr_version() is not None
    with pytest.raises(TypeError):
        lib.pbr_version(0)
    with pytest.raises(TypeError):
        lib.pbr_reduce_blocks()
