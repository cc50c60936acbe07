"""CPU-side checks of the C ABI library: it builds, loads, and exports every
entry point the header declares (no compute without a GPU)."""
import ctypes
import os
import re

import pytest

from radiobear_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, 'include', 'radiobear_gb300.h')) as fp:
        src = fp.read()
    return sorted(set(re.findall(r'^\s*(?:int|const char\*)\s+(rb_\w+)\s*\(', src, re.M)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert 'rb_forward' in syms and 'rb_alpha' in syms and len(syms) >= 12
    with open(os.path.join(ROOT, 'include', 'radiobear_gb300.h')) as fp:
        ver = re.search(r'#define RB_ABI_VERSION (\d+)', fp.read())
    assert ver and int(ver.group(1)) == _native.ABI_VERSION


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(_native.EXPORTS) <= set(declared_symbols())


def test_abi_version_and_error_path_without_gpu():
    lib = _native.load_library()
    assert lib.rb_abi_version() == _native.ABI_VERSION == 2
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip('a GPU is present; the no-GPU error path is not reachable')
    with pytest.raises(_native.RBError):
        _native.Engine(0)
    assert lib.rb_last_error()


def test_missing_library_fails_loudly(tmp_path):
    """The product path has no CPU fallback: without the built library the
    binding raises instead of computing anything."""
    with pytest.raises(_native.RBError, match='not built'):
        _native.load_library(str(tmp_path / 'librbgpu.so'))
    # the cached library of the other tests is untouched
    assert _native.load_library() is _native.load_library()
