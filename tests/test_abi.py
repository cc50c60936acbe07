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
    assert lib.rb_abi_version() == _native.ABI_VERSION == 3
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


def test_header_is_plain_c99_and_links(tmp_path):
    """A C caller (cgo, N-API, a C application) includes the header under
    strict C99 and links every entry point against the library."""
    import shutil
    import subprocess
    if shutil.which('gcc') is None:
        pytest.skip('gcc not available')
    lib = build.build()
    syms = declared_symbols()
    src = tmp_path / 'caller.c'
    src.write_text(
        '#include "radiobear_gb300.h"\n#include <stdio.h>\n'
        'typedef void (*rb_fn)(void);\n'
        'int main(void) {\n  const rb_fn entry[] = {\n' +
        ''.join('    (rb_fn)&{},\n'.format(s) for s in syms) +
        '  };\n  printf("%d %d\\n", (int)(sizeof entry / sizeof entry[0]), rb_abi_version());\n'
        '  return 0;\n}\n')
    exe = tmp_path / 'caller'
    libdir = os.path.dirname(lib)
    r = subprocess.run(['gcc', '-std=c99', '-Wall', '-Wextra', '-Werror', '-pedantic',
                        '-I' + os.path.join(ROOT, 'include'), str(src), '-o', str(exe),
                        '-L' + libdir, '-l' + os.path.basename(lib)[3:-3],
                        '-Wl,-rpath,' + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == [str(len(syms)), str(_native.ABI_VERSION)]
