"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports every entry point
declared in include/*.h; the ctypes table covers the same set. No compute calls (no GPU here)."""
import glob
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, 'include', '*.h')):
        txt = open(h).read()
        names |= set(re.findall(r'^\s*int\s+(ocmp_\w+)\s*\(', txt, re.M))
    return names


@pytest.fixture(scope='module')
def lib_path():
    from opencmp_gb300 import build
    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(['nm', '-D', '--defined-only', lib_path], capture_output=True, text=True).stdout
    exported = set(re.findall(r'\sT\s+(ocmp_\w+)', out))
    missing = declared() - exported
    assert not missing, missing
    assert len(declared()) >= 20


def test_library_loads_and_ctypes_table_complete(lib_path):
    from opencmp_gb300 import _lib
    L = _lib.load()
    assert L.ocmp_abi_version() == 1
    assert declared() <= set(_lib.SIGNATURES), declared() - set(_lib.SIGNATURES)


def test_errors_do_not_cross_the_abi(lib_path):
    from opencmp_gb300 import _lib
    import ctypes as C
    L = _lib.load()
    h = C.c_void_p()
    st = L.ocmp_space_create(None, 0, 2, 0, C.byref(h))
    assert st == _lib.ERR_ARG
    assert 'null' in _lib.last_error()
    st = L.ocmp_mesh_create(None, 0, 2, None, 0, None, None, 0, C.byref(h))
    assert st == _lib.ERR_ARG
