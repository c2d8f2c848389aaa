"""CPU checks of the drop-in boundary: the library builds, loads without a GPU
and exports exactly the C ABI that include/mkf_gb300.h declares."""
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names |= set(re.findall(r"\b(mkf_[a-z0-9_]+)\s*\(", txt))
    return names


def test_header_matches_binding_and_exports():
    from mkfbodytracker_pdaf_gb300 import build, _native
    build.build()
    declared = _declared()
    assert declared == set(_native.SIGNATURES), declared ^ set(_native.SIGNATURES)
    L = _native.lib()
    for name in declared:
        assert hasattr(L, name), name


def test_host_entry_points_without_gpu(olib):
    from mkfbodytracker_pdaf_gb300 import _native
    L = _native.lib()
    assert b"sm_103a" in L.mkf_version()
    out = np.zeros(4, np.uint32)
    for seed, track, frame, item, stream in [(0, 0, 0, 0, 0), (2 ** 40 + 5, 3, 7, 11, 2),
                                             (123456789, 0xFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0x100)]:
        assert L.mkf_philox_block(seed, track, frame, item, stream, out.ctypes.data) == 0
        np.testing.assert_array_equal(out, olib.draw_block(seed, track, frame, item, stream))


def test_bad_arguments_are_rejected_without_gpu():
    import ctypes as C
    from mkfbodytracker_pdaf_gb300 import _native
    L = _native.lib()
    assert L.mkf_philox_block(0, 0, 0, 0, 0, None) == 1
    assert b"null" in L.mkf_last_error()
    h = C.c_void_p()
    assert L.mkf_bpf_create(None, None, C.byref(h)) == 1


def test_product_fails_loudly_without_the_library(tmp_path):
    """No CPU fallback: with the library missing, the first call raises."""
    import subprocess
    import sys
    code = ("import mkfbodytracker_pdaf_gb300._native as N\n"
            "N.LIB_PATH = %r\n"
            "N._lib = None\n"
            "try:\n"
            "    N.lib()\n"
            "except N.MkfError as e:\n"
            "    print('raised', e)\n" % str(tmp_path / "missing.so"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=120)
    assert "raised" in r.stdout and "no CPU fallback" in r.stdout, r.stdout + r.stderr


def test_product_package_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "mkfbodytracker_pdaf_gb300")
    for fn in os.listdir(pkg):
        if fn.endswith(".py"):
            src = open(os.path.join(pkg, fn)).read()
            assert not re.search(r"^\s*(import oracle|from oracle)", src, flags=re.M), fn
