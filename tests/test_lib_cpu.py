"""CPU checks of the C ABI: the library loads, exports every entry point
declared in include/mpet_gpu.h, and the ctypes struct layouts match C."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "mpet_gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mpet_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from waterscapes_gb300 import build
    build.build()
    from waterscapes_gb300 import _lib
    return _lib.load()


def test_library_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_every_declared_symbol():
    from waterscapes_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_struct_layout_matches_c():
    from waterscapes_gb300 import _lib
    src = r'''
#include <stdio.h>
#include <stddef.h>
#include "mpet_gpu.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(mpet_params), offsetof(mpet_params, theta),
         offsetof(mpet_params, check_every), sizeof(mpet_stats), offsetof(mpet_stats, relres_true));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    P, S = _lib.MpetParams, _lib.MpetStats
    assert int(out[0]) == ctypes.sizeof(P)
    assert int(out[1]) == P.theta.offset
    assert int(out[2]) == P.check_every.offset
    assert int(out[3]) == ctypes.sizeof(S)
    assert int(out[4]) == S.relres_true.offset


def test_context_creation_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from waterscapes_gb300 import _lib
    with pytest.raises(_lib.MpetError):
        _lib.Context(0)
