"""CPU tests: the CUDA library builds for sm_103a and exports every C-ABI symbol."""
import ctypes
import os
import re

from movfem_gb300 import api, build

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared():
    names = set()
    for f in os.listdir(HDR):
        if f.endswith(".h"):
            txt = open(os.path.join(HDR, f)).read()
            names |= set(re.findall(r"\b(mvf_[a-z_0-9]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(declared()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(api.EXPORTS) <= declared()


def test_header_compiles_as_c():
    import subprocess
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        open(src, "w").write('#include "movfem_gpu.h"\nint main(void){mvf_mesh m; (void)m; return 0;}\n')
        subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", HDR, "-c", src, "-o", os.path.join(d, "t.o")])
