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


def test_mesh_struct_layout_matches_the_header():
    """The ctypes mirror of mvf_mesh has the C struct's size and field offsets."""
    import subprocess
    import tempfile
    fields = [f for f, _ in api._Mesh._fields_]
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        body = "".join(f'printf("%zu\\n", offsetof(mvf_mesh, {f}));' for f in fields)
        open(src, "w").write('#include <stddef.h>\n#include <stdio.h>\n#include "movfem_gpu.h"\n'
                             'int main(void){printf("%zu\\n", sizeof(mvf_mesh));' + body + 'return 0;}\n')
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-std=c99", "-I", HDR, src, "-o", exe])
        out = [int(v) for v in subprocess.check_output([exe]).split()]
    assert out[0] == ctypes.sizeof(api._Mesh)
    assert out[1:] == [getattr(api._Mesh, f).offset for f in fields]


def test_model_struct_layout_matches_the_header():
    """The ctypes mirrors of mvf_model (library and oracle) have the C struct's size and
    field offsets."""
    import subprocess
    import tempfile

    import oracle
    fields = [f for f, _ in api._Model._fields_]
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        body = "".join(f'printf("%zu\\n", offsetof(mvf_model, {f}));' for f in fields)
        open(src, "w").write('#include <stddef.h>\n#include <stdio.h>\n#include "movfem_gpu.h"\n'
                             'int main(void){printf("%zu\\n", sizeof(mvf_model));' + body + 'return 0;}\n')
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-std=c99", "-I", HDR, src, "-o", exe])
        out = [int(v) for v in subprocess.check_output([exe]).split()]
    for S in (api._Model, oracle._Model):
        assert [f for f, _ in S._fields_] == fields
        assert out[0] == ctypes.sizeof(S)
        assert out[1:] == [getattr(S, f).offset for f in fields]
