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


def test_c_host_links_and_gets_errors_without_a_gpu():
    """A plain C host (no Python) links libmovfem_gpu.so through include/movfem_gpu.h and
    gets status codes and messages back from calls the library refuses before any
    device work: the drop-in boundary as a C or Fortran caller sees it."""
    import subprocess
    import tempfile
    lib = build.build()
    libdir = os.path.dirname(lib)
    cuda_lib = "/usr/local/cuda/lib64"
    src = r'''
#include <stdio.h>
#include <string.h>
#include "movfem_gpu.h"
int main(void) {
    mvf_ctx *ctx = 0;
    mvf_mesh mesh;
    mvf_model model;
    double xp[2] = {0, 1}, sig[12], mu[6];
    int rc;
    memset(&mesh, 0, sizeof mesh);
    memset(&model, 0, sizeof model);
    if (mvf_create(&ctx, NULL, -1) != MVF_E_ARG) return 1;
    if (mvf_map_model(NULL, &model, 1.0, sig, mu, NULL, -1) != MVF_E_ARG) return 2;
    if (strstr(mvf_last_error(NULL), "null") == NULL) return 3;
    mesh.nodes_per_elem = 8; mesh.nx = mesh.ny = mesh.nz = 1;
    mesh.xp = mesh.yp = mesh.zp = xp;
    mesh.nextd = 0;
    rc = mvf_map_model(&mesh, &model, 1.0, sig, mu, NULL, -1);
    if (rc != MVF_E_ARG || strstr(mvf_last_error(NULL), "nextd") == NULL) return 4;
    printf("ok %d %s\n", rc, mvf_last_error(NULL));
    return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "host.c")
        exe = os.path.join(d, "host")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-I", HDR, c, "-o", exe, "-L", libdir,
                               "-lmovfem_gpu", "-L", cuda_lib, "-lcudart", f"-Wl,-rpath,{libdir}:{cuda_lib}"])
        out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.startswith("ok -1")
