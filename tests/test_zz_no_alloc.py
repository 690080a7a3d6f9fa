"""mvf_spmv_noalloc: the matrix-vector product for callers that cannot let the
library allocate device memory (their device memory belongs to their own pool
allocator).

It must give the same product as mvf_spmv (the allocating entry point) and as the
oracle's assembled matrix, on two calls in a row -- the second call reuses the shared
fixed-size staging array left behind by the first -- and it must leave the device's
free memory unchanged.  This file is collected last so that a failure here leaves the
rest of the suite already run; it also passes on its own in a fresh process.
"""
import math

import numpy as np
import pytest

import oracle
from movfem_gb300 import api
from movfem_gb300 import mesh as M

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_noalloc_spmv_matches_spmv_twice():
    torch = pytest.importorskip("torch")
    m = M.plain_linear_block(ncells=8, d=250.0, n_air=4, dz_air=500.0, nrx=2)
    w = 2 * math.pi * np.array([0.5, 4.0])
    p = api.MTProblem(m, device=0)
    p.assemble(w)
    o = oracle.Oracle(m)
    rng = np.random.Generator(np.random.PCG64(11))
    # the 16 MiB array is part of the library's device image: CUDA loads it (lazily) with
    # the module's first kernel on this device, not at the call's request; one warm-up
    # call does that before free memory is compared across the two checked calls
    xw = torch.zeros((2, p.nne), dtype=torch.complex128, device="cuda:0")
    yw = torch.zeros_like(xw)
    torch.cuda.synchronize()
    p.spmv_noalloc(0, xw.data_ptr(), yw.data_ptr())
    for call, f in enumerate([1, 0]):
        x = rng.normal(size=(2, p.nne)) + 1j * rng.normal(size=(2, p.nne))
        ref = p.spmv(f, x)
        A, _ = o.matrix(w[f])
        ref_oracle = np.stack([A @ x[0], A @ x[1]])
        xd = torch.from_numpy(x).to("cuda:0")
        yd = torch.full((2, p.nne), complex(float("nan"), float("nan")), dtype=torch.complex128, device="cuda:0")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        p.spmv_noalloc(f, xd.data_ptr(), yd.data_ptr())
        free1 = torch.cuda.mem_get_info(0)[0]
        y = yd.cpu().numpy()
        assert free1 == free0, f"call {call}: device free memory changed by {free0 - free1} bytes"
        assert _rel(y, ref) < 1e-12, f"call {call}"
        # the oracle's matrix: FP64 on both sides, assembled in a different order
        assert _rel(y, ref_oracle) < 1e-10, f"call {call}"


def test_noalloc_after_a_side_stream_event():
    """The documented stream contract: x written on the caller's own (non-default)
    stream, that stream's event waited for on the host -- no device-wide synchronise --
    then the call; y is complete when the call returns."""
    torch = pytest.importorskip("torch")
    m = M.plain_linear_block(ncells=6, d=250.0, n_air=3, dz_air=500.0, nrx=2)
    w = 2 * math.pi * 2.0
    p = api.MTProblem(m, device=0)
    p.assemble([w])
    rng = np.random.Generator(np.random.PCG64(13))
    x = rng.normal(size=(2, p.nne)) + 1j * rng.normal(size=(2, p.nne))
    ref = p.spmv(0, x)
    side = torch.cuda.Stream(device=0)
    with torch.cuda.stream(side):
        xh = torch.from_numpy(x).pin_memory()
        xd = xh.to("cuda:0", non_blocking=True)
        yd = torch.zeros((2, p.nne), dtype=torch.complex128, device="cuda:0")
        done = torch.cuda.Event()
        done.record(side)
    done.synchronize()
    p.spmv_noalloc(0, xd.data_ptr(), yd.data_ptr())
    assert _rel(yd.cpu().numpy(), ref) < 1e-12


def test_noalloc_rejects_models_above_its_limit():
    torch = pytest.importorskip("torch")
    # 46^3 earth cells + 10 air layers: about 355,000 free DOFs, above the 262,144 limit
    m = M.plain_linear_block(ncells=46, d=100.0, n_air=10, dz_air=200.0, nrx=2)
    p = api.MTProblem(m, device=0)
    p.assemble([2 * math.pi])
    assert p.nne > 262144
    xd = torch.zeros((2, p.nne), dtype=torch.complex128, device="cuda:0")
    yd = torch.zeros_like(xd)
    with pytest.raises(api.MVFError) as e:
        p.spmv_noalloc(0, xd.data_ptr(), yd.data_ptr())
    assert e.value.code == api.E_ARG
    assert "262144" in str(e.value)
