"""The allocation-free rconv entry point (opaw_rconv_noalloc) against the
allocating one (opaw_rconv), through the C ABI, on two calls in a row.

opaw_rconv_noalloc exists for callers that cannot call cudaMalloc (a host
program with a device memory budget fixed at start-up, code running under
CUDA stream capture, a process whose allocator a library must not touch): it
takes caller-allocated device buffers and keeps its scratch in a fixed
file-scope device array.  This file is named to be collected last.
"""
import os

import numpy as np
import pytest

import opaw_tddft_gb300 as pkg

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12


def run_noalloc(torch, gin, bk):
    a = torch.from_numpy(np.ascontiguousarray(gin)).to("cuda")
    b = torch.from_numpy(np.ascontiguousarray(bk)).to("cuda")
    out = torch.full_like(a, float("nan"))
    n2, n1, n0 = gin.shape
    torch.cuda.synchronize()
    st = pkg.lib().opaw_rconv_noalloc(n0, n1, n2, a.data_ptr(), b.data_ptr(), out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 0, pkg.lib().opaw_last_error().decode()
    return out.cpu().numpy()


def test_rconv_noalloc_matches_rconv_twice():
    torch = pytest.importorskip("torch")
    f = np.load(os.path.join(GOLDEN, "rconv_8x6x3.npz"))
    rng = np.random.default_rng(17)
    gin2 = rng.standard_normal((20, 28, 30))
    bk2 = np.abs(rng.standard_normal((20, 28, 30)))
    for gin, bk in [(f["gin"], f["bk"]), (gin2, bk2)]:
        ref = pkg.rconv(gin, bk)
        got = run_noalloc(torch, gin, bk)
        assert np.abs(got - ref).max() <= TOL64 * np.abs(ref).max()
    # the reference's own known answer, through the allocation-free path
    got = run_noalloc(torch, f["gin"], f["bk"])
    assert np.abs(got - f["gana"]).sum() < 1e-11 * np.abs(f["gana"]).sum()


def test_rconv_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    L = pkg.lib()
    one = np.zeros(1)
    p = one.ctypes.data
    assert L.opaw_rconv_noalloc(128, 64, 64, p, p, p, None) == 1  # 524288 points > 262144
    assert b"exceed the fixed scratch" in L.opaw_last_error()
    assert L.opaw_rconv_noalloc(512, 2, 2, p, p, p, None) == 1  # extent > 256
