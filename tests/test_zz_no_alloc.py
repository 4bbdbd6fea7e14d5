"""The allocation-free rconv entry point (opaw_rconv_noalloc) against the
allocating one (opaw_rconv), through the C ABI, on two calls in a row.

opaw_rconv_noalloc exists for callers that cannot call cudaMalloc: a host
program whose device memory budget was fixed at start-up, or a process whose
device allocator belongs to another runtime that a library must not touch.
It takes caller-allocated device buffers and keeps its scratch in a fixed
file-scope device array.  This file is named to be collected last.
"""
import os

import numpy as np
import pytest

import opaw_tddft_gb300 as pkg

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL64 = 1e-12


def to_dev(torch, gin, bk):
    a = torch.from_numpy(np.ascontiguousarray(gin)).to("cuda")
    b = torch.from_numpy(np.ascontiguousarray(bk)).to("cuda")
    out = torch.full_like(a, float("nan"))
    torch.cuda.synchronize()
    return a, b, out


def call_noalloc(torch, a, b, out):
    n2, n1, n0 = a.shape
    st = pkg.lib().opaw_rconv_noalloc(n0, n1, n2, a.data_ptr(), b.data_ptr(), out.data_ptr(),
                                      torch.cuda.current_stream().cuda_stream)
    assert st == 0, pkg.lib().opaw_last_error().decode()


def run_noalloc(torch, gin, bk):
    a, b, out = to_dev(torch, gin, bk)
    call_noalloc(torch, a, b, out)
    return out.cpu().numpy()


def cases():
    f = np.load(os.path.join(GOLDEN, "rconv_8x6x3.npz"))
    rng = np.random.default_rng(17)
    # generic lengths (radix 2, 3, 5, 7 stages) and lengths with their own
    # compile-time FFT kernels (32, 48, 64)
    gin2 = rng.standard_normal((20, 28, 30))
    bk2 = np.abs(rng.standard_normal((20, 28, 30)))
    gin3 = rng.standard_normal((64, 48, 32))
    bk3 = np.abs(rng.standard_normal((64, 48, 32)))
    return f, [(f["gin"], f["bk"]), (gin2, bk2), (gin3, bk3)]


def test_rconv_noalloc_matches_rconv_twice():
    torch = pytest.importorskip("torch")
    f, cs = cases()
    for gin, bk in cs:
        ref = pkg.rconv(gin, bk)
        for _ in range(2):  # two calls in a row: the shared scratch keeps the last call's contents
            got = run_noalloc(torch, gin, bk)
            assert np.abs(got - ref).max() <= TOL64 * np.abs(ref).max(), gin.shape
    # the reference's own known answer, through the allocation-free path
    got = run_noalloc(torch, f["gin"], f["bk"])
    assert np.abs(got - f["gana"]).sum() < 1e-11 * np.abs(f["gana"]).sum()


def test_rconv_noalloc_allocates_nothing():
    """After a warm call, a second call on the largest case leaves the device's
    free memory and torch's reserved pool unchanged."""
    torch = pytest.importorskip("torch")
    _, cs = cases()
    a, b, out = to_dev(torch, *cs[-1])
    call_noalloc(torch, a, b, out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    res0 = torch.cuda.memory_reserved()
    call_noalloc(torch, a, b, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert torch.cuda.memory_reserved() == res0
    assert np.isfinite(out.cpu().numpy()).all()


def test_rconv_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    L = pkg.lib()
    one = np.zeros(1)
    p = one.ctypes.data
    assert L.opaw_rconv_noalloc(128, 64, 64, p, p, p, None) == 1  # 524288 points > 262144
    assert b"exceed the fixed scratch" in L.opaw_last_error()
    assert L.opaw_rconv_noalloc(512, 2, 2, p, p, p, None) == 1  # extent > 256
    assert L.opaw_rconv_noalloc(11, 2, 2, p, p, p, None) == 1  # prime factor 11
