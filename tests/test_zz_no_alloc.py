"""The allocation-free bulk apply, symeig_apply_givens_f64_noalloc.

It serves callers that cannot allocate device memory at call time, e.g. because another
allocator already owns the device's memory.  Its scratch (the wave table) is a fixed
file-scope device array shared by all calls.  This test calls it through the C ABI and checks
its output against the handle-based entry point symeig_apply_givens_f64_dev on two calls in
a row, with the bit-exact tolerance the other apply tests use, and checks that a size beyond
the array is rejected.  The file name sorts last so a failure here stops a run only after
every other test has run.  It also covers the 27-warp tile shape the apply takes from 15000
rows on, a leading dimension larger than the row count, the explicit set-up call and the
read-and-clear status query of the entry point's error word.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(torch, m, n, k, seed, lda=None):
    lda = m if lda is None else lda
    g = torch.Generator(device="cpu").manual_seed(seed)
    Qt = torch.rand(n, lda, generator=g, dtype=torch.float64) * 2 - 1      # column-major Q = Qt.T
    th = torch.rand(k, n - 1, generator=g, dtype=torch.float64) * 2 * np.pi
    cs = torch.stack([torch.cos(th), torch.sin(th)], -1).contiguous()      # Julia layout
    return Qt.cuda(), cs.cuda()


@pytest.mark.parametrize("m,n,k,lda", [(300, 129, 70, 300), (64, 1000, 64, 64), (5, 3, 1, 5),
                                       (15360, 257, 8, 15360), (301, 130, 65, 304)])
def test_noalloc_matches_handle_entry_two_calls(cuda, pkg, m, n, k, lda):
    torch = cuda
    lib = pkg.load_library()
    assert lib.symeig_noalloc_init() == 0
    h = pkg.Handle(0)
    stream = torch.cuda.current_stream().cuda_stream
    h.set_stream(stream)
    Qt, cs = _inputs(torch, m, n, k, seed=m + n + k, lda=lda)
    A_ref = Qt.clone()
    A_new = Qt.clone()
    for call in range(2):   # two calls in a row: the shared array keeps the previous contents
        rc = lib.symeig_apply_givens_f64_dev(h.ptr, ctypes.c_void_p(A_ref.data_ptr()), lda, m, n,
                                             ctypes.c_void_p(cs.data_ptr()), k)
        assert rc == 0
        rc = lib.symeig_apply_givens_f64_noalloc(ctypes.c_void_p(A_new.data_ptr()), lda, m, n,
                                                 ctypes.c_void_p(cs.data_ptr()), k,
                                                 ctypes.c_void_p(stream))
        assert rc == 0
        assert lib.symeig_noalloc_status(ctypes.c_void_p(stream)) == 0   # no wait gave up
        torch.cuda.synchronize()
        assert torch.equal(A_new, A_ref), f"call {call}: max diff {(A_new - A_ref).abs().max().item()}"
    if lda > m:   # the rows between m and lda are not touched
        assert torch.equal(A_new[:, m:], Qt[:, m:])
    h.close()


def test_noalloc_rejects_sizes_beyond_its_array(cuda, pkg):
    torch = cuda
    lib = pkg.load_library()
    n, m, k = 40000, 1, 1       # ceil((n + 71) / 9) * 10368 bytes > 32 MiB
    A = torch.zeros(n, dtype=torch.float64, device="cuda")
    cs = torch.zeros(2 * (n - 1), dtype=torch.float64, device="cuda")
    rc = lib.symeig_apply_givens_f64_noalloc(ctypes.c_void_p(A.data_ptr()), 1, m, n,
                                             ctypes.c_void_p(cs.data_ptr()), k, None)
    assert rc == 2                          # SYMEIG_ERR_SIZE, nothing launched
    assert lib.symeig_apply_givens_f64_noalloc(None, 1, 1, 4, None, 1, None) == 1  # NULL A
