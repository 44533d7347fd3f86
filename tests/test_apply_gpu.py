"""Parity of the wave-window Givens kernel (bulk_wave_order_2x2_rmul!, src/wave.jl:36-162)
with the CPU oracle.  The kernel and the oracle use the same fused-multiply-add pattern, so
the comparison is bit-exact (signed zeros compare equal)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rotation_grid, to_device_colmajor

pytestmark = pytest.mark.gpu

SHAPES = [  # (m, n, k)
    (1, 2, 1), (3, 2, 2), (5, 3, 1), (32, 4, 2), (33, 5, 3), (7, 8, 4), (64, 33, 7),
    (129, 34, 8), (100, 9, 20),   # k > n-1, which the reference cannot do
    (257, 65, 64), (130, 200, 65), (31, 129, 130),
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,k", SHAPES)
def test_apply_device_matches_oracle(cuda, pkg, oracle, m, n, k, dtype):
    rng = np.random.default_rng(m * 1000 + n * 10 + k)
    g = rotation_grid(pkg, rng, n, k, dtype)
    A = np.asfortranarray((rng.random((m, n)) * 2 - 1).astype(dtype))
    ref = A.copy(order="F")
    oracle.apply_seq(ref, g)
    dA = to_device_colmajor(cuda, A)
    pkg.bulk_wave_order_2x2_rmul_(dA, cuda.from_numpy(np.ascontiguousarray(g)).cuda())
    got = dA.cpu().numpy()
    assert np.array_equal(got, ref), np.max(np.abs(got - ref))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_apply_host_buffers_with_leading_dimension(cuda, pkg, oracle, dtype):
    rng = np.random.default_rng(5)
    m, n, k, ld = 45, 20, 9, 53
    big = np.asfortranarray((rng.random((ld, n)) * 2 - 1).astype(dtype))
    A = big[:m, :]  # column-major view with leading dimension 53
    g = rotation_grid(pkg, rng, n, k, dtype)
    ref = np.asfortranarray(A.copy())
    oracle.apply_seq(ref, g)
    untouched = big[m:, :].copy()
    pkg.bulk_wave_order_2x2_rmul_(A, g)
    assert np.array_equal(A, ref)
    assert np.array_equal(big[m:, :], untouched)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,k,ld", [(4100, 300, 64, 4100), (4099, 129, 40, 4111), (4096, 70, 1, 4096),
                                      (5000, 200, 65, 5000), (2100, 90, 64, 2100), (4096, 2001, 64, 4096),
                                      (15360, 600, 64, 15363), (4097, 3, 2, 4097), (4096, 2, 64, 4096),
                                      (8200, 150, 64, 8201), (10001, 97, 33, 10001)])
def test_apply_host_pipelined_column_segments(cuda, pkg, oracle, m, n, k, ld, dtype):
    """Host Q with k <= 64 and m >= 4096 runs as 16 launches over column segments of one pass
    (copies in, kernels and copies out on three streams; each launch carries its registers to
    the next through a state buffer): the result is the oracle's bits, and the rows beyond m of
    a leading dimension are untouched.  Small n gives one table chunk per segment (every
    boundary a segment boundary).  The default tile choice by rows takes FP64 shape 0 below
    9728 rows and the 27-warp shape 2 above, FP32 shape 0 below 7168, 1 up to 14336 (m = 8200,
    10001) and 4 above.  k = 65 and m = 2100 take the unpipelined path."""
    rng = np.random.default_rng(m + n + k)
    big = np.asfortranarray((rng.random((ld, n)) * 2 - 1).astype(dtype))
    A = big[:m, :]
    g = rotation_grid(pkg, rng, n, k, dtype)
    ref = np.asfortranarray(A.copy())
    oracle.apply_seq(ref, g)
    untouched = big[m:, :].copy()
    pkg.bulk_wave_order_2x2_rmul_(A, g)
    assert np.array_equal(A, ref)
    assert np.array_equal(big[m:, :], untouched)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,k", [(7167, 64), (7168, 64), (9727, 64), (9728, 64), (14335, 64), (14336, 64),
                                 (15000, 64), (15500, 64), (16417, 64), (1000, 128), (3071, 128), (3072, 96),
                                 (7167, 128), (7168, 128)])
def test_apply_auto_shape_by_rows(cuda, pkg, oracle, m, k, dtype):
    """The default tile choice by rows, on each side of its thresholds: FP64 shape 0 below 9728
    rows, CTAs of 27 warps (one per SM at 16384 rows) from there, and below 7168 rows one pass
    of 128 layers (shape 3) for more than 64 layers, with the integer-pipe products from 3072
    rows; FP32 shape 0 below 7168, 1 below 14336, CTAs of 14 warps from there.  The last CTA
    is partial.  Bits as the oracle's, device path."""
    rng = np.random.default_rng(m + k)
    n = 40
    g = rotation_grid(pkg, rng, n, k, dtype)
    A = np.asfortranarray((rng.random((m, n)) * 2 - 1).astype(dtype))
    ref = A.copy(order="F")
    oracle.apply_seq(ref, g)
    dA = to_device_colmajor(cuda, A)
    pkg.bulk_wave_order_2x2_rmul_(dA, cuda.from_numpy(np.ascontiguousarray(g)).cuda())
    assert np.array_equal(dA.cpu().numpy(), ref)


def test_apply_host_pipelined_scaled_form(cuda, pkg, oracle):
    rng = np.random.default_rng(77)
    m, n, k = 4352, 257, 64
    A = np.asfortranarray(rng.random((m, n)) * 2 - 1)
    g = rotation_grid(pkg, rng, n, k, np.float64)
    ref = A.copy(order="F")
    oracle.apply_scaled(ref, g)
    pkg.bulk_wave_order_2x2_rmul_(A, g, form=1)
    assert np.array_equal(A, ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,n,k", [(2, 1, 1), (9, 5, 3), (65, 40, 64), (130, 33, 70)])
def test_left_apply_matches_oracle(cuda, pkg, oracle, m, n, k, dtype):
    """Bulk lmul! (row rotations) == the oracle's column rotations of the transpose."""
    rng = np.random.default_rng(m + 7 * n + k)
    g = rotation_grid(pkg, rng, m, k, dtype)          # (m-1) x k grid
    A = np.asfortranarray((rng.random((m, n)) * 2 - 1).astype(dtype))
    refT = np.asfortranarray(A.T.copy())
    oracle.apply_seq(refT, g)
    dA = to_device_colmajor(cuda, A)
    pkg.bulk_wave_order_2x2_lmul_(dA, cuda.from_numpy(np.ascontiguousarray(g)).cuda())
    assert np.array_equal(dA.cpu().numpy(), refT.T)
    B = A.copy(order="F")
    pkg.bulk_wave_order_2x2_lmul_(B, g)
    assert np.array_equal(B, refT.T)


@pytest.mark.parametrize("dtype,shape", [(np.float64, 0), (np.float64, 1), (np.float64, 2), (np.float64, 3),
                                         (np.float32, 0), (np.float32, 1), (np.float32, 2), (np.float32, 3),
                                         (np.float32, 4)])
def test_apply_every_tile_shape(cuda, pkg, oracle, dtype, shape):
    """Every tile shape of the single-matrix wave kernel gives the oracle's bits (FP32 shapes 2
    and 3 hold two rows per thread, FP32 shape 4 is a CTA of 14 warps, FP64 shape 2 one of 27
    warps, FP64 shape 3 runs passes of 128 layers -- k = 130 is one such pass and a 2-layer pass
    in shape 0, k = 100 one pass of 100 layers; the row counts leave partial tiles and partial
    warps)."""
    import ctypes
    lib = pkg.load_library()
    fp64 = int(dtype == np.float64)
    old = ctypes.c_int32()
    assert lib.symeig_apply_tuning(fp64, ctypes.byref(old), 0) == 0
    v = ctypes.c_int32(shape)
    assert lib.symeig_apply_tuning(fp64, ctypes.byref(v), 1) == 0
    try:
        rng = np.random.default_rng(99 + shape)
        for (m, n, k) in [(33, 70, 64), (100, 129, 130), (7, 20, 5), (77, 40, 64), (333, 90, 64), (15100, 50, 64),
                          (3100, 60, 100)]:
            g = rotation_grid(pkg, rng, n, k, dtype)
            A = np.asfortranarray((rng.random((m, n)) * 2 - 1).astype(dtype))
            ref = A.copy(order="F")
            oracle.apply_seq(ref, g)
            dA = to_device_colmajor(cuda, A)
            pkg.bulk_wave_order_2x2_rmul_(dA, cuda.from_numpy(np.ascontiguousarray(g)).cuda())
            assert np.array_equal(dA.cpu().numpy(), ref)
    finally:
        assert lib.symeig_apply_tuning(fp64, ctypes.byref(old), 1) == 0
