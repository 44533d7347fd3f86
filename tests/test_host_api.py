"""Host-side logic of the Python mirror that needs no GPU: argument validation raises before
any library call, layouts are recognised, and the packing helpers are consistent."""
from __future__ import annotations

import numpy as np
import pytest


def test_symtridiagonal_dense_and_copy(pkg):
    H = pkg.SymTridiagonal(np.array([1.0, 2.0, 3.0]), np.array([0.5, -0.25]))
    T = H.dense()
    assert np.array_equal(T, np.array([[1, 0.5, 0], [0.5, 2, -0.25], [0, -0.25, 3.0]]))
    H2 = H.copy()
    H2.dv[0] = 9.0
    assert H.dv[0] == 1.0 and H.n == 3


def test_givens_buffer_is_julia_layout(pkg):
    g = pkg.givens_buffer(5, 3)
    assert g.shape == (5, 3, 2)
    # pair, then i, then L: strides 8, 16, 16*(n-1) bytes
    assert g.strides == (16, 80, 8)


def test_row_major_matrix_is_rejected(pkg):
    A = np.zeros((4, 5))                  # C order: not column-major
    with pytest.raises(ValueError):
        pkg.bulk_wave_order_2x2_rmul_(A, pkg.givens_buffer(4, 1))


def test_apply_shape_mismatch_is_rejected(pkg):
    A = np.asfortranarray(np.zeros((4, 5)))
    with pytest.raises(ValueError):
        pkg.bulk_wave_order_2x2_rmul_(A, pkg.givens_buffer(3, 1))   # needs n-1 = 4 rows
    with pytest.raises(ValueError):
        pkg.bulk_wave_order_2x2_lmul_(A, pkg.givens_buffer(4, 1))   # needs m-1 = 3 rows


def test_qr_arguments_are_checked(pkg):
    H = pkg.SymTridiagonal(np.zeros(4), np.zeros(2))         # ev must have n-1 entries
    with pytest.raises(ValueError):
        pkg.qr_algorithm_(H, None)
    H = pkg.SymTridiagonal(np.zeros(4, dtype=np.float32), np.zeros(3, dtype=np.float32))
    with pytest.raises(TypeError):
        pkg.qr_algorithm_(H, None)
    H = pkg.SymTridiagonal(np.zeros(4), np.zeros(3))
    with pytest.raises(ValueError):
        pkg.qr_algorithm_(H, np.asfortranarray(np.zeros((4, 3))))  # Q needs n columns


def test_batched_packing_is_checked(pkg):
    n = [3, 4]
    with pytest.raises(ValueError):
        pkg.qr_algorithm_batched_(np.zeros(6), np.zeros(5), n)      # d has sum(n) = 7
    with pytest.raises(ValueError):
        pkg.qr_algorithm_batched_(np.zeros(7), np.zeros(5), n, np.zeros(24))   # Q has 25
    with pytest.raises(TypeError):
        pkg.qr_algorithm_batched_(np.zeros(7, dtype=np.float32), np.zeros(5), n)
    with pytest.raises(TypeError):   # Q float16
        pkg.qr_algorithm_batched_(np.zeros(7), np.zeros(5), n, np.zeros(25, dtype=np.float16))


def test_batched_tuning_per_dtype(pkg):
    """The batched tuning is kept per precision of Q; tiles 0..2 are accepted, others and a
    split below 1 are refused (SYMEIG_ERR_SIZE) and leave the tuning unchanged.  No device."""
    old64, old32 = pkg.batched_tuning(fp64=True), pkg.batched_tuning(fp64=False)
    try:
        pkg.batched_tuning(fp64=True, split=300, shape_small=2, shape_large=1)
        pkg.batched_tuning(fp64=False, split=100, shape_small=1, shape_large=2)
        assert pkg.batched_tuning(fp64=True) == {"split": 300, "shape_small": 2, "shape_large": 1}
        assert pkg.batched_tuning(fp64=False) == {"split": 100, "shape_small": 1, "shape_large": 2}
        for bad in ({"shape_small": 3}, {"shape_large": -1}, {"split": 0}):
            with pytest.raises(pkg.SymeigError):
                pkg.batched_tuning(fp64=True, **bad)
        assert pkg.batched_tuning(fp64=True) == {"split": 300, "shape_small": 2, "shape_large": 1}
    finally:
        pkg.batched_tuning(fp64=True, **old64)
        pkg.batched_tuning(fp64=False, **old32)


def test_wave_port_threads_do_not_change_bits(oracle, pkg):
    """The oracle's row-slab threading (src/wave.jl:44-57) gives the same bits for any count."""
    rng = np.random.default_rng(4)
    m, n, k = 100, 34, 8
    th = rng.random((n - 1, k)) * 2 * np.pi
    g = pkg.givens_buffer(n - 1, k)
    g[..., 0], g[..., 1] = np.cos(th), np.sin(th)
    A = np.asfortranarray(rng.random((m, n)))
    outs = []
    for t in (1, 2, 3, 7):
        B = A.copy(order="F")
        oracle.apply_wave(B, g, nthreads=t)
        outs.append(B)
    for B in outs[1:]:
        assert np.array_equal(B, outs[0])


def test_oracle_fp32_q_variant(oracle):
    """FP32-Q oracle: the chase is FP64 (eigenvalues bit-equal to the FP64 run) and Q is the
    FP32 product of the FP32-rounded rotations."""
    rng = np.random.default_rng(8)
    n = 50
    d, e = rng.standard_normal(n), rng.random(n - 1)
    d1, e1, d2, e2 = d.copy(), e.copy(), d.copy(), e.copy()
    Q64 = np.asfortranarray(np.eye(n))
    Q32 = np.asfortranarray(np.eye(n, dtype=np.float32))
    oracle.qr_algorithm(d1, e1, Q64)
    oracle.qr_algorithm(d2, e2, Q32)
    assert np.array_equal(d1, d2)
    assert np.max(np.abs(Q32.astype(np.float64) - Q64)) < 1e-4


def test_oracle_flush_generator(oracle):
    """qr_flushes walks the reference's outer loop: flushes with rotations, then converged."""
    rng = np.random.default_rng(3)
    n = 30
    d, e = rng.standard_normal(n), rng.random(n - 1)
    statuses = []
    for rc, grid, thick, place, it in oracle.qr_flushes(d, e, max_layers=4):
        statuses.append(rc)
        if rc == 1:
            assert thick.max() <= 4 and place.max() >= 1
            assert grid.shape == (n - 1, 8, 2)   # exact-order grids hold 2 * max_layers
    assert statuses[-1] == 0 and all(s == 1 for s in statuses[:-1]) and len(statuses) > 2


def test_dense_entry_points_validate_arguments(pkg):
    """sytrd / orgtr / syev reject bad handles and sizes before touching a device."""
    lib = pkg.load_library()
    import ctypes
    buf = (ctypes.c_double * 16)()
    c32, c64 = ctypes.c_int32(), ctypes.c_int64()
    assert lib.symeig_sytrd_f64(None, 4, buf, 4, buf, buf, buf) == 5          # SYMEIG_ERR_HANDLE
    assert lib.symeig_orgtr_f64(None, 4, buf, 4, buf, buf, 4) == 5
    assert lib.symeig_syev_f64(None, 4, buf, 4, buf, buf, 4, ctypes.byref(c32), ctypes.byref(c64)) == 5
    assert lib.symeig_sytrd_f64_dev(None, 4, buf, 4, buf, buf, buf) == 5


def test_apply_tuning_shapes_per_precision(pkg):
    """symeig_apply_tuning keeps the tile shape per precision: FP64 has shapes 0-3 (2: one CTA
    of 27 warps, 3: passes of 128 layers), FP32 0-4 (2 and 3 hold two rows per thread, 4 is a CTA of 14 warps), and -1
    (the default) chooses by the rows of each launch; out-of-range shapes are refused and
    leave it as it was.  Setting the shape touches no device."""
    import ctypes
    lib = pkg.load_library()
    v = ctypes.c_int32()
    assert lib.symeig_apply_tuning(1, ctypes.byref(v), 0) == 0 and v.value == -1
    assert lib.symeig_apply_tuning(0, ctypes.byref(v), 0) == 0 and v.value == -1
    for fp64, bad in ((1, 4), (1, -2), (0, 5)):
        v = ctypes.c_int32(bad)
        assert lib.symeig_apply_tuning(fp64, ctypes.byref(v), 1) == 2      # SYMEIG_ERR_SIZE
    v = ctypes.c_int32(3)
    assert lib.symeig_apply_tuning(0, ctypes.byref(v), 1) == 0
    assert lib.symeig_apply_tuning(0, ctypes.byref(v), 0) == 0 and v.value == 3
    v = ctypes.c_int32(-1)
    assert lib.symeig_apply_tuning(0, ctypes.byref(v), 1) == 0
    assert lib.symeig_apply_tuning(0, ctypes.byref(v), 0) == 0 and v.value == -1
    assert lib.symeig_apply_tuning(1, ctypes.byref(v), 0) == 0 and v.value == -1
