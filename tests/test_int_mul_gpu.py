"""The canonical FP64 apply computes each rotation's two products s*y and s*x on GB300's
integer pipes (csrc/int_mul.cuh) and falls back to the FP64 pipe where the integer path does
not apply.  symeig_mul_rn_f64_dev exposes that arithmetic elementwise; it must give the IEEE
round-to-nearest-even product bit for bit (the host's multiply, and the device's FP64
multiply) on random operands, exact ties, operands with extreme significands, signed zeros,
subnormals, infinities, NaNs, underflowing and overflowing products.  The apply itself is
then checked bit for bit against the oracle in both arithmetic forms (form 0: integer-pipe
products, form 2: FP64-pipe products)."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import rotation_grid, to_device_colmajor

pytestmark = pytest.mark.gpu


def _device_products(torch, pkg, a, b, form):
    lib = pkg.load_library()
    h = pkg.Handle(0)
    try:
        da = torch.from_numpy(a).cuda()
        db = torch.from_numpy(b).cuda()
        out = torch.empty_like(da)
        h.set_stream(torch.cuda.current_stream().cuda_stream)
        rc = lib.symeig_mul_rn_f64_dev(h.ptr, a.size, ctypes.c_void_p(da.data_ptr()),
                                       ctypes.c_void_p(db.data_ptr()), ctypes.c_void_p(out.data_ptr()), form)
        assert rc == 0
        torch.cuda.synchronize()
        return out.cpu().numpy()
    finally:
        h.close()


def _operands(rng):
    """Pairs (a, b): random, ties, extremes and specials."""
    A, B = [], []
    n = 1 << 20
    # rotation-like factors times values over the whole exponent range
    A.append(rng.uniform(-1, 1, n))
    B.append(rng.uniform(-1, 1, n) * 10.0 ** rng.integers(-300, 300, n))
    # uniform bit patterns (every exponent, both signs)
    bits = rng.integers(0, 2**64, size=(2, n), dtype=np.uint64).view(np.float64)
    A.append(bits[0])
    B.append(bits[1])
    # exact ties and near-ties: a 53-bit integer times 1 + j/2^k (k <= 3) discards 1-3 bits
    a53 = rng.integers(2**52, 2**53, n).astype(np.float64) * 2.0 ** rng.integers(-80, 80, n)
    k = rng.integers(1, 4, n)
    j = rng.integers(1, 8, n) % (2 ** k)
    j[j == 0] = 1
    A.append((1 + j / 2.0 ** k) * rng.choice([-1.0, 1.0], n))
    B.append(a53)
    # extreme significands: all-ones and implicit-bit-only, at many exponents
    ext = np.array([1.0, np.nextafter(2.0, 0), np.nextafter(1.0, 2), 1.5, 0.75, np.nextafter(1.0, 0)])
    ea, eb = np.meshgrid(ext, ext)
    scale = 2.0 ** np.arange(-1074, 1024, 37, dtype=np.float64)
    for s in scale:
        A.append(ea.ravel())
        B.append(eb.ravel() * s)
    # specials
    sp = np.array([0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, np.nextafter(2.2250738585072014e-308, 0),
                   np.inf, -np.inf, np.nan, 1.0, -1.0, 1.7976931348623157e308, 1e-300, 1e300, 0.5, 2.0 ** -537])
    sa, sb = np.meshgrid(sp, sp)
    A.append(sa.ravel())
    B.append(sb.ravel())
    # zero factors (the grid's identity padding, the zeros of Q = I) against every kind of value
    z = np.array([0.0, -0.0])
    vals = np.concatenate([sp, rng.uniform(-1, 1, 64) * 10.0 ** rng.integers(-300, 300, 64)])
    za, zb = np.meshgrid(z, vals)
    A += [za.ravel(), zb.ravel()]
    B += [zb.ravel(), za.ravel()]
    # underflow / overflow boundaries: products around 2^-1022 and 2^1024
    m = 1 << 16
    A.append(rng.uniform(1, 2, m) * 2.0 ** rng.integers(-540, -480, m))
    B.append(rng.uniform(1, 2, m) * 2.0 ** rng.integers(-560, -500, m))
    A.append(rng.uniform(1, 2, m) * 2.0 ** rng.integers(500, 520, m))
    B.append(rng.uniform(1, 2, m) * 2.0 ** rng.integers(500, 524, m))
    return np.concatenate(A), np.concatenate(B)


def test_integer_products_match_ieee_multiply(cuda, pkg):
    torch = cuda
    rng = np.random.default_rng(2024)
    a, b = _operands(rng)
    got = _device_products(torch, pkg, a, b, 0)
    native = _device_products(torch, pkg, a, b, 1)
    with np.errstate(all="ignore"):
        host = a * b
    nan = np.isnan(host)
    assert np.array_equal(np.isnan(got), nan) and np.array_equal(np.isnan(native), nan)
    # every non-NaN product has the host multiply's bits (signed zeros and infinities included)
    assert np.array_equal(got[~nan].view(np.int64), host[~nan].view(np.int64))
    # and the device FP64 multiply's bits everywhere (NaN payloads included)
    assert np.array_equal(got.view(np.int64), native.view(np.int64))


@pytest.mark.parametrize("m,n,k", [(257, 65, 64), (3072, 90, 64), (4100, 300, 64), (15360, 129, 64), (33, 5, 3)])
@pytest.mark.parametrize("form", [0, 2])
def test_apply_forms_bit_exact(cuda, pkg, oracle, m, n, k, form):
    """Form 0 (the default: integer-pipe products from 3072 rows on) and form 2 (FP64-pipe
    products) give the oracle's bits; Q with zero columns, subnormal and tiny entries, and
    rotations with s = 0 and c = 0 exercise the inline zero path and the fall-back lanes."""
    torch = cuda
    rng = np.random.default_rng(m + n + k + form)
    g = rotation_grid(pkg, rng, n, k)
    A = np.asfortranarray(rng.random((m, n)) * 2 - 1)
    A[:, n // 3] = 0.0
    A[: m // 2, n // 2] = 1e-310
    A[m // 3, :] *= 2.0 ** -1000
    g[n // 4, 0] = (0.0, 1.0)
    g[n // 5, k - 1] = (1.0, 0.0)
    ref = A.copy(order="F")
    oracle.apply_seq(ref, g)
    dA = to_device_colmajor(torch, A)
    pkg.bulk_wave_order_2x2_rmul_(dA, torch.from_numpy(np.ascontiguousarray(g)).cuda(), form=form)
    assert np.array_equal(dA.cpu().numpy(), ref)


@pytest.mark.parametrize("shape", [0, 1, 2, 3])
def test_apply_fp64_tile_shapes_bit_exact(cuda, pkg, oracle, shape):
    """Every FP64 tile shape (symeig_apply_tuning) with the integer-pipe products (shape 3 with
    k = 17 runs as shape 0; with k = 100 as one 128-layer pass)."""
    torch = cuda
    lib = pkg.load_library()
    old = ctypes.c_int32()
    assert lib.symeig_apply_tuning(1, ctypes.byref(old), 0) == 0
    sh = ctypes.c_int32(shape)
    assert lib.symeig_apply_tuning(1, ctypes.byref(sh), 1) == 0
    try:
        rng = np.random.default_rng(shape)
        for (m, n, k) in [(1000, 200, 64), (16384, 40, 17), (4000, 50, 100)]:
            g = rotation_grid(pkg, rng, n, k)
            A = np.asfortranarray(rng.random((m, n)) * 2 - 1)
            ref = A.copy(order="F")
            oracle.apply_seq(ref, g)
            dA = to_device_colmajor(torch, A)
            pkg.bulk_wave_order_2x2_rmul_(dA, torch.from_numpy(np.ascontiguousarray(g)).cuda())
            assert np.array_equal(dA.cpu().numpy(), ref), (m, n, k)
    finally:
        assert lib.symeig_apply_tuning(1, ctypes.byref(old), 1) == 0
