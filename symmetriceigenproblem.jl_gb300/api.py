"""Host-side mirror of SymmetricEigenProblem.jl's public functions for the hot path.

Same names (with ``!`` spelled ``_``), argument meaning and results as the reference:

  qr_algorithm_(H, Q, max_layers=128, tol=eps, maxiter=100n) -> (H, converged, iter)
      src/bulge_chasing.jl:146-288
  bulk_wave_order_2x2_rmul_(A, givens)            src/wave.jl:62-162
  bulk_wave_order_2x2_rmul_parallel_(A, givens)   src/wave.jl:36-60
  eigen_decomp_(H) -> (eigenvalues, Q)            src/bulge_chasing.jl:290-299

Every call goes to libsymeig.so on the GPU.  Arrays may be numpy (host buffers: the library
copies them to the device and back) or CUDA torch tensors (device buffers, no copies).
Matrices are column-major like Julia's: a numpy array in Fortran order, or a torch tensor
with stride(0) == 1 (e.g. ``torch.empty(n, m).T``).  A rotation grid ``givens`` is the
Julia ``Matrix{Tuple{T,T}}``: shape (n-1, k, 2), entry [i, L] = (c, s), with memory laid out
as Julia lays it out (pair, then i, then L) -- ``givens_buffer`` builds one.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import check, default_handle, Handle, c_i32, c_i64, load as load_library

try:  # torch is optional for host-buffer use
    import torch
except Exception:  # pragma: no cover
    torch = None

EPS64 = float(np.finfo(np.float64).eps)


@dataclass
class SymTridiagonal:
    """LinearAlgebra.SymTridiagonal(dv, ev): dv (n,) and ev (n-1,) float64 (numpy or CUDA torch)."""
    dv: object
    ev: object

    @property
    def n(self) -> int:
        return int(self.dv.shape[0])

    def copy(self) -> "SymTridiagonal":
        if _is_torch(self.dv):
            return SymTridiagonal(self.dv.clone(), self.ev.clone())
        return SymTridiagonal(np.array(self.dv, copy=True), np.array(self.ev, copy=True))

    def dense(self) -> np.ndarray:
        d = _to_numpy(self.dv)
        e = _to_numpy(self.ev)
        return np.diag(d) + np.diag(e, 1) + np.diag(e, -1)


def _is_torch(x) -> bool:
    return torch is not None and isinstance(x, torch.Tensor)


def _to_numpy(x):
    return x.detach().cpu().numpy() if _is_torch(x) else np.asarray(x)


def _colmajor_info(A):
    """(pointer, ld, m, n, dtype-name, on_device) of a column-major matrix."""
    if _is_torch(A):
        if not A.is_cuda:
            raise ValueError("torch matrices must live on a CUDA device")
        if A.dim() != 2:
            raise ValueError("matrix must be 2-D")
        m, n = A.shape
        if n > 0 and m > 1 and A.stride(0) != 1:
            raise ValueError("matrix must be column-major (stride(0) == 1), e.g. torch.empty(n, m).T")
        ld = A.stride(1) if n > 1 else max(m, 1)
        dt = {torch.float64: "f64", torch.float32: "f32"}.get(A.dtype)
        if dt is None:
            raise TypeError(f"unsupported dtype {A.dtype}")
        return A.data_ptr(), max(ld, m, 1), m, n, dt, True
    if not isinstance(A, np.ndarray) or A.ndim != 2:
        raise ValueError("matrix must be a 2-D numpy array or CUDA torch tensor")
    m, n = A.shape
    if not A.flags.writeable or (m > 1 and n > 0 and A.strides[0] != A.itemsize):
        raise ValueError("matrix must be a writeable column-major (Fortran-ordered) array")
    ld = A.strides[1] // A.itemsize if n > 1 else max(m, 1)
    dt = {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}.get(A.dtype)
    if dt is None:
        raise TypeError(f"unsupported dtype {A.dtype}")
    return A.ctypes.data, max(ld, m, 1), m, n, dt, False


def get_rotation(f, g, handle: Handle | None = None, form: int = 0):
    """get_rotation(f, g) -> (c, s, r) elementwise (src/simple_givens.jl:20-23,
    LinearAlgebra.givensAlgorithm), computed on the device the way the chase computes them:
    form 0 the proved Newton form, form 1 the reference form.  f, g: float64 numpy arrays
    (host) or CUDA tensors (device) of one shape."""
    dev = _is_torch(f)
    h = handle or default_handle(f.device.index if dev else 0)
    h.set_chase_mode(1 if form == 1 else 0)
    try:
        if dev:
            if f.dtype != torch.float64 or g.dtype != torch.float64 or f.shape != g.shape:
                raise TypeError("f, g must be float64 CUDA tensors of one shape")
            fc, gc = f.contiguous().reshape(-1), g.contiguous().reshape(-1)
            c, s, r = (torch.empty_like(fc) for _ in range(3))
            with h.on_stream(torch.cuda.current_stream(f.device).cuda_stream):
                h.call("symeig_get_rotation_f64_dev", int(fc.numel()), ctypes.c_void_p(fc.data_ptr()),
                       ctypes.c_void_p(gc.data_ptr()), ctypes.c_void_p(c.data_ptr()),
                       ctypes.c_void_p(s.data_ptr()), ctypes.c_void_p(r.data_ptr()))
            return c.reshape(f.shape), s.reshape(f.shape), r.reshape(f.shape)
        fa = np.ascontiguousarray(f, dtype=np.float64).reshape(-1)
        ga = np.ascontiguousarray(g, dtype=np.float64).reshape(-1)
        if fa.shape != ga.shape:
            raise ValueError("f and g must have one shape")
        c, s, r = (np.empty_like(fa) for _ in range(3))
        h.call("symeig_get_rotation_f64", int(fa.size), fa.ctypes.data, ga.ctypes.data, c.ctypes.data,
               s.ctypes.data, r.ctypes.data)
        shp = np.shape(f)
        return c.reshape(shp), s.reshape(shp), r.reshape(shp)
    finally:
        h.set_chase_mode(0)


def givens_buffer(n_minus_1: int, k: int, dtype=np.float64) -> np.ndarray:
    """An uninitialised Julia-layout Matrix{Tuple{T,T}} of shape (n-1, k, 2)."""
    return np.empty((k, n_minus_1, 2), dtype=dtype).transpose(1, 0, 2)


def _givens_ptr(givens, dtype_name: str, on_device: bool):
    """Pointer to a Julia-layout (n-1, k, 2) rotation grid, plus a keep-alive object."""
    if _is_torch(givens):
        if not on_device or not givens.is_cuda:
            raise ValueError("givens and A must both be host arrays or both CUDA tensors")
        g = givens.permute(1, 0, 2).contiguous()  # (k, n-1, 2) row-major == Julia layout
        want = torch.float64 if dtype_name == "f64" else torch.float32
        if g.dtype != want:
            raise TypeError("givens must have the dtype of A")
        return g.data_ptr(), g, int(givens.shape[1])
    g = np.asarray(givens)
    if on_device:
        raise ValueError("givens and A must both be host arrays or both CUDA tensors")
    want = np.float64 if dtype_name == "f64" else np.float32
    if g.dtype != want:
        raise TypeError("givens must have the dtype of A")
    if g.ndim != 3 or g.shape[2] != 2:
        raise ValueError("givens must have shape (n-1, k, 2)")
    buf = np.ascontiguousarray(g.transpose(1, 0, 2))
    return buf.ctypes.data, buf, int(g.shape[1])


def bulk_wave_order_2x2_rmul_(A, givens, handle: Handle | None = None, form: int = 0) -> None:
    """A <- A * prod(G) for the (n-1) x k rotation grid, in the reference's wave order
    (src/wave.jl:62-162).  Unlike the reference, any n and any k are accepted.  form=1 uses
    the scaled (fast-Givens) form for FP64 A (symeig_set_apply_form): two FMAs per rotation
    and row, a few ulps from form 0."""
    ptr, ld, m, n, dt, dev = _colmajor_info(A)
    gn = int(givens.shape[0])
    if n >= 2 and gn != n - 1:
        raise ValueError(f"givens has {gn} rows, expected n-1 = {n - 1}")
    if n < 2 or m == 0 or int(givens.shape[1]) == 0:
        return None
    h = handle or default_handle(A.device.index if _is_torch(A) else 0)
    gptr, keep, k = _givens_ptr(givens, dt, dev)
    name = f"symeig_apply_givens_{dt}" + ("_dev" if dev else "")
    h.set_apply_form(form)
    try:
        if dev:  # run on torch's current stream: ordered after the producers of A and givens
            with h.on_stream(torch.cuda.current_stream(A.device).cuda_stream):
                h.call(name, ctypes.c_void_p(ptr), ld, m, n, ctypes.c_void_p(gptr), k)
        else:
            h.call(name, ctypes.c_void_p(ptr), ld, m, n, ctypes.c_void_p(gptr), k)
    finally:
        h.set_apply_form(0)
    if dev:
        # keep the temporary Julia-layout copy alive until the kernels that read it finish
        torch.cuda.current_stream(A.device).synchronize()
    del keep
    return None


def bulk_wave_order_2x2_rmul_parallel_(A, givens, handle: Handle | None = None, form: int = 0) -> None:
    """src/wave.jl:36-60: the row-slab threaded variant.  On the GPU every row already has
    its own thread, so this is the same call."""
    return bulk_wave_order_2x2_rmul_(A, givens, handle, form)


def qr_algorithm_(H: SymTridiagonal, Q=None, max_layers: int = 128, tol: float | None = None,
                  maxiter: int | None = None, handle: Handle | None = None,
                  exact_order: bool = True, chase_mode: int = 0, apply_form: int = 0):
    """qr_algorithm!(H, Q, max_layers=128, tol=eps(T), maxiter=100n) -> (H, converged, iter)
    (src/bulge_chasing.jl:146-288).  H.dv becomes the (unsorted) eigenvalues, Q <- Q*prod(G).
    Q may be None (eigenvalues only), float64 or float32 (the FP32-Q variant: FP64 chase,
    (c,s) rounded to float).  exact_order=False places rotations in the grid as the reference
    does (grid[i, ++layer_thickness[i]]), which loses accuracy in Q when a split block
    re-merges within a flush; the default places each sweep at one layer so Q is exact.
    chase_mode selects how the chase computes rotations (symeig_set_chase_mode); modes 0-2
    give the reference's bits, mode 3 (multishift batches of concurrent bulges) meets the
    reference's error bounds with a different sweep sequence.  apply_form=1 applies each flush to an FP64 Q in the scaled form
    (symeig_set_apply_form)."""
    n = H.n
    tol = EPS64 if tol is None else float(tol)
    maxiter = 100 * n if maxiter is None else int(maxiter)
    dev = _is_torch(H.dv)
    if dev:
        if not (H.dv.is_cuda and H.ev.is_cuda) or H.dv.dtype != torch.float64 or H.ev.dtype != torch.float64:
            raise TypeError("H.dv / H.ev must be CUDA float64 tensors")
        if not (H.dv.is_contiguous() and H.ev.is_contiguous()):
            raise ValueError("H.dv / H.ev must be contiguous")
        dptr, eptr = H.dv.data_ptr(), (H.ev.data_ptr() if H.ev.numel() else None)
    else:
        for a in (H.dv, H.ev):
            if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable:
                raise TypeError("H.dv / H.ev must be writeable contiguous float64 numpy arrays")
        dptr, eptr = H.dv.ctypes.data, (H.ev.ctypes.data if H.ev.size else None)
    if H.ev.shape[0] != max(n - 1, 0):
        raise ValueError("ev must have n-1 entries")
    if Q is None:
        qptr, ld, m, dt = None, 1, 0, "f64"
    else:
        qptr, ld, m, nq, dt, qdev = _colmajor_info(Q)
        if qdev != dev:
            raise ValueError("H and Q must both be host arrays or both CUDA tensors")
        if nq != n:
            raise ValueError(f"Q has {nq} columns, expected n = {n}")
    h = handle or default_handle(H.dv.device.index if dev else 0)
    conv, it = c_i32(), c_i64()
    name = "symeig_qr_f64" + ("_q32" if dt == "f32" else "") + ("_dev" if dev else "")
    h.set_exact_order(exact_order)
    h.set_chase_mode(chase_mode)
    h.set_apply_form(apply_form)
    try:
        args = (ctypes.c_void_p(dptr), ctypes.c_void_p(eptr), n, ctypes.c_void_p(qptr), ld, m,
                int(max_layers), tol, maxiter, ctypes.byref(conv), ctypes.byref(it))
        if dev:  # ordered after torch's pending work on H and Q; returns when the solve is done
            with h.on_stream(torch.cuda.current_stream(H.dv.device).cuda_stream):
                h.call(name, *args)
        else:
            h.call(name, *args)
    finally:
        h.set_exact_order(True)
        h.set_chase_mode(0)
        h.set_apply_form(0)
    return H, bool(conv.value), int(it.value)


def eigen_decomp_(H: SymTridiagonal, handle: Handle | None = None, chase_mode: int = 0,
                  apply_form: int = 0):
    """eigen_decomp!(H) (src/bulge_chasing.jl:290-299): Q = I, qr_algorithm!, returns
    (eigenvalues, Q).  The reference returns Diagonal(H.dv); here the 1-D array H.dv.
    chase_mode and apply_form as for qr_algorithm_.  Host arrays go through the C entry point
    symeig_eigen_decomp_f64 (which sets Q = I itself); device tensors through qr_algorithm_."""
    n = H.n
    if _is_torch(H.dv):
        Q = torch.eye(n, dtype=torch.float64, device=H.dv.device).T  # column-major view
        qr_algorithm_(H, Q, handle=handle, chase_mode=chase_mode, apply_form=apply_form)
        return H.dv, Q
    for a in (H.dv, H.ev):
        if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable:
            raise TypeError("H.dv / H.ev must be writeable contiguous float64 numpy arrays")
    if H.ev.shape[0] != max(n - 1, 0):
        raise ValueError("ev must have n-1 entries")
    Q = np.empty((n, n), dtype=np.float64, order="F")
    h = handle or default_handle(0)
    conv, it = c_i32(), c_i64()
    h.set_chase_mode(chase_mode)
    h.set_apply_form(apply_form)
    try:
        h.call("symeig_eigen_decomp_f64", ctypes.c_void_p(H.dv.ctypes.data),
               ctypes.c_void_p(H.ev.ctypes.data if H.ev.size else None), n, ctypes.c_void_p(Q.ctypes.data), n,
               ctypes.byref(conv), ctypes.byref(it))
    finally:
        h.set_chase_mode(0)
        h.set_apply_form(0)
    return H.dv, Q


def qr_algorithm_batched_(d, e, n, Q=None, max_layers: int = 128, tol: float | None = None,
                          maxiter_factor: int = 100, handle: Handle | None = None):
    """Batched qr_algorithm!: count independent solves in one call (no reference counterpart;
    it replaces a loop of qr_algorithm! calls, src/bulge_chasing.jl:146).

    d, e, Q are packed: matrix i has order n[i], its diagonal/off-diagonal follow the previous
    matrices' in d (sum n) and e (sum n-1), and its Q (n_i x n_i column-major) follows the
    previous ones in Q (sum n^2, flat).  All three are numpy arrays (host) or CUDA torch
    tensors (device); Q may be None (eigenvalues only).  d and e are float64; Q is float64 or
    float32 (the FP32-Q variant: the chase stays FP64 and each (c,s) is rounded to float).
    Returns (converged, iters) numpy arrays of length count."""
    n = np.ascontiguousarray(np.asarray(n, dtype=np.int64))
    count = int(n.shape[0])
    conv = np.zeros(count, dtype=np.int32)
    iters = np.zeros(count, dtype=np.int64)
    tol = EPS64 if tol is None else float(tol)
    dev = _is_torch(d)
    for a, what in ((d, "d"), (e, "e")) + (((Q, "Q"),) if Q is not None else ()):
        if dev:
            ok = _is_torch(a) and a.is_cuda and a.is_contiguous() and (
                a.dtype == torch.float64 or (what == "Q" and a.dtype == torch.float32))
            if not ok:
                raise TypeError("d, e must be contiguous CUDA float64 tensors, Q float64 or float32")
        else:
            ok = isinstance(a, np.ndarray) and a.flags.c_contiguous and a.flags.writeable and (
                a.dtype == np.float64 or (what == "Q" and a.dtype == np.float32))
            if not ok:
                raise TypeError("d, e must be writeable contiguous float64 numpy arrays, Q float64 or float32")
    q32 = Q is not None and (Q.dtype == torch.float32 if dev else Q.dtype == np.float32)
    if int(d.shape[0]) != int(n.sum()) or int(e.shape[0]) != int((n - 1).sum()):
        raise ValueError("packed d / e sizes do not match n")
    if Q is not None and int(Q.numel() if dev else Q.size) != int((n * n).sum()):
        raise ValueError("packed Q size does not match n")
    ptr = (lambda a: a.data_ptr()) if dev else (lambda a: a.ctypes.data)
    h = handle or default_handle(d.device.index if dev else 0)
    args = (count, ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(ptr(d)),
            ctypes.c_void_p(ptr(e) if int(e.shape[0]) else None),
            ctypes.c_void_p(ptr(Q) if Q is not None else None), int(max_layers), tol,
            int(maxiter_factor), ctypes.c_void_p(conv.ctypes.data), ctypes.c_void_p(iters.ctypes.data))
    fn = "symeig_qr_batched_f64_q32" if q32 else "symeig_qr_batched_f64"
    if dev:
        with h.on_stream(torch.cuda.current_stream(d.device).cuda_stream):
            h.call(fn + "_dev", *args)
    else:
        if int(e.shape[0]) == 0:
            ebuf = np.zeros(1)
            args = args[:3] + (ctypes.c_void_p(ebuf.ctypes.data),) + args[4:]
        h.call(fn, *args)
    return conv.astype(bool), iters


BATCHED_TILES = 3   # 0: 16 rows x 64 layers, 1: 32 rows x 64 layers, 2: 8 rows x 128 layers


def batched_tuning(fp64: bool = True, split: int | None = None, shape_small: int | None = None,
                   shape_large: int | None = None, handle: Handle | None = None):
    """Read, or with any argument given write, the batched tuning of FP64 (fp64=True) or FP32 Q:
    {"split", "shape_small", "shape_large"} (tiles 0..2).  Process-wide; needs no device."""
    lib = handle._lib if handle is not None else load_library()
    sp, s0, s1 = c_i64(), c_i32(), c_i32()
    check("symeig_batched_tuning_dtype",
          lib.symeig_batched_tuning_dtype(int(fp64), ctypes.byref(sp), ctypes.byref(s0), ctypes.byref(s1), 0))
    if split is not None or shape_small is not None or shape_large is not None:
        sp = c_i64(sp.value if split is None else int(split))
        s0 = c_i32(s0.value if shape_small is None else int(shape_small))
        s1 = c_i32(s1.value if shape_large is None else int(shape_large))
        check("symeig_batched_tuning_dtype",
              lib.symeig_batched_tuning_dtype(int(fp64), ctypes.byref(sp), ctypes.byref(s0), ctypes.byref(s1), 1))
    return {"split": sp.value, "shape_small": s0.value, "shape_large": s1.value}


def batched_autotune(sizes=None, handle: Handle | None = None):
    """Run the batched-apply autotuner over the tiles (rows per tile and layers per pass) for FP64
    and FP32 Q, on matrices of the orders `sizes` (those of the batch to be solved; None: a
    spread of orders over each size class).  Returns ({"f64": tuning, "f32": tuning},
    {"f64": ms, "f32": ms}) where ms[class][tile] is the time of one 128-layer flush of every
    matrix of that class."""
    h = handle or default_handle(0)
    nt = BATCHED_TILES
    ms = (ctypes.c_double * (4 * nt))()
    if sizes is None:
        h.call("symeig_batched_autotune", ms)
    else:
        nn = np.ascontiguousarray(np.asarray(sizes, dtype=np.int64))
        h.call("symeig_batched_autotune_sizes", int(nn.shape[0]), ctypes.c_void_p(nn.ctypes.data), ms)
    tun, times = {}, {}
    for dt, name in ((0, "f64"), (1, "f32")):
        tun[name] = batched_tuning(fp64=(dt == 0), handle=h)
        times[name] = [list(ms[(dt * 2 + c) * nt:(dt * 2 + c + 1) * nt]) for c in range(2)]
    return tun, times


def _dense_square(A, what="A"):
    ptr, ld, m, n, dt, dev = _colmajor_info(A)
    if m != n:
        raise ValueError(f"{what} must be square")
    if dt != "f64":
        raise TypeError(f"{what} must be float64")
    return ptr, ld, n, dev


def sytrd_(A, handle: Handle | None = None):
    """Dense symmetric -> tridiagonal (LAPACK dsytrd, lower; no reference counterpart: the
    step before qr_algorithm! for a dense symmetric A).  A (n x n, both triangles, column-major,
    float64; numpy or CUDA torch) is overwritten as by dsytrd.  Returns (d, e, tau) with
    A = Q SymTridiagonal(d, e) Q^T, Q = orgtr(A, tau)."""
    ptr, ld, n, dev = _dense_square(A)
    h = handle or default_handle(A.device.index if dev else 0)
    if dev:
        d = torch.empty(n, dtype=torch.float64, device=A.device)
        e = torch.empty(max(n - 1, 0), dtype=torch.float64, device=A.device)
        tau = torch.empty(max(n - 1, 0), dtype=torch.float64, device=A.device)
        with h.on_stream(torch.cuda.current_stream(A.device).cuda_stream):
            h.call("symeig_sytrd_f64_dev", n, ctypes.c_void_p(ptr), ld, ctypes.c_void_p(d.data_ptr()),
                   ctypes.c_void_p(e.data_ptr() if n > 1 else None), ctypes.c_void_p(tau.data_ptr() if n > 1 else None))
        return d, e, tau
    d, e, tau = np.empty(n), np.empty(max(n - 1, 0)), np.empty(max(n - 1, 0))
    h.call("symeig_sytrd_f64", n, ctypes.c_void_p(ptr), ld, d.ctypes.data,
           ctypes.c_void_p(e.ctypes.data if n > 1 else None), ctypes.c_void_p(tau.ctypes.data if n > 1 else None))
    return d, e, tau


def orgtr(A, tau, handle: Handle | None = None):
    """Q of sytrd_ (LAPACK dorgtr, lower) as a new column-major matrix."""
    ptr, ld, n, dev = _dense_square(A)
    h = handle or default_handle(A.device.index if dev else 0)
    if dev:
        Q = torch.empty(n, n, dtype=torch.float64, device=A.device).T
        t = tau.contiguous()
        with h.on_stream(torch.cuda.current_stream(A.device).cuda_stream):
            h.call("symeig_orgtr_f64_dev", n, ctypes.c_void_p(ptr), ld,
                   ctypes.c_void_p(t.data_ptr() if n > 1 else None), ctypes.c_void_p(Q.data_ptr()), n)
        return Q
    Q = np.empty((n, n), order="F")
    t = np.ascontiguousarray(tau, dtype=np.float64)
    h.call("symeig_orgtr_f64", n, ctypes.c_void_p(ptr), ld, ctypes.c_void_p(t.ctypes.data if n > 1 else None),
           Q.ctypes.data, n)
    return Q


def syev(A, handle: Handle | None = None):
    """Dense symmetric eigensolve on the device: sytrd, orgtr, then qr_algorithm! on the
    tridiagonal with Q = the orthogonal factor.  Returns (lam, V, converged, iters): lam
    unsorted as the reference's H.dv, V the eigenvectors (column-major).  A CUDA tensor A is
    overwritten (as by sytrd_); a numpy A is left unchanged."""
    ptr, ld, n, dev = _dense_square(A)
    h = handle or default_handle(A.device.index if dev else 0)
    conv, it = c_i32(), c_i64()
    if dev:
        lam = torch.empty(n, dtype=torch.float64, device=A.device)
        V = torch.empty(n, n, dtype=torch.float64, device=A.device).T
        with h.on_stream(torch.cuda.current_stream(A.device).cuda_stream):
            h.call("symeig_syev_f64_dev", n, ctypes.c_void_p(ptr), ld, ctypes.c_void_p(lam.data_ptr()),
                   ctypes.c_void_p(V.data_ptr()), n, ctypes.byref(conv), ctypes.byref(it))
        return lam, V, bool(conv.value), int(it.value)
    lam = np.empty(n)
    V = np.empty((n, n), order="F")
    h.call("symeig_syev_f64", n, ctypes.c_void_p(ptr), ld, lam.ctypes.data, V.ctypes.data, n,
           ctypes.byref(conv), ctypes.byref(it))
    return lam, V, bool(conv.value), int(it.value)


def eig_adjoint(lam, Q, glam, gQ=None, handle: Handle | None = None):
    """dL/d(d, e) of the tridiagonal eigensolve from dL/dlam and dL/dQ (symeig_eig_adjoint_f64*).

    Single matrix: lam (n,), Q (n, n) column-major, glam (n,), gQ (n, n) or None.  Batch of B
    matrices of one order: lam (B, n), Q (B, n, n) with each Q[b] column-major (i.e.
    Q[b].stride(0) == 1), glam (B, n), gQ like Q or None.  numpy (host) or CUDA torch (device).
    Returns (gd, ge) with shapes (n,), (n-1,) or (B, n), (B, n-1)."""
    dev = _is_torch(lam)
    batched = lam.ndim == 2
    B = int(lam.shape[0]) if batched else 1
    n = int(lam.shape[-1])
    h = handle or default_handle(lam.device.index if dev else 0)

    def colmajor_flat(M):
        # the column-major memory of each n x n matrix, back to back
        if dev:
            return (M.transpose(-1, -2).contiguous() if M.ndim == 2 else M.transpose(-1, -2).contiguous()).reshape(-1)
        return np.ascontiguousarray(np.swapaxes(M, -1, -2)).reshape(-1)

    if dev:
        zl = lambda *s: torch.empty(*s, dtype=torch.float64, device=lam.device)
        lam_c, glam_c = lam.contiguous().reshape(-1), glam.contiguous().reshape(-1)
        Qf = colmajor_flat(Q)
        gQf = colmajor_flat(gQ) if gQ is not None else None
        gd, ge = zl(B * n), zl(max(B * (n - 1), 1))
        ptr = lambda a: ctypes.c_void_p(a.data_ptr() if a is not None else None)
        with h.on_stream(torch.cuda.current_stream(lam.device).cuda_stream):
            h.call("symeig_eig_adjoint_f64_dev", B, n, ptr(lam_c), ptr(Qf), ptr(glam_c), ptr(gQf), ptr(gd), ptr(ge))
    else:
        lam_c = np.ascontiguousarray(lam, dtype=np.float64).reshape(-1)
        glam_c = np.ascontiguousarray(glam, dtype=np.float64).reshape(-1)
        Qf = colmajor_flat(np.asarray(Q, dtype=np.float64))
        gQf = colmajor_flat(np.asarray(gQ, dtype=np.float64)) if gQ is not None else None
        gd, ge = np.empty(B * n), np.empty(max(B * (n - 1), 1))
        ptr = lambda a: ctypes.c_void_p(a.ctypes.data if a is not None else None)
        h.call("symeig_eig_adjoint_f64", B, n, ptr(lam_c), ptr(Qf), ptr(glam_c), ptr(gQf), ptr(gd), ptr(ge))
    ge = ge[: B * (n - 1)]
    if batched:
        return gd.reshape(B, n), ge.reshape(B, n - 1)
    return gd, ge


if torch is not None:
    class TridiagEigh(torch.autograd.Function):
        """(lam, Q) = eigen-decomposition of SymTridiagonal(d, e) by the GB300 qr_algorithm!,
        differentiable: the backward is symeig_eig_adjoint_f64_dev.  lam is unsorted (as
        H.dv of the reference); Q is returned as a column-major view.  The counterpart of the
        Julia ChainRulesCore rrule of the Julia binding.  apply(d, e[, chase_mode[, apply_form]]):
        the forward solve's chase mode and apply form as for qr_algorithm_ (default: the
        reference's sweep sequence, canonical apply); the backward does not depend on them."""

        @staticmethod
        def forward(ctx, d, e, chase_mode=0, apply_form=0):
            n = d.shape[0]
            dd, ee = d.detach().clone().contiguous(), e.detach().clone().contiguous()
            Q = torch.eye(n, dtype=torch.float64, device=d.device).T.contiguous().T
            _, conv, _ = qr_algorithm_(SymTridiagonal(dd, ee), Q, chase_mode=int(chase_mode),
                                       apply_form=int(apply_form))
            if not conv:
                raise RuntimeError("qr_algorithm! did not converge")
            ctx.save_for_backward(dd, Q)
            return dd, Q

        @staticmethod
        def backward(ctx, glam, gQ):
            lam, Q = ctx.saved_tensors
            if glam is None:
                glam = torch.zeros_like(lam)
            gd, ge = eig_adjoint(lam, Q, glam.contiguous(), gQ)
            return gd, ge, None, None

    class TridiagEighBatched(torch.autograd.Function):
        """Batched TridiagEigh: d (B, n), e (B, n-1) -> lam (B, n), Q (B, n, n) (each Q[b]
        column-major), via symeig_qr_batched_f64_dev and the batched adjoint."""

        @staticmethod
        def forward(ctx, d, e):
            B, n = d.shape
            dd, ee = d.detach().clone().contiguous(), e.detach().clone().contiguous()
            Qf = torch.eye(n, dtype=torch.float64, device=d.device).reshape(1, n, n).repeat(B, 1, 1).reshape(-1)
            conv, _ = qr_algorithm_batched_(dd.reshape(-1), ee.reshape(-1), [n] * B, Qf)
            if not conv.all():
                raise RuntimeError("qr_algorithm! did not converge")
            Q = Qf.reshape(B, n, n).transpose(1, 2)   # column-major per matrix
            ctx.save_for_backward(dd, Q)
            return dd, Q

        @staticmethod
        def backward(ctx, glam, gQ):
            lam, Q = ctx.saved_tensors
            if glam is None:
                glam = torch.zeros_like(lam)
            return eig_adjoint(lam, Q, glam.contiguous(), gQ)


def bulk_wave_order_2x2_lmul_(A, givens, handle: Handle | None = None) -> None:
    """A <- (row rotations) * A: the bulk form of lmul!(G, A) (src/simple_givens.jl:38-51) for an
    (m-1) x k grid, layer-major (for L, for i: rows i, i+1).  The reference has only the
    single-rotation lmul!.  Same array conventions as bulk_wave_order_2x2_rmul_, with givens of
    shape (m-1, k, 2)."""
    ptr, ld, m, n, dt, dev = _colmajor_info(A)
    gm = int(givens.shape[0])
    if m >= 2 and gm != m - 1:
        raise ValueError(f"givens has {gm} rows, expected m-1 = {m - 1}")
    if m < 2 or n == 0 or int(givens.shape[1]) == 0:
        return None
    h = handle or default_handle(A.device.index if _is_torch(A) else 0)
    gptr, keep, k = _givens_ptr(givens, dt, dev)
    name = f"symeig_apply_givens_left_{dt}" + ("_dev" if dev else "")
    if dev:
        with h.on_stream(torch.cuda.current_stream(A.device).cuda_stream):
            h.call(name, ctypes.c_void_p(ptr), ld, m, n, ctypes.c_void_p(gptr), k)
        torch.cuda.current_stream(A.device).synchronize()
    else:
        h.call(name, ctypes.c_void_p(ptr), ld, m, n, ctypes.c_void_p(gptr), k)
    del keep
    return None
