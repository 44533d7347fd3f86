"""GB300-native (sm_103a) hot path of SymmetricEigenProblem.jl.

The package holds the CUDA sources of libsymeig.so (``csrc/``), its in-tree build
(``build.py``), the ctypes binding of its C ABI (``_lib.py``) and the host-side mirror of
the reference's functions (``api.py``).  The directory name carries a dot, so Python code
loads it by path (see ``__graft_entry__.load_package``).
"""
from .api import (  # noqa: F401
    SymTridiagonal,
    bulk_wave_order_2x2_lmul_,
    bulk_wave_order_2x2_rmul_,
    bulk_wave_order_2x2_rmul_parallel_,
    eig_adjoint,
    batched_autotune,
    batched_tuning,
    qr_algorithm_batched_,
    eigen_decomp_,
    get_rotation,
    givens_buffer,
    orgtr,
    qr_algorithm_,
    syev,
    sytrd_,
)
from ._lib import Handle, SymeigError, default_handle, load as load_library, load_checked  # noqa: F401
from .build import build, LIB as LIBRARY_PATH  # noqa: F401

try:  # the autograd Functions need torch
    from .api import TridiagEigh, TridiagEighBatched  # noqa: F401
except ImportError:  # pragma: no cover
    pass
