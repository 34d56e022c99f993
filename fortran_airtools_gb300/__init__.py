"""fortran_airtools_gb300 -- GB300-native (sm_103a) AIR reconstruction hot path.

The package mirrors the reference's three Fortran modules on top of the
C-ABI library libfair_gb300.so (include/fair_gpu.h):

* ``sparse_matrices``   -- type(csr_matrix) on the GPU and its procedures;
* ``system_generation`` -- paralleltomo / fanlineartomo ray tracing, noise;
* ``airms``             -- art, twin_art, sirt, gradient_descent, normest;
* ``phantomgallery``    -- Shepp-Logan and seeded synthetic phantoms.

All O(nnz) work runs in hand-written CUDA kernels; without the library the
import of any of these modules raises at first use.
"""
from ._clib import FairError, Opts, lib  # noqa: F401
from . import airms, batch, mfree, phantomgallery, sparse_matrices, system_generation  # noqa: F401
from .batch import Batch  # noqa: F401
from .mfree import MatrixFree  # noqa: F401
from .sparse_matrices import CSRMatrix  # noqa: F401
from .system_generation import Data, fanlineartomo, linspace, paralleltomo, paralleltomo_f32  # noqa: F401

__all__ = ["FairError", "Opts", "lib", "airms", "batch", "mfree", "phantomgallery",
           "sparse_matrices", "system_generation", "Batch", "CSRMatrix", "Data", "MatrixFree",
           "fanlineartomo", "linspace", "paralleltomo", "paralleltomo_f32"]
