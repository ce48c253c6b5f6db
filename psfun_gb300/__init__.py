"""psfun_gb300 -- GB300-native (sm_103a) implementation of PSFUN's f(A)x path.

The compute lives in the in-tree shared library lib/libpsfun_gb300.so (CUDA
kernels behind a C-ABI, include/psfun_gb300.h); this package is the Python
mirror of the reference's Fortran API over that C-ABI.
"""
from .api import (  # noqa: F401
    CsrMatrix,
    KrylovResult,
    PsfunDKrylov,
    PsfunDSerial,
    PsfunError,
    PsfunZQuadrature,
    ellipj,
    ellipkkp,
    expm_adjoint,
    hhtmethod1,
    talbot_rule,
    krylov_batch,
    quadrature_batch,
    horner,
    psb_krylov,
)

__version__ = "0.1.0"
