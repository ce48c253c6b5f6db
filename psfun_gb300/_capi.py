"""ctypes binding of libpsfun_gb300.so (include/psfun_gb300.h).

The library is built in-tree by psfun_gb300/build.py.  There is no CPU
fallback: if the shared library is missing or cannot be loaded this module
raises, and every compute entry point needs a CUDA device.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libpsfun_gb300.so"

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)
vp = C.c_void_p
USERF = C.CFUNCTYPE(C.c_double, C.c_double, C.c_int)
ZFUN = C.CFUNCTYPE(None, dp, dp, C.c_void_p)

class BatchItem(C.Structure):
    """psfun_batch_item"""
    _fields_ = [("a", C.c_void_p), ("nrhs", C.c_int), ("x", C.c_void_p), ("y", C.c_void_p),
                ("scaling", C.c_double)]


class QuadItem(C.Structure):
    """psfun_quad_item"""
    _fields_ = [("a", C.c_void_p), ("nrhs", C.c_int), ("x", C.c_void_p), ("y", C.c_void_p), ("N", C.c_int),
                ("xi", C.c_void_p), ("c", C.c_void_p), ("eta", C.c_double), ("sign", C.c_double)]


# name -> (restype, argtypes)
PROTOS = {
    "psfun_gpu_version": (C.c_char_p, []),
    "psfun_gpu_last_error": (C.c_char_p, []),
    "psfun_gpu_kernel_launches": (C.c_longlong, []),
    "psfun_gpu_set_stream": (C.c_int, [vp]),
    "psfun_gpu_get_stream": (vp, []),
    "psfun_gpu_profile_enable": (C.c_int, [C.c_int]),
    "psfun_gpu_profile_read": (C.c_int, [C.c_int, C.POINTER(C.c_longlong), dp]),
    "psfun_gpu_csr_create": (C.c_int, [C.c_int64, C.c_int64, ip, ip, dp, C.c_int, C.POINTER(vp)]),
    "psfun_gpu_csr_destroy": (C.c_int, [vp]),
    "psfun_gpu_csr_info": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64), dp]),
    "psfun_gpu_csr_is_symmetric": (C.c_int, [vp, C.POINTER(C.c_int)]),
    "psfun_gpu_csr_spmv_device": (C.c_int, [vp, C.c_double, vp, C.c_double, vp]),
    "psfun_gpu_csr_spmv": (C.c_int, [vp, C.c_double, dp, C.c_double, dp]),
    "psfun_gpu_serial_create": (C.c_int, [C.POINTER(vp)]),
    "psfun_gpu_serial_destroy": (C.c_int, [vp]),
    "psfun_gpu_serial_set_string": (C.c_int, [vp, C.c_char_p, C.c_char_p]),
    "psfun_gpu_serial_set_real": (C.c_int, [vp, C.c_char_p, C.c_double]),
    "psfun_gpu_serial_set_integer": (C.c_int, [vp, C.c_char_p, C.c_int]),
    "psfun_gpu_serial_set_function": (C.c_int, [vp, C.c_char_p, USERF]),
    "psfun_gpu_serial_get": (C.c_int, [vp, C.c_char_p, C.c_char_p, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "psfun_gpu_serial_apply": (C.c_int, [vp, C.c_int, dp, C.c_int, dp, dp]),
    "psfun_gpu_serial_apply_sparse": (C.c_int, [vp, vp, dp, dp]),
    "psfun_gpu_serial_apply_device_static": (C.c_int, [vp, C.c_int, vp, C.c_int, vp, vp]),
    "psfun_gpu_krylov_create": (C.c_int, [C.POINTER(vp)]),
    "psfun_gpu_krylov_destroy": (C.c_int, [vp]),
    "psfun_gpu_krylov_set_string": (C.c_int, [vp, C.c_char_p, C.c_char_p]),
    "psfun_gpu_krylov_set_integer": (C.c_int, [vp, C.c_char_p, C.c_int]),
    "psfun_gpu_krylov_set_real": (C.c_int, [vp, C.c_char_p, C.c_double]),
    "psfun_gpu_krylov_precinit": (C.c_int, [vp, C.c_char_p]),
    "psfun_gpu_selftest_wait": (C.c_int, [C.c_int]),
    "psfun_gpu_krylov_precbuild": (C.c_int, [vp, vp]),
    "psfun_gpu_d_krylov_apply": (C.c_int, [vp, vp, vp, dp, dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                           C.POINTER(C.c_int), dp, dp, C.c_int, C.POINTER(C.c_int)]),
    "psfun_gpu_d_krylov_apply_device": (C.c_int, [vp, vp, vp, vp, vp, C.c_double, C.c_int, C.c_int, C.c_int,
                                                  C.POINTER(C.c_int), dp, dp, C.c_int, C.POINTER(C.c_int)]),
    "psfun_gpu_d_krylov_batch": (C.c_int, [vp, vp, C.c_int, C.POINTER(BatchItem), C.c_double, C.c_int, C.c_int,
                                            C.POINTER(C.c_int), dp, C.POINTER(C.c_int)]),
    "psfun_gpu_z_quadrature_batch": (C.c_int, [C.c_int, C.POINTER(QuadItem), C.c_double, C.c_int, C.POINTER(C.c_int),
                                                dp, C.POINTER(C.c_int)]),
    "psfun_gpu_talbot_rule": (C.c_int, [C.c_int, dp, dp]),
    "psfun_gpu_d_expm_adjoint_device": (C.c_int, [vp, C.c_double, vp, vp, C.c_int, C.c_double, C.c_int, C.c_int, vp,
                                                  vp, dp, vp, C.POINTER(C.c_int)]),
    "psfun_gpu_dcg": (C.c_int, [C.c_char_p, vp, C.c_char_p, dp, C.c_double, C.c_double, dp, C.c_double, C.c_int,
                                C.c_int, C.POINTER(C.c_int), dp]),
    "psfun_gpu_dcg_device": (C.c_int, [C.c_char_p, vp, C.c_char_p, vp, C.c_double, C.c_double, vp, C.c_double,
                                       C.c_int, C.c_int, C.POINTER(C.c_int), dp]),
    "psfun_gpu_dcg_ex": (C.c_int, [C.c_char_p, vp, C.c_char_p, dp, C.c_double, C.c_double, dp, C.c_double, C.c_int,
                                   C.c_int, C.c_int, C.POINTER(C.c_int), dp, dp]),
    "psfun_gpu_dcg_ex_device": (C.c_int, [C.c_char_p, vp, C.c_char_p, vp, C.c_double, C.c_double, vp, C.c_double,
                                          C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), dp, dp]),
    "psfun_gpu_hhtmethod1": (C.c_int, [ZFUN, C.c_void_p, C.c_int, dp, dp, dp, dp, dp]),
    "psfun_gpu_ellipkkp": (C.c_int, [C.c_double, dp]),
    "psfun_gpu_d_ellipj": (C.c_int, [C.c_double, C.c_double, dp, dp, dp]),
    "psfun_gpu_z_ellipj": (C.c_int, [dp, C.c_double, dp, dp, dp]),
    "psfun_gpu_horner": (C.c_double, [dp, C.c_int, C.c_double]),
    "psfun_gpu_z_quadrature_apply": (C.c_int, [vp, C.c_int, dp, dp, C.c_double, C.c_double, dp, dp, C.c_double,
                                               C.c_int, C.POINTER(C.c_int), dp]),
    "psfun_gpu_z_quadrature_apply_device": (C.c_int, [vp, C.c_int, dp, dp, C.c_double, C.c_double, vp, vp,
                                                      C.c_double, C.c_int, C.POINTER(C.c_int), dp]),
}

_lib = None


def load(path: Path | None = None):
    """Loads the in-tree library; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(psfun_gb300 has no CPU fallback)")
    L = C.CDLL(str(p))
    for name, (res, args) in PROTOS.items():
        fn = getattr(L, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load().psfun_gpu_last_error().decode()


def kernel_launches() -> int:
    return int(load().psfun_gpu_kernel_launches())
