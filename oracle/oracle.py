"""ctypes wrapper of the C restatement (oracle/psfun_oracle.c) plus dense
FP64 SciPy oracles.  TEST INFRASTRUCTURE ONLY: the parity checker, never the
product path.

Parity pin: horner / ellipkkp / ellipj against the control values of
examples/utils/utiltest.f90:63-87 (tests/golden/utiltest_control.json).  The
Krylov, Pade, CRAM and CG restatements have no golden vectors in the reference
(it cannot be built here); they are pinned against the dense oracles below.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "lib" / "libpsfun_oracle.so"

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)

ERR = {
    "SUCCESS": 0,
    "INVALID_ARGS_COMBINATION": 111,
    "INVALID_VECT_STATE": 1124,
    "FROM_SUBROUTINE": 4010,
    "FROM_SUBROUTINE_NON": 4011,
    "INVALID_ISTOP": 5001,
}


class OrcCsr(C.Structure):
    _fields_ = [("n", C.c_int64), ("nnz", C.c_int64), ("irp", _ip), ("ja", _ip), ("val", _dp)]


USERF = C.CFUNCTYPE(C.c_double, C.c_double, C.c_int)
ZFUN = C.CFUNCTYPE(None, _dp, _dp, C.c_void_p)


class OrcSerial(C.Structure):
    _fields_ = [("fname", C.c_char * 24), ("variant", C.c_char * 24), ("scaling", C.c_double),
                ("padedegree", C.c_int), ("phiorder", C.c_int), ("f_ptr", USERF)]


def build() -> Path:
    if not LIB.exists() or LIB.stat().st_mtime < (HERE / "psfun_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_dgpadm.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, C.POINTER(C.c_int)]
        L.orc_dnchbv.argtypes = [C.c_int, C.c_double, _dp, C.c_int, _dp]
        L.orc_dnchbv.restype = None
        L.orc_dschbv.argtypes = [C.c_int, C.c_double, _dp, C.c_int, _dp]
        L.orc_dgchbv.argtypes = [C.c_int, C.c_double, _dp, C.c_int, _dp]
        L.orc_expm_sasq.argtypes = [C.c_int, _dp, _dp]
        L.orc_expm_taylor.argtypes = [C.c_int, _dp, _dp]
        L.orc_phi_augmented.argtypes = [C.c_int, C.c_int, C.c_double, _dp, C.c_int, _dp, _dp, C.c_int]
        L.orc_sym_eig.argtypes = [C.c_int, _dp, C.c_int, _dp, _dp]
        L.orc_serial_apply.argtypes = [C.POINTER(OrcSerial), C.c_int, _dp, C.c_int, _dp, _dp]
        for f in (L.orc_arnoldi, L.orc_lanczos):
            f.argtypes = [C.POINTER(OrcSerial), C.POINTER(OrcCsr), _dp, _dp, C.c_double, C.c_int, C.c_int,
                          C.c_int, C.POINTER(C.c_int), _dp, _dp, C.c_int, C.POINTER(C.c_int)]
        L.orc_saiarnoldi.argtypes = [C.POINTER(OrcSerial), C.POINTER(OrcCsr), _dp, C.c_double, C.c_int, C.c_int, _dp,
                                     _dp, C.c_double, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                     C.POINTER(C.c_double), _dp, C.c_int, C.POINTER(C.c_int)]
        L.orc_dcg.argtypes = [C.POINTER(OrcCsr), _dp, _dp, C.c_double, C.c_double, _dp, C.c_double, C.c_int,
                              C.c_int, C.POINTER(C.c_int), _dp]
        L.orc_dcg_hist.argtypes = [C.POINTER(OrcCsr), _dp, _dp, C.c_double, C.c_double, _dp, C.c_double, C.c_int,
                                   C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, C.POINTER(C.c_int), _dp]
        L.orc_bjac_build.argtypes = [C.POINTER(OrcCsr), C.c_int, C.POINTER(C.c_void_p)]
        L.orc_bjac_free.argtypes = [C.c_void_p]
        L.orc_bjac_free.restype = None
        L.orc_bjac_apply.argtypes = [C.c_void_p, _dp, _dp]
        L.orc_bjac_apply.restype = None
        L.orc_bjac_export.argtypes = [C.c_void_p, _ip, _ip, _dp, _ip, _dp]
        L.orc_bjac_export.restype = C.c_int64
        L.orc_dcg_bjac_hist.argtypes = [C.POINTER(OrcCsr), C.c_void_p, _dp, C.c_double, C.c_double, _dp, C.c_double,
                                        C.c_int, C.c_int, C.POINTER(C.c_int), _dp, _dp, _dp, C.POINTER(C.c_int), _dp]
        L.orc_saiarnoldi_bjac.argtypes = [C.POINTER(OrcSerial), C.POINTER(OrcCsr), C.c_void_p, C.c_double, C.c_int,
                                          C.c_int, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int,
                                          C.POINTER(C.c_int), C.POINTER(C.c_double), _dp, C.c_int,
                                          C.POINTER(C.c_int)]
        L.orc_horner.argtypes = [_dp, C.c_int, C.c_double]
        L.orc_horner.restype = C.c_double
        L.orc_ellipkkp.argtypes = [C.c_double, _dp]
        L.orc_ellipkkp.restype = None
        L.orc_d_ellipj.argtypes = [C.c_double, C.c_double, _dp, _dp, _dp]
        L.orc_d_ellipj.restype = None
        L.orc_z_ellipj.argtypes = [_dp, C.c_double, _dp, _dp, _dp]
        L.orc_z_ellipj.restype = None
        L.orc_hhtmethod1.argtypes = [ZFUN, C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_spmv.argtypes = [C.POINTER(OrcCsr), C.c_double, _dp, C.c_double, _dp]
        L.orc_spmv.restype = None
        L.orc_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_dp)


def set_threads(n: int) -> int:
    return lib().orc_set_threads(int(n))


class Csr:
    """Keeps the numpy arrays alive behind an OrcCsr."""

    def __init__(self, irp, ja, val):
        self.irp = np.ascontiguousarray(irp, dtype=np.int32)
        self.ja = np.ascontiguousarray(ja, dtype=np.int32)
        self.val = np.ascontiguousarray(val, dtype=np.float64)
        self.s = OrcCsr(len(self.irp) - 1, len(self.ja), self.irp.ctypes.data_as(_ip),
                        self.ja.ctypes.data_as(_ip), _p(self.val))

    @classmethod
    def from_scipy(cls, m):
        m = m.tocsr()
        m.sort_indices()
        return cls(m.indptr, m.indices, m.data)


def serial(fname="EXP", variant="EXPOKIT", scaling=1.0, padedegree=6, phiorder=1, f=None):
    s = OrcSerial()
    s.fname = fname.encode()
    s.variant = variant.encode()
    s.scaling = scaling
    s.padedegree = padedegree
    s.phiorder = phiorder
    if f is not None:
        cb = USERF(f)
        s.f_ptr = cb
        s._keep = cb
    return s


def serial_apply(fun, a, x):
    a = np.asfortranarray(a, dtype=np.float64)
    n = a.shape[0]
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(n)
    info = lib().orc_serial_apply(C.byref(fun), n, _p(a), n, _p(y), _p(x))
    return y, info


def dgpadm(H, t=1.0, ideg=6):
    H = np.asfortranarray(H, dtype=np.float64)
    m = H.shape[0]
    E = np.zeros((m, m), order="F")
    ns = C.c_int(0)
    info = lib().orc_dgpadm(ideg, m, t, _p(H), m, _p(E), C.byref(ns))
    return E, info, ns.value


def krylov(method, fun, A: Csr, x, eps, itmax=200, istop=1, drop_last=True):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    it = C.c_int(0)
    err = C.c_double(0.0)
    res = np.zeros(itmax + 2)
    nres = C.c_int(0)
    f = lib().orc_arnoldi if method.upper() == "ARNOLDI" else lib().orc_lanczos
    info = f(C.byref(fun), C.byref(A.s), _p(y), _p(x), eps, itmax, istop, 1 if drop_last else 0,
             C.byref(it), C.byref(err), _p(res), len(res), C.byref(nres))
    return dict(y=y, info=info, iter=it.value, err=err.value, res=res[: nres.value].copy())


def diag_inv(A: Csr):
    """Inverse diagonal of A for the DIAG preconditioner (a zero entry -> 1)."""
    n = len(A.irp) - 1
    d = np.zeros(n)
    for i in range(n):
        lo, hi = A.irp[i], A.irp[i + 1]
        sel = A.ja[lo:hi] == i
        d[i] = A.val[lo:hi][sel].sum()
    return np.where(d != 0.0, 1.0 / np.where(d != 0.0, d, 1.0), 1.0)


BJAC_BLOCK_ROWS = 32  # rows per diagonal block of the BJAC preconditioner


class Bjac:
    """Block-Jacobi ILU(0) factors of A (orc_bjac_build), blocks of bs rows."""

    def __init__(self, A: Csr, bs: int = BJAC_BLOCK_ROWS):
        self.A = A
        h = C.c_void_p()
        info = lib().orc_bjac_build(C.byref(A.s), int(bs), C.byref(h))
        if info != 0:
            raise ValueError(f"orc_bjac_build: info={info}")
        self.h = h

    def apply(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.zeros_like(r)
        lib().orc_bjac_apply(self.h, _p(r), _p(z))
        return z

    def factors(self):
        n = len(self.A.irp) - 1
        irp = np.zeros(n + 1, dtype=np.int32)
        lib().orc_bjac_export(self.h, irp.ctypes.data_as(_ip), None, None, None, None)
        nz = int(irp[-1])
        ja = np.zeros(nz, dtype=np.int32)
        val = np.zeros(nz)
        dpos = np.zeros(n, dtype=np.int32)
        udinv = np.zeros(n)
        lib().orc_bjac_export(self.h, irp.ctypes.data_as(_ip), ja.ctypes.data_as(_ip), _p(val),
                              dpos.ctypes.data_as(_ip), _p(udinv))
        return dict(irp=irp, ja=ja, val=val, dpos=dpos, udinv=udinv)

    def __del__(self):
        try:
            lib().orc_bjac_free(self.h)
        except Exception:
            pass


def saiarnoldi(fun, A: Csr, x, eps, tau=0.0, prec="NONE", initmax=200, inistop=1, itmax=200, istop=1,
               drop_last=True):
    """psfun_d_saiarnoldi with kmethd 'CG' (krylov/rational/psfun_d_sai.f90)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros_like(x)
    it = C.c_int(0)
    err = C.c_double(0.0)
    res = np.zeros(itmax + 2)
    nres = C.c_int(0)
    if prec.upper() == "BJAC":
        P = Bjac(A)
        info = lib().orc_saiarnoldi_bjac(C.byref(fun), C.byref(A.s), P.h, float(tau), int(initmax), int(inistop),
                                         _p(y), _p(x), eps, itmax, istop, 1 if drop_last else 0, C.byref(it),
                                         C.byref(err), _p(res), len(res), C.byref(nres))
        return dict(y=y, info=info, iter=it.value, err=err.value, res=res[: nres.value].copy())
    dinv = diag_inv(A) if prec.upper() == "DIAG" else None
    info = lib().orc_saiarnoldi(C.byref(fun), C.byref(A.s), _p(dinv) if dinv is not None else None, float(tau),
                                int(initmax), int(inistop), _p(y), _p(x), eps, itmax, istop, 1 if drop_last else 0,
                                C.byref(it), C.byref(err), _p(res), len(res), C.byref(nres))
    return dict(y=y, info=info, iter=it.value, err=err.value, res=res[: nres.value].copy())


def dcg(A: Csr, b, eta, zeta, x0=None, eps=1e-7, itmax=1000, istop=2, prec="NONE"):
    if prec.upper() == "BJAC":
        r = dcg_cond(A, b, eta, zeta, x0, eps, itmax, istop, prec)
        return dict(x=r["x"], info=r["info"], iter=r["iter"], err=r["err"])
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    dinv = diag_inv(A) if prec.upper() == "DIAG" else None
    it = C.c_int(0)
    err = C.c_double(0.0)
    info = lib().orc_dcg(C.byref(A.s), _p(dinv) if dinv is not None else None, _p(b), eta, zeta, _p(x), eps,
                         itmax, istop, C.byref(it), C.byref(err))
    return dict(x=x, info=info, iter=it.value, err=err.value)


def dcg_cond(A: Csr, b, eta, zeta, x0=None, eps=1e-7, itmax=1000, istop=2, prec="NONE"):
    """dcg with the reference's optional cond (psfun_dcg.F90:237-246, 312-320,
    336-353): the CG tridiagonal td/tu, its extreme eigenvalues by LAPACK's
    symmetric tridiagonal solver (scipy), cond = eig(max) / eig(min); and the
    per-iteration errnum/errden."""
    import scipy.linalg as sla
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
    dinv = diag_inv(A) if prec.upper() == "DIAG" else None
    it = C.c_int(0)
    err = C.c_double(0.0)
    nt = C.c_int(0)
    td = np.zeros(max(itmax, 1))
    tu = np.zeros(max(itmax, 1))
    eh = np.zeros(max(itmax, 1))
    if prec.upper() == "BJAC":
        P = Bjac(A)
        info = lib().orc_dcg_bjac_hist(C.byref(A.s), P.h, _p(b), eta, zeta, _p(x), eps, itmax, istop, C.byref(it),
                                       C.byref(err), _p(td), _p(tu), C.byref(nt), _p(eh))
    else:
        info = lib().orc_dcg_hist(C.byref(A.s), _p(dinv) if dinv is not None else None, _p(b), eta, zeta, _p(x),
                                  eps, itmax, istop, C.byref(it), C.byref(err), _p(td), _p(tu), C.byref(nt), _p(eh))
    m = nt.value
    cond = 0.0
    if m > 0:
        ev = sla.eigvalsh_tridiagonal(td[:m], tu[:m - 1]) if m > 1 else td[:1]
        cond = float(ev[-1] / ev[0])
    return dict(x=x, info=info, iter=it.value, err=err.value, cond=cond, td=td[:m].copy(), tu=tu[:max(m - 1, 0)].copy(),
                errh=eh[: it.value].copy())


def spmv(A: Csr, x, alpha=1.0, beta=0.0, y=None):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(A.s.n) if y is None else np.array(y, dtype=np.float64)
    lib().orc_spmv(C.byref(A.s), alpha, _p(x), beta, _p(y))
    return y


def horner(coeffs, x):
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    return lib().orc_horner(_p(c), len(c), x)


def ellipkkp(L):
    K = np.zeros(2)
    lib().orc_ellipkkp(L, _p(K))
    return K


def d_ellipj(u, L):
    sn, cn, dn = C.c_double(), C.c_double(), C.c_double()
    lib().orc_d_ellipj(u, L, C.byref(sn), C.byref(cn), C.byref(dn))
    return sn.value, cn.value, dn.value


def z_ellipj(u, L):
    uu = np.array([u.real, u.imag])
    sn, cn, dn = np.zeros(2), np.zeros(2), np.zeros(2)
    lib().orc_z_ellipj(_p(uu), L, _p(sn), _p(cn), _p(dn))
    return complex(*sn), complex(*cn), complex(*dn)


def hhtmethod1(zfun, N, rparams):
    @ZFUN
    def cb(z, res, ctx):
        v = complex(zfun(complex(z[0], z[1])))
        res[0] = v.real
        res[1] = v.imag

    rp = np.ascontiguousarray(rparams, dtype=np.float64)
    xi = np.zeros(2 * N)
    c = np.zeros(2 * N)
    eta = C.c_double()
    sign = C.c_double()
    info = lib().orc_hhtmethod1(cb, None, N, _p(rp), _p(xi), _p(c), C.byref(eta), C.byref(sign))
    return xi[0::2] + 1j * xi[1::2], c[0::2] + 1j * c[1::2], eta.value, sign.value, info


# ---------------------------------------------------------------------------
# dense FP64 oracles (library calls, not restatements)
# ---------------------------------------------------------------------------
def dense_expm_times(A, x, t=1.0):
    import scipy.linalg as sl
    return sl.expm(t * np.asarray(A, dtype=np.float64)) @ x


def dense_phi1_times(A, x, t=1.0):
    """phi_1(tA) x from the last column of expm([[tA, x],[0, 0]])."""
    import scipy.linalg as sl
    n = A.shape[0]
    M = np.zeros((n + 1, n + 1))
    M[:n, :n] = t * np.asarray(A)
    M[:n, n] = x
    return sl.expm(M)[:n, n]


def kron_expm_2d_times(T, X, t=1.0):
    """exp(-t (T (+) T)) vec(X) for a 2-D Kronecker-sum Laplacian (dense 1-D factor)."""
    import scipy.linalg as sl
    E = sl.expm(-t * T)
    return (E @ X @ E.T)
