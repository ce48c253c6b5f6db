"""Python mirror of PSFUN's Fortran API for the f(A)x path, over the C-ABI.

Names, argument meaning, defaults and `info` codes follow the reference:

  PsfunDKrylov      type(psfun_d_krylov)     krylov/psfun_d_krylov_mod.F90:42-60
  PsfunDSerial      type(psfun_d_serial)     serial/psfun_d_serial_mod.F90:43-61
  PsfunZQuadrature  type(psfun_z_quadrature) quadratures/psfun_z_quadrature_mod.F90:42-55
  hhtmethod1        quadratures/psfun_z_quadrules_mod.f90:40-85
  ellipkkp, ellipj, horner                   utils/psfun_utils_mod.f90:38-73
  psb_krylov        shifted CG generic       krylov/psfun_krylov_mod.f90:39-142

Where the Fortran routine returns through intent(out) arguments, the Python
method returns them (a result object carrying `info`).  Vectors may be numpy
arrays (host: copied in and out inside the call) or CUDA torch tensors
(device: used in place).  Every computation runs on the GPU; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi

SUCCESS = 0
ERR_INVALID_ARGS_COMBINATION = 111
ERR_INVALID_VECT_STATE = 1124
ERR_FROM_SUBROUTINE = 4010
ERR_FROM_SUBROUTINE_NON = 4011
ERR_INVALID_ISTOP = 5001
ERR_CUDA = 9001
ERR_DEVICE_TIMEOUT = 9002
ERR_INVALID_MATRIX = 9003


def _lib():
    return _capi.load()


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_capi.dp)


def _is_device(v) -> bool:
    return hasattr(v, "is_cuda") and bool(v.is_cuda)


def _sync_stream():
    """Run the library on torch's current stream when torch drives the device."""
    try:
        import torch
        if torch.cuda.is_available() and torch.cuda.is_initialized():
            _lib().psfun_gpu_set_stream(C.c_void_p(torch.cuda.current_stream().cuda_stream))
    except ImportError:
        pass


class PsfunError(RuntimeError):
    def __init__(self, info: int, where: str):
        super().__init__(f"{where}: info={info} ({_capi.last_error()})")
        self.info = info


# ---------------------------------------------------------------------------
class CsrMatrix:
    """Device CSR matrix: the local storage of a psb_dspmat_type (irp/ja/val).

    index_base = 1 accepts PSBLAS (Fortran) arrays unchanged.  Index arrays
    are validated and stored bit-exactly (int32)."""

    def __init__(self, irp, ja, val, index_base: int = 0, n: int | None = None):
        irp = np.ascontiguousarray(irp, dtype=np.int32)
        ja = np.ascontiguousarray(ja, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=np.float64)
        self.n = int(len(irp) - 1 if n is None else n)
        self.nnz = int(len(ja))
        h = C.c_void_p()
        info = _lib().psfun_gpu_csr_create(self.n, self.nnz, irp.ctypes.data_as(_capi.ip),
                                           ja.ctypes.data_as(_capi.ip), _dp(val), index_base, C.byref(h))
        if info != SUCCESS:
            raise PsfunError(info, "psfun_gpu_csr_create")
        self.handle = h
        nt = C.c_int64()
        ninf = C.c_double()
        _lib().psfun_gpu_csr_info(h, None, None, C.byref(nt), C.byref(ninf))
        self.ntiles = nt.value
        self.norm_inf = ninf.value

    @classmethod
    def from_scipy(cls, m):
        m = m.tocsr()
        m.sort_indices()
        return cls(m.indptr, m.indices, m.data)

    def is_symmetric(self) -> bool:
        """A == A^T entry by entry (checked once per handle on the host)."""
        v = C.c_int(0)
        info = _lib().psfun_gpu_csr_is_symmetric(self.handle, C.byref(v))
        if info != SUCCESS:
            raise PsfunError(info, "psfun_gpu_csr_is_symmetric")
        return bool(v.value)

    def spmv(self, x, alpha: float = 1.0, beta: float = 0.0, y=None):
        """y = alpha*A*x + beta*y (psb_spmm)."""
        if _is_device(x):
            import torch
            out = torch.zeros_like(x) if y is None else y
            _sync_stream()
            info = _lib().psfun_gpu_csr_spmv_device(self.handle, alpha, C.c_void_p(x.data_ptr()), beta,
                                                     C.c_void_p(out.data_ptr()))
        else:
            xx = np.ascontiguousarray(x, dtype=np.float64)
            out = np.zeros(self.n) if y is None else np.ascontiguousarray(y, dtype=np.float64).copy()
            info = _lib().psfun_gpu_csr_spmv(self.handle, alpha, _dp(xx), beta, _dp(out))
        if info != SUCCESS:
            raise PsfunError(info, "psfun_gpu_csr_spmv")
        return out

    def close(self):
        if getattr(self, "handle", None):
            _lib().psfun_gpu_csr_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
class PsfunDSerial:
    """type(psfun_d_serial): fname 'EXP', variant 'EXPOKIT', scaling 1,
    padedegree 6, phiorder 1 (serial/psfun_d_serial_mod.F90:44-48)."""

    def __init__(self):
        h = C.c_void_p()
        _lib().psfun_gpu_serial_create(C.byref(h))
        self.handle = h
        self._cb = None

    def set(self, what: str, val) -> int:
        """Generic set(what, val, info): string / real / integer / procedure."""
        L = _lib()
        w = what.encode()
        if isinstance(val, str):
            return L.psfun_gpu_serial_set_string(self.handle, w, val.encode())
        if isinstance(val, (bool, int, np.integer)):
            return L.psfun_gpu_serial_set_integer(self.handle, w, int(val))
        if isinstance(val, (float, np.floating)):
            return L.psfun_gpu_serial_set_real(self.handle, w, float(val))
        if callable(val):
            cb = _capi.USERF(lambda x, k: float(val(x, k)))
            info = L.psfun_gpu_serial_set_function(self.handle, w, cb)
            if info == SUCCESS:
                self._cb = cb
            return info
        return ERR_INVALID_ARGS_COMBINATION

    def get(self):
        fn = C.create_string_buffer(32)
        var = C.create_string_buffer(32)
        sc = C.c_double()
        pd = C.c_int()
        po = C.c_int()
        _lib().psfun_gpu_serial_get(self.handle, fn, var, C.byref(sc), C.byref(pd), C.byref(po))
        return dict(fname=fn.value.decode(), variant=var.value.decode(), scaling=sc.value, padedegree=pd.value,
                    phiorder=po.value)

    def apply(self, a, x):
        """y = f(scaling*a) x; a dense (n x n) array or a CsrMatrix.  Returns (y, info)."""
        xx = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros_like(xx)
        if isinstance(a, CsrMatrix):
            info = _lib().psfun_gpu_serial_apply_sparse(self.handle, a.handle, _dp(y), _dp(xx))
        else:
            aa = np.asfortranarray(a, dtype=np.float64)
            n = aa.shape[0]
            info = _lib().psfun_gpu_serial_apply(self.handle, n, _dp(aa), n, _dp(y), _dp(xx))
        return y, info

    def __del__(self):
        try:
            _lib().psfun_gpu_serial_destroy(self.handle)
        except Exception:
            pass


@dataclass
class KrylovResult:
    y: object
    info: int
    iter: int = 0
    err: float = 0.0
    res: np.ndarray = field(default_factory=lambda: np.zeros(0))


class PsfunDKrylov:
    """type(psfun_d_krylov): kname 'ARNOLDI', kmethd 'CG', tau 0, itmax 200,
    itrace 0, istopc 1, irst 10 (krylov/psfun_d_krylov_mod.F90:43-50)."""

    def __init__(self):
        h = C.c_void_p()
        _lib().psfun_gpu_krylov_create(C.byref(h))
        self.handle = h
        self.kname = "ARNOLDI"

    def set(self, what: str, val) -> int:
        """set(what, val): KNAME, KMETHD, PREC ('NONE' / 'DIAG') as strings;
        ITMAX, ITRACE, ISTOPC, IRST, KEEPLAST, BATCHMAP (the batched Lanczos'
        SpMM mapping, -1 = autotuned) as integers; TAU (the public component
        meth%tau of the reference) as a real."""
        if isinstance(val, str):
            info = _lib().psfun_gpu_krylov_set_string(self.handle, what.encode(), val.encode())
            if info == 0 and what.strip().upper() == "KNAME":
                self.kname = val
            return info
        if isinstance(val, (bool, int, np.integer)):
            return _lib().psfun_gpu_krylov_set_integer(self.handle, what.encode(), int(val))
        if isinstance(val, (float, np.floating)):
            return _lib().psfun_gpu_krylov_set_real(self.handle, what.encode(), float(val))
        return ERR_INVALID_ARGS_COMBINATION

    def precinit(self, ptype: str) -> int:
        """meth%precinit(ctxt, ptype, info) (psfun_d_prec_init,
        krylov/psfun_d_krylov_mod.F90:326-361): 'NOPREC'/'NONE', 'DIAG' or 'BJAC'
        (block Jacobi, ILU(0) on the diagonal blocks of 32 rows)."""
        return _lib().psfun_gpu_krylov_precinit(self.handle, ptype.encode())

    def precbuild(self, a: CsrMatrix) -> int:
        """meth%precbuild(a, desc_a, info) (psfun_d_prec_build, :363-403)."""
        return _lib().psfun_gpu_krylov_precbuild(self.handle, a.handle)

    def plot(self, fun: PsfunDSerial, iter: int, res, directory: str = ".") -> int:
        """meth%plot(fun, iter, res, info) (psfun_d_plot_info, :271-324): the
        residual history res(1:min(size(res), iter+1)) on a log scale, written
        to '<KNAME>-<FNAME>-<VARIANT>-Residual'.  The reference drives gnuplot
        to a PDF; this writes an SVG of the same plot with no external tool."""
        return plot_residual(self.kname, fun, iter, res, directory)

    def apply(self, fun: PsfunDSerial, a: CsrMatrix, x, eps: float, itmax: int | None = None,
              itrace: int | None = None, istop: int | None = None, y=None) -> KrylovResult:
        """kmethd%apply(fun,a,desc_a,y,x,eps,info,itmax,itrace,istop,iter,err,res)
        (psfun_d_parallel_apply, krylov/psfun_d_krylov_mod.F90:225-269)."""
        itmax_ = 200 if itmax is None else int(itmax)
        itrace_ = 0 if itrace is None else int(itrace)
        istop_ = 1 if istop is None else int(istop)
        it = C.c_int(0)
        err = C.c_double(0.0)
        cap = max(itmax_ + 2, 2)
        res = np.zeros(cap)
        nres = C.c_int(0)
        if _is_device(x):
            import torch
            out = torch.empty_like(x) if y is None else y
            _sync_stream()
            info = _lib().psfun_gpu_d_krylov_apply_device(
                self.handle, fun.handle, a.handle, C.c_void_p(out.data_ptr()), C.c_void_p(x.data_ptr()), eps,
                itmax_, itrace_, istop_, C.byref(it), C.byref(err), _dp(res), cap, C.byref(nres))
        else:
            xx = np.ascontiguousarray(x, dtype=np.float64)
            out = np.zeros_like(xx) if y is None else y
            info = _lib().psfun_gpu_d_krylov_apply(
                self.handle, fun.handle, a.handle, _dp(out), _dp(xx), eps, itmax_, itrace_, istop_, C.byref(it),
                C.byref(err), _dp(res), cap, C.byref(nres))
        return KrylovResult(out, info, it.value, err.value, res[: nres.value].copy())

    def __del__(self):
        try:
            _lib().psfun_gpu_krylov_destroy(self.handle)
        except Exception:
            pass


def plot_residual(kname: str, fun: PsfunDSerial, iter: int, res, directory: str = ".") -> int:
    """Residual history plot of psfun_d_plot_info (krylov/psfun_d_krylov_mod.F90:271-324):
    points (j, res(j)) for j = 1..indplot, indplot = size(res) if size(res) <= iter+1
    else iter+1 (:289-296), y on a log scale, lines with points, file and title
    '<kname>-<fname>-<variant>-Residual' (:300-304).  Written as SVG by hand
    (gnuplot is not a dependency); non-positive residuals are left out, as a
    log axis cannot show them.  Returns 0, or PSFUN_ERR_FROM_SUBROUTINE when
    the file cannot be written."""
    import math
    import os
    res = np.asarray(res, dtype=np.float64).ravel()
    n = res.size
    indplot = n if n <= iter + 1 else iter + 1
    st = fun.get()
    tag = f"{kname.strip()}-{st['fname'].strip()}-{st['variant'].strip()}"
    pts = [(j + 1, float(res[j])) for j in range(indplot) if res[j] > 0 and math.isfinite(res[j])]
    W, H, L, R, T, B = 640, 480, 80, 20, 40, 50
    if pts:
        lo = math.floor(math.log10(min(v for _, v in pts)))
        hi = math.ceil(math.log10(max(v for _, v in pts)))
    else:
        lo, hi = -16, 0
    hi = max(hi, lo + 1)
    xmax = max(indplot, 2)

    def px(j):
        return L + (W - L - R) * (j - 1) / (xmax - 1)

    def py(v):
        return T + (H - T - B) * (hi - math.log10(v)) / (hi - lo)

    out = [f'<svg xmlns="http://www.w3.org/2000/svg" width="{W}" height="{H}" font-family="sans-serif" font-size="12">',
           f'<text x="{W / 2}" y="20" text-anchor="middle" font-size="14">Residual history {tag}</text>',
           f'<rect x="{L}" y="{T}" width="{W - L - R}" height="{H - T - B}" fill="none" stroke="black"/>',
           f'<text x="{(W + L - R) / 2}" y="{H - 12}" text-anchor="middle">Iteration</text>',
           f'<text x="18" y="{(H + T - B) / 2}" text-anchor="middle" transform="rotate(-90 18 {(H + T - B) / 2})">'
           'Relative Residual</text>']
    step = max(1, (hi - lo) // 8)
    for e in range(lo, hi + 1, step):
        y = py(10.0 ** e)
        out.append(f'<line x1="{L - 4}" y1="{y:.1f}" x2="{L}" y2="{y:.1f}" stroke="black"/>'
                   f'<text x="{L - 8}" y="{y + 4:.1f}" text-anchor="end">10^{e}</text>')
    xstep = max(1, int(math.ceil((xmax - 1) / 10)))
    for j in range(1, xmax + 1, xstep):
        x = px(j)
        out.append(f'<line x1="{x:.1f}" y1="{H - B}" x2="{x:.1f}" y2="{H - B + 4}" stroke="black"/>'
                   f'<text x="{x:.1f}" y="{H - B + 18}" text-anchor="middle">{j}</text>')
    if pts:
        poly = " ".join(f"{px(j):.1f},{py(v):.1f}" for j, v in pts)
        out.append(f'<polyline points="{poly}" fill="none" stroke="#d62728"/>')
        out.extend(f'<circle cx="{px(j):.1f}" cy="{py(v):.1f}" r="3" fill="#d62728"/>' for j, v in pts)
    out.append("</svg>")
    try:
        with open(os.path.join(directory, tag + "-Residual.svg"), "w") as f:
            f.write("\n".join(out) + "\n")
    except OSError:
        return ERR_FROM_SUBROUTINE
    return 0


def krylov_batch(meth: "PsfunDKrylov", fun: "PsfunDSerial", items, eps: float, itmax: int = 200,
                 istop: int = 1):
    """Batched Lanczos f(t_k A_k) X_k for items [(CsrMatrix, X, Y, t_k), ...] in one
    persistent launch.  X, Y: CUDA float64 tensors of shape (nrhs, n) (column-major
    n x nrhs, the same nrhs for every item).  Returns (info, infos, iters, errs), the
    per-pair arrays shaped (count, nrhs)."""
    count = len(items)
    arr = (_capi.BatchItem * count)()
    R = int(items[0][1].shape[0])
    for k, (a, X, Y, t) in enumerate(items):
        if not (_is_device(X) and _is_device(Y)):
            raise TypeError("krylov_batch takes CUDA tensors")
        arr[k] = _capi.BatchItem(a.handle, int(X.shape[0]), X.data_ptr(), Y.data_ptr(), float(t))
    iters = np.zeros(count * R, dtype=np.int32)
    errs = np.zeros(count * R)
    infos = np.zeros(count * R, dtype=np.int32)
    _sync_stream()
    info = _lib().psfun_gpu_d_krylov_batch(meth.handle, fun.handle, count, arr, eps, int(itmax), int(istop),
                                           iters.ctypes.data_as(C.POINTER(C.c_int)), _dp(errs),
                                           infos.ctypes.data_as(C.POINTER(C.c_int)))
    return info, infos.reshape(count, R), iters.reshape(count, R), errs.reshape(count, R)


def quadrature_batch(items, eps: float = 1e-10, itmax: int = 2000):
    """The quadrature sum y = eta A Im(sum_j c_j (xi_j I + sign A)^{-1} x) for
    items [(CsrMatrix, X, Y, PsfunZQuadrature), ...] in one persistent launch
    (the quadrature's own poles xi, weights c, eta and sign per item).  X, Y:
    CUDA float64 tensors of shape (nrhs, n), the same nrhs for every item.
    Returns (info, infos, iters, errs) with the per-pair arrays shaped
    (count, nrhs)."""
    count = len(items)
    arr = (_capi.QuadItem * count)()
    keep = []
    R = int(items[0][1].shape[0])
    for k, (a, X, Y, q) in enumerate(items):
        if not (_is_device(X) and _is_device(Y)):
            raise TypeError("quadrature_batch takes CUDA tensors")
        N = len(q.xi)
        xi = np.empty(2 * N)
        xi[0::2], xi[1::2] = np.real(q.xi), np.imag(q.xi)
        cw = np.empty(2 * N)
        cw[0::2], cw[1::2] = np.real(q.c), np.imag(q.c)
        keep += [xi, cw]
        arr[k] = _capi.QuadItem(a.handle, int(X.shape[0]), X.data_ptr(), Y.data_ptr(), N, xi.ctypes.data,
                                cw.ctypes.data, float(q.eta), float(q.sign))
    iters = np.zeros(count * R, dtype=np.int32)
    errs = np.zeros(count * R)
    infos = np.zeros(count * R, dtype=np.int32)
    _sync_stream()
    info = _lib().psfun_gpu_z_quadrature_batch(count, arr, float(eps), int(itmax),
                                               iters.ctypes.data_as(C.POINTER(C.c_int)), _dp(errs),
                                               infos.ctypes.data_as(C.POINTER(C.c_int)))
    return info, infos.reshape(count, R), iters.reshape(count, R), errs.reshape(count, R)


def talbot_rule(N: int = 32):
    """Nodes z_k and weights c_k (N/2 of each) of the optimized Talbot rule:
    exp(M) b ~ Re sum_k c_k (z_k I - M)^{-1} b."""
    z = np.zeros(N)
    c = np.zeros(N)
    info = _lib().psfun_gpu_talbot_rule(int(N), _dp(z), _dp(c))
    if info != SUCCESS:
        raise PsfunError(info, "psfun_gpu_talbot_rule")
    return z[0::2] + 1j * z[1::2], c[0::2] + 1j * c[1::2]


def expm_adjoint(a: CsrMatrix, t: float, x, g=None, nquad: int = 32, eps: float = 1e-15, itmax: int = 300,
                 recompute: bool = False, want=("y", "grad_x", "grad_t", "grad_vals")):
    """y = exp(tA) x and, given g = dL/dy, the gradients dL/dx = exp(tA^T) g,
    dL/dt = g^T A y and dL/dA on the CSR pattern of A (one value per stored
    entry).  Symmetric A: two Lanczos bases and the nquad-point Talbot rule;
    nonsymmetric A: Arnoldi on A and A^T and Van Loan's block exponential.
    x, g: CUDA float64 tensors.  Returns a dict of CUDA tensors / floats."""
    import torch
    out = {}
    y = torch.empty_like(x) if "y" in want else None
    gx = torch.empty_like(x) if (g is not None and "grad_x" in want) else None
    gv = torch.empty(a.nnz, dtype=torch.float64, device=x.device) if (g is not None and "grad_vals" in want) else None
    gt = C.c_double(0.0)
    it = (C.c_int * 2)()
    gg = g if g is not None else x
    _sync_stream()
    info = _lib().psfun_gpu_d_expm_adjoint_device(
        a.handle, float(t), C.c_void_p(x.data_ptr()), C.c_void_p(gg.data_ptr()), int(nquad), float(eps), int(itmax),
        1 if recompute else 0, C.c_void_p(y.data_ptr()) if y is not None else None,
        C.c_void_p(gx.data_ptr()) if gx is not None else None,
        C.byref(gt) if (g is not None and "grad_t" in want) else None,
        C.c_void_p(gv.data_ptr()) if gv is not None else None, it)
    if info != SUCCESS:
        raise PsfunError(info, "psfun_gpu_d_expm_adjoint_device")
    out.update(y=y, grad_x=gx, grad_t=gt.value if g is not None else None, grad_vals=gv, iters=(it[0], it[1]))
    return out


# ---------------------------------------------------------------------------
def psb_krylov(method: str, a: CsrMatrix, prec: str, b, eta: float, zeta: float, x, eps: float,
               itmax: int = 1000, istop: int = 2, itrace: int = 0, cond: bool = False):
    """psb_krylov(method,a,prec,b,eta,zeta,x,eps,desc_a,info,itmax,iter,err,itrace,istop,cond)
    for (eta A + zeta I) x = b (psfun_dkrylov_vect).  prec is 'NONE', 'DIAG' or 'BJAC'.
    x is the initial guess.  Returns (x, info, iter, err), and cond as a fifth
    element when cond=True (the reference's optional condition estimate)."""
    it = C.c_int(0)
    err = C.c_double(0.0)
    cv = C.c_double(0.0)
    pc = C.byref(cv) if cond else None
    if _is_device(b):
        _sync_stream()
        info = _lib().psfun_gpu_dcg_ex_device(method.encode(), a.handle, prec.encode(), C.c_void_p(b.data_ptr()),
                                              eta, zeta, C.c_void_p(x.data_ptr()), eps, itmax, itrace, istop,
                                              C.byref(it), C.byref(err), pc)
        out = x
    else:
        bb = np.ascontiguousarray(b, dtype=np.float64)
        out = np.ascontiguousarray(x, dtype=np.float64).copy()
        info = _lib().psfun_gpu_dcg_ex(method.encode(), a.handle, prec.encode(), _dp(bb), eta, zeta, _dp(out), eps,
                                       itmax, itrace, istop, C.byref(it), C.byref(err), pc)
    if cond:
        return out, info, it.value, err.value, cv.value
    return out, info, it.value, err.value


# ---------------------------------------------------------------------------
def horner(coeffs, x: float) -> float:
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    return float(_lib().psfun_gpu_horner(_dp(c), len(c), float(x)))


def ellipkkp(L: float) -> np.ndarray:
    K = np.zeros(2)
    _lib().psfun_gpu_ellipkkp(float(L), _dp(K))
    return K


def ellipj(u, L: float):
    """Real or complex Jacobi sn, cn, dn at parameter m = exp(-2 pi L)."""
    if isinstance(u, complex) or np.iscomplexobj(u):
        uu = np.array([complex(u).real, complex(u).imag])
        sn, cn, dn = np.zeros(2), np.zeros(2), np.zeros(2)
        _lib().psfun_gpu_z_ellipj(_dp(uu), float(L), _dp(sn), _dp(cn), _dp(dn))
        return complex(*sn), complex(*cn), complex(*dn)
    sn, cn, dn = C.c_double(), C.c_double(), C.c_double()
    _lib().psfun_gpu_d_ellipj(float(u), float(L), C.byref(sn), C.byref(cn), C.byref(dn))
    return sn.value, cn.value, dn.value


def hhtmethod1(zfun, N: int, rparams):
    """Method 1 of Hale-Higham-Trefethen: returns (xi, c, eta, sign, info)."""

    @_capi.ZFUN
    def cb(z, res, ctx):
        v = complex(zfun(complex(z[0], z[1])))
        res[0] = v.real
        res[1] = v.imag

    rp = np.ascontiguousarray(rparams, dtype=np.float64)
    xi = np.zeros(2 * N)
    c = np.zeros(2 * N)
    eta = C.c_double()
    sign = C.c_double()
    info = _lib().psfun_gpu_hhtmethod1(cb, None, int(N), _dp(rp), _dp(xi), _dp(c), C.byref(eta), C.byref(sign))
    return xi[0::2] + 1j * xi[1::2], c[0::2] + 1j * c[1::2], eta.value, sign.value, info


class PsfunZQuadrature:
    """type(psfun_z_quadrature): poles xi, weights c, eta, sign, matrix, prec.
    apply() forms y = eta * A * Im(sum_j c_j (xi_j I + sign A)^{-1} x) on the
    GPU with one shared Lanczos basis (the reference stores these fields but
    has no routine that forms the sum)."""

    def __init__(self):
        self.xi = None
        self.c = None
        self.eta = 0.0
        self.sign = 0.0
        self.a = None
        self.prec = None

    def computepoles(self, quadformula, zfun, N: int, cparams=None, rparams=None) -> int:
        """psfun_z_computepoles (quadratures/psfun_z_quadrature_mod.F90:114-142)."""
        if rparams is None:
            return ERR_INVALID_ARGS_COMBINATION
        xi, c, eta, sign, info = quadformula(zfun, N, rparams)
        if info == SUCCESS:
            self.xi, self.c, self.eta, self.sign = xi, c, eta, sign
        return info

    def setmatrix(self, a: CsrMatrix):
        self.a = a

    def setpreconditioner(self, prec):
        self.prec = prec

    def set(self, obj):
        if isinstance(obj, CsrMatrix):
            self.setmatrix(obj)
        else:
            self.setpreconditioner(obj)

    def apply(self, x, eps: float = 1e-10, itmax: int = 2000, y=None):
        """Returns (y, info, iter, err); err is the largest relative shifted residual."""
        if self.a is None or self.xi is None:
            return None, ERR_INVALID_ARGS_COMBINATION, 0, 0.0
        N = len(self.xi)
        xi = np.empty(2 * N)
        xi[0::2], xi[1::2] = np.real(self.xi), np.imag(self.xi)
        cw = np.empty(2 * N)
        cw[0::2], cw[1::2] = np.real(self.c), np.imag(self.c)
        it = C.c_int(0)
        err = C.c_double(0.0)
        if _is_device(x):
            import torch
            out = torch.empty_like(x) if y is None else y
            _sync_stream()
            info = _lib().psfun_gpu_z_quadrature_apply_device(self.a.handle, N, _dp(xi), _dp(cw), self.eta,
                                                              self.sign, C.c_void_p(x.data_ptr()),
                                                              C.c_void_p(out.data_ptr()), eps, itmax, C.byref(it),
                                                              C.byref(err))
        else:
            xx = np.ascontiguousarray(x, dtype=np.float64)
            out = np.zeros_like(xx)
            info = _lib().psfun_gpu_z_quadrature_apply(self.a.handle, N, _dp(xi), _dp(cw), self.eta, self.sign,
                                                       _dp(xx), _dp(out), eps, itmax, C.byref(it), C.byref(err))
        return out, info, it.value, err.value
