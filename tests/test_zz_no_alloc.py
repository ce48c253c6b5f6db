"""psfun_gpu_serial_apply_device_static (static device scratch, no allocation)
against psfun_gpu_serial_apply on the same inputs, for consecutive calls that
share the scratch array.  Collected last so that it also runs after every
other test in the same process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-11  # the dense f(H)x tolerance of the serial parity tests


def mk(fname, variant, scaling, k=1):
    import psfun_gb300 as pg
    s = pg.PsfunDSerial()
    s.set("FNAME", fname); s.set("VARIANT", variant); s.set("SCALING", float(scaling)); s.set("PHIORDER", k)
    return s


def case(m, seed):
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((m, m))
    return -(B @ B.T / m + np.eye(m)), rng.standard_normal(m)


def static_apply(lib, fun, H, x):
    import torch
    m = H.shape[0]
    # column-major a with lda = m + 3 (a padded leading dimension)
    lda = m + 3
    a = torch.zeros((m, lda), dtype=torch.float64, device="cuda")
    a[:, :m] = torch.from_numpy(np.ascontiguousarray(H.T)).cuda()
    xd = torch.from_numpy(x).cuda()
    yd = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = lib.psfun_gpu_serial_apply_device_static(fun.handle, m, C.c_void_p(a.data_ptr()), lda,
                                                  C.c_void_p(yd.data_ptr()), C.c_void_p(xd.data_ptr()))
    return rc, yd.cpu().numpy()


def test_static_scratch_matches_allocating_entry_point(lib):
    calls = [("EXP", "GENPADE", 0.6, 1, 48, 1), ("PHI", "", 0.6, 3, 20, 2), ("EXP", "CHBGEN", 0.6, 1, 64, 3),
             ("EXP", "GENPADE", 0.6, 1, 48, 1)]
    prev = None
    for fname, variant, sc, k, m, seed in calls:
        fun = mk(fname, variant, sc, k)
        H, x = case(m, seed)
        ref, info = fun.apply(H, x)
        assert info == 0
        rc, y = static_apply(lib, fun, H, x)
        assert rc == 0, lib.psfun_gpu_last_error()
        assert np.linalg.norm(y - ref) <= RTOL * np.linalg.norm(ref), (fname, variant, m)
        if seed == 1 and prev is not None:
            # the repeated first call, after the array held other contents
            assert np.array_equal(y, prev)
        if seed == 1:
            prev = y


def test_static_scratch_rejects_oversize(lib):
    import torch
    fun = mk("EXP", "GENPADE", 0.5)
    m = 65
    buf = torch.zeros(m * m + 2 * m, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    rc = lib.psfun_gpu_serial_apply_device_static(fun.handle, m, C.c_void_p(p), m, C.c_void_p(p + 8 * m * m),
                                                  C.c_void_p(p + 8 * (m * m + m)))
    assert rc == 111
    assert b"static scratch" in lib.psfun_gpu_last_error()


def test_static_scratch_limits_follow_the_function(lib):
    """PHIORDER limits PHI only: an EXP call at n = 64 whose handle still holds
    a large PHIORDER runs; PHI with phiorder 9 and USERF are refused."""
    import torch
    H, x = case(64, 4)
    fun = mk("EXP", "GENPADE", 0.6, 20)
    ref, info = fun.apply(H, x)
    assert info == 0
    rc, y = static_apply(lib, fun, H, x)
    assert rc == 0, lib.psfun_gpu_last_error()
    assert np.linalg.norm(y - ref) <= RTOL * np.linalg.norm(ref)
    H, x = case(16, 5)
    rc, _ = static_apply(lib, mk("PHI", "", 0.6, 9), H, x)
    assert rc == 111 and b"phiorder" in lib.psfun_gpu_last_error()
    fu = mk("USERF", "SYM", 0.6)
    assert fu.set("FPOINTER", lambda v, k: np.exp(v)) == 0
    rc, _ = static_apply(lib, fu, H, x)
    assert rc == 111 and b"USERF" in lib.psfun_gpu_last_error()
    torch.cuda.synchronize()
