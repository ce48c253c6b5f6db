"""Dense f(H) on the device (psfun_d_serial%apply) against the oracle."""
from pathlib import Path

import numpy as np
import pytest

from psfun_gb300 import matrices

pytestmark = pytest.mark.gpu
FIX = np.load(Path(__file__).parent / "golden" / "driver_scenarios.npz")


def mk(fname, variant, scaling, k=1, f=None):
    import psfun_gb300 as pg
    s = pg.PsfunDSerial()
    s.set("FNAME", fname); s.set("VARIANT", variant); s.set("SCALING", float(scaling)); s.set("PHIORDER", k)
    if f is not None:
        s.set("FPOINTER", f)
    return s


@pytest.mark.parametrize("fname,variant,k", [("EXP", "GENPADE", 1), ("EXP", "CHBHES", 1), ("EXP", "CHBGEN", 1),
                                             ("EXP", "CHBSYM", 1), ("EXP", "SASQ", 1), ("EXP", "TAYLOR", 1),
                                             ("PHI", "", 1), ("PHI", "", 3)])
@pytest.mark.parametrize("m", [1, 5, 33, 80])
def test_serial_vs_oracle(lib, orc, fname, variant, k, m):
    rng = np.random.default_rng(m)
    B = rng.standard_normal((m, m))
    H = -(B @ B.T / m + np.eye(m))
    if variant == "CHBHES":
        H = np.triu(H, -1)
    x = rng.standard_normal(m)
    y, info = mk(fname, variant, 0.6, k).apply(H, x)
    yo, io = orc.serial_apply(orc.serial(fname, variant, 0.6, phiorder=k), H, x)
    assert info == 0 and io == 0
    assert np.linalg.norm(y - yo) <= 1e-11 * np.linalg.norm(yo)


def test_serial_errors(lib):
    y, info = mk("EXP", "EXPOKIT", 1.0).apply(np.eye(4), np.ones(4))
    assert info == 4010
    y, info = mk("LOG", "GENPADE", 1.0).apply(np.eye(4), np.ones(4))
    assert info == 4010


def test_serialtest_scenario_sparse(lib):
    """serialtest.f90:106 (apply on the sparse laplacian.mtx, exp(A) 1)."""
    import psfun_gb300 as pg
    T = -matrices.laplacian_1d(50)
    y, info = mk("EXP", "GENPADE", 1.0).apply(pg.CsrMatrix.from_scipy(T), np.ones(50))
    assert info == 0
    assert np.linalg.norm(y - FIX["serial_y"]) <= 1e-12 * np.linalg.norm(FIX["serial_y"])


def test_userf_serial(lib, orc):
    H = -np.diag(np.arange(1.0, 9.0)) + 0.1 * np.ones((8, 8))
    f = lambda v, k: float(np.cos(v))
    y, info = mk("USERF", "SYM", 0.7, f=f).apply(H, np.ones(8))
    yo, io = orc.serial_apply(orc.serial("USERF", "SYM", 0.7, f=f), H, np.ones(8))
    assert info == 0 and io == 0 and np.linalg.norm(y - yo) <= 1e-12 * np.linalg.norm(yo)
