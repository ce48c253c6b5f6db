"""Without a CUDA device the library has no fallback: a compute call returns
a PSBLAS-style error code with the CUDA error in psfun_gpu_last_error, and
creating a device matrix raises.  Runs only where no GPU is present."""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import has_gpu

pytestmark = pytest.mark.skipif(has_gpu(), reason="checks the behaviour without a CUDA device")


def test_serial_apply_reports_cuda_error(lib):
    import psfun_gb300 as pg
    f = pg.PsfunDSerial()
    assert f.set("VARIANT", "GENPADE") == 0
    y, info = f.apply(-np.eye(3), np.ones(3))
    assert info != 0
    assert b"cuda" in lib.psfun_gpu_last_error().lower()


def test_csr_create_raises(lib):
    import psfun_gb300 as pg
    with pytest.raises(pg.api.PsfunError) as e:
        pg.CsrMatrix.from_scipy(sp.identity(4, format="csr"))
    assert e.value.args and "psfun_gpu_csr_create" in str(e.value)
