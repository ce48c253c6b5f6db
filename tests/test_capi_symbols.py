"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares."""
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        src = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(psfun_gpu_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_all_declared_symbols_exported(lib):
    names = declared_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_prototypes_cover_header(lib):
    from psfun_gb300 import _capi
    missing = [n for n in declared_symbols() if n not in _capi.PROTOS]
    assert not missing, missing


def test_version_string(lib):
    assert b"sm_103a" in lib.psfun_gpu_version()


def test_setters_without_gpu(lib):
    """Handle set-up and the reference's set() semantics are host logic."""
    import psfun_gb300 as pg
    f = pg.PsfunDSerial()
    assert f.get()["fname"] == "EXP" and f.get()["variant"] == "EXPOKIT" and f.get()["padedegree"] == 6
    assert f.set("fname", "PHI") == 0 and f.get()["fname"] == "PHI"
    assert f.set("scaling", -0.5) == 0 and f.get()["scaling"] == -0.5
    assert f.set("Pade_Degree", 8) == 0 and f.get()["padedegree"] == 8
    assert f.set("NOPE", "x") == 111 and f.set("SCALING", 1) == 111
    k = pg.PsfunDKrylov()
    assert k.set("kname", "LANCZOS") == 0 and k.set("itmax", 10) == 0 and k.set("BAD", 1) == 111
    assert k.set("ITMAX", "x") == 111
    # the batched Lanczos' SpMM mapping: -1 (autotuned) or 0..2
    assert all(k.set("BATCHMAP", v) == 0 for v in (-1, 0, 1, 2))
    assert k.set("BATCHMAP", 3) == 111 and k.set("batchmap", -2) == 111


def test_precinit_types_without_gpu(lib):
    """precinit (psfun_d_prec_init) accepts the preconditioners that exist here
    and reports the AMG4PSBLAS-only types as a failed subroutine."""
    import psfun_gb300 as pg
    k = pg.PsfunDKrylov()
    assert k.precinit("NOPREC") == 0 and k.precinit("diag") == 0 and k.precinit("NONE") == 0
    assert k.precinit("bjac") == 0
    assert k.precinit("ML") == pg.api.ERR_FROM_SUBROUTINE
    assert b"ML" in lib.psfun_gpu_last_error()


def test_plot_residual_history(lib, tmp_path):
    """plot (psfun_d_plot_info): min(size(res), iter+1) points, file named
    <kname>-<fname>-<variant>-Residual, log axis skipping non-positive values."""
    import psfun_gb300 as pg
    f = pg.PsfunDSerial()
    assert f.set("VARIANT", "GENPADE") == 0
    k = pg.PsfunDKrylov()
    assert k.set("KNAME", "Lanczos") == 0
    res = np.array([1.0, 1e-3, 1e-6, 0.0, 1e-9, 5.0])
    assert k.plot(f, 4, res, directory=str(tmp_path)) == 0
    svg = (tmp_path / "Lanczos-EXP-GENPADE-Residual.svg").read_text()
    assert "Residual history Lanczos-EXP-GENPADE" in svg
    # iter = 4: the first 5 entries, of which the zero is left out
    assert svg.count("<circle") == 4
    assert k.plot(f, 10, res, directory=str(tmp_path)) == 0
    assert (tmp_path / "Lanczos-EXP-GENPADE-Residual.svg").read_text().count("<circle") == 5
    assert k.plot(f, 1, res, directory=str(tmp_path / "missing")) == pg.api.ERR_FROM_SUBROUTINE


def test_missing_library_raises(tmp_path):
    """No fallback: a missing library is an error (fresh interpreter, since the
    loader caches the library it opened)."""
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, sys.argv[1])\n"
            "from psfun_gb300 import _capi\n"
            "try:\n    _capi.load(sys.argv[2])\nexcept RuntimeError as e:\n    print('raised:', e)\n")
    r = subprocess.run([sys.executable, "-c", code, str(ROOT), str(tmp_path / "absent.so")], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "raised:" in r.stdout and "no CPU fallback" in r.stdout
