"""The C-ABI from plain C: include/psfun_gb300.h compiles as C11 and as
C++17, and a C program links libpsfun_gb300.so and uses its host entry points
(version string, serial handle set-up with the reference's set() semantics,
the utiltest control value of the Horner routine) without a GPU and without
Python or torch in the process.  CPU only."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
INC = ROOT / "include"
LIBDIR = ROOT / "psfun_gb300" / "lib"

PROG = r"""
#include <stdio.h>
#include <string.h>
#include "psfun_gb300.h"
int main(void) {
  const char* v = psfun_gpu_version();
  if (!v || !strstr(v, "sm_103a")) return 10;
  psfun_serial* f = NULL;
  if (psfun_gpu_serial_create(&f) != 0 || !f) return 11;
  if (psfun_gpu_serial_set_string(f, "fname", "PHI") != 0) return 12;
  if (psfun_gpu_serial_set_integer(f, "PHIORDER", 2) != 0) return 13;
  if (psfun_gpu_serial_set_real(f, "SCALING", -0.5) != 0) return 14;
  if (psfun_gpu_serial_set_string(f, "NOPE", "x") != 111) return 15;
  if (psfun_gpu_serial_destroy(f) != 0) return 16;
  /* utiltest.f90's control: Horner on (132, 42, 14, 5, 2, 1, 0) at 1 is 196 */
  const double c[7] = {132.0, 42.0, 14.0, 5.0, 2.0, 1.0, 0.0};
  if (psfun_gpu_horner(c, 7, 1.0) != 196.0) return 17;
  printf("ok %s\n", v);
  return 0;
}
"""


def _cc():
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    return cc


def test_header_compiles_as_c_and_cxx(tmp_path):
    src = tmp_path / "h.c"
    src.write_text('#include "psfun_gb300.h"\nint main(void) { return 0; }\n')
    cc = _cc()
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-I", str(INC), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx:
        r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-fsyntax-only", "-x", "c++", "-I", str(INC),
                            str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_c_program_links_and_runs(lib, tmp_path):
    src = tmp_path / "prog.c"
    src.write_text(PROG)
    exe = tmp_path / "prog"
    r = subprocess.run([_cc(), "-std=c11", "-Wall", "-Werror", "-I", str(INC), str(src), "-o", str(exe),
                        "-L", str(LIBDIR), "-lpsfun_gb300", f"-Wl,-rpath,{LIBDIR}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    assert r.stdout.startswith("ok ")
