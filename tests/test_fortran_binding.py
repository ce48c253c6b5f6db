"""The Fortran side of the boundary (psfun_gb300/fortran) against the C header,
on the CPU.  No Fortran compiler is available, so the ISO_C_BINDING interface
module is checked by reading it: every entry point of include/psfun_gb300.h has
a bind(C) interface with the same name, the same number of arguments and
argument-by-argument compatible types (value scalars, arrays, handles,
strings, function pointers), the bind(C) psfun_batch_item and psfun_quad_item
match the header's structs field by field, and the shim calls only bound
entry points."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "psfun_gb300.h"
CABI = ROOT / "psfun_gb300" / "fortran" / "psfun_gb300_cabi.f90"
SHIM = ROOT / "psfun_gb300" / "fortran" / "psfun_gb300_shim.F90"

HANDLES = {"psfun_csr", "psfun_serial", "psfun_krylov", "void"}


def c_prototypes():
    src = HEADER.read_text()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"^\s*#.*$", " ", src, flags=re.M)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(psfun_gpu_\w+)\s*\(([^;{]*?)\)\s*;", src):
        ret, name, args = " ".join(m.group(1).split()), m.group(2), " ".join(m.group(3).split())
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret, params)
    return out


def c_class(param: str) -> str:
    """Class of a C parameter: 'int', 'double', 'ptr' (a handle or any other
    single pointer that a Fortran caller passes as c_ptr), 'ptrptr', 'funptr',
    or a normalised pointer type such as 'const double*'."""
    p = param.replace("*", " * ")
    toks = p.split()[:-1]  # drop the parameter name
    stars = toks.count("*")
    base = [t for t in toks if t != "*"]
    const = "const" in base
    base = [t for t in base if t != "const"]
    tname = " ".join(base)
    if tname in ("psfun_userf", "psfun_zfun"):
        return "funptr"
    if stars == 2:
        return "ptrptr"
    if stars == 0:
        return tname
    if tname in HANDLES:
        return "ptr"
    return ("const " if const else "") + tname + "*"


FTYPE = {
    "integer(c_int)": "int", "integer(c_int64_t)": "int64_t", "integer(c_int32_t)": "int32_t",
    "integer(c_long_long)": "long long", "real(c_double)": "double", "complex(c_double_complex)": "double",
    "character(kind=c_char)": "char", "type(psfun_batch_item)": "psfun_batch_item",
    "type(psfun_quad_item)": "psfun_quad_item",
}


def f_interfaces():
    src = CABI.read_text()
    src = re.sub(r"!.*$", "", src, flags=re.M)
    src = re.sub(r"&\s*\n\s*", " ", src)
    out = {}
    for m in re.finditer(r"^[ \t]*([^\n]+?)[ \t]+function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end function",
                         src, flags=re.S | re.M):
        ret, fname, args, cname, body = m.group(1).strip(), m.group(2), m.group(3), m.group(4), m.group(5)
        assert fname == cname, (fname, cname)
        names = [a.strip() for a in args.split(",") if a.strip()]
        decl = {}
        for line in body.splitlines():
            if "::" not in line:
                continue
            spec, vars_ = line.split("::")
            spec = spec.strip()
            parts = [p.strip() for p in re.split(r",(?![^(]*\))", spec)]
            ftype, attrs = parts[0], set(parts[1:])
            for v in re.split(r",(?![^(]*\))", vars_):
                v = v.strip()
                if v:
                    arr = v.endswith("(*)")
                    decl[v.replace("(*)", "").strip()] = (ftype, attrs, arr)
        out[cname] = (ret, [(n,) + decl[n] for n in names])
    return out


def f_class(ftype: str, attrs: set, arr: bool) -> str:
    if ftype == "type(c_ptr)":
        return "ptr" if "value" in attrs else "ptrptr"
    if ftype == "type(c_funptr)":
        assert "value" in attrs
        return "funptr"
    base = FTYPE[ftype]
    if "value" in attrs:
        assert not arr
        return base
    const = "intent(in)" in attrs
    return ("const " if const else "") + base + "*"


def compatible(cc: str, fc: str) -> bool:
    if cc == fc:
        return True
    if fc == "ptr" and (cc == "ptr" or cc.endswith("*")):
        return True  # a device pointer or an optional host scalar passed as c_ptr
    return False


def test_every_entry_point_is_bound_with_matching_arguments():
    cp = c_prototypes()
    fi = f_interfaces()
    assert len(cp) >= 45
    assert set(cp) == set(fi), (sorted(set(cp) - set(fi)), sorted(set(fi) - set(cp)))
    for name, (cret, cparams) in cp.items():
        fret, fparams = fi[name]
        assert len(cparams) == len(fparams), (name, cparams, fparams)
        for cpar, (fname, ftype, attrs, arr) in zip(cparams, fparams):
            cc, fc = c_class(cpar), f_class(ftype, attrs, arr)
            assert compatible(cc, fc), (name, cpar, fname, ftype, attrs, cc, fc)
        want = {"int": "integer(c_int)", "double": "real(c_double)", "long long": "integer(c_long_long)",
                "const char*": "type(c_ptr)", "void*": "type(c_ptr)"}[cret]
        assert fret == want, (name, cret, fret)


def struct_fields(name):
    hdr = re.search(r"typedef struct \{([^{}]*)\} " + name + ";", HEADER.read_text()).group(1)
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    cfields = [f.split()[-1].lstrip("*") for f in hdr.split(";") if f.strip()]
    body = re.search(r"type, bind\(C\) :: " + name + r"\n(.*?)end type", CABI.read_text(), flags=re.S).group(1)
    ffields = [line.split("::")[1].strip() for line in body.splitlines() if "::" in line]
    return cfields, ffields


def test_batch_item_layout():
    cfields, ffields = struct_fields("psfun_batch_item")
    assert cfields == ffields == ["a", "nrhs", "x", "y", "scaling"]
    cfields, ffields = struct_fields("psfun_quad_item")
    assert [f.lower() for f in cfields] == [f.lower() for f in ffields] == ["a", "nrhs", "x", "y", "n", "xi", "c",
                                                                           "eta", "sign"]


def test_shim_calls_only_bound_entry_points():
    fi = f_interfaces()
    called = set(re.findall(r"\b(psfun_gpu_\w+)\s*\(", re.sub(r"!.*$", "", SHIM.read_text(), flags=re.M)))
    assert called and called <= set(fi), sorted(called - set(fi))
    # the drop-in keeps the reference routine's argument list after the method name
    sig = re.search(r"subroutine psfun_gb300_krylov_apply\(([^)]*)\)", SHIM.read_text()).group(1)
    assert [a.strip() for a in sig.split(",")] == ["kname", "fun", "a", "desc_a", "y", "x", "eps", "info", "itmax",
                                                   "itrace", "istop", "iter", "err", "res"]
