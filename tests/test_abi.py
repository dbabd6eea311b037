"""CPU tests of the C-ABI boundary: the library loads, exports every function declared in
include/gturbo.h, its structs have the layout of the header, and the host-only entry points
behave like the reference (no GPU work is launched here)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from gturbo_gb300 import _lib, build
from gturbo_gb300.params import GtInfo, GtParams, Params
from oracle.coracle import rann

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_library_exports_every_header_function(lib):
    names = _lib.header_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    for n in names:
        assert hasattr(lib, n)


def _c_layout(struct, fields):
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "gturbo.h"', "int main(void){",
           f'printf("%zu\\n", sizeof({struct}));']
    src += [f'printf("%zu\\n", offsetof({struct}, {f}));' for f in fields]
    src.append("return 0;}")
    tmp = os.path.join(build.BUILD, f"layout_{struct}")
    os.makedirs(build.BUILD, exist_ok=True)
    with open(tmp + ".c", "w") as f:
        f.write("\n".join(src))
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), tmp + ".c", "-o", tmp], check=True)
    vals = [int(x) for x in subprocess.run([tmp], capture_output=True, text=True, check=True).stdout.split()]
    return vals[0], vals[1:]


@pytest.mark.parametrize("ctype,cname", [(GtParams, "gt_params"), (GtInfo, "gt_info")])
def test_struct_layout_matches_header(ctype, cname):
    fields = [f for f, _ in ctype._fields_]
    size, offs = _c_layout(cname, fields)
    assert size == ctypes.sizeof(ctype)
    assert offs == [getattr(ctype, f).offset for f in fields]


def test_fortran_module_matches_header():
    """include/gturbo_c.f90 (the bind(C) module for the Fortran driver; no Fortran compiler
    here): every bound name is declared in gturbo.h with the same number of arguments, and its
    gt_params type lists the C struct's fields in order with matching kinds."""
    import re
    text = open(os.path.join(ROOT, "include", "gturbo_c.f90")).read()
    header = open(_lib.HEADER).read()
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    binds = re.findall(r"function\s+(\w+)\s*\(([^)]*)\)\s*&?\s*bind\(C, name=\"(\w+)\"\)", text)
    assert len(binds) >= 19
    for fname, args, cname in binds:
        assert fname == cname
        m = re.search(r"\b%s\s*\(([^)]*)\)" % cname, header)
        assert m, cname
        n_c = len([a for a in m.group(1).split(",") if a.strip()])
        n_f = len([a for a in args.split(",") if a.strip()])
        assert n_c == n_f, (cname, n_c, n_f)
    ftype = re.search(r"type, bind\(C\) :: gt_params(.*?)end type", text, re.S).group(1)
    fields = []
    for line in ftype.strip().splitlines():
        kind, names = line.split("::")
        fields += [(kind.strip(), n.strip()) for n in names.split(",")]
    assert [n for _, n in fields] == [f for f, _ in GtParams._fields_]
    for (kind, name), (_, ct) in zip(fields, GtParams._fields_):
        assert ("c_int32_t" in kind) == (ct is ctypes.c_int32), name
        assert ("c_double" in kind) == (ct is ctypes.c_double), name


def test_gt_rann_is_the_reference_lcg(lib):
    s = ctypes.c_int32(481929)
    got = np.array([lib.gt_rann(ctypes.byref(s)) for _ in range(500)], np.float32)
    ref, last = rann(481929, 500)
    assert np.array_equal(got, ref) and s.value == last


def test_create_rejects_bad_grid_size(lib):
    h = ctypes.c_void_p()
    cp = Params(n=100).to_ctypes()
    assert lib.gt_create(ctypes.byref(cp), ctypes.byref(h)) == 1
    assert b"power of two" in lib.gt_last_error(None)


def test_create_rejects_bad_non_square_grids(lib):
    """A non-square grid has NX, NY >= 32 and NY <= 4096 (the column variants with the column
    count at run time stop at 4096); every side a power of two."""
    h = ctypes.c_void_p()
    for n, ny in ((64, 16), (16, 64), (64, 8192), (64, 48), (64, -2)):
        cp = Params(n=n, ny=ny).to_ctypes()
        assert lib.gt_create(ctypes.byref(cp), ctypes.byref(h)) == 1, (n, ny)
        assert b"power of two" in lib.gt_last_error(None)


def test_params_struct_carries_ny():
    assert Params(n=64, ny=32).field_shape == (32, 66)
    assert Params(n=64).field_shape == (66 - 2, 66) and Params(n=64).rows == 64
    assert Params(n=256, ny=1024).to_ctypes().ny == 1024


def test_create_reports_nforc_overflow(lib):
    """More than NFORC=2048 forced modes: the reference stops with 'NFORC too small !'
    (src/iniforcing.f90:22); the C-ABI returns GT_ERR_NFORC before touching the device."""
    h = ctypes.c_void_p()
    cp = Params(n=512, k1f=0.0, k2f=60.0).to_ctypes()
    assert lib.gt_create(ctypes.byref(cp), ctypes.byref(h)) == 3
    assert b"NFORC" in lib.gt_last_error(None)


def test_null_arguments_are_errors_not_crashes(lib):
    assert lib.gt_create(None, None) == 1
    assert lib.gt_fft_dir(None, None) == 1
    assert lib.gt_step_rk2(None, None, None, None, None) == 1
    assert lib.gt_diag(None, None, None, None, None, None, None, None) == 1


def test_variant_table(lib):
    """Launch variants by grid size: 0 always, 1 up to 8192, 2-4 up to 1024, 5 from 32 to 512
    (host only)."""
    for n in (16, 32, 64, 512, 1024, 2048, 4096, 8192):
        got = [lib.gt_variant_supported(n, v) for v in range(6)]
        assert got == [1, int(n <= 8192)] + [int(n <= 1024)] * 3 + [int(32 <= n <= 512)], n
    assert lib.gt_variant_supported(100, 0) == 0 and lib.gt_variant_supported(64, 6) == 0
    for n in (16, 64, 512, 2048, 8192):
        assert [lib.gt_row_variant_supported(n, r) for r in range(7)] == \
            [1, int(n <= 8192)] + [int(n <= 1024)] * 3 + [int(32 <= n <= 512), 0], n
    assert lib.gt_set_variant(None, 0) == 1 and lib.gt_autotune(None, 1, None, None) == 1


def test_read_params_dat_format():
    from gturbo_gb300.params import read_params_dat
    text = """6.2831853071795864769d0\t6.2831853071795864769d0
4.5d-46\t8.0d0\t0.1d0\t0.0d0\t1.0d0
2.0d-5\t2
2000\t100000\t100
0.6666666666666666667d0\t1
0.4d0\t20.0d0\t22.0d0

xlx   yly
"""
    p = read_params_dat(text, 2048)
    assert p.n == 2048 and p.rko == 2 and p.truncate == 1 and p.imix == 100
    assert p.nu == 4.5e-46 and p.alpnu == 8.0 and p.alpv == 1.0 and p.dt == 2e-5
    assert p.xlx == 2 * np.pi and p.k1f == 20.0 and p.famp == 0.4


# ---- the bind(C) module's calling convention, argument by argument ---------------------------
# ISO_C_BINDING passes a dummy with the VALUE attribute by value and every other dummy (scalar or
# array) by address; type(c_ptr) is a C object pointer. So a Fortran dummy implies a C parameter
# of a given base type and pointer depth, and a Fortran function result a C return type.
_F_KIND = {"c_int": "int", "c_int32_t": "int32", "c_int64_t": "int64", "c_double": "double",
           "c_float": "float", "c_ptr": "ptr", "gt_params": "gt_params", "gt_info": "gt_info"}
_C_BASE = {"int": "int", "int32_t": "int32", "int64_t": "int64", "uint64_t": "int64", "double": "double",
           "float": "float", "gt_params": "gt_params", "gt_info": "gt_info"}


def _fortran_interfaces(text):
    """{name: (result kind, [(arg, kind, by_value, is_array)])} of every bind(C) interface."""
    import re
    text = re.sub(r"&\s*\n\s*", " ", text)
    out = {}
    for m in re.finditer(r"^\s*(integer|real|type)\((\w+)\)\s+function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C[^)]*\)"
                         r"(.*?)end function", text, re.S | re.M):
        kind, name, args, body = _F_KIND[m.group(2)], m.group(3), m.group(4), m.group(5)
        decl = {}
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if "::" not in line or line.startswith("import"):
                continue
            spec, ents = line.split("::")
            km = re.match(r"(integer|real|type)\((\w+)\)", spec.strip())
            by_value = "value" in spec
            for ent in re.findall(r"(\w+)\s*(\([^)]*\))?", ents):
                decl[ent[0]] = (_F_KIND[km.group(2)], by_value, bool(ent[1]))
        names = [a.strip() for a in args.split(",") if a.strip()]
        out[name] = (kind, [(a, *decl[a]) for a in names])
    return out


def _c_prototypes(header):
    """{name: (return (base, depth), [(base, depth)])} of every gt_ function in the header."""
    import re
    header = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    out = {}
    for m in re.finditer(r"([\w\s\*]+?)\b(gt_\w+)\s*\(([^)]*)\)\s*;", header):
        def parse(t):
            depth = t.count("*")
            words = [w for w in re.sub(r"[\*]", " ", t).split() if w not in ("const", "struct")]
            base = words[0] if words else "void"
            if len(words) > 1 and words[-1] not in _C_BASE and words[-1] != base:
                base = words[0]  # "type name": the first word is the type
            return _C_BASE.get(base, "ptr" if depth else base), depth
        ret = parse(m.group(1).strip().split("\n")[-1])
        params = [parse(p) for p in m.group(3).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(2)] = (ret, params)
    return out


def test_fortran_module_calling_convention_matches_header():
    """Every bind(C) interface of include/gturbo_c.f90 passes each argument the way the C
    prototype in gturbo.h receives it: VALUE dummies as C values of the same type, other
    dummies as pointers to it, type(c_ptr) VALUE as an object pointer, type(c_ptr) arrays or
    non-VALUE scalars as pointers to pointers; and the result kinds match the C return types."""
    fi = _fortran_interfaces(open(os.path.join(ROOT, "include", "gturbo_c.f90")).read())
    cp = _c_prototypes(open(_lib.HEADER).read())
    assert len(fi) >= 19
    for name, (fres, fargs) in fi.items():
        assert name in cp, name
        (cret, cdepth), cparams = cp[name]
        if fres == "ptr":
            assert cdepth >= 1, name
        else:
            assert (fres, 0) == (cret, cdepth), (name, fres, cret, cdepth)
        assert len(fargs) == len(cparams), name
        for (arg, kind, by_value, is_array), (cbase, depth) in zip(fargs, cparams):
            where = f"{name}({arg})"
            if kind == "ptr":
                want = 1 if by_value else 2
                assert depth == want, (where, depth, want)
            elif by_value:
                assert (cbase, depth) == (kind, 0), (where, cbase, depth, kind)
            else:
                assert (cbase, depth) == (kind, 1), (where, cbase, depth, kind)


def test_calling_convention_check_catches_planted_mistakes():
    """The check above fails on a copy of the module with a VALUE attribute dropped or a kind
    changed (the mistakes a hand-written bind(C) block makes)."""
    text = open(os.path.join(ROOT, "include", "gturbo_c.f90")).read()
    cp = _c_prototypes(open(_lib.HEADER).read())

    def consistent(t):
        for name, (fres, fargs) in _fortran_interfaces(t).items():
            _, cparams = cp[name]
            for (arg, kind, by_value, is_array), (cbase, depth) in zip(fargs, cparams):
                if kind == "ptr":
                    if depth != (1 if by_value else 2):
                        return False
                elif (cbase, depth) != (kind, 0 if by_value else 1):
                    return False
        return True

    assert consistent(text)
    old = 'function gt_destroy(h) bind(C, name="gt_destroy")\n      import :: c_int, c_ptr\n      type(c_ptr), value :: h'
    assert old in text
    assert not consistent(text.replace(old, old.replace("type(c_ptr), value :: h", "type(c_ptr) :: h")))
    old = "integer(c_int32_t) :: seed"
    assert old in text
    assert not consistent(text.replace(old, "integer(c_int64_t) :: seed", 1))
