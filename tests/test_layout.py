"""The C structs of include/gw_gb300.h, as the compiler lays them out, against
the two bindings that mirror them by hand: the ctypes classes of
geothermalwells_gb300/_lib.py and the Julia structs of
julia/GB300Backend/src/GB300Backend.jl (whose isbits structs take the C
layout: each field at the next multiple of its alignment).

A tiny C program is compiled against the header with gcc and prints sizeof
and offsetof of every field; the Julia struct definitions are read from the
package source and laid out by the same rule."""
import ctypes
import json
import os
import re
import shutil
import subprocess

import pytest

from geothermalwells_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gw_gb300.h")
JULIA = os.path.join(ROOT, "julia", "GB300Backend", "src", "GB300Backend.jl")

# C struct -> (ctypes class, Julia struct name, fields in declaration order)
STRUCTS = {
    "gw_borehole_desc": (_lib.BoreholeDesc, "BoreholeDesc"),
    "gw_material_desc": (_lib.MaterialDesc, "MaterialDesc"),
    "gw_desc": (_lib.Desc, "Desc"),
    "gw_info_t": (_lib.Info, "GwInfo"),
    "gw_adjoint_info_t": (_lib.AdjointInfo, "AdjointInfo"),
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    gcc = shutil.which("gcc") or shutil.which("cc")
    if gcc is None:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("layout")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gw_gb300.h"', 'int main(void) {',
             '  printf("{");']
    first = True
    for cname, (cls, _) in STRUCTS.items():
        fields = [f[0] for f in cls._fields_]
        parts = ['\\"%s\\": [%%zu' % cname] + [', %zu' for _ in fields] + [']']
        fmt = ("" if first else ", ") + "".join(parts)
        args = ["sizeof(%s)" % cname] + ["offsetof(%s, %s)" % (cname, f) for f in fields]
        lines.append('  printf("%s", %s);' % (fmt, ", ".join(args)))
        first = False
    lines += ['  printf("}\\n");', '  return 0;', '}']
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([gcc, "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def ctypes_layout(cls):
    return [ctypes.sizeof(cls)] + [getattr(cls, f[0]).offset for f in cls._fields_]


# sizes (= alignments) of the field types the Julia structs use
JL_SIZES = {"Cint": 4, "Cdouble": 8, "Clonglong": 8, "Float64": 8, "Int32": 4, "Int64": 8}


def julia_structs():
    """Field lists of the isbits structs in the Julia package source."""
    src = open(JULIA).read()
    out = {}
    for m in re.finditer(r"^struct\s+(\w+)\s*\n(.*?)^end", src, re.S | re.M):
        name, body = m.group(1), m.group(2)
        fields = []
        for line in body.split("\n"):
            line = line.split("#")[0]
            for decl in line.split(";"):
                decl = decl.strip()
                if "::" in decl:
                    fn, ty = [x.strip() for x in decl.split("::", 1)]
                    fields.append((fn, ty))
        out[name] = fields
    return out


def julia_layout(structs, name):
    """(size, alignment, offsets) of a Julia isbits struct by the C rule."""
    off, align, offsets = 0, 1, []
    for _, ty in structs[name]:
        if ty.startswith("Ptr{"):
            sz = al = 8
        elif ty in JL_SIZES:
            sz = al = JL_SIZES[ty]
        else:
            sz, al, _ = julia_layout(structs, ty)
        off = (off + al - 1) // al * al
        offsets.append(off)
        off += sz
        align = max(align, al)
    size = (off + align - 1) // align * align
    return size, align, offsets


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_ctypes_mirror_matches_header(cname, c_layout):
    cls, _ = STRUCTS[cname]
    assert ctypes_layout(cls) == c_layout[cname]


@pytest.mark.parametrize("cname", list(STRUCTS))
def test_julia_mirror_matches_header(cname, c_layout):
    cls, jname = STRUCTS[cname]
    structs = julia_structs()
    assert jname in structs, "struct %s missing from the Julia package" % jname
    names = [f[0] for f in structs[jname]]
    assert len(names) == len(cls._fields_)
    size, _, offsets = julia_layout(structs, jname)
    assert [size] + offsets == c_layout[cname]


def test_julia_package_binds_declared_symbols():
    """Every gw_* symbol the Julia package calls is declared in the header."""
    src = open(JULIA).read()
    header = open(HEADER).read()
    called = set(re.findall(r":(gw_\w+)", src))
    assert called, "no ccall symbols found"
    declared = set(re.findall(r"\b(gw_\w+)\s*\(", header))
    assert called <= declared, sorted(called - declared)
