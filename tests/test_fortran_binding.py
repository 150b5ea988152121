"""The Fortran ISO_C_BINDING module (scone_gb300/fortran/scone_gpu_mod.f90) agrees with the C ABI.

No Fortran compiler is available, so the module is checked by reading it: every bind(C) derived type
is laid out by C's rules (each component at the next multiple of its alignment, the size rounded up
to the largest alignment) and compared with the offsets and sizes a C program built against
include/scone_gpu.h prints; every prototype of the header has an interface block whose arguments
pass the same kinds in the same way (by value or by reference).  No GPU is used."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MOD = os.path.join(ROOT, "scone_gb300", "fortran", "scone_gpu_mod.f90")
HEADER = os.path.join(ROOT, "include", "scone_gpu.h")
SCALAR = {"c_int32_t": (4, 4), "c_int64_t": (8, 8), "c_double": (8, 8), "c_size_t": (8, 8)}


def fortran_types():
    """{type name: [(component, (size, align), count, nested type or None)]}, in declaration order."""
    text = open(MOD).read()
    out = {}
    for name, body in re.findall(r"type, bind\(C\) :: (\w+)\n(.*?)end type \1", text, re.S):
        comps = []
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            decl, names = line.split("::")
            m = re.match(r"(integer|real)\((c_\w+)\)|type\((\w+)\)", decl.strip())
            for nm in [x.strip() for x in re.split(r",(?![^(]*\))", names)]:
                mm = re.match(r"(\w+)(?:\((\d+)\))?$", nm)
                count = int(mm.group(2) or 1)
                if m.group(2):
                    comps.append((mm.group(1), SCALAR[m.group(2)], count, None))
                elif m.group(3) == "c_ptr":
                    comps.append((mm.group(1), (8, 8), count, None))
                else:
                    comps.append((mm.group(1), None, count, m.group(3)))
        out[name] = comps
    return out


def c_layout(types, name, cache):
    if name in cache:
        return cache[name]
    off, align, offsets = 0, 1, {}
    for comp, sa, count, nested in types[name]:
        if nested:
            size, a, _ = c_layout(types, nested, cache)
        else:
            size, a = sa
        off = (off + a - 1) // a * a
        offsets[comp] = off
        off += size * count
        align = max(align, a)
    size = (off + align - 1) // align * align
    cache[name] = (size, align, offsets)
    return cache[name]


def test_fortran_types_match_the_c_structs(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    types = fortran_types()
    assert len(types) >= 16
    cache = {}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "scone_gpu.h"', 'int main(void) {']
    for t, comps in types.items():
        lines.append(f'  printf("{t} size %zu\\n", sizeof({t}));')
        for comp, _, _, _ in comps:
            lines.append(f'  printf("{t} {comp} %zu\\n", offsetof({t}, {comp}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "f_layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "f_layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {tuple(l.split()[:2]): int(l.split()[2])
           for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines() if l}
    for t in types:
        size, _, offsets = c_layout(types, t, cache)
        assert got[(t, "size")] == size, t
        for comp, off in offsets.items():
            assert got[(t, comp)] == off, (t, comp)


def header_prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"^\s*(int32_t|uint64_t|double)\s+(sg_\w+)\s*\(([^;]*?)\)\s*;", text, re.M | re.S):
        args = " ".join(args.split())
        params = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (ret, [re.match(r"(?:const\s+)?(\w+)\s*(\*?)\s*\w+$", p).groups() for p in params])
    return out


def fortran_interfaces():
    text = re.sub(r"&[ \t]*\n[ \t]*", "", open(MOD).read())        # join continued lines
    out = {}
    for name, args, body in re.findall(r'function (sg_\w+)\(([^)]*)\) bind\(C, name="\1"\)\n(.*?)end function \1', text, re.S):
        names = [a.strip() for a in args.split(",") if a.strip()]
        decl = {}
        ret = None
        for line in body.splitlines():
            line = line.strip()
            if "::" not in line:
                continue
            spec, nm = [x.strip() for x in line.split("::")]
            if nm == name:
                ret = spec
            else:
                decl[nm] = spec
        out[name] = (ret, [decl[n] for n in names])
    return out


C2F = {"int32_t": "integer(c_int32_t)", "int64_t": "integer(c_int64_t)", "uint64_t": "integer(c_int64_t)",
       "double": "real(c_double)", "size_t": "integer(c_size_t)"}


def test_every_entry_point_has_a_matching_interface():
    protos, ifaces = header_prototypes(), fortran_interfaces()
    assert len(protos) >= 50
    assert set(protos) == set(ifaces), set(protos) ^ set(ifaces)
    for name, (ret, params) in protos.items():
        fret, fargs = ifaces[name]
        assert fret == C2F[ret], name
        assert len(params) == len(fargs), name
        for (ty, ptr), spec in zip(params, fargs):
            if ty in ("sg_handle", "sg_batch"):
                assert spec == ("type(c_ptr), intent(out)" if ptr else "type(c_ptr), value"), (name, spec)
            elif ty.startswith("sg_"):
                assert ptr and spec.startswith(f"type({ty})"), (name, spec)
            elif ty == "char":
                assert ptr and spec.startswith("character(kind=c_char), dimension(*)"), (name, spec)
            elif ptr:
                assert spec.startswith(C2F[ty]) and "value" not in spec, (name, spec)   # by reference
            else:
                assert spec == f"{C2F[ty]}, value", (name, spec)


def test_fortran_lines_fit_free_form():
    """Free-form Fortran allows 132 characters a line (gfortran's default)."""
    for path in (MOD, os.path.join(os.path.dirname(MOD), "transportOperatorGPU_class.f90")):
        for i, line in enumerate(open(path).read().splitlines(), 1):
            assert len(line) <= 132, (os.path.basename(path), i, len(line))
