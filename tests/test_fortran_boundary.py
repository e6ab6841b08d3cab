"""The Fortran side of the boundary (fortran/hande_gpu_m.f90) against the C
header (include/hande_gpu.h), checked on the CPU without a Fortran compiler:

- every bind(c) derived type has the fields of its C struct in the same order,
  with the same interoperable kind and array length;
- the module declares an interface for every entry point of the header, under
  the same binding name, with the same number of arguments, each of the same
  kind and passed the same way (by value or by reference).

A HANDE build that uses the module (do_fciqmc calling hgpu_run_cycles,
hgpu_end_report, hgpu_get_state / hgpu_set_state for restarts) therefore sees
the C layout the library was compiled with."""

import os
import re

from tests.conftest import ROOT

HEADER = open(os.path.join(ROOT, "include", "hande_gpu.h")).read()
FORTRAN = open(os.path.join(ROOT, "fortran", "hande_gpu_m.f90")).read()
STRUCTS = ["hgpu_system", "hgpu_config", "hgpu_report", "hgpu_state", "hgpu_launch"]
CONST = {"HGPU_MAX_WORDS": 2, "HGPU_MAX_SPACES": 2}

C_KIND = {"int32_t": "i32", "int64_t": "i64", "uint64_t": "i64", "double": "f64", "char": "char", "void": "void"}
F_KIND = {"c_int32_t": "i32", "c_int64_t": "i64", "c_uint64_t": "i64", "c_double": "f64", "c_char": "char"}


def strip_c_comments(t):
    return re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", t, flags=re.S))


def c_struct_fields(name):
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), strip_c_comments(HEADER), re.S).group(1)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(?:const\s+)?(\w+)\s+(.*)", decl)
        base, rest = m.group(1), m.group(2)
        for item in rest.split(","):
            item = item.strip()
            ptr = item.startswith("*")
            item = item.lstrip("*").strip()
            am = re.match(r"(\w+)(?:\[(\w+)\])?", item)
            n = CONST.get(am.group(2), am.group(2)) if am.group(2) else 1
            out.append((am.group(1).lower(), "ptr" if ptr else C_KIND[base], int(n)))
    return out


def f_type_fields(name):
    body = re.search(r"type, bind\(c\) :: %s\n(.*?)end type %s" % (name, name), FORTRAN, re.S).group(1)
    out = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        m = re.match(r"(integer|real|type)\((\w+)\)\s*::\s*(.*)", line)
        kind = "ptr" if m.group(1) == "type" and m.group(2) == "c_ptr" else F_KIND[m.group(2)]
        for item in re.findall(r"(\w+)(?:\((\w+)\))?", m.group(3)):
            n = CONST.get(item[1], item[1]) if item[1] else 1
            out.append((item[0].lower(), kind, int(n)))
    return out


def c_functions():
    out = {}
    for m in re.finditer(r"^(int32_t|const char \*)\s*(hgpu_\w+)\s*\(([^)]*)\)\s*;", strip_c_comments(HEADER), re.M):
        args = []
        for a in m.group(3).split(","):
            a = a.strip()
            if a in ("", "void"):
                continue
            depth = a.count("*")
            base = re.sub(r"\bconst\b", "", a.replace("*", " ")).split()[0]
            if base.startswith("hgpu_") and base not in STRUCTS:  # opaque handle / batch
                base, depth = "opaque", depth
            kind = base if base in STRUCTS or base == "opaque" else C_KIND.get(base, base)
            if kind == "void":
                kind = "opaque"
            args.append((kind, depth))
        out[m.group(2)] = ("i32" if m.group(1) == "int32_t" else "ptr", args)
    return out


def f_functions():
    out = {}
    for m in re.finditer(r"(integer\(c_int32_t\)|type\(c_ptr\)) function (\w+)\(([^)]*)\)\s*&?\s*(?:\n\s*)?"
                         r"(?:[\w, &()=']*?)bind\(c, name='(\w+)'\)(.*?)end function \2", FORTRAN, re.S):
        ret = "i32" if m.group(1).startswith("integer") else "ptr"
        names = [x.strip().lower() for x in m.group(3).replace("&", " ").split(",") if x.strip()]
        decls = {}
        for line in m.group(5).splitlines():
            line = line.strip()
            dm = re.match(r"(integer|real|type|character)\((?:kind=)?(\w+)\)(.*?)::\s*(.*)", line)
            if not dm:
                continue
            attrs = dm.group(3)
            for v in re.findall(r"(\w+)(?:\([^)]*\))?", dm.group(4)):
                decls[v.lower()] = (dm.group(1), dm.group(2), "value" in attrs)
        args = []
        for n in names:
            cls, kind, byval = decls[n]
            if cls == "type" and kind == "c_ptr":
                args.append(("opaque", 1 if byval else 2))
            elif cls == "type":
                args.append((kind, 0 if byval else 1))
            else:
                args.append((F_KIND[kind], 0 if byval else 1))
        out[m.group(4)] = (ret, args)
    return out


def test_derived_types_match_structs():
    for name in STRUCTS:
        c = c_struct_fields(name)
        f = f_type_fields(name)
        assert [x[0] for x in f] == [x[0] for x in c], name
        assert f == c, name


def test_interfaces_cover_every_entry_point():
    c = c_functions()
    f = f_functions()
    assert sorted(f) == sorted(c)
    for name in c:
        cret, cargs = c[name]
        fret, fargs = f[name]
        assert fret == cret, name
        # a pointer to an opaque handle or a stream is a type(c_ptr) passed by
        # value (a handle's address: by reference); the device buffers of the
        # allocation-free entry point are type(c_ptr) too
        device = {0, 4} if name == "hgpu_self_annihilate_noalloc" else set()
        norm = [("opaque", 1) if i in device else (k, d) for i, (k, d) in enumerate(cargs)]
        assert len(fargs) == len(norm), name
        assert fargs == norm, "%s: %s != %s" % (name, fargs, norm)
