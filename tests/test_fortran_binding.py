"""The Fortran interface module include/sps_gb300.f90 against the C header include/sps.h.

No Fortran compiler exists on the machines this library is built on, so the module is
checked by reading it: the bind(C) derived type sps_params must list the C struct's
fields in the same order with the same element kinds and counts, which makes every byte
offset and the total size equal (the offsets of the Fortran type are computed with the
C layout rules that bind(C) types follow; the C offsets come from gcc).  Every bind(C)
interface must name a function of the header with the same number of arguments.
"""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "sps_gb300.f90")
HDR = os.path.join(ROOT, "include", "sps.h")

# iso_c_binding kinds: (size, alignment)
FKIND = {"integer(c_int32_t)": 4, "integer(c_int)": 4, "integer(c_int64_t)": 8,
         "real(c_double)": 8, "real(c_float)": 4, "type(c_ptr)": 8}
CTYPE = {"int32_t": 4, "double": 8, "float": 4, "int64_t": 8}


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def fortran_fields(text):
    """[(name, element size, count)] of the sps_params derived type."""
    m = re.search(r"type\s*,\s*bind\(C\)\s*::\s*sps_params\s*\n(.*?)\n\s*end type", text,
                  re.S | re.I)
    assert m, "no bind(C) type sps_params"
    out = []
    for line in m.group(1).splitlines():
        line = line.split("!")[0].strip()
        if not line:
            continue
        kind, names = [s.strip() for s in line.split("::")]
        kind = re.sub(r"\s+", "", kind.lower())
        size = FKIND[kind]
        for part in re.findall(r"\w+(?:\(\d+\))?", names):
            mm = re.match(r"(\w+)(?:\((\d+)\))?", part)
            out.append((mm.group(1).lower(), size, int(mm.group(2) or 1)))
    return out


def c_fields(text):
    """[(name, element size, count)] of the C struct sps_params."""
    body = re.search(r"typedef struct sps_params \{(.*?)\} sps_params;", _strip_c(text), re.S)
    assert body
    out = []
    for decl in body.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ptr = "*" in decl
        decl = decl.replace("const", "").replace("*", " ")
        toks = decl.split(None, 1)
        size = 8 if ptr else CTYPE[toks[0]]
        for part in toks[1].split(","):
            mm = re.match(r"\s*(\w+)\s*(?:\[(\d+)\])?", part)
            out.append((mm.group(1), size, int(mm.group(2) or 1)))
    return out


def layout(fields):
    """Byte offsets and the total size under the C rules (each element aligned to its
    size, the struct to its largest element)."""
    off, offs, align = 0, [], 1
    for _, size, count in fields:
        off = (off + size - 1) // size * size
        offs.append(off)
        off += size * count
        align = max(align, size)
    return offs, (off + align - 1) // align * align


def gcc_offsets(tmp_path, names):
    src = tmp_path / "off.c"
    src.write_text("#include <stddef.h>\n#include <stdio.h>\n#include \"sps.h\"\nint main(void){\n" +
                   "".join('printf("%%zu\\n", offsetof(sps_params, %s));\n' % n for n in names) +
                   'printf("%zu\\n", sizeof(sps_params));\nreturn 0;}\n')
    exe = tmp_path / "off"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)],
                   check=True, capture_output=True)
    vals = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                           text=True).stdout.split()]
    return vals[:-1], vals[-1]


def mismatches(ff, cf, c_offs, c_size):
    bad = []
    if [f[0] for f in ff] != [c[0].lower() for c in cf]:
        bad.append("field names/order differ")
    for f, c in zip(ff, cf):  # Fortran names are case-insensitive
        if f[1:] != c[1:]:
            bad.append("%s: Fortran %s vs C %s" % (f[0], f[1:], c[1:]))
    f_offs, f_size = layout(ff)
    if f_offs != c_offs[:len(f_offs)] or len(f_offs) != len(c_offs):
        bad.append("offsets differ")
    if f_size != c_size:
        bad.append("size %d vs C %d" % (f_size, c_size))
    return bad


def test_params_type_matches_c_struct(tmp_path):
    ff = fortran_fields(open(F90).read())
    cf = c_fields(open(HDR).read())
    c_offs, c_size = gcc_offsets(tmp_path, [c[0] for c in cf])
    # the C rules reproduce gcc's own layout of the header
    assert layout(cf) == (c_offs, c_size)
    assert mismatches(ff, cf, c_offs, c_size) == []


def test_a_short_type_is_caught(tmp_path):
    # a type that stops before the trailing fields (as a binding that ends at
    # max_neighbours would) passes a struct shorter than the C one
    ff = fortran_fields(open(F90).read())
    cf = c_fields(open(HDR).read())
    c_offs, c_size = gcc_offsets(tmp_path, [c[0] for c in cf])
    k = [f[0] for f in ff].index("max_neighbours") + 1
    assert mismatches(ff[:k], cf, c_offs, c_size)
    swapped = ff[:]
    swapped[0], swapped[1] = swapped[1], swapped[0]
    assert mismatches(swapped, cf, c_offs, c_size)


def _c_arity():
    text = _strip_c(open(HDR).read())
    out = {}
    for m in re.finditer(r"\b(?:int|void)\s+(sps_\w+)\s*\(([^)]*)\)\s*;", text):
        args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        out[m.group(1)] = len(args)
    return out


def test_interfaces_match_header():
    text = open(F90).read()
    arity = _c_arity()
    found = re.findall(r"(?:function|subroutine)\s+(sps_\w+)\s*\(([^)]*)\)\s*&?\s*(?:\n\s*)?bind\(C,"
                       r"\s*name=\"(\w+)\"\)", text, re.I)
    assert len(found) >= 10
    for fname, args, cname in found:
        assert fname == cname
        assert cname in arity, cname
        nargs = len([a for a in args.replace("&", " ").split(",") if a.strip()])
        assert nargs == arity[cname], (cname, nargs, arity[cname])
