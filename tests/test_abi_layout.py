"""The C-ABI's POD structs agree on all three sides of the boundary (CPU):
the C compiler's layout of include/swave.h (tests/abi_layout.c), the ctypes
mirror in seismic_gb300, and the Fortran bind(C) types of
include/swave_iface.f90 (field order, kinds and the offsets C alignment
gives them); and every entry point of swave.h has a Fortran interface and a
ctypes signature."""
import os
import re
import shutil
import subprocess

import pytest

import seismic_gb300 as sw

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

CTYPES = {"sw_genpar": sw.SwGenpar, "sw_prop_desc": sw.SwPropDesc, "sw_prop_io": sw.SwPropIO,
          "sw_shot": sw.SwShot, "sw_window": sw.SwWindow, "sw_fwi_shot": sw.SwFwiShot,
          "sw_fwi_desc": sw.SwFwiDesc, "sw_reg_desc": sw.SwRegDesc,
          "sw_reg_state": sw.SwRegState, "sw_tuning": sw.SwTuning, "sw_stats": sw.SwStats,
          "sw_lbfgs_oc_state": sw.SwLbfgsOcState, "sw_lbfgs_oc_desc": sw.SwLbfgsOcDesc}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("abi") / "abi_layout")
    subprocess.run([cc, "-std=c11", "-I", INC, "-o", exe,
                    os.path.join(ROOT, "tests", "abi_layout.c")], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    layout, cur = {}, None
    for line in out.splitlines():
        p = line.split()
        if p[0] == "struct":
            cur = p[1]
            layout[cur] = {"size": int(p[2]), "fields": []}
        else:
            layout[cur]["fields"].append((p[1], int(p[2]), int(p[3])))
    return layout


def _fortran_types():
    """name -> [(field, bytes, align)] in declaration order."""
    src = open(os.path.join(INC, "swave_iface.f90")).read()
    kinds = {"integer(c_int)": (4, 4), "real(c_float)": (4, 4), "real(c_double)": (8, 8),
             "integer(c_int64_t)": (8, 8), "type(c_ptr)": (8, 8)}
    types = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)end type \1", src, re.S):
        name, body = m.group(1), m.group(2)
        fields = []
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            decl, names = [x.strip() for x in line.split("::")]
            for nm in [x.strip() for x in names.split(",")]:
                count = 1
                am = re.match(r"(\w+)\((\d+)\)", nm)
                if am:
                    nm, count = am.group(1), int(am.group(2))
                if decl.startswith("type(sw_"):
                    inner = decl[5:-1]
                    fields.append((nm, ("struct", inner), count))
                else:
                    fields.append((nm, kinds[decl], count))
        types[name] = fields
    return types


def _layout_of(types, name, memo):
    if name in memo:
        return memo[name]
    off, align, out = 0, 1, []
    for nm, kind, count in types[name]:
        if kind[0] == "struct":
            size, al, _ = _layout_of(types, kind[1], memo)
        else:
            size, al = kind
        off = (off + al - 1) // al * al
        out.append((nm, off, size * count))
        off += size * count
        align = max(align, al)
    total = (off + align - 1) // align * align
    memo[name] = (total, align, out)
    return memo[name]


def test_ctypes_mirror_matches_c(c_layout):
    import ctypes
    for name, cls in CTYPES.items():
        c = c_layout[name]
        assert ctypes.sizeof(cls) == c["size"], name
        names = [f[0] for f in cls._fields_]
        assert names == [f[0] for f in c["fields"]], name
        for fname, off, size in c["fields"]:
            assert getattr(cls, fname).offset == off, (name, fname)
            assert getattr(cls, fname).size == size, (name, fname)


def test_fortran_types_match_c(c_layout):
    types = _fortran_types()
    assert set(types) == set(CTYPES)
    memo = {}
    for name in CTYPES:
        size, _, fields = _layout_of(types, name, memo)
        c = c_layout[name]
        assert size == c["size"], name
        # Fortran names are case-insensitive.
        assert [(f[0].lower(), f[1], f[2]) for f in fields] == \
            [(f[0].lower(), f[1], f[2]) for f in c["fields"]], name


def test_every_entry_point_is_bound():
    hdr = open(os.path.join(INC, "swave.h")).read()
    funcs = set(re.findall(r"^(?:int|const char \*)\s*(sw_\w+)\(", hdr, re.M))
    assert len(funcs) >= 45
    f90 = open(os.path.join(INC, "swave_iface.f90")).read()
    bound = set(re.findall(r'bind\(C, name="(sw_\w+)"\)', f90))
    assert funcs == bound, (funcs - bound, bound - funcs)
    assert funcs <= set(sw._SIGS), funcs - set(sw._SIGS)
