"""The Python mirror (poisson_caustic_design_gb300._lib) agrees with the C ABI
header include/pcd.h: every enumerator has the same value, and every ctypes
structure has the C structure's fields in the same order with the same
scalar kinds.  Pure text checks: no library load, no device."""
import os
import re

from conftest import ROOT

C_TYPES = {"int": "c_int", "double": "c_double", "long long": "c_longlong", "float": "c_float"}


def header():
    src = open(os.path.join(ROOT, "include", "pcd.h")).read()
    return re.sub(r"/\*.*?\*/", "", src, flags=re.S)


def enumerators():
    return {name: int(val) for name, val in re.findall(r"\b(PCD_[A-Z0-9_]+)\s*=\s*(-?\d+)", header())}


def structs():
    """typedef struct { ... } name;  ->  {name: [(field, kind), ...]}"""
    out = {}
    for body, name in re.findall(r"typedef struct \{(.*?)\}\s*(\w+)\s*;", header(), flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(const )?(long long|int|double|float|[a-z_]+ ?\*?)\s*(\*?)\s*(.*)$", decl)
            assert m, decl
            base, ptr, names = m.group(2).strip(), m.group(3), m.group(4)
            for nm in names.split(","):
                nm = nm.strip()
                star = ptr == "*" or nm.startswith("*") or base.endswith("*")
                nm = nm.lstrip("*").strip()
                arr = re.match(r"(\w+)\[(\d+)\]", nm)
                kind = "ptr" if star else C_TYPES.get(base.rstrip("*").strip(), base)
                if arr:
                    fields.append((arr.group(1), (kind, int(arr.group(2)))))
                else:
                    fields.append((nm, kind))
        out[name] = fields
    return out


def test_enumerators_match_python_constants():
    from poisson_caustic_design_gb300 import _lib
    from poisson_caustic_design_gb300.caustic_design import GRID, VERT

    en = enumerators()
    assert len(en) >= 35
    prefixes = {"PCD_STOP_": "STOP_", "PCD_PREC_": "PREC_", "PCD_SCHED_": "SCHED_", "PCD_WARM_": "WARM_"}
    unmatched = []
    for name, val in en.items():
        cp = next((c for c in prefixes if name.startswith(c)), None)
        if cp:
            py = prefixes[cp] + name[len(cp):]
            assert getattr(_lib, py) == val, (name, val, getattr(_lib, py, None))
        elif name.startswith("PCD_GRID_"):
            assert GRID[name[len("PCD_GRID_"):].lower()] == val, name
        elif name.startswith("PCD_VERT_"):
            key = name[len("PCD_VERT_"):].lower()
            assert VERT.get(key, VERT.get("vertex_" + key)) == val, name
        elif hasattr(_lib, name):  # status codes keep their C names
            assert getattr(_lib, name) == val, (name, val)
        else:
            unmatched.append(name)
    assert not unmatched, unmatched


def test_ctypes_structures_follow_the_header():
    import ctypes as C

    from poisson_caustic_design_gb300 import _lib

    st = structs()
    pairs = {"pcd_solve_opts": _lib.SolveOpts, "pcd_solve_stats": _lib.SolveStats, "pcd_instance": _lib.Instance,
             "pcd_instance_stats": _lib.InstanceStats, "pcd_batch_stats": _lib.BatchStats,
             "pcd_design_params": _lib.DesignParams}
    nested = {cname: py for cname, py in pairs.items()}
    for cname, py in pairs.items():
        assert cname in st, cname
        cf = st[cname]
        pf = py._fields_
        assert [n for n, _ in cf] == [n for n, _ in pf], (cname, cf, pf)
        for (n, kind), (_, ctype) in zip(cf, pf):
            if kind == "ptr":
                assert ctype in (C.c_void_p,) or hasattr(ctype, "contents") or ctype is C.c_char_p, (cname, n, ctype)
            elif isinstance(kind, tuple):
                assert issubclass(ctype, C.Array) and ctype._length_ == kind[1], (cname, n, ctype)
                assert ctype._type_ is getattr(C, kind[0]), (cname, n, ctype)
            elif kind in nested:
                assert ctype is nested[kind], (cname, n, kind, ctype)
            else:
                assert ctype is getattr(C, kind), (cname, n, kind, ctype)
