"""The Fortran binding include/m_hbi_gpu.f90 against the C ABI it wraps.

No Fortran compiler exists on either machine of this build, so the module is
checked by reading it: every bind(c) interface names an entry point that
include/hbi_gpu.h declares, with the same number of arguments; the bind(c)
mirror of hbi_bemv lists the C struct's fields in the C order; and the
HACApK routines carry the reference's names and dummy-argument lists, so that
HBI's driver needs only its `use` lines changed:

  HACApK_init(nd,st_ctl,st_bemv,icomma)                    m_HACApK_base.f90:246
  HACApK_generate(st_leafmtxp,st_bemv,st_ctl,coord,ztol)   m_HACApK_use.f90:133
  HACApK_construct_LH(st_LHp,st_leafmtxp,st_bemv,st_ctl,coord,ztol)  m_HACApK_use.f90:263
  HACApK_gen_lattice_vector(st_vec,st_leafmtxp,st_ctl)     m_HACApK_base.f90:3449
  HACApK_adot_lattice_hyp(st_au,st_LHp,st_ctl,wws,st_u)    m_HACApK_solve.f90:220
  HACApK_free_leafmtxp(st_leafmtxp)                        m_HACApK_base.f90:3084
  HACApK_finalize(st_ctl)                                  m_HACApK_base.f90:385
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = open(os.path.join(ROOT, "include", "m_hbi_gpu.f90")).read()
HDR = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "hbi_gpu.h")).read(), flags=re.S)

REFERENCE_ARGS = {
    "HACApK_init": ["nd", "st_ctl", "st_bemv", "icomma"],
    "HACApK_generate": ["st_leafmtxp", "st_bemv", "st_ctl", "coord", "ztol"],
    "HACApK_construct_LH": ["st_LHp", "st_leafmtxp", "st_bemv", "st_ctl", "coord", "ztol"],
    "HACApK_gen_lattice_vector": ["st_vec", "st_leafmtxp", "st_ctl"],
    "HACApK_adot_lattice_hyp": ["st_au", "st_LHp", "st_ctl", "wws", "st_u"],
    "HACApK_free_leafmtxp": ["st_leafmtxp"],
    "HACApK_finalize": ["st_ctl"],
}


def _code(src):
    """Fortran source without comments, continuation lines joined."""
    lines = [l.split("!")[0].rstrip() for l in src.splitlines()]
    out, cur = [], ""
    for l in lines:
        if cur:
            l = l.lstrip().lstrip("&")
        if l.endswith("&"):
            cur += l[:-1]
            continue
        out.append(cur + l)
        cur = ""
    return out


def c_prototypes():
    protos = {}
    for m in re.finditer(r"\b(?:int|void\*|const char\*)\s+(hbi_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", HDR):
        args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
        protos[m.group(1)] = len(args)
    return protos


def fortran_bindings():
    b = {}
    for line in _code(F90):
        m = re.search(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\s*\(\s*c\s*,\s*name\s*=\s*'(\w+)'", line, re.I)
        if m:
            args = [a for a in m.group(2).split(",") if a.strip()]
            b[m.group(3)] = len(args)
    return b


def test_every_binding_names_a_declared_entry_point_with_its_arity():
    protos = c_prototypes()
    binds = fortran_bindings()
    assert len(binds) >= 14
    for name, nargs in binds.items():
        if name == "strlen":
            continue
        assert name in protos, f"{name} is not declared in include/hbi_gpu.h"
        assert protos[name] == nargs, (name, protos[name], nargs)


def test_hot_path_entries_are_bound():
    binds = fortran_bindings()
    for name in ("hbi_init", "hbi_generate", "hbi_construct_lh", "hbi_gen_lattice_vector",
                 "hbi_adot_lattice_hyp", "hbi_free_leafmtxp", "hbi_finalize", "hbi_lh_check_error"):
        assert name in binds, name


def test_hacapk_routines_keep_the_reference_argument_lists():
    code = "\n".join(_code(F90))
    for name, args in REFERENCE_ARGS.items():
        m = re.search(r"(?:integer\s+function|subroutine)\s+" + name + r"\s*\(([^)]*)\)", code)
        assert m, name
        got = [a.strip() for a in m.group(1).split(",")]
        assert got == args, (name, got)


def test_bemv_mirror_follows_the_c_struct():
    cs = re.search(r"typedef struct \{(.*?)\} hbi_bemv;", HDR, re.S).group(1)
    c_fields = []
    for decl in cs.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names = decl.split(None, 1)[1] if not decl.startswith("const") else decl.split("double", 1)[1]
        c_fields += [n.strip().lstrip("*").strip() for n in names.split(",")]
    fm = re.search(r"type, bind\(c\) :: hbi_bemv_c(.*?)end type hbi_bemv_c", F90, re.S).group(1)
    f_fields = []
    for line in _code(fm):
        if "::" in line:
            f_fields += [n.strip() for n in line.split("::")[1].split(",")]
    assert f_fields == c_fields


def test_problem_names_cover_the_hot_path_kinds():
    code = "\n".join(_code(F90))
    for name in ("'2dvs'", "'3dph'", "'3dnr'", "'3dnt'", "'2dph'", "'2dn'", "'3dht'"):
        assert name in code, name
    defs = dict((k.strip(), int(v)) for k, v in re.findall(r"(HBI_[0-9A-Z_]+) = (\d+)", code))
    hdr = dict((k, int(v)) for k, v in re.findall(r"#define (HBI_[0-9A-Z_]+) (\d+)", HDR))
    for k in ("HBI_2DVS", "HBI_3DPH", "HBI_3DNR", "HBI_3DNT", "HBI_2DPH", "HBI_2DN", "HBI_3DHT", "HBI_STORE_F64",
              "HBI_STORE_F32", "HBI_STORE_BF16"):
        assert defs[k] == hdr[k], k
