"""The Fortran binding (fesom2_gb300/fortran/fesom_gpu_mod.F90) against the C ABI it binds.

No Fortran compiler exists here or on the GPU host, so the module is checked as text: every
bind(C) interface names a function the header declares and the library exports, with the same
number of arguments, and the bind(C) derived types hold the fields of the C structs in order.
"""
import os
import re

from fesom2_gb300 import gpu as G
from tests.test_abi import declared_functions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MOD = os.path.join(ROOT, "fesom2_gb300", "fortran", "fesom_gpu_mod.F90")
HDR = os.path.join(ROOT, "include", "fesom_gpu.h")


def _fortran_interfaces():
    src = re.sub(r"&\s*\n\s*", " ", open(MOD).read())  # join continuation lines
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", src):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        out[m.group(3)] = (m.group(1), args)
    return out


def _c_arg_counts():
    hdr = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(fesom_gpu_\w+)\s*\(([^;{]*?)\)\s*;", hdr):
        params = m.group(2).strip()
        out[m.group(1)] = 0 if params in ("", "void") else len(params.split(","))
    return out


def _struct_fields(name):
    hdr = re.sub(r"/\*.*?\*/", "", open(HDR).read(), flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}", hdr, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        names = decl.split(None, 1)[1] if not decl.startswith("const") else decl.split(None, 2)[2]
        # arrays: x[4] in C is x(4) in Fortran
        fields += [re.sub(r"\[(\d+)\]", r"(\1)", n.strip().lstrip("*")) for n in names.split(",")]
    return fields


def _fortran_type_fields(name):
    src = re.sub(r"&\s*\n\s*", " ", open(MOD).read())
    body = re.search(r"type, bind\(C\) :: " + name + r"\n(.*?)end type", src, flags=re.S).group(1)
    fields = []
    for line in body.splitlines():
        line = line.split("!")[0].strip()
        if "::" in line:
            fields += [f.strip() for f in line.split("::")[1].split(",")]
    return fields


def test_every_fortran_interface_binds_a_declared_exported_function():
    ifaces = _fortran_interfaces()
    assert len(ifaces) >= 25
    declared = declared_functions()
    counts = _c_arg_counts()
    lib = G.load()
    for cname, (fname, args) in ifaces.items():
        assert cname == fname, cname
        assert cname in declared, cname
        assert hasattr(lib, cname), cname
        assert counts[cname] == len(args), (cname, counts[cname], len(args))


def test_the_drop_in_routines_are_bound():
    ifaces = _fortran_interfaces()
    for name in ("fesom_gpu_init", "fesom_gpu_adv_tra", "fesom_gpu_vdiff_impl", "fesom_gpu_vdiff_impl_wi",
                 "fesom_gpu_init_tracers_ab", "fesom_gpu_tracer_step", "fesom_gpu_diff_hor",
                 "fesom_gpu_diff_ver_expl", "fesom_gpu_tracer_tail", "fesom_gpu_vdiff_impl_noalloc"):
        assert name in ifaces, name


def test_bind_c_types_follow_the_c_structs():
    for c_name, f_name in (("fesom_tra_cfg", "fesom_tra_cfg"), ("fesom_mesh_desc", "fesom_mesh_desc"),
                           ("fesom_tail_cfg", "fesom_tail_cfg"), ("fesom_tune_result", "fesom_tune_result")):
        assert [f.lower() for f in _struct_fields(c_name)] == [f.lower() for f in _fortran_type_fields(f_name)]
