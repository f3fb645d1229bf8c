"""The C-ABI library loads and exports every entry point include/gb_gmg.h
declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

from aspect_gb300 import build, gmg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "gb_gmg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]*?\b(gb_gmg_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ["gb_gmg_create", "gb_gmg_set_level_mesh", "gb_gmg_set_level_constraints",
                     "gb_gmg_set_transfer", "gb_gmg_set_viscosity", "gb_gmg_build_preconditioner",
                     "gb_gmg_vmult", "gb_gmg_solve", "gb_gmg_adjoint_gradient", "gb_gmg_last_error",
                     "gb_gmg_destroy"]:
        assert required in names


def test_library_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(gmg.EXPORTS) == declared_functions()


# the public structs of include/gb_gmg.h and their ctypes mirrors in aspect_gb300.gmg
ABI_STRUCTS = {"gb_gmg_options": gmg.Options, "gb_gmg_solve_params": gmg.SolveParams,
               "gb_gmg_outputs": gmg.Outputs, "gb_gmg_newton_terms": gmg.NewtonTerms}


def test_ctypes_structs_match_the_header_layout(tmp_path):
    """Each struct's size and every field's name and offset, as the C compiler
    lays out include/gb_gmg.h, equal those of the Python front end's ctypes
    Structure: a field added, dropped or reordered on one side only fails here."""
    import shutil
    import subprocess

    import pytest

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "gb_gmg.h"', "int main(void) {"]
    for cname, py in ABI_STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines():
        cname, key, value = line.split()
        got[(cname, key)] = int(value)
    for cname, py in ABI_STRUCTS.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for field, _ in py._fields_:
            assert got[(cname, field)] == getattr(py, field).offset, (cname, field)


def test_ctypes_structs_name_every_header_field():
    """The header's struct members, in order, are the ctypes fields (the layout
    test above compiles only the fields the ctypes side names)."""
    src = open(os.path.join(ROOT, "include", "gb_gmg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    for cname, py in ABI_STRUCTS.items():
        body = re.search(r"typedef struct " + cname + r"\s*\{(.*?)\}\s*" + cname + ";", src, flags=re.S).group(1)
        members = [m.group(1) for decl in body.split(";") if decl.strip()
                   for m in [re.search(r"(\w+)\s*(?:\[[^\]]*\])?\s*$", decl.strip())]]
        assert members == [f for f, _ in py._fields_], cname
