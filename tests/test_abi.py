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
