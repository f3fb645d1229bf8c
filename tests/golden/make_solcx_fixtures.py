"""Generates tests/golden/solcx_exact.npz and solcx_golden.json.

Run in a container where the reference tree is present:
    python tests/golden/make_solcx_fixtures.py
It builds the reference's own SolCx analytic solution (oracle/ref_build.sh ->
oracle/_ref/libsolcx.so), evaluates it at the QGauss(4) points of the 4x4 and
16x16 meshes the reference tests use, and records the numbers printed in the
reference's committed outputs tests/sol_cx_{2,4}_gmg/screen-output and
tests/sol_cx_4_gmg_no_avg/screen-output (no material averaging) and
tests/no_cheap_gmg/screen-output (expensive solver only, density averaged too).
"""
import ctypes
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from aspect_gb300 import fe, problems  # noqa: E402

# the reference tree: $ASPECT_REFERENCE, else a directory "reference" beside the repository
REF = os.environ.get("ASPECT_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


def main():
    so = subprocess.check_output(["sh", os.path.join(ROOT, "oracle", "ref_build.sh")]).decode().split()[-1]
    lib = ctypes.CDLL(so)
    out = {}
    for nref in (2, 4):
        P = problems.solcx(nref)
        f = P.fine
        pts, _ = fe.quadrature(2, 4)
        xq = f.map_points(pts).reshape(-1, 2)
        u = np.zeros((len(xq), 2))
        p = np.zeros(len(xq))
        vel = (ctypes.c_double * 2)()
        pr = ctypes.c_double()
        ts = (ctypes.c_double * 3)()
        sr = (ctypes.c_double * 3)()
        for i, x in enumerate(xq):
            pos = (ctypes.c_double * 2)(x[0], x[1])
            lib._Velic_solCx(pos, ctypes.c_double(1.0), ctypes.c_double(1e6), ctypes.c_double(0.5),
                             ctypes.c_int(1), vel, ctypes.byref(pr), ts, sr)
            u[i] = vel[0], vel[1]
            p[i] = pr.value
        n = 2 ** nref
        out[f"u_{n}"] = u.reshape(f.n_cells, -1, 2)
        out[f"p_{n}"] = p.reshape(f.n_cells, -1)
    np.savez_compressed(os.path.join(HERE, "solcx_exact.npz"), **out)
    golden = {}
    for test, n in (("sol_cx_2_gmg", 4), ("sol_cx_4_gmg", 16), ("sol_cx_4_gmg_no_avg", "16_no_avg"),
                    ("no_cheap_gmg", "16_no_cheap")):
        txt = open(os.path.join(REF, "tests", test, "screen-output")).read()
        its = re.search(r"Solving Stokes system \(GMG\)\.\.\. (\d+)\+(\d+) iterations", txt)
        errs = re.search(r"Errors u_L1, p_L1, u_L2, p_L2: ([^\n]+)", txt).group(1)
        dofs = re.search(r"Number of degrees of freedom: [\d,]+ \(([\d,]+)\+([\d,]+)", txt)
        golden[str(n)] = dict(test=test, cheap_iterations=int(its.group(1)),
                              expensive_iterations=int(its.group(2)),
                              errors=[float(v) for v in errs.split(",")],
                              n_u=int(dofs.group(1).replace(",", "")),
                              n_p=int(dofs.group(2).replace(",", "")))
    with open(os.path.join(HERE, "solcx_golden.json"), "w") as fh:
        json.dump(golden, fh, indent=1)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
