"""Generates tests/golden/nsinker_golden.json.

Run in a container where the reference tree is present:
    python tests/golden/make_nsinker_fixtures.py
It reads the NSinker benchmark's input data from the reference -- the number of
sinkers and the viscosity ratio of benchmarks/nsinker/nsinker_gmg.prm, the
sinker density default, delta, omega and the first n_sinkers sinker centres of
benchmarks/nsinker/nsinker.cc -- and the solver outputs the reference committed
for three of its tests on the 4^3 mesh: tests/nsinker_gmg_gc/screen-output (the
first solve, GMRES, before the adaptive step), tests/nsinker_gmg_idr/screen-output
(IDR(2)) and tests/nsinker_gmg_no_avg/screen-output (GMRES, no averaging).
"""
import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference tree: $ASPECT_REFERENCE, else a directory "reference" beside the repository
REF = os.environ.get("ASPECT_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))


def prm_value(txt, key):
    return re.search(r"set\s+" + re.escape(key) + r"\s*=\s*([^\s#]+)", txt).group(1)


def main():
    prm = open(os.path.join(REF, "benchmarks", "nsinker", "nsinker_gmg.prm")).read()
    src = open(os.path.join(REF, "benchmarks", "nsinker", "nsinker.cc")).read()
    n_sinkers = int(prm_value(prm, "Number of sinkers"))
    ratio = float(prm_value(prm, "Dynamic viscosity ratio"))
    density = float(re.search(r'declare_entry \("Sinker density", "([^"]+)"', src).group(1))
    delta = float(re.search(r"delta = ([0-9.eE+-]+);", src).group(1))
    omega = float(re.search(r"omega = ([0-9.eE+-]+);", src).group(1))
    centres = {}
    for m in re.finditer(r"centers\[(\d+)\] = Point<3>\(([^,]+), ([^,]+), ([^)]+)\);", src):
        centres[int(m.group(1))] = [float(m.group(k)) for k in (2, 3, 4)]
    golden = dict(n_sinkers=n_sinkers, dynamic_viscosity_ratio=ratio, sinker_density=density, delta=delta,
                  omega=omega, centres=[centres[i] for i in range(n_sinkers)],
                  linear_solver_tolerance=float(prm_value(prm, "Linear solver tolerance")),
                  n_cheap_steps=int(prm_value(prm, "Number of cheap Stokes solver steps")),
                  restart=int(prm_value(prm, "GMRES solver restart length")))
    for test, key in (("nsinker_gmg_gc", "gmres"), ("nsinker_gmg_idr", "idr2"), ("nsinker_gmg_no_avg", "no_avg")):
        txt = open(os.path.join(REF, "tests", test, "screen-output")).read()
        its = re.search(r"Stokes solver \((GMRES|IDR\(\d+\))\): (\d+)\+(\d+) iterations", txt)
        schur = re.search(r"Schur complement preconditioner: (\d+)\+(\d+) iterations", txt)
        dofs = re.search(r"Number of degrees of freedom: [\d,]+ \(([\d,]+)\+([\d,]+)", txt)
        vrange = re.search(r"Viscosity range: ([0-9.eE+-]+) - ([0-9.eE+-]+)", txt)
        golden[key] = dict(test=test, solver=its.group(1), cheap_iterations=int(its.group(2)),
                           expensive_iterations=int(its.group(3)), schur_applications=int(schur.group(1)),
                           n_u=int(dofs.group(1).replace(",", "")), n_p=int(dofs.group(2).replace(",", "")),
                           viscosity_range=[float(vrange.group(1)), float(vrange.group(2))])
    with open(os.path.join(HERE, "nsinker_golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    print(json.dumps(golden, indent=1))


if __name__ == "__main__":
    main()
