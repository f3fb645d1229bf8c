"""GB300-native matrix-free geometric-multigrid Stokes solver (Q2-Q1).

The compute path is the CUDA library ``libgb_gmg.so`` behind the C ABI in
``include/gb_gmg.h``; this package holds its ctypes front end
(:mod:`aspect_gb300.gmg`), the caller-side mesh/DoF/constraint builders that
stand in for deal.II (:mod:`aspect_gb300.mesh`) and the synthetic problems
(:mod:`aspect_gb300.problems`).
"""
