"""Helpers shared by the GPU parity tests (GPU solver vs CPU oracle on the same inputs)."""
import numpy as np

from aspect_gb300 import mesh


def rel_err(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def p_err(a, b):
    """Relative difference of two pressure vectors with their means removed: with
    free slip (or no slip) on the whole boundary the pressure is determined only
    up to a constant, which the caller fixes afterwards by normalisation."""
    a, b = np.asarray(a), np.asarray(b)
    return rel_err(a - a.mean(), b - b.mean())


def hierarchy(dim, n, geometry="box", permute=False, seed=0):
    levels = mesh.box_hierarchy(dim, n)
    if geometry == "q2":
        levels = [mesh.to_q2_geometry(l) for l in levels]
    elif geometry == "q2-distorted":
        levels = [mesh.to_q2_geometry(l, mesh.smooth_distortion()) for l in levels]
    if permute:
        levels = [mesh.permute_dofs(l, seed + i)[0] for i, l in enumerate(levels)]
    return levels


def random_eta(level, per_q, seed=1, contrast=3.0):
    rng = np.random.default_rng(seed)
    nq = 3 ** level.dim
    shape = (level.n_cells, nq) if per_q else (level.n_cells,)
    return np.exp(contrast * rng.uniform(-1, 1, size=shape))
