"""Per-replica starting structures for ``--init_npz``.

The file format is the reference's interface (``neuralce/mc/init_structures.py`` documents it): ``numbers (R, N)``
atomic numbers of each replica's starting structure, ``positions (N, 3)`` Cartesian positions shared by all
replicas, ``cell (3, 3)`` (the MC cell), ``temps (R,)`` the temperature of each structure (the run's ladder).

Sites may come in any order.  Here they are matched onto the MC cell geometrically: both site sets are taken to
fractional coordinates of the MC cell and wrapped into the unit cube, and every MC site is paired with the nearest
file site under periodic boundaries (a k-d tree on the 3-torus).  The pairing must be one-to-one and every pair must
lie within ``tol_A`` angstrom; the result is the file's numbers re-ordered into the MC cell's atom order.
"""
from __future__ import annotations

import numpy as np


def _wrapped_fractional(cell, positions):
    f = np.asarray(positions, float) @ np.linalg.inv(np.asarray(cell, float))
    f -= np.floor(f)
    f[f >= 1.0] -= 1.0                                   # -1e-17 wraps to exactly 1.0 in floating point
    return f


def site_order(cell, mc_positions, file_positions, tol_A=0.2):
    """perm (N,): file site perm[i] occupies MC site i.  Raises ValueError when the file's sites are not the MC
    cell's sites."""
    from scipy.spatial import cKDTree
    mc_positions = np.asarray(mc_positions, float); file_positions = np.asarray(file_positions, float)
    if file_positions.shape != mc_positions.shape:
        raise ValueError(f"the --init_npz file lists {len(file_positions)} sites; the MC cell has {len(mc_positions)}")
    f_mc, f_file = _wrapped_fractional(cell, mc_positions), _wrapped_fractional(cell, file_positions)
    tree = cKDTree(f_file, boxsize=1.0)
    dist, perm = tree.query(f_mc, k=1)
    # fractional distance -> an upper bound in angstrom (the longest cell vector scales every component)
    worst = float(np.max(dist, initial=0.0)) * float(np.max(np.linalg.norm(np.asarray(cell, float), axis=1)))
    if worst > tol_A:
        i = int(np.argmax(dist))
        raise ValueError(f"MC site {i} at {mc_positions[i].round(3).tolist()} A has no --init_npz site within {tol_A} A")
    if len(np.unique(perm)) != len(perm):
        raise ValueError("two MC sites pair with the same --init_npz site: the file's sites are not the MC lattice")
    return perm.astype(np.int64)


def load_init_npz(path, ref, temps, tol_T=0.5, tol_A=0.2):
    """(numbers (R, N) in the atom order of the MC structure ``ref``, the file's temperatures).

    Checked: the file's cell is the MC cell (1e-3 A), its sites are the MC cell's sites, it holds one structure per
    run temperature in ladder order (within max(tol_T, 1e-5 T) kelvin), and each structure has the MC cell's
    composition (swaps conserve it)."""
    with np.load(path) as z:
        missing = [k for k in ("numbers", "positions", "cell", "temps") if k not in z.files]
        if missing:
            raise ValueError(f"{path}: missing array(s) {missing} (need numbers, positions, cell, temps)")
        numbers = np.asarray(z["numbers"]); positions = np.asarray(z["positions"], float)
        cell = np.asarray(z["cell"], float); T_file = np.asarray(z["temps"], float).reshape(-1)
    if numbers.ndim != 2 or numbers.shape[0] != T_file.size:
        raise ValueError(f"{path}: numbers of shape {numbers.shape} need one row per temperature ({T_file.size})")
    if cell.shape != (3, 3) or np.abs(cell - np.asarray(ref.cell, float)).max() > 1e-3:
        raise ValueError(f"{path}: the structures' cell\n{cell}\nis not the MC cell\n{np.asarray(ref.cell, float)}")
    run_T = np.asarray(temps, float).reshape(-1)
    if run_T.size != T_file.size or np.any(np.abs(run_T - T_file) > np.maximum(tol_T, 1e-5 * run_T)):
        raise ValueError(f"{path}: structures for T = {np.round(T_file, 1).tolist()} K, but the run's ladder is "
                         f"T = {np.round(run_T, 1).tolist()} K")
    perm = site_order(ref.cell, ref.positions, positions, tol_A)
    out = numbers[:, perm]
    want = np.unique(np.asarray(ref.numbers, np.int64), return_counts=True)
    for r, row in enumerate(out):
        have = np.unique(row.astype(np.int64), return_counts=True)
        if not (np.array_equal(have[0], want[0]) and np.array_equal(have[1], want[1])):
            raise ValueError(f"{path}: structure {r} (T = {T_file[r]:.1f} K) has composition "
                             f"{dict(zip(have[0].tolist(), have[1].tolist()))}, the MC cell "
                             f"{dict(zip(want[0].tolist(), want[1].tolist()))}")
    return out, T_file
