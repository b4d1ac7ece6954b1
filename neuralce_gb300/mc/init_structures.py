"""Per-replica starting structures (``--init_npz``), after ``neuralce/mc/init_structures.py``.

npz format: ``numbers (R, N)`` atomic numbers of replica r's starting structure, ``positions (N, 3)`` and
``cell (3, 3)`` of one geometry for all replicas (the cell must equal the MC cell), ``temps (R,)`` the temperature
each structure belongs to (must equal the run's).  Sites may be listed in any order: they are matched onto the MC
cell by lattice site (basis index + primitive-cell offset reduced into the supercell), never by atom index.
"""
from __future__ import annotations

import numpy as np

from ..lattice import site_decompose


def _site_keys(prim, cell, positions):
    basis, off_red, T, _ = site_decompose(prim.cell, prim.frac, cell, positions)
    S = 1 << 17
    if np.abs(off_red).max(initial=0) >= S or basis.max(initial=0) >= 256:
        raise ValueError("cell too large for the lattice-site key")
    o = np.asarray(off_red, np.int64) + S
    keys = (np.asarray(basis, np.int64) << 54) | (o[:, 0] << 36) | (o[:, 1] << 18) | o[:, 2]
    if len(np.unique(keys)) != len(keys):
        raise ValueError("two atoms occupy the same lattice site")
    return keys, T


def map_to_reference(prim, ref, cell, positions):
    """idx (N,): site idx[i] of the given geometry sits on the lattice site of ``ref`` atom i."""
    cell = np.asarray(cell, float); positions = np.asarray(positions, float)
    if cell.shape != (3, 3) or not np.allclose(cell, ref.cell, rtol=0, atol=1e-3):
        raise ValueError(f"init_npz cell differs from the MC cell:\n{cell}\nvs\n{ref.cell}")
    if len(positions) != len(ref):
        raise ValueError(f"init_npz has {len(positions)} sites, the MC cell {len(ref)}")
    k_ref, T_ref = _site_keys(prim, ref.cell, ref.positions)
    k_oth, T_oth = _site_keys(prim, ref.cell, positions)
    if not np.array_equal(T_ref, T_oth):
        raise ValueError(f"supercell matrices differ: {T_ref.tolist()} vs {T_oth.tolist()}")
    o_ref, o_oth = np.argsort(k_ref, kind="stable"), np.argsort(k_oth, kind="stable")
    if not np.array_equal(k_ref[o_ref], k_oth[o_oth]):
        raise ValueError("init_npz sites do not coincide with the MC cell's lattice sites")
    idx = np.empty(len(k_ref), np.int64); idx[o_ref] = o_oth
    return idx


def load_init_npz(path, prim, ref, temps, tol_T=0.5):
    """(numbers (R, N) in the atom order of ``ref``, npz temperatures); checks the cell, the lattice sites, one
    structure per run temperature and every replica's composition against ``ref``."""
    z = np.load(path)
    numbers = np.asarray(z["numbers"]); T_npz = np.asarray(z["temps"], float).reshape(-1)
    temps = np.asarray(temps, float).reshape(-1)
    if numbers.ndim != 2 or numbers.shape[0] != len(T_npz):
        raise ValueError(f"init_npz numbers {numbers.shape} / temps {T_npz.shape} inconsistent")
    if len(temps) != len(T_npz) or np.any(np.abs(temps - T_npz) > np.maximum(tol_T, 1e-5 * T_npz)):
        raise ValueError(f"init_npz temperatures {np.round(T_npz, 1).tolist()} != run temperatures "
                         f"{np.round(temps, 1).tolist()}")
    idx = map_to_reference(prim, ref, z["cell"], z["positions"])
    out = numbers[:, idx]
    comp = np.bincount(np.asarray(ref.numbers, np.int64), minlength=256)
    for r in range(out.shape[0]):
        if not np.array_equal(np.bincount(out[r].astype(np.int64), minlength=256), comp):
            raise ValueError(f"init_npz replica {r}: composition differs from the MC cell")
    return out, T_npz
