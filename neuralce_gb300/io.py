"""File formats of the reference, read and written without icet or ase.

* icet ``.ce`` files (``ClusterExpansion.read``, used at ``neuralce/ce/icet_mc.py:131``): a tar archive with
  ``items`` (pickled dict with ``parameters``) and ``cluster_space`` (a nested tar with ``items`` -- cutoffs,
  chemical_symbols, tolerances -- and ``atoms``, the primitive structure in ase's JSON database layout).
* NeuralCE ``model.pkl`` (``neuralce/nce/mc_model.py:20-21``): a plain pickle whose ``primitive`` entry is an
  ``ase.Atoms``; it is unpickled here with a restricted unpickler that turns ``ase.atoms.Atoms`` and
  ``ase.cell.Cell`` into small stand-ins carrying the cell, positions and numbers.
* cif files in the P1 layout the reference writes (``_atom_site_fract_*`` loop) and reads through ase.
"""
from __future__ import annotations

import io
import json
import pickle
import tarfile
from dataclasses import dataclass, field

import numpy as np

from .lattice import Primitive

SYMBOLS = ("X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu "
           "Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr").split()
Z_OF = {s: i for i, s in enumerate(SYMBOLS)}


@dataclass
class Structure:
    """Periodic structure: cell rows (A), cartesian positions (A), atomic numbers."""
    cell: np.ndarray
    positions: np.ndarray
    numbers: np.ndarray

    def __len__(self):
        return len(self.numbers)

    def copy(self):
        return Structure(self.cell.copy(), self.positions.copy(), self.numbers.copy())

    def scaled_positions(self):
        return self.positions @ np.linalg.inv(self.cell)

    def repeat(self, reps):
        nx, ny, nz = (int(r) for r in reps)
        shifts = np.array([[i, j, k] for i in range(nx) for j in range(ny) for k in range(nz)], float) @ self.cell
        pos = (shifts[:, None, :] + self.positions[None]).reshape(-1, 3)
        nums = np.tile(self.numbers, len(shifts))
        cell = self.cell * np.array([nx, ny, nz], float)[:, None]
        return Structure(cell, pos, nums)

    @property
    def symbols(self):
        return [SYMBOLS[int(z)] for z in self.numbers]


def fcc_conventional(a, reps=(1, 1, 1), symbol="Ni"):
    """Cubic 4-site fcc cell of edge ``a`` repeated ``reps`` times (ase ``bulk(.., 'fcc', cubic=True)`` order)."""
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    cell = np.eye(3) * a
    s = Structure(cell, basis @ cell, np.full(4, Z_OF[symbol], np.int64))
    return s.repeat(reps)


def fcc_primitive(a, symbols=("Ni", "Pt")):
    h = a / 2.0
    return Primitive(cell=np.array([[0, h, h], [h, 0, h], [h, h, 0]], float), frac=np.zeros((1, 3)),
                     species=[sorted(symbols, key=lambda s: Z_OF[s])], numbers=np.array([Z_OF[symbols[0]]]))


# ───────────────────────────── icet .ce ────────────────────────────────────────────────────────

@dataclass
class ClusterExpansionFile:
    """Contents of an icet .ce file."""
    parameters: np.ndarray
    cutoffs: list
    chemical_symbols: list            # per primitive site, allowed species
    primitive: Primitive
    metadata: dict = field(default_factory=dict)


def _ase_json_atoms(text):
    d = json.loads(text)
    row = d[str(d["ids"][0])]

    def arr(v):
        if isinstance(v, dict) and "__ndarray__" in v:
            shape, dtype, flat = v["__ndarray__"]
            return np.asarray(flat, dtype=dtype).reshape(shape)
        return np.asarray(v)
    cell = row["cell"]
    cell = arr(cell["array"]) if isinstance(cell, dict) and "array" in cell else arr(cell)
    return np.asarray(cell, float), arr(row["positions"]).astype(float), arr(row["numbers"]).astype(np.int64)


def read_ce(path):
    """icet ClusterExpansion.read without icet: parameters, cutoffs, species and the primitive structure."""
    with tarfile.open(path) as tf:
        items = pickle.loads(tf.extractfile("items").read())
        cs_bytes = tf.extractfile("cluster_space").read()
    with tarfile.open(fileobj=io.BytesIO(cs_bytes)) as tf:
        cs_items = pickle.loads(tf.extractfile("items").read())
        cell, pos, nums = _ase_json_atoms(tf.extractfile("atoms").read().decode())
    chem = [sorted(list(s), key=lambda x: Z_OF[x]) for s in cs_items["chemical_symbols"]]
    if len(chem) == 1 and len(nums) > 1:
        chem = chem * len(nums)
    frac = pos @ np.linalg.inv(cell)
    prim = Primitive(cell=cell, frac=frac, species=chem, numbers=nums)
    meta = dict(items.get("metadata", {}))
    return ClusterExpansionFile(parameters=np.asarray(items["parameters"], float), cutoffs=list(cs_items["cutoffs"]),
                                chemical_symbols=chem, primitive=prim, metadata=meta)


def write_ce(path, ce: ClusterExpansionFile):
    """Write a .ce archive with the same layout icet uses (items + nested cluster_space tar)."""
    def add(tf, name, data):
        ti = tarfile.TarInfo(name); ti.size = len(data); tf.addfile(ti, io.BytesIO(data))
    p = ce.primitive
    atoms = {"1": {"cell": {"array": {"__ndarray__": [[3, 3], "float64", np.asarray(p.cell, float).ravel().tolist()]},
                            "__ase_objtype__": "cell"},
                   "numbers": {"__ndarray__": [[p.nB], "int64", [int(x) for x in (p.numbers if p.numbers is not None
                                                                              else [Z_OF[s[0]] for s in p.species])]]},
                   "pbc": {"__ndarray__": [[3], "bool", [True, True, True]]},
                   "positions": {"__ndarray__": [[p.nB, 3], "float64", (np.asarray(p.frac) @ p.cell).ravel().tolist()]}},
             "ids": [1], "nextid": 2}
    inner = io.BytesIO()
    with tarfile.open(fileobj=inner, mode="w") as tf:
        add(tf, "items", pickle.dumps({"cutoffs": list(ce.cutoffs), "chemical_symbols": ce.chemical_symbols,
                                       "pruning_history": [], "symprec": 1e-5, "position_tolerance": 1e-5}))
        add(tf, "atoms", json.dumps(atoms).encode())
    with tarfile.open(path, "w") as tf:
        add(tf, "items", pickle.dumps({"parameters": np.asarray(ce.parameters, float), "metadata": ce.metadata}))
        add(tf, "cluster_space", inner.getvalue())


# ───────────────────────────── NeuralCE model.pkl ──────────────────────────────────────────────

class _Stand:
    """stand-in for ase.Atoms / ase.Cell inside model.pkl"""
    def __init__(self, *a, **k):
        pass

    def __setstate__(self, st):
        self.__dict__.update(st)


class _AtomsStand(_Stand):
    pass


class _CellStand(_Stand):
    pass


class _ModelUnpickler(pickle.Unpickler):
    def find_class(self, module, name):
        if module.startswith("ase"):
            return _CellStand if name == "Cell" else _AtomsStand
        if module.startswith(("numpy", "builtins", "collections", "copyreg")) or module == "_codecs":
            return super().find_class(module, name)
        raise pickle.UnpicklingError(f"model.pkl refers to {module}.{name}, which this reader does not load")


def _stand_to_primitive(a, chem):
    cellobj = a.__dict__.get("_cellobj")
    cell = np.asarray(getattr(cellobj, "array", cellobj.__dict__.get("array")), float)
    arrays = a.__dict__["arrays"]
    pos = np.asarray(arrays["positions"], float); nums = np.asarray(arrays["numbers"], np.int64)
    chem = [sorted(list(s), key=lambda x: Z_OF[x]) for s in chem]
    if len(chem) == 1 and len(nums) > 1:
        chem = chem * len(nums)
    return Primitive(cell=cell, frac=pos @ np.linalg.inv(cell), species=chem, numbers=nums)


def load_model(path):
    """Load a NeuralCE model.pkl (``neuralce/nce/mc_model.py:20-21``); ``primitive`` becomes a Primitive."""
    with open(path, "rb") as f:
        mdl = _ModelUnpickler(f).load()
    if "primitive" in mdl and not isinstance(mdl["primitive"], Primitive):
        mdl["primitive"] = _stand_to_primitive(mdl["primitive"], mdl["chemical_symbols"])
    return mdl


# ───────────────────────────── cif (P1) ────────────────────────────────────────────────────────

def read_cif(path):
    """Minimal P1 cif reader: cell lengths/angles and the _atom_site_fract_* loop."""
    vals = {}; cols = []; rows = []; in_loop = False
    for line in open(path):
        s = line.strip()
        if not s or s.startswith("#"):
            continue
        if s.startswith("loop_"):
            in_loop = True; cols = []; continue
        if in_loop and s.startswith("_"):
            cols.append(s.split()[0]); continue
        if in_loop and cols and "_atom_site_fract_x" in cols:
            rows.append(s.split()); continue
        if in_loop and cols:
            in_loop = False
        if s.startswith("_"):
            parts = s.split(None, 1)
            if len(parts) == 2:
                vals[parts[0]] = parts[1]
    a, b, c = (float(vals[f"_cell_length_{x}"].split("(")[0]) for x in "abc")
    al, be, ga = (np.radians(float(vals[f"_cell_angle_{x}"].split("(")[0])) for x in ("alpha", "beta", "gamma"))
    cx = np.cos(be); cy = (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    cell = np.array([[a, 0, 0], [b * np.cos(ga), b * np.sin(ga), 0], [c * cx, c * cy, c * np.sqrt(max(1 - cx * cx - cy * cy, 0))]])
    cell[np.abs(cell) < 1e-12] = 0.0
    ix = cols.index("_atom_site_fract_x"); iy = cols.index("_atom_site_fract_y"); iz = cols.index("_atom_site_fract_z")
    it = cols.index("_atom_site_type_symbol") if "_atom_site_type_symbol" in cols else cols.index("_atom_site_label")
    frac = np.array([[float(r[ix].split("(")[0]), float(r[iy].split("(")[0]), float(r[iz].split("(")[0])] for r in rows])
    sym = ["".join(ch for ch in r[it] if ch.isalpha()) for r in rows]
    nums = np.array([Z_OF[s] for s in sym], np.int64)
    return Structure(cell, frac @ cell, nums)


def write_cif(path, s: Structure):
    L = np.linalg.norm(s.cell, axis=1)
    ang = [np.degrees(np.arccos(np.dot(s.cell[(i + 1) % 3], s.cell[(i + 2) % 3]) / (L[(i + 1) % 3] * L[(i + 2) % 3]))) for i in range(3)]
    if not np.allclose(s.cell, np.diag(np.diag(s.cell))):
        raise ValueError("write_cif writes orthorhombic cells only")
    frac = s.scaled_positions()
    with open(path, "w") as f:
        f.write("data_image0\n")
        for k, v in zip("abc", L):
            f.write(f"_cell_length_{k} {v:.10g}\n")
        for k, v in zip(("alpha", "beta", "gamma"), ang):
            f.write(f"_cell_angle_{k} {v:.10g}\n")
        f.write("_space_group_name_H-M_alt 'P 1'\n_space_group_IT_number 1\n\nloop_\n  _atom_site_type_symbol\n"
                "  _atom_site_label\n  _atom_site_fract_x\n  _atom_site_fract_y\n  _atom_site_fract_z\n  _atom_site_occupancy\n")
        for i, (z, fr) in enumerate(zip(s.numbers, frac)):
            sy = SYMBOLS[int(z)]
            f.write(f"  {sy} {sy}{i + 1} {fr[0]:.12f} {fr[1]:.12f} {fr[2]:.12f} 1.0\n")
