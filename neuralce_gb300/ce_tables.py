"""Template-only cluster-expansion tables for one supercell (host setup).

Restates ``build_ce_gpu_implicit`` (``neuralce/ce/ce_gpu_implicit.py:50-126``) from an orbit list computed by
``lattice.enumerate_orbits``:

* sites in canonical order ``i = cell * nB + basis``, ``cell = (k0*d1 + k1)*d2 + k2`` with ``k = U n mod d``
  (SNF of the transposed supercell matrix), ``perm`` canonical -> input, ``inv_perm`` input -> canonical;
* template rows ``T_b, T_uo, T_bf, T_st, T_eci`` with eci_row = eci * energy_scale / (n_instances * n_cells)
  (``ce_gpu_implicit.py:81-85``); padded members repeat the row's first member with point-function index 0;
* reverse rows ``Rv_*`` per basis site (every (row, slot) whose member has that basis, written relative to the
  slot, ``ce_gpu_implicit.py:96-107``); padded entries point at the site itself with eci 0;
* point-function table ``pf[sublattice, bf, species]`` with bf 0 = 1 and bf p+1 = theta(M, p, s)
  (``neuralce/ce/classical_ce_gpu.py:80-141``).

On top of the reference layout it derives the GPU form used by the kernels: for every basis site the
distinct member offsets of its reverse rows become a *neighbourhood* list ``nb_b / nb_uo`` (``n_nbr`` entries,
entry 0 = the site itself), and each reverse-row member is stored as a 16-bit index into that list
(``Rv_loc``) plus an 8-bit point-function column (``Rv_pfc`` = sublattice * (max_bf+1) + bf).  A swap then
gathers ``n_nbr`` occupancies per site instead of ``J * mo``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .io import Z_OF, Structure
from .lattice import Primitive, canonical_cells, enumerate_orbits, site_decompose, smith_normal_form, theta


@dataclass
class ClusterSpace:
    """Primitive + cutoffs + its orbit list (the part of icet's ClusterSpace the MC path uses)."""
    primitive: Primitive
    cutoffs: list
    orbits: list

    @classmethod
    def build(cls, primitive, cutoffs):
        return cls(primitive, list(cutoffs), enumerate_orbits(primitive, list(cutoffs)))

    @property
    def n_params(self):
        return 1 + len(self.orbits)

    # sublattices: basis sites with the same allowed-species list (icet's get_sublattices)
    def sublattices(self):
        keys = []
        b_sl = np.zeros(self.primitive.nB, np.int32)
        for b, sp in enumerate(self.primitive.species):
            k = tuple(sp)
            if k not in keys:
                keys.append(k)
            b_sl[b] = keys.index(k)
        return b_sl, [list(k) for k in keys]

    def point_functions(self):
        """pf[sl, bf, s]: bf 0 -> 1, bf p+1 -> theta(M_sl, p, s)."""
        b_sl, sl_species = self.sublattices()
        max_sp = max(len(s) for s in sl_species)
        act = [len(s) for s in sl_species if len(s) > 1]
        max_bf = max([m - 1 for m in act], default=0)
        pf = np.zeros((len(sl_species), max_bf + 1, max_sp), np.float64)
        pf[:, 0, :] = 1.0
        for sl, sp in enumerate(sl_species):
            M = len(sp)
            if M < 2:
                continue
            for p in range(M - 1):
                for s in range(M):
                    pf[sl, p + 1, s] = theta(M, p, s)
        return pf


def _check_binary(cs):
    for sp in cs.primitive.species:
        if len(sp) > 2:
            raise NotImplementedError("multicomponent (>2 species) cluster-vector elements are not enumerated; "
                                      "binary sublattices only")


def encode_species(cs, structure: Structure, basis):
    """species index per site (input order): rank of Z within the site's allowed species (sorted by Z)."""
    sig = np.zeros(len(structure), np.int8)
    for b in range(cs.primitive.nB):
        m = basis == b
        lut = {Z_OF[s]: i for i, s in enumerate(cs.primitive.species[b])}
        z = structure.numbers[m]
        bad = sorted(set(int(x) for x in np.unique(z)) - set(lut))
        if bad:
            raise ValueError(f"basis {b}: atomic numbers {bad} not in {cs.primitive.species[b]}")
        tab = np.zeros(256, np.int8)
        for zz, k in lut.items():
            tab[zz] = k
        sig[m] = tab[z]
    return sig


def build_tables(cs: ClusterSpace, structure: Structure, parameters, energy_scale=1.0):
    """All implicit tables for ``structure`` (an integer supercell of ``cs.primitive``)."""
    _check_binary(cs)
    prim = cs.primitive; nB = prim.nB
    params = np.asarray(parameters, np.float64)
    if len(params) != cs.n_params:
        raise ValueError(f"{len(params)} parameters for a cluster space of {cs.n_params}")
    eci_full = params * float(energy_scale)
    zerolet = float(eci_full[0])
    b_sl, sl_species = cs.sublattices()
    pf = cs.point_functions()
    nbf = pf.shape[1]
    basis, off_red, T, n_cells = site_decompose(prim.cell, prim.frac, structure.cell, structure.positions)
    N = len(structure)
    if N != nB * n_cells:
        raise ValueError(f"{N} sites for {nB} basis sites x {n_cells} cells")
    U, d, _ = smith_normal_form(T.T)
    _, cell_idx = canonical_cells(off_red, U, d)
    canon = cell_idx * nB + basis
    if len(np.unique(canon)) != N:
        raise ValueError("sites do not form a clean tiling of the primitive")
    perm = np.argsort(canon).astype(np.int64)
    inv_perm = np.empty(N, np.int64); inv_perm[perm] = np.arange(N)
    # template rows
    tb, to, tbf, teci, tcol = [], [], [], [], []
    for k, o in enumerate(cs.orbits):
        ev = float(eci_full[k + 1]) / (len(o.clusters) * n_cells)
        for inst in o.clusters:
            tb.append([s[0] for s in inst]); to.append([s[1] for s in inst])
            tbf.append([1] * len(inst)); teci.append(ev); tcol.append(k)  # binary: multicomponent vector 0 -> bf 1
    Rt = len(tb); mo = max(len(r) for r in tb)
    T_b = np.zeros((Rt, mo), np.int32); T_off = np.zeros((Rt, mo, 3), np.int64)
    T_bf = np.zeros((Rt, mo), np.int32); T_msk = np.zeros((Rt, mo), bool)
    for r in range(Rt):
        n = len(tb[r]); T_b[r, :n] = tb[r]; T_off[r, :n] = to[r]; T_bf[r, :n] = tbf[r]; T_msk[r, :n] = True
    for r in range(Rt):
        for m in range(mo):
            if not T_msk[r, m]:
                T_b[r, m] = T_b[r, 0]; T_off[r, m] = T_off[r, 0]
    T_uo = np.mod(T_off @ U.T, d).astype(np.int32)
    T_st = b_sl[T_b].astype(np.int32)
    T_eci = np.asarray(teci, np.float64)
    # reverse rows
    ent = [[] for _ in range(nB)]
    for r in range(Rt):
        for m in range(mo):
            if T_msk[r, m]:
                ent[T_b[r, m]].append((r, m))
    J = max(len(e) for e in ent)
    Rv_b = np.zeros((nB, J, mo), np.int32); Rv_off = np.zeros((nB, J, mo, 3), np.int64)
    Rv_bf = np.zeros((nB, J, mo), np.int32); Rv_eci = np.zeros((nB, J), np.float64)
    Rv_col = np.full((nB, J), len(cs.orbits), np.int32)      # padded rows: an extra column whose eci is 0
    Rv_slot = np.full((nB, J), -1, np.int8)                    # slot of the site in the template row (0: the anchor)
    Rv_len = np.array([len(e) for e in ent], np.int32)
    for b in range(nB):
        Rv_b[b] = b
        for j, (r, m) in enumerate(ent[b]):
            Rv_b[b, j] = T_b[r]; Rv_off[b, j] = T_off[r] - T_off[r, m]; Rv_bf[b, j] = T_bf[r]; Rv_eci[b, j] = T_eci[r]
            Rv_col[b, j] = tcol[r]; Rv_slot[b, j] = m
    Rv_uo = np.mod(Rv_off @ U.T, d).astype(np.int32)
    Rv_st = b_sl[Rv_b].astype(np.int32)
    # neighbourhood-compressed GPU layout (cell independent offsets; uo depends on the supercell)
    nb_list = []
    loc = np.zeros((nB, J, mo), np.int32)
    for b in range(nB):
        idx = {(b, (0, 0, 0)): 0}
        for j in range(J):
            for m in range(mo):
                key = (int(Rv_b[b, j, m]), tuple(int(x) for x in Rv_off[b, j, m]))
                if key not in idx:
                    idx[key] = len(idx)
                loc[b, j, m] = idx[key]
        nb_list.append(list(idx))
    n_nbr = max(len(x) for x in nb_list)
    if n_nbr > 65535:
        raise ValueError(f"neighbourhood of {n_nbr} sites exceeds the 16-bit index")
    nb_b = np.zeros((nB, n_nbr), np.int32); nb_off = np.zeros((nB, n_nbr, 3), np.int64)
    for b in range(nB):
        nb_b[b] = b
        for q, (bb, o) in enumerate(nb_list[b]):
            nb_b[b, q] = bb; nb_off[b, q] = o
    nb_uo = np.mod(nb_off @ U.T, d).astype(np.int32)
    Rv_pfc = (Rv_st * nbf + Rv_bf).astype(np.int32)
    # swap groups (active sublattices with their basis sites), O(1) proposal (ce_gpu_implicit.py:108-114)
    act = [sl for sl, sp in enumerate(sl_species) if len(sp) > 1]
    maxb = max(int((b_sl == sl).sum()) for sl in act)
    act_b = np.zeros((len(act), maxb), np.int32); act_nb = np.zeros(len(act), np.int32)
    for a, sl in enumerate(act):
        bs = np.where(b_sl == sl)[0]; act_b[a, :len(bs)] = bs; act_nb[a] = len(bs)
    site_to_sl = b_sl[np.arange(N) % nB]
    return dict(nB=nB, n_cells=n_cells, N=N, d=d.astype(np.int64), U=U, T=T, perm=perm, inv_perm=inv_perm,
                basis_in=basis, zerolet=zerolet, energy_scale=float(energy_scale), pf=pf, n_bf=nbf,
                max_sp=pf.shape[2], b_sl=b_sl, sl_species=sl_species, site_to_sl=site_to_sl,
                T_b=T_b, T_uo=T_uo, T_bf=T_bf, T_st=T_st, T_eci=T_eci, T_msk=T_msk, T_off=T_off, Rt=Rt, mo=mo,
                Rv_b=Rv_b, Rv_uo=Rv_uo, Rv_bf=Rv_bf, Rv_st=Rv_st, Rv_eci=Rv_eci, Rv_len=Rv_len, J=J, Rv_off=Rv_off,
                Rv_col=Rv_col, n_cols=len(cs.orbits) + 1, Rv_slot=Rv_slot,
                Rv_loc=loc, Rv_pfc=Rv_pfc, nb_b=nb_b, nb_uo=nb_uo, nb_off=nb_off, n_nbr=n_nbr,
                act_sl=act, act_b=act_b, act_nb=act_nb)


def synthetic_eci(cs: ClusterSpace, seed, sigma0=0.05):
    """Per-orbit ECIs of the synthetic benchmark cluster set: ECI_k ~ N(0, (sigma0/k)^2) eV per atom, k = 1-based
    rank of the orbit in (order, radius) order starting at the singlet; zerolet 0."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, len(cs.orbits) + 1, dtype=np.float64)
    return np.concatenate([[0.0], rng.normal(0.0, 1.0, len(cs.orbits)) * (sigma0 / k)])
