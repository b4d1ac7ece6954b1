"""GPUClusterExpansion: the reference's CE boundary object on the GB300 engine.

Mirrors ``neuralce/ce/classical_ce_gpu.py:496-593`` (implicit branch ``:515-535``): the constructor builds the
template-only tables for a supercell, sites are in canonical order (``perm`` canonical -> input,
``inv_perm`` input -> canonical), and ``energy_a`` / ``delta_energy_a`` / ``energy`` / ``batched_energy`` /
``encode`` / ``sublattices`` keep the reference's meaning.  Arithmetic runs in libnce_gb300 (CUDA);
torch only holds device buffers.
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from . import _lib
from .ce_tables import ClusterSpace, build_tables, encode_species
from .io import ClusterExpansionFile, Structure


_SERIAL = itertools.count(1)      # identity of a model for launch-shape caches (never reused, unlike id())


def _arr(x, dtype):
    return np.ascontiguousarray(np.asarray(x, dtype=dtype))


class CETables:
    """Host copy of the tables in the C-ABI layout, kept alive while the struct points at them."""

    def __init__(self, tb):
        self.tb = tb
        nB, J, mo = tb["nB"], tb["J"], tb["mo"]
        self.Rv_len = _arr(tb["Rv_len"], np.int32)
        self.Rv_loc = _arr(tb["Rv_loc"], np.uint16)
        self.Rv_pfc = _arr(tb["Rv_pfc"], np.uint8)
        self.Rv_eci = _arr(tb["Rv_eci"], np.float64)
        self.nb_b = _arr(tb["nb_b"], np.int32)
        self.nb_uo = _arr(tb["nb_uo"], np.int32)
        self.T_b = _arr(tb["T_b"], np.int32)
        self.T_uo = _arr(tb["T_uo"], np.int32)
        self.T_pfc = _arr(tb["T_st"] * tb["n_bf"] + tb["T_bf"], np.uint8)
        self.T_eci = _arr(tb["T_eci"], np.float64)
        self.pf = _arr(tb["pf"].reshape(-1, tb["max_sp"]), np.float64)
        self.act_b = _arr(tb["act_b"], np.int32)
        self.act_nb = _arr(tb["act_nb"], np.int32)
        w = self.act_nb.astype(np.float64) * 1.0
        cum = np.cumsum(w) / w.sum()
        g = np.floor(cum * 2.0 ** 32).astype(np.uint64); g[-1] = np.uint64(2 ** 32)
        self.grp_cum = _arr(g, np.uint64)
        self.Rv_col = _arr(tb["Rv_col"], np.int32)
        self.Rv_slot = _arr(tb["Rv_slot"], np.int8)
        s = _lib.NceCeTables()
        s.nB, s.J, s.mo, s.n_nbr = nB, J, mo, tb["n_nbr"]
        s.n_pfc, s.max_sp = self.pf.shape[0], tb["max_sp"]
        for c in range(3):
            s.d[c] = int(tb["d"][c])
        s.n_cells = int(tb["n_cells"]); s.zerolet = float(tb["zerolet"])
        s.Rv_len, s.Rv_loc, s.Rv_pfc, s.Rv_eci = (_lib.ptr(a) for a in (self.Rv_len, self.Rv_loc, self.Rv_pfc, self.Rv_eci))
        s.nb_b, s.nb_uo = _lib.ptr(self.nb_b), _lib.ptr(self.nb_uo)
        s.Rt = tb["Rt"]
        s.T_b, s.T_uo, s.T_pfc, s.T_eci = (_lib.ptr(a) for a in (self.T_b, self.T_uo, self.T_pfc, self.T_eci))
        s.pf = _lib.ptr(self.pf)
        s.n_groups, s.max_gb = self.act_b.shape
        s.act_b, s.act_nb, s.grp_cum = _lib.ptr(self.act_b), _lib.ptr(self.act_nb), _lib.ptr(self.grp_cum)
        s.Rv_col, s.n_cols = _lib.ptr(self.Rv_col), int(tb["n_cols"])
        s.Rv_slot = _lib.ptr(self.Rv_slot)
        self.struct = s


class GPUClusterExpansion:
    """Template-only CE on the GPU for one supercell (the reference's ``table_mode='implicit'``).

    ce: a ClusterExpansionFile (``io.read_ce``) or a tuple (ClusterSpace, parameters).
    energy_scale: E is the total energy of ``energy_scale`` copies of the cell the parameters refer to
    (``classical_ce_gpu.py:500-505``)."""

    implicit = True

    def __init__(self, ce, supercell: Structure, table_mode="implicit", energy_scale=1.0, cluster_space=None):
        if table_mode not in (None, "implicit"):
            raise ValueError("only the implicit (template-only) tables are implemented on this engine")
        if isinstance(ce, ClusterExpansionFile):
            cs = cluster_space or ClusterSpace.build(ce.primitive, ce.cutoffs)
            params = ce.parameters
        else:
            cs, params = ce
        self.ce = ce
        self.cs = cs
        self.parameters = np.asarray(params, np.float64)
        self.supercell = supercell
        self.energy_scale = float(energy_scale)
        self.info = build_tables(cs, supercell, self.parameters, energy_scale)
        tb = self.info
        self.perm, self.inv_perm = tb["perm"], tb["inv_perm"]
        self.site_to_sl = tb["site_to_sl"]
        self._n_atoms = tb["N"]
        self.sublattices = []
        nB = tb["nB"]
        for sl in tb["act_sl"]:
            bs = np.where(tb["b_sl"] == sl)[0]
            idx = (np.arange(tb["n_cells"])[:, None] * nB + bs[None]).reshape(-1).astype(np.int32)
            sp = tb["sl_species"][sl]
            self.sublattices.append({"indices": np.sort(idx), "n_species": len(sp), "chemical_symbols": list(sp),
                                     "name": "".join(sp)})
        self.host_tables = CETables(tb)
        self._handle = None
        self.serial = next(_SERIAL)

    # ── reference attributes ──
    @property
    def n_atoms(self):
        return self._n_atoms

    @property
    def tp(self):
        return self

    @property
    def has_spin(self):
        return False

    @property
    def n_instances(self):
        return self.info["Rt"] * self.info["n_cells"]

    @property
    def max_size(self):
        return self.info["mo"]

    def __repr__(self):
        return (f"GPUClusterExpansion(n_atoms={self.n_atoms}, n_instances={self.n_instances}, max_size={self.max_size}, "
                f"sublattices={len(self.sublattices)})")

    # ── device handle ──
    @property
    def handle(self):
        if self._handle is None:
            h = C.c_void_p()
            _lib.check(_lib.lib().nce_ce_create(C.byref(self.host_tables.struct), C.byref(h)), "nce_ce_create")
            self._handle = h
        return self._handle

    def close(self):
        if self._handle is not None:
            _lib.lib().nce_ce_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ── encoding ──
    def encode(self, structure: Structure):
        """species index per site in canonical order (sigma_canon = sigma_orig[perm])."""
        from .lattice import site_decompose
        prim = self.cs.primitive
        basis, _, _, _ = site_decompose(prim.cell, prim.frac, structure.cell, structure.positions)
        return encode_species(self.cs, structure, basis)[self.perm]

    def check_errors(self):
        """Raise NceError if a kernel on this model flagged an error since the last check (and clear the flags)."""
        _lib.raise_device_errors(_lib.lib().nce_ce_errors, self.handle, _lib.CE_ERROR_FLAGS, "CE kernels")

    # ── energies ──
    def _sigma_dev(self, sigma):
        import torch
        if isinstance(sigma, torch.Tensor) and sigma.is_cuda and sigma.dtype == torch.int8:
            return sigma.reshape(-1, self.n_atoms).contiguous()      # already on the device: no round trip
        s = torch.as_tensor(np.asarray(sigma.cpu() if hasattr(sigma, "cpu") else sigma), dtype=torch.int8)
        return s.reshape(-1, self.n_atoms).contiguous().cuda()

    def batched_energy(self, sigma_batch, precision=64):
        import torch
        sd = sigma_batch if (hasattr(sigma_batch, "is_cuda") and sigma_batch.is_cuda and sigma_batch.dtype == torch.int8) \
            else self._sigma_dev(sigma_batch)
        sd = sd.reshape(-1, self.n_atoms).contiguous()
        R = sd.shape[0]
        E = torch.empty(R, dtype=torch.float64, device=sd.device)
        _lib.check(_lib.lib().nce_ce_energy(self.handle, sd.data_ptr(), R, precision, E.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_energy")
        return E

    @property
    def has_local_field(self):
        """True when the local-field kernel can run on this cell (+-1 point functions, no aliasing)."""
        ok = C.c_int32(0)
        _lib.check(_lib.lib().nce_ce_has_local_field(self.handle, C.byref(ok), None), "nce_ce_has_local_field")
        return bool(ok.value)

    @property
    def field_scale(self):
        """eV per unit of the local fields (2^-S of the fixed point)."""
        ok, sc = C.c_int32(0), C.c_double(0.0)
        _lib.check(_lib.lib().nce_ce_has_local_field(self.handle, C.byref(ok), C.byref(sc)), "nce_ce_has_local_field")
        return sc.value

    def field_init(self, sigma_batch, field=None):
        """Local fields (R, N) int64 of R configurations (``nce_ce_field_init``): G(i) = sum over the cluster instances
        containing site i of 2 eci Pi, fixed point x 2^S."""
        import torch
        sd = self._sigma_dev(sigma_batch)
        if field is None:
            field = torch.empty(sd.shape, dtype=torch.int64, device=sd.device)
        _lib.check(_lib.lib().nce_ce_field_init(self.handle, sd.data_ptr(), sd.shape[0], field.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_field_init")
        return field

    def cluster_counts(self, sigma_batch):
        """(R, n_cols) int64 cluster-vector sums of device configurations (point functions in {-1, +1})."""
        import torch
        sd = sigma_batch.reshape(-1, self.n_atoms).contiguous()
        cv = torch.empty((sd.shape[0], self.info["n_cols"]), dtype=torch.int64, device=sd.device)
        _lib.check(_lib.lib().nce_ce_cluster_counts(self.handle, sd.data_ptr(), sd.shape[0], cv.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_cluster_counts")
        return cv

    def energy_from_counts(self, cv):
        """float64 energies E = zerolet + sum_c eci_c cv[:, c]."""
        import torch
        E = torch.empty(cv.shape[0], dtype=torch.float64, device=cv.device)
        _lib.check(_lib.lib().nce_ce_energy_from_counts(self.handle, cv.data_ptr(), cv.shape[0], E.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_energy_from_counts")
        return E

    def energy(self, sigma, precision=64):
        return float(self.batched_energy(sigma, precision)[0].item())

    def energy_a(self, tp, sigma):
        return self.energy(sigma)

    def delta_energy_batch(self, sigma_batch, rep, ia, ib, sa_new, sb_new, precision=64, warps=8):
        """dE of independent swaps on device configurations sigma_batch (R, N)."""
        import torch
        dev = sigma_batch.device
        n = len(ia)
        rep = torch.as_tensor(np.asarray(rep), dtype=torch.int32, device=dev)
        ia = torch.as_tensor(np.asarray(ia), dtype=torch.int64, device=dev)
        ib = torch.as_tensor(np.asarray(ib), dtype=torch.int64, device=dev)
        sa = torch.as_tensor(np.asarray(sa_new), dtype=torch.int8, device=dev)
        sb = torch.as_tensor(np.asarray(sb_new), dtype=torch.int8, device=dev)
        out = torch.empty(n, dtype=torch.float64, device=dev)
        _lib.check(_lib.lib().nce_ce_delta(self.handle, sigma_batch.data_ptr(), sigma_batch.shape[0], n, rep.data_ptr(),
                                           ia.data_ptr(), ib.data_ptr(), sa.data_ptr(), sb.data_ptr(), precision, warps,
                                           out.data_ptr(), _lib.stream_ptr()), "nce_ce_delta")
        return out

    def delta_energy_a(self, tp, i_a, i_b, sigma, s_a_new, s_b_new, precision=64):
        """E(after sigma[i_a]=s_a_new, sigma[i_b]=s_b_new) - E(before) (``ce_gpu_implicit.py:181-191``)."""
        sd = self._sigma_dev(sigma)
        return float(self.delta_energy_batch(sd, [0], [int(i_a)], [int(i_b)], [int(s_a_new)], [int(s_b_new)], precision)[0].item())


def proposal_stream(gce_or_tables, R, n_steps, seed):
    """Seeded host proposal stream (numpy PCG64) in the engine's [step][slot] layout: for each step and slot a
    sublattice group chosen with probability proportional to its size, two uniform sites of that group and a
    uniform u in (0, 1] (``ce_gpu_implicit.py:194-211`` with numpy in place of jax.random)."""
    tb = gce_or_tables.info if hasattr(gce_or_tables, "info") else gce_or_tables
    rng = np.random.default_rng(seed)
    nB, n_cells = tb["nB"], tb["n_cells"]
    act_b, act_nb = tb["act_b"], tb["act_nb"]
    shape = (n_steps, R)
    if len(act_nb) == 1:
        g = np.zeros(shape, np.int64)
    else:
        g = rng.choice(len(act_nb), size=shape, p=act_nb / act_nb.sum())
    def draw():
        c = rng.integers(0, n_cells, size=shape)
        q = np.floor(rng.random(shape) * act_nb[g]).astype(np.int64)
        return (c * nB + act_b[g, q]).astype(np.int32)
    a = draw(); b = draw()
    u = 1.0 - rng.random(shape)
    return a, b, u
