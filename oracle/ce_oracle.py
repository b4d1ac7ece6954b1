"""CPU oracle for the cluster-expansion PT path -- TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs of ``bench.py``
may import this module.  It checks the product path and is never part of it.

Two independent restatements of the reference, both in float64:

* ``energy_explicit`` -- total energy from an explicit enumeration of every cluster instance of the
  supercell (the role of the reference's tiled tables, ``neuralce/ce/ce_gpu_tiled.py:20-105``, and of
  icet's ``ClusterExpansion.predict``): E = zerolet + sum_k eci_k * scale * <prod theta>_k.
* ``energy_implicit`` / ``delta_implicit`` -- literal restatements of ``energy_a`` and ``delta_energy_a``
  (``neuralce/ce/ce_gpu_implicit.py:147-191``) on the implicit tables, including the reference's handling of
  rows of i_b that also contain i_a.

The compiled C restatement of the same delta path plus the Metropolis step and slot exchange
(``oracle/ce_oracle.c``) is loaded by ``load_c_oracle``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def energy_explicit(cs, parameters, structure, energy_scale=1.0):
    """Total CE energy of ``structure`` by enumerating every cluster instance of every orbit in every
    primitive cell of the supercell (float64)."""
    from neuralce_gb300.lattice import site_decompose, theta
    from neuralce_gb300.ce_tables import encode_species
    prim = cs.primitive
    basis, off, T, n_cells = site_decompose(prim.cell, prim.frac, structure.cell, structure.positions)
    sig = encode_species(cs, structure, basis).astype(np.int64)
    Tinv = np.linalg.inv(T)
    lookup = {}
    for i in range(len(structure)):
        lookup[(int(basis[i]),) + tuple(int(x) for x in off[i])] = i
    cells = np.unique(off, axis=0)
    assert len(cells) == n_cells

    def site(b, n):
        n = np.asarray(n, np.int64)
        nr = n - np.floor(n @ Tinv + 1e-9).astype(np.int64) @ T
        return lookup[(int(b),) + tuple(int(x) for x in nr)]
    params = np.asarray(parameters, np.float64) * float(energy_scale)
    E = params[0]
    for k, o in enumerate(cs.orbits):
        acc = 0.0
        for inst in o.clusters:
            for c in cells:
                pr = 1.0
                for (b, n) in inst:
                    i = site(b, c + np.asarray(n))
                    pr *= theta(len(prim.species[b]), 0, sig[i])
                acc += pr
        E += params[k + 1] * acc / (len(o.clusters) * n_cells)
    return float(E)


def _site(tb, b, k):
    d = tb["d"]
    return ((k[..., 0] * d[1] + k[..., 1]) * d[2] + k[..., 2]) * tb["nB"] + b


def _k_of(tb, i):
    d = tb["d"]; nB = tb["nB"]; c = i // nB
    return i % nB, np.stack([c // (d[1] * d[2]), (c // d[2]) % d[1], c % d[2]], axis=-1)


def energy_implicit(tb, sigma):
    """energy_a restated: zerolet + sum over cells and template rows of eci * prod pf (float64)."""
    sigma = np.asarray(sigma, np.int64)
    n_cells = tb["n_cells"]; d = tb["d"]
    c = np.arange(n_cells)
    k = np.stack([c // (d[1] * d[2]), (c // d[2]) % d[1], c % d[2]], axis=-1)
    tot = 0.0
    for r in range(tb["Rt"]):
        kk = (k[:, None, :] + tb["T_uo"][r][None]) % d
        sites = _site(tb, tb["T_b"][r][None], kk)
        pr = np.prod(tb["pf"][tb["T_st"][r][None], tb["T_bf"][r][None], sigma[sites]], axis=-1)
        tot += tb["T_eci"][r] * pr.sum()
    return tb["zerolet"] + tot


def delta_implicit(tb, sigma, i_a, i_b, s_a_new, s_b_new):
    """delta_energy_a restated (float64): rows of i_a, plus rows of i_b that do not contain i_a."""
    sigma = np.asarray(sigma, np.int64)

    def entries(i):
        b, k = _k_of(tb, i)
        kk = (k[None, None, :] + tb["Rv_uo"][b]) % tb["d"]
        return _site(tb, tb["Rv_b"][b], kk), tb["Rv_st"][b], tb["Rv_bf"][b], tb["Rv_eci"][b]

    def species(sites):
        sp = sigma[sites].copy()
        sp = np.where(sites == i_a, s_a_new, sp)
        sp = np.where(sites == i_b, s_b_new, sp)
        return sp
    pf = tb["pf"]
    sa, st_a, bf_a, ec_a = entries(i_a)
    da = ec_a * (np.prod(pf[st_a, bf_a, species(sa)], -1) - np.prod(pf[st_a, bf_a, sigma[sa]], -1))
    sb, st_b, bf_b, ec_b = entries(i_b)
    db = ec_b * (np.prod(pf[st_b, bf_b, species(sb)], -1) - np.prod(pf[st_b, bf_b, sigma[sb]], -1))
    both = np.any(sb == i_a, axis=1)
    return float(np.sum(da) + np.sum(np.where(both, 0.0, db)))


# ───────────────────────────── compiled C oracle ───────────────────────────────────────────────

_vp = ctypes.c_void_p
_i32, _i64, _u64, _f64 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_double


class OrcTables(ctypes.Structure):
    _fields_ = [("nB", _i32), ("J", _i32), ("mo", _i32), ("Rt", _i32), ("n_bf", _i32), ("max_sp", _i32),
                ("d", _i64 * 3), ("n_cells", _i64), ("zerolet", _f64),
                ("Rv_b", _vp), ("Rv_uo", _vp), ("Rv_st", _vp), ("Rv_bf", _vp), ("Rv_eci", _vp),
                ("T_b", _vp), ("T_uo", _vp), ("T_st", _vp), ("T_bf", _vp), ("T_eci", _vp), ("pf", _vp),
                ("n_groups", _i32), ("max_gb", _i32), ("act_b", _vp), ("act_nb", _vp), ("grp_cum", _vp)]


class OrcState(ctypes.Structure):
    _fields_ = [("R", _i32), ("N", _i64), ("sigma", _vp), ("E", _vp), ("beta_slot", _vp), ("rep_of_slot", _vp),
                ("slot_of_rep", _vp), ("ladder_id", _vp), ("E_min_rep", _vp), ("n_acc", _vp), ("n_ex", _vp),
                ("n_near", _vp)]


class OrcChunk(ctypes.Structure):
    _fields_ = [("n_steps", _i64), ("step0", _i64), ("prop_a", _vp), ("prop_b", _vp), ("prop_u", _vp), ("seed", _u64),
                ("sample_interval", _i64), ("E_samples", _vp), ("do_exchange", _i32), ("ex_parity", _i32),
                ("ex_u", _vp), ("n_threads", _i32), ("rounds", _i32), ("near_eV", _f64)]


def _p(a):
    return None if a is None else a.ctypes.data


class _COracle:
    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        L = self.lib
        L.orc_ce_energy.restype = _f64
        L.orc_ce_energy.argtypes = [ctypes.POINTER(OrcTables), _vp]
        L.orc_ce_delta.restype = _f64
        L.orc_ce_delta.argtypes = [ctypes.POINTER(OrcTables), _vp, _i64, _i64, _i32, _i32]
        L.orc_ce_run.restype = ctypes.c_int
        L.orc_ce_run.argtypes = [ctypes.POINTER(OrcTables), ctypes.POINTER(OrcState), ctypes.POINTER(OrcChunk)]
        L.orc_philox4x32.restype = None
        L.orc_philox4x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3

    def philox(self, ctr, key):
        c = (ctypes.c_uint32 * 4)(*ctr); k = (ctypes.c_uint32 * 2)(*key); o = (ctypes.c_uint32 * 4)()
        self.lib.orc_philox4x32(c, k, o)
        return [int(x) for x in o]


class OracleCE:
    """C oracle bound to one set of implicit tables (reference layout)."""

    def __init__(self, tb):
        self.c = load_c_oracle()
        self.tb = tb
        a = lambda x, dt: np.ascontiguousarray(np.asarray(x, dt))
        self.keep = dict(Rv_b=a(tb["Rv_b"], np.int32), Rv_uo=a(tb["Rv_uo"], np.int32), Rv_st=a(tb["Rv_st"], np.int32),
                         Rv_bf=a(tb["Rv_bf"], np.int32), Rv_eci=a(tb["Rv_eci"], np.float64), T_b=a(tb["T_b"], np.int32),
                         T_uo=a(tb["T_uo"], np.int32), T_st=a(tb["T_st"], np.int32), T_bf=a(tb["T_bf"], np.int32),
                         T_eci=a(tb["T_eci"], np.float64), pf=a(tb["pf"], np.float64), act_b=a(tb["act_b"], np.int32),
                         act_nb=a(tb["act_nb"], np.int32))
        w = self.keep["act_nb"].astype(np.float64)
        g = np.floor(np.cumsum(w) / w.sum() * 2.0 ** 32).astype(np.uint64); g[-1] = np.uint64(2 ** 32)
        self.keep["grp_cum"] = np.ascontiguousarray(g)
        s = OrcTables()
        s.nB, s.J, s.mo, s.Rt = tb["nB"], tb["J"], tb["mo"], tb["Rt"]
        s.n_bf, s.max_sp = tb["pf"].shape[1], tb["pf"].shape[2]
        for i in range(3):
            s.d[i] = int(tb["d"][i])
        s.n_cells = int(tb["n_cells"]); s.zerolet = float(tb["zerolet"])
        for k, v in self.keep.items():
            setattr(s, k, v.ctypes.data)
        s.n_groups, s.max_gb = self.keep["act_b"].shape
        self.s = s

    def energy(self, sigma):
        sig = np.ascontiguousarray(sigma, np.int8)
        return self.c.lib.orc_ce_energy(ctypes.byref(self.s), sig.ctypes.data)

    def delta(self, sigma, ia, ib, sa_new, sb_new):
        sig = np.ascontiguousarray(sigma, np.int8)
        return self.c.lib.orc_ce_delta(ctypes.byref(self.s), sig.ctypes.data, int(ia), int(ib), int(sa_new), int(sb_new))

    def run(self, state, n_steps, step0, seed=0, proposals=None, sample_interval=1, E_samples=None, do_exchange=False,
            ex_parity=0, ex_u=None, n_threads=1, rounds=1, near_eV=0.0):
        """run one chunk in place on the numpy arrays of ``state`` (dict: sigma, E, beta_slot, rep_of_slot,
        slot_of_rep, ladder_id, E_min_rep, n_acc, n_ex, optional n_near).  ``rounds`` exchange rounds at the chunk
        end (host uniforms: ex_u (rounds, ceil((R-1)/2)), parity bit q of ex_parity); ``state["n_near"]`` (when
        present) counts the steps with |dE + ln(u) / beta| < near_eV."""
        st = OrcState()
        st.R, st.N = state["sigma"].shape
        for k in ("sigma", "E", "beta_slot", "rep_of_slot", "slot_of_rep", "ladder_id", "E_min_rep", "n_acc", "n_ex"):
            setattr(st, k, state[k].ctypes.data)
        st.n_near = state["n_near"].ctypes.data if "n_near" in state else None
        ck = OrcChunk()
        ck.n_steps, ck.step0, ck.seed = int(n_steps), int(step0), int(seed) & 0xFFFFFFFFFFFFFFFF
        if proposals is not None:
            pa, pb, pu = (np.ascontiguousarray(x) for x in proposals)
            proposals = (pa, pb, pu)
            ck.prop_a, ck.prop_b, ck.prop_u = pa.ctypes.data, pb.ctypes.data, pu.ctypes.data
        ck.sample_interval = int(sample_interval); ck.E_samples = _p(E_samples)
        ck.do_exchange = int(bool(do_exchange)); ck.ex_parity = int(ex_parity); ck.ex_u = _p(ex_u)
        ck.n_threads = int(n_threads); ck.rounds = int(rounds); ck.near_eV = float(near_eV)
        self.c.lib.orc_ce_run(ctypes.byref(self.s), ctypes.byref(st), ctypes.byref(ck))


def new_state(sigma, E, beta_slot, ladder_id=None):
    """numpy PT state for the C oracle (same layout as the engine's)."""
    R = sigma.shape[0]
    Emr = np.full(R, np.inf); Emr[0] = E[0]
    return dict(sigma=np.ascontiguousarray(sigma, np.int8).copy(), E=np.ascontiguousarray(E, np.float64).copy(),
                beta_slot=np.ascontiguousarray(beta_slot, np.float32), rep_of_slot=np.arange(R, dtype=np.int32),
                slot_of_rep=np.arange(R, dtype=np.int32),
                ladder_id=np.zeros(R, np.int32) if ladder_id is None else np.ascontiguousarray(ladder_id, np.int32),
                E_min_rep=Emr, n_acc=np.zeros(R, np.int64), n_ex=np.zeros(1, np.int64), n_near=np.zeros(R, np.int64))


def c_oracle_path():
    return os.path.join(HERE, "_build", "libce_oracle.so")


def build_c_oracle(force=False):
    """Compile oracle/ce_oracle.c into oracle/_build/libce_oracle.so with gcc."""
    import subprocess
    out = c_oracle_path()
    src = os.path.join(HERE, "ce_oracle.c")
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11", src, "-o", out, "-lm"])
    return out


_C = None


def load_c_oracle():
    global _C
    if _C is None:
        _C = _COracle(build_c_oracle())
    return _C
