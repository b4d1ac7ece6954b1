"""Parallel-tempering driver of the CE path on the GB300 engine.

Host-side mirror of ``neuralce/ce/pt_mcmc_ce.py``: ``MCMCConfig`` / ``MCMCResult`` (``:37-104,587-598``),
temperature ladders (``:223-260``), chunk / exchange-interval reconciliation (``:646-674``), equilibration then
production with the E_min reset (``:897-939``), checkpoint / resume with a run fingerprint (``:869-931``) and the
``energies.npz`` / ``mcmc_result.npz`` outputs (``:969-1018``).  Each chunk is one call of
``nce_ce_run_chunk``: the persistent CUDA kernel runs every step of every replica, then a one-CTA kernel
exchanges temperature slots on the device.  Random numbers are Philox4x32-10 keyed by ``cfg.seed`` and
counted by (global step, slot) -- a run resumed from a checkpoint is bit-identical to an uninterrupted one.
A host-supplied proposal stream can replace the device RNG (parity runs).
"""
from __future__ import annotations

import ctypes as C
import os
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import _lib

KB_EV_PER_K = 8.617333e-5


@dataclass
class MCMCConfig:
    ce_path: str = ''
    supercell_matrix: list = field(default_factory=list)
    T_min: float = 100.0
    T_max: float = 2000.0
    n_replicas: int = 64
    n_steps: int = 100000
    n_equilib: int = 10000
    sample_interval: int = 100
    exchange_interval: int = 10
    chunk_size: int = 1000
    spin_orbits_pkl: str = ''
    spin_states: dict = field(default_factory=dict)
    spin_move_prob: float = 0.0
    initial_composition: dict = field(default_factory=dict)
    swap_pairs: Optional[list] = None
    initial_sigma: Optional[np.ndarray] = None
    n_ladders: int = 1
    seed: int = 42
    output_dir: str = 'mcmc_results'
    energy_mode: str = 'delta'
    checkpoint_every: int = 0
    T_grid: Optional[np.ndarray] = None
    run_id: str = ''
    # engine options (not in the reference)
    precision: int = 64
    warps: int = 0
    cluster: int = 1                 # CTAs per replica (thread-block cluster, sign-parity path)
    reanchor_every: int = 0          # chunks between float64 full-energy re-anchors (0 = never, as the reference)


@dataclass
class MCMCResult:
    energies: np.ndarray
    temperatures: np.ndarray
    swap_accept_rate: float
    flip_accept_rate: float
    exchange_accept_rate: float
    sigma_final: np.ndarray
    sigma_min: np.ndarray
    E_min: float
    spins_final: Optional[np.ndarray]
    wall_time: float
    # steps whose Metropolis margin |dE + ln(u)/beta| was below the precision form's stated dE bound (a decision there
    # may differ from a float64 reference's); not in the reference's result
    near_threshold_steps: int = 0


def make_temperature_ladder(T_min, T_max, n_replicas):
    temps = np.array([T_min]) if n_replicas == 1 else np.geomspace(T_min, T_max, n_replicas)
    betas = 1.0 / (KB_EV_PER_K * temps)
    return temps.astype(np.float32), betas.astype(np.float32)


def build_interleaved_ladders(T_min, T_max, n_per_ladder, n_ladders):
    n_total = n_per_ladder * n_ladders
    tg = np.array([T_min], np.float64) if n_total == 1 else np.geomspace(T_min, T_max, n_total, dtype=np.float64)
    i = np.arange(n_total, dtype=np.int64)
    lid = (i // n_per_ladder).astype(np.int32); lpos = (i % n_per_ladder).astype(np.int32)
    temps = tg[lid.astype(np.int64) + lpos.astype(np.int64) * n_ladders].astype(np.float32)
    betas = (1.0 / (KB_EV_PER_K * temps)).astype(np.float32)
    return temps, betas, lid, lpos


class PTState:
    """Device state of one PT job (torch buffers) in the C-ABI layout."""

    def __init__(self, sigma, E, beta_slot, ladder_id, device="cuda"):
        import torch
        R, N = sigma.shape
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt).to(device)
        self.R, self.N = R, N
        self.sigma = t(sigma, torch.int8)
        self.E = t(E, torch.float64)
        self.beta_slot = t(beta_slot, torch.float32)
        self.rep_of_slot = torch.arange(R, dtype=torch.int32, device=device)
        self.slot_of_rep = torch.arange(R, dtype=torch.int32, device=device)
        self.ladder_id = t(ladder_id, torch.int32)
        Emr = np.full(R, np.inf); Emr[0] = float(np.asarray(E)[0])
        self.E_min_rep = t(Emr, torch.float64)
        self.n_acc = torch.zeros(R, dtype=torch.int64, device=device)
        self.n_ex = torch.zeros(1, dtype=torch.int64, device=device)
        self.n_near = torch.zeros(R, dtype=torch.int64, device=device)   # near-threshold steps (stated dE bound)
        self.field = None                                                  # local fields (enable_field)
        # chunk-end exchange inside the chunk kernel (the counter of replicas done); None: a separate exchange launch
        self.ex_sync = torch.zeros(1, dtype=torch.int32, device=device)
        self._min = torch.zeros(1, dtype=torch.float64, device=device)
        self._arg = torch.zeros(1, dtype=torch.int32, device=device)
        self.cv = None

    def track_counts(self, gce):
        """Keep the replicas' cluster-vector sums (exact integers, sign-parity tables) current from now on; the
        carried energies can then be re-anchored exactly with ``reanchor_from_counts``."""
        self.cv = gce.cluster_counts(self.sigma)
        return self

    def enable_field(self, gce):
        """Give the state its local fields (when the cell supports them): precision-64 chunks then run the local-field
        kernel, which keeps them current.  Call again after changing ``sigma`` by hand."""
        if gce.has_local_field:
            import torch
            if self.field is None or self.field.shape != self.sigma.shape:
                self.field = torch.empty(self.sigma.shape, dtype=torch.int64, device=self.sigma.device)
            gce.field_init(self.sigma, self.field)
        return self

    def reanchor_from_counts(self, gce):
        """float64 energies from the tracked sums; returns the largest change of a carried energy."""
        E = gce.energy_from_counts(self.cv)
        drift = float((E - self.E).abs().max().item())
        self.E.copy_(E)
        return drift

    def struct(self):
        s = _lib.NcePtState()
        s.R, s.N = self.R, self.N
        for f in ("sigma", "E", "beta_slot", "rep_of_slot", "slot_of_rep", "ladder_id", "E_min_rep", "n_acc", "n_ex", "n_near"):
            setattr(s, f, getattr(self, f).data_ptr())
        s.cv = self.cv.data_ptr() if self.cv is not None else None
        s.field = self.field.data_ptr() if self.field is not None else None
        s.ex_sync = self.ex_sync.data_ptr() if self.ex_sync is not None else None
        return s

    def minimum(self, stream=None):
        """(running minimum over replicas, argmin of the current energies) on the device."""
        st = self.struct()
        _lib.check(_lib.lib().nce_pt_minimum(C.byref(st), self._min.data_ptr(), self._arg.data_ptr(),
                                             _lib.stream_ptr(stream)), "nce_pt_minimum")
        return self._min, self._arg

    def reset_minimum(self, idx):
        import torch
        v = torch.full((self.R,), float("inf"), dtype=torch.float64, device=self.E.device)
        v[idx] = self.E[idx]
        self.E_min_rep.copy_(v)


def make_chunk(n_steps, step0, seed, precision=64, warps=0, proposals=None, sample_interval=1, E_samples=None,
               do_exchange=False, ex_parity=0, ex_u=None, path=0, cluster=1, near_eV=0.0):
    c = _lib.NcePtChunk()
    c.n_steps, c.step0, c.seed = int(n_steps), int(step0), int(seed) & 0xFFFFFFFFFFFFFFFF
    if proposals is not None:
        c.prop_a, c.prop_b, c.prop_u = (_lib.ptr(p) for p in proposals)
    c.sample_interval = int(sample_interval)
    c.E_samples = _lib.ptr(E_samples)
    c.do_exchange = int(bool(do_exchange)); c.ex_parity = int(ex_parity); c.ex_u = _lib.ptr(ex_u)
    c.precision = int(precision); c.warps = int(warps); c.path = int(path); c.cluster = int(cluster)
    c.near_eV = float(near_eV)
    return c


def run_chunk(gce, st: PTState, n_steps, step0, seed, precision=64, warps=0, proposals=None, sample_interval=1,
              E_samples=None, do_exchange=False, ex_parity=0, ex_u=None, stream=None, path=0, cluster=1, near_eV=0.0):
    """One chunk of the persistent kernel (+ chunk-end exchange) for one job.  path: 0 auto (local field when the state
    has fields, else sign parity when the point functions are +-1), 1 general products, 2 sign parity, 3 local field.
    ``st.n_near`` counts the steps whose Metropolis margin |dE + ln(u) / beta| is below ``near_eV`` (0: the precision form's stated dE bound)."""
    ck = make_chunk(n_steps, step0, seed, precision, warps, proposals, sample_interval, E_samples, do_exchange,
                    ex_parity, ex_u, path, cluster, near_eV)
    s = st.struct()
    _lib.check(_lib.lib().nce_ce_run_chunk(gce.handle, C.byref(s), C.byref(ck), _lib.stream_ptr(stream)),
               "nce_ce_run_chunk")


def initial_state(gce, n_replicas, composition, seed):
    """Random configurations per replica at the given composition per sublattice (``pt_mcmc_ce.py:266-308``
    with numpy's PCG64 seeded by ``seed`` in place of the jax key)."""
    rng = np.random.default_rng(seed)
    N = gce.n_atoms
    tmpl = np.zeros(N, np.int8)
    for sl in gce.sublattices:
        idx = np.asarray(sl["indices"]); n = len(idx); ns = sl["n_species"]
        fr = composition.get(sl["name"]) if composition else None
        if fr is None:
            fr = [1.0 / ns] * ns
        elif not isinstance(fr, (list, tuple)):
            fr = [1.0 - fr, fr]
        cnt = np.round(np.asarray(fr) * n).astype(int); cnt[0] += n - cnt.sum()
        arr = np.concatenate([np.full(c, k, np.int8) for k, c in enumerate(cnt)])
        rng.shuffle(arr); tmpl[idx] = arr
    out = np.tile(tmpl, (n_replicas, 1))
    for r in range(n_replicas):
        for sl in gce.sublattices:
            idx = np.asarray(sl["indices"]); sub = out[r, idx].copy(); rng.shuffle(sub); out[r, idx] = sub
    return out


def run_pt_mcmc(gce, cfg: MCMCConfig, verbose=True):
    """Run PT-MCMC on the GPU; same outputs and files as the reference."""
    import torch
    log = print if verbose else (lambda *a, **k: None)
    os.makedirs(cfg.output_dir, exist_ok=True)
    if cfg.energy_mode != "delta":
        raise ValueError("this engine implements the delta (local) energy mode only")
    if cfg.spin_orbits_pkl or cfg.spin_states:
        raise ValueError("spin cluster expansions are not on this engine's path (delta mode is compositional only)")
    n_ladders = max(int(cfg.n_ladders), 1)
    n_per = int(cfg.n_replicas); n_total = n_per * n_ladders
    if cfg.T_grid is not None:
        if n_ladders != 1:
            raise ValueError("cfg.T_grid is one ladder; n_ladders must be 1")
        tg = np.asarray(cfg.T_grid, np.float64).reshape(-1)
        n_per = n_total = len(tg)
        temps = tg.astype(np.float32); betas = (1.0 / (KB_EV_PER_K * tg)).astype(np.float32)
        lid = np.zeros(n_total, np.int32); lpos = np.arange(n_total, dtype=np.int32)
    elif n_ladders == 1:
        temps, betas = make_temperature_ladder(cfg.T_min, cfg.T_max, n_per)
        lid = np.zeros(n_per, np.int32); lpos = np.arange(n_per, dtype=np.int32)
    else:
        temps, betas, lid, lpos = build_interleaved_ladders(cfg.T_min, cfg.T_max, n_per, n_ladders)
    chunk = int(cfg.chunk_size); si = int(cfg.sample_interval); ex_int = int(cfg.exchange_interval)
    if ex_int <= 0:                   # independent chains (single-T / multi-T runs): no exchange
        ex_int = 0
    elif n_total > 1 and ex_int % chunk != 0:
        import math
        if ex_int < chunk:
            chunk = ex_int
            if chunk % si != 0:
                si = math.gcd(chunk, si)
            log(f"  chunk_size -> {chunk} (= exchange interval); sample_interval {si}", flush=True)
        else:
            ex_int = int(round(ex_int / chunk)) * chunk
            log(f"  exchange_interval -> {ex_int} (whole chunks of {chunk})", flush=True)
    n_prod = cfg.n_steps - cfg.n_equilib
    if cfg.n_equilib % chunk != 0:
        raise ValueError(f"n_equilib ({cfg.n_equilib}) must be a multiple of chunk_size ({chunk})")
    if n_prod % chunk != 0:
        raise ValueError(f"(n_steps - n_equilib) = {n_prod} must be a multiple of chunk_size ({chunk})")
    if chunk % si != 0:
        raise ValueError(f"chunk_size ({chunk}) must be a multiple of sample_interval ({si})")
    if cfg.swap_pairs:
        sets = [set(sl["chemical_symbols"]) for sl in gce.sublattices]
        bad = [(a, b) for (a, b) in cfg.swap_pairs if not any({a, b} <= s for s in sets)]
        if bad:
            raise ValueError(f"swap_pairs {bad} do not lie within any single sublattice")
    log(f"PT-MCMC: {n_total} replicas, T=[{temps.min():.0f}, {temps.max():.0f}] K, n_steps={cfg.n_steps:,}, "
        f"n_equilib={cfg.n_equilib:,}, chunk={chunk}, exchange_interval={ex_int}, sample_interval={si}, "
        f"precision=fp{cfg.precision}", flush=True)
    # initial configurations
    if cfg.initial_sigma is not None:
        s0 = np.asarray(cfg.initial_sigma, np.int8)
        if s0.shape == (gce.n_atoms,):
            sig0 = np.broadcast_to(s0, (n_total, gce.n_atoms)).copy()
        elif s0.shape == (n_total, gce.n_atoms):
            sig0 = s0.copy()
        else:
            raise ValueError(f"initial_sigma shape {s0.shape} must be ({gce.n_atoms},) or ({n_total}, {gce.n_atoms})")
    else:
        sig0 = initial_state(gce, n_total, cfg.initial_composition, cfg.seed)
    sig_dev = torch.as_tensor(sig0, dtype=torch.int8).cuda()
    E0 = gce.batched_energy(sig_dev).cpu().numpy()
    st = PTState(sig0, E0, betas, lid)
    sigma_min = st.sigma[0].clone(); E_min = float(E0[0])
    n_eq = cfg.n_equilib // chunk; n_pc = n_prod // chunk; spc = chunk // si
    energy_samples = np.zeros((n_pc * spc, n_total), np.float64)
    Es_dev = torch.zeros((spc, n_total), dtype=torch.float64, device="cuda")
    si_ = 0; c0 = 0; step = 0
    ck_every = int(cfg.checkpoint_every or 0); ck_path = os.path.join(cfg.output_dir, "checkpoint.npz")
    if ck_every and os.path.exists(ck_path):
        ck = np.load(ck_path)
        want = dict(n_steps=cfg.n_steps, chunk=chunk, n_total=n_total, n_atoms=gce.n_atoms, sample_interval=si,
                    seed=cfg.seed, precision=cfg.precision)
        have = {k: int(ck["cfg_" + k]) for k in want}
        want["run_id"] = str(cfg.run_id or ""); have["run_id"] = str(ck["cfg_run_id"])
        if not np.allclose(ck["cfg_temps"], temps, rtol=0, atol=1e-6):
            have["temps"] = "differ"; want["temps"] = "same"
        if have != want:
            raise RuntimeError(f"{ck_path} was written by another run (it records {have}, this run is {want}); remove the "
                               "file or choose another output directory")
        c0 = int(ck["chunk"]); si_ = int(ck["si"]); energy_samples[:si_] = ck["energy_samples"]; step = int(ck["step"])
        st.sigma.copy_(torch.as_tensor(ck["sigma"]).cuda()); st.E.copy_(torch.as_tensor(ck["E"]).cuda())
        st.rep_of_slot.copy_(torch.as_tensor(ck["rep_of_slot"]).cuda()); st.slot_of_rep.copy_(torch.as_tensor(ck["slot_of_rep"]).cuda())
        st.E_min_rep.copy_(torch.as_tensor(ck["E_min_rep"]).cuda()); st.n_acc.copy_(torch.as_tensor(ck["n_acc"]).cuda())
        st.n_ex.copy_(torch.as_tensor(ck["n_ex"]).cuda())
        sigma_min = torch.as_tensor(ck["sigma_min"]).cuda(); E_min = float(ck["E_min"])
        log(f"  resumed from {ck_path}: production chunk {c0}/{n_pc}, {si_} samples", flush=True)
    t0 = time.time()

    def one_chunk(record):
        nonlocal step, sigma_min, E_min
        do_ex = n_total > 1 and ex_int > 0 and (step + chunk) % ex_int == 0
        E_before = E_min
        run_chunk(gce, st, chunk, step, cfg.seed, cfg.precision, cfg.warps, None, si, Es_dev if record else None,
                  do_ex, cluster=cfg.cluster)
        step += chunk
        mn, arg = st.minimum()
        m = float(mn.item())
        if m < E_before:
            E_min = m
            sigma_min = st.sigma[int(arg.item())].clone()
        if cfg.reanchor_every and (step // chunk) % cfg.reanchor_every == 0:
            st.E.copy_(gce.batched_energy(st.sigma))

    if c0 == 0:
        for c in range(n_eq):
            one_chunk(False)
        if n_eq > 0:
            idx0 = int(torch.argmin(st.E).item())
            sigma_min = st.sigma[idx0].clone(); E_min = float(st.E[idx0].item()); st.reset_minimum(idx0)
            log("  -> equilibration complete; reset E_min for production.", flush=True)
    for c in range(c0, n_pc):
        one_chunk(True)
        energy_samples[si_:si_ + spc] = Es_dev.cpu().numpy(); si_ += spc
        if ck_every and (c + 1) % ck_every == 0 and c + 1 < n_pc:
            np.savez(ck_path + ".tmp.npz", chunk=c + 1, si=si_, step=step, energy_samples=energy_samples[:si_],
                     sigma=st.sigma.cpu().numpy(), E=st.E.cpu().numpy(), rep_of_slot=st.rep_of_slot.cpu().numpy(),
                     slot_of_rep=st.slot_of_rep.cpu().numpy(), E_min_rep=st.E_min_rep.cpu().numpy(),
                     n_acc=st.n_acc.cpu().numpy(), n_ex=st.n_ex.cpu().numpy(), sigma_min=sigma_min.cpu().numpy(),
                     E_min=E_min, cfg_n_steps=cfg.n_steps, cfg_chunk=chunk, cfg_n_total=n_total,
                     cfg_n_atoms=gce.n_atoms, cfg_sample_interval=si, cfg_seed=cfg.seed, cfg_precision=cfg.precision,
                     cfg_temps=temps, cfg_run_id=str(cfg.run_id or ""))
            os.replace(ck_path + ".tmp.npz", ck_path)
    torch.cuda.synchronize()
    gce.check_errors()                                    # device error flags raise here, as the reference's errors
    wall = time.time() - t0
    n_sw = cfg.n_steps * n_total
    pairs = (n_per // 2) * n_ladders
    n_ex_att = (cfg.n_steps // ex_int) * pairs if ex_int else 0
    swap_rate = float(st.n_acc.sum().item()) / max(1, n_sw)
    ex_rate = float(st.n_ex.item()) / max(1, n_ex_att)
    log(f"\nDone in {wall:.1f}s  ({n_sw / max(wall, 1e-9):,.0f} swap attempts/s)\n  swap acceptance     : {swap_rate:.4f}\n"
        f"  exchange acceptance : {ex_rate:.4f}\n  E_min (production)  : {E_min:.4f}\n"
        f"  near-threshold steps: {int(st.n_near.sum().item())}", flush=True)
    np.savez(os.path.join(cfg.output_dir, "energies.npz"), energies=energy_samples[:si_], temperatures=temps,
             ladder_id=lid, n_atoms=np.int32(gce.n_atoms), swap_accept_rate=swap_rate, exchange_accept_rate=ex_rate,
             flip_accept_rate=0.0, E_min=E_min, wall_time=wall)
    ros = st.rep_of_slot.cpu().numpy()
    sigma_final = st.sigma.cpu().numpy()[ros][:, gce.inv_perm]
    smin = sigma_min.cpu().numpy()[gce.inv_perm]
    res = MCMCResult(energies=energy_samples[:si_], temperatures=temps.astype(np.float32), swap_accept_rate=swap_rate,
                     flip_accept_rate=0.0, exchange_accept_rate=ex_rate, sigma_final=sigma_final, sigma_min=smin,
                     E_min=E_min, spins_final=None, wall_time=wall, near_threshold_steps=int(st.n_near.sum().item()))
    np.savez(os.path.join(cfg.output_dir, "mcmc_result.npz"), energies=res.energies, temperatures=res.temperatures,
             ladder_id=lid, ladder_pos=lpos, n_ladders=np.int32(n_ladders), sigma_final=res.sigma_final,
             sigma_min=res.sigma_min, E_min=res.E_min, spins_final=np.array([]), swap_accept_rate=swap_rate,
             flip_accept_rate=0.0, exchange_accept_rate=ex_rate, wall_time=wall)
    if ck_every and os.path.exists(ck_path):
        os.remove(ck_path)
    return res
