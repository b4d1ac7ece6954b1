"""NeuralCE ("nce" framework) drivers of the command line, after ``neuralce/nce/mcmc.py:24-475``.

``_run_replicas`` is the reference's generic driver: R replicas, one chunk of ``chunk`` steps per launch
(``nce_nce_run_chunk``), the full caches and carried energies rebuilt every ``anchor_every`` chunks (default
ceil(N / chunk)) with the drift logged, PT exchange rounds every ``exchange_every`` steps.  Exchanges permute
temperature slots on the device instead of moving configurations; every output here is reported per temperature
(slot order), as the reference's are.  Outputs: ``energies.npz`` (E_chunk, acc_chunk, drift, drift_eV, traj,
betas, temps), ``final_sigma.npy`` (input atom order), ``final_T*_r*.cif``, ``checkpoint.npz`` while running.
"""
from __future__ import annotations

import hashlib
import os
import time

import numpy as np

from ..ce_tables import encode_species
from ..io import Z_OF, Structure, load_model, read_cif, write_cif
from ..lattice import site_decompose

KB = 8.617333262e-5


def _log(*a):
    print(*a, flush=True)


def _prepare(model_path, init_cif, supercell=(1, 1, 1), seed_idx=0, dtype="float32", seed=0):
    from ..nce import setup
    mdl = load_model(model_path) if isinstance(model_path, str) else model_path
    if int(mdl.get("spin", 0) or 0):
        raise NotImplementedError("spin models are not on this engine's path")
    atoms = read_cif(init_cif) if isinstance(init_cif, str) else init_cif
    prim = mdl["primitive"]
    site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)          # ideal lattice of the model primitive
    sc = tuple(int(x) for x in supercell)
    if sc != (1, 1, 1):
        atoms = atoms.repeat(sc)
        if os.environ.get("CE_CNN_SUPERCELL_PERIODIC", "0") != "1":
            basis, _, _, _ = site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)
            rng = np.random.default_rng(seed)
            Z = atoms.numbers.copy()
            keys = [tuple(sp) for sp in prim.species]
            for key in dict.fromkeys(keys):
                m = np.isin(basis, [b for b, k in enumerate(keys) if k == key])
                Z[m] = rng.permutation(Z[m])
            atoms.numbers = Z
            _log(f"[nce] cif repeated {sc}: {len(atoms)} sites; each sublattice's species permuted at random (seed {seed})")
        else:
            _log(f"[nce] cif repeated {sc}: {len(atoms)} sites, the ordered copies left as they are")
    t0 = time.time()
    mc = setup(mdl, atoms, seed_idx=seed_idx, dtype=dtype)
    mc["mdl"], mc["atoms"] = mdl, atoms
    _log(f"[nce] network of {mc['depth']} layer(s) on {mc['n_atoms']} sites ({mc['n_active']} swappable); set up in "
         f"{time.time() - t0:.1f} s; starting energy {mc['energy'](mc['sig0']):.6f} eV/atom")
    return mc


def _fingerprint(mc, sig):
    h = hashlib.md5()
    P = mc["P"]
    for lay in P["layers"]:
        for k in sorted(lay):
            v = lay[k]
            if v is not None:
                h.update(np.ascontiguousarray(np.asarray(v, np.float64)).tobytes())
    h.update(np.ascontiguousarray(np.asarray(sig), dtype=np.int32).tobytes())
    return h.hexdigest()[:16]


def _init_sig_from_npz(mc, path, temps, R):
    from .init_structures import load_init_npz
    model, atoms = mc["model"], mc["atoms"]
    nums, _ = load_init_npz(path, atoms, temps)
    if nums.shape[0] != R:
        raise ValueError(f"init_npz has {nums.shape[0]} structures for {R} replicas")
    prim = mc["mdl"]["primitive"]
    basis, _, _, _ = site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)
    return np.stack([encode_species(mc["cs"], Structure(atoms.cell, atoms.positions, nums[r].astype(np.int64)), basis)
                     [model.perm] for r in range(R)]).astype(np.int8)


def _write_cifs(mc, sig_in, temps, out_dir):
    """final_T{T}_r{r}.cif per temperature; sig_in in input atom order."""
    atoms = mc["atoms"]; prim = mc["mdl"]["primitive"]
    basis, _, _, _ = site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)
    lut = [np.array([Z_OF[s] for s in prim.species[b]], np.int64) for b in range(len(prim.species))]
    for r in range(sig_in.shape[0]):
        Z = atoms.numbers.copy()
        for b, zs in enumerate(lut):
            m = basis == b
            if len(zs) > 1:
                Z[m] = zs[sig_in[r, m].astype(np.int64)]
        write_cif(os.path.join(out_dir, f"final_T{temps[r]:.0f}_r{r}.cif"), Structure(atoms.cell, atoms.positions, Z))


def _run_replicas(mc, betas, n_steps, seed, chunk, log_every, sample_interval, out_dir, tag, exchange_every=0,
                  anchor_every=None, init_npz=None, checkpoint_every=0, cluster=1):
    import torch

    model = mc["model"]
    R = len(betas); betas = np.asarray(betas, np.float32)
    temps = 1.0 / (KB * betas.astype(np.float64))
    N = mc["n_atoms"]
    if init_npz:
        sig = _init_sig_from_npz(mc, init_npz, temps, R)
        _log(f"[{tag}] starting structures read from {init_npz}, one per temperature (sites paired by position)")
    else:
        sig = np.stack([model.sig0] * R).astype(np.int8)
    n_chunks = max(n_steps // chunk, 1)
    if anchor_every is None:
        anchor_every = max(1, int(np.ceil(N / chunk)))
    si = max(1, min(int(sample_interval), chunk))
    rounds = max(chunk // exchange_every, 1) if (exchange_every > 0 and R > 1) else 0
    ys, ym = mc["ys"], mc["ym"]
    E_chunk, acc_chunk, drift_log, traj = [], [], [], []
    drift = 0.0
    ck_every = int(checkpoint_every or 0); ck_path = os.path.join(out_dir, "checkpoint.npz"); c0 = 0
    st = mc["new_state"](sig, betas)                    # one model, or the ensemble of every trained seed
    want = None
    if ck_every:
        ck_every = int(np.ceil(ck_every / anchor_every)) * anchor_every
        want = dict(n_steps=int(n_steps), chunk=int(chunk), R=int(R), n_atoms=int(N), sample_interval=int(si),
                    seed=int(seed), anchor_every=int(anchor_every), exchange_every=int(exchange_every))
        ints = list(want)
        want["model"] = _fingerprint(mc, sig)
        if os.path.exists(ck_path):
            ck = np.load(ck_path)
            have = {k: int(ck["cfg_" + k]) for k in ints}; have["model"] = str(ck["cfg_model"])
            same_T = np.allclose(np.asarray(ck["cfg_betas"], np.float64), betas.astype(np.float64), rtol=0, atol=1e-6)
            if have != want or not same_T:
                raise RuntimeError(f"{ck_path} was written by another run (it records {have}, this run is {want}, "
                                   f"ladder unchanged: {same_T}); remove the file or choose another output directory")
            c0 = int(ck["chunk"]); drift = float(ck["drift"])
            st.sigma.copy_(torch.as_tensor(ck["sig"]).cuda())
            st.rep_of_slot.copy_(torch.as_tensor(ck["rep_of_slot"]).cuda())
            st.slot_of_rep.copy_(torch.as_tensor(ck["slot_of_rep"]).cuda())
            st.n_acc.copy_(torch.as_tensor(ck["n_acc"]).cuda()); st.n_ex.copy_(torch.as_tensor(ck["n_ex"]).cuda())
            E_chunk = list(ck["E_chunk"]); acc_chunk = list(ck["acc_chunk"]); drift_log = [float(x) for x in ck["drift_log"]]
            traj = [np.asarray(ck["traj"])] if ck["traj"].shape[1] else []
            if hasattr(st, "broadcast"):
                st.broadcast()
            _log(f"[{tag}] resumed from {ck_path}: chunk {c0}/{n_chunks}")
    st.full_cache()
    _log(f"[{tag}] {R} replicas, {n_chunks} chunks of {chunk} steps; full re-anchor every {anchor_every} chunk(s)"
         + (f"; checkpoint every {ck_every} chunks" if ck_every else ""))
    Es = torch.zeros((chunk // si, R), dtype=torch.float64, device="cuda")
    n_acc_prev = st.n_acc.clone()
    t0 = time.time()
    for c in range(c0, n_chunks):
        st.run_chunk(chunk, c * chunk, seed=seed, sample_interval=si, E_samples=Es, exchange_rounds=rounds, cluster=cluster)
        if (c + 1) % anchor_every == 0 or c == n_chunks - 1:
            E_car = st.E.clone()
            st.full_cache()
            drift = float((st.E - E_car).abs().max().item())
        ros = st.rep_of_slot.long()
        E_eV = (st.E[ros].cpu().numpy() * ys + ym)
        nacc = (st.n_acc - n_acc_prev)[ros].cpu().numpy(); n_acc_prev = st.n_acc.clone()
        E_chunk.append(E_eV); acc_chunk.append(nacc / chunk); drift_log.append(drift)
        traj.append(Es.cpu().numpy().T * ys + ym)
        if log_every and ((c + 1) % max(log_every // chunk, 1) == 0 or c == n_chunks - 1):
            _log(f"[{tag}] chunk {c+1}/{n_chunks}  E(eV/atom) mean {E_eV.mean():.6f} [{E_eV.min():.6f},{E_eV.max():.6f}]  "
                 f"acc {np.mean(acc_chunk[-1]):.3f}  drift {drift:.1e}  {R*chunk*(c+1-c0)/(time.time()-t0):,.0f} steps/s")
        if ck_every and (c + 1) % ck_every == 0 and c + 1 < n_chunks:
            os.makedirs(out_dir, exist_ok=True)
            traj = [np.concatenate(traj, axis=1)] if traj else []
            np.savez(ck_path + ".tmp.npz", chunk=c + 1, sig=st.sigma.cpu().numpy(), rep_of_slot=st.rep_of_slot.cpu().numpy(),
                     slot_of_rep=st.slot_of_rep.cpu().numpy(), n_acc=st.n_acc.cpu().numpy(), n_ex=st.n_ex.cpu().numpy(),
                     drift=drift, E_chunk=np.array(E_chunk), acc_chunk=np.array(acc_chunk),
                     drift_log=np.array(drift_log, np.float64), traj=(traj[0] if traj else np.zeros((R, 0))),
                     cfg_betas=betas.astype(np.float64), **{"cfg_" + k: v for k, v in want.items()})
            os.replace(ck_path + ".tmp.npz", ck_path)
    (st.check_errors if hasattr(st, "check_errors") else st.model.check_errors)()   # device error flags raise here
    wall = time.time() - t0
    os.makedirs(out_dir, exist_ok=True)
    E_chunk = np.array(E_chunk); acc_chunk = np.array(acc_chunk); traj = np.concatenate(traj, axis=1)
    np.savez(os.path.join(out_dir, "energies.npz"), E_chunk=E_chunk, acc_chunk=acc_chunk, drift=np.array(drift_log),
             drift_eV=np.array(drift_log) * ys, traj=traj, betas=betas, temps=temps)
    ros = st.rep_of_slot.long().cpu().numpy()
    sig_in = st.sigma.cpu().numpy()[ros][:, model.inv_perm]
    np.save(os.path.join(out_dir, "final_sigma.npy"), sig_in)
    if N <= int(os.environ.get("CE_CNN_CIF_MAX", "200000")):
        _write_cifs(mc, sig_in, temps, out_dir)
    if ck_every and os.path.exists(ck_path):
        os.remove(ck_path)
    n_ex = int(st.n_ex.item())
    n_try = (n_chunks - c0) * rounds * (R - 1) / 2.0
    return dict(steps_per_s=float(R * chunk * (n_chunks - c0) / max(wall, 1e-9)), n_replicas=R, n_steps=int(n_steps),
                chunk=int(chunk), E_final=[float(x) for x in E_chunk[-1]], acc_mean=float(acc_chunk.mean()),
                drift_max=float(np.max(drift_log)), exchange_acc=(n_ex / n_try if n_try else None),
                near_threshold_steps=int(st.n_near.sum().item()),
                model_depth=int(mc["depth"]), n_atoms=int(N))


def run_mc(model_path, init_cif, n_steps=10000, temperature=300.0, seed=0, log_every=0, out_dir=".", n_replicas=1,
           chunk=1000, sample_interval=100, supercell=(1, 1, 1), seed_idx=0, dtype="float32", anchor_every=None,
           init_npz=None, checkpoint_every=0, cluster=1, **_):
    mc = _prepare(model_path, init_cif, supercell, seed_idx, dtype, seed)
    betas = [1.0 / (KB * temperature)] * n_replicas
    res = _run_replicas(mc, betas, n_steps, seed, min(chunk, n_steps), log_every, sample_interval, out_dir,
                        f"ce_cnn T={temperature:.0f}", anchor_every=anchor_every, init_npz=init_npz,
                        checkpoint_every=checkpoint_every, cluster=cluster)
    res.update(temperature=float(temperature))
    return res


def run_multiT_mc(model_path, init_cif, temps, n_steps=10000, seed=0, log_every=0, out_dir=".", chunk=1000,
                  sample_interval=100, supercell=(1, 1, 1), seed_idx=0, dtype="float32", anchor_every=None, init_npz=None,
                  checkpoint_every=0, cluster=1, **_):
    mc = _prepare(model_path, init_cif, supercell, seed_idx, dtype, seed)
    betas = [1.0 / (KB * t) for t in temps]
    res = _run_replicas(mc, betas, n_steps, seed, min(chunk, n_steps), log_every, sample_interval, out_dir,
                        "ce_cnn multiT", anchor_every=anchor_every, init_npz=init_npz, checkpoint_every=checkpoint_every,
                        cluster=cluster)
    res.update(temps=[float(t) for t in temps])
    return res


def run_pt_mc(model_path, init_cif, n_steps=10000, T_min=100.0, T_max=2000.0, n_replicas=32, T_grid=None,
              exchange_every=100, seed=0, log_every=0, out_dir=".", chunk=1000, sample_interval=100, supercell=(1, 1, 1),
              seed_idx=0, dtype="float32", anchor_every=None, init_npz=None, checkpoint_every=0, cluster=1, **_):
    mc = _prepare(model_path, init_cif, supercell, seed_idx, dtype, seed)
    temps = np.asarray(T_grid, float) if T_grid is not None else np.geomspace(T_min, T_max, n_replicas)
    betas = [1.0 / (KB * t) for t in temps]
    res = _run_replicas(mc, betas, n_steps, seed, min(chunk, n_steps), log_every, sample_interval, out_dir, "ce_cnn PT",
                        exchange_every=exchange_every, anchor_every=anchor_every, init_npz=init_npz,
                        checkpoint_every=checkpoint_every, cluster=cluster)
    res.update(temps=[float(t) for t in temps], exchange_every=int(exchange_every))
    return res
