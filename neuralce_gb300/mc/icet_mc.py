"""CE ("icet" framework) drivers of the command line, after ``neuralce/ce/icet_mc.py:76-250``.

The cell is the init cif (an integer supercell of the ``.ce`` primitive, sites on the ideal lattice), optionally
tiled ``supercell_reps`` times with the species re-shuffled within every sublattice (seeded; the environment
variable ``CE_SUPERCELL_PERIODIC=1`` keeps the periodic images instead), ``energy_scale`` = number of copies.
Every run goes through ``pt.run_pt_mcmc`` on the GPU engine: PT over a ladder, or independent chains (single
temperature / a temperature list) with the exchange switched off.
"""
from __future__ import annotations

import hashlib
import os

import numpy as np

from ..ce import GPUClusterExpansion
from ..io import Structure, read_ce, read_cif
from ..lattice import site_decompose
from ..pt import MCMCConfig, run_pt_mcmc


def _unsupported(**kw):
    bad = [k for k, v in kw.items() if v not in (None, "", {}, [], 0, 0.0)]
    if bad:
        raise NotImplementedError(f"{', '.join(bad)}: spin cluster expansions and primitive detection of non-ideal "
                                  "cells are not on this engine's path (ideal-lattice binary CE only)")


def prepare_cell(ce_file, init_cif, supercell_reps=None, seed=0, log=print):
    """(structure, energy_scale) of the MC cell."""
    prim = ce_file.primitive
    atoms = read_cif(init_cif) if isinstance(init_cif, str) else init_cif
    site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)          # raises unless on the ideal lattice
    energy_scale = 1.0
    reps = tuple(int(r) for r in supercell_reps) if supercell_reps is not None else (1, 1, 1)
    if reps != (1, 1, 1):
        atoms = atoms.repeat(reps)
        energy_scale = float(np.prod(reps))
        if os.environ.get("CE_SUPERCELL_PERIODIC", "0") != "1":
            basis, _, _, _ = site_decompose(prim.cell, prim.frac, atoms.cell, atoms.positions)
            rng = np.random.default_rng(seed)
            Z = atoms.numbers.copy()
            keys = [tuple(sp) for sp in prim.species]
            for key in dict.fromkeys(keys):                                      # sublattices: same allowed species
                bs = [b for b, k in enumerate(keys) if k == key]
                m = np.isin(basis, bs)
                Z[m] = rng.permutation(Z[m])
            atoms.numbers = Z
            log(f"[ce] cif repeated {reps}: {len(atoms)} sites; each sublattice's species permuted at random "
                f"(seed {seed})", flush=True)
        else:
            log(f"[ce] cif repeated {reps}: {len(atoms)} sites, the ordered copies left as they are", flush=True)
    return atoms, energy_scale


def run_pt_mc(ce_path, init_cif, n_steps, T_min=100.0, T_max=2000.0, n_replicas=32, n_ladders=1, swap_mode="uniform",
              seed=0, log_every=0, n_equilib=0, exchange_every=100, chunk_size=1000, sample_interval=100, out_dir=".",
              ideal_map=None, inert_species=None, symprec=1e-2, swap_pairs=None, ref_cif=None,
              fractional_position_tolerance=None, energy_mode="delta", spin_move_prob=0.0, spin_orbits_pkl="",
              spin_states=None, supercell_reps=None, table_mode=None, checkpoint_every=0, T_grid=None, init_npz=None,
              precision=64, warps=0, cluster=1, verbose=True):
    """PT-MCMC of a fitted ``.ce`` on the GPU engine (reference ``icet_mc.run_pt_mc``)."""
    log = print if verbose else (lambda *a, **k: None)
    _unsupported(ideal_map=ideal_map, inert_species=inert_species, spin_orbits_pkl=spin_orbits_pkl,
                 spin_states=spin_states)
    if swap_mode not in ("uniform", "weighted"):
        raise ValueError(f"swap_mode must be 'uniform' or 'weighted'; got {swap_mode!r}")
    if energy_mode == "local":
        raise ValueError("--energy_mode local is the nce path; icet uses --energy_mode delta (or full)")
    if energy_mode == "full":
        log("PT-MC: energy_mode 'full' runs the delta engine (the same Markov chain; the energy is recomputed "
            "exactly at the end)", flush=True)
    if table_mode not in (None, "implicit"):
        raise ValueError("only the implicit (template-only) tables are implemented on this engine")
    os.makedirs(out_dir, exist_ok=True)
    ce = read_ce(ce_path)
    atoms, energy_scale = prepare_cell(ce, init_cif, supercell_reps, seed, log)
    gce = GPUClusterExpansion(ce, atoms, energy_scale=energy_scale)
    log(f"PT-MC: {gce}  energy_scale {energy_scale:g}", flush=True)
    initial_sigma = gce.encode(atoms)
    log(f"PT-MC: init E (from cif) = {gce.energy(initial_sigma[None]):.4f} eV", flush=True)
    if init_npz:
        if n_ladders != 1:
            raise ValueError("--init_npz assigns one structure per temperature of a single ladder; n_ladders must be 1")
        from .init_structures import load_init_npz
        run_T = np.asarray(T_grid, float) if T_grid is not None else np.geomspace(T_min, T_max, n_replicas)
        nums, _ = load_init_npz(init_npz, atoms, run_T)
        rows = []
        for r in range(nums.shape[0]):
            a_r = Structure(atoms.cell, atoms.positions, nums[r].astype(np.int64))
            rows.append(gce.encode(a_r))
        initial_sigma = np.stack(rows)
        log(f"PT-MC: per-replica starting structures from {init_npz} ({initial_sigma.shape[0]} replicas)", flush=True)
    h = hashlib.md5(np.ascontiguousarray(ce.parameters, dtype=np.float64).tobytes())
    h.update(np.ascontiguousarray(initial_sigma, dtype=np.int32).tobytes())
    cfg = MCMCConfig(T_min=T_min, T_max=T_max, n_replicas=(len(T_grid) if T_grid is not None else n_replicas),
                     n_ladders=n_ladders, n_steps=n_steps, n_equilib=n_equilib, exchange_interval=exchange_every,
                     chunk_size=chunk_size, sample_interval=sample_interval, output_dir=out_dir, seed=seed,
                     swap_pairs=swap_pairs, initial_sigma=initial_sigma, energy_mode="delta",
                     checkpoint_every=checkpoint_every,
                     T_grid=(np.asarray(T_grid, float) if T_grid is not None else None), run_id=h.hexdigest()[:16],
                     precision=precision, warps=warps, cluster=cluster)
    return run_pt_mcmc(gce, cfg, verbose=verbose)


def run_mc(ce_path, init_cif, n_steps, temperature=300.0, seed=0, log_every=0, swap_mode="uniform", energy_mode="delta",
           out_dir=".", **kw):
    """One chain at ``temperature`` (reference single-T ``run_mc``), as a one-slot run without exchange."""
    kw.pop("exchange_every", None)
    return run_pt_mc(ce_path, init_cif, n_steps, seed=seed, log_every=log_every, swap_mode=swap_mode,
                     energy_mode=energy_mode, out_dir=out_dir, T_grid=[float(temperature)], exchange_every=0,
                     sample_interval=kw.pop("sample_interval", 100), chunk_size=kw.pop("chunk_size", 1000), **kw)


def run_multiT_mc(ce_path, init_cif, temps, n_steps, seed=0, log_every=0, swap_mode="uniform", energy_mode="delta",
                  out_dir=".", **kw):
    """Independent chains, one per temperature (reference ``run_multiT_mc``)."""
    kw.pop("exchange_every", None)
    return run_pt_mc(ce_path, init_cif, n_steps, seed=seed, log_every=log_every, swap_mode=swap_mode,
                     energy_mode=energy_mode, out_dir=out_dir, T_grid=[float(t) for t in temps], exchange_every=0,
                     sample_interval=kw.pop("sample_interval", 100), chunk_size=kw.pop("chunk_size", 1000), **kw)
