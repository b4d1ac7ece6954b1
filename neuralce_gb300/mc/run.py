"""``neuralce-mc``: the reference's central Monte Carlo command line (``neuralce/mc/run.py:31-195``) on the GB300
engine.  Same flags and outputs (``mcmc_summary.json`` beside each driver's files).

    neuralce-mc --framework icet --ce models/ce/ptni/icet_c8_6_5.ce --init_cif ref_L10_NiPt.cif --supercell 2 2 2 \\
        --pt --T_min 300 --T_max 1400 --n_replicas 32 --n_steps 200000 --energy_mode delta --out_dir runs/icet
    neuralce-mc --framework nce --ckpt models/nce/<tag>/model.pkl --init_cif ref_L10_NiPt.cif --supercell 2 2 2 \\
        --pt --T_min 300 --T_max 1400 --n_replicas 32 --n_steps 200000 --energy_mode local --out_dir runs/nce

Flags that select machinery off this engine's path (spin models, primitive detection of relaxed or decorated
cells) are accepted by the parser and rejected with an error when set.  ``--platform`` is accepted for
compatibility: the engine always runs on the GPU.  Engine options (not in the reference): ``--precision``,
``--warps``, ``--cluster``.
"""
from __future__ import annotations

import argparse
import json
from pathlib import Path


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description="Central MC / parallel-tempering entry for the cluster-expansion models.")
    ap.add_argument("--framework", required=True, choices=["nce", "ce_cnn", "icet"],
                    help="nce = neural cluster expansion (alias ce_cnn); icet = orthonormal cluster expansion")
    ap.add_argument("--ce", default=None, help="(icet) fitted .ce file")
    ap.add_argument("--ckpt", default=None, help="(nce) models/nce/<tag>/model.pkl")
    ap.add_argument("--init_cif", required=True, help="initial structure (cif)")
    ap.add_argument("--T", type=float, default=300.0, help="single-replica temperature in K")
    ap.add_argument("--temps", nargs="+", type=float, default=None,
                    help="list of temperatures: one independent chain per temperature (overrides --T)")
    ap.add_argument("--n_steps", type=int, default=10000)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--log_every", type=int, default=0)
    ap.add_argument("--swap_mode", default="uniform", choices=["uniform", "weighted"],
                    help="(icet) sublattice sampling: 50:50 / proportional to size")
    ap.add_argument("--pt", action="store_true", help="parallel tempering over a temperature ladder")
    ap.add_argument("--n_replicas", type=int, default=32, help="(PT) replicas per ladder")
    ap.add_argument("--n_ladders", type=int, default=1, help="(icet PT) independent interleaved ladders")
    ap.add_argument("--T_min", type=float, default=100.0)
    ap.add_argument("--T_max", type=float, default=2000.0)
    ap.add_argument("--T_grid_file", default=None,
                    help="(PT) text file with one temperature (K) per line, ascending; overrides T_min/T_max/n_replicas")
    ap.add_argument("--init_npz", default=None, help="(PT) per-replica starting structures (numbers, positions, cell, temps)")
    ap.add_argument("--exchange_every", type=int, default=100, help="(PT) replica-exchange interval in steps")
    ap.add_argument("--sample_interval", type=int, default=100, help="energy sub-sampling interval of the trajectory")
    ap.add_argument("--chunk", type=int, default=1000, help="steps per device launch")
    ap.add_argument("--checkpoint_every", type=int, default=0,
                    help="save the MC state to out_dir/checkpoint.npz every K production chunks and resume from it")
    ap.add_argument("--supercell", nargs=3, type=int, default=[1, 1, 1], metavar=("NX", "NY", "NZ"),
                    help="tile init_cif NX*NY*NZ times in memory (species re-shuffled unless "
                         "CE_SUPERCELL_PERIODIC=1 / CE_CNN_SUPERCELL_PERIODIC=1)")
    ap.add_argument("--out_dir", default=".", help="directory for trajectory and summary outputs")
    ap.add_argument("--ideal_map", default=None, help="(icet) species -> idealised species for primitive detection")
    ap.add_argument("--inert_species", nargs="*", default=None, help="(icet) species excluded from swaps")
    ap.add_argument("--swap_pairs", default=None, help='(icet) JSON list of swap pairs, e.g. \'[["Ni","Pt"]]\'')
    ap.add_argument("--ref_cif", default=None, help="(icet) reference cif for primitive detection (default: init_cif)")
    ap.add_argument("--symprec", type=float, default=1e-2)
    ap.add_argument("--frac_tol", type=float, default=None)
    ap.add_argument("--spin_move_prob", type=float, default=0.5,
                    help="probability of a spin move per step; 0 for spin-free models")
    ap.add_argument("--spin_orbits_pkl", default=None)
    ap.add_argument("--spin_states", default=None)
    ap.add_argument("--spin_allowed_file", default="")
    ap.add_argument("--spin_init", choices=["random", "fm", "zero"], default="random")
    ap.add_argument("--energy_mode", choices=["full", "delta", "local"], default="full",
                    help="full = recompute every step (runs the equivalent local update here); delta (icet); local (nce)")
    ap.add_argument("--dtype", choices=["float32", "float64"], default="float32")
    ap.add_argument("--anchor_every", type=int, default=None, help="(nce) full cache/energy recompute every K chunks")
    ap.add_argument("--model_seed", type=int, default=0, help="(nce) which saved parameter set to use; -1 = ensemble mean")
    ap.add_argument("--platform", choices=["auto", "cpu", "cuda"], default="auto", help="accepted; the engine runs on the GPU")
    ap.add_argument("--precision", type=int, choices=[32, 64], default=64, help="(icet) dE precision of the engine")
    ap.add_argument("--warps", type=int, default=0, help="warps per CTA (0 = default)")
    ap.add_argument("--cluster", type=int, default=1, help="CTAs per replica (thread-block cluster)")
    return ap.parse_args(argv)


def _load_T_grid(path):
    import numpy as np
    return np.atleast_1d(np.loadtxt(path, comments="#", dtype=np.float64))


def dispatch_icet(args):
    from . import icet_mc
    if args.energy_mode == "local":
        raise ValueError("--energy_mode local is the nce path; icet uses --energy_mode delta (or full)")
    kw = dict(ideal_map=json.loads(args.ideal_map) if args.ideal_map else None, inert_species=args.inert_species,
              symprec=args.symprec, ref_cif=args.ref_cif, swap_pairs=json.loads(args.swap_pairs) if args.swap_pairs else None,
              fractional_position_tolerance=args.frac_tol, precision=args.precision, warps=args.warps,
              cluster=args.cluster, sample_interval=args.sample_interval, chunk_size=args.chunk,
              checkpoint_every=args.checkpoint_every)
    reps = tuple(int(x) for x in args.supercell) if list(args.supercell) != [1, 1, 1] else None
    if args.pt:
        T_grid = _load_T_grid(args.T_grid_file) if args.T_grid_file else None
        spin_states = json.loads(args.spin_states) if args.spin_states else None
        return icet_mc.run_pt_mc(ce_path=args.ce, init_cif=args.init_cif, n_steps=args.n_steps, T_min=args.T_min,
                                 T_max=args.T_max, n_replicas=args.n_replicas, n_ladders=args.n_ladders,
                                 swap_mode=args.swap_mode, seed=args.seed, log_every=args.log_every,
                                 exchange_every=args.exchange_every, out_dir=args.out_dir, energy_mode=args.energy_mode,
                                 spin_orbits_pkl=args.spin_orbits_pkl or "", spin_states=spin_states, supercell_reps=reps,
                                 T_grid=T_grid, init_npz=args.init_npz, **kw)
    if args.temps:
        return icet_mc.run_multiT_mc(args.ce, args.init_cif, args.temps, args.n_steps, seed=args.seed,
                                     log_every=args.log_every, swap_mode=args.swap_mode, energy_mode=args.energy_mode,
                                     out_dir=args.out_dir, supercell_reps=reps, **kw)
    return icet_mc.run_mc(args.ce, args.init_cif, args.n_steps, temperature=args.T, seed=args.seed,
                          log_every=args.log_every, swap_mode=args.swap_mode, energy_mode=args.energy_mode,
                          out_dir=args.out_dir, supercell_reps=reps, **kw)


def dispatch_nce(args):
    from . import nce_mc
    if not args.ckpt:
        raise ValueError("--framework nce requires --ckpt models/nce/<tag>/model.pkl")
    if args.energy_mode not in ("local", "full"):
        raise ValueError("nce supports --energy_mode local (recommended) or full")
    if args.spin_allowed_file:
        raise NotImplementedError("spin models are not on this engine's path")
    common = dict(model_path=args.ckpt, init_cif=args.init_cif, seed=args.seed, log_every=args.log_every,
                  out_dir=args.out_dir, chunk=args.chunk, sample_interval=args.sample_interval,
                  supercell=tuple(args.supercell), seed_idx=args.model_seed, dtype=args.dtype,
                  anchor_every=args.anchor_every, init_npz=args.init_npz, checkpoint_every=args.checkpoint_every,
                  cluster=args.cluster)
    if args.pt:
        T_grid = _load_T_grid(args.T_grid_file) if args.T_grid_file else None
        return nce_mc.run_pt_mc(n_steps=args.n_steps, T_min=args.T_min, T_max=args.T_max, n_replicas=args.n_replicas,
                                T_grid=T_grid, exchange_every=args.exchange_every, **common)
    if args.temps:
        return nce_mc.run_multiT_mc(temps=args.temps, n_steps=args.n_steps, **common)
    return nce_mc.run_mc(n_steps=args.n_steps, temperature=args.T, n_replicas=args.n_replicas, **common)


def summarize(result):
    """The JSON-able scalars and lists of a driver's result (``run.py:181-195``)."""
    if result is not None and not isinstance(result, dict) and hasattr(result, "__dataclass_fields__"):
        result = {k: getattr(result, k) for k in result.__dataclass_fields__}
    if not isinstance(result, dict):
        return None
    out = {}
    for k, v in result.items():
        if hasattr(v, "shape") and getattr(v, "shape", None) == ():
            v = float(v)
        if isinstance(v, (int, float, str, bool, list)):
            out[k] = v
    return out


def main(argv=None):
    args = parse_args(argv)
    if args.framework == "ce_cnn":
        args.framework = "nce"
    if args.framework == "icet" and not args.ce:
        raise SystemExit("--ce is required for --framework icet")
    Path(args.out_dir).mkdir(parents=True, exist_ok=True)
    print(f"== mcmc: framework={args.framework}, pt={args.pt}, energy_mode={args.energy_mode} ==", flush=True)
    result = dispatch_icet(args) if args.framework == "icet" else dispatch_nce(args)
    summary = summarize(result)
    if summary is not None:
        out_json = Path(args.out_dir) / "mcmc_summary.json"
        with open(out_json, "w") as f:
            json.dump(summary, f, indent=2, default=float)
        print(f"\nwrote {out_json}", flush=True)
    return result


if __name__ == "__main__":
    main()
