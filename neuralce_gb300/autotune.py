"""Launch-shape autotuner of the CE chunk kernel: warps per replica (CTA size).

Per-step latency, not throughput, bounds a Markov chain, and the best CTA size depends on the number of rows
per site, the replica count relative to the 152 SMs and the precision.  The tuner times a short chunk of the
real kernel for each candidate on a scratch copy of the state (the job's own state is untouched) and keeps the
fastest; results are cached per (tables, R, precision, path)."""
from __future__ import annotations

_cache = {}


def best_warps(gce, st, precision=64, path=0, candidates=(2, 4, 8, 16, 32), steps=300, seed=12345):
    import torch
    from .pt import PTState, run_chunk
    key = (id(gce), st.R, precision, path)
    if key in _cache:
        return _cache[key]
    scratch = PTState(st.sigma.cpu().numpy(), st.E.cpu().numpy(), st.beta_slot.cpu().numpy(), st.ladder_id.cpu().numpy())
    timings = {}
    for w in candidates:
        run_chunk(gce, scratch, 20, 0, seed, precision, w, path=path)          # warm-up / attribute set-up
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(); run_chunk(gce, scratch, steps, 20, seed, precision, w, path=path); b.record()
        torch.cuda.synchronize()
        timings[w] = a.elapsed_time(b)
    best = min(timings, key=timings.get)
    _cache[key] = (best, timings)
    return best, timings
