"""Launch-shape autotuner of the CE chunk kernels: warps per CTA, CTAs per replica (thread-block cluster) and,
optionally, the kernel (sign parity or local field).

Per-step latency, not throughput, bounds a Markov chain, and the best shape depends on the number of rows per
site, the replica count relative to the 152 SMs and the precision: with few replicas, spreading each replica
over a cluster of 2-8 CTAs puts idle SMs to work on the row phase at the price of one cluster barrier per
evaluated swap.  The tuner times a short chunk of the real kernel for each candidate on a scratch copy of the
state (the job's own state is untouched) and keeps the fastest; results are cached per (tables, R, precision,
path); the key names the model by its serial number, which no later model reuses."""
from __future__ import annotations

_cache = {}


def best_launch(gce, st, precision=64, path=0, warps=(2, 4, 8, 16, 32), clusters=(1,), steps=300, seed=12345, paths=None,
                reps=3):
    """((warps, cluster), {(warps, cluster): ms}) of the fastest candidate (each timed ``reps`` times on a chunk of
    ``steps`` steps, the fastest kept); with ``paths`` (e.g. (2, 3)) the path is tuned too: ((warps, cluster, path),
    {(warps, cluster, path): ms})."""
    import torch
    from . import _lib
    from .pt import PTState, run_chunk
    key = (gce.serial, st.R, precision, path, tuple(warps), tuple(clusters), tuple(paths or ()))
    if key in _cache:
        return _cache[key]
    if paths:
        timings = {}
        for p in paths:
            _, t = best_launch(gce, st, precision, p, warps, clusters, steps, seed, reps=reps)
            timings.update({k + (p,): v for k, v in t.items()})    # (a path that cannot run adds nothing)
        best = min(timings, key=timings.get)
        _cache[key] = (best, timings)
        return best, timings
    scratch = PTState(st.sigma.cpu().numpy(), st.E.cpu().numpy(), st.beta_slot.cpu().numpy(), st.ladder_id.cpu().numpy())
    if path == 3:
        if not gce.has_local_field or precision != 64:
            _cache[key] = (None, {})
            return _cache[key]
        scratch.enable_field(gce)
        clusters = (1,)                                   # one CTA per replica: the decider warp is the chain
        warps = tuple(w for w in warps if w <= 16) or (16,)   # the kernel's CTAs hold at most 16 warps
    timings = {}
    for cl in clusters:
        for w in warps:
            try:
                run_chunk(gce, scratch, 20, 0, seed, precision, w, path=path, cluster=cl)  # warm-up / attribute set-up
            except _lib.NceError:
                continue                                  # shape not launchable (cluster does not fit a GPC)
            best_ms = None
            for k in range(reps):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(); run_chunk(gce, scratch, steps, 20 + k * steps, seed, precision, w, path=path, cluster=cl); b.record()
                torch.cuda.synchronize()
                best_ms = a.elapsed_time(b) if best_ms is None else min(best_ms, a.elapsed_time(b))
            timings[(w, cl)] = best_ms
    best = min(timings, key=timings.get)
    _cache[key] = (best, timings)
    return best, timings


def best_warps(gce, st, precision=64, path=0, candidates=(2, 4, 8, 16, 32), steps=300, seed=12345):
    """Warps per replica with one CTA per replica: (warps, {warps: ms})."""
    (w, _), t = best_launch(gce, st, precision, path, candidates, (1,), steps, seed)
    return w, {k[0]: v for k, v in t.items()}
