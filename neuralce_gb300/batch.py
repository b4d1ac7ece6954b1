"""Batched parallel tempering: many independent CE jobs (different cells, compositions and ladders) advanced by
one persistent launch per chunk (``nce_ce_run_batch``, up to 64 jobs per launch), CUDA-graph capturable.

Mirrors running the reference's ``run_chunk`` (``neuralce/ce/pt_mcmc_ce.py:798-818``) for every job, with each job's
own Philox stream (seed, global step, slot), its own chunk-end exchange and, optionally, a float64 full-energy
re-anchor of the carried energies every ``reanchor_every`` steps (the precision form: float32 dE, float64 E).
A job's trajectory is identical alone and inside any batch (tested)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .pt import PTState, make_chunk

MAX_JOBS = 64


class CEBatch:
    def __init__(self, jobs, precision=32, warps=0, path=0, seeds=None):
        import torch
        self.jobs = jobs
        self.precision, self.path = precision, path
        self.states = []
        for j in jobs:
            sd = torch.as_tensor(j["sigma"]).cuda()
            E0 = j["gce"].batched_energy(sd).cpu().numpy()
            self.states.append(PTState(j["sigma"], E0, j["beta"], np.zeros(len(j["beta"]), np.int32)))
        self.seeds = seeds if seeds is not None else [7919 * (k + 1) for k in range(len(jobs))]
        self.warps = warps if warps else 8
        self.step = 0

    def run_chunk(self, n_steps, do_exchange=True, stream=None):
        """one chunk of every job, 64 jobs per launch"""
        for a in range(0, len(self.jobs), MAX_JOBS):
            js = list(range(a, min(a + MAX_JOBS, len(self.jobs))))
            n = len(js)
            hs = (C.c_void_p * n)(*[self.jobs[k]["gce"].handle.value for k in js])
            ss = (_lib.NcePtState * n)(*[self.states[k].struct() for k in js])
            cks = (_lib.NcePtChunk * n)(*[make_chunk(n_steps, self.step, self.seeds[k], self.precision, self.warps, None, 1, None,
                                                     do_exchange, path=self.path) for k in js])
            _lib.check(_lib.lib().nce_ce_run_batch(n, hs, ss, cks, _lib.stream_ptr(stream)), "nce_ce_run_batch")
        self.step += n_steps

    def reanchor(self):
        """float64 full-energy recompute of every replica's carried energy; returns the largest drift."""
        drift = 0.0
        for j, st in zip(self.jobs, self.states):
            E = j["gce"].batched_energy(st.sigma, precision=64)
            drift = max(drift, float((E - st.E).abs().max().item()))
            st.E.copy_(E)
        return drift

    @property
    def attempts_per_step(self):
        return sum(int(j["R"]) for j in self.jobs)


def tune_warps(jobs, precision=32, candidates=(4, 8, 16, 32), steps=200):
    """Autotune warps per replica for a batch: time a short chunk of the real batch for each candidate on
    scratch states."""
    import torch
    best, times = None, {}
    for w in candidates:
        b = CEBatch(jobs, precision, w)
        b.run_chunk(10, False)
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(); b.run_chunk(steps, False); s1.record(); torch.cuda.synchronize()
        times[w] = s0.elapsed_time(s1)
    best = min(times, key=times.get)
    return best, times
