"""Batched parallel tempering: many independent CE jobs (different cells, compositions and ladders) advanced by
one persistent launch per chunk (``nce_ce_run_batch``, up to 64 jobs per launch), captured in a CUDA graph.

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
SPLIT_SITES = 48 * 1024       # a job whose occupancy fits the batch kernel's per-job shared memory can be split over CTAs


class CEBatch:
    def __init__(self, jobs, precision=32, warps=0, path=0, seeds=None, track=True, cluster=1):
        import torch
        self.jobs = jobs
        self.precision, self.path = precision, path
        self.states = []
        for j in jobs:
            sd = torch.as_tensor(j["sigma"]).cuda()
            E0 = j["gce"].batched_energy(sd).cpu().numpy()
            st = PTState(j["sigma"], E0, j["beta"], np.zeros(len(j["beta"]), np.int32))
            if track:
                st.track_counts(j["gce"])
            self.states.append(st)
        self.track, self.cluster = track, cluster
        self.seeds = seeds if seeds is not None else [7919 * (k + 1) for k in range(len(jobs))]
        self.warps = warps if warps else 8
        self.step = 0

    def launch_groups(self):
        """(job indices, CTAs per replica) of each launch: with a split (cluster > 1) the jobs whose occupancy fits the
        per-job shared memory are launched split over thread-block clusters, the larger ones one CTA per replica;
        at most 64 jobs per launch."""
        if self.cluster <= 1:
            idx = [(list(range(len(self.jobs))), 1)]
        else:
            small = [k for k, j in enumerate(self.jobs) if j["gce"].n_atoms <= SPLIT_SITES]
            large = [k for k, j in enumerate(self.jobs) if j["gce"].n_atoms > SPLIT_SITES]
            idx = [(g, c) for g, c in ((small, self.cluster), (large, 1)) if g]
        return [(g[a:a + MAX_JOBS], c) for g, c in idx for a in range(0, len(g), MAX_JOBS)]

    def run_chunk(self, n_steps, do_exchange=True, stream=None, step_dev=None):
        """one chunk of every job (launch_groups).  step_dev: (n_jobs,) int64 device step counters that the launch
        reads and advances (used inside captured graphs) instead of the host step."""
        for js, cl in self.launch_groups():
            n = len(js)
            hs = (C.c_void_p * n)(*[self.jobs[k]["gce"].handle.value for k in js])
            ss = (_lib.NcePtState * n)(*[self.states[k].struct() for k in js])
            cks = (_lib.NcePtChunk * n)(*[make_chunk(n_steps, self.step, self.seeds[k], self.precision, self.warps, None, 1, None,
                                                     do_exchange, path=self.path, cluster=cl) for k in js])
            if step_dev is not None:
                for i, k in enumerate(js):
                    cks[i].step_dev = step_dev.data_ptr() + 8 * k
            _lib.check(_lib.lib().nce_ce_run_batch(n, hs, ss, cks, _lib.stream_ptr(stream)), "nce_ce_run_batch")
        if step_dev is None:
            self.step += n_steps

    def _reanchor_into(self, stream=None):
        for j, st in zip(self.jobs, self.states):
            _lib.check(_lib.lib().nce_ce_energy_from_counts(j["gce"].handle, st.cv.data_ptr(), st.R, st.E.data_ptr(),
                                                            _lib.stream_ptr(stream)), "nce_ce_energy_from_counts")

    def capture(self, n_steps, chunks=1, reanchor=True, do_exchange=True):
        """Capture ``chunks`` chunks of every job (+ the exact float64 re-anchor from the tracked sums) in one CUDA
        graph; ``replay()`` then advances the whole batch by chunks * n_steps steps with one graph launch."""
        import torch
        if reanchor and not self.track:
            raise ValueError("the captured re-anchor needs tracked cluster-vector sums (track=True)")
        self._step_dev = torch.full((len(self.jobs),), self.step, dtype=torch.int64, device="cuda")
        torch.cuda.synchronize()
        self._graph = torch.cuda.CUDAGraph()
        self._graph_steps = n_steps * chunks
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            with torch.cuda.graph(self._graph, stream=side):
                for _ in range(chunks):
                    self.run_chunk(n_steps, do_exchange, stream=side, step_dev=self._step_dev)
                if reanchor:
                    self._reanchor_into(side)
        torch.cuda.current_stream().wait_stream(side)
        return self

    def replay(self):
        self._graph.replay()
        self.step += self._graph_steps

    def reanchor(self, full=False):
        """float64 re-anchor of every replica's carried energy; returns the largest drift.  With tracked
        cluster-vector sums the energies follow exactly from them (O(n_cols) per replica); ``full`` or an
        untracked batch recomputes them from the occupancies."""
        drift = 0.0
        if self.track and not full:
            for j, st in zip(self.jobs, self.states):
                drift = max(drift, st.reanchor_from_counts(j["gce"]))
            return drift
        for j, st in zip(self.jobs, self.states):
            E = j["gce"].batched_energy(st.sigma, precision=64)
            drift = max(drift, float((E - st.E).abs().max().item()))
            st.E.copy_(E)
        return drift

    @property
    def attempts_per_step(self):
        return sum(int(j["R"]) for j in self.jobs)


def tune_launch(jobs, precision=32, warps=(4, 8, 16, 32), clusters=(1, 2, 4), steps=200):
    """Autotune a batch's launch shape, warps per CTA and the split (CTAs per replica of the jobs that can be split):
    time a short chunk of the real batch for each candidate on scratch states.  Returns ((warps, cluster), {...: ms})."""
    import torch
    times = {}
    for cl in clusters:
        for w in warps:
            b = CEBatch(jobs, precision, w, track=False, cluster=cl)
            try:
                b.run_chunk(10, False)
            except _lib.NceError:
                continue                                   # a split that does not launch on this GPU
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(); b.run_chunk(steps, False); s1.record(); torch.cuda.synchronize()
            times[(w, cl)] = s0.elapsed_time(s1)
    return min(times, key=times.get), times


def tune_warps(jobs, precision=32, candidates=(4, 8, 16, 32), steps=200):
    """Warps per replica for a batch with one CTA per replica: (warps, {warps: ms})."""
    (w, _), t = tune_launch(jobs, precision, candidates, (1,), steps)
    return w, {k[0]: v for k, v in t.items()}
