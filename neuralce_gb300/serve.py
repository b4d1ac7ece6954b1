"""Serving form: a resident job server for parallel-tempering jobs (``nce_server_*`` / ``nce_job_*`` in
libnce_gb300).

Jobs of different cells, replica counts, compositions and models (CE or NeuralCE) are submitted while others run;
the server admits them in submission order as device memory within its budget frees up, keeps their state on
the device, advances the running CE jobs with persistent batch launches on eight lanes (a job joins the next
launch on an idle lane as soon as its previous one has completed: continuous batching) and each NeuralCE job chunk
by chunk on side streams, and copies each job's final state into host arrays when it finishes.  A job's
chunks (exchange interval, Philox key and global step of every chunk) depend only on its own parameters, so its
result is the same alone and in any mix.  The reference has no serving mode: a job here is one
``run_pt_mcmc`` call (``neuralce/ce/pt_mcmc_ce.py:587-601``) or NeuralCE ``_run_replicas``
(``neuralce/nce/mcmc.py:288-422``) without the file outputs.

Every call here is host-only and returns at once; ``wait`` polls with sleeps.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import _lib

STATUS = {0: "queued", 1: "running", 2: "done", 3: "cancelled", 4: "failed"}


class Job:
    """Handle of a submitted job; ``result()`` holds the final state once ``done``."""

    def __init__(self, server, kind, model, R, N, sigma_out=None, borrowed=None):
        self.server, self.kind, self.model, self.R, self.N = server, kind, model, R, N
        self.sigma = np.zeros((R, N), np.int8) if sigma_out is None else sigma_out
        self._borrowed = borrowed              # the caller's initial occupancies, read by the server at admission
        self.E = np.zeros(R, np.float64)
        self.n_acc = np.zeros(R, np.int64)
        self.rep_of_slot = np.zeros(R, np.int32)
        self.n_ex = np.zeros(1, np.int64)
        self.id = None

    def info(self):
        return self.server.poll(self)

    @property
    def status(self):
        return self.info()["status"]

    def result(self):
        inf = self.info()
        if inf["status"] != "done":
            raise RuntimeError(f"job {self.id} is {inf['status']}")
        return dict(sigma=self.sigma, E=self.E, n_acc=self.n_acc, rep_of_slot=self.rep_of_slot, n_ex=int(self.n_ex[0]),
                    latency_s=inf["t_end"] - inf["t_submit"])


class Server:
    """ce_kernel: 0 = every CE job on the sign-parity kernel at ``precision``; 3 = jobs whose cell allows it on the
    local-field kernel (exact fixed-point dE; 8 more bytes of device memory per site and replica), the rest on the
    sign-parity kernel."""

    def __init__(self, hbm_budget=0, max_batch=64, precision=32, warps=8, nce_cluster=1, nce_streams=4, starve_s=5.0,
                 ce_kernel=0, ce_lf_warps=0):
        cfg = _lib.NceServerConfig()
        cfg.hbm_budget, cfg.max_batch, cfg.precision, cfg.warps = int(hbm_budget), int(max_batch), int(precision), int(warps)
        cfg.nce_cluster, cfg.nce_streams, cfg.starve_s = int(nce_cluster), int(nce_streams), float(starve_s)
        cfg.ce_kernel, cfg.ce_lf_warps = int(ce_kernel), int(ce_lf_warps)
        h = C.c_void_p()
        _lib.check(_lib.lib().nce_server_create(C.byref(cfg), C.byref(h)), "nce_server_create")
        self._h = h
        self._jobs = {}

    def _submit(self, kind, model_handle, model, sigma, beta_slot, n_steps, exchange_every, seed, ladder_id,
                reanchor_chunks=0, sigma_out=None, borrow=False):
        sigma = np.ascontiguousarray(np.asarray(sigma, np.int8))
        R, N = sigma.shape
        beta = np.ascontiguousarray(np.asarray(beta_slot, np.float32))
        if beta.shape != (R,):
            raise ValueError(f"beta_slot must have {R} entries")
        lid = None if ladder_id is None else np.ascontiguousarray(np.asarray(ladder_id, np.int32))
        if sigma_out is not None and (sigma_out.shape != (R, N) or sigma_out.dtype != np.int8
                                      or not sigma_out.flags["C_CONTIGUOUS"] or not sigma_out.flags["WRITEABLE"]):
            raise ValueError(f"sigma_out must be a writeable C-contiguous ({R}, {N}) int8 array")
        job = Job(self, kind, model, R, N, sigma_out, sigma if borrow else None)
        d = _lib.NceJobDesc()
        d.flags = 1 if borrow else 0
        d.kind, d.model, d.R = kind, model_handle, R
        d.sigma, d.beta_slot, d.ladder_id = sigma.ctypes.data, beta.ctypes.data, (lid.ctypes.data if lid is not None else None)
        d.n_steps, d.exchange_every, d.seed = int(n_steps), int(exchange_every), int(seed) & 0xFFFFFFFFFFFFFFFF
        d.reanchor_chunks = int(reanchor_chunks)
        d.sigma_out, d.E_out, d.n_acc_out = job.sigma.ctypes.data, job.E.ctypes.data, job.n_acc.ctypes.data
        d.rep_of_slot_out, d.n_ex_out = job.rep_of_slot.ctypes.data, job.n_ex.ctypes.data
        jid = C.c_int64()
        _lib.check(_lib.lib().nce_job_submit(self._h, C.byref(d), C.byref(jid)), "nce_job_submit")
        job.id = int(jid.value)
        self._jobs[job.id] = job
        return job

    def submit_ce(self, gce, sigma, beta_slot, n_steps, exchange_every=5000, seed=0, ladder_id=None, sigma_out=None,
                  borrow=False):
        """A CE parallel-tempering job: ``sigma`` (R, N) species indices in canonical site order.  ``sigma_out``: the
        array that receives the final occupancies (default: a new one); ``borrow``: the server reads ``sigma`` in
        place when it admits the job instead of copying it now; the job keeps a reference, and the caller must not
        change it until the job has left the queued and running states.  Both avoid host copies of large cells;
        in page-locked memory (e.g. ``torch.empty(..., pin_memory=True).numpy()``) the uploads and downloads are
        direct copies."""
        return self._submit(0, gce.handle.value, gce, sigma, beta_slot, n_steps, exchange_every, seed, ladder_id,
                            sigma_out=sigma_out, borrow=borrow)

    def submit_nce(self, model, sigma, beta_slot, n_steps, exchange_every=1000, seed=0, ladder_id=None, reanchor_chunks=0,
                   sigma_out=None, borrow=False):
        """A NeuralCE parallel-tempering job on an ``nce.NCEModel``; the full caches are rebuilt every
        ``reanchor_chunks`` chunks (0: ceil(N / exchange_every), the reference driver's default).  ``sigma_out`` and
        ``borrow`` as in ``submit_ce``."""
        return self._submit(1, model.handle.value, model, sigma, beta_slot, n_steps, exchange_every, seed, ladder_id,
                            reanchor_chunks, sigma_out=sigma_out, borrow=borrow)

    def poll(self, job):
        inf = _lib.NceJobInfo()
        _lib.check(_lib.lib().nce_job_poll(self._h, int(job.id), C.byref(inf)), "nce_job_poll")
        out = {k: getattr(inf, k) for k, _ in inf._fields_}
        out["status"] = STATUS[inf.status]
        if inf.status == 4:
            buf = C.create_string_buffer(2048)
            _lib.lib().nce_job_error(self._h, int(job.id), buf, len(buf))
            out["message"] = buf.value.decode(errors="replace")
        return out

    def cancel(self, job):
        _lib.check(_lib.lib().nce_job_cancel(self._h, int(job.id)), "nce_job_cancel")

    def wait(self, jobs, timeout=None, poll_s=0.0005):
        """Poll until every job has left the queued/running states; returns their infos."""
        t0 = time.time()
        jobs = list(jobs)
        while True:
            infos = [self.poll(j) for j in jobs]
            if all(i["status"] not in ("queued", "running") for i in infos):
                return infos
            if timeout is not None and time.time() - t0 > timeout:
                raise TimeoutError(f"{sum(i['status'] in ('queued', 'running') for i in infos)} jobs still open")
            time.sleep(poll_s)

    def stats(self):
        s = _lib.NceServerStats()
        _lib.check(_lib.lib().nce_server_query(self._h, C.byref(s)), "nce_server_query")
        return {k: getattr(s, k) for k, _ in s._fields_}

    def close(self):
        if self._h is not None:
            _lib.lib().nce_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
