"""One temperature ladder over several GPUs (one process per GPU): replicas are sharded into contiguous ranges,
configurations never leave their GPU, and at every exchange the ranks all-gather the R float64 energies and
recompute the same slot permutation (``neuralce/ce/pt_mcmc_ce.py:748-760``): one collective of R x 8 bytes per
exchange and no data-path collective.

On a rank, the chunk kernel runs its local replicas with ``slot_of_rep`` holding their GLOBAL temperature slots
and ``beta_slot`` the global ladder, so every proposal is keyed by (seed, global step, global slot) exactly as in
a single-process run: a sharded run reproduces the single-GPU trajectory bit for bit.  The exchange is computed
on the host from the gathered energies with the kernels' Philox counters (round q of the exchange: parity from
counter word 2 = 0xFFFFFFFF - 2q, uniform of pair k from word 2 = 0xFFFFFFFE - 2q and word 3 = k; words 0-1 = the
global step after the chunk).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib


def _u01(hi, lo):
    m = ((int(hi) & 0xFFFFFFFF) << 21) | ((int(lo) & 0xFFFFFFFF) >> 11)
    return (m + 1) * 2.0 ** -53


def exchange_slots(E, beta_slot, ladder_id, rep_of_slot, seed, g_end, q=0):
    """Round q of the neighbour-slot exchange on the host: E (R,) float64 per replica, beta_slot (R,) float32 per
    slot, rep_of_slot (R,) int; returns (new rep_of_slot, accepted swaps).  Each round draws its own parity and
    uniforms, as ce_exchange_kernel does."""
    R = len(rep_of_slot)
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    c0, c1 = g_end & 0xFFFFFFFF, (g_end >> 32) & 0xFFFFFFFF
    cq = (0xFFFFFFFF - 2 * q) & 0xFFFFFFFF
    parity = _lib.philox4x32([c0, c1, cq, 0], [k0, k1])[0] & 1
    perm = np.arange(R)
    n = 0
    for k in range(R // 2 + 1):
        i = 2 * k + parity; j = i + 1
        if 2 * k >= R - 1 or j >= R:
            continue
        if ladder_id[i] != ladder_id[j]:
            continue
        log_acc = (float(np.float32(beta_slot[j])) - float(np.float32(beta_slot[i]))) * (float(E[rep_of_slot[j]]) - float(E[rep_of_slot[i]]))
        w = _lib.philox4x32([c0, c1, (cq - 1) & 0xFFFFFFFF, k], [k0, k1])
        if math.log(_u01(w[0], w[1])) < log_acc:
            perm[i], perm[j] = j, i
            n += 1
    return np.asarray(rep_of_slot)[perm].copy(), n


class ShardedLadder:
    """Global slot bookkeeping of a ladder of R replicas sharded over ``world`` ranks (contiguous replica ranges)."""

    def __init__(self, beta_slot, ladder_id=None, rank=0, world=1, group=None):
        self.beta_slot = np.asarray(beta_slot, np.float32)
        self.R = len(self.beta_slot)
        self.ladder_id = np.zeros(self.R, np.int32) if ladder_id is None else np.asarray(ladder_id, np.int32)
        self.rank, self.world, self.group = rank, world, group
        bounds = np.linspace(0, self.R, world + 1).round().astype(int)
        self.bounds = bounds
        self.r0, self.r1 = int(bounds[rank]), int(bounds[rank + 1])
        self.rep_of_slot = np.arange(self.R)
        self.n_ex = 0

    @property
    def slot_of_rep(self):
        s = np.empty(self.R, np.int64); s[self.rep_of_slot] = np.arange(self.R)
        return s

    def local_slots(self):
        return self.slot_of_rep[self.r0:self.r1].astype(np.int32)

    def gather(self, E_local):
        """all ranks' replica energies in global replica order (float64)."""
        E_local = np.asarray(E_local, np.float64)
        if self.world == 1:
            return E_local.copy()
        import torch
        import torch.distributed as dist
        n = int(self.bounds[1:].__sub__(self.bounds[:-1]).max())
        buf = torch.zeros(n, dtype=torch.float64)
        buf[:len(E_local)] = torch.from_numpy(E_local)
        backend = dist.get_backend(self.group)
        if backend == "nccl":
            buf = buf.cuda()
        out = [torch.zeros_like(buf) for _ in range(self.world)]
        dist.all_gather(out, buf, group=self.group)
        return np.concatenate([o.cpu().numpy()[:self.bounds[q + 1] - self.bounds[q]] for q, o in enumerate(out)])

    def exchange(self, E_local, seed, g_end, rounds=1):
        E = self.gather(E_local)
        for q in range(rounds):
            self.rep_of_slot, n = exchange_slots(E, self.beta_slot, self.ladder_id, self.rep_of_slot, seed, g_end, q)
            self.n_ex += n
        return E


def run_sharded_chunks(gce, shard, sigma_local, n_chunks, chunk, seed, precision=64, warps=0, path=0, step0=0):
    """The rank's replicas on its GPU for ``n_chunks`` chunks with a ladder-wide exchange after each; returns the
    local PTState (energies, occupancies) and the global energies after the last exchange."""
    import torch
    from .pt import PTState, run_chunk
    E0 = gce.batched_energy(torch.as_tensor(sigma_local).cuda()).cpu().numpy()
    st = PTState(sigma_local, E0, shard.beta_slot, shard.ladder_id)
    st.slot_of_rep = torch.as_tensor(shard.local_slots()).cuda()
    E = None
    for c in range(n_chunks):
        run_chunk(gce, st, chunk, step0 + c * chunk, seed, precision, warps, None, 1, None, False, path=path)
        E = shard.exchange(st.E.cpu().numpy(), seed, step0 + (c + 1) * chunk)
        st.slot_of_rep.copy_(torch.as_tensor(shard.local_slots()).cuda())
    return st, E
