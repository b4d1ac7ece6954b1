"""Synthetic, seeded workloads of the benchmark configurations (no dataset is involved).

ce_config(L):  fcc Ni/Pt, a = 3.924 A, 4-site conventional cell repeated L x L x L (L = 8: 2,048 sites),
               cluster set cut at pairs 8 A / triplets 6 A / quadruplets 5 A (the shipped PtNi .ce's cutoffs),
               one ECI per orbit ~ N(0, (0.05 eV / k)^2) with k the 1-based rank of the orbit (order, radius),
               zerolet 0.  ECIs are per-atom energies; the cell's total energy uses energy_scale = N, as the
               shipped .ce does for its 256-site base cell.  Occupancy int8, exactly N/2 Pt by a seeded
               permutation (numpy default_rng).
ladder(R):     geometric 300-1400 K, beta = 1/(kB T) in float32 (``neuralce/ce/pt_mcmc_ce.py:223-229``).
"""
from __future__ import annotations

import functools

import numpy as np

from .ce_tables import ClusterSpace, synthetic_eci
from .io import Z_OF, fcc_conventional, fcc_primitive

A_FCC = 3.924
CUTOFFS = (8.0, 6.0, 5.0)


@functools.lru_cache(maxsize=4)
def cluster_space(cutoffs=CUTOFFS):
    return ClusterSpace.build(fcc_primitive(A_FCC), list(cutoffs))


def ce_structure(L, seed=0, x_pt=0.5):
    s = fcc_conventional(A_FCC, (L, L, L))
    N = len(s)
    rng = np.random.default_rng(seed)
    n_pt = int(round(x_pt * N))
    z = np.full(N, Z_OF["Ni"], np.int64)
    z[rng.permutation(N)[:n_pt]] = Z_OF["Pt"]
    s.numbers = z
    return s


def ce_config(L=8, seed=0, x_pt=0.5, eci_seed=0):
    """(GPUClusterExpansion, canonical sigma) of the synthetic CE workload on an L^3 conventional fcc cell."""
    from .ce import GPUClusterExpansion
    cs = cluster_space()
    eci = synthetic_eci(cs, eci_seed)
    s = ce_structure(L, seed, x_pt)
    gce = GPUClusterExpansion((cs, eci), s, energy_scale=len(s))
    return gce, gce.encode(s)


def ladder(R, T_min=300.0, T_max=1400.0):
    temps = np.geomspace(T_min, T_max, R) if R > 1 else np.array([T_min])
    return temps, (1.0 / (8.617333e-5 * temps)).astype(np.float32)


def replica_configs(sigma, R, seed):
    """R independent shuffles of sigma (same composition), one per replica."""
    rng = np.random.default_rng(seed)
    return np.stack([sigma[rng.permutation(len(sigma))] for _ in range(R)]).astype(np.int8)


def nce_config(L=8, depth=3, width=64, seed=0, x_pt=0.5, model_seed=0):
    """(NCEModel, canonical sigma) of the synthetic NeuralCE workload: the CE workload's cell and cluster set as
    layer 0 (38 channels), ``depth`` graph-convolution layers of ``width`` over the 12-neighbour shell, SiLU,
    sum readout, weights ~ N(0, 1/fan_in) from ``model_seed``."""
    from .nce import NCEModel, synthetic_model
    cs = cluster_space()
    s = ce_structure(L, seed, x_pt)
    P = synthetic_model(len(cs.orbits) + 1, depth, width, 1, model_seed)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum")
    return m, m.sig0


def ce_batch_config(n_jobs=64, seed=2, L_range=(4, 32), R_choices=(16, 32, 64), T_min=300.0, T_max=1400.0):
    """Batched CE workload: ``n_jobs`` independent cells with edge L ~ U{4..32} conventional cells (256 to 131,072
    sites), Pt fraction ~ U[0.1, 0.9], replicas ~ U{16, 32, 64} on a geometric 300-1400 K ladder each; the CE
    workload's cluster set and ECIs.  Returns a list of dicts (gce, sigma (R, N) int8, beta (R,), L, x_pt)."""
    from .ce import GPUClusterExpansion
    rng = np.random.default_rng(seed)
    cs = cluster_space()
    eci = synthetic_eci(cs, 0)
    jobs = []
    for k in range(n_jobs):
        L = int(rng.integers(L_range[0], L_range[1] + 1))
        x = float(rng.uniform(0.1, 0.9))
        R = int(rng.choice(R_choices))
        s = ce_structure(L, seed=1000 + k, x_pt=x)
        gce = GPUClusterExpansion((cs, eci), s, energy_scale=len(s))
        sig0 = gce.encode(s)
        _, beta = ladder(R, T_min, T_max)
        jobs.append(dict(gce=gce, sigma=replica_configs(sig0, R, 2000 + k), beta=beta, L=L, x_pt=x, R=R, N=len(s)))
    return jobs
