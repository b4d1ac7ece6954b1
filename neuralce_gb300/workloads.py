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


def nce_config(L=8, depth=3, width=64, seed=0, x_pt=0.5, model_seed=0, mma=0):
    """(NCEModel, canonical sigma) of the synthetic NeuralCE workload: the CE workload's cell and cluster set as
    layer 0 (38 channels), ``depth`` graph-convolution layers of ``width`` over the 12-neighbour shell, SiLU,
    sum readout, weights ~ N(0, 1/fan_in) from ``model_seed``."""
    from .nce import NCEModel, synthetic_model
    cs = cluster_space()
    s = ce_structure(L, seed, x_pt)
    P = synthetic_model(len(cs.orbits) + 1, depth, width, 1, model_seed)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum", mma=mma)
    return m, m.sig0


def shipped_nce_config(path, L=8, seed=0, x_pt=0.5, mma=0):
    """(NCEModel, canonical sigma): the reference's shipped PtNi NeuralCE model (its model.pkl content stored as
    JSON: depth 1, width 16, three shells, sigmoid gate, tanh, mean readout; the model its published GPU
    throughput is quoted on) on an L^3 conventional fcc cell at x_pt, a = 3.924 A."""
    import json
    from .lattice import Primitive
    from .nce import NCEModel, expand_params
    with open(path) as f:
        g = json.load(f)
    arr = lambda x: np.asarray(x, float)
    P = g["params0"]
    params = dict(lin=arr(P["lin"]), layers=[{k: arr(v) for k, v in lay.items()} for lay in P["layers"]],
                  head={k: (float(v) if np.ndim(v) == 0 else arr(v)) for k, v in P["head"].items()})
    prim = Primitive(cell=arr(g["primitive_cell"]), frac=arr(g["primitive_frac"]),
                     species=g["chemical_symbols"] * len(g["primitive_numbers"]), numbers=np.array(g["primitive_numbers"]))
    mdl = dict(params=[params], mu=arr(g["mu"]), sd=arr(g["sd"]), keep=np.array(g["keep"]), K_chem=g["K_chem"])
    cs = ClusterSpace.build(prim, g["cutoffs"])
    Pm, mu, sd = expand_params(mdl, 0)
    m = NCEModel(cs, ce_structure(L, seed, x_pt), Pm, mu, sd, shell_edges=g["shell_edges"], act="tanh", pool="mean",
                 ys=g["ys"], ym=g["ym"], mma=mma)
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


def serve_stream(rate=50.0, seconds=600.0, seed=4, ce_scale=1.0, nce_scale=1.0, nce_max_sites=1 << 20,
                 N_range=(256, 1 << 20), R_range=(8, 128), steps_range=(10_000, 1_000_000)):
    """Serving workload: Poisson arrivals at ``rate`` jobs/s for ``seconds``; model CE or NeuralCE 50/50; sites
    log-uniform in N_range rounded to 4 L^3 (NeuralCE cells capped at ``nce_max_sites``); Pt fraction ~ U[0.1, 0.9];
    replicas ~ U{8..128}; steps per replica log-uniform in steps_range, multiplied by ``ce_scale`` / ``nce_scale``.
    Returns a list of job descriptions (arrival time, kind, L, N, x_pt, R, steps, seed)."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= seconds:
            break
        kind = "ce" if rng.random() < 0.5 else "nce"
        N = float(np.exp(rng.uniform(np.log(N_range[0]), np.log(N_range[1]))))
        if kind == "nce":
            N = min(N, nce_max_sites)
        L = max(4, int(round((N / 4.0) ** (1.0 / 3.0))))
        x = float(rng.uniform(0.1, 0.9))
        R = int(rng.integers(R_range[0], R_range[1] + 1))
        steps = float(np.exp(rng.uniform(np.log(steps_range[0]), np.log(steps_range[1]))))
        steps = max(1, int(round(steps * (ce_scale if kind == "ce" else nce_scale))))
        jobs.append(dict(t=t, kind=kind, L=L, N=4 * L ** 3, x_pt=x, R=R, steps=steps, seed=int(rng.integers(1 << 62))))
    return jobs


def random_occupancy(N, x_pt, R, seed):
    """(R, N) int8 canonical occupancies of a binary fcc cell, each replica an independent random arrangement
    with round(x_pt N) Pt (species index 1)."""
    rng = np.random.default_rng(seed)
    n_pt = int(round(x_pt * N))
    base = np.zeros(N, np.int8); base[:n_pt] = 1
    return np.stack([rng.permutation(base) for _ in range(R)])


class ServeModels:
    """Per-cell models of the serving workload, built once and shared by every job on that cell (a job's model
    must stay valid while it runs; jobs on one CE model share the CE worker's stream)."""

    def __init__(self, depth=3, width=64, eci_seed=0, model_seed=0, mma=0):
        self.depth, self.width, self.eci_seed, self.model_seed, self.mma = depth, width, eci_seed, model_seed, mma
        self._ce, self._nce = {}, {}

    def ce(self, L):
        if L not in self._ce:
            from .ce import GPUClusterExpansion
            cs = cluster_space()
            s = fcc_conventional(A_FCC, (L, L, L))
            self._ce[L] = GPUClusterExpansion((cs, synthetic_eci(cs, self.eci_seed)), s, energy_scale=len(s))
        return self._ce[L]

    def nce(self, L):
        if L not in self._nce:
            from .nce import NCEModel, synthetic_model
            cs = cluster_space()
            s = fcc_conventional(A_FCC, (L, L, L))
            s.numbers = np.full(len(s), Z_OF["Ni"], np.int64)
            P = synthetic_model(len(cs.orbits) + 1, self.depth, self.width, 1, self.model_seed)
            self._nce[L] = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum", mma=self.mma)
        return self._nce[L]
