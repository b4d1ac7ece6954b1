"""Thermodynamic estimates from parallel-tempering energy series: <E>(T), C_V(T) and their standard errors.

The reference's analysis (``scripts/bench/ptni_exact_pt_analyze.py:36-60``) compares per-temperature means and
variances of the sampled energies with an exact enumeration.  Here, per temperature slot:

* burn-in: the first ``burn`` fraction of the samples is dropped;
* statistical inefficiency g = 1 + 2 sum_t rho(t), summed up to the first window M with M >= c g(M) (Sokal's
  automatic windowing, A. D. Sokal, "Monte Carlo methods in statistical mechanics", 1997), with the
  autocorrelation from an FFT of the zero-padded series;
* <E> per atom with standard error sqrt(g var / n), and the same error from ``blocks`` batch means; the larger
  of the two is reported;
* C_V = N beta^2 var(e) in k_B per atom (e the energy per atom), its error from the batch means of C_V.
"""
from __future__ import annotations

import numpy as np

KB = 8.617333262e-5


def stat_ineff(x, c=6.0):
    x = np.asarray(x, np.float64)
    n = len(x)
    x = x - x.mean()
    v = float(x @ x)
    if n < 8 or v <= 0.0:
        return 1.0
    nf = 1 << int(np.ceil(np.log2(2 * n)))
    f = np.fft.rfft(x, nf)
    acf = np.fft.irfft(f * np.conj(f), nf)[:n]
    acf /= acf[0]
    g = 2.0 * np.cumsum(acf) - 1.0
    ok = np.arange(n) >= c * g
    w = int(np.argmax(ok)) if ok.any() else n - 1
    return float(max(g[w], 1.0))


def batch_means(x, blocks):
    L = len(x) // blocks
    if L < 2:
        return None
    return np.asarray(x[:blocks * L], np.float64).reshape(blocks, L)


def estimates(traj, temps, N, burn=0.2, blocks=16):
    """traj (R, S) energies per atom (eV) of each temperature slot, temps (R,) K -> dict of arrays."""
    traj = np.asarray(traj, np.float64)
    R, S = traj.shape
    s0 = int(burn * S)
    out = {k: np.zeros(R) for k in ("E", "E_se", "Cv", "Cv_se", "g", "n")}
    for r in range(R):
        x = traj[r, s0:]
        beta = 1.0 / (KB * float(temps[r]))
        g = stat_ineff(x)
        n = len(x)
        m = float(x.mean())
        se_g = float(np.sqrt(g * x.var() / n))
        b = batch_means(x, blocks)
        se_b = float(b.mean(1).std(ddof=1) / np.sqrt(blocks)) if b is not None else np.inf
        cv = N * beta ** 2 * float(x.var())
        cv_b = N * beta ** 2 * b.var(1) if b is not None else None
        cv_se = float(cv_b.std(ddof=1) / np.sqrt(blocks)) if cv_b is not None else np.inf
        out["E"][r], out["E_se"][r], out["Cv"][r], out["Cv_se"][r] = m, max(se_g, se_b), cv, cv_se
        out["g"][r], out["n"][r] = g, n
    return out
