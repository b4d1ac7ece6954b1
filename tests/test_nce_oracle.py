"""CPU tests of the NeuralCE oracle and host geometry, pinned by the reference's exact-enumeration energy, and the
reference's local-update checks (tests/test_nce_local_update.py: local dE == full-recompute difference, chained
cache == full rebuild, float64 1e-9)."""
import numpy as np
import pytest

from tests.conftest import l10_cell, random_cell


def _oracle(mdl, s):
    from neuralce_gb300.ce_tables import ClusterSpace
    from neuralce_gb300.nce import expand_params
    from neuralce_gb300.nce_geometry import build_geometry
    from oracle.nce_oracle import NCEOracle
    cs = ClusterSpace.build(mdl["primitive"], mdl["cutoffs"])
    P, mu, sd = expand_params(mdl, 0)
    geo = build_geometry(cs, s, mdl["shell_edges"], len(P["layers"]))
    return NCEOracle(geo, P, mu, sd, act="tanh", pool="mean"), geo


def test_golden_exact_enumeration_L10(nipt_model):
    mdl, g = nipt_model
    orc, geo = _oracle(mdl, l10_cell())
    E = orc.energy(geo["sig"]) * mdl["ys"] + mdl["ym"]
    assert abs(E - g["E_L10"]) < 1e-12, (E, g["E_L10"])


def test_oracle_expand_params_matches_package(nipt_model):
    from neuralce_gb300.nce import expand_params as pkg
    from oracle.nce_oracle import expand_params as orc
    mdl, _ = nipt_model
    a, mu1, sd1 = pkg(mdl, 0); b, mu2, sd2 = orc(mdl, 0)
    assert np.array_equal(a["lin"], b["lin"]) and np.array_equal(mu1, mu2) and np.array_equal(sd1, sd2)


def _chain_check(orc, geo, n, seed, tol=1e-9):
    sig = geo["sig"].astype(np.int64).copy()
    cache = orc.full_cache(sig); E = orc.energy_of(cache)
    rng = np.random.RandomState(seed)
    act = np.arange(geo["N"])
    done = 0
    while done < n:
        i, j = (int(x) for x in rng.choice(act, 2, replace=False))
        if sig[i] == sig[j]:
            continue
        dE, patch = orc.local_delta(cache, sig, [(i, int(sig[j])), (j, int(sig[i]))])
        sig1 = sig.copy(); sig1[i], sig1[j] = sig[j], sig[i]
        E1 = orc.energy(sig1)
        assert abs(dE - (E1 - E)) < tol, (dE, E1 - E)
        cache = orc.commit(cache, patch, True); sig = sig1; E = E1
        done += 1
    full = orc.full_cache(sig)
    assert abs(orc.energy_of(cache) - orc.energy_of(full)) < tol
    for l in range(len(cache["hmid"])):
        assert np.abs(cache["hmid"][l] - full["hmid"][l]).max() < tol
    assert np.abs(cache["e"] - full["e"]).max() < tol


def test_local_delta_equals_full_recompute_reference_model(nipt_model):
    mdl, _ = nipt_model
    orc, geo = _oracle(mdl, random_cell((4, 4, 4), 1))
    _chain_check(orc, geo, 10, 0)


def test_local_delta_equals_full_recompute_benchmark_model():
    """depth 3, width 64, SiLU, sum readout, one 12-neighbour shell, config-0 cluster set (38 channels)."""
    from neuralce_gb300.nce import synthetic_model
    from neuralce_gb300.nce_geometry import build_geometry
    from neuralce_gb300.workloads import cluster_space
    from oracle.nce_oracle import NCEOracle
    cs = cluster_space()
    s = random_cell((3, 3, 3), 2)
    P = synthetic_model(len(cs.orbits) + 1, 3, 64, 1, 0)
    geo = build_geometry(cs, s, [0.0, 3.3], 3)
    assert geo["W"] == 12
    orc = NCEOracle(geo, P, act="silu", pool="sum")
    _chain_check(orc, geo, 4, 3)
