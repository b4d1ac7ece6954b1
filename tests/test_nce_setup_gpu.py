"""The reference's NeuralCE ``setup()`` interface on the engine (``neuralce/nce/mc_model.py:175-228``):
``full_cache`` / ``local_delta`` / ``commit`` / ``propose`` / ``energy_of`` through the C ABI's nce_nce_local_delta and
nce_nce_commit.  The first test is the reference's own check (``tests/test_nce_local_update.py:27-53``: 30 swaps on a
256-atom cell, local dE == difference of two full energies, chained cache == rebuild) run through those keys, with
the float64 oracle beside it.  Tolerances are the float32 engine's: dE within 1e-4 eV of the total energy."""
import numpy as np
import pytest

from tests.conftest import random_cell

pytestmark = pytest.mark.gpu


def _oracle(mc, mdl, k=0):
    from neuralce_gb300.nce import expand_params
    from oracle.nce_oracle import NCEOracle
    P, mu, sd = expand_params(mdl, k)
    return NCEOracle(mc["model"].geo, P, mu, sd, act="tanh", pool="mean")


def test_setup_local_delta_commit_chain(cuda, nipt_model):
    torch = cuda
    from neuralce_gb300.nce import setup
    mdl, _ = nipt_model
    mc = setup(mdl, random_cell((4, 4, 4), 2))
    N = mc["n_atoms"]; assert N == 256
    to_eV = mc["ys"] * N                                   # dE in the model's units -> eV of the cell
    orc = _oracle(mc, mdl)
    sig = np.asarray(mc["sig0"], np.int64).copy()
    cache = mc["full_cache"](sig); ocache = orc.full_cache(sig)
    e_i = mc["energy_of"](cache)
    assert abs(e_i - orc.energy_of(ocache)) * to_eV < 1e-4
    rng = np.random.default_rng(0)
    worst_full = worst_orc = 0.0; n = 0
    for _ in range(200):
        i, j = (int(x) for x in rng.choice(N, 2, replace=False))
        if sig[i] == sig[j]:
            continue
        flips = np.array([[i, sig[j]], [j, sig[i]]])
        dE, patch, sig_back = mc["local_delta"](cache, sig, flips)
        assert sig_back is sig
        sig1 = sig.copy(); sig1[i], sig1[j] = sig[j], sig[i]
        E1 = mc["energy_of"](mc["full_cache"](sig1))
        dEo, opatch = orc.local_delta(ocache, sig, [(i, int(sig[j])), (j, int(sig[i]))])
        worst_full = max(worst_full, abs(float(dE) - (E1 - e_i)) * to_eV)
        worst_orc = max(worst_orc, abs(float(dE) - dEo) * to_eV)
        cache = mc["commit"](cache, patch, True); ocache = orc.commit(ocache, opatch, True)
        sig = sig1; e_i = E1; n += 1
        if n == 30:
            break
    assert n == 30
    print(f"30 swaps: max |dE - full difference| = {worst_full:.2e} eV, max |dE - oracle| = {worst_orc:.2e} eV")
    assert worst_full < 1e-4 and worst_orc < 1e-4
    assert np.array_equal(cache.sigma.cpu().numpy(), sig.astype(np.int8))
    rebuilt = mc["full_cache"](sig)
    assert abs(mc["energy_of"](cache) - mc["energy_of"](rebuilt)) * to_eV < 1e-4
    assert np.abs(cache.states[0].e[0].cpu().numpy() - rebuilt.states[0].e[0].cpu().numpy()).max() < 1e-5
    assert int(cache.states[0].n_acc[0].item()) == 30


def test_setup_rejected_commit_and_stale_patch(cuda, nipt_model):
    """commit(accept=False) leaves the cache and occupancy unchanged; a patch replaced by a later local_delta is
    refused instead of committing the wrong swap."""
    from neuralce_gb300.nce import setup
    mdl, _ = nipt_model
    mc = setup(mdl, random_cell((4, 4, 4), 3))
    sig = np.asarray(mc["sig0"], np.int64).copy()
    cache = mc["full_cache"](sig)
    e0 = mc["energy_of"](cache)
    a, b = int(np.flatnonzero(sig == 0)[3]), int(np.flatnonzero(sig == 1)[5])
    dE, patch, _ = mc["local_delta"](cache, sig, [[a, sig[b]], [b, sig[a]]])
    mc["commit"](cache, patch, False)
    assert mc["energy_of"](cache) == e0 and np.array_equal(cache.sigma.cpu().numpy(), sig.astype(np.int8))
    _, p1, _ = mc["local_delta"](cache, sig, [[a, sig[b]], [b, sig[a]]])
    _, p2, _ = mc["local_delta"](cache, sig, [[b, sig[a]], [a, sig[b]]])
    with pytest.raises(RuntimeError, match="no longer held"):
        mc["commit"](cache, p1, True)
    mc["commit"](cache, p2, True)
    assert abs(mc["energy_of"](cache) - (e0 + float(dE))) < 1e-6
    with pytest.raises(ValueError, match="swaps"):
        mc["local_delta"](cache, sig, [[a, sig[a]], [b, sig[b]]])


def test_setup_propose_is_the_kernels_draw(cuda, nipt_model):
    """propose((seed, step, slot)) returns the pair the chunk kernel draws for that slot at that step: one forced
    step of a Philox chunk swaps exactly those two sites."""
    torch = cuda
    from neuralce_gb300.nce import NCEState, setup
    mdl, _ = nipt_model
    mc = setup(mdl, random_cell((4, 4, 4), 4))
    m = mc["model"]
    sig = np.asarray(mc["sig0"], np.int8)
    checked = 0
    for g in range(40):
        i, j = mc["propose"]((77, g, 0))
        assert 0 <= i < m.N and 0 <= j < m.N
        st = NCEState(m, sig[None], np.ones(1)).full_cache()
        st.run_chunk(1, g, seed=77, force=1)
        torch.cuda.synchronize()
        got = st.sigma[0].cpu().numpy()
        want = sig.copy(); want[i], want[j] = sig[j], sig[i]
        assert np.array_equal(got, want)
        checked += sig[i] != sig[j]
    assert checked > 5


def test_setup_ensemble_is_the_mean_of_the_seeds(cuda, nipt_model):
    """seed_idx = -1 (the reference's ensemble): energy and every local dE are the mean over the trained seeds' models
    (a second seed is made here by perturbing the shipped weights)."""
    import copy
    from neuralce_gb300.nce import setup
    mdl, _ = nipt_model
    mdl2 = copy.deepcopy(mdl)
    p1 = copy.deepcopy(mdl["params"][0]); rng = np.random.default_rng(1)
    for L in p1["layers"]:
        for k in L:
            L[k] = np.asarray(L[k]) * (1.0 + 0.05 * rng.standard_normal(np.shape(L[k])))
    mdl2["params"] = [mdl["params"][0], p1]
    atoms = random_cell((4, 4, 4), 5)
    ens = setup(mdl2, atoms, seed_idx=-1)
    one = [setup(mdl2, atoms, seed_idx=k) for k in (0, 1)]
    assert ens["ensemble"] and len(ens["models"]) == 2
    sig = np.asarray(ens["sig0"], np.int64)
    assert abs(ens["energy"](sig) - np.mean([o["energy"](sig) for o in one])) < 1e-6
    ce, c0, c1 = ens["full_cache"](sig), one[0]["full_cache"](sig), one[1]["full_cache"](sig)
    a, b = int(np.flatnonzero(sig == 0)[1]), int(np.flatnonzero(sig == 1)[2])
    fl = [[a, sig[b]], [b, sig[a]]]
    de = float(ens["local_delta"](ce, sig, fl)[0])
    d0, d1 = float(one[0]["local_delta"](c0, sig, fl)[0]), float(one[1]["local_delta"](c1, sig, fl)[0])
    assert abs(de - 0.5 * (d0 + d1)) < 1e-9


def _two_seed_model(mdl):
    import copy
    mdl2 = copy.deepcopy(mdl)
    p1 = copy.deepcopy(mdl["params"][0]); rng = np.random.default_rng(1)
    for L in p1["layers"]:
        for k in L:
            L[k] = np.asarray(L[k]) * (1.0 + 0.05 * rng.standard_normal(np.shape(L[k])))
    mdl2["params"] = [mdl["params"][0], p1]
    return mdl2


def test_ensemble_chain_matches_oracle(cuda, nipt_model):
    """seed_idx = -1 chains of 3 replicas (device local_delta on both seeds' models, accept on the mean dE, commit on
    both) against the oracle's two models driven with the same proposals, uniforms and rule: occupancies bit-exact,
    energies within the float32 bound; then a chunk-end exchange on the mean energies."""
    torch = cuda
    from neuralce_gb300.nce import expand_params, proposal_block, setup
    from neuralce_gb300.workloads import ladder
    from oracle.nce_oracle import NCEOracle
    mdl, _ = nipt_model
    mdl2 = _two_seed_model(mdl)
    mc = setup(mdl2, random_cell((4, 4, 4), 6), seed_idx=-1)
    R, T, seed = 3, 25, 17
    _, beta = ladder(R, 500.0, 1200.0)
    rng = np.random.default_rng(2)
    sig = np.stack([mc["sig0"][rng.permutation(mc["n_atoms"])] for _ in range(R)]).astype(np.int8)
    st = mc["new_state"](sig, beta).full_cache()
    st.run_chunk(T, 0, seed=seed)
    torch.cuda.synchronize()
    st.check_errors()
    orcs = []
    for k in range(2):
        P, mu, sd = expand_params(mdl2, k)
        orcs.append(NCEOracle(mc["model"].geo, P, mu, sd, act="tanh", pool="mean"))
    pi, pj, pu = proposal_block(mc["model"], seed, 0, T, np.arange(R))
    scale = mc["model"].scale_eV
    for r in range(R):
        s = sig[r].astype(np.int64).copy()
        caches = [o.full_cache(s) for o in orcs]
        E = np.mean([o.energy_of(c) for o, c in zip(orcs, caches)])
        nacc = 0
        for k in range(T):
            i, j = int(pi[k, r]), int(pj[k, r])
            if s[i] == s[j]:
                nacc += 1; continue
            out = [o.local_delta(c, s, [(i, int(s[j])), (j, int(s[i]))]) for o, c in zip(orcs, caches)]
            dEeV = np.mean([d for d, _ in out]) * scale
            if dEeV <= 0 or pu[k, r] < np.exp(-float(beta[r]) * dEeV):
                caches = [o.commit(c, p, True) for o, c, (_, p) in zip(orcs, caches, out)]
                s[i], s[j] = s[j], s[i]; nacc += 1; E += dEeV / scale
        assert np.array_equal(st.sigma[r].cpu().numpy(), s.astype(np.int8))
        assert int(st.n_acc[r].item()) == nacc
        assert abs(float(st.E[r].item()) - E) * scale < 1e-4
    # a chunk that ends with exchange rounds keeps every model's slots in step
    st.run_chunk(5, T, seed=seed, exchange_rounds=2)
    torch.cuda.synchronize()
    for s_ in st.states[1:]:
        assert torch.equal(s_.rep_of_slot, st.rep_of_slot) and torch.equal(s_.sigma, st.sigma)


def test_ensemble_driver_runs(cuda, nipt_model, tmp_path):
    """The NeuralCE PT driver with seed_idx = -1 (the CLI's --model_seed -1) runs and writes its outputs."""
    from neuralce_gb300.mc import nce_mc
    mdl, _ = nipt_model
    res = nce_mc.run_pt_mc(_two_seed_model(mdl), random_cell((3, 3, 3), 7), n_steps=60, T_min=500.0, T_max=1500.0,
                           n_replicas=3, exchange_every=20, chunk=30, sample_interval=10, seed_idx=-1,
                           out_dir=str(tmp_path))
    assert (tmp_path / "energies.npz").exists() and (tmp_path / "final_sigma.npy").exists()
    assert res["n_replicas"] == 3 and np.isfinite(res["E_final"]).all()
