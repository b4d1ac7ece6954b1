"""GPU parity of the NeuralCE engine against the float64 oracle, through the C ABI.

Tolerances (float32 engine): energies within 2e-5 eV/atom of the oracle; per-swap dE within 1e-4 eV
(the stated NeuralCE bound) in eV of the total energy; occupancy trajectories on a seeded stream bit-exact except at
steps whose Metropolis margin |beta dE_eV + ln u| is below 1e-4 (counted: none occur for these seeds).
"""
import numpy as np
import pytest

from tests.conftest import l10_cell, random_cell

pytestmark = pytest.mark.gpu


def _model_pkl(mdl, s):
    from neuralce_gb300.ce_tables import ClusterSpace
    from neuralce_gb300.nce import NCEModel, expand_params
    from oracle.nce_oracle import NCEOracle
    cs = ClusterSpace.build(mdl["primitive"], mdl["cutoffs"])
    P, mu, sd = expand_params(mdl, 0)
    m = NCEModel(cs, s, P, mu, sd, shell_edges=mdl["shell_edges"], act="tanh", pool="mean", ys=mdl["ys"], ym=mdl["ym"])
    return m, NCEOracle(m.geo, P, mu, sd, act="tanh", pool="mean")


def _model_bench(L=3, seed=0, reps=None):
    from neuralce_gb300.nce import NCEModel, synthetic_model
    from neuralce_gb300.workloads import cluster_space
    from oracle.nce_oracle import NCEOracle
    cs = cluster_space()
    s = random_cell(reps or (L, L, L), seed)
    P = synthetic_model(len(cs.orbits) + 1, 3, 64, 1, 0)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum")
    return m, NCEOracle(m.geo, P, act="silu", pool="sum")


def test_full_cache_golden_L10(cuda, nipt_model):
    from neuralce_gb300.nce import NCEState
    mdl, g = nipt_model
    m, orc = _model_pkl(mdl, l10_cell())
    st = NCEState(m, m.sig0[None], np.ones(1)).full_cache()
    E = float(st.E[0].item()) * mdl["ys"] + mdl["ym"]
    assert abs(E - g["E_L10"]) < 2e-5, (E, g["E_L10"])


@pytest.mark.parametrize("which", ["pkl", "bench", "long"])
def test_full_cache_matches_oracle(cuda, nipt_model, which):
    """Full caches (layer 0 bit-sliced over 32-site words along the last cell axis) vs the oracle; "long" is a
    1 x 6 x 78 cell: three words per row, the last one ragged (14 sites)."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    if which == "pkl":
        m, orc = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 1))
    elif which == "long":
        m, orc = _model_bench(seed=4, reps=(3, 3, 13))
        assert tuple(m.geo["d"]) == (1, 6, 78)
    else:
        m, orc = _model_bench(3, 2)
    rng = np.random.default_rng(0)
    sig = np.stack([m.sig0[rng.permutation(m.N)] for _ in range(3)]).astype(np.int8)
    st = NCEState(m, sig, np.ones(3)).full_cache()
    torch.cuda.synchronize()
    for r in range(3):
        c = orc.full_cache(sig[r].astype(np.int64))
        assert abs(float(st.E[r]) - orc.energy_of(c)) * m.scale_eV < 1e-4 * max(1.0, m.N / 64)
        assert np.abs(st.h0[r].cpu().numpy() - c["h0"]).max() < 2e-5
        assert np.abs(st.e[r].cpu().numpy() - c["e"]).max() < 1e-4


@pytest.mark.parametrize("which,cluster", [("pkl", 1), ("bench", 1), ("pkl", 4), ("bench", 2)])
def test_local_chain_matches_oracle(cuda, nipt_model, which, cluster):
    """Every proposal accepted (force=1): per-step dE vs the oracle's local_delta chain, then the carried energy
    and the caches vs a full rebuild."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from oracle.nce_oracle import run_chain
    if which == "pkl":
        m, orc = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 3))
        T = 24
    else:
        m, orc = _model_bench(3, 4)
        T = 8
    rng = np.random.default_rng(7)
    pi = rng.integers(0, m.N, T).astype(np.int32); pj = rng.integers(0, m.N, T).astype(np.int32); pu = np.full(T, 0.5)
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    dE = torch.zeros((T, 1), dtype=torch.float64, device="cuda")
    props = tuple(torch.as_tensor(x.reshape(T, 1)).cuda() for x in (pi, pj, pu))
    st.run_chunk(T, 0, proposals=props, dE_out=dE, force=1, cluster=cluster)
    torch.cuda.synchronize()
    cache = orc.full_cache(m.sig0.astype(np.int64))
    E0 = orc.energy_of(cache)
    # oracle with every move accepted: beta = 0 and u = 0.5 accepts dE <= 0 and (u < 1) all others
    cache, sig, dsum, nacc, dEs, _ = run_chain(orc, cache, m.sig0, pi, pj, np.full(T, 0.5), 0.0, m.scale_eV)
    got = dE.cpu().numpy()[:, 0]
    assert np.abs((got - dEs) * m.scale_eV).max() < 1e-4, np.abs((got - dEs) * m.scale_eV).max()
    assert np.array_equal(st.sigma[0].cpu().numpy(), sig.astype(np.int8))
    Ecar = float(st.E[0].item())
    st2 = NCEState(m, st.sigma.cpu().numpy(), np.ones(1)).full_cache()
    torch.cuda.synchronize()
    assert abs(Ecar - float(st2.E[0].item())) * m.scale_eV < 1e-4
    assert abs(Ecar - (E0 + dsum)) * m.scale_eV < 1e-4
    assert np.abs(st.e[0].cpu().numpy() - st2.e[0].cpu().numpy()).max() < 1e-4
    assert int(st.n_acc[0].item()) == T


def _metropolis_vs_oracle(torch, m, orc, R, T, seed, cluster=1, temps=(500.0, 1400.0)):
    """Seeded host stream, Metropolis on R replicas over a geometric ladder: every step checked against the oracle
    (``trace_chain``): per-step dE within 1e-4 eV; decisions equal except at steps within the stated bound of
    their threshold, which the kernel counts in n_near; final occupancies equal the followed chain bit for bit."""
    from neuralce_gb300.nce import NCEState
    from oracle.nce_oracle import trace_chain
    beta = (1.0 / (8.617333e-5 * np.geomspace(temps[0], temps[1], R))).astype(np.float32)
    rng = np.random.default_rng(seed)
    sig = np.stack([m.sig0[rng.permutation(m.N)] for _ in range(R)]).astype(np.int8)
    pi = rng.integers(0, m.N, (T, R)).astype(np.int32); pj = rng.integers(0, m.N, (T, R)).astype(np.int32)
    pu = 1.0 - rng.random((T, R))
    st = NCEState(m, sig, beta).full_cache()
    dE = torch.zeros((T, R), dtype=torch.float64, device="cuda")
    st.run_chunk(T, 0, proposals=tuple(torch.as_tensor(x).cuda() for x in (pi, pj, pu)), dE_out=dE, cluster=cluster)
    torch.cuda.synchronize()
    m.check_errors()
    near_eV = 1e-2 if m.mma in (1, 2) else 1e-4
    dEg = dE.cpu().numpy()
    counted, excused = 0, 0
    for r in range(R):
        cache = orc.full_cache(sig[r].astype(np.int64))
        tr = trace_chain(orc, cache, sig[r], pi[:, r], pj[:, r], pu[:, r], float(beta[r]), m.scale_eV, dEg[:, r], near_eV)
        assert not tr["mismatch"], f"replica {r}: decisions differ away from the threshold at steps {tr['mismatch']}"
        assert np.abs((dEg[:, r] - tr["dE"]) * m.scale_eV).max() < (1e-2 if m.mma in (1, 2) else 1e-4)
        assert np.array_equal(st.sigma[r].cpu().numpy(), tr["sig"].astype(np.int8))
        assert int(st.n_acc[r].item()) == tr["nacc"]
        assert int(st.n_near[r].item()) == tr["near_engine"]
        counted += tr["near_engine"]; excused += len(tr["excused"])
    print(f"{R} x {T} steps: {counted} near-threshold steps counted, {excused} decisions excused")
    return counted


@pytest.mark.parametrize("which,cluster", [("pkl", 1), ("pkl", 4), ("bench", 1), ("bench", 2)])
def test_metropolis_trajectory_matches_oracle(cuda, nipt_model, which, cluster):
    """Metropolis chains of 4 replicas, 40 steps each, checked step by step against the oracle."""
    if which == "pkl":
        m, orc = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 5))
    else:
        m, orc = _model_bench(3, 5)
    _metropolis_vs_oracle(cuda, m, orc, 4, 40, 11, cluster)


def test_near_threshold_steps_are_counted(cuda, nipt_model):
    """A step planted near its threshold (u chosen from the oracle's dE so that the margin is 5e-5 eV, inside the
    1e-4 eV bound and beyond the float32 engine's dE error) is counted in n_near; a step 1e-2 eV away is not."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    m, orc = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 8))
    beta = np.array([1.0 / (8.617333e-5 * 800.0)], np.float32)
    sig = m.sig0.astype(np.int64)
    cache = orc.full_cache(sig)
    rng = np.random.default_rng(2)
    found = []
    while len(found) < 2:                                 # two swaps with dE_eV > 0.05 eV (u < 1 at the threshold)
        i, j = (int(x) for x in rng.integers(0, m.N, 2))
        if sig[i] == sig[j]:
            continue
        dE, _ = orc.local_delta(cache, sig, [(i, int(sig[j])), (j, int(sig[i]))])
        if dE * m.scale_eV > 0.05:
            found.append((i, j, dE * m.scale_eV))
    # step 0: margin +5e-5 eV (rejected, near); step 1: the same swap (state unchanged), margin +1e-2 eV (not near)
    (i, j, de), b = found[0], float(beta[0])
    u0 = np.exp(-b * (de - 5e-5)); u1 = np.exp(-b * (de - 1e-2))
    pi = np.array([[i], [i]], np.int32); pj = np.array([[j], [j]], np.int32); pu = np.array([[u0], [u1]])
    st = NCEState(m, sig[None].astype(np.int8), beta).full_cache()
    st.run_chunk(2, 0, proposals=tuple(torch.as_tensor(x).cuda() for x in (pi, pj, pu)))
    torch.cuda.synchronize()
    assert int(st.n_near[0].item()) == 1 and int(st.n_acc[0].item()) == 0


@pytest.mark.parametrize("cluster,per_sm,shipped", [(4, 1, False), (1, 2, False), (4, 2, False), (8, 2, False),
                                                   (4, 1, True), (8, 1, True)])
def test_cluster_equals_single_cta(cuda, nipt_model, cluster, per_sm, shipped):
    """Philox stream with exchanges: a replica spread over a cluster of CTAs, and CTAs sharing an SM two by two
    (128 registers a thread), give the same trajectory as one CTA per replica; the configuration-1 network and
    the reference's shipped model (three shells of up to 24 partners)."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from neuralce_gb300.workloads import ladder, replica_configs
    m, orc = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 6)) if shipped else _model_bench(3, 6)
    R = 4
    _, beta = ladder(R)
    sig = replica_configs(m.sig0, R, 3)
    a = NCEState(m, sig, beta).full_cache(); b = NCEState(m, sig, beta).full_cache()
    a.run_chunk(40, 0, seed=5, exchange_rounds=2, cluster=1)
    b.run_chunk(40, 0, seed=5, exchange_rounds=2, cluster=cluster, ctas_per_sm=per_sm)
    torch.cuda.synchronize()
    assert torch.equal(a.sigma, b.sigma) and torch.equal(a.rep_of_slot, b.rep_of_slot)
    assert torch.equal(a.n_acc, b.n_acc) and torch.allclose(a.E, b.E, rtol=0, atol=0)


def _model_bench_mma(L, seed, mma, width=64):
    from neuralce_gb300.nce import NCEModel, synthetic_model
    from neuralce_gb300.workloads import cluster_space
    from oracle.nce_oracle import NCEOracle
    cs = cluster_space()
    s = random_cell((L, L, L), seed)
    P = synthetic_model(len(cs.orbits) + 1, 3, width, 1, 0)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum", mma=mma)
    return m, NCEOracle(m.geo, P, act="silu", pool="sum")


@pytest.mark.parametrize("mma,width", [(3, 64), (3, 128), (1, 64), (3, 32), (4, 64), (4, 32), (4, 128), (2, 64),
                                       (2, 128), (2, 16)])
def test_tensor_core_forms_vs_oracle(cuda, mma, width):
    """Layer contractions on tensor cores (mma.sync: 1, 3; tcgen05 with tensor-memory accumulators: 2, 4).  The split
    bf16 forms (3, 4) -- the precision form -- stay within the NeuralCE per-swap bound of 1e-4 eV and the float32
    energy bound; at width 128 the tcgen05 split form stages its A operand in two K slices.  Plain bf16 operands
    (1, 2) are a labelled comparison point with their own stated bound of 1e-2 eV per swap (measured ~5e-3 eV on
    this model, whose total energy is ~1e2 eV).  A chain of forced moves keeps the carried energy equal to a rebuild
    of the caches in the same form."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from oracle.nce_oracle import run_chain
    m, orc = _model_bench_mma(3, 4, mma, width)
    tol_E, tol_dE = (1e-4 * max(1.0, m.N / 64), 1e-4) if mma in (3, 4) else (5e-1, 1e-2)
    rng = np.random.default_rng(3)
    sig = np.stack([m.sig0[rng.permutation(m.N)] for _ in range(2)]).astype(np.int8)
    st = NCEState(m, sig, np.ones(2)).full_cache()
    torch.cuda.synchronize()
    for r in range(2):
        c = orc.full_cache(sig[r].astype(np.int64))
        assert abs(float(st.E[r]) - orc.energy_of(c)) * m.scale_eV < tol_E, (float(st.E[r]), orc.energy_of(c))
    T = 8
    pi = rng.integers(0, m.N, T).astype(np.int32); pj = rng.integers(0, m.N, T).astype(np.int32)
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    dE = torch.zeros((T, 1), dtype=torch.float64, device="cuda")
    props = tuple(torch.as_tensor(x.reshape(T, 1)).cuda() for x in (pi, pj, np.full(T, 0.5)))
    st.run_chunk(T, 0, proposals=props, dE_out=dE, force=1)
    torch.cuda.synchronize()
    cache = orc.full_cache(m.sig0.astype(np.int64))
    _, sig_ref, _, _, dEs, _ = run_chain(orc, cache, m.sig0, pi, pj, np.full(T, 0.5), 0.0, m.scale_eV)
    err = np.abs((dE.cpu().numpy()[:, 0] - dEs) * m.scale_eV).max()
    print(f"mma {mma} width {width}: max |dE - oracle| = {err:.3e} eV")
    assert err < tol_dE, err
    assert np.array_equal(st.sigma[0].cpu().numpy(), sig_ref.astype(np.int8))
    Ecar = float(st.E[0].item())
    st2 = NCEState(m, st.sigma.cpu().numpy(), np.ones(1)).full_cache()
    torch.cuda.synchronize()
    assert abs(Ecar - float(st2.E[0].item())) * m.scale_eV < 1e-4 * max(1.0, m.N / 64)


@pytest.mark.parametrize("mma,width", [(3, 64), (4, 64), (2, 64), (4, 128)])
def test_tensor_core_cluster_equals_single_cta(cuda, mma, width):
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from neuralce_gb300.workloads import ladder, replica_configs
    m, _ = _model_bench_mma(3, 6, mma, width)
    _, beta = ladder(4)
    sig = replica_configs(m.sig0, 4, 3)
    a = NCEState(m, sig, beta).full_cache(); b = NCEState(m, sig, beta).full_cache()
    a.run_chunk(30, 0, seed=5, exchange_rounds=2, cluster=1)
    b.run_chunk(30, 0, seed=5, exchange_rounds=2, cluster=4)
    torch.cuda.synchronize()
    assert torch.equal(a.sigma, b.sigma) and torch.equal(a.rep_of_slot, b.rep_of_slot) and torch.equal(a.E, b.E)


@pytest.mark.parametrize("K,N", [(16, 64), (76, 64), (128, 64), (256, 64), (128, 128), (80, 128), (40, 16)])
def test_tc_gemm_matches_fp32(cuda, K, N):
    """The tcgen05 tile GEMM (bf16 operands in the core-matrix layout, float32 accumulation in tensor memory)
    against float64 products of the same bf16-rounded operands; the split form against the float64 product of
    the float32 operands (hi*hi + hi*lo + lo*hi drops lo*lo: ~2^-16 relative)."""
    torch = cuda
    from neuralce_gb300.nce import tc_gemm
    g = torch.Generator(device="cpu").manual_seed(K * 1000 + N)
    A = torch.randn(256, K, generator=g).cuda()
    B = (torch.randn(K, N, generator=g) / K ** 0.5).cuda()
    C = tc_gemm(A, B)
    ref = (A.bfloat16().double() @ B.bfloat16().double())
    scale = (A.abs().double() @ B.abs().double())
    assert ((C.double() - ref).abs() <= 1e-5 * scale + 1e-6).all(), float((C.double() - ref).abs().max())
    Cs = tc_gemm(A, B, split=True)
    ref64 = A.double() @ B.double()
    err = ((Cs.double() - ref64).abs() / (scale + 1e-30)).max().item()
    assert err < 2e-5, err
    # the plain bf16 form is much further from the float32 product than the split form
    err1 = ((C.double() - ref64).abs() / (scale + 1e-30)).max().item()
    assert err1 > 4 * err


def test_two_ctas_per_sm_refused_when_too_large(cuda, nipt_model):
    """The shipped model's tiles (73 partner rows per site) need more than half an SM's shared memory: a chunk
    asking for two CTAs per SM fails with a message and changes nothing."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.nce import NCEState
    m, _ = _model_pkl(nipt_model[0], random_cell((4, 4, 4), 6))
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    sig0 = st.sigma.clone()
    with pytest.raises(_lib.NceError, match="shared memory"):
        st.run_chunk(10, 0, seed=1, cluster=2, ctas_per_sm=2)
    torch.cuda.synchronize()
    assert torch.equal(st.sigma, sig0)


def test_out_of_range_proposal_is_reported(cuda):
    """A host proposal naming a site outside the cell is turned into a no-op by the kernel's bounds check and
    reported: check_errors raises NceError once, naming the flag, and clears it; the chain equals the one where
    that proposal picks the same site twice."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.nce import NCEState
    from neuralce_gb300.workloads import ladder, replica_configs
    m, _ = _model_bench(3, 9)
    R, T = 3, 30
    _, beta = ladder(R)
    sig = replica_configs(m.sig0, R, 4)
    rng = np.random.default_rng(2)
    pi = rng.integers(0, m.N, (T, R)).astype(np.int32); pj = rng.integers(0, m.N, (T, R)).astype(np.int32)
    pu = 1.0 - rng.random((T, R))
    bad = pi.copy(); bad[11, 1] = m.N
    same = pj.copy(); same[11, 1] = pi[11, 1]
    a = NCEState(m, sig, beta).full_cache(); b = NCEState(m, sig, beta).full_cache()
    a.run_chunk(T, 0, proposals=tuple(torch.as_tensor(x).cuda() for x in (bad, pj, pu)))
    torch.cuda.synchronize()
    with pytest.raises(_lib.NceError, match="proposal index was out of range"):
        m.check_errors()
    m.check_errors()
    b.run_chunk(T, 0, proposals=tuple(torch.as_tensor(x).cuda() for x in (pi, same, pu)))
    torch.cuda.synchronize()
    m.check_errors()
    assert torch.equal(a.sigma, b.sigma) and torch.equal(a.E, b.E) and torch.equal(a.n_acc, b.n_acc)


def _ternary_model(seed=1, mma=0):
    from neuralce_gb300.ce_tables import ClusterSpace
    from neuralce_gb300.io import Z_OF, fcc_conventional, fcc_primitive
    from neuralce_gb300.nce import NCEModel, synthetic_model
    from oracle.nce_oracle import NCEOracle
    cs = ClusterSpace.build(fcc_primitive(3.924, ("Ni", "Pt", "Cu")), [6.0, 4.5])
    s = fcc_conventional(3.924, (3, 3, 3))
    r = np.random.RandomState(seed)
    s.numbers = np.array([Z_OF[x] for x in r.choice(["Ni", "Pt", "Cu"], len(s))], np.int64)
    P = synthetic_model(len(cs.orbits) + 1, 2, 32, 1, 0)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum", mma=mma)
    return m, NCEOracle(m.geo, P, act="silu", pool="sum")


@pytest.mark.parametrize("cluster", [1, 4])
def test_ternary_point_functions(cuda, cluster):
    """Three species per site: point functions -cos(2 pi s / 3) are not +-1, so layer 0 runs the general float64
    row products (full cache) and the int64 fixed-point row changes (step).  Full cache and a forced-move chain
    against the oracle; a cluster of CTAs equals one CTA."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from oracle.nce_oracle import run_chain
    m, orc = _ternary_model()
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    torch.cuda.synchronize()
    c = orc.full_cache(m.sig0.astype(np.int64))
    assert np.abs(st.h0[0].cpu().numpy() - c["h0"]).max() < 2e-5
    assert abs(float(st.E[0]) - orc.energy_of(c)) * m.scale_eV < 1e-4 * max(1.0, m.N / 64)
    T = 10
    rng = np.random.default_rng(8)
    pi = rng.integers(0, m.N, T).astype(np.int32); pj = rng.integers(0, m.N, T).astype(np.int32)
    dE = torch.zeros((T, 1), dtype=torch.float64, device="cuda")
    props = tuple(torch.as_tensor(x.reshape(T, 1)).cuda() for x in (pi, pj, np.full(T, 0.5)))
    st.run_chunk(T, 0, proposals=props, dE_out=dE, force=1, cluster=cluster)
    torch.cuda.synchronize()
    _, sig_ref, _, _, dEs, _ = run_chain(orc, c, m.sig0, pi, pj, np.full(T, 0.5), 0.0, m.scale_eV)
    assert np.abs((dE.cpu().numpy()[:, 0] - dEs) * m.scale_eV).max() < 1e-4
    assert np.array_equal(st.sigma[0].cpu().numpy(), sig_ref.astype(np.int8))
    m.check_errors()


@pytest.mark.parametrize("mma,width", [(0, 64), (4, 64), (4, 128), (3, 128)])
def test_config_cell_chain_matches_oracle(cuda, mma, width):
    """The configuration-1 cell itself (8 x 8 x 8 conventional fcc, 2,048 sites: receptive fields of 141 / 321 / 603
    / 1,007 sites that no longer wrap onto themselves), depth 3, SiLU, sum readout, at width 64 (configuration 1)
    and 128 (configuration 3's width): 16 forced moves against the oracle's local_delta chain, per step within
    1e-4 eV, then carried energy vs a rebuild of the caches."""
    torch = cuda
    from neuralce_gb300.nce import NCEState
    from oracle.nce_oracle import run_chain
    m, orc = _model_bench_mma(8, 4, mma, width)
    assert m.N == 2048
    T = 16
    rng = np.random.default_rng(9)
    pi = rng.integers(0, m.N, T).astype(np.int32); pj = rng.integers(0, m.N, T).astype(np.int32)
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    dE = torch.zeros((T, 1), dtype=torch.float64, device="cuda")
    props = tuple(torch.as_tensor(x.reshape(T, 1)).cuda() for x in (pi, pj, np.full(T, 0.5)))
    st.run_chunk(T, 0, proposals=props, dE_out=dE, force=1, cluster=2)
    torch.cuda.synchronize()
    m.check_errors()
    cache = orc.full_cache(m.sig0.astype(np.int64))
    E0 = orc.energy_of(cache)
    cache, sig_ref, dsum, _, dEs, _ = run_chain(orc, cache, m.sig0, pi, pj, np.full(T, 0.5), 0.0, m.scale_eV)
    err = np.abs((dE.cpu().numpy()[:, 0] - dEs) * m.scale_eV).max()
    print(f"2048 sites, mma {mma}, width {width}: max |dE - oracle| = {err:.3e} eV")
    assert err < 1e-4, err
    assert np.array_equal(st.sigma[0].cpu().numpy(), sig_ref.astype(np.int8))
    Ecar = float(st.E[0].item())
    E0g = float(NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache().E[0].item())
    # energies of the whole cell: float32 site energies summed over 2,048 sites (the bound scales with N, as above)
    assert abs(E0g - E0) * m.scale_eV < 1e-4 * m.N / 64
    assert abs(Ecar - (E0g + float(dE.sum().item()))) * m.scale_eV < 1e-9
    st2 = NCEState(m, st.sigma.cpu().numpy(), np.ones(1)).full_cache()
    torch.cuda.synchronize()
    assert abs(Ecar - float(st2.E[0].item())) * m.scale_eV < 1e-3
    assert abs(float(st2.E[0].item()) - (E0 + dsum)) * m.scale_eV < 1e-4 * m.N / 64
    assert np.abs(st2.e[0].cpu().numpy() - cache["e"]).max() < 1e-4


@pytest.mark.parametrize("mma,width,cluster", [(0, 64, 4), (4, 64, 8), (4, 128, 4)])
def test_config_cell_metropolis_matches_oracle(cuda, mma, width, cluster):
    """Metropolis chains of 4 replicas on the 2,048-site configuration-1 cell, checked step by step against the
    oracle (decisions equal except at counted near-threshold steps; occupancies bit-exact)."""
    m, orc = _model_bench_mma(8, 5, mma, width)
    _metropolis_vs_oracle(cuda, m, orc, 4, 24, 13, cluster)


def test_tensor_core_wait_timeout_is_reported(cuda):
    """A tensor-core completion wait that nothing completes (no MMA issued) gives up after a bounded number of polls:
    the kernel returns, flag 32 reaches check_errors() as an NceError, the flags clear, and the context stays usable
    (a tcgen05 chunk afterwards still matches its float32 counterpart within the bf16 bound)."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.nce import NCEState
    m, _ = _model_bench_mma(3, 4, 2, 32)
    _lib.check(_lib.lib().nce_nce_tc_wait_selftest(m.handle, 1000, _lib.stream_ptr()), "nce_nce_tc_wait_selftest")
    torch.cuda.synchronize()
    with pytest.raises(_lib.NceError, match="tensor-core completion wait timed out"):
        m.check_errors()
    m.check_errors()                                       # cleared
    st = NCEState(m, m.sig0[None].astype(np.int8), np.ones(1)).full_cache()
    st.run_chunk(4, 0, seed=3, force=1)
    torch.cuda.synchronize()
    m.check_errors()
    Ecar = float(st.E[0].item())
    assert abs(Ecar - float(NCEState(m, st.sigma.cpu().numpy(), np.ones(1)).full_cache().E[0].item())) < 1e-3
