"""GPU parity of the CE engine against the C oracle (float64), through the C-ABI.

Tolerances: float64 kernel dE within 1e-10 eV of the oracle (only the summation order differs); float32
kernel dE within 1e-6 eV (the stated CE bound).  Occupancy trajectories on a seeded stream are bit-exact.  A step
is near its threshold when its Metropolis margin |dE + ln(u) / beta| is below the precision form's stated dE bound
(1e-9 eV at float64, 1e-6 eV at float32): only there could a decision differ from the oracle's.  The kernels
count such steps (``n_near``) and the oracle counts them with the same definition; the trajectory tests require
the counts to agree, and ``test_near_threshold_steps_are_counted`` plants steps on both sides of the band.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(L, seed=0, R=4):
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    from oracle.ce_oracle import OracleCE
    gce, sig = ce_config(L, seed=seed)
    orc = OracleCE(gce.info)
    sig_r = replica_configs(sig, R, seed + 1)
    _, beta = ladder(R)
    return gce, orc, sig_r, beta


@pytest.mark.parametrize("L", [2, 3, 8])
def test_energy_matches_oracle(cuda, L):
    torch = cuda
    gce, orc, sig_r, _ = _setup(L)
    E = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
    E32 = gce.batched_energy(torch.as_tensor(sig_r).cuda(), precision=32).cpu().numpy()
    for r in range(len(sig_r)):
        e = orc.energy(sig_r[r])
        assert abs(E[r] - e) < 1e-10 * max(1.0, abs(e)), (E[r], e)
        assert abs(E32[r] - e) < 1e-5, (E32[r], e)


@pytest.mark.parametrize("L,warps", [(2, 8), (3, 4), (8, 8), (8, 32)])
def test_delta_matches_oracle(cuda, L, warps):
    """Random swaps (L=2: the 8 A pair shell wraps onto periodic images of the 16-site cell)."""
    torch = cuda
    gce, orc, sig_r, _ = _setup(L)
    rng = np.random.default_rng(L * 100 + warps)
    N = gce.n_atoms
    q = []
    while len(q) < 200:
        r = int(rng.integers(0, len(sig_r))); ia, ib = (int(x) for x in rng.integers(0, N, 2))
        if sig_r[r, ia] != sig_r[r, ib]:
            q.append((r, ia, ib))
    rep, ia, ib = (np.array(x) for x in zip(*q))
    sa_new = sig_r[rep, ib]; sb_new = sig_r[rep, ia]
    sd = torch.as_tensor(sig_r).cuda()
    d64 = gce.delta_energy_batch(sd, rep, ia, ib, sa_new, sb_new, precision=64, warps=warps).cpu().numpy()
    d32 = gce.delta_energy_batch(sd, rep, ia, ib, sa_new, sb_new, precision=32, warps=warps).cpu().numpy()
    want = np.array([orc.delta(sig_r[r], a, b, sa, sb) for r, a, b, sa, sb in zip(rep, ia, ib, sa_new, sb_new)])
    assert np.abs(d64 - want).max() < 1e-10
    assert np.abs(d32 - want).max() < 1e-6


def _engine_state(sig_r, E, beta):
    from neuralce_gb300.pt import PTState
    return PTState(sig_r, E, beta, np.zeros(len(beta), np.int32))


def _compare(st, ref, E_tol):
    assert np.array_equal(st.n_near.cpu().numpy(), ref["n_near"]), (st.n_near.cpu().numpy(), ref["n_near"])
    assert np.array_equal(st.sigma.cpu().numpy(), ref["sigma"])
    assert np.abs(st.E.cpu().numpy() - ref["E"]).max() < E_tol
    assert np.array_equal(st.n_acc.cpu().numpy(), ref["n_acc"])
    assert np.array_equal(st.rep_of_slot.cpu().numpy(), ref["rep_of_slot"])
    assert np.array_equal(st.slot_of_rep.cpu().numpy(), ref["slot_of_rep"])
    assert int(st.n_ex.item()) == int(ref["n_ex"][0])


@pytest.mark.parametrize("precision,path,warps,cluster", [(64, 1, 8, 1), (32, 1, 8, 1), (64, 2, 8, 1), (32, 2, 4, 1),
                                                          (64, 2, 1, 1), (64, 2, 8, 2), (32, 2, 4, 4), (64, 2, 16, 8),
                                                          (32, 2, 16, 2)])
def test_trajectory_host_stream(cuda, precision, path, warps, cluster):
    """Seeded host proposal stream + exchange uniforms: bit-exact occupancy trajectory, energies, acceptance,
    slot permutation and slot-ordered samples vs the oracle (cluster > 1: each replica spread over that many
    CTAs of a thread-block cluster)."""
    torch = cuda
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T, si = 8, 1500, 50
    gce, orc, sig_r, beta = _setup(8, seed=3, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta)
    ref = new_state(sig_r, E0, beta)
    step = 0
    for chunk in range(2):
        pa, pb, pu = proposal_stream(gce, R, T, seed=10 + chunk)
        exu = np.random.default_rng(50 + chunk).random((R - 1 + 1) // 2)
        exu = 1.0 - exu
        par = chunk % 2
        Es = torch.zeros((T // si, R), dtype=torch.float64, device="cuda")
        dev = tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))
        run_chunk(gce, st, T, step, 0, precision, warps, dev, si, Es, True, par, torch.as_tensor(exu).cuda(), path=path,
                  cluster=cluster)
        Es_ref = np.zeros((T // si, R))
        orc.run(ref, T, step, 0, (pa, pb, pu), si, Es_ref, True, par, exu, n_threads=4,
                near_eV=1e-9 if precision == 64 else 1e-6)
        torch.cuda.synchronize()
        tol = 1e-9 if precision == 64 else 1e-4
        _compare(st, ref, tol)
        assert np.abs(Es.cpu().numpy() - Es_ref).max() < tol
        step += T
    assert int(st.n_acc.sum()) > 0


@pytest.mark.parametrize("path", [1, 2])
def test_trajectory_philox_multichunk(cuda, path):
    """Device Philox stream, 3 chunks with exchanges: equals the oracle's Philox restatement."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 16, 1000
    gce, orc, sig_r, beta = _setup(4, seed=5, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta); ref = new_state(sig_r, E0, beta)
    for c in range(3):
        Es = torch.zeros((T // 100, R), dtype=torch.float64, device="cuda")
        Es_ref = np.zeros((T // 100, R))
        run_chunk(gce, st, T, c * T, 1234, 64, 4, None, 100, Es, True, path=path)
        orc.run(ref, T, c * T, 1234, None, 100, Es_ref, True, n_threads=4, near_eV=1e-9)
        torch.cuda.synchronize()
        _compare(st, ref, 1e-9)
        assert np.abs(Es.cpu().numpy() - Es_ref).max() < 1e-9
    # running energies equal full recomputes
    Ef = gce.batched_energy(st.sigma).cpu().numpy()
    assert np.abs(Ef - st.E.cpu().numpy()).max() < 1e-9


def test_batch_equals_alone(cuda):
    """Jobs with different cells and replica counts in one launch give the same results as alone."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import make_chunk
    jobs = []
    for k, (L, R) in enumerate([(3, 2), (4, 5), (5, 3)]):
        gce, orc, sig_r, beta = _setup(L, seed=20 + k, R=R)
        E0 = np.array([orc.energy(x) for x in sig_r])
        jobs.append((gce, sig_r, E0, beta))
    T = 700
    alone = []
    for k, (gce, sig_r, E0, beta) in enumerate(jobs):
        st = _engine_state(sig_r, E0, beta)
        ck = make_chunk(T, 0, 77 + k, 64, 4, None, 1, None, True)
        _lib.check(_lib.lib().nce_ce_run_chunk(gce.handle, C.byref(st.struct()), C.byref(ck), _lib.stream_ptr()), "alone")
        alone.append(st)
    sts = [_engine_state(sig_r, E0, beta) for (_, sig_r, E0, beta) in jobs]
    hs = (C.c_void_p * 3)(*[j[0].handle.value for j in jobs])
    ss = (_lib.NcePtState * 3)(*[s.struct() for s in sts])
    cks = (_lib.NcePtChunk * 3)(*[make_chunk(T, 0, 77 + k, 64, 4, None, 1, None, True) for k in range(3)])
    _lib.check(_lib.lib().nce_ce_run_batch(3, hs, ss, cks, _lib.stream_ptr()), "batch")
    torch.cuda.synchronize()
    for a, b in zip(alone, sts):
        assert torch.equal(a.sigma, b.sigma) and torch.equal(a.E, b.E) and torch.equal(a.rep_of_slot, b.rep_of_slot)


@pytest.mark.parametrize("cluster,path", [(2, 2), (4, 2), (8, 2), (16, 2)])
def test_cluster_equals_single_cta(cuda, cluster, path):
    """Philox stream with exchanges, 3 chunks: a replica spread over a thread-block cluster gives the same
    trajectory as one CTA, alone and in a batch of jobs."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import make_chunk, run_chunk
    R, T = 8, 2000
    gce, orc, sig_r, beta = _setup(8, seed=12, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    a = _engine_state(sig_r, E0, beta); b = _engine_state(sig_r, E0, beta)
    for c in range(3):
        Ea = torch.zeros((T // 10, R), dtype=torch.float64, device="cuda"); Eb = torch.zeros_like(Ea)
        run_chunk(gce, a, T, c * T, 99, 64, 8, None, 10, Ea, True, path=path, cluster=1)
        run_chunk(gce, b, T, c * T, 99, 64, 8, None, 10, Eb, True, path=path, cluster=cluster)
        torch.cuda.synchronize()
        assert torch.equal(a.sigma, b.sigma) and torch.equal(a.E, b.E) and torch.equal(Ea, Eb)
        assert torch.equal(a.n_acc, b.n_acc) and torch.equal(a.rep_of_slot, b.rep_of_slot)
        assert torch.equal(a.E_min_rep, b.E_min_rep)
    assert int(a.n_acc.sum()) > 0
    # two jobs in one clustered launch equal the same jobs alone
    jobs = []
    for k, (L, RR) in enumerate([(3, 3), (4, 2)]):
        g2, o2, s2, b2 = _setup(L, seed=40 + k, R=RR)
        jobs.append((g2, s2, np.array([o2.energy(x) for x in s2]), b2))
    alone = []
    for k, (g2, s2, e2, b2) in enumerate(jobs):
        st = _engine_state(s2, e2, b2)
        run_chunk(g2, st, 500, 0, 7 + k, 64, 8, None, 1, None, True, path=path, cluster=1)
        alone.append(st)
    sts = [_engine_state(s2, e2, b2) for (_, s2, e2, b2) in jobs]
    hs = (C.c_void_p * 2)(*[j[0].handle.value for j in jobs])
    ss = (_lib.NcePtState * 2)(*[s.struct() for s in sts])
    cks = (_lib.NcePtChunk * 2)(*[make_chunk(500, 0, 7 + k, 64, 8, None, 1, None, True, path=path, cluster=cluster)
                                  for k in range(2)])
    _lib.check(_lib.lib().nce_ce_run_batch(2, hs, ss, cks, _lib.stream_ptr()), "batch")
    torch.cuda.synchronize()
    for x, y in zip(alone, sts):
        assert torch.equal(x.sigma, y.sigma) and torch.equal(x.E, y.E) and torch.equal(x.rep_of_slot, y.rep_of_slot)


def test_host_buffer_entry_point(cuda):
    """nce_ce_run_chunk_host (host buffers, copies inside) equals the device-pointer call."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import make_chunk, run_chunk
    R, T = 4, 600
    gce, orc, sig_r, beta = _setup(3, seed=8, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta)
    run_chunk(gce, st, T, 0, 5, 64, 4, None, 100, None, True)
    h_sig = sig_r.copy(); h_E = E0.copy(); ros = np.arange(R, dtype=np.int32); sor = ros.copy()
    lid = np.zeros(R, np.int32); emr = np.full(R, np.inf); emr[0] = E0[0]; nacc = np.zeros(R, np.int64); nex = np.zeros(1, np.int64)
    samples = np.zeros((T // 100, R))
    ck = make_chunk(T, 0, 5, 64, 4, None, 100, None, True)
    p = _lib.ptr
    _lib.check(_lib.lib().nce_ce_run_chunk_host(gce.handle, R, p(h_sig), p(h_E), p(beta), p(ros), p(sor), p(lid), p(emr),
                                                p(nacc), p(nex), C.byref(ck), p(samples)), "host")
    torch.cuda.synchronize()
    assert np.array_equal(h_sig, st.sigma.cpu().numpy()) and np.array_equal(h_E, st.E.cpu().numpy())
    assert np.array_equal(ros, st.rep_of_slot.cpu().numpy()) and np.array_equal(nacc, st.n_acc.cpu().numpy())


@pytest.mark.parametrize("L", [2, 3])
def test_sign_parity_small_cells(cuda, L):
    """Tiny periodic cells (neighbourhood entries alias onto the same sites): sign-parity == general == oracle."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 4, 400
    gce, orc, sig_r, beta = _setup(L, seed=9, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    a, b, c = (_engine_state(sig_r, E0, beta) for _ in range(3))
    ref = new_state(sig_r, E0, beta)
    run_chunk(gce, a, T, 0, 31, 64, 2, None, 1, None, True, path=1)
    run_chunk(gce, b, T, 0, 31, 64, 2, None, 1, None, True, path=2)
    run_chunk(gce, c, T, 0, 31, 64, 2, None, 1, None, True, path=2, cluster=2)   # partial dE pushed over a cluster
    orc.run(ref, T, 0, 31, None, 1, None, True, near_eV=1e-9)
    torch.cuda.synchronize()
    _compare(a, ref, 1e-9); _compare(b, ref, 1e-9); _compare(c, ref, 1e-9)


def test_chunk_of_two_billion_steps_is_refused(cuda):
    """The chunk kernels count steps in 32 bits: a chunk of 2^31 - 1 steps or more is refused before any launch."""
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import run_chunk
    gce, orc, sig_r, beta = _setup(3, R=2)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta)
    with pytest.raises(_lib.NceError, match="n_steps"):
        run_chunk(gce, st, 2 ** 31, 0, 0, 64, 4, path=2)
    assert np.array_equal(st.sigma.cpu().numpy(), sig_r)


def test_out_of_range_proposal_is_flagged(cuda):
    """A proposal index outside [0, N) is rejected by the kernel's bounds check and reported, not read."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import run_chunk
    R, T = 2, 10
    gce, orc, sig_r, beta = _setup(3, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta)
    pa = np.zeros((T, R), np.int32); pb = np.ones((T, R), np.int32); pu = np.full((T, R), 0.5)
    pa[3, 1] = gce.n_atoms + 5
    dev = tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))
    run_chunk(gce, st, T, 0, 0, 64, 4, dev)
    flags = _lib.i32()
    _lib.check(_lib.lib().nce_ce_errors(gce.handle, C.byref(flags)), "errors")
    assert flags.value & 1


def test_tracked_cluster_vector_sums(cuda):
    """Sign-parity chunks keep the replicas' cluster-vector sums exact: after Philox chunks with exchanges the
    tracked integers equal a recount of the final occupancies, and the energies that follow from them equal a
    float64 full recompute; fp32 carried energies re-anchor onto them."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    R, T = 8, 3000
    gce, orc, sig_r, beta = _setup(5, seed=13, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    for precision, cluster, path in ((64, 1, 2), (32, 2, 2), (64, 8, 2), (32, 4, 2)):
        st = _engine_state(sig_r, E0, beta).track_counts(gce)
        assert np.abs(gce.energy_from_counts(st.cv).cpu().numpy() - E0).max() < 1e-9
        for c in range(3):
            run_chunk(gce, st, T, c * T, 4321, precision, 8, None, 1, None, True, path=path, cluster=cluster)
        torch.cuda.synchronize()
        assert torch.equal(st.cv, gce.cluster_counts(st.sigma))
        Ef = gce.batched_energy(st.sigma).cpu().numpy()
        assert np.abs(gce.energy_from_counts(st.cv).cpu().numpy() - Ef).max() < 1e-9
        drift = st.reanchor_from_counts(gce)
        assert drift < (1e-9 if precision == 64 else 1e-3)
        assert np.abs(st.E.cpu().numpy() - Ef).max() < 1e-9
        assert int(st.n_acc.sum()) > 0


def test_graph_replay_equals_eager_batch(cuda):
    """A CUDA graph of batch chunks (device step counters, exact re-anchor) replays to the same trajectories as
    eager launches of the same chunks."""
    torch = cuda
    from neuralce_gb300.batch import CEBatch
    from neuralce_gb300.workloads import ladder, replica_configs, ce_config
    jobs = []
    for k, (L, R) in enumerate([(3, 4), (4, 6), (5, 2)]):
        gce, sig = ce_config(L, seed=60 + k)
        _, beta = ladder(R)
        jobs.append({"gce": gce, "sigma": replica_configs(sig, R, 61 + k), "beta": beta, "R": R, "N": gce.n_atoms})
    a = CEBatch(jobs, precision=32, warps=8)
    b = CEBatch(jobs, precision=32, warps=8).capture(400, chunks=2, reanchor=True)
    for _ in range(3):
        a.run_chunk(400); a.run_chunk(400); a.reanchor()
        b.replay()
    torch.cuda.synchronize()
    assert a.step == b.step == 2400
    for x, y in zip(a.states, b.states):
        assert torch.equal(x.sigma, y.sigma) and torch.equal(x.cv, y.cv) and torch.equal(x.rep_of_slot, y.rep_of_slot)
        assert torch.equal(x.E, y.E) and torch.equal(x.n_acc, y.n_acc)


def test_sharded_runner_equals_device_exchange(cuda):
    """One rank of the multi-GPU ladder layout (global slots in slot_of_rep, host exchange from gathered energies)
    runs the same trajectory as the single-GPU kernel with its device exchange."""
    torch = cuda
    from neuralce_gb300.dist import ShardedLadder, run_sharded_chunks
    from neuralce_gb300.pt import run_chunk
    R, T = 8, 800
    gce, orc, sig_r, beta = _setup(4, seed=31, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    a = _engine_state(sig_r, E0, beta)
    for c in range(3):
        run_chunk(gce, a, T, c * T, 55, 64, 8, None, 1, None, True, path=2)
    shard = ShardedLadder(beta)
    b, _ = run_sharded_chunks(gce, shard, sig_r, 3, T, 55, 64, 8, path=2)
    torch.cuda.synchronize()
    assert torch.equal(a.sigma, b.sigma) and torch.allclose(a.E, b.E, rtol=0, atol=1e-9)
    assert np.array_equal(a.rep_of_slot.cpu().numpy(), shard.rep_of_slot)
    assert int(a.n_ex.item()) == shard.n_ex > 0


@pytest.mark.parametrize("path", [1, 2])
def test_out_of_range_proposal_is_rejected_and_reported(cuda, path):
    """A host proposal naming a site outside the cell is rejected by the kernel's own bounds check (the chain
    continues as if the two sites had the same species) and reported: check_errors raises NceError once, naming
    the flag, and clears it."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    R, T = 4, 200
    gce, orc, sig_r, beta = _setup(4, seed=5, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    pa, pb, pu = proposal_stream(gce, R, T, seed=3)
    bad_a = pa.copy(); bad_a[17, 2] = gce.n_atoms                 # one entry one past the last site
    a = _engine_state(sig_r, E0, beta); b = _engine_state(sig_r, E0, beta)
    same_b = pb.copy(); same_b[17, 2] = pa[17, 2]                  # the rejected move, written as a same-site draw
    run_chunk(gce, a, T, 0, 0, 64, 8, tuple(torch.as_tensor(x).cuda() for x in (bad_a, pb, pu)), path=path)
    torch.cuda.synchronize()
    with pytest.raises(_lib.NceError, match="proposal index was out of range"):
        gce.check_errors()
    gce.check_errors()                                             # cleared
    run_chunk(gce, b, T, 0, 0, 64, 8, tuple(torch.as_tensor(x).cuda() for x in (pa, same_b, pu)), path=path)
    torch.cuda.synchronize()
    gce.check_errors()
    assert torch.equal(a.sigma, b.sigma) and torch.equal(a.E, b.E)


@pytest.mark.parametrize("precision,path", [(64, 1), (64, 2), (32, 1), (32, 2)])
def test_near_threshold_steps_are_counted(cuda, precision, path):
    """Steps planted at a known Metropolis margin (u chosen from the oracle's dE): a margin inside the stated band
    (1e-9 eV at float64, 1e-6 eV at float32) is counted in n_near, one outside it is not; both are rejected, as the
    oracle decides."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    gce, orc, sig_r, beta = _setup(8, seed=21, R=2)
    rng = np.random.default_rng(4)
    sig = sig_r[0]
    while True:                                           # a swap that raises the energy by more than 0.01 eV
        ia, ib = (int(x) for x in rng.integers(0, gce.n_atoms, 2))
        if sig[ia] != sig[ib]:
            de = orc.delta(sig, ia, ib, sig[ib], sig[ia])
            if de > 0.01:
                break
    band = 1e-9 if precision == 64 else 1e-6
    b = float(beta[0])
    margins = [0.5 * band, 3.0 * band, 1e-3]                # near, not near, far
    T = len(margins)
    pa = np.zeros((T, 2), np.int32); pb = np.zeros((T, 2), np.int32); pu = np.ones((T, 2))
    pa[:, 0], pb[:, 0] = ia, ib                              # replica 1 draws same-site moves (no-ops)
    pu[:, 0] = [np.exp(-b * (de - x)) for x in margins]
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta)
    run_chunk(gce, st, T, 0, 0, precision, 8, tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu)), path=path)
    torch.cuda.synchronize()
    assert st.n_near.cpu().tolist() == [1, 0]
    assert st.n_acc.cpu().tolist() == [0, 0]
    assert np.array_equal(st.sigma.cpu().numpy(), sig_r)


@pytest.mark.parametrize("precision", [64, 32])
def test_trajectory_occupancy_in_global_memory(cuda, precision):
    """A cell too large for shared memory (36^3 conventional = 186,624 sites: the sign-parity kernel reads and writes
    the replica's occupancy in global memory): host proposal stream, two chunks with exchanges, bit-exact against
    the oracle, near-threshold counts equal."""
    torch = cuda
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 4, 400
    gce, orc, sig_r, beta = _setup(36, seed=17, R=R)
    assert gce.n_atoms == 186_624
    E0 = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
    assert abs(E0[0] - orc.energy(sig_r[0])) < 1e-9 * max(1.0, abs(E0[0]))
    st = _engine_state(sig_r, E0, beta); ref = new_state(sig_r, E0, beta)
    step = 0
    for chunk in range(2):
        pa, pb, pu = proposal_stream(gce, R, T, seed=70 + chunk)
        dev = tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))
        run_chunk(gce, st, T, step, 0, precision, 8, dev, 1, None, True, chunk % 2,
                  torch.as_tensor(1.0 - np.random.default_rng(chunk).random(R // 2)).cuda(), path=2)
        orc.run(ref, T, step, 0, (pa, pb, pu), 1, None, True, chunk % 2, 1.0 - np.random.default_rng(chunk).random(R // 2),
                n_threads=4, near_eV=1e-9 if precision == 64 else 1e-6)
        torch.cuda.synchronize()
        _compare(st, ref, 1e-9 if precision == 64 else 1e-4)
        step += T
    assert int(st.n_acc.sum()) > 0


def test_batch_with_a_job_in_global_memory(cuda):
    """A batch whose shared-memory budget holds the small jobs' occupancies (3^3, 4^3 conventional) but not the large
    one's (24^3 = 55,296 sites, above the 48 KB per-job budget): every job bit-exact against the oracle."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import make_chunk
    from oracle.ce_oracle import new_state
    T = 300
    jobs = []
    for k, (L, R) in enumerate([(3, 3), (24, 4), (4, 2)]):
        gce, orc, sig_r, beta = _setup(L, seed=80 + k, R=R)
        E0 = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
        pa, pb, pu = proposal_stream(gce, R, T, seed=90 + k)
        jobs.append(dict(gce=gce, orc=orc, st=_engine_state(sig_r, E0, beta), ref=new_state(sig_r, E0, beta),
                         props=(pa, pb, pu), dev=tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))))
    assert jobs[1]["gce"].n_atoms > 48 * 1024
    hs = (C.c_void_p * 3)(*[j["gce"].handle.value for j in jobs])
    ss = (_lib.NcePtState * 3)(*[j["st"].struct() for j in jobs])
    cks = (_lib.NcePtChunk * 3)(*[make_chunk(T, 0, 0, 64, 8, j["dev"], 1, None, True) for j in jobs])
    _lib.check(_lib.lib().nce_ce_run_batch(3, hs, ss, cks, _lib.stream_ptr()), "batch")
    for j in jobs:
        j["orc"].run(j["ref"], T, 0, 0, j["props"], 1, None, True, n_threads=4, near_eV=1e-9)
    torch.cuda.synchronize()
    for j in jobs:
        _compare(j["st"], j["ref"], 1e-9)


# ── local-field kernel ───────────────────────────────────────────────────────────────────────────────

def test_local_field_init_is_the_flip_energy(cuda):
    """G(i) of nce_ce_field_init is minus the energy change of flipping site i alone (the oracle's float64 delta with
    both sites of the swap at i), in fixed point: within 1e-12 eV for every site of two configurations."""
    torch = cuda
    gce, orc, sig_r, _ = _setup(5, seed=2, R=2)
    assert gce.has_local_field
    G = gce.field_init(torch.as_tensor(sig_r).cuda()).cpu().numpy().astype(np.float64) * gce.field_scale
    for r in range(2):
        for i in range(gce.n_atoms):
            s = int(sig_r[r, i]); f = 1 - s
            assert abs(-G[r, i] - orc.delta(sig_r[r], i, i, f, f)) < 1e-12


@pytest.mark.parametrize("L", [2, 3])
def test_local_field_refused_on_aliasing_cells(cuda, L):
    """Cells so small that a site's neighbourhood wraps onto itself have no local-field path: path 3 is refused with
    a message, path 0 falls back to the sign-parity kernel."""
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import run_chunk
    gce, orc, sig_r, beta = _setup(L, seed=1, R=2)
    assert not gce.has_local_field
    st = _engine_state(sig_r, np.array([orc.energy(x) for x in sig_r]), beta).enable_field(gce)
    assert st.field is None
    with pytest.raises(_lib.NceError, match="local-field"):
        run_chunk(gce, st, 10, 0, 1, 64, 8, path=3)


@pytest.mark.parametrize("warps", [4, 16, 32])
def test_local_field_trajectory_host_stream(cuda, warps):
    """Host proposal stream with exchanges, two chunks: the local-field kernel is bit-exact against the oracle
    (occupancies, energies, acceptance, slot permutation, samples, near-threshold counts), and its fields equal a
    fresh nce_ce_field_init of the final occupancies."""
    torch = cuda
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T, si = 8, 1500, 50
    gce, orc, sig_r, beta = _setup(8, seed=3, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta).enable_field(gce)
    ref = new_state(sig_r, E0, beta)
    step = 0
    for chunk in range(2):
        pa, pb, pu = proposal_stream(gce, R, T, seed=10 + chunk)
        exu = 1.0 - np.random.default_rng(50 + chunk).random(R // 2)
        Es = torch.zeros((T // si, R), dtype=torch.float64, device="cuda")
        dev = tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))
        run_chunk(gce, st, T, step, 0, 64, warps, dev, si, Es, True, chunk % 2, torch.as_tensor(exu).cuda(), path=3)
        Es_ref = np.zeros((T // si, R))
        orc.run(ref, T, step, 0, (pa, pb, pu), si, Es_ref, True, chunk % 2, exu, n_threads=4, near_eV=1e-9)
        torch.cuda.synchronize()
        _compare(st, ref, 1e-9)
        assert np.abs(Es.cpu().numpy() - Es_ref).max() < 1e-9
        step += T
    assert torch.equal(st.field, gce.field_init(st.sigma))
    assert int(st.n_acc.sum()) > 0


def test_local_field_philox_equals_sign_parity(cuda):
    """Device Philox stream, three chunks with exchanges, 16 replicas: the local-field kernel and the sign-parity
    kernel give the same trajectory (and both the oracle's)."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 16, 1000
    gce, orc, sig_r, beta = _setup(5, seed=5, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    a = _engine_state(sig_r, E0, beta).enable_field(gce); b = _engine_state(sig_r, E0, beta); ref = new_state(sig_r, E0, beta)
    for c in range(3):
        Ea = torch.zeros((T // 100, R), dtype=torch.float64, device="cuda"); Eb = torch.zeros_like(Ea)
        run_chunk(gce, a, T, c * T, 1234, 64, 8, None, 100, Ea, True, path=3)
        run_chunk(gce, b, T, c * T, 1234, 64, 8, None, 100, Eb, True, path=2)
        orc.run(ref, T, c * T, 1234, None, 100, None, True, n_threads=4, near_eV=1e-9)
        torch.cuda.synchronize()
        assert torch.equal(a.sigma, b.sigma) and torch.equal(a.E, b.E) and torch.equal(Ea, Eb)
        assert torch.equal(a.n_acc, b.n_acc) and torch.equal(a.rep_of_slot, b.rep_of_slot)
        assert torch.equal(a.E_min_rep, b.E_min_rep) and torch.equal(a.n_near, b.n_near)
        _compare(a, ref, 1e-9)
    assert torch.equal(a.field, gce.field_init(a.sigma))


def test_local_field_in_global_memory_and_batch(cuda):
    """Fields and occupancies in global memory (a 24^3 cell in a batch beside small ones, whose fields fit the
    shared-memory budget), with tracked cluster-vector sums: every job bit-exact against the oracle, fields equal a
    fresh initialisation, tracked sums equal a recount."""
    torch = cuda
    from neuralce_gb300 import _lib
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import make_chunk
    from oracle.ce_oracle import new_state
    T = 400
    jobs = []
    for k, (L, R) in enumerate([(5, 3), (24, 4), (6, 2)]):
        gce, orc, sig_r, beta = _setup(L, seed=110 + k, R=R)
        E0 = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
        pa, pb, pu = proposal_stream(gce, R, T, seed=120 + k)
        st = _engine_state(sig_r, E0, beta).enable_field(gce).track_counts(gce)
        jobs.append(dict(gce=gce, orc=orc, st=st, ref=new_state(sig_r, E0, beta), props=(pa, pb, pu),
                         dev=tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu))))
    hs = (C.c_void_p * 3)(*[j["gce"].handle.value for j in jobs])
    ss = (_lib.NcePtState * 3)(*[j["st"].struct() for j in jobs])
    cks = (_lib.NcePtChunk * 3)(*[make_chunk(T, 0, 0, 64, 8, j["dev"], 1, None, True, path=3) for j in jobs])
    _lib.check(_lib.lib().nce_ce_run_batch(3, hs, ss, cks, _lib.stream_ptr()), "batch")
    for j in jobs:
        j["orc"].run(j["ref"], T, 0, 0, j["props"], 1, None, True, n_threads=4, near_eV=1e-9)
    torch.cuda.synchronize()
    for j in jobs:
        _compare(j["st"], j["ref"], 1e-9)
        assert torch.equal(j["st"].field, j["gce"].field_init(j["st"].sigma))
        assert torch.equal(j["st"].cv, j["gce"].cluster_counts(j["st"].sigma))


def test_local_field_large_cell_single_job(cuda):
    """One 36^3 cell (186,624 sites: occupancy and fields in global memory), host stream with an exchange: bit-exact
    against the oracle."""
    torch = cuda
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 4, 400
    gce, orc, sig_r, beta = _setup(36, seed=19, R=R)
    E0 = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
    st = _engine_state(sig_r, E0, beta).enable_field(gce); ref = new_state(sig_r, E0, beta)
    pa, pb, pu = proposal_stream(gce, R, T, seed=71)
    run_chunk(gce, st, T, 0, 0, 64, 16, tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu)), 1, None, True, path=3)
    orc.run(ref, T, 0, 0, (pa, pb, pu), 1, None, True, n_threads=4, near_eV=1e-9)
    torch.cuda.synchronize()
    _compare(st, ref, 1e-9)
    assert torch.equal(st.field, gce.field_init(st.sigma))


def test_batch_split_equals_unsplit(cuda):
    """A batch launched with a split (small jobs over 2-CTA clusters, the large one a CTA per replica, two launches per
    chunk) gives every job the trajectory of the unsplit batch."""
    torch = cuda
    from neuralce_gb300.batch import CEBatch
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    jobs = []
    for k, (L, R) in enumerate([(3, 4), (24, 3), (5, 2)]):
        gce, sig = ce_config(L, seed=130 + k)
        _, beta = ladder(R)
        jobs.append({"gce": gce, "sigma": replica_configs(sig, R, 131 + k), "beta": beta, "R": R, "N": gce.n_atoms})
    a = CEBatch(jobs, precision=32, warps=8, cluster=1)
    b = CEBatch(jobs, precision=32, warps=8, cluster=2)
    assert [c for _, c in b.launch_groups()] == [2, 1]
    for _ in range(2):
        a.run_chunk(300); b.run_chunk(300)
    torch.cuda.synchronize()
    for x, y in zip(a.states, b.states):
        assert torch.equal(x.sigma, y.sigma) and torch.equal(x.E, y.E) and torch.equal(x.rep_of_slot, y.rep_of_slot)
        assert torch.equal(x.cv, y.cv)


@pytest.mark.parametrize("path", [1, 2, 3])
def test_fused_exchange_equals_exchange_kernel(cuda, path):
    """The chunk-end exchange inside the chunk kernel (the last replica to finish performs it) equals the separate
    exchange launch: three chunks with exchanges and energy samples, host exchange uniforms in the middle one."""
    torch = cuda
    from neuralce_gb300.pt import run_chunk
    R, T = 12, 500
    gce, orc, sig_r, beta = _setup(5, seed=41, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    a = _engine_state(sig_r, E0, beta); b = _engine_state(sig_r, E0, beta)
    b.ex_sync = None                                       # the separate exchange kernel
    if path == 3:
        a.enable_field(gce); b.enable_field(gce)
    for c in range(3):
        Ea = torch.zeros((T // 50, R), dtype=torch.float64, device="cuda"); Eb = torch.zeros_like(Ea)
        exu = torch.as_tensor(1.0 - np.random.default_rng(c).random(R // 2)).cuda() if c == 1 else None
        for st, Es in ((a, Ea), (b, Eb)):
            run_chunk(gce, st, T, c * T, 2024, 64, 8, None, 50, Es, True, c % 2, exu, path=path)
        torch.cuda.synchronize()
        assert torch.equal(a.rep_of_slot, b.rep_of_slot) and torch.equal(a.slot_of_rep, b.slot_of_rep)
        assert torch.equal(a.n_ex, b.n_ex) and torch.equal(Ea, Eb) and torch.equal(a.E, b.E)
        assert int(a.ex_sync.item()) == 0
    assert int(a.n_ex.item()) > 0


@pytest.mark.parametrize("cluster", [1, 4])
def test_sign_parity_fp32_per_swap_error(cuda, cluster):
    """Per-swap dE of the float32 sign-parity chunk kernel (the batching and serving form) against the oracle: with an
    energy sample after every step, the change of the carried energy at each accepted step is the kernel's dE there;
    every one is within the stated 1e-6 eV of the oracle's float64 dE, and the trajectory is the oracle's."""
    torch = cuda
    from neuralce_gb300.ce import proposal_stream
    from neuralce_gb300.pt import run_chunk
    from oracle.ce_oracle import new_state
    R, T = 8, 600
    gce, orc, sig_r, beta = _setup(8, seed=51, R=R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = _engine_state(sig_r, E0, beta); ref = new_state(sig_r, E0, beta)
    pa, pb, pu = proposal_stream(gce, R, T, seed=52)
    Es = torch.zeros((T, R), dtype=torch.float64, device="cuda")
    run_chunk(gce, st, T, 0, 0, 32, 8, tuple(torch.as_tensor(x).cuda() for x in (pa, pb, pu)), 1, Es, False, path=2,
              cluster=cluster)
    Es_ref = np.zeros((T, R))
    orc.run(ref, T, 0, 0, (pa, pb, pu), 1, Es_ref, False, n_threads=4, near_eV=1e-6)
    torch.cuda.synchronize()
    _compare(st, ref, 1e-4)
    g = np.diff(np.concatenate([E0[None], Es.cpu().numpy()]), axis=0)      # per step, slot order = replica order
    o = np.diff(np.concatenate([E0[None], Es_ref]), axis=0)
    moved = o != 0.0
    assert moved.sum() > 100
    err = np.abs(g - o)[moved].max()
    print(f"float32 sign parity: {moved.sum()} accepted swaps, max |dE - oracle| = {err:.2e} eV")
    assert err < 1e-6
    assert np.all(g[~moved] == 0.0)
