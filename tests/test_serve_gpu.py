"""Serving form on the GPU: the job server's results are the same alone and in a mix of CE and NeuralCE jobs,
equal the direct chunk API, admission respects the device-memory budget, and cancellation frees the slot."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ce_jobs():
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    out = []
    for k, (L, R, x, steps, ex) in enumerate([(3, 4, 0.5, 3000, 1000), (4, 6, 0.3, 5000, 1000), (5, 8, 0.7, 2500, 500),
                                             (6, 5, 0.5, 4000, 2000)]):
        gce, sig = ce_config(L, seed=80 + k, x_pt=x)
        _, beta = ladder(R)
        out.append(dict(kind="ce", model=gce, sigma=replica_configs(sig, R, 90 + k), beta=beta, steps=steps, ex=ex, seed=500 + k))
    return out


def _nce_jobs():
    from neuralce_gb300.nce import NCEModel, synthetic_model
    from neuralce_gb300.workloads import cluster_space, ladder, replica_configs
    from tests.conftest import random_cell
    cs = cluster_space()
    out = []
    for k, (L, R, steps, ex) in enumerate([(3, 4, 60, 20), (3, 3, 45, 15)]):
        s = random_cell((L, L, L), 70 + k)
        m = NCEModel(cs, s, synthetic_model(len(cs.orbits) + 1, 3, 32, 1, k), shell_edges=(0.0, 3.3), act="silu", pool="sum")
        _, beta = ladder(R)
        out.append(dict(kind="nce", model=m, sigma=replica_configs(m.sig0, R, 75 + k), beta=beta, steps=steps, ex=ex, seed=600 + k))
    return out


def _submit(srv, j):
    if j["kind"] == "ce":
        return srv.submit_ce(j["model"], j["sigma"], j["beta"], j["steps"], j["ex"], j["seed"])
    return srv.submit_nce(j["model"], j["sigma"], j["beta"], j["steps"], j["ex"], j["seed"], reanchor_chunks=2)


def _same(a, b):
    assert np.array_equal(a["sigma"], b["sigma"])
    assert np.array_equal(a["E"], b["E"])
    assert np.array_equal(a["n_acc"], b["n_acc"]) and np.array_equal(a["rep_of_slot"], b["rep_of_slot"])
    assert a["n_ex"] == b["n_ex"]


@pytest.mark.parametrize("ce_kernel", [0, 3])
def test_results_same_alone_and_in_mix(cuda, ce_kernel):
    """ce_kernel 3: the two larger CE cells run the local-field kernel, the two smaller (aliasing) ones the sign-parity
    kernel, in separate launches of the same rounds."""
    from neuralce_gb300.serve import Server
    jobs = _ce_jobs() + _nce_jobs()
    alone = []
    with Server(precision=32, ce_kernel=ce_kernel) as srv:
        for j in jobs:
            h = _submit(srv, j)
            info, = srv.wait([h], timeout=300)
            assert info["status"] == "done", info
            alone.append(h.result())
    with Server(precision=32, ce_kernel=ce_kernel) as srv:
        hs = [_submit(srv, j) for j in jobs]
        infos = srv.wait(hs, timeout=300)
        assert all(i["status"] == "done" for i in infos), infos
        # jobs overlapped on the device: some job started before another had finished
        iv = sorted((i["t_start"], i["t_end"]) for i in infos)
        assert any(s1 < e0 for (_, e0), (s1, _) in zip(iv, iv[1:]))
        st = srv.stats()
        assert st["done"] == len(jobs) and st["bytes_used"] == 0
        assert st["attempts"] == sum(j["steps"] * len(j["beta"]) for j in jobs)
        for h, a in zip(hs, alone):
            _same(h.result(), a)
    for j, a in zip(jobs, alone):
        assert int(a["n_acc"].sum()) > 0


def test_borrowed_page_locked_buffers(cuda):
    """Jobs whose occupancies are read in place at admission (borrow) from page-locked memory, with the final
    occupancies written into caller buffers, give the same results as jobs whose inputs were copied at submission."""
    torch = cuda
    from neuralce_gb300.serve import Server
    jobs = _ce_jobs() + _nce_jobs()
    with Server(precision=32) as srv:
        hs = [_submit(srv, j) for j in jobs]
        assert all(i["status"] == "done" for i in srv.wait(hs, timeout=300))
        want = [h.result() for h in hs]
    pins, outs = [], []
    for j in jobs:
        p = torch.empty(j["sigma"].shape, dtype=torch.int8, pin_memory=True).numpy()
        p[...] = j["sigma"]
        pins.append(p)
        outs.append(torch.empty(j["sigma"].shape, dtype=torch.int8, pin_memory=True).numpy())
    with Server(precision=32) as srv:
        hs = []
        for j, p, o in zip(jobs, pins, outs):
            if j["kind"] == "ce":
                hs.append(srv.submit_ce(j["model"], p, j["beta"], j["steps"], j["ex"], j["seed"], sigma_out=o, borrow=True))
            else:
                hs.append(srv.submit_nce(j["model"], p, j["beta"], j["steps"], j["ex"], j["seed"], reanchor_chunks=2,
                                         sigma_out=o, borrow=True))
        assert all(i["status"] == "done" for i in srv.wait(hs, timeout=300))
        for h, o, w in zip(hs, outs, want):
            r = h.result()
            assert r["sigma"] is o
            _same(r, w)
    for p, j in zip(pins, jobs):                   # the borrowed inputs are read, never written
        assert np.array_equal(p, j["sigma"])


@pytest.mark.parametrize("ce_kernel", [0, 3])
def test_ce_job_equals_direct_chunks(cuda, ce_kernel):
    """A served CE job = the chunk API driven by hand: chunks of the exchange interval, exact re-anchor of the
    carried energies from the tracked cluster-vector sums after every chunk; ce_kernel 0: sign parity in fp32,
    ce_kernel 3: the local-field kernel (exact fixed point) on this cell."""
    torch = cuda
    from neuralce_gb300.pt import PTState, run_chunk
    from neuralce_gb300.serve import Server
    j = _ce_jobs()[2]
    gce, R = j["model"], len(j["beta"])
    E0 = gce.batched_energy(torch.as_tensor(j["sigma"]).cuda()).cpu().numpy()
    st = PTState(j["sigma"], E0, j["beta"], np.zeros(R, np.int32)).track_counts(gce)
    lf = ce_kernel == 3
    assert gce.has_local_field
    if lf:
        st.enable_field(gce)
    done = 0
    while done < j["steps"]:
        n = min(j["ex"], j["steps"] - done)
        run_chunk(gce, st, n, done, j["seed"], 64 if lf else 32, 8, None, 1, None, (done + n) % j["ex"] == 0,
                  path=3 if lf else 0)
        st.reanchor_from_counts(gce)
        done += n
    torch.cuda.synchronize()
    with Server(precision=32, warps=8, ce_kernel=ce_kernel) as srv:
        h = _submit(srv, j)
        srv.wait([h], timeout=120)
        r = h.result()
    assert np.array_equal(r["sigma"], st.sigma.cpu().numpy())
    assert np.array_equal(r["E"], st.E.cpu().numpy())
    assert np.array_equal(r["n_acc"], st.n_acc.cpu().numpy())
    # the exact energies equal a float64 full recompute
    Ef = gce.batched_energy(torch.as_tensor(r["sigma"]).cuda()).cpu().numpy()
    assert np.abs(Ef - r["E"]).max() < 1e-9


def test_admission_by_budget_and_cancel(cuda):
    from neuralce_gb300 import _lib
    from neuralce_gb300.serve import Server
    jobs = _ce_jobs()
    sizes = []
    with Server() as probe:
        for j in jobs:
            h = _submit(probe, j)
            sizes.append(probe.poll(h)["device_bytes"])
        probe.wait(probe._jobs.values(), timeout=120)
    budget = max(sizes) + min(sizes) // 2          # room for the largest job and little else
    with Server(hbm_budget=budget) as srv:
        big = dict(jobs[0]); big["sigma"] = np.tile(jobs[0]["sigma"], (40, 1)); big["beta"] = np.tile(jobs[0]["beta"], 40)
        with pytest.raises(_lib.NceError, match="budget"):
            _submit(srv, big)
        hs = [_submit(srv, j) for j in jobs]
        infos = srv.wait(hs, timeout=300)
        assert all(i["status"] == "done" for i in infos)
        # the resident jobs never held more than the budget
        for i in infos:
            held = sum(k["device_bytes"] for k in infos if k["t_start"] <= i["t_start"] < k["t_end"])
            assert held <= budget, (held, budget)
        # cancel a long job while it is queued or running; the server keeps serving
        long = dict(jobs[1]); long["steps"] = 10 ** 9
        hl = _submit(srv, long)
        h2 = _submit(srv, jobs[2])
        srv.cancel(hl)
        infos = srv.wait([hl, h2], timeout=120)
        assert infos[0]["status"] == "cancelled" and infos[1]["status"] == "done"
        assert srv.stats()["bytes_used"] == 0


def test_nce_jobs_sharing_a_model(cuda):
    """Several NeuralCE jobs on one model, re-anchored after every chunk, submitted together: admissions (full
    caches on the io stream) overlap other jobs' re-anchors on their streams; every result equals the job alone.
    Run in the bf16 tcgen05 form."""
    from neuralce_gb300.nce import NCEModel, synthetic_model
    from neuralce_gb300.serve import Server
    from neuralce_gb300.workloads import cluster_space, ladder, replica_configs
    from tests.conftest import random_cell
    cs = cluster_space()
    m = NCEModel(cs, random_cell((3, 3, 3), 90), synthetic_model(len(cs.orbits) + 1, 3, 32, 1, 4), shell_edges=(0.0, 3.3),
                 act="silu", pool="sum", mma=2)
    jobs = []
    for k in range(6):
        R = 3 + k % 3
        jobs.append(dict(sigma=replica_configs(m.sig0, R, 300 + k), beta=ladder(R)[1], steps=40 + 10 * k, seed=700 + k))
    def run(srv, j):
        return srv.submit_nce(m, j["sigma"], j["beta"], j["steps"], 10, j["seed"], reanchor_chunks=1)
    alone = []
    with Server(precision=32) as srv:
        for j in jobs:
            h = run(srv, j)
            info, = srv.wait([h], timeout=300)
            assert info["status"] == "done", info
            alone.append(h.result())
    with Server(precision=32) as srv:
        hs = [run(srv, j) for j in jobs]
        infos = srv.wait(hs, timeout=300)
        assert all(i["status"] == "done" for i in infos), infos
        for h, a in zip(hs, alone):
            _same(h.result(), a)


def test_submit_refuses_unknown_flags_and_bad_output_buffers(cuda):
    """Descriptor flags other than NCE_JOB_BORROW_SIGMA are refused at submission, and so is an output buffer of the
    wrong shape; nothing is queued."""
    import ctypes as C
    from neuralce_gb300 import _lib
    from neuralce_gb300.serve import Server
    j = _ce_jobs()[0]
    with Server() as srv:
        R, N = j["sigma"].shape
        with pytest.raises(ValueError, match="sigma_out"):
            srv.submit_ce(j["model"], j["sigma"], j["beta"], 100, 50, 1, sigma_out=np.zeros((R, N + 1), np.int8))
        sig = np.ascontiguousarray(j["sigma"]); beta = np.ascontiguousarray(j["beta"], np.float32)
        out = np.zeros_like(sig)
        d = _lib.NceJobDesc()
        d.kind, d.model, d.R = 0, j["model"].handle.value, R
        d.sigma, d.beta_slot, d.n_steps, d.exchange_every, d.seed = sig.ctypes.data, beta.ctypes.data, 100, 50, 1
        d.sigma_out = out.ctypes.data
        d.flags = 2
        jid = C.c_int64()
        assert _lib.lib().nce_job_submit(srv._h, C.byref(d), C.byref(jid)) == -1      # NCE_ERR_INVALID
        assert srv.stats()["queued"] == 0 and srv.stats()["running"] == 0
