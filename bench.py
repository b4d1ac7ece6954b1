"""Benchmark of the parallel-tempering hot path on GB300 (one JSON line on rank 0).

Workload (default, the reference's published CE configuration): fcc Ni/Pt, 8x8x8 conventional cells = 2,048
sites, synthetic per-orbit ECIs (cutoffs 8/6/5 A), int8 occupancy 50/50, R = 32 replicas on a geometric
300-1400 K ladder, replica exchange every 5,000 steps, 200,000 steps per replica.  A bench "step" is one
chunk of 5,000 MC steps for all 32 replicas followed by the on-device exchange (160,000 swap attempts);
the whole job is 40 such steps.  Proposals come from the device Philox stream.

  value     swap attempts/s with the state resident in HBM, CUDA events around each chunk on its stream,
            L2 flushed (256 MB write) between timed chunks outside the events
  e2e       the same chunks through nce_ce_run_chunk_host: pinned host buffers in and out every chunk
  roofline  dominant kernel ce_bin_chunk_kernel (sign-parity form); algorithmic bytes per attempt = 14,996 B
            of int8 member-occupancy reads (2 x 7,498 member slots of the rows of both sites)
  cpu_baseline  the oracle's C restatement on the host cores (bounded sample, all threads)
  side lines  nce (configuration 1, float32), nce_tcgen05_split / nce_tcgen05_bf16 (the same on tcgen05
            tensor cores), nce_shipped_model (the reference's shipped PtNi model on the same cell), batch
            (configuration 2), serve (configuration 4, scaled)
--workload nce | nce-shipped | ce-batch | ce-large | nce-large | serve | ce-energy prints one of them alone.
--impl reference times the oracle port on the host cores (the reference's own CPU paths, JAX and icet,
are not installed on this image) with the same metric.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MC swap attempts/s (CE, NCE) vs plain FP64 form; p50/p99 PT-job latency"
CONTRACTIONS = ["fp32 CUDA cores", "bf16 mma.sync tensor cores (fp32 accumulation)",
                "bf16 tcgen05 tensor cores (fp32 accumulation in tensor memory)", "split-bf16 mma.sync tensor cores",
                "split-bf16 tcgen05 tensor cores"]
H100_PUBLISHED = 1_231_993.0          # reference CE PT, 2,048 sites, R=32, H100 (results/bench_stage/gpu_icet_*H100*.json)
B_GATHER = 14_996                     # bytes of member occupancy per attempt, config-0 cluster set
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu capture of the headline kernel,
# keyed by (path, L, R, steps per chunk): profiles/ holds the capture (a 1000-step chunk; the tables and occupancy
# are read once per launch, so the figure does not grow with the steps)
TRAFFIC = {(2, 8, 32, 5000): 166_912}
SMEM_PIPE = {(2, 8, 32, 5000): 0.178}       # the same capture's shared-memory wavefronts, fraction of the pipe's peak


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32])
    ap.add_argument("--warps", type=int, default=0, help="warps per replica (0 = autotune)")
    ap.add_argument("--cluster", type=int, default=0, help="CTAs per replica, thread-block cluster (0 = autotune)")
    ap.add_argument("--path", type=int, default=0, help="0 auto, 1 general products, 2 sign parity, 3 local field")
    ap.add_argument("--L", type=int, default=8)
    ap.add_argument("--R", type=int, default=32)
    ap.add_argument("--chunk", type=int, default=5000)
    ap.add_argument("--workload", choices=["ce", "nce", "ce-batch", "serve", "ce-large", "nce-large", "ce-energy", "nce-shipped"], default="ce")
    ap.add_argument("--nce-mma", type=int, default=-1, help="NeuralCE contractions: 0 fp32 CUDA cores; bf16 / split bf16 "
                    "on tensor cores: 1 / 3 mma.sync, 2 / 4 tcgen05 (-1: workload default)")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window of the serving side measurement (0 = skip)")
    ap.add_argument("--batch-steps", type=int, default=3, help="chunks of the batched-form side measurement (0 = skip)")
    ap.add_argument("--nce-steps", type=int, default=3, help="chunks of the NeuralCE side measurement (0 = skip)")
    ap.add_argument("--nce-chunk", type=int, default=1000, help="MC steps per NeuralCE chunk")
    ap.add_argument("--nce-width", type=int, default=64, help="layer width of the --workload nce network")
    ap.add_argument("--large-steps", type=int, default=2, help="chunks of each configuration-3 side measurement (0 = skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0")); world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index; self.p = None; self.path = None

    def start(self):
        import tempfile
        fd, self.path = tempfile.mkstemp(suffix=".csv"); os.close(fd)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
        os.unlink(self.path)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1])); mx = max(mx, float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def bf16_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p))["bf16_tflops"], "measured"
    return 1900.0, "fallback"


def nce_flops_per_attempt(m):
    """Layer-contraction FLOPs of one attempt, upper bound before the two flips' receptive fields are merged:
    2 flops x sum over layers l = 1..depth of 2 ball_l sites x ((1 + P) Cin_l) x D (exact ball sizes of the
    cell's tables; basis 0)."""
    ends = [int(x) for x in m.keep["ball_end"][0]]
    P = int(m.geo["P"])
    f = 0
    for lvl in range(1, m.depth + 1):
        cin = m.C0 if lvl == 1 else m.D
        f += 2 * ends[lvl] * (1 + P) * cin * m.D
    return 2 * f


def cpu_oracle_rate(L, R, target_s=10.0, threads=None):
    """attempts/s of the C oracle on the host cores for the same workload (bounded sample)."""
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    from oracle.ce_oracle import OracleCE, new_state
    threads = threads or os.cpu_count() or 1
    gce, sig = ce_config(L, seed=0)
    orc = OracleCE(gce.info)
    sig_r = replica_configs(sig, R, 1)
    _, beta = ladder(R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = new_state(sig_r, E0, beta)
    t = time.perf_counter(); orc.run(st, 20, 0, seed=7, n_threads=threads); dt = time.perf_counter() - t
    steps = max(20, int(20 * target_s / max(dt, 1e-6)))
    t = time.perf_counter(); orc.run(st, steps, 20, seed=7, n_threads=threads); dt = time.perf_counter() - t
    return R * steps / dt, threads, f"{R} replicas x {steps} steps of the {gce.n_atoms}-site job ({dt:.1f} s)"


def run_reference(args, rank, world):
    if rank != 0:
        return
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    from oracle.ce_oracle import OracleCE, new_state
    threads = os.cpu_count() or 1
    gce, sig = ce_config(args.L, seed=0)
    orc = OracleCE(gce.info)
    sig_r = replica_configs(sig, args.R, 1)
    _, beta = ladder(args.R)
    E0 = np.array([orc.energy(x) for x in sig_r])
    st = new_state(sig_r, E0, beta)
    t = time.perf_counter(); orc.run(st, 10, 0, seed=7, n_threads=threads); dt = time.perf_counter() - t
    per = max(10, int(10 * 2.0 / max(dt, 1e-6)))          # ~2 s per bench step
    step0 = 10
    for _ in range(args.warmup):
        orc.run(st, per, step0, seed=7, n_threads=threads); step0 += per
    times = []
    for _ in range(args.steps):
        t = time.perf_counter(); orc.run(st, per, step0, seed=7, n_threads=threads, do_exchange=True)
        times.append(time.perf_counter() - t); step0 += per
    tot = sum(times); value = args.R * per * args.steps / tot
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "swap attempts/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, gce),
            "cpu_baseline": {"value": value, "unit": "swap attempts/s", "cores": threads, "kind": "port",
                             "sample": f"{args.R} replicas x {per} steps per bench step of the {gce.n_atoms}-site job; "
                                       "C restatement of the reference delta path (JAX/icet CPU paths not installed)"},
            "e2e": {"value": value, "unit": "swap attempts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def bench_nce(L=8, R=32, depth=3, width=64, chunk=1000, exchange_every=100, steps=3, warmup=1, seed=0, cluster=0, mma=0,
              shipped=False):
    """NeuralCE configuration 1: local receptive-field update, float32, R replicas 300-1400 K; a step is one
    chunk of ``chunk`` MC steps + chunk//exchange_every exchange rounds; full re-anchor every ceil(N/chunk)
    chunks (the reference driver's default).  ``shipped``: the reference's shipped PtNi model instead of the
    configuration-1 network (the model of its published 144,636 steps/s at 2,048 sites, R = 32, H100)."""
    exchange_every = min(exchange_every, chunk)
    import torch
    from neuralce_gb300.nce import NCEState
    from neuralce_gb300.workloads import ladder, nce_config, replica_configs, shipped_nce_config
    if shipped:
        m, sig = shipped_nce_config(os.path.join(ROOT, "tests", "golden", "nipt_v3_nomax_sel.json"), L, seed, mma=mma)
    else:
        m, sig = nce_config(L, depth, width, seed, mma=mma)
    _, beta = ladder(R)
    st = NCEState(m, replica_configs(sig, R, 1 + seed), beta).full_cache()
    tune = None
    per_sm = 1
    if cluster == 0:            # CTAs per replica and per SM: time a short chunk for each candidate that fits
        from neuralce_gb300 import _lib
        from neuralce_gb300.nce import NCEState as _S
        tune = {}
        for cl, ps in ((1, 1), (2, 1), (4, 1), (8, 1), (2, 2), (4, 2), (8, 2)):
            sc = _S(m, replica_configs(sig, R, 1 + seed), beta).full_cache()
            try:
                sc.run_chunk(4, 0, seed=1, cluster=cl, ctas_per_sm=ps)
            except _lib.NceError:
                continue
            a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_.record(); sc.run_chunk(20, 4, seed=1, cluster=cl, ctas_per_sm=ps); b_.record(); torch.cuda.synchronize()
            tune[f"{cl}x{ps}"] = a_.elapsed_time(b_)
        cluster, per_sm = (int(x) for x in min(tune, key=tune.get).split("x"))
    anchor = max(1, -(-m.N // chunk))
    step = 0
    def one(k):
        nonlocal step
        st.run_chunk(chunk, step, seed=99, exchange_rounds=max(chunk // exchange_every, 1), cluster=cluster,
                     ctas_per_sm=per_sm); step += chunk
        if (k + 1) % anchor == 0:
            st.full_cache()
    for k in range(warmup):
        one(k)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stream = torch.cuda.current_stream()
    for k in range(steps):
        ev[k][0].record(stream); one(warmup + k); ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    tot = sum(ms) / 1e3
    net = ("the reference's shipped PtNi model (depth 1, width 16, 3 shells, sigmoid gate, tanh, mean readout)" if shipped
           else f"depth {depth}, width {width}, SiLU, sum readout, 12-NN shell")
    value = R * chunk * steps / tot
    flops = nce_flops_per_attempt(m)
    pk, src = bf16_peak()
    roof = {"bound": "tensor", "achieved": value * flops / 1e12, "peak": pk, "unit": "TFLOP/s",
            "frac": value * flops / 1e12 / pk, "traffic": None, "peak_source": src, "flops_per_attempt": flops,
            "note": "layer contractions only, against the measured dense bf16 peak; the step is bound by the "
                    "receptive-field gathers and per-level barriers of the Markov chain"}
    return {"value": value, "unit": "swap attempts/s", "ms_per_step": float(np.mean(ms)),
            "config": f"NeuralCE: {m.N} sites, R={R}, {net}, "
                      f"chunk {chunk} steps + {max(chunk // exchange_every, 1)} exchange rounds, re-anchor every {anchor} chunks",
            "vs_h100_published_144636": (value / 144_636) if (shipped and m.N == 2048 and R == 32) else None,
            "receptive_field": [int(x) for x in m.keep['ball_end'][0]], "accept_rate": float(st.n_acc.sum().item()) / (R * step),
            "ctas_per_replica": cluster, "ctas_per_sm": per_sm, "autotune_ms": tune, "roofline": roof,
            "contractions": CONTRACTIONS[mma]}


def bench_energy(L=64, R=128, reps=5, seed=0):
    """Full energy (the re-anchor / set-up kernel) of R configurations of an L^3 conventional fcc cell on the
    sign-parity tables: bit planes + exact column sums + float64 energies."""
    import torch
    from neuralce_gb300.workloads import ServeModels, random_occupancy
    gce = ServeModels().ce(L)
    sig = torch.as_tensor(random_occupancy(gce.n_atoms, 0.5, R, seed)).cuda()
    gce.batched_energy(sig)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        gce.batched_energy(sig)
    b.record(); torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    return {"value": gce.n_atoms * R / (ms / 1e3), "unit": "site-replicas/s", "ms_per_step": ms,
            "config": f"full energy, bit-sliced: fcc {L}^3 conventional ({gce.n_atoms} sites) x {R} configurations",
            "rows_per_site": int(gce.info["Rt"]) // int(gce.info["nB"])}


def bench_batch(steps=3, warmup=1, chunk=5000, reanchor=10000, n_jobs=64, alone_jobs=8, alone_steps=2000):
    """Configuration 2: 64 independent CE cells (L ~ U{4..32}, x_Pt ~ U[0.1, 0.9], R ~ U{16,32,64}) advanced by one
    CUDA-graph replay per ``reanchor`` steps: reanchor/chunk persistent batch launches (float32 dE, every job's
    exchange at each chunk end) and the exact float64 re-anchor of every carried energy from the tracked
    cluster-vector sums.  Compared with the plain float64 kernels running the first ``alone_jobs`` jobs alone."""
    import torch
    from neuralce_gb300.batch import CEBatch, tune_launch
    from neuralce_gb300.pt import PTState, run_chunk
    from neuralce_gb300.workloads import ce_batch_config
    from neuralce_gb300.autotune import best_warps
    t0 = time.time()
    jobs = ce_batch_config(n_jobs)
    setup = time.time() - t0
    (w, cl), tune = tune_launch(jobs, 32)
    # float32 drift between re-anchors and exactness of the float64 re-anchor, measured eagerly on a copy
    chk = CEBatch(jobs, precision=32, warps=w, cluster=cl)
    for _ in range(reanchor // chunk):
        chk.run_chunk(chunk)
    drift = chk.reanchor()
    full_err = max(float((j["gce"].batched_energy(st.sigma) - st.E).abs().max().item()) for j, st in zip(jobs, chk.states))
    del chk
    b = CEBatch(jobs, precision=32, warps=w, cluster=cl).capture(chunk, chunks=max(1, reanchor // chunk), reanchor=True)
    for _ in range(warmup):
        b.replay()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stream = torch.cuda.current_stream()
    for k in range(steps):
        ev[k][0].record(stream); b.replay(); ev[k][1].record(stream)
    torch.cuda.synchronize()
    tot = sum(a.elapsed_time(c) for a, c in ev) / 1e3
    value = b.attempts_per_step * b._graph_steps * steps / tot
    # the first jobs alone in the plain float64 kernels: general point-function products, and sign parity
    alone = {}
    for path in (1, 2):
        att = 0; secs = 0.0
        for j in jobs[:alone_jobs]:
            st = PTState(j["sigma"], j["gce"].batched_energy(torch.as_tensor(j["sigma"]).cuda()).cpu().numpy(), j["beta"],
                         np.zeros(j["R"], np.int32))
            wj, _ = best_warps(j["gce"], st, 64, path)
            run_chunk(j["gce"], st, 50, 0, 5, 64, wj, do_exchange=True, path=path)
            a_, c_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_.record(); run_chunk(j["gce"], st, alone_steps, 50, 5, 64, wj, do_exchange=True, path=path); c_.record()
            torch.cuda.synchronize()
            secs += a_.elapsed_time(c_) / 1e3; att += j["R"] * alone_steps
        alone[path] = att / secs
    return {"value": value, "unit": "swap attempts/s", "ms_per_step": 1e3 * tot / steps,
            "config": f"{n_jobs} CE jobs, one CUDA graph per {b._graph_steps} steps: L~U{{4..32}} "
                      f"({min(j['N'] for j in jobs)}-{max(j['N'] for j in jobs)} sites), x_Pt~U[0.1,0.9], R~U{{16,32,64}} "
                      f"({b.attempts_per_step} replicas), fp32 dE, {max(1, reanchor // chunk)} batch launches of {chunk} steps "
                      f"+ exchange, then the fp64 re-anchor from exact cluster-vector sums",
            "fp64_single_job_alone": alone[1], "ratio_vs_fp64_single_job": value / alone[1],
            "fp64_sign_parity_single_job_alone": alone[2], "ratio_vs_fp64_sign_parity_single_job": value / alone[2],
            "max_fp32_drift_before_reanchor_eV": drift, "max_reanchored_vs_full_recompute_eV": full_err,
            "warps_per_replica": w, "ctas_per_replica_of_split_jobs": cl,
            "autotune_ms": {f"{a}x{b_}": round(v, 3) for (a, b_), v in tune.items()}, "setup_s": setup}


def bench_serve(seconds=10.0, rate=50.0, ce_scale=0.01, nce_scale=0.0002, nce_max_sites=32768, seed=4, alone_jobs=0,
                ce_exchange=500, nce_exchange=20, nce_mma=4):
    """Configuration 4 (serving), scaled: Poisson arrivals at ``rate`` jobs/s for ``seconds``, CE or NeuralCE 50/50,
    sites log-uniform 256..1,048,576 (NeuralCE capped at ``nce_max_sites``), x_Pt ~ U[0.1, 0.9], R ~ U{8..128},
    steps log-uniform 10k..1M times ``ce_scale`` / ``nce_scale``.  Jobs are submitted to the job server at their
    arrival times (models and occupancies prepared beforehand); reports p50/p99 job latency (submission to
    results on the host) and the aggregate swap attempts/s over the makespan.  Capacity: the stream's CE jobs
    submitted at once, against the same jobs run one after another in the plain float64 kernel (``alone_jobs``
    limits that to the first jobs; 0 = all).  NeuralCE jobs run the precision form ``nce_mma`` (4: split bf16 operands on
    the tcgen05 tensor cores, float32 accumulation, within 1e-4 eV per swap; 2: plain bf16)."""
    import torch
    from neuralce_gb300.pt import PTState, run_chunk
    from neuralce_gb300.serve import Server
    from neuralce_gb300.workloads import ServeModels, ladder, random_occupancy, serve_stream
    t0 = time.time()
    jobs = serve_stream(rate, seconds, seed, ce_scale, nce_scale, nce_max_sites)
    models = ServeModels(mma=nce_mma)
    for j in jobs:
        j["model"] = models.ce(j["L"]) if j["kind"] == "ce" else models.nce(j["L"])
        # the job's occupancies and its result buffer in page-locked host memory, prepared with the job; the server
        # reads the occupancies in place at admission (borrow) and writes the final ones into the result buffer
        sig = random_occupancy(j["N"], j["x_pt"], j["R"], j["seed"] & 0xFFFFFFFF)
        j["sigma"] = torch.empty(sig.shape, dtype=torch.int8, pin_memory=True).numpy()
        j["sigma"][...] = sig
        j["out"] = torch.empty(sig.shape, dtype=torch.int8, pin_memory=True).numpy()
        j["beta"] = ladder(j["R"])[1]
    setup = time.time() - t0
    ce_jobs = [j for j in jobs if j["kind"] == "ce"]

    def burst(w):
        """every CE job of the stream submitted at once: (attempts/s over the makespan, makespan)"""
        with Server(precision=32, warps=w) as sv:
            bh = [sv.submit_ce(j["model"], j["sigma"], j["beta"], j["steps"], ce_exchange, j["seed"], sigma_out=j["out"],
                               borrow=True) for j in ce_jobs]
            binf = sv.wait(bh, timeout=1800)
        span = max(i["t_end"] for i in binf) - min(i["t_submit"] for i in binf)
        return sum(j["R"] * j["steps"] for j in ce_jobs) / span, span
    burst(8)                                               # warm-up: kernels loaded, pools grown
    cap = {w: burst(w) for w in (8, 16, 32)}               # the launch shape of the served CE rounds
    w_best = max(cap, key=lambda w: cap[w][0])
    srv = Server(precision=32, warps=w_best)
    hs = []
    start = time.perf_counter()
    for j in jobs:
        while time.perf_counter() - start < j["t"]:
            time.sleep(0.0002)
        if j["kind"] == "ce":
            hs.append(srv.submit_ce(j["model"], j["sigma"], j["beta"], j["steps"], ce_exchange, j["seed"], sigma_out=j["out"],
                                    borrow=True))
        else:
            hs.append(srv.submit_nce(j["model"], j["sigma"], j["beta"], j["steps"], nce_exchange, j["seed"], sigma_out=j["out"],
                                     borrow=True))
    infos = srv.wait(hs, timeout=1800)
    st = srv.stats()
    failures = [i.get("message", "") for i in infos if i["status"] == "failed"][:3]
    srv.close()
    ok = [i for i in infos if i["status"] == "done"]
    lat = np.array([i["t_end"] - i["t_submit"] for i in ok])
    makespan = max(i["t_end"] for i in ok) - min(i["t_submit"] for i in ok)
    kinds = {k: np.array([i["t_end"] - i["t_submit"] for i, j in zip(infos, jobs) if j["kind"] == k and i["status"] == "done"])
             for k in ("ce", "nce")}
    att = {k: sum(j["R"] * j["steps"] for j in jobs if j["kind"] == k) for k in ("ce", "nce")}
    # capacity (above): every CE job of the stream submitted at once; against each alone, one after another, in the
    # plain float64 kernel (general point-function products), chunks of the same exchange interval
    burst_s = cap[w_best][1]
    a_att, a_s = 0, 0.0
    for j in ce_jobs[:alone_jobs] if alone_jobs else ce_jobs:
        gce = j["model"]
        E0 = gce.batched_energy(torch.as_tensor(j["sigma"]).cuda()).cpu().numpy()
        stt = PTState(j["sigma"], E0, j["beta"], np.zeros(j["R"], np.int32))
        run_chunk(gce, stt, 20, 0, 1, 64, 8, None, 1, None, False, path=1)
        torch.cuda.synchronize()
        e0 = time.perf_counter()
        done = 0
        while done < j["steps"]:
            n = min(ce_exchange, j["steps"] - done)
            run_chunk(gce, stt, n, done, j["seed"], 64, 8, None, 1, None, (done + n) % ce_exchange == 0, path=1)
            done += n
        torch.cuda.synchronize()
        a_s += time.perf_counter() - e0; a_att += j["R"] * j["steps"]
    pct = lambda a, q: float(np.percentile(a, q)) if len(a) else None
    ce_rate = att["ce"] / makespan
    return {"value": st["attempts"] / makespan, "unit": "swap attempts/s", "ms_per_step": 1e3 * makespan,
            "config": f"serving: Poisson {rate:g} jobs/s for {seconds:g} s ({len(jobs)} jobs), CE/NeuralCE 50/50, "
                      f"sites log-U 256..1M (NeuralCE <= {nce_max_sites}), x_Pt U[0.1,0.9], R U{{8..128}}, steps log-U "
                      f"10k..1M x {ce_scale:g} (CE) / x {nce_scale:g} (NeuralCE), exchange every {ce_exchange} / {nce_exchange}; "
                      f"CE fp32 with exact fp64 re-anchor per chunk, NeuralCE {CONTRACTIONS[nce_mma]}",
            "jobs": len(jobs), "done": len(ok), "failed": st["failed"], "failures": failures,
            "latency_s": {"p50": pct(lat, 50), "p99": pct(lat, 99), "max": float(lat.max()) if len(lat) else None,
                          "ce_p50": pct(kinds["ce"], 50), "ce_p99": pct(kinds["ce"], 99),
                          "nce_p50": pct(kinds["nce"], 50), "nce_p99": pct(kinds["nce"], 99)},
            "makespan_s": makespan, "attempts": st["attempts"], "attempts_ce": att["ce"], "attempts_nce": att["nce"],
            "ce_attempts_per_s_poisson": ce_rate,
            "ce_capacity_attempts_per_s": att["ce"] / burst_s, "ce_capacity_makespan_s": burst_s,
            "ce_warps": w_best, "ce_capacity_by_warps": {str(w): v[0] for w, v in cap.items()},
            "fp64_single_job_alone": (a_att / a_s) if a_s else None,
            "ratio_ce_capacity_vs_fp64_alone": (att["ce"] / burst_s) / (a_att / a_s) if a_s else None,
            "rounds": {"ce": st["rounds_ce"], "nce": st["rounds_nce"]}, "setup_s": setup}


def bench_large(L=136, R=256, chunk=5000, steps=3, warmup=1, precision=64, seed=0, path=0):
    """Configuration 3 (CE part): fcc L^3 conventional cell (L = 136: 10,061,824 sites), 50/50, R temperatures
    300-1400 K; dE in the float64 kernels' exact fixed point (the local-field kernel when the tuner picks it, fields
    in global memory), float64 exchange, and carried energies re-anchored exactly from the tracked cluster-vector
    sums after every chunk.  Occupancies are drawn on the device (one seeded permutation per replica).  A step is one
    chunk of ``chunk`` MC steps per replica + exchange + re-anchor."""
    import torch
    from neuralce_gb300.autotune import best_launch
    from neuralce_gb300.pt import PTState, run_chunk
    from neuralce_gb300.workloads import ServeModels, ladder
    t0 = time.time()
    gce = ServeModels().ce(L)
    N = gce.n_atoms
    setup_tables = time.time() - t0
    g = torch.Generator(device="cuda"); g.manual_seed(seed)
    n_pt = N // 2
    sig = torch.empty((R, N), dtype=torch.int8, device="cuda")
    for r in range(R):
        sig[r] = (torch.randperm(N, device="cuda", generator=g) < n_pt).to(torch.int8)
    _, beta = ladder(R)
    st = PTState(np.zeros((R, 1), np.int8), np.zeros(R), beta, np.zeros(R, np.int32))
    st.sigma, st.N = sig, N
    st.E = gce.batched_energy(sig)
    st.E_min_rep = torch.full((R,), float("inf"), dtype=torch.float64, device="cuda"); st.E_min_rep[0] = st.E[0]
    st.n_near = torch.zeros(R, dtype=torch.int64, device="cuda")
    st.track_counts(gce)
    torch.cuda.synchronize()
    setup = time.time() - t0
    paths = (2, 3) if path == 0 and precision == 64 else ((2,) if path == 0 else (path,))
    (w, cl, path), tune = best_launch(gce, st, precision, 0, (8, 16, 32), (1,), steps=200, paths=paths)
    field_ms = None
    if path == 3:
        a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_.record(); st.enable_field(gce); b_.record(); torch.cuda.synchronize()
        field_ms = a_.elapsed_time(b_)
    step = 0
    from neuralce_gb300 import _lib

    def one():
        nonlocal step
        run_chunk(gce, st, chunk, step, 77, precision, w, None, 1, None, True, path=path)
        _lib.check(_lib.lib().nce_ce_energy_from_counts(gce.handle, st.cv.data_ptr(), R, st.E.data_ptr(), _lib.stream_ptr()),
                   "nce_ce_energy_from_counts")             # exact float64 re-anchor, in place
        step += chunk
    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stream = torch.cuda.current_stream()
    for k in range(steps):
        ev[k][0].record(stream); one(); ev[k][1].record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    tot = sum(ms) / 1e3
    value = R * chunk * steps / tot
    # exactness: tracked sums vs a recount, re-anchored energies vs a float64 full recompute, fields vs a rebuild
    cv_ok = bool(torch.equal(st.cv, gce.cluster_counts(st.sigma)))
    Ef = gce.batched_energy(st.sigma)
    field_ok = bool(torch.equal(st.field, gce.field_init(st.sigma))) if path == 3 else None
    torch.cuda.synchronize()
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record(); gce.batched_energy(st.sigma); b_.record(); torch.cuda.synchronize()
    hbm, src = peaks()
    achieved = value * B_GATHER / 1e9
    return {"value": value, "unit": "swap attempts/s", "ms_per_step": float(np.mean(ms)),
            "config": f"CE large cell: fcc {L}^3 conventional ({N} sites), R={R} 300-1400 K, "
                      f"{'local-field' if path == 3 else 'sign-parity'} kernel, fp{precision} (exact fixed point) dE, "
                      f"chunk {chunk} steps + fp64 exchange + exact fp64 re-anchor from cluster-vector sums",
            "sites": N, "replicas": R, "state_bytes": R * N * (9 if path == 3 else 1), "warps_per_replica": w,
            "path": {2: "sign-parity", 3: "local-field"}[path], "autotune_ms": {str(k): round(v, 3) for k, v in tune.items()},
            "tracked_sums_equal_recount": cv_ok, "fields_equal_rebuild": field_ok,
            "max_E_vs_full_recompute_eV": float((Ef - st.E).abs().max().item()), "field_init_ms": field_ms,
            "full_energy_ms": a_.elapsed_time(b_), "full_energy_site_replicas_per_s": R * N / (a_.elapsed_time(b_) / 1e3),
            "accept_rate": float(st.n_acc.sum().item()) / (R * step),
            "near_threshold_steps": int(st.n_near.sum().item()),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_source": src, "bytes_per_attempt": B_GATHER},
            "setup_s": setup, "tables_s": setup_tables, "vs_h100_published_4344547": value / 4_344_547}


def bench_nce_large(L=64, R=64, width=128, depth=3, chunk=100, steps=3, warmup=1, mma=4, seed=0, cluster=0):
    """Configuration 3 (NeuralCE part): fcc L^3 conventional cell (L = 64: 1,048,576 sites), R replicas 300-1400 K,
    the configuration-1 architecture widened to ``width``; layer contractions as split bf16 on the tcgen05 tensor
    cores with float32 accumulation in tensor memory (``mma`` 4, the precision form: per-swap dE within 1e-4 eV of the
    float64 oracle, tests/test_nce_gpu.py::test_config_cell_chain_matches_oracle); 2 = plain bf16 (stated bound
    1e-2 eV), 1 / 3 = bf16 / split bf16 on mma.sync, 0 = float32 CUDA cores.  Occupancies drawn on the device.  A step
    is one chunk of ``chunk`` MC steps per replica + one exchange round; the full caches are built once (timed
    separately)."""
    import torch
    from neuralce_gb300.nce import NCEModel, NCEState, synthetic_model
    from neuralce_gb300.workloads import A_FCC, cluster_space, ladder
    from neuralce_gb300.io import Z_OF, fcc_conventional
    t0 = time.time()
    cs = cluster_space()
    s = fcc_conventional(A_FCC, (L, L, L)); s.numbers = np.full(len(s), Z_OF["Ni"], np.int64)
    P = synthetic_model(len(cs.orbits) + 1, depth, width, 1, seed)
    m = NCEModel(cs, s, P, shell_edges=(0.0, 3.3), act="silu", pool="sum", mma=mma)
    N = m.N
    setup_model = time.time() - t0
    g = torch.Generator(device="cuda"); g.manual_seed(seed)
    sig = torch.empty((R, N), dtype=torch.int8, device="cuda")
    for r in range(R):
        sig[r] = (torch.randperm(N, device="cuda", generator=g) < N // 2).to(torch.int8)
    _, beta = ladder(R)
    st = NCEState(m, np.zeros((R, 1), np.int8), beta)
    st.N = N; st.sigma = sig
    st.h0 = torch.zeros((R, N, m.C0), dtype=torch.float32, device="cuda")
    st.hmid = torch.zeros((max(depth - 1, 0), R, N, m.D), dtype=torch.float32, device="cuda") if depth >= 2 else None
    st.e = torch.zeros((R, N), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record(); st.full_cache(); b_.record(); torch.cuda.synchronize()
    full_ms = a_.elapsed_time(b_)
    tune = None
    if cluster == 0:
        tune = {}
        for cl in (1, 2, 4):
            st.run_chunk(2, 0, seed=1, cluster=cl)
            a_.record(); st.run_chunk(10, 2, seed=1, cluster=cl); b_.record(); torch.cuda.synchronize()
            tune[cl] = a_.elapsed_time(b_)
        cluster = min(tune, key=tune.get)
    step = 100
    for _ in range(warmup):
        st.run_chunk(chunk, step, seed=99, exchange_rounds=1, cluster=cluster); step += chunk
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        ev[k][0].record(); st.run_chunk(chunk, step, seed=99, exchange_rounds=1, cluster=cluster); ev[k][1].record(); step += chunk
    torch.cuda.synchronize()
    ms = [x.elapsed_time(y) for x, y in ev]
    tot = sum(ms) / 1e3
    E_car = st.E.clone(); st.full_cache(); torch.cuda.synchronize()
    drift = float((st.E - E_car).abs().max().item())
    value = R * chunk * steps / tot
    flops = nce_flops_per_attempt(m)
    pk, psrc = bf16_peak()
    return {"value": value, "unit": "swap attempts/s", "ms_per_step": float(np.mean(ms)),
            "roofline": {"bound": "tensor", "achieved": value * flops / 1e12, "peak": pk, "unit": "TFLOP/s",
                         "frac": value * flops / 1e12 / pk, "peak_source": psrc, "flops_per_attempt": flops},
            "dE_error_bound_eV": 1e-4 if mma in (0, 3, 4) else 1e-2,
            "near_threshold_steps": int(st.n_near.sum().item()),
            "config": f"NeuralCE large cell: fcc {L}^3 conventional ({N} sites), R={R}, depth {depth}, width {width}, SiLU, sum, "
                      f"{CONTRACTIONS[mma]}, "
                      f"chunk {chunk} steps + 1 exchange round",
            "sites": N, "replicas": R, "full_cache_ms": full_ms, "ctas_per_replica": cluster, "autotune_ms": tune,
            "carried_vs_rebuilt_energy_eV": drift, "device_state_GB": (R * N * (1 + 4 * m.C0 + 4 + 4 * m.D * max(depth - 1, 0))) / 1e9,
            "setup_model_s": setup_model}


def workload_config(args, gce):
    return {"workload": f"CE parallel tempering fp{args.precision}: fcc Ni/Pt {args.L}x{args.L}x{args.L} conventional "
                        f"({gce.n_atoms} sites), R={args.R} replicas 300-1400 K, exchange every {args.chunk} steps, "
                        f"{args.chunk * args.steps} steps per replica timed",
            "sites": gce.n_atoms, "replicas": args.R, "steps_per_chunk": args.chunk, "cluster_set": "8/6/5 A (37 orbits)",
            "proposals": "device Philox4x32-10", "l2": "flushed between timed chunks (256 MB write)",
            "parallelism": f"replicas only: {args.gpus} independent job(s), one per GPU"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(local)
    if args.workload == "ce-batch":
        from neuralce_gb300 import _lib
        _lib.lib()
        r = bench_batch(steps=args.steps, warmup=args.warmup)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["value"], "unit": "swap attempts/s", "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": r["config"]},
                              "batch": r}), flush=True)
        return
    if args.workload == "ce-large":
        from neuralce_gb300 import _lib
        _lib.lib()
        r = bench_large(steps=args.steps if args.steps != 40 else 3, warmup=max(1, min(args.warmup, 2)))
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["value"], "unit": "swap attempts/s", "n_gpus": world,
                              "steps": args.steps if args.steps != 40 else 3, "warmup": max(1, min(args.warmup, 2)),
                              "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": r["config"]},
                              "large": r}), flush=True)
        return
    if args.workload == "ce-energy":
        from neuralce_gb300 import _lib
        _lib.lib()
        r = bench_energy(L=64 if args.L == 8 else args.L, R=128 if args.R == 32 else args.R)
        if rank == 0:
            print(json.dumps({"metric": "full-energy site-replicas/s", "value": r["value"], "unit": r["unit"], "n_gpus": world,
                              "steps": 5, "warmup": 1, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
                              "scaling": "weak", "vs_baseline": None, "dtype": "int32/f64", "data": "synthetic",
                              "config": {"workload": r["config"]}, "energy": r}), flush=True)
        return
    if args.workload == "nce-large":
        from neuralce_gb300 import _lib
        _lib.lib()
        st_, wu_ = (args.steps if args.steps != 40 else 3), max(1, min(args.warmup, 2))
        r = bench_nce_large(steps=st_, warmup=wu_, mma=(4 if args.nce_mma < 0 else args.nce_mma))
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["value"], "unit": "swap attempts/s", "n_gpus": world, "steps": st_,
                              "warmup": wu_, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "bf16" if args.nce_mma in (-1, 1, 2, 3, 4) else "f32", "data": "synthetic",
                              "config": {"workload": r["config"]}, "large": r}), flush=True)
        return
    if args.workload == "serve":
        from neuralce_gb300 import _lib
        _lib.lib()
        r = bench_serve(seconds=args.serve_seconds or 10.0)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["value"], "unit": "swap attempts/s", "n_gpus": world, "steps": 1,
                              "warmup": 0, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": r["config"]},
                              "serve": r}), flush=True)
        return
    if args.workload in ("nce", "nce-shipped"):
        from neuralce_gb300 import _lib
        _lib.lib()
        r = bench_nce(L=args.L, R=args.R, chunk=args.nce_chunk, steps=args.steps, warmup=args.warmup, seed=rank,
                      width=args.nce_width,
                      mma=max(args.nce_mma, 0), shipped=args.workload == "nce-shipped")
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": r["value"], "unit": "swap attempts/s", "n_gpus": world, "steps": args.steps,
                              "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                              "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": r["config"]},
                              "nce": r}), flush=True)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from neuralce_gb300 import _lib
    from neuralce_gb300.pt import PTState, run_chunk, make_chunk
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    _lib.lib()
    gce, sig = ce_config(args.L, seed=rank)
    R, T = args.R, args.chunk
    sig_r = replica_configs(sig, R, 1 + rank)
    _, beta = ladder(R)
    E0 = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
    st = PTState(sig_r, E0, beta, np.zeros(R, np.int32))
    tuned = None
    if args.warps == 0 or args.cluster == 0:
        from neuralce_gb300.autotune import best_launch
        ws = (args.warps,) if args.warps else (4, 8, 16, 32)
        cls = (args.cluster,) if args.cluster else ((1, 2, 4, 8, 16) if args.path != 1 else (1,))
        paths = (2, 3) if args.path == 0 else (args.path,)
        (args.warps, args.cluster, args.path), t = best_launch(gce, st, args.precision, args.path, ws, cls, steps=1000,
                                                               paths=paths)
        tuned = {f"{w}x{c}/p{p}": round(v, 3) for (w, c, p), v in t.items()}
    if args.path == 3:
        st.enable_field(gce)                               # local fields of the replicas' occupancies
    si = 100                                               # energy samples every 100 steps (the CLI default)
    Es = torch.zeros((T // si, R), dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()
    step = 0
    for _ in range(args.warmup):
        run_chunk(gce, st, T, step, 42 + rank, args.precision, args.warps, None, si, Es, True, path=args.path,
                  cluster=args.cluster); step += T
    torch.cuda.synchronize()
    clk = Clocks(local); clk.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        ev[k][0].record(stream)
        run_chunk(gce, st, T, step, 42 + rank, args.precision, args.warps, None, si, Es, True, path=args.path,
                  cluster=args.cluster)
        ev[k][1].record(stream)
        step += T
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = clk.stop()
    per_ms = [a.elapsed_time(b) for a, b in ev]
    tot_s = sum(per_ms) / 1e3
    if world > 1:
        t = torch.tensor([tot_s], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX); tot_s = float(t.item())
    attempts = R * T * args.steps * world
    value = attempts / tot_s
    # e2e: same chunks with host buffers through the C-ABI (pinned host memory)
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        h_sig = pin(st.sigma.cpu().numpy()); h_E = pin(st.E.cpu().numpy()); h_b = pin(beta)
        h_ros = pin(st.rep_of_slot.cpu().numpy()); h_sor = pin(st.slot_of_rep.cpu().numpy()); h_lid = pin(np.zeros(R, np.int32))
        h_emr = pin(st.E_min_rep.cpu().numpy()); h_nacc = pin(st.n_acc.cpu().numpy()); h_nex = pin(st.n_ex.cpu().numpy())
        h_samp = pin(np.zeros((T // si, R)))
        torch.cuda.synchronize()
        ck = make_chunk(T, step, 42 + rank, args.precision, args.warps, None, si, None, True, path=args.path, cluster=args.cluster)
        def host_call():
            _lib.check(_lib.lib().nce_ce_run_chunk_host(gce.handle, R, h_sig.data_ptr(), h_E.data_ptr(), h_b.data_ptr(),
                                                        h_ros.data_ptr(), h_sor.data_ptr(), h_lid.data_ptr(), h_emr.data_ptr(),
                                                        h_nacc.data_ptr(), h_nex.data_ptr(), C.byref(ck), h_samp.data_ptr()),
                       "nce_ce_run_chunk_host")
        host_call(); ck.step0 += T      # warm the staging buffers
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_call(); ck.step0 += T
        e2e_s = time.perf_counter() - t0
        h2d = R * gce.n_atoms + R * (8 + 4 + 4 + 4 + 4 + 8 + 8) + 8
        d2h = R * gce.n_atoms + R * (8 + 4 + 4 + 8 + 8) + 8 + 8 * R * (T // si)
        e2e = {"value": R * T * args.steps * world / e2e_s, "unit": "swap attempts/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "api": "nce_ce_run_chunk_host"}
    hbm, src = peaks()
    ms_chunk = float(np.mean(per_ms))
    achieved = R * T * B_GATHER / (ms_chunk / 1e3) / 1e9
    # DRAM bytes per launch from one ncu capture of this workload (dram__bytes_read.sum + dram__bytes_write.sum of
    # ce_bin_chunk_kernel, 2,048 sites, R = 32, 16 warps x 4 CTAs): the tables and occupancies live in shared memory;
    # the same capture's shared-memory pipe use (l1tex__data_pipe_lsu_wavefronts_mem_shared.sum.pct_of_peak_sustained
    # _elapsed), the on-chip roofline that the gathered bytes actually meet
    traffic = TRAFFIC.get((args.path, args.L, args.R, T))
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
            "kernel": {1: "ce_pt_chunk_kernel", 3: "ce_lf_chunk_kernel"}.get(args.path, "ce_bin_chunk_kernel"),
            "peak_source": src,
            "algorithmic_bytes_per_launch": R * T * B_GATHER,
            "shared_pipe_frac_ncu": SMEM_PIPE.get((args.path, args.L, args.R, T))}
    nce_line = nce_tc_line = nce_bf16_line = nce_shipped_line = None
    if rank == 0 and args.nce_steps > 0:
        nce_line = bench_nce(steps=args.nce_steps)
        nce_tc_line = bench_nce(steps=args.nce_steps, mma=4)
        nce_bf16_line = bench_nce(steps=args.nce_steps, mma=2)
        nce_shipped_line = bench_nce(steps=args.nce_steps, shipped=True)
    large_ce_line = large_nce_line = None
    if rank == 0 and args.large_steps > 0:
        large_ce_line = bench_large(steps=args.large_steps, warmup=1)
        torch.cuda.empty_cache()
        large_nce_line = bench_nce_large(steps=args.large_steps, warmup=1)
        torch.cuda.empty_cache()
    batch_line = None
    if rank == 0 and args.batch_steps > 0:
        batch_line = bench_batch(steps=args.batch_steps)
    serve_line = None
    if rank == 0 and args.serve_seconds > 0:
        serve_line = bench_serve(seconds=args.serve_seconds)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, cores, sample = cpu_oracle_rate(args.L, R)
        cpu = {"value": v, "unit": "swap attempts/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "swap attempts/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_chunk, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": value / H100_PUBLISHED if (args.L == 8 and args.R == 32) else None,
                "dtype": "f64" if args.precision == 64 else "f32", "data": "synthetic (seeded lattice, random-normal ECIs)",
                "config": workload_config(args, gce), "clocks": clocks, "e2e": e2e, "gpu_launches": 2 * args.steps,
                "roofline": roof, "cpu_baseline": cpu, "nce": nce_line, "nce_tcgen05_split": nce_tc_line, "nce_tcgen05_bf16": nce_bf16_line, "nce_shipped_model": nce_shipped_line, "batch": batch_line, "serve": serve_line,
                "large_ce": large_ce_line, "large_nce": large_nce_line,
                "launch": {"warps_per_cta": args.warps, "ctas_per_replica": args.cluster,
                           "path": ["auto", "general", "sign-parity", "local-field"][args.path],
                           "autotune_ms": tuned},
                "accept_rate": float(st.n_acc.sum().item()) / max(1, R * step),
                "near_threshold_steps": {"count": int(st.n_near.sum().item()), "of_attempts": R * step,
                                         "band_eV": 1e-9 if args.precision == 64 else 1e-6}}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
