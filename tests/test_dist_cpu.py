"""Multi-rank host logic on the CPU (gloo, world size 2): a ladder sharded over two ranks, each advancing its own
replicas (the C oracle stands in for the chunk kernel) and all-gathering the energies at every exchange, gives
the single-process trajectory bit for bit; the host exchange equals the oracle's in-process exchange, with one
exchange round per chunk and with two (each round drawing its own parity and uniforms)."""
import multiprocessing as mp
import socket

import numpy as np
import pytest

R, T, CHUNKS, SEED = 8, 300, 4, 17


def _setup():
    from neuralce_gb300.workloads import ce_config, ladder, replica_configs
    from oracle.ce_oracle import OracleCE
    gce, sig = ce_config(3, seed=5)
    sig_r = replica_configs(sig, R, 6)
    _, beta = ladder(R)
    orc = OracleCE(gce.info)
    E0 = np.array([orc.energy(x) for x in sig_r])
    return orc, sig_r, E0, beta


def _local_state(shard, sig_r, E0, beta):
    r0, r1 = shard.r0, shard.r1
    n = r1 - r0
    Emr = np.full(n, np.inf)
    return dict(sigma=np.ascontiguousarray(sig_r[r0:r1]).copy(), E=E0[r0:r1].copy(), beta_slot=np.asarray(beta, np.float32),
                rep_of_slot=np.arange(n, dtype=np.int32), slot_of_rep=shard.local_slots(),
                ladder_id=np.zeros(R, np.int32), E_min_rep=Emr, n_acc=np.zeros(n, np.int64), n_ex=np.zeros(1, np.int64))


def _sharded(rank, world, port, q, rounds=1):
    import torch.distributed as dist
    from neuralce_gb300.dist import ShardedLadder
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    orc, sig_r, E0, beta = _setup()
    shard = ShardedLadder(beta, rank=rank, world=world)
    st = _local_state(shard, sig_r, E0, beta)
    for c in range(CHUNKS):
        st["slot_of_rep"] = shard.local_slots()
        orc.run(st, T, c * T, SEED, do_exchange=False)
        shard.exchange(st["E"], SEED, (c + 1) * T, rounds=rounds)
    q.put((rank, st["sigma"], st["E"], st["n_acc"], shard.rep_of_slot, shard.n_ex))
    dist.destroy_process_group()


def _reference(rounds=1):
    from oracle.ce_oracle import new_state
    orc, sig_r, E0, beta = _setup()
    ref = new_state(sig_r, E0, beta)
    for c in range(CHUNKS):
        orc.run(ref, T, c * T, SEED, do_exchange=True, rounds=rounds)
    return ref


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("rounds", [1, 2])
def test_host_exchange_equals_oracle_single_rank(rounds):
    from neuralce_gb300.dist import ShardedLadder
    orc, sig_r, E0, beta = _setup()
    shard = ShardedLadder(beta)
    st = _local_state(shard, sig_r, E0, beta)
    for c in range(CHUNKS):
        st["slot_of_rep"] = shard.local_slots()
        orc.run(st, T, c * T, SEED, do_exchange=False)
        shard.exchange(st["E"], SEED, (c + 1) * T, rounds=rounds)
    ref = _reference(rounds)
    assert np.array_equal(st["sigma"], ref["sigma"]) and np.array_equal(st["E"], ref["E"])
    assert np.array_equal(shard.rep_of_slot, ref["rep_of_slot"]) and shard.n_ex == int(ref["n_ex"][0])
    assert shard.n_ex > 0


@pytest.mark.timeout(300)
def test_two_rank_ladder_equals_single_process():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_sharded, args=(r, 2, port, q, 2)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted([q.get(timeout=240) for _ in ps], key=lambda x: x[0])
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = _reference(2)
    sigma = np.concatenate([o[1] for o in out]); E = np.concatenate([o[2] for o in out])
    n_acc = np.concatenate([o[3] for o in out])
    assert np.array_equal(sigma, ref["sigma"]) and np.array_equal(E, ref["E"]) and np.array_equal(n_acc, ref["n_acc"])
    for o in out:
        assert np.array_equal(o[4], ref["rep_of_slot"]) and o[5] == int(ref["n_ex"][0])
