"""The ``neuralce-mc`` command line and its drivers on the GPU engine: reference output files and keys, energies
consistent with a full recompute, and checkpoint/resume after a run killed between chunks (the failure is
made on the host: the chunk call raises) continuing to the same results as an uninterrupted run."""
import json

import numpy as np
import pytest

from tests.conftest import l10_cell

pytestmark = pytest.mark.gpu


def _files(tmp_path, ptni_ce, reps=(1, 1, 1)):
    from neuralce_gb300.io import write_ce, write_cif
    ce, _ = ptni_ce
    ce_path = tmp_path / "ptni.ce"
    write_ce(str(ce_path), ce)
    cif = tmp_path / "l10.cif"
    write_cif(str(cif), l10_cell(reps))
    return str(ce_path), str(cif)


def _flaky(real, fail_at):
    calls = {"n": 0}

    def f(*a, **k):
        calls["n"] += 1
        if calls["n"] == fail_at:
            raise RuntimeError("simulated kill between chunks")
        return real(*a, **k)
    return f


def test_icet_pt_cli_outputs_and_resume(cuda, tmp_path, ptni_ce, monkeypatch):
    torch = cuda
    import neuralce_gb300.pt as ptmod
    from neuralce_gb300.ce import GPUClusterExpansion
    from neuralce_gb300.io import read_ce
    from neuralce_gb300.mc import icet_mc, run
    ce_path, cif = _files(tmp_path, ptni_ce)
    args = ["--framework", "icet", "--ce", ce_path, "--init_cif", cif, "--supercell", "3", "3", "3", "--pt",
            "--T_min", "300", "--T_max", "1400", "--n_replicas", "6", "--n_steps", "3000", "--chunk", "500",
            "--exchange_every", "500", "--sample_interval", "100", "--energy_mode", "delta", "--seed", "3"]
    a = tmp_path / "a"
    run.main(args + ["--out_dir", str(a)])
    e, r = np.load(a / "energies.npz"), np.load(a / "mcmc_result.npz")
    summary = json.load(open(a / "mcmc_summary.json"))
    assert e["energies"].shape == (30, 6) and e["temperatures"].shape == (6,)
    for k in ("energies", "temperatures", "ladder_id", "ladder_pos", "sigma_final", "sigma_min", "E_min",
              "swap_accept_rate", "exchange_accept_rate", "wall_time"):
        assert k in r.files, k
    assert 0.0 < summary["swap_accept_rate"] < 1.0 and "E_min" in summary
    assert summary["near_threshold_steps"] >= 0                # counted by the chunk kernels, reported
    # the last slot-ordered samples are the energies of the final configurations
    atoms, scale = icet_mc.prepare_cell(read_ce(ce_path), cif, (3, 3, 3), 3, log=lambda *x, **k: None)
    gce = GPUClusterExpansion(read_ce(ce_path), atoms, energy_scale=scale)
    canon = r["sigma_final"][:, gce.perm]
    E = gce.batched_energy(torch.as_tensor(canon).cuda()).cpu().numpy()
    assert np.abs(E - e["energies"][-1]).max() < 1e-8
    # killed after three chunks with a checkpoint every chunk, then restarted: same results
    b = tmp_path / "b"
    monkeypatch.setattr(ptmod, "run_chunk", _flaky(ptmod.run_chunk, 4))
    with pytest.raises(RuntimeError, match="simulated kill"):
        run.main(args + ["--out_dir", str(b), "--checkpoint_every", "1"])
    assert (b / "checkpoint.npz").exists()
    monkeypatch.undo()
    run.main(args + ["--out_dir", str(b), "--checkpoint_every", "1"])
    assert not (b / "checkpoint.npz").exists()
    e2, r2 = np.load(b / "energies.npz"), np.load(b / "mcmc_result.npz")
    assert np.array_equal(e["energies"], e2["energies"])
    assert np.array_equal(r["sigma_final"], r2["sigma_final"]) and float(r["E_min"]) == float(r2["E_min"])
    # a checkpoint of a different run is refused
    c = tmp_path / "c"
    monkeypatch.setattr(ptmod, "run_chunk", _flaky(ptmod.run_chunk, 3))
    with pytest.raises(RuntimeError):
        run.main(args + ["--out_dir", str(c), "--checkpoint_every", "1"])
    monkeypatch.undo()
    with pytest.raises(RuntimeError, match="another run"):
        run.main([x if x != "3" else "4" for x in args] + ["--out_dir", str(c), "--checkpoint_every", "1"])


def test_icet_single_and_multi_temperature(cuda, tmp_path, ptni_ce):
    from neuralce_gb300.mc import run
    ce_path, cif = _files(tmp_path, ptni_ce)
    base = ["--framework", "icet", "--ce", ce_path, "--init_cif", cif, "--supercell", "3", "3", "3", "--n_steps", "1000",
            "--chunk", "500", "--energy_mode", "delta"]
    run.main(base + ["--T", "600", "--out_dir", str(tmp_path / "s")])
    assert np.load(tmp_path / "s" / "energies.npz")["energies"].shape == (10, 1)
    run.main(base + ["--temps", "400", "800", "1200", "--out_dir", str(tmp_path / "m")])
    r = np.load(tmp_path / "m" / "mcmc_result.npz")
    assert r["sigma_final"].shape[0] == 3 and float(r["exchange_accept_rate"]) == 0.0


def test_nce_pt_driver_outputs_and_resume(cuda, tmp_path, nipt_model, monkeypatch):
    from neuralce_gb300.io import write_cif
    from neuralce_gb300.mc import nce_mc
    from neuralce_gb300.nce import NCEState
    mdl, g = nipt_model
    cif = tmp_path / "l10.cif"
    write_cif(str(cif), l10_cell((3, 3, 4)))
    kw = dict(model_path=mdl, init_cif=str(cif), n_steps=400, T_min=300.0, T_max=1400.0, n_replicas=4, exchange_every=50,
              chunk=100, sample_interval=20, seed=5)
    a = tmp_path / "a"
    res = nce_mc.run_pt_mc(out_dir=str(a), **kw)
    e = np.load(a / "energies.npz")
    for k in ("E_chunk", "acc_chunk", "drift", "drift_eV", "traj", "betas", "temps"):
        assert k in e.files, k
    assert e["E_chunk"].shape == (4, 4) and e["traj"].shape == (4, 20)
    assert (a / "final_sigma.npy").exists() and len(list(a.glob("final_T*_r*.cif"))) == 4
    assert res["drift_max"] < 1e-4 and 0.0 < res["acc_mean"] < 1.0
    # the L1_0 start: first samples near the exact E_L10 at low T
    assert abs(e["traj"][0, 0] - g["E_L10"]) < 0.05
    b = tmp_path / "b"
    monkeypatch.setattr(NCEState, "run_chunk", _flaky(NCEState.run_chunk, 3))
    with pytest.raises(RuntimeError, match="simulated kill"):
        nce_mc.run_pt_mc(out_dir=str(b), checkpoint_every=1, **kw)
    monkeypatch.undo()
    nce_mc.run_pt_mc(out_dir=str(b), checkpoint_every=1, **kw)
    e2 = np.load(b / "energies.npz")
    assert np.array_equal(e["E_chunk"], e2["E_chunk"]) and np.array_equal(e["traj"], e2["traj"])
    assert np.array_equal(np.load(a / "final_sigma.npy"), np.load(b / "final_sigma.npy"))
