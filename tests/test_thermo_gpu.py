"""Thermodynamics of the NeuralCE PT path against the reference's exact enumeration: the shipped model on the
48-atom 2x2x3 conventional cell at 24 Pt / 24 Ni (``results/ptni_exact/exact_N48.json``, fixture
``tests/golden/exact_N48.json``).  <E>(T) and C_V(T) of a seeded PT run agree with the exact values within
their statistical errors (5 standard errors, plus 3e-5 eV/atom for the float32 engine and 5% of C_V for the
error of its error estimate)."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, l10_cell

pytestmark = pytest.mark.gpu


def test_pt_thermodynamics_match_exact_enumeration(cuda, nipt_model):
    torch = cuda
    from neuralce_gb300.nce import NCEState, setup
    from neuralce_gb300.thermo import KB, estimates
    mdl, _ = nipt_model
    ex = json.load(open(os.path.join(GOLDEN, "exact_N48.json")))
    mc = setup(mdl, l10_cell())
    model = mc["model"]
    assert model.N == ex["N"] == 48
    temps = np.geomspace(500.0, 1600.0, 16)
    betas = (1.0 / (KB * temps)).astype(np.float32)
    R = len(temps)
    st = NCEState(model, np.stack([model.sig0] * R).astype(np.int8), betas).full_cache()
    chunk, si, n_chunks = 1000, 10, 200
    Es = torch.zeros((chunk // si, R), dtype=torch.float64, device="cuda")
    traj = []
    for c in range(n_chunks):
        st.run_chunk(chunk, c * chunk, seed=2024, sample_interval=si, E_samples=Es, exchange_rounds=chunk // 100)
        traj.append(Es.cpu().numpy().T.copy())
        st.full_cache()                                         # re-anchor every chunk (N < chunk)
    traj = np.concatenate(traj, axis=1) * mc["ys"] + mc["ym"]
    est = estimates(traj, temps, model.N)
    E_ex = np.interp(temps, ex["T"], ex["E"])
    C_ex = np.interp(temps, ex["T"], ex["Cv"])
    for t, e, ee, se, cv, ce, cse, g in zip(temps, est["E"], E_ex, est["E_se"], est["Cv"], C_ex, est["Cv_se"], est["g"]):
        print(f"T {t:7.1f} K  <E> {e:.6f} exact {ee:.6f} (se {se:.1e})  C_V {cv:.4f} exact {ce:.4f} (se {cse:.3f})  g {g:.1f}")
    dE = np.abs(est["E"] - E_ex)
    assert np.all(dE <= 5 * est["E_se"] + 3e-5), list(zip(temps.round(), dE, est["E_se"]))
    dC = np.abs(est["Cv"] - C_ex)
    assert np.all(dC <= 5 * est["Cv_se"] + 0.05 * C_ex), list(zip(temps.round(), est["Cv"], C_ex, est["Cv_se"]))
    assert int(st.n_ex.item()) > 0
