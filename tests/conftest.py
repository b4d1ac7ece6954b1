"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the in-tree libnce_gb300.so; the rest run
on the CPU (the oracle, host-side setup, the C-ABI's exported symbols)."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


@pytest.fixture(scope="session")
def ptni_ce():
    """The shipped PtNi cluster expansion (golden fixture) as a ClusterExpansionFile + its reference energies."""
    from neuralce_gb300.io import ClusterExpansionFile
    from neuralce_gb300.lattice import Primitive
    g = json.load(open(os.path.join(GOLDEN, "ptni_ce_c8_6_5.json")))
    prim = Primitive(cell=np.array(g["primitive_cell"]), frac=np.array(g["primitive_frac"]),
                     species=g["chemical_symbols"] * len(g["primitive_numbers"]), numbers=np.array(g["primitive_numbers"]))
    return ClusterExpansionFile(parameters=np.array(g["parameters"]), cutoffs=g["cutoffs"],
                                chemical_symbols=g["chemical_symbols"], primitive=prim), g


@pytest.fixture(scope="session")
def ptni_cs(ptni_ce):
    from neuralce_gb300.ce_tables import ClusterSpace
    ce, _ = ptni_ce
    return ClusterSpace.build(ce.primitive, ce.cutoffs)


def ordered_refs(a=3.924):
    """The ordered fcc references of the PtNi fit on a 4x4x4 conventional cell (L1_2, DO22, L1_0, L1_1), built
    from the sublattice rules the reference's fit script uses (scripts/train/fit_ce_ptni.py:30-35)."""
    from neuralce_gb300.io import Z_OF, fcc_conventional
    conv = fcc_conventional(a, (4, 4, 4))
    frac = conv.scaled_positions() * 4
    code = ((np.round(frac * 2).astype(int) % 2) * np.array([1, 2, 4])).sum(1)
    sub = np.array([{0: 0, 3: 1, 5: 2, 6: 3}[int(c)] for c in code])
    h = np.round(frac.sum(1) * 2).astype(int)
    zc = np.floor(frac[:, 2] + 1e-6).astype(int)

    def mk(mask):
        s = conv.copy(); s.numbers = np.where(mask, Z_OF["Pt"], Z_OF["Ni"]).astype(np.int64); return s
    do22 = np.where((zc // 2) % 2 == 0, sub == 0, sub == 1)
    return {"L12_Ni3Pt": mk(sub == 0), "DO22_Ni3Pt": mk(do22), "L12_Pt3Ni": mk(sub != 0), "DO22_Pt3Ni": mk(~do22),
            "L10_NiPt": mk(np.isin(sub, [0, 1])), "L11_NiPt": mk((h // 2) % 2 == 0)}


@pytest.fixture(scope="session")
def nipt_model():
    """The shipped NeuralCE model (golden fixture) in model.pkl form (seed 0) + its exact-enumeration energies."""
    from neuralce_gb300.lattice import Primitive
    g = json.load(open(os.path.join(GOLDEN, "nipt_v3_nomax_sel.json")))
    a = lambda x: np.asarray(x, float)
    P = g["params0"]
    params = dict(lin=a(P["lin"]), layers=[{k: a(v) for k, v in L.items()} for L in P["layers"]],
                  head={k: (float(v) if np.ndim(v) == 0 else a(v)) for k, v in P["head"].items()})
    prim = Primitive(cell=a(g["primitive_cell"]), frac=a(g["primitive_frac"]),
                     species=g["chemical_symbols"] * len(g["primitive_numbers"]), numbers=np.array(g["primitive_numbers"]))
    mdl = dict(params=[params], mu=a(g["mu"]), sd=a(g["sd"]), keep=np.array(g["keep"]), K_chem=g["K_chem"], ys=g["ys"],
               ym=g["ym"], cutoffs=g["cutoffs"], shell_edges=g["shell_edges"], chemical_symbols=g["chemical_symbols"],
               primitive=prim, spin=0)
    return mdl, g


def l10_cell(reps=(2, 2, 3), a=3.924):
    """L1_0 NiPt on a conventional fcc cell: Pt on the odd (001) half-layers (scripts/bench/ptni_exact_enum.py:358-359)."""
    from neuralce_gb300.io import Z_OF, fcc_conventional
    s = fcc_conventional(a, reps)
    z = s.scaled_positions()[:, 2] * reps[2] * 2
    s.numbers = np.where(np.round(z).astype(int) % 2 == 1, Z_OF["Pt"], Z_OF["Ni"]).astype(np.int64)
    return s


def random_cell(reps, seed, a=3.924):
    from neuralce_gb300.io import Z_OF, fcc_conventional
    s = fcc_conventional(a, reps)
    r = np.random.RandomState(seed)
    z = np.full(len(s), Z_OF["Pt"], np.int64); z[r.choice(len(s), len(s) // 2, replace=False)] = Z_OF["Ni"]
    s.numbers = z
    return s


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from neuralce_gb300 import _lib
    _lib.lib()           # fails loudly if the library is missing
    return torch
