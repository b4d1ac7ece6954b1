"""Writes the golden fixtures of the tests from the reference's shipped files (run in a checkout that has
the reference mounted; the fixtures are committed, so the tests never read the reference).

  ptni_ce_c8_6_5.json   the shipped PtNi cluster expansion (models/ce/ptni/icet_c8_6_5.ce: parameters, cutoffs,
                        species, primitive) and its ordered-structure energies (models/ce/ptni/fits.json "refs",
                        eV/atom, computed by icet's ClusterExpansion.predict with the per-atom ECIs = parameters/256)

  nipt_v3_nomax_sel.json  the shipped NeuralCE model (models/nce/nipt_v3_nomax_sel/model.pkl: seed-0 parameters,
                        standardisation, channel selection, cutoffs, shells, primitive) and its L1_0 energy on the
                        2x2x3 conventional cell from results/ptni_exact/exact_N48.json ("E_L10", eV/atom)

  exact_N48.json        the exact (enumerated) thermodynamics of that model on that cell at 24 Pt / 24 Ni, from
                        results/ptni_exact/exact_N48.json: temperature grid (K), <E> (eV/atom), C_V (k_B/atom)

Usage: python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def main(ref):
    from neuralce_gb300.io import read_ce
    ce = read_ce(os.path.join(ref, "models/ce/ptni/icet_c8_6_5.ce"))
    fits = json.load(open(os.path.join(ref, "models/ce/ptni/fits.json")))["icet_c8_6_5"]
    out = dict(source="models/ce/ptni/icet_c8_6_5.ce + models/ce/ptni/fits.json", parameters=ce.parameters.tolist(),
               cutoffs=ce.cutoffs, chemical_symbols=ce.chemical_symbols, primitive_cell=ce.primitive.cell.tolist(),
               primitive_frac=ce.primitive.frac.tolist(), primitive_numbers=ce.primitive.numbers.tolist(),
               eci_scale=fits["eci_scale"], refs=fits["refs"], n_params=fits["n_params"])
    json.dump(out, open(os.path.join(HERE, "ptni_ce_c8_6_5.json"), "w"), indent=1)
    from neuralce_gb300.io import load_model
    import numpy as np
    mdl = load_model(os.path.join(ref, "models/nce/nipt_v3_nomax_sel/model.pkl"))
    ex = json.load(open(os.path.join(ref, "results/ptni_exact/exact_N48.json")))
    tl = lambda x: np.asarray(x, float).tolist()
    P = mdl["params"][0]
    layers = [{k: tl(v) for k, v in L.items()} for L in P["layers"]]
    nce = dict(source="models/nce/nipt_v3_nomax_sel/model.pkl + results/ptni_exact/exact_N48.json",
               params0=dict(lin=tl(P["lin"]), layers=layers, head={k: tl(v) for k, v in P["head"].items()}),
               mu=tl(mdl["mu"]), sd=tl(mdl["sd"]), keep=np.asarray(mdl["keep"]).tolist(), K_chem=int(mdl["K_chem"]),
               ys=float(mdl["ys"]), ym=float(mdl["ym"]), cutoffs=list(mdl["cutoffs"]), shell_edges=list(mdl["shell_edges"]),
               chemical_symbols=mdl["chemical_symbols"], primitive_cell=mdl["primitive"].cell.tolist(),
               primitive_frac=mdl["primitive"].frac.tolist(), primitive_numbers=mdl["primitive"].numbers.tolist(),
               cell=[2, 2, 3], E_L10=float(ex["E_L10"]), E_min=float(ex["E_min"]), E_max=float(ex["E_max"]), N=int(ex["N"]))
    json.dump(nce, open(os.path.join(HERE, "nipt_v3_nomax_sel.json"), "w"))
    th = dict(source="results/ptni_exact/exact_N48.json", N=int(ex["N"]), nPt=int(ex["nPt"]), cell=[2, 2, 3],
              T=tl(ex["T"]), E=tl(ex["E"]), Cv=tl(ex["Cv"]), E_L10=float(ex["E_L10"]))
    json.dump(th, open(os.path.join(HERE, "exact_N48.json"), "w"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the neuralce reference checkout>")
    main(sys.argv[1])
