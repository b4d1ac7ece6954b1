"""Writes the golden fixtures of the tests from the reference's shipped files (run in a checkout that has
the reference mounted; the fixtures are committed, so the tests never read the reference).

  ptni_ce_c8_6_5.json   the shipped PtNi cluster expansion (models/ce/ptni/icet_c8_6_5.ce: parameters, cutoffs,
                        species, primitive) and its ordered-structure energies (models/ce/ptni/fits.json "refs",
                        eV/atom, computed by icet's ClusterExpansion.predict with the per-atom ECIs = parameters/256)

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


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
