"""CPU tests: host setup (SNF, symmetry, orbits, tables) and the oracle, pinned by the reference's golden
energies.  Port of the reference's ``tests/test_ce_implicit.py`` checks onto the oracle."""
import numpy as np
import pytest

from tests.conftest import ordered_refs


def test_smith_normal_form_properties():
    from neuralce_gb300.lattice import smith_normal_form
    rng = np.random.default_rng(3)
    mats = [np.diag([2, 3, 4]), np.array([[-1, 1, 1], [1, -1, 1], [1, 1, -1]]) * 8, np.array([[0, 2, 2], [2, 0, 2], [2, 2, 0]])]
    for _ in range(20):
        m = rng.integers(-4, 5, (3, 3))
        if abs(round(np.linalg.det(m))) > 0:
            mats.append(m)
    for T in mats:
        U, d, V = smith_normal_form(T)
        assert np.array_equal(U @ T @ V, np.diag(d))
        assert d[1] % d[0] == 0 and d[2] % d[1] == 0
        assert abs(round(np.linalg.det(U))) == 1 and abs(round(np.linalg.det(V))) == 1
        assert np.prod(d) == abs(round(np.linalg.det(T)))


def test_fcc_space_group_and_orbit_counts(ptni_cs):
    from neuralce_gb300.lattice import space_group
    assert len(space_group(ptni_cs.primitive)) == 48
    orb = ptni_cs.orbits
    assert len(orb) == 37 and ptni_cs.n_params == 38                 # n_params of the shipped c8_6_5 model
    by_order = {k: sum(1 for o in orb if o.order == k) for k in (1, 2, 3, 4)}
    assert by_order == {1: 1, 2: 8, 3: 12, 4: 16}
    # rows containing one site: 140 pairs + 630 triplet + 1332 quadruplet memberships (+ the singlet)
    memb = {k: sum(len(o.clusters) * o.order for o in orb if o.order == k) for k in (2, 3, 4)}
    assert memb == {2: 140, 3: 630, 4: 1332}


def test_golden_reference_energies(ptni_ce, ptni_cs):
    """Ordered-structure energies of the shipped PtNi .ce (fits.json refs, eV/atom) through the explicit
    enumeration AND the implicit tables."""
    from neuralce_gb300.ce_tables import build_tables, encode_species
    from oracle.ce_oracle import energy_explicit, energy_implicit
    ce, g = ptni_ce
    scale = g["eci_scale"]
    for name, s in ordered_refs().items():
        e_ex = energy_explicit(ptni_cs, ce.parameters / scale, s)
        tb = build_tables(ptni_cs, s, ce.parameters / scale, energy_scale=len(s))
        sig = encode_species(ptni_cs, s, tb["basis_in"])[tb["perm"]]
        e_im = energy_implicit(tb, sig) / len(s)
        assert abs(e_ex - g["refs"][name]) < 1e-12, (name, e_ex, g["refs"][name])
        assert abs(e_im - g["refs"][name]) < 1e-12, (name, e_im, g["refs"][name])


def test_c_oracle_matches_restatement_and_full_energy(ptni_ce, ptni_cs):
    """30 random swaps on a random 256-site Ni0.5Pt0.5 cell: C oracle dE == numpy restatement, and dE == the
    difference of two full energies (reference tolerances 1e-4 / 2e-3 eV, here float64: 1e-9)."""
    from neuralce_gb300.ce_tables import build_tables
    from neuralce_gb300.io import Z_OF, fcc_conventional
    from oracle.ce_oracle import OracleCE, delta_implicit, energy_implicit
    ce, _ = ptni_ce
    s = fcc_conventional(3.924, (4, 4, 4))
    r = np.random.RandomState(1)
    z = np.full(len(s), Z_OF["Pt"], np.int64); z[r.choice(len(s), len(s) // 2, replace=False)] = Z_OF["Ni"]
    s.numbers = z
    tb = build_tables(ptni_cs, s, ce.parameters)
    orc = OracleCE(tb)
    from neuralce_gb300.ce_tables import encode_species
    sig = encode_species(ptni_cs, s, tb["basis_in"])[tb["perm"]]
    E = orc.energy(sig)
    assert abs(E - energy_implicit(tb, sig)) < 1e-9
    rng = np.random.RandomState(0)
    n = 0
    while n < 30:
        ia, ib = rng.randint(0, len(s), 2)
        if sig[ia] == sig[ib]:
            continue
        d = orc.delta(sig, ia, ib, sig[ib], sig[ia])
        assert abs(d - delta_implicit(tb, sig, ia, ib, sig[ib], sig[ia])) < 1e-9
        s1 = sig.copy(); s1[ia], s1[ib] = sig[ib], sig[ia]
        E1 = orc.energy(s1)
        assert abs(d - (E1 - E)) < 1e-9
        sig, E = s1, E1
        n += 1


def test_extensive_under_tiling(ptni_ce, ptni_cs):
    """The periodic 2x2x2 image has 8x the energy (energy_scale 8) and a swap keeps its dE
    (reference test_energy_extensive_under_tiling: ratios within 1e-4 / 1e-3)."""
    from neuralce_gb300.ce_tables import build_tables, encode_species
    from oracle.ce_oracle import OracleCE
    ce, _ = ptni_ce
    s4 = ordered_refs()["L11_NiPt"]
    r = np.random.RandomState(2)
    s4.numbers = s4.numbers[r.permutation(len(s4))]
    s8 = s4.repeat((2, 2, 2))
    t4 = build_tables(ptni_cs, s4, ce.parameters); t8 = build_tables(ptni_cs, s8, ce.parameters, energy_scale=8.0)
    g4 = encode_species(ptni_cs, s4, t4["basis_in"])[t4["perm"]]
    g8 = encode_species(ptni_cs, s8, t8["basis_in"])[t8["perm"]]
    o4, o8 = OracleCE(t4), OracleCE(t8)
    e4, e8 = o4.energy(g4), o8.energy(g8)
    assert abs(e8 / e4 - 8.0) < 1e-9
    ia, ib = 3, 7
    while g4[ia] == g4[ib]:
        ib += 1
    d4 = o4.delta(g4, ia, ib, g4[ib], g4[ia])
    ja, jb = int(t8["inv_perm"][int(t4["perm"][ia])]), int(t8["inv_perm"][int(t4["perm"][ib])])
    d8 = o8.delta(g8, ja, jb, g8[jb], g8[ja])
    assert abs(d8 / d4 - 1.0) < 1e-3      # the periodic image only changes rows that see both copies


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors (Random123 kat_vectors) in the oracle and in libnce_gb300's host copy."""
    from oracle.ce_oracle import load_c_oracle
    kat = [([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
           ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
           ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
            [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1])]
    c = load_c_oracle()
    for ctr, key, want in kat:
        assert c.philox(ctr, key) == want
    import os
    from neuralce_gb300 import _lib
    if os.path.exists(_lib.LIB_PATH):
        for ctr, key, want in kat:
            assert _lib.philox4x32(ctr, key) == want


def test_oracle_chunk_exchange_and_resume():
    """A chunk split in two (with the Philox stream) equals the same steps in one chunk: resumable trajectories."""
    from neuralce_gb300.workloads import cluster_space, ladder, replica_configs
    from neuralce_gb300.ce_tables import build_tables, synthetic_eci
    from neuralce_gb300.io import fcc_conventional
    from oracle.ce_oracle import OracleCE, new_state
    cs = cluster_space()
    s = fcc_conventional(3.924, (3, 3, 3))
    tb = build_tables(cs, s, synthetic_eci(cs, 0), energy_scale=len(s))
    orc = OracleCE(tb)
    sig0 = np.zeros(len(s), np.int8); sig0[: len(s) // 2] = 1
    R = 4
    sig = replica_configs(sig0, R, 1)
    E = np.array([orc.energy(x) for x in sig])
    _, beta = ladder(R)
    a = new_state(sig, E, beta); b = new_state(sig, E, beta)
    orc.run(a, 40, 0, seed=9, do_exchange=True, n_threads=2)
    orc.run(b, 25, 0, seed=9); orc.run(b, 15, 25, seed=9, do_exchange=True)
    for k in ("sigma", "E", "rep_of_slot", "slot_of_rep", "n_acc", "n_ex"):
        assert np.array_equal(a[k], b[k]), k
    # running energy equals a full recompute
    for r in range(R):
        assert abs(a["E"][r] - orc.energy(a["sigma"][r])) < 1e-9
