"""Lattices with several sublattices: a B2 (CsCl-type) cell with two binary sublattices, and a rocksalt-type cell
with one active and one inert sublattice.  CPU: explicit enumeration == implicit tables == C oracle, swap dE ==
difference of full energies.  GPU (general and sign-parity paths, one CTA and a cluster): energies, swap dE and
Philox trajectories with exchanges == the C oracle."""
import numpy as np
import pytest


def _system(kind, L=4, seed=0):
    from neuralce_gb300.ce_tables import ClusterSpace
    from neuralce_gb300.io import Z_OF, Structure
    from neuralce_gb300.lattice import Primitive
    a = 3.0
    species = [["Ni", "Pt"], ["Al", "Cu"]] if kind == "b2" else [["Ni", "Pt"], ["O"]]
    frac = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.5]])
    prim = Primitive(cell=np.eye(3) * a, frac=frac, species=species,
                     numbers=np.array([Z_OF[species[0][0]], Z_OF[species[1][0]]]))
    cs = ClusterSpace.build(prim, [5.0, 3.5])
    rng = np.random.default_rng(seed)
    params = np.concatenate([[0.0], rng.normal(0.0, 0.05, len(cs.orbits)) / np.arange(1, len(cs.orbits) + 1)])
    n = np.array([(i, j, k) for i in range(L) for j in range(L) for k in range(L)], float)
    pos, z = [], []
    for b in range(2):
        pos.append((n + frac[b]) @ prim.cell)
        sp = species[b]
        zz = np.full(len(n), Z_OF[sp[0]], np.int64)
        if len(sp) > 1:
            zz[rng.permutation(len(n))[: len(n) // 2]] = Z_OF[sp[1]]
        z.append(zz)
    s = Structure(prim.cell * L, np.concatenate(pos), np.concatenate(z))
    return cs, params, s


@pytest.mark.parametrize("kind", ["b2", "rocksalt"])
def test_oracle_multisublattice(kind):
    from neuralce_gb300.ce_tables import build_tables, encode_species
    from oracle.ce_oracle import OracleCE, delta_implicit, energy_explicit, energy_implicit
    cs, params, s = _system(kind)
    tb = build_tables(cs, s, params)
    assert tb["nB"] == 2 and len(tb["act_nb"]) == (2 if kind == "b2" else 1)
    sig = encode_species(cs, s, tb["basis_in"])[tb["perm"]]
    orc = OracleCE(tb)
    E = orc.energy(sig)
    assert abs(E - energy_implicit(tb, sig)) < 1e-10
    assert abs(E - energy_explicit(cs, params, s)) < 1e-10
    rng = np.random.default_rng(1)
    sl = tb["site_to_sl"]
    n = 0
    while n < 20:
        ia, ib = (int(x) for x in rng.integers(0, len(sig), 2))
        if sl[ia] != sl[ib] or sig[ia] == sig[ib] or len(tb["sl_species"][sl[ia]]) < 2:
            continue
        d = orc.delta(sig, ia, ib, sig[ib], sig[ia])
        assert abs(d - delta_implicit(tb, sig, ia, ib, sig[ib], sig[ia])) < 1e-10
        s1 = sig.copy(); s1[ia], s1[ib] = sig[ib], sig[ia]
        E1 = orc.energy(s1)
        assert abs(d - (E1 - E)) < 1e-10
        sig, E = s1, E1
        n += 1


@pytest.mark.gpu
@pytest.mark.parametrize("kind,path,cluster", [("b2", 1, 1), ("b2", 2, 1), ("b2", 2, 4), ("rocksalt", 1, 1),
                                               ("rocksalt", 2, 2)])
def test_gpu_multisublattice(cuda, kind, path, cluster):
    torch = cuda
    from neuralce_gb300.ce import GPUClusterExpansion
    from neuralce_gb300.pt import PTState, run_chunk
    from neuralce_gb300.workloads import ladder
    from oracle.ce_oracle import OracleCE, new_state
    cs, params, s = _system(kind, seed=3)
    gce = GPUClusterExpansion((cs, params), s)
    orc = OracleCE(gce.info)
    sig = gce.encode(s)
    R = 6
    rng = np.random.default_rng(4)
    sl = gce.info["site_to_sl"]
    sig_r = np.stack([sig] * R).astype(np.int8)
    for r in range(R):                                   # shuffle within each sublattice
        for k in np.unique(sl):
            idx = np.where(sl == k)[0]
            sig_r[r, idx] = sig_r[r, idx[rng.permutation(len(idx))]]
    E = gce.batched_energy(torch.as_tensor(sig_r).cuda()).cpu().numpy()
    E0 = np.array([orc.energy(x) for x in sig_r])
    assert np.abs(E - E0).max() < 1e-10
    _, beta = ladder(R)
    st = PTState(sig_r, E0, beta, np.zeros(R, np.int32))
    ref = new_state(sig_r, E0, beta)
    T = 600
    for c in range(3):
        run_chunk(gce, st, T, c * T, 21, 64, 8, None, 1, None, True, path=path, cluster=cluster)
        orc.run(ref, T, c * T, 21, None, 1, None, True)
    torch.cuda.synchronize()
    assert np.array_equal(st.sigma.cpu().numpy(), ref["sigma"])
    assert np.abs(st.E.cpu().numpy() - ref["E"]).max() < 1e-9
    assert np.array_equal(st.n_acc.cpu().numpy(), ref["n_acc"]) and np.array_equal(st.rep_of_slot.cpu().numpy(), ref["rep_of_slot"])
    assert int(st.n_acc.sum()) > 0
    # inert sites never move
    inert = np.where([len(gce.info["sl_species"][k]) < 2 for k in sl])[0]
    if len(inert):
        assert np.array_equal(st.sigma.cpu().numpy()[:, inert], sig_r[:, inert])
