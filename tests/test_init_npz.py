"""--init_npz on the CPU: a file whose sites are listed in another order (and shifted by lattice vectors, with
rounding noise) is read back in the MC cell's atom order for every replica; wrong cells, sites, temperatures and
compositions are refused with a message."""
import numpy as np
import pytest

from tests.conftest import random_cell


def _write(tmp_path, s, numbers, temps, perm, shift=True, name="init.npz", cell=None):
    rng = np.random.default_rng(3)
    pos = s.positions[perm].copy()
    if shift:                                          # whole lattice vectors and 1e-4 A noise change nothing
        pos += rng.integers(-2, 3, (len(pos), 3)) @ s.cell + rng.normal(0, 1e-4, pos.shape)
    p = tmp_path / name
    np.savez(p, numbers=numbers[:, perm].astype(np.uint8), positions=pos, cell=s.cell if cell is None else cell,
             temps=np.asarray(temps, float))
    return str(p)


def test_round_trip_in_shuffled_order(tmp_path):
    from neuralce_gb300.mc.init_structures import load_init_npz
    s = random_cell((3, 3, 3), 1)
    rng = np.random.default_rng(0)
    temps = [300.0, 650.0, 1400.0]
    numbers = np.stack([s.numbers[rng.permutation(len(s))] for _ in temps])
    perm = rng.permutation(len(s))
    out, T = load_init_npz(_write(tmp_path, s, numbers, temps, perm), s, temps)
    assert np.array_equal(out, numbers) and np.allclose(T, temps)


def test_refusals(tmp_path):
    from neuralce_gb300.mc.init_structures import load_init_npz
    s = random_cell((3, 3, 3), 2)
    rng = np.random.default_rng(1)
    temps = [400.0, 800.0]
    numbers = np.stack([s.numbers[rng.permutation(len(s))] for _ in temps])
    ident = np.arange(len(s))
    with pytest.raises(ValueError, match="ladder"):
        load_init_npz(_write(tmp_path, s, numbers, temps, ident), s, [400.0, 900.0])
    with pytest.raises(ValueError, match="not the MC cell"):
        load_init_npz(_write(tmp_path, s, numbers, temps, ident, cell=s.cell * 1.01), s, temps)
    bad = numbers.copy(); bad[1, :] = 78
    with pytest.raises(ValueError, match="composition"):
        load_init_npz(_write(tmp_path, s, bad, temps, ident), s, temps)
    off = s.copy(); off.positions = off.positions + np.array([0.9, 0.0, 0.0])   # not the lattice's sites
    p = tmp_path / "off.npz"
    np.savez(p, numbers=numbers, positions=off.positions, cell=s.cell, temps=np.asarray(temps))
    with pytest.raises(ValueError, match="no --init_npz site"):
        load_init_npz(str(p), s, temps)
