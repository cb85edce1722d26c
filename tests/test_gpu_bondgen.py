"""GPU bond generation (dem_generate_bonds) against the oracle's literal
restatement of State::regen_bonds (src/state.rs:291-367): the same bonds in
the same order (status, angle and length bits) and the same contact records,
bit for bit."""
import numpy as np
import pytest

import dem
import dem_scenes
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def _packing(n, seed, pitch=2.0, rlo=0.7, rhi=1.3):
    rng = np.random.default_rng(seed)
    cols = int(np.sqrt(n))
    idx = np.arange(n)
    pos = np.zeros((n, 2), np.float32)
    pos[:, 0] = (idx % cols) * pitch + rng.uniform(-0.15, 0.15, n)
    pos[:, 1] = (idx // cols) * pitch + rng.uniform(-0.15, 0.15, n)
    radii = rng.uniform(rlo, rhi, n).astype(np.float32)
    # shuffle so that index order and space order differ
    perm = rng.permutation(n)
    return pos[perm].copy(), radii[perm].copy()


@pytest.mark.parametrize("max_bonds", [1, 6, 14])
def test_generated_bonds_equal_regen_bonds(max_bonds):
    pos, radii = _packing(4000, seed=max_bonds)
    gb, gc = dem.generate_bonds(pos, radii, max_bonds=max_bonds)
    ob, oc = oracle.regen_bonds(pos.reshape(-1), radii, max_bonds=max_bonds)
    assert gb.size > 3 * 1000
    assert np.array_equal(gb, ob)
    assert np.array_equal(gc, oc)


def test_slot_cap_when_many_smaller_partners_bond_first():
    # a large disk (last index) ringed by 40 small ones with lower indices:
    # every ring member bonds to it before it makes bonds of its own, so its
    # 14 slots fill and later bonds exist without slots
    k = 40
    ang = np.arange(k) * 2 * np.pi / k
    R, r = 6.0, 0.45
    pos = np.zeros((k + 1, 2), np.float32)
    pos[:k, 0] = (R + r) * np.cos(ang)
    pos[:k, 1] = (R + r) * np.sin(ang)
    radii = np.full(k + 1, r, np.float32)
    radii[k] = R
    gb, gc = dem.generate_bonds(pos.reshape(-1), radii)
    ob, oc = oracle.regen_bonds(pos.reshape(-1), radii)
    assert np.array_equal(gb, ob) and np.array_equal(gc, oc)
    c = gc.reshape(-1, 14, 6)
    assert (c[k, :, 1] != -1).sum() == 14
    assert gb.size // 3 > 14


def test_chain_scene_bonds():
    sc, p, ext = dem_scenes.c1_chains(chains=5, length=50, seed=2)
    gb, gc = dem.generate_bonds(sc["pos"], sc["radii"])
    assert np.array_equal(gb, sc["bonds"])
    assert np.array_equal(gc, sc["contacts"])


def test_no_bonds_and_empty():
    pos = np.array([0.0, 0.0, 10.0, 0.0], np.float32)
    radii = np.array([1.0, 1.0], np.float32)
    gb, gc = dem.generate_bonds(pos, radii)
    assert gb.tolist() == [-1] and (gc == -1).all()
    gb, gc = dem.generate_bonds(np.zeros(0, np.float32), np.zeros(0, np.float32))
    assert gb.tolist() == [-1] and gc.size == 0
