"""The bench's workloads are what its JSON lines and the measured numbers
describe: the seeded generators must keep producing the same scenes (a
changed generator would silently change what every number measures)."""
import numpy as np

import dem_scenes


def test_c3_batch_mix():
    items = dem_scenes.c3_batch(512)
    sizes = np.array([int(sc["radii"].shape[0]) for sc, _, _ in items])
    bonds = sum(int(sc["bonds"].size // 3) for sc, _, _ in items if sc["bonds"].size >= 3)
    assert len(items) == 512
    assert int(sizes.sum()) == 8645025
    assert (int(sizes.min()), int(sizes.max())) == (1001, 63261)
    assert bonds == 2152857
    models = sorted({int(p["bonds"]) for _, p, _ in items})
    assert models == [0, 3]  # loose settles without bonds, chains with parallel bonds


def test_c2_impact_scene():
    sc, p, ext = dem_scenes.c2_impact()
    n = int(sc["radii"].shape[0])
    assert n == 4194305 and int(sc["bonds"].size // 3) == 1182950
    assert p["bonds"] == 3
    r = sc["radii"]
    assert float(r.max()) == 40.0 and int((r > 4.0).sum()) == 1  # the projectile
    assert abs(float(np.median(r)) - 1.0) < 0.01
