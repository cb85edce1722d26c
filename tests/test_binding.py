"""The ctypes binding's marshalling, checked without a GPU: scene structs
point at the dicts' arrays, a wrong array length is refused before any call
reaches the library, and a prepared SceneTable lays out its structs the way
the bulk calls read them."""
import ctypes as C

import numpy as np
import pytest

import dem
import dem_scenes


def test_scene_struct_points_at_the_arrays():
    sc, p, ext = dem_scenes.dense_bed(300, seed=1)
    st = dem.make_scene(sc)
    assert st.n_particles == 300
    for k in dem.F32_KEYS + dem.I32_KEYS:
        assert getattr(st, k) == sc[k].ctypes.data, k
    assert list(st.coll_cont) == [int(v) for v in sc["coll_cont"]]


def test_wrong_length_is_refused():
    sc, p, ext = dem_scenes.dense_bed(300, seed=1)
    bad = dict(sc)
    bad["contacts"] = sc["contacts"][:-6].copy()
    with pytest.raises(ValueError):
        dem.make_scene(bad)
    bad = dict(sc)
    bad["vel"] = sc["vel"].astype(np.float64)
    with pytest.raises(TypeError):
        dem.make_scene(bad)


def test_direct_data_pointer_matches_numpy():
    for a in (np.zeros(7, np.float32), np.arange(12, dtype=np.int32)[3:], np.ones((4, 3), np.float32)):
        assert dem._addr(a) == a.ctypes.data


def test_scene_table_layout():
    scenes = [dem_scenes.dense_bed(100 + 50 * k, seed=k)[0] for k in range(5)]
    pairs = [(4 - k, sc) for k, sc in enumerate(scenes)]
    t = dem.SceneTable(pairs)
    assert t.n == 5 and list(t.idx) == [4, 3, 2, 1, 0]
    for k, (_, sc) in enumerate(pairs):
        st = dem.Scene.from_address(int(t.ptrs[k]))
        assert st.n_particles == len(sc["radii"]) and st.pos == sc["pos"].ctypes.data
    # control words written into the structs come back into the dicts
    for k in range(5):
        t.structs[k].coll_cont[:] = [k, k + 1, k + 2, 0]
    t.read_control()
    for k, (_, sc) in enumerate(pairs):
        assert list(sc["coll_cont"]) == [k, k + 1, k + 2, 0]
