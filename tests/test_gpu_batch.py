"""Batches of independent scenes: each scene's result in a batch is the
result of the same scene run alone, bit for bit (and the oracle's)."""
import numpy as np
import pytest

import dem
import dem_scenes
import oracle
from gpu_backend import assert_same_state, copy_scene

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def _items():
    specs = [(600, 0.0, 1), (1500, 0.3, 2), (900, 0.5, 3), (2500, 0.1, 4), (1200, 0.45, 5)]
    items = [dem_scenes.c3_mix_scene(n, f, sd) for n, f, sd in specs]
    items.append(dem_scenes.dense_bed(800, seed=6))
    items.append(dem_scenes.c1_chains(chains=3, length=20, seed=7, pull_velocity=20.0))
    # scenes with large particles (their own cell and partner records)
    items.append(dem_scenes.c2_impact(cols=32, rows=64, seed=8, projectile_radius=8.0, projectile_speed=400.0,
                                      projectiles=2))
    items.append(dem_scenes.c2_impact(cols=40, rows=40, seed=9, projectile_radius=7.0, projectile_speed=300.0))
    return items


def _ev_tuples(ev, scene=None):
    out = []
    for e in ev:
        if scene is None or int(e["scene"]) == scene:
            out.append((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])))
    return sorted(out)


def test_batch_scene_equals_scene_alone():
    items = _items()
    steps = 140
    with dem.Batch(items, reorder_interval=35) as b:
        b.step(steps)
        got = [b.download(k) for k in range(len(items))]
        bev = b.break_events()
    for k, (sc, p, ext) in enumerate(items):
        with dem.Context(sc, p, reorder_interval=35, **ext) as ctx:
            ctx.step(steps)
            alone = ctx.download()
            aev = ctx.break_events()
        assert_same_state(got[k], alone, "scene %d: " % k)
        assert _ev_tuples(bev, k) == _ev_tuples(aev)


def test_batch_with_an_f64_scene_equals_scenes_alone():
    """One scene with F64 distances puts the whole batch on the Simulation
    kernels that carry them (the others alone run kernels compiled without
    them, for their one bond model); every result is still the scene's
    result alone, bit for bit."""
    items = _items()[:4]
    sc, p, ext = dem_scenes.c1_chains(chains=3, length=20, seed=31, pull_velocity=20.0)
    items.insert(2, (sc, p, dict(ext, use_f64=True)))
    steps = 105
    with dem.Batch(items, reorder_interval=35) as b:
        b.step(steps)
        got = [b.download(k) for k in range(len(items))]
        bev = b.break_events()
    for k, (sc, p, ext) in enumerate(items):
        with dem.Context(sc, p, reorder_interval=35, **ext) as ctx:
            ctx.step(steps)
            alone = ctx.download()
            aev = ctx.break_events()
        assert_same_state(got[k], alone, "scene %d: " % k)
        assert _ev_tuples(bev, k) == _ev_tuples(aev)


@pytest.mark.parametrize("scenes", [1, 9])
def test_plain_launches_equal_graphs(scenes):
    """Plain launches (the rebuild kernels launched at every step on grids the
    SMs hold at once, doing nothing unless a rebuild is due) give the graphs'
    results bit for bit, rebuilds included; one scene groups by contact count
    in windows of 1024, several in windows of 128."""
    items = _items()[:scenes]
    runs = []
    for plain in (0, 1):
        with dem.Batch(items, reorder_interval=35, plain_launches=plain) as b:
            b.step(140)
            runs.append(([b.download(k) for k in range(len(items))], b.stats()["reorders"],
                         _ev_tuples(b.break_events())))
    (g, g_re, g_ev), (p, p_re, p_ev) = runs
    assert g_re == p_re and g_re > 0
    for k in range(len(items)):
        assert_same_state(p[k], g[k], "scene %d: " % k)
    assert p_ev == g_ev


def test_batch_matches_oracle():
    items = _items()[:3]
    steps = 90
    with dem.Batch(items) as b:
        b.step(steps)
        got = [b.download(k) for k in range(len(items))]
    for k, (sc, p, ext) in enumerate(items):
        o = copy_scene(sc)
        kw = {}
        if "bond_lambda" in ext:
            kw["bond_lambda"] = ext["bond_lambda"]
        if "bond_sn" in ext:
            kw["bond_sn"], kw["bond_ss"] = ext["bond_sn"], ext["bond_ss"]
        oracle.step(o, p, steps, **kw)
        assert_same_state(got[k], o, "scene %d: " % k)


def test_batch_upload_replaces_one_scene_only():
    items = _items()[:4]
    with dem.Batch(items) as b:
        b.step(40)
        before = [b.download(k) for k in range(4)]
        b.upload(2, items[2][0])
        b.step(0)
        after = [b.download(k) for k in range(4)]
    for k in (0, 1, 3):
        assert_same_state(after[k], before[k], "scene %d: " % k)
    assert np.array_equal(after[2]["pos"], items[2][0]["pos"])


def test_bulk_upload_and_download_equal_per_scene_calls():
    items = _items()
    with dem.Batch(items) as b:
        b.step(70)
        per = [b.download(k) for k in range(len(items))]
        bulk = [b.download(k) for k in range(len(items))]
        for x in bulk:
            for key in ("pos", "vel", "contacts", "data"):
                x[key][:] = 0
        table = dem.SceneTable(list(enumerate(bulk)))  # built once, used twice
        b.download_many(table)
        for x in bulk:
            x["vel"][:] = 0
        b.download_many(table)
        for k in range(len(items)):
            assert_same_state(bulk[k], per[k], "download_many scene %d: " % k)
            assert np.array_equal(bulk[k]["fixity"], per[k]["fixity"])
            assert np.array_equal(bulk[k]["coll_cont"], per[k]["coll_cont"])
        # restore every scene in one call and step on: equal to per-scene restores
        b.upload_many(list(enumerate(per)))
        b.step(35)
        got = [b.download(k) for k in range(len(items))]
    with dem.Batch(items) as c:
        c.step(70)
        for k in range(len(items)):
            c.upload(k, per[k])
        c.step(35)
        ref = [c.download(k) for k in range(len(items))]
    for k in range(len(items)):
        assert_same_state(got[k], ref[k], "upload_many scene %d: " % k)


@pytest.mark.parametrize("host_copies", [0, 1])
def test_transfer_routes_agree(host_copies):
    """Direct device access to the callers' arrays (where the device reaches
    pageable host memory) and copies through the page-locked block give the
    same bytes, for bulk and single-scene calls, both ways."""
    items = _items()
    with dem.Batch(items) as a, dem.Batch(items, host_copies=host_copies) as b:
        a.step(70)
        b.step(70)
        sa = [a.download(k) for k in range(len(items))]
        sb = [b.download(k) for k in range(len(items))]
        bulk = [copy_scene(x) for x in sb]
        for x in bulk:
            for key in ("pos", "fixity", "contacts", "data"):
                x[key][:] = 0
            if x["bonds"].size >= 3:  # not the placeholder of a scene without bonds
                x["bonds"][:] = 0
        b.download_many(list(enumerate(bulk)))
        for k in range(len(items)):
            assert_same_state(sb[k], sa[k], "download scene %d: " % k)
            assert_same_state(bulk[k], sa[k], "download_many scene %d: " % k)
            for key in ("fixity", "bonds", "coll_cont", "material_pointers"):
                assert np.array_equal(bulk[k][key], sa[k][key]), key
        # scenes swapped between the two routes, then stepped on
        a.upload_many([(k, sb[k]) for k in range(len(items))])
        for k in range(len(items)):
            b.upload(k, sa[k])
        a.step(35)
        b.step(35)
        for k in range(len(items)):
            assert_same_state(b.download(k), a.download(k), "after upload, scene %d: " % k)


def _empty_like(sc):
    """A scene of the same settings and materials with no particles."""
    e = {k: (v[:0].copy() if hasattr(v, "shape") and k not in ("materials", "bonds", "coll_cont") else v)
         for k, v in sc.items()}
    e["materials"] = sc["materials"].copy()
    e["bonds"] = np.array([-1], dtype=np.int32)
    e["coll_cont"] = sc["coll_cont"].copy()
    return e


def test_empty_scene_in_a_batch():
    """A scene without particles sits in a batch without disturbing the
    others, downloads as empty, and takes part in bulk transfers."""
    a, p, ext = dem_scenes.dense_bed(700, seed=21)
    b_sc, bp, bext = dem_scenes.c3_mix_scene(900, 0.3, 22)
    items = [(a, p, ext), (_empty_like(a), p, ext), (b_sc, bp, bext)]
    with dem.Batch(items) as bt:
        bt.step(70)
        got = [bt.download(k) for k in range(3)]
        assert got[1]["radii"].size == 0
        bt.upload_many(list(enumerate(got)))
        bt.step(35)
        again = [bt.download(k) for k in range(3)]
    for k in (0, 2):
        sc, pp, ee = items[k]
        with dem.Context(sc, pp, **ee) as ctx:
            ctx.step(70)
            ctx.upload(ctx.download())
            ctx.step(35)
            assert_same_state(again[k], ctx.download(), "scene %d: " % k)


def test_bulk_upload_rejects_a_bad_scene_and_writes_nothing():
    items = _items()[:3]
    with dem.Batch(items) as b:
        b.step(35)
        before = [b.download(k) for k in range(3)]
        bad = copy_scene(before[2])
        bad["contacts"] = bad["contacts"].copy()
        c = bad["contacts"].reshape(-1, 14, 6)
        c[0, 0, 1] = 10 ** 6          # partner out of range
        good = copy_scene(before[0])
        good["vel"] = good["vel"] + np.float32(1.0)
        with pytest.raises(dem.DemError):
            b.upload_many([(0, good), (2, bad)])
        after = [b.download(k) for k in range(3)]
    for k in range(3):
        assert_same_state(after[k], before[k], "scene %d: " % k)


def test_record_one_scene_of_a_batch_equals_the_scene_alone():
    """dem_batch_record of one scene (every scene steps) gives the rows
    dem_record gives for that scene alone."""
    a = dem_scenes.dense_bed(n=800, seed=21)
    b = dem_scenes.c3_mix_scene(1200, 0.3, 22)
    sel = np.zeros(800, np.int32)
    sel[[3, 100, 555]] = 1
    with dem.Batch([a, b]) as bt:
        bt.step(10)
        got = bt.record(0, 60, sel)
        none = bt.record(1, 5, np.zeros(1200, np.int32))
    with dem.Context(a[0], a[1], **a[2]) as ctx:
        ctx.step(10)
        ref = ctx.record(60, sel)
    assert none is None
    assert got.shape == (60, 10) and np.array_equal(got, ref)


def test_dashpot_scene_in_a_batch_equals_the_oracle():
    """A scene with the normal dashpot (restitution 0.5) batched with scenes
    without it: the batch runs the generic kernels and each scene equals the
    oracle with its own setting."""
    a = dem_scenes.dense_bed(n=900, seed=23)
    a = (a[0], a[1], dict(a[2], restitution=0.5))
    b = dem_scenes.c3_mix_scene(1500, 0.3, 24)
    c = dem_scenes.dense_bed(n=600, seed=25)
    items = [a, b, c]
    with dem.Batch(items) as bt:
        bt.step(150)
        got = [bt.download(k) for k in range(3)]
    for k, (sc, p, ext) in enumerate(items):
        o = copy_scene(sc)
        okw = {kk: ext[kk] for kk in ("bond_lambda", "bond_sn", "bond_ss", "restitution") if kk in ext}
        oracle.step(o, p, 150, **okw)
        assert_same_state(got[k], o, "scene %d: " % k)
