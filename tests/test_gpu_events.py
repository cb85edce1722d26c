"""Fix / Drop / Release events and the device datum.

The events are restated on the oracle's scene arrays from the shaders
(src/shaders/event_handling/Fix.wgsl:44-54, Drop.wgsl:34-41,
Release.wgsl:77-92); both sides then step on and must stay bit-identical.
get_datum (src/state.rs:708-737) is restated as a double loop in index order
and must equal dem_get_datum exactly."""
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


def _fix(o, sel):
    for i in np.nonzero(sel == 1)[0]:
        sel[i] = 2
        o["fixity"][6 * i:6 * i + 6] = 1
        o["vel"][2 * i:2 * i + 2] = 0.0
        o["rot_vel"][i] = 0.0


def _drop(o, sel):
    for i in np.nonzero(sel == 2)[0]:
        sel[i] = 1
        o["fixity"][6 * i:6 * i + 6] = 0


def _release(o, sel, dT, throw, dx, dy, ticks):
    q = np.float32(dT) * np.float32(ticks)
    for i in np.nonzero(sel != 0)[0]:
        f = o["fixity"]
        f[6 * i:6 * i + 3] = f[6 * i + 3:6 * i + 6]
        if throw:
            o["vel"][2 * i] = np.float32(dx) / q
            o["vel"][2 * i + 1] = np.float32(dy) / q


def _datum(st, sel):
    s = [0.0] * 10
    idx = [i for i in range(sel.size) if sel[i] != 0]
    if not idx:
        return None
    d = st["data"]
    for i in idx:
        s[0] += float(st["pos"][2 * i]); s[1] += float(st["pos"][2 * i + 1])
        s[2] += float(d[7 * i + 4]); s[3] += float(d[7 * i + 5]); s[4] += float(st["rot"][i])
        s[5] += float(d[7 * i + 6]); s[6] += abs(float(d[7 * i])); s[7] += float(d[7 * i + 1])
        s[8] += float(d[7 * i + 2]); s[9] += float(d[7 * i + 3])
    return np.array([v if k == 6 else v / len(idx) for k, v in enumerate(s)])


def test_fix_drop_release_and_datum_match_oracle():
    sc, p, ext = dem_scenes.dense_bed(n=900, seed=21)
    rng = np.random.default_rng(5)
    fx = sc["fixity"].reshape(-1, 6)
    some = rng.random(fx.shape[0]) < 0.3
    fx[some, 3:6] = rng.integers(0, 3, size=(some.sum(), 3))
    sc["data"][3::7] = rng.random(fx.shape[0]).astype(np.float32)
    o = copy_scene(sc)
    n = sc["radii"].size
    sel_g = np.zeros(n, np.int32)
    sel_g[::9] = 1
    sel_o = sel_g.copy()
    step_base = 0
    with dem.Context(sc, p) as ctx:
        def both(k):
            nonlocal step_base
            ctx.step(k)
            oracle.step(o, p, k, step_base=step_base)
            step_base += k
        both(40)
        ctx.event(dem.EVENT_FIX, sel_g)
        _fix(o, sel_o)
        assert np.array_equal(sel_g, sel_o) and (sel_g == 2).sum() == (n + 8) // 9
        both(60)
        assert_same_state(ctx.download(), o, "after fix: ")
        ctx.event(dem.EVENT_DROP, sel_g)
        _drop(o, sel_o)
        assert np.array_equal(sel_g, sel_o)
        both(60)
        assert_same_state(ctx.download(), o, "after drop: ")
        rel = np.zeros(n, np.int32)
        rel[some] = 1
        ctx.event(dem.EVENT_RELEASE, rel, throw=True, del_x=0.3, del_y=-0.7, ticks=12)
        _release(o, rel, p["dT"], True, 0.3, -0.7, 12)
        both(80)
        st = ctx.download()
        assert_same_state(st, o, "after release: ")
        assert np.array_equal(st["fixity"], o["fixity"])
        got = ctx.datum(sel_g)
        assert got is not None
        assert np.array_equal(got, _datum(st, sel_g))
        assert np.array_equal(got, _datum(o, sel_g))
        assert ctx.datum(np.zeros(n, np.int32)) is None
