"""Serving: scenes admitted while others run, each stopping at its own
horizon, give exactly the results of running them alone."""
import numpy as np
import pytest

import dem
import dem_scenes
from gpu_backend import assert_same_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def _alone(sc, p, ext, steps):
    with dem.Context(sc, p, **ext) as ctx:
        ctx.step(steps)
        return ctx.download(), ctx.break_events()


def _ev(ev):
    return sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in ev)


@pytest.mark.parametrize("borrow", [False, True])
def test_each_result_equals_the_scene_alone(borrow):
    """Requests admitted while others run equal each scene run alone, whether
    the server copies each request's scene at submit or refers to the
    caller's arrays until the request is done (dem_server_submit_borrowed)."""
    reqs = [
        (dem_scenes.c3_mix_scene(1500, 0.3, 11), 100),
        (dem_scenes.dense_bed(900, seed=12), 70),
        (dem_scenes.c1_chains(chains=3, length=24, seed=13, pull_velocity=20.0), 130),
        (dem_scenes.c3_mix_scene(2200, 0.0, 14), 45),
        (dem_scenes.c3_mix_scene(700, 0.5, 15), 60),
    ]
    with dem.Server(memory_budget_bytes=1 << 30, max_active_particles=4000, max_scenes=8,
                    reorder_interval=35) as sv:
        ids = {}
        # two requests up front, the others arrive while those run
        for k in (0, 1):
            (sc, p, ext), h = reqs[k]
            ids[sv.submit(sc, p, h, borrow=borrow, **ext)] = k
        sv.advance(35)
        (sc, p, ext), h = reqs[2]
        ids[sv.submit(sc, p, h, borrow=borrow, **ext)] = 2
        sv.advance(35)
        for k in (3, 4):
            (sc, p, ext), h = reqs[k]
            ids[sv.submit(sc, p, h, borrow=borrow, **ext)] = k
        done = {}
        for _ in range(40):
            sv.advance(35)
            for rid in sv.poll():
                done[rid] = sv.fetch(rid)
            if len(done) == len(reqs):
                break
        st = sv.stats()
    assert len(done) == len(reqs), st
    admits = {}
    for rid, (got, times, ev) in done.items():
        k = ids[rid]
        (sc, p, ext), h = reqs[k]
        ref, rev = _alone(sc, p, ext, h)
        assert_same_state(got, ref, "request %d: " % k)
        assert _ev(ev) == _ev(rev)
        admits[k] = times[1]
        assert times[0] <= times[1] <= times[2]
    # max_active_particles = 4000 delays request 3 (2200 particles) until room frees
    assert admits[3] >= admits[2]


def test_f64_request_joins_and_leaves_a_running_world():
    """An F64 request admitted among FP32 scenes moves the world onto the
    Simulation kernels that carry the F64 paths, and its retirement moves it
    back, while the others run on; every result equals the scene alone."""
    chains = dem_scenes.c1_chains(chains=3, length=20, seed=22, pull_velocity=20.0)
    reqs = [
        (dem_scenes.c3_mix_scene(1200, 0.3, 21), 175),
        ((chains[0], chains[1], dict(chains[2], use_f64=True)), 70),
        (dem_scenes.dense_bed(700, seed=23), 105),
    ]
    with dem.Server(memory_budget_bytes=1 << 30, max_scenes=4, reorder_interval=35) as sv:
        ids = {}
        (sc, p, ext), h = reqs[0]
        ids[sv.submit(sc, p, h, **ext)] = 0
        sv.advance(35)
        (sc, p, ext), h = reqs[1]
        ids[sv.submit(sc, p, h, **ext)] = 1
        sv.advance(35)
        (sc, p, ext), h = reqs[2]
        ids[sv.submit(sc, p, h, **ext)] = 2
        done = {}
        for _ in range(20):
            sv.advance(35)
            for rid in sv.poll():
                done[rid] = sv.fetch(rid)
            if len(done) == len(reqs):
                break
    assert len(done) == len(reqs)
    for rid, (got, times, ev) in done.items():
        k = ids[rid]
        (sc, p, ext), h = reqs[k]
        ref, rev = _alone(sc, p, ext, h)
        assert_same_state(got, ref, "request %d: " % k)
        assert _ev(ev) == _ev(rev)


def test_capacity_refuses_nothing_and_queues():
    sc, p, ext = dem_scenes.dense_bed(3000, seed=21)
    with dem.Server(memory_budget_bytes=1 << 30, max_active_particles=3000, max_scenes=4) as sv:
        a = sv.submit(sc, p, 40)
        b = sv.submit(sc, p, 40)
        sv.advance(35)
        s1 = sv.stats()
        assert s1["running"] == 1 and s1["queued"] == 1
        out = {}
        for _ in range(10):
            sv.advance(35)
            for rid in sv.poll():
                out[rid] = sv.fetch(rid)
        assert set(out) == {a, b}
        ga, _, _ = out[a]
        gb, _, _ = out[b]
        assert_same_state(ga, gb)


def test_request_beyond_the_arenas_is_refused_and_the_queue_moves_on():
    """A request larger than the particle arena is refused at submit; one whose
    bonds cannot fit even into empty arenas is failed at admission (poll lists
    it, fetch raises the admission error) and the requests behind it run."""
    small, p, ext = dem_scenes.dense_bed(900, seed=31)
    chains = dem_scenes.c1_chains(chains=20, length=64, seed=32, pull_velocity=0.0)
    with dem.Server(memory_budget_bytes=1 << 30, max_active_particles=2048, max_scenes=4,
                    bonds_per_particle=0.0) as sv:
        cap = sv.stats()["capacity_particles"]
        big, pb, eb = dem_scenes.dense_bed(cap + 1000, seed=33)
        with pytest.raises(dem.DemError) as e:
            sv.submit(big, pb, 10, **eb)
        assert e.value.code == -7
        (csc, cp, cext) = chains
        bad = sv.submit(csc, cp, 10, **cext)      # 20 x 63 bonds; the bond arena holds 1024
        good = sv.submit(small, p, 40, **ext)
        seen = set()
        for _ in range(6):
            sv.advance(35)
            seen.update(sv.poll())
        assert seen == {bad, good}
        with pytest.raises(dem.DemError) as e:
            sv.fetch(bad)
        assert e.value.code == -7
        sv.release(bad)
        got, _, _ = sv.fetch(good)
    ref, _ = _alone(small, p, ext, 40)
    assert_same_state(got, ref)


def test_cancel_queued_and_running_requests():
    """Cancelling a running request frees its ranges and a queued one never
    runs; the requests left give the results of running alone."""
    a_sc, a_p, a_ext = dem_scenes.dense_bed(1500, seed=41)
    b_sc, b_p, b_ext = dem_scenes.c3_mix_scene(1400, 0.3, 42)
    c_sc, c_p, c_ext = dem_scenes.c3_mix_scene(1200, 0.2, 43)
    with dem.Server(memory_budget_bytes=1 << 30, max_active_particles=1600, max_scenes=4) as sv:
        a = sv.submit(a_sc, a_p, 400, **a_ext)
        b = sv.submit(b_sc, b_p, 50, **b_ext)   # waits: a holds the particle budget
        sv.advance(35)
        st = sv.stats()
        assert st["running"] == 1 and st["queued"] == 1
        sv.cancel(b)
        assert sv.stats()["queued"] == 0
        sv.cancel(a)
        st = sv.stats()
        assert st["running"] == 0 and st["active_particles"] == 0
        c = sv.submit(c_sc, c_p, 70, **c_ext)
        done = {}
        for _ in range(8):
            sv.advance(35)
            for rid in sv.poll():
                done[rid] = sv.fetch(rid)
        assert set(done) == {c}
        with pytest.raises(dem.DemError):
            sv.events(a)                         # the cancelled id is unknown
    ref, _ = _alone(c_sc, c_p, c_ext, 70)
    assert_same_state(done[c][0], ref)
