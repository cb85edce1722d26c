"""The oracle's results do not depend on how it is run: one host thread or
many, all steps in one call or split over several, give byte-identical
states and break-event lists.  It is the checker of every parity test."""
import numpy as np
import pytest

import dem_scenes
import oracle
from gpu_backend import copy_scene


def _run(sc, p, steps, threads, **kw):
    o = copy_scene(sc)
    ev, _ = oracle.step(o, p, steps, threads=threads, **kw)
    return o, ev


@pytest.mark.parametrize("workload", ["settle", "chains"])
def test_thread_count_does_not_change_results(workload):
    if workload == "settle":
        sc, p, ext = dem_scenes.c0_settle(n=3000, seed=11, box=(60, 120), spacing=2.05)
        kw = {}
        steps = 120
    else:
        sc, p, ext = dem_scenes.c1_chains(chains=8, length=64, seed=12, pull_velocity=30.0)
        kw = {"bond_lambda": ext["bond_lambda"], "bond_sn": ext["bond_sn"], "bond_ss": ext["bond_ss"]}
        steps = 200
    runs = [_run(sc, p, steps, t, **kw) for t in (1, 3, 0)]
    (a, ea) = runs[0]
    for b, eb in runs[1:]:
        for k in a:
            if k == "grid":
                continue
            assert np.asarray(a[k]).tobytes() == np.asarray(b[k]).tobytes(), k
        assert np.asarray(ea).tobytes() == np.asarray(eb).tobytes()
    if workload == "chains":
        assert len(ea) > 0, "the pulled chains should break bonds"


@pytest.mark.parametrize("interval", [1, 3])
def test_chunked_calls_equal_one_call(interval):
    """Stepping in chunks (as the parity tests do on both sides) equals one
    call of all the steps: the control words carry the interval schedule
    across calls, and the events keep their step numbers."""
    sc, p, ext = dem_scenes.c1_chains(chains=6, length=48, seed=13, pull_velocity=30.0)
    p = dict(p, collision_interval=interval)
    kw = {"bond_lambda": ext["bond_lambda"], "bond_sn": ext["bond_sn"], "bond_ss": ext["bond_ss"]}
    whole, ew = _run(sc, p, 210, 0, **kw)
    part = copy_scene(sc)
    evs = []
    done = 0
    for k in (1, 40, 69, 100):
        ev, _ = oracle.step(part, p, k, step_base=done, **kw)
        evs.append(ev)
        done += k
    for k in whole:
        if k == "grid":
            continue
        assert np.asarray(whole[k]).tobytes() == np.asarray(part[k]).tobytes(), k
    ep = np.concatenate(evs)
    assert len(ew) > 0
    assert np.asarray(ew).tobytes() == np.asarray(ep).tobytes()
