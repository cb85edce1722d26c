"""GPU parity on the benchmark workloads themselves, not only on crops and
short runs: the c0 settle over its whole 2,000-step horizon (and on until
the bottom rows land), the c2 bed crop with the configured r = 40, v = 50
projectile until its contact set is capped, and scenes drawn from the c3 mix
the bench times, batched with the bench's autotuned knobs.  Whole states and
break-event lists are compared bit for bit against the oracle."""
import numpy as np
import pytest

import dem
import dem_scenes
import oracle
from gpu_backend import assert_same_state, contact_pairs, copy_scene, run_both

pytestmark = pytest.mark.gpu

# the knobs the autotuner picked for the 512-scene mix in the bench line
BENCH_KNOBS = {"search_cell_factor": 0.85, "list_skin": 0.2, "block_size": 128, "reorder_interval": 70,
               "split_narrow": 0, "unfused_lom": 0}


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def _events(ev):
    return sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in ev)


def test_c0_settle_whole_horizon_bit_exact():
    """c0 (4,096 disks, dt 1e-4): its 2,000 steps move every disk ~0.2 down,
    less than any lattice gap, so the first disk-disk contacts appear only
    after ~7,000 steps, when the bottom rows have landed on the floor; the
    run is compared at 2,000 steps and again at 10,000, by then in contact."""
    sc, p, ext = dem_scenes.c0_settle(n=4096, seed=0)
    o = copy_scene(sc)
    with dem.Context(sc, p) as ctx:
        ctx.step(2000)
        g = ctx.download()
        oracle.step(o, p, 2000)
        assert_same_state(g, o, "c0 at 2000 steps: ")
        ctx.step(8000)
        g = ctx.download()
        oracle.step(o, p, 8000, step_base=2000)
    assert len(contact_pairs(o)) > 50, "the bottom rows must be in contact"
    assert_same_state(g, o, "c0 at 10000 steps: ")


def test_c2_crop_with_the_configured_projectile_bit_exact():
    """The c2 bed model (log-normal radii, 30 % bonded clusters, Weibull
    strengths) on 128 x 256 lattice sites with the configured projectile,
    r = 40 at v = 50 (dt 5e-5): after 800 steps its contact set is at the
    cap of 14 while more bed disks touch it, thousands of bonds have broken,
    and state and break events equal the oracle's."""
    sc, p, ext = dem_scenes.c2_impact(cols=128, rows=256)
    n = sc["radii"].size
    g, o, gev, oev = run_both(sc, p, 800, chunk=200, **ext)
    assert_same_state(g, o)
    assert _events(gev) == _events(oev)
    assert len(oev) > 1000
    c = g["contacts"].reshape(-1, 14, 6)
    assert (c[n - 1, :, 1] != -1).sum() == 14, "the projectile's contact set must reach the cap"
    assert (c[:, :, 1] == n - 1).sum() > 14


def test_c3_mix_scenes_batched_with_the_bench_knobs_bit_exact():
    """16 scenes of the c3 mix (seed 0, every 32nd of the 512, so sizes span
    the log-uniform range) in one batch with the bench's knobs, 400 steps:
    each scene equals the oracle's run of it."""
    idx = list(range(0, 512, 32))
    items = dem_scenes.c3_batch(n_scenes=512, seed=0, indices=idx)
    sizes = [it[0]["radii"].size for it in items]
    assert min(sizes) < 4000 and max(sizes) > 30000
    with dem.Batch(items, **BENCH_KNOBS) as b:
        b.step(400)
        got = [b.download(k) for k in range(len(items))]
        gev = b.break_events()
    for k, (sc, p, ext) in enumerate(items):
        o = copy_scene(sc)
        okw = {kk: ext[kk] for kk in ("bond_lambda", "bond_sn", "bond_ss") if kk in ext}
        oev, _ = oracle.step(o, p, 400, **okw)
        assert_same_state(got[k], o, "c3 scene %d: " % idx[k])
        assert _events(gev[gev["scene"] == k]) == _events(oev), "c3 scene %d: break events differ" % idx[k]
