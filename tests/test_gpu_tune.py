"""Autotuner and the knobs it turns: search-cell size (3 x 3 or 5 x 5 cell
searches), candidate-list skin (re-sort frequency), particle-kernel block
size, steps per captured graph and the one- or two-kernel Simulation pass
change speed only -- every scene's state and bond-break events are the same
bit for bit under any setting.  So does how often a rebuild reorders the
particle arrays into cell order (every rebuild, or only the first)."""
import pytest

import dem
import dem_scenes
from gpu_backend import assert_same_state

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def _items():
    specs = [(700, 0.0, 11), (1800, 0.4, 12), (3000, 0.2, 13)]
    items = [dem_scenes.c3_mix_scene(n, f, sd) for n, f, sd in specs]
    items.append(dem_scenes.dense_bed(1500, seed=14))
    items.append(dem_scenes.c1_chains(chains=4, length=30, seed=15, pull_velocity=20.0))
    items.append(dem_scenes.c2_impact(cols=32, rows=48, seed=16, projectile_radius=8.0, projectile_speed=300.0))
    return items


def _run(items, steps, **kw):
    with dem.Batch(items, **kw) as b:
        b.step(steps)
        states = [b.download(k) for k in range(len(items))]
        ev = b.break_events()
    evs = sorted((int(e["scene"]), int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"]))
                 for e in ev)
    return states, evs


@pytest.mark.parametrize("knobs", [
    dict(search_cell_factor=0.68, list_skin=0.45, block_size=128, reorder_interval=21, split_narrow=1),
    dict(search_cell_factor=1.36, list_skin=0.1, block_size=512, reorder_interval=70, unfused_lom=1),
    dict(list_skin=0.1, reorder_every=1),
    dict(list_skin=0.1, reorder_every=100000, plain_launches=1),
])
def test_knobs_do_not_change_results(knobs):
    items = _items()
    steps = 210
    ref, ref_ev = _run(items, steps)
    got, got_ev = _run(items, steps, **knobs)
    for k in range(len(items)):
        assert_same_state(got[k], ref[k], "scene %d: " % k)
    assert got_ev == ref_ev


def test_autotune_picks_listed_values_and_keeps_results():
    items = _items()
    chosen, info = dem.autotune(items, sample_particles=6000, trial_steps=70)
    assert chosen["search_cell_factor"] in (pytest.approx(0.68), pytest.approx(0.85), 1.0, pytest.approx(1.36))
    assert chosen["list_skin"] in (pytest.approx(0.1), pytest.approx(0.2), pytest.approx(0.3), pytest.approx(0.45))
    assert chosen["block_size"] in (128, 256, 512)
    assert chosen["reorder_interval"] in (21, 35, 70)
    assert chosen["split_narrow"] in (0, 1) and chosen["unfused_lom"] in (0, 1)
    assert info["trials"] >= 10 and info["ms_per_step"] <= info["default_ms_per_step"]
    ref, ref_ev = _run(items, 105)
    got, got_ev = _run(items, 105, **chosen)
    for k in range(len(items)):
        assert_same_state(got[k], ref[k], "scene %d: " % k)
    assert got_ev == ref_ev


def _dense_items():
    # beds of c2's model (about two particles a search cell at the default
    # cell size): their candidate lists come from neighbour cells staged in
    # shared memory, whose runs of 128 cell-list entries here also straddle
    # scene boundaries and wrap grid rows
    items = [dem_scenes.c2_impact(cols=40, rows=90, seed=20 + k, projectile_radius=5.0, projectile_speed=250.0)
             for k in range(3)]
    items.append(dem_scenes.c2_impact(cols=17, rows=120, seed=30, projectile_radius=5.0, projectile_speed=200.0))
    return items


@pytest.mark.parametrize("knobs", [
    dict(search_cell_factor=1.36, list_skin=0.2),   # larger cells: staged, 3 x 3
    dict(search_cell_factor=0.68, list_skin=0.2),   # 5 x 5 search of smaller cells
    dict(search_cell_factor=1.0, list_skin=0.45, plain_launches=1),
])
def test_dense_batch_lists_do_not_depend_on_the_cell_size(knobs):
    """The staged list build (dense worlds) and the cell-table scan (sparse
    ones) build the same candidate lists: a batch of dense beds with a fast
    projectile each (rebuilds every few steps) steps bit for bit alike under
    cell sizes on both sides of the density threshold and both stencils."""
    items = _dense_items()
    sc, p, ext = items[0]
    with dem.Context(sc, p, **ext) as ctx:  # default cell size: a dense world
        gw, gh = ctx.search_grid()[3:5]
    assert 2 * sc["radii"].shape[0] >= 3 * gw * gh
    ref, ref_ev = _run(items, 280)
    got, got_ev = _run(items, 280, **knobs)
    for k in range(len(items)):
        assert_same_state(got[k], ref[k], "scene %d: " % k)
    assert got_ev == ref_ev
