"""GPU parity: the CUDA path against the CPU oracle on identical inputs.

Both follow the reference's expressions with the same float rounding (no
contraction on either side), and both resolve the reference's races the same
way, so whole states are compared bit for bit: positions, velocities,
accelerations, diagnostics, every contact record (pairs, slot positions,
tangential histories) and every bond record, plus the bond-break event list.
"""
import os

import numpy as np
import pytest

import dem
import dem_scenes
import state_io
import oracle
import replay
from gpu_backend import GpuBackend, assert_same_state, contact_pairs, copy_scene, run_both

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build_lib
    build_lib.build()


def test_texps_replay_equals_oracle_and_golden(golden_dir):
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "TEXPS.bin"))
    gb = GpuBackend(scene, uni, info["use_f64"])
    gx = replay.Replayer(gb, info["scripts"], len(scene["radii"])).run()
    ob = replay.OracleBackend(scene, uni, info["use_f64"])
    ox = replay.Replayer(ob, info["scripts"], len(scene["radii"])).run()
    traces = np.load(os.path.join(golden_dir, "traces.npz"))
    assert set(gx) == set(ox)
    for k in gx:
        assert np.array_equal(gx[k], ox[k]), k
    assert np.array_equal(gx["TEXP_1"][:, 7], traces["TEXP_1"][:, 7])


def test_record_path_reproduces_the_texp_exports(golden_dir, tmp_path):
    """Advance with Record on through the device record path (dem_record:
    the datum of every step gathered on the device, read back once per
    call) gives every exported trace of the TEXPS experiments exactly as a
    state readback after every step does; TEXP_1's Data1 equals the
    reference's export bit for bit, and the CSV export reads back to the
    same numbers."""
    import record
    from gpu_backend import RecordingGpuBackend
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "TEXPS.bin"))
    n = len(scene["radii"])
    gx = replay.Replayer(GpuBackend(scene, uni, info["use_f64"]), info["scripts"], n).run()
    rx = replay.Replayer(RecordingGpuBackend(scene, uni, info["use_f64"]), info["scripts"], n).run()
    assert set(gx) == set(rx) and len(rx) >= 13
    for k in gx:
        assert np.array_equal(gx[k], rx[k]), k
    traces = np.load(os.path.join(golden_dir, "traces.npz"))
    assert np.array_equal(rx["TEXP_1"][:, 7], traces["TEXP_1"][:, 7])
    path = tmp_path / "TEXP_1.csv"
    record.write_csv(str(path), rx["TEXP_1"])
    assert open(path).readline().strip() == record.HEADER
    back = np.loadtxt(str(path), delimiter=",", skiprows=1, dtype=np.float64, ndmin=2)
    assert np.array_equal(back[:, :11], rx["TEXP_1"])


def test_chain_texp_replay_equals_oracle(golden_dir):
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "Chain_TEXP.bin"))
    gx = replay.Replayer(GpuBackend(scene, uni, info["use_f64"]), info["scripts"], 3).run()
    ox = replay.Replayer(replay.OracleBackend(scene, uni, info["use_f64"]), info["scripts"], 3).run()
    for k in ox:
        assert np.array_equal(gx[k], ox[k]), k


@pytest.mark.parametrize("n,steps", [(600, 400), (2000, 150)])
def test_dense_settle_bit_exact(n, steps):
    sc, p, ext = dem_scenes.dense_bed(n=n, seed=1)
    g, o, _, _ = run_both(sc, p, steps, chunk=50, reorder_interval=7)
    assert len(contact_pairs(o)) > n  # the scene is in contact
    assert_same_state(g, o)


def test_c0_default_scene_bit_exact():
    sc, p, ext = dem_scenes.c0_settle(n=4096, seed=0)
    g, o, _, _ = run_both(sc, p, 60)
    assert_same_state(g, o)


def test_chains_with_breaks_bit_exact():
    sc, p, ext = dem_scenes.c1_chains(chains=6, length=40, seed=3, pull_velocity=20.0)
    g, o, gev, oev = run_both(sc, p, 700, chunk=100, **ext)
    assert len(oev) > 0, "the pull must break bonds"
    assert_same_state(g, o)
    got = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in gev)
    ref = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in oev)
    assert got == ref


def test_large_world_end_of_step_kernels_bit_exact():
    """Above 131072 particles the step ends in separate one-warp kernels
    (rebuild decision, break application, counters) instead of the last warp
    of the LOM and Simulation kernels; breaks, events and state must not
    change."""
    sc, p, ext = dem_scenes.c1_chains(chains=640, length=256, seed=3, pull_velocity=20.0)
    assert sc["radii"].size > 131072
    g, o, gev, oev = run_both(sc, p, 300, chunk=100, **ext)
    assert len(oev) > 0, "the pull must break bonds"
    assert_same_state(g, o)
    got = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in gev)
    ref = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in oev)
    assert got == ref


@pytest.mark.parametrize("projectiles", [1, 3])
def test_large_particle_impact_bit_exact(projectiles):
    """A bonded, polydisperse bed hit by projectiles of radius 12 (12x the
    median): the projectiles live outside the search cells and get their
    partners from one thread block each; their contact sets hit the cap of 14
    while more bed particles touch them, and side by side they touch each
    other."""
    sc, p, ext = dem_scenes.c2_impact(cols=64, rows=128, seed=1, projectile_radius=12.0,
                                      projectile_speed=400.0, projectiles=projectiles)
    n = sc["radii"].size
    with dem.Context(sc, p, **ext) as ctx:
        keys, _, _ = ctx.broad_phase()
        _, _, _, gw, gh = ctx.search_grid()
    assert (keys[n - projectiles:] == gw * gh).all(), "projectiles must sit in the large-particle cell"
    g, o, gev, oev = run_both(sc, p, 600, chunk=100, **ext)
    assert_same_state(g, o)
    got = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in gev)
    ref = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in oev)
    assert got == ref
    c = g["contacts"].reshape(-1, 14, 6)
    assert (c[n - 1, :, 1] != -1).sum() == 14, "the projectile's contact set must reach the cap"
    assert (c[:, :, 1] == n - 1).sum() > 14
    if projectiles > 1:
        assert (c[n - 1, :, 1] >= n - projectiles).any() or (c[n - 2, :, 1] >= n - projectiles).any()


@pytest.mark.parametrize("reorder_every", [1, 100000])
def test_rebuilds_with_and_without_reorder_bit_exact(reorder_every):
    """A rebuild every one or two steps (skin 0.02 r_max) on a bonded bed hit
    by two projectiles: with the particle arrays reordered into cell order at
    every rebuild, or only at the first (the large particles then found
    through the cell list, not by position), the run equals the oracle."""
    sc, p, ext = dem_scenes.c2_impact(cols=48, rows=64, seed=7, projectile_radius=10.0,
                                      projectile_speed=300.0, projectiles=2)
    g, o, gev, oev = run_both(sc, p, 300, chunk=100, list_skin=0.02, reorder_every=reorder_every, **ext)
    assert_same_state(g, o)
    got = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in gev)
    ref = sorted((int(e["step"]), int(e["bond"]), int(e["code"]), int(e["a"]), int(e["b"])) for e in oev)
    assert got == ref
    with dem.Context(sc, p, list_skin=0.02, reorder_every=reorder_every, **ext) as ctx:
        ctx.step(50)
        assert ctx.stats()["reorders"] >= 20


def test_dashpot_extension_bit_exact():
    """The normal dashpot (dem_ext.restitution, an extension: the
    reference's contacts are springs only) runs in the generic Simulation
    kernels; a packed bed with restitution 0.5 equals the oracle's step with
    the same dashpot over 300 steps, and loses kinetic energy the undamped
    run keeps."""
    sc, p, ext = dem_scenes.dense_bed(n=1500, seed=12)
    g, o, _, _ = run_both(sc, p, 300, chunk=100, restitution=0.5)
    assert_same_state(g, o)
    u, _, _, _ = run_both(sc, p, 300, chunk=300)
    ke = lambda st: float((st["radii"].astype(np.float64) ** 2 * (st["vel"].reshape(-1, 2).astype(np.float64) ** 2).sum(1)).sum())
    assert ke(g) < ke(u)


@pytest.mark.parametrize("model", [1, 2, 3])
def test_bond_models_bit_exact(model):
    sc, p, ext = dem_scenes.c1_chains(chains=3, length=24, seed=5, pull_velocity=8.0)
    p = dict(p)
    p["bonds"] = model
    p["bond_normal_strength"] = 2e3 if model != 1 else 3e3
    ext = {"bond_lambda": 0.8}
    g, o, gev, oev = run_both(sc, p, 400, chunk=80, **ext)
    assert_same_state(g, o)
    assert len(gev) == len(oev)


def test_bond_model_changes_between_calls_bit_exact():
    """The Simulation kernels are compiled per bond model; a context whose
    model changes between calls (parallel -> none -> linear -> parallel)
    changes kernels and recaptures its graphs, and still gives the oracle's
    results under the same parameter sequence."""
    sc, p, _ = dem_scenes.c1_chains(chains=3, length=24, seed=5, pull_velocity=8.0)
    p = dict(p)
    p["bond_normal_strength"] = 2e3
    o = copy_scene(sc)
    done = 0
    oev = []
    with dem.Context(sc, dict(p, bonds=3), bond_lambda=0.8, reorder_interval=35) as ctx:
        for model, k in ((3, 70), (0, 70), (1, 105), (3, 70)):
            q = dict(p, bonds=model)
            ctx.set_params(q)
            ctx.step(k)
            ev, _ = oracle.step(o, q, k, step_base=done, bond_lambda=0.8)
            oev.append(ev)
            done += k
        g = ctx.download()
        gev = ctx.break_events()
    assert_same_state(g, o)
    assert len(gev) == len(np.concatenate(oev))


@pytest.mark.parametrize("variant", ["planet", "round_walls", "interval3", "f64", "fixity_mix"])
def test_setting_variants_bit_exact(variant):
    sc, p, ext = dem_scenes.c0_settle(n=500, seed=7, box=(50, 60), spacing=2.3)
    p = dict(p)
    kw = {}
    if variant == "planet":
        p["planet_mode"] = 1
    elif variant == "round_walls":
        p["round_bounds"] = 1
        p["bound_radius"] = 26.0
    elif variant == "interval3":
        p["collision_interval"] = 3
    elif variant == "f64":
        kw["use_f64"] = True
    elif variant == "fixity_mix":
        fx = sc["fixity"].reshape(-1, 6)
        fx[::7, 0] = 1
        fx[::11, 1] = 1
        fx[::5, 2] = 2
        sc["vel"].reshape(-1, 2)[::7, 0] = 3.0
        sc["forces"].reshape(-1, 6)[::13, :3] = [50.0, -20.0, 1.0]
    g, o, _, _ = run_both(sc, p, 200, chunk=40, **kw)
    assert_same_state(g, o, variant + ": ")


def test_strings_scene_bit_exact(golden_dir):
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "Strings.bin"))
    g, o, gev, oev = run_both(scene, uni, 300, chunk=60, use_f64=info["use_f64"])
    assert_same_state(g, o)
    assert len(gev) == len(oev)


def test_nan_velocity_and_broken_bonds_scene_bit_exact(golden_dir):
    """The reference's MicroStrings state: 2048 particles in strings, 4193
    bonds already broken (code -9) and one NaN velocity; NaN compares equal
    to NaN, every other bit must match."""
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "MicroStrings.bin"))
    assert np.isnan(scene["vel"]).any()
    g, o, gev, oev = run_both(scene, uni, 200, chunk=50, use_f64=info["use_f64"])
    assert_same_state(g, o)
    assert len(gev) == len(oev)


def test_out_of_grid_and_nan_particles_bit_exact():
    """Particles beyond the reference bucket grid find no partners (the
    reference's clamped bucket loops are empty for them; circular bounds of
    radius 1e6 keep them out there, since the rectangle walls always act,
    2D_LOM.wgsl:101-145), and a NaN velocity turns its particle's position
    NaN; GPU and oracle agree."""
    sc, p, ext = dem_scenes.dense_bed(900, seed=5)
    p = dict(p)
    p["round_bounds"] = 1
    p["bound_radius"] = 1.0e6
    sc = copy_scene(sc)
    pos = sc["pos"].reshape(-1, 2)
    far = np.argsort(pos[:, 0])[-40:]          # the 40 right-most particles, still touching
    pos[far, 0] += np.float32(2 * p["hor_bound"])   # one another, moved beyond the grid
    sc["vel"].reshape(-1, 2)[450, 0] = np.float32("nan")
    g, o, _, _ = run_both(sc, p, 120, chunk=40, reorder_interval=7)
    assert np.isnan(g["pos"]).any()
    assert not contact_pairs(o) & {(int(a), int(b)) for a in far for b in far}
    assert_same_state(g, o)


def _append_particles(sc, pos, radii, vel):
    """The scene with particles appended (no contacts, no fixity, material 0)."""
    m = radii.shape[0]
    out = copy_scene(sc)
    add = {"pos": pos.astype(np.float32).reshape(-1), "radii": radii.astype(np.float32),
           "vel": vel.astype(np.float32).reshape(-1), "acc": np.zeros(2 * m, np.float32),
           "rot": np.zeros(m, np.float32), "rot_vel": np.zeros(m, np.float32), "rot_acc": np.zeros(m, np.float32),
           "forces": np.zeros(6 * m, np.float32), "fixity": np.zeros(6 * m, np.int32),
           "del_pos": np.zeros(2 * m, np.float32), "del_rot": np.zeros(m, np.float32),
           "contacts": np.full(6 * 14 * m, -1, np.int32), "material_pointers": np.zeros(m, np.int32),
           "data": np.zeros(7 * m, np.float32)}
    for k, v in add.items():
        out[k] = np.concatenate([sc[k], v])
    return out


def test_crowded_cells_sort_in_linear_time():
    """The cell order is a stable counting sort whose cost does not depend on
    how many particles share a cell.  A packed bed plus 50,000 zero-radius
    particles (one dead cell) and 50,000 particles thrown out of the search
    grid at 1,000 units a step, so that every rebuild (one per step: they
    move beyond the skin) clamps them all into the grid's corner cell: the
    run takes well under a second of GPU time for 40 steps and equals the
    oracle bit for bit (the thrown particles are beyond the reference's
    bucket grid, so they find no partners in either)."""
    import time
    sc, p, ext = dem_scenes.dense_bed(2000, seed=5)
    p = dict(p)
    p["round_bounds"] = 1
    p["bound_radius"] = 1.0e6
    rng = np.random.default_rng(11)
    nz = 50000
    zpos = rng.uniform(-40.0, 40.0, size=(nz, 2))
    side = 224
    gx, gy = np.meshgrid(np.arange(side), np.arange(side))
    x0 = sc["pos"].reshape(-1, 2).max(axis=0) + 10.0
    tpos = np.stack([x0[0] + 4.0 * gx.ravel(), x0[1] + 4.0 * gy.ravel()], axis=1)
    nt = tpos.shape[0]
    tvel = np.full((nt, 2), 1.0e7)
    sc = _append_particles(sc, zpos, np.zeros(nz), np.zeros((nz, 2)))
    sc = _append_particles(sc, tpos, np.full(nt, 1.0), tvel)
    n = sc["radii"].shape[0]
    o = copy_scene(sc)
    with dem.Context(sc, p) as ctx:
        _, _, _, gw, gh = ctx.search_grid()
        ctx.step(1)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.step(40)
        ctx.synchronize()
        dt = time.perf_counter() - t0
        keys, order, cs = ctx.broad_phase()
        g = ctx.download()
        stats = ctx.stats()
    oracle.step(o, p, 41)
    assert stats["reorders"] >= 40
    assert np.count_nonzero(keys == gw * gh - 1) == nt, "the thrown particles share the corner cell"
    assert np.count_nonzero(keys == gw * gh) == nz
    assert np.array_equal(order, np.lexsort((np.arange(n), keys)))
    assert dt < 2.0, "40 steps with 40 rebuilds took %.2f s" % dt
    assert_same_state(g, o)


def test_large_scene_layout_on_host_threads_bit_exact():
    """Above 2^18 particles the layout is derived on host threads (the median
    radius from a histogram of the radii's float bits, then a selection in
    one bucket): the large particles are those of the serial rule (4x the
    median of the nonzero radii, at most max(64, n/256) of them), and the
    run equals the oracle."""
    sc, p, ext = dem_scenes.c2_impact(cols=512, rows=600, seed=3, projectile_radius=12.0,
                                      projectile_speed=80.0, projectiles=3)
    n = len(sc["radii"])
    assert n >= 1 << 18
    r = sc["radii"]
    nz = r[r > 0]
    med = np.partition(nz, nz.size // 2)[nz.size // 2]
    big = set(np.nonzero(r > 4 * med)[0].tolist())
    assert 0 < len(big) <= max(64, n // 256)
    with dem.Context(sc, p, **ext) as ctx:
        keys, order, cell_start = ctx.broad_phase()
    last = set(np.nonzero(keys == keys.max())[0].tolist())
    assert last == big | set(np.nonzero(r == 0)[0].tolist())
    g, o, _, _ = run_both(sc, p, 12, **ext)
    assert_same_state(g, o)


@pytest.mark.parametrize("split", [0, 1])
def test_list_overflow_cell_search_bit_exact(split):
    """A skin of 2 r_max puts more than 15 candidates on most particles of a
    packed bed: they search the rebuild's cell table every step instead of a
    candidate list (both Simulation-kernel forms), with the oracle's results."""
    sc, p, ext = dem_scenes.dense_bed(n=1500, seed=9)
    g, o, _, _ = run_both(sc, p, 120, chunk=40, list_skin=2.0, split_narrow=split, reorder_interval=7)
    with dem.Context(sc, p, list_skin=2.0, split_narrow=split) as ctx:
        ctx.step(10)
        assert ctx.stats()["list_overflows"] > 0
    assert_same_state(g, o)


def test_broad_phase_keys_and_order():
    sc, p, ext = dem_scenes.c0_settle(n=3000, seed=2, box=(80, 120), spacing=2.3)
    with dem.Context(sc, p) as ctx:
        ctx.step(25)
        st = ctx.download()
        keys, order, cs = ctx.broad_phase()
        x0, y0, inv, gw, gh = ctx.search_grid()
    pos = st["pos"].reshape(-1, 2)
    f = np.float32
    qx = np.floor((pos[:, 0] - f(x0)) * f(inv)).astype(np.int64)
    qy = np.floor((pos[:, 1] - f(y0)) * f(inv)).astype(np.int64)
    ref_keys = np.clip(qy, 0, gh - 1) * gw + np.clip(qx, 0, gw - 1)
    ref_keys[st["radii"] == 0] = gw * gh
    assert np.array_equal(keys, ref_keys)
    ref_order = np.lexsort((np.arange(len(keys)), ref_keys))
    assert np.array_equal(order, ref_order)
    counts = np.bincount(ref_keys, minlength=gw * gh + 1)
    assert np.array_equal(cs, np.concatenate([[0], np.cumsum(counts)]))


def test_upload_download_roundtrip(golden_dir):
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, "Strings.bin"))
    with dem.Context(scene, uni, use_f64=info["use_f64"]) as ctx:
        d = ctx.download()
        for k in ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "fixity",
                  "del_pos", "del_rot", "bonds", "contacts", "material_pointers", "materials"):
            assert np.array_equal(d[k].view(np.int32), scene[k].view(np.int32)), k
        ctx.step(40)
        mid = ctx.download()
        ctx.upload(scene)
        back = ctx.download()
        assert np.array_equal(back["contacts"], scene["contacts"])
        assert not np.array_equal(mid["pos"], scene["pos"])


def test_set_properties_matches_oracle():
    sc, p, ext = dem_scenes.c0_settle(n=400, seed=4, box=(40, 60), spacing=2.3)
    o = copy_scene(sc)
    sel = np.zeros(400, np.int32)
    sel[10:30] = 1
    words = np.zeros(28, np.int32)
    words[[0, 3, 10, 6]] = 1
    f = words.view(np.float32)
    f[14] = 3.5
    f[17] = -1.25
    f[20] = 40.0
    words[24] = 1
    with dem.Context(sc, p) as ctx:
        ctx.step(10)
        oracle.step(o, p, 10)
        gsel = ctx.set_properties(sel, words)
        osel = oracle.set_properties(o, sel.copy(), words)
        assert np.array_equal(gsel, osel)
        ctx.step(30)
        oracle.step(o, p, 30, step_base=10)
        g = ctx.download()
    assert_same_state(g, o)
    assert np.array_equal(g["fixity"], o["fixity"]) and np.array_equal(g["forces"], o["forces"])


def test_fp64_twin_error_is_reported():
    """Per-particle FP32 accelerations of one step against the FP64 twin of the
    same step, scaled by the particle's force magnitude (sum |F_n| + m g).
    Against the reference's own FP32 arithmetic the path is exact (every
    other parity test); against FP64 it carries FP32's rounding.  Bounds, on
    a packed bed in contact: median 1e-5 (the workload definition's
    tolerance), 99th percentile 1e-3 and maximum 1e-2 -- FP32 positions of
    magnitude ~30 carry ~2e-6 absolute rounding, so the overlap of a
    near-grazing contact (~1e-3) is only known to ~1e-3 relative."""
    sc, p, ext = dem_scenes.dense_bed(n=1500, seed=9)
    with dem.Context(sc, p) as ctx:
        ctx.step(30)
        s30 = ctx.download()
        ctx.step(1)
        s31 = ctx.download()
    twin = oracle.step_f64(s30, p, 1)
    r = s30["radii"].astype(np.float64)
    mass = np.pi * r * r
    a32 = s31["acc"].reshape(-1, 2).astype(np.float64)
    a64 = twin["acc"].reshape(-1, 2)
    f_abs = np.abs(s31["data"].reshape(-1, 7)[:, 0]).astype(np.float64)
    scale = (f_abs + mass * 9.81) / mass
    err = np.linalg.norm(a32 - a64, axis=1) / scale
    print("fp32 vs fp64 one-step acceleration error: max %.3g p99 %.3g median %.3g"
          % (err.max(), np.percentile(err, 99), np.median(err)))
    assert np.median(err) < 1e-5
    assert np.percentile(err, 99) < 1e-3
    assert err.max() < 1e-2


def test_zero_radius_and_empty_slots_edge_cases():
    sc, p, ext = dem_scenes.c0_settle(n=300, seed=6, box=(40, 50), spacing=2.3)
    sc["radii"][::17] = 0.0
    g, o, _, _ = run_both(sc, p, 120, chunk=30)
    assert_same_state(g, o)


def test_checkpoint_through_a_saved_state_resumes_bit_exact():
    """State::save -> file -> State::load -> restore (state_io + dem_upload)
    in the middle of a run: the resumed run equals the uninterrupted one."""
    import state_io
    sc, p, ext = dem_scenes.dense_bed(n=1200, seed=31)
    with dem.Context(sc, p) as a:
        a.step(100)
        buf = state_io.save_state(a.download(), p)
        a.step(100)
        ref = a.download()
    sc2, uni, info = state_io.load_state(buf)
    assert uni["dT"] == float(np.float32(p["dT"])) and uni["collision_interval"] == 1
    with dem.Context(sc2, p) as b:
        b.step(100)
        got = b.download()
    assert_same_state(got, ref, "resumed: ")
