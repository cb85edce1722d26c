"""The oracle's results do not depend on how it is run: one host thread or
many, all steps in one call or split over several, give byte-identical
states and break-event lists, and its FP32 step agrees with its FP64 twin to
rounding; and, as physics, it conserves linear momentum where nothing
external acts.  It is the checker of every parity test."""
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


@pytest.mark.parametrize("workload", ["settle", "chains"])
def test_fp32_step_agrees_with_the_fp64_twin(workload):
    """The oracle's FP32 step and its separately written FP64 twin agree to
    rounding over one step from a state with contacts and bonds: a
    transcription error in either would show far above these bounds
    (measured: positions 4e-8, velocities 5e-7, spins 7e-8 of the field's
    scale; accelerations, sums of nearly cancelling forces, 7e-4)."""
    if workload == "settle":
        sc, p, ext = dem_scenes.c0_settle(n=2000, seed=5, box=(50, 100), spacing=2.05)
        kw = {}
    else:
        sc, p, ext = dem_scenes.c1_chains(chains=6, length=48, seed=13, pull_velocity=30.0)
        kw = {"bond_lambda": ext["bond_lambda"], "bond_sn": ext["bond_sn"], "bond_ss": ext["bond_ss"]}
    base, _ = _run(sc, p, 50, 0, **kw)
    a, _ = _run(base, p, 1, 0, **kw)
    d = oracle.step_f64(copy_scene(base), p, 1, **kw)
    tol = {"pos": 1e-6, "vel": 1e-5, "rot_vel": 1e-5, "acc": 1e-2}
    for k, t in tol.items():
        x = np.asarray(a[k], np.float64)
        scale = max(np.abs(d[k]).max(), 1e-30)
        assert np.abs(x - d[k]).max() / scale <= t, k


@pytest.mark.parametrize("workload", ["contacts", "bonds"])
def test_linear_momentum_is_conserved(workload):
    """With gravity and local damping off, no particle fixed and the walls out
    of reach, contact and bond forces act in equal and opposite pairs, so
    total linear momentum (mass = density x pi r^2) stays constant to
    rounding over 200 steps, bond breaks included (measured: 2e-8 of the
    total |m v|)."""
    if workload == "contacts":
        sc, p, ext = dem_scenes.c0_settle(n=900, seed=7, box=(400, 400), spacing=1.9)
        kw, sd = {}, 5.0
    else:
        sc, p, ext = dem_scenes.c1_chains(chains=6, length=48, seed=13, pull_velocity=30.0)
        kw = {"bond_lambda": ext["bond_lambda"], "bond_sn": ext["bond_sn"], "bond_ss": ext["bond_ss"]}
        sd = 20.0
    p = dict(p, gravity=0, local_damping=0)
    o = copy_scene(sc)
    o["fixity"][:] = 0
    o["forces"][:] = 0
    rng = np.random.default_rng(3)
    o["vel"][:] = rng.normal(0.0, sd, size=o["vel"].size).astype(np.float32)
    mats = o["materials"].reshape(-1, 6)
    m = mats[o["material_pointers"], 3].astype(np.float64) * np.pi * o["radii"].astype(np.float64) ** 2

    def momentum():
        v = o["vel"].reshape(-1, 2).astype(np.float64)
        return (m[:, None] * v).sum(0), (m[:, None] * np.abs(v)).sum()

    p0, _ = momentum()
    breaks = 0
    for k in range(5):
        ev, _ = oracle.step(o, p, 40, step_base=40 * k, **kw)
        breaks += len(ev)
        pk, total = momentum()
        assert np.abs(pk - p0).max() <= 1e-6 * total, k
    if workload == "bonds":
        assert breaks > 0


def _head_on(restitution, steps=3000):
    """Two equal disks closing at speed 2 (no gravity, walls far away):
    the ratio of separating to closing speed after the contact."""
    sc = dem_scenes.empty_scene(2, [1, 1, 1, 1.0, 1e5, 5e4])
    sc["pos"][:] = [-1.1, 0.0, 1.1, 0.0]
    sc["radii"][:] = 1.0
    sc["vel"][:] = [1.0, 0.0, -1.0, 0.0]
    p = dem_scenes.reference_defaults(2)
    p.update({"hor_bound": 100.0, "vert_bound": 100.0, "gravity": 0, "planet_mode": 0, "dT": 1e-4,
              "friction_coefficient": 0.5, "bonds": 0})
    sc["grid"] = dem_scenes.grid_capacity(100.0, 100.0, sc["radii"], 2)
    oracle.step(sc, p, steps, restitution=restitution)
    v = sc["vel"].reshape(2, 2)
    return float((v[1, 0] - v[0, 0]) / 2.0)


def test_dashpot_extension_restitution():
    """The normal dashpot (an extension; the reference's contacts are pure
    springs): restitution 0 keeps the reference's elastic contact, and a
    head-on collision of two disks comes out with about the requested
    restitution (higher for strong damping, where the no-pull clamp cuts the
    dashpot's tension off)."""
    assert abs(_head_on(0.0) - 1.0) < 1e-4
    assert 0.5 <= _head_on(0.5) <= 0.6
    assert 0.79 <= _head_on(0.8) <= 0.83
    assert abs(_head_on(0.95) - 0.95) < 0.01


def test_dashpot_off_is_the_reference_arithmetic():
    """restitution 0 gives the default step byte for byte."""
    sc, p, ext = dem_scenes.dense_bed(n=400, seed=3)
    a, b = copy_scene(sc), copy_scene(sc)
    oracle.step(a, p, 60)
    oracle.step(b, p, 60, restitution=0.0)
    for k in ("pos", "vel", "acc", "data", "contacts"):
        assert np.array_equal(a[k].view(np.int32), b[k].view(np.int32)), k
