"""Shared helpers for the GPU parity tests (test infrastructure)."""
import numpy as np

import dem
import oracle

FLOAT_KEYS = ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "del_pos", "del_rot", "data")


class GpuBackend:
    """Replayer backend over the CUDA library (dem.Context)."""

    def __init__(self, scene, settings, use_f64, **ext):
        self.ctx = dem.Context(scene, settings, use_f64=use_f64, **ext)
        self.dt = np.float32(settings["dT"])

    def download(self):
        return self.ctx.download()

    def upload(self, scene):
        self.ctx.upload(scene)

    def set_properties(self, selections, words):
        return self.ctx.set_properties(selections, words)

    def step(self, n):
        self.ctx.step(n)


class RecordingGpuBackend(GpuBackend):
    """The same backend with the device record path (dem_record) for
    Advance with Record on, instead of a state readback per step."""

    def record(self, ticks, selections):
        return self.ctx.record(ticks, selections)


def copy_scene(sc):
    return {k: (v.copy() if hasattr(v, "copy") else v) for k, v in sc.items()}


def assert_same_state(got, ref, what=""):
    """Bit-for-bit equality of every state array (floats compared by value, so
    that +0 and -0 are equal; NaN equals NaN)."""
    for k in FLOAT_KEYS:
        a, b = got[k], ref[k]
        if not np.array_equal(a, b, equal_nan=True):
            d = np.nonzero(~((a == b) | (np.isnan(a) & np.isnan(b))))[0]
            raise AssertionError("%s%s differs at %d entries, first %s: gpu %r oracle %r" % (
                what, k, d.size, d[:5], a[d[:5]], b[d[:5]]))
    # contacts: ints bitwise, the three float fields by value
    ca = got["contacts"].reshape(-1, 6)
    cb = ref["contacts"].reshape(-1, 6)
    for f in (0, 1, 5):
        if not np.array_equal(ca[:, f], cb[:, f]):
            d = np.nonzero(ca[:, f] != cb[:, f])[0]
            raise AssertionError("%scontacts field %d differs at %d slots, first %s: gpu %r oracle %r" % (
                what, f, d.size, d[:5], ca[d[:5]], cb[d[:5]]))
    fa = ca[:, 2:5].copy().view(np.float32)
    fb = cb[:, 2:5].copy().view(np.float32)
    if not np.array_equal(fa, fb, equal_nan=True):
        d = np.nonzero(~((fa == fb) | (np.isnan(fa) & np.isnan(fb))).all(axis=1))[0]
        raise AssertionError("%scontact forces differ at %d slots, first %s: gpu %r oracle %r" % (
            what, d.size, d[:5], fa[d[:5]], fb[d[:5]]))
    assert np.array_equal(got["bonds"], ref["bonds"]), what + "bond records differ"


def contact_pairs(sc):
    c = sc["contacts"].reshape(-1, 6)
    occ = c[:, 1] != -1
    return set(zip(c[occ, 0].tolist(), c[occ, 1].tolist()))


def run_both(scene, params, steps, chunk=None, **ext):
    """Advance the same scene on the GPU and on the oracle; return both states
    and both break-event lists (oracle events as dem.BREAK_DTYPE-like tuples)."""
    o = copy_scene(scene)
    okw = {k: ext[k] for k in ("use_f64", "restitution") if k in ext}
    if "bond_lambda" in ext:
        okw["bond_lambda"] = ext["bond_lambda"]
    if "bond_sn" in ext:
        okw["bond_sn"] = ext["bond_sn"]
        okw["bond_ss"] = ext["bond_ss"]
    ctx = dem.Context(scene, params, **ext)
    chunk = chunk or steps
    done = 0
    oev = []
    while done < steps:
        k = min(chunk, steps - done)
        ctx.step(k)
        ev, _ = oracle.step(o, params, k, step_base=done, **okw)
        oev.append(ev)
        done += k
    g = ctx.download()
    gev = ctx.break_events()
    ctx.close()
    oev = np.concatenate(oev) if oev else np.zeros(0, oracle.BREAK_DTYPE)
    return g, o, gev, oev
