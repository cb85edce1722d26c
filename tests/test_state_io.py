"""FlatBuffers saved states (state_io): reading both schemas, writing the new
one the way State::save does (src/state.rs:369-493), and the round trip."""
import glob
import os
import struct

import numpy as np
import pytest

import dem_scenes
import state_io

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _same_scene(a, b):
    """Every array bit for bit (a saved NaN must come back as the same NaN)."""
    for k in a:
        if k == "grid":
            assert a[k] == b[k]
        else:
            x, y = np.asarray(a[k]), np.asarray(b[k])
            assert x.dtype == y.dtype and x.shape == y.shape and x.tobytes() == y.tobytes(), k


# the experiment states (Default.bin is in neither schema: its own test below)
EXPERIMENT_STATES = sorted(p for p in glob.glob(os.path.join(GOLDEN, "*.bin")) if not p.endswith("Default.bin"))


@pytest.mark.parametrize("path", EXPERIMENT_STATES, ids=os.path.basename)
def test_golden_states_round_trip_through_the_writer(path):
    sc, uni, info = state_io.load_state(path)
    out = state_io.save_state(sc, uni, info)
    sc2, uni2, info2 = state_io.load_state(out)
    _same_scene(sc, sc2)
    assert uni == uni2
    # every settings byte, padding included, as the reference wrote it
    assert info2["settings_raw"] == info["settings_raw"]
    assert info2["scripts"] == info["scripts"]
    assert np.array_equal(info2["groups"], info["groups"])
    assert len(out) % 4 == 0


def test_layouts_follow_the_flatbuffers_struct_rules():
    names = {n: o for n, _, o in state_io.SETTINGS_NEW}
    assert names["particles"] == 76 and names["timestep"] == 116 and names["gravity"] == 156
    assert names["use_f64"] == 116 + 36 and names["bond_tearing"] == 156 + 24
    old = {n: o for n, _, o in state_io.SETTINGS_OLD}
    assert old["gravity"] == 152 and old["bond_normal_stiffness"] == 152 + 24
    assert "use_f64" not in old and "bond_tearing" not in old


def _write_old(scene, settings_values):
    """A State of schema.fbs (14 vectors, then the 204-byte settings; no
    scripts), written with the same front-to-back layout."""
    raw = bytearray(state_io.SETTINGS_OLD_SIZE)
    for name, kind, off in state_io.SETTINGS_OLD:
        v = settings_values.get(name, 0)
        if kind == "b":
            raw[off] = 1 if v else 0
        elif kind == "i":
            struct.pack_into("<i", raw, off, int(v))
        else:
            struct.pack_into("<f", raw, off, float(v))
    nf = 15
    vt_pos, vt_size = 4, 4 + 2 * nf
    table_pos = (vt_pos + vt_size + 3) // 4 * 4
    b = state_io._Builder()
    b.buf += struct.pack("<I", table_pos)
    b.buf += struct.pack("<%dH" % (nf + 2), vt_size, 4 + 4 * 14 + len(raw), *[4 + 4 * i for i in range(nf)])
    b.align()
    b.buf += struct.pack("<i", table_pos - vt_pos) + b"\0" * (4 * 14) + bytes(raw)
    keys = ["pos", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "radii", "fixity", "bonds", "contacts",
            "material_pointers", "materials"]
    targets = [b.vector(np.asarray(scene[k])) for k in keys] + [b.vector(np.zeros(3, np.int32))]
    for i, t in enumerate(targets):
        fo = table_pos + 4 + 4 * i
        struct.pack_into("<I", b.buf, fo, t - fo)
    return bytes(b.buf)


def test_old_schema_state_is_read():
    sc, p, ext = dem_scenes.c1_chains(chains=2, length=10)
    vals = {"particles": 20, "max_radius": 1.0, "timestep": 1e-4, "gen_per_frame": 105, "width": 60.0,
            "height": 30.0, "x_timesteps": 7, "gravity": True, "g_force": 1.0, "collisions": True,
            "collision_interval": 1, "friction_coef": 0.5, "bond": 3, "bond_normal_stiffness": 1e5,
            "bond_shear_stiffness": 5e4, "bond_normal_strength": 5e3, "bond_shear_strength": 5e3,
            "moment_contribution_factor": 1.0, "local_damping_alpha": 0.1}
    buf = _write_old(sc, vals)
    sc2, uni, info = state_io.load_state(buf)
    assert info["schema"] == "old" and info["scripts"] == ""
    assert info["use_f64"] is False and info["bond_tearing"] is False
    assert info["x_timesteps"] == 7 and uni["bonds"] == 3 and uni["bonds_tear"] == 0
    for k in ("pos", "radii", "fixity", "bonds", "contacts", "materials"):
        assert np.array_equal(sc2[k], sc[k]), k
    assert np.array_equal(sc2["del_pos"], sc2["vel"])


def test_fresh_scene_saves_and_loads():
    sc, p, ext = dem_scenes.c0_settle(n=400, seed=3)
    buf = state_io.save_state(sc, p, use_f64=True)
    sc2, uni, info = state_io.load_state(buf)
    assert info["particles"] == 400 and info["use_f64"] is True
    for k in ("pos", "radii", "vel", "fixity", "contacts", "material_pointers", "materials"):
        assert np.array_equal(sc2[k], np.asarray(sc[k])), k
    for k in ("dT", "hor_bound", "vert_bound", "friction_coefficient", "gravity_acc"):
        assert uni[k] == float(np.float32(p[k])), k
    for k in ("gravity", "planet_mode", "collisions", "collision_interval", "bonds"):
        assert uni[k] == p[k], k


def test_truncated_buffers_raise():
    sc, uni, info = state_io.load_state(os.path.join(GOLDEN, "TEXPS.bin"))
    buf = state_io.save_state(sc, uni, info)
    for cut in (3, 40, len(buf) // 2):
        with pytest.raises(ValueError):
            state_io.load_state(buf[:cut])


def test_random_scenes_round_trip_bit_for_bit():
    """Any scene, its floats random bit patterns (NaNs and infinities
    included), any particle, bond and material counts: save then load gives
    back every saved array byte for byte; del_pos and del_rot come back as
    the reference's restore uploads them, copies of vel and rot_vel, and the
    diagnostics, which State does not save, as zeros."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies
    _, p, _ = dem_scenes.c0_settle(n=16, seed=0)
    widths = {"pos": 2, "radii": 1, "vel": 2, "acc": 2, "rot": 1, "rot_vel": 1, "rot_acc": 1, "forces": 6,
              "fixity": 6, "del_pos": 2, "del_rot": 1, "contacts": 84, "data": 7}
    ints = ("fixity", "contacts")

    @hyp.settings(max_examples=60, deadline=None, derandomize=True)
    @hyp.given(n=st.integers(1, 64), nb=st.integers(0, 40), nm=st.integers(1, 5), seed=st.integers(0, 2**31 - 1))
    def check(n, nb, nm, seed):
        rng = np.random.default_rng(seed)

        def bits(size):
            return rng.integers(0, 2**32, size=size, dtype=np.uint64).astype(np.uint32)

        sc = {k: (bits(w * n).view(np.int32) if k in ints else bits(w * n).view(np.float32)) for k, w in widths.items()}
        sc["materials"] = bits(6 * nm).view(np.float32)
        sc["material_pointers"] = rng.integers(0, nm, size=n, dtype=np.int64).astype(np.int32)
        sc["bonds"] = bits(3 * nb).view(np.int32) if nb else np.array([-1], dtype=np.int32)
        sc["coll_cont"] = bits(4).view(np.int32)
        sc["grid"] = {"cell_size": 2.5, "cell_cap": 8, "w": 4, "h": 4}
        sc2, _, _ = state_io.load_state(state_io.save_state(sc, dict(p, particles=n)))
        expect = dict(sc, del_pos=sc["vel"], del_rot=sc["rot_vel"], data=np.zeros(7 * n, np.float32))
        for k in expect:
            if k in ("grid", "coll_cont"):
                continue
            x, y = np.asarray(expect[k]), np.asarray(sc2[k])
            assert x.dtype == y.dtype and x.shape == y.shape and x.tobytes() == y.tobytes(), k

    check()


def _root_vectors(buf):
    """Field count of a FlatBuffers root table and, per field, the length
    word of the vector it points to (None for an absent field)."""
    import struct
    root = struct.unpack_from("<I", buf, 0)[0]
    vt = root - struct.unpack_from("<i", buf, root)[0]
    vlen = struct.unpack_from("<H", buf, vt)[0]
    out = []
    for k in range((vlen - 4) // 2):
        o = struct.unpack_from("<H", buf, vt + 4 + 2 * k)[0]
        if o == 0:
            out.append(None)
            continue
        tgt = root + o + struct.unpack_from("<I", buf, root + o)[0]
        out.append(struct.unpack_from("<I", buf, tgt)[0] if tgt + 4 <= len(buf) else None)
    return out


def test_default_bin_is_in_neither_schema_and_is_refused(golden_dir):
    """The Default.bin at the root of the reference checkout is not the scene
    the reference starts with: its code reads saved states only from files
    the user or a script picks (State::load_from_file from client.rs:917 and
    1151).  It follows neither schema in the reference: a 256-particle state
    whose root table holds 15 fields in an order of neither State table, with
    a contact vector of 14,336 words -- 4 words a record, where both schemas
    store 6 (contacts = 14 records x 6 words a particle).  The reader refuses
    it instead of misreading it."""
    buf = open(os.path.join(golden_dir, "Default.bin"), "rb").read()
    lens = _root_vectors(buf)
    assert len(lens) == 15
    assert 14336 in lens and 256 * 14 * 4 == 14336 and 256 * 14 * 6 not in lens
    with pytest.raises(ValueError):
        state_io.load_state(os.path.join(golden_dir, "Default.bin"))
    for name in ("TEXPS.bin", "Strings.bin"):   # the experiment states: 6 words a record
        s, _, _ = state_io.load_state(os.path.join(golden_dir, name))
        assert s["contacts"].size == 14 * 6 * s["radii"].size
