"""Reader for the reference's FlatBuffers saved states (test infrastructure).

Wire format of `table State` in new_schema.fbs:86-104 (root_type State) with the
field ids pinned by new_schema_generated.rs:2500-2515 (VT_POS=4 .. VT_SETTINGS=34)
and the inline `struct Settings` of 212 bytes (new_schema_generated.rs:2364-2480):
view 0..76, setup 76..116, sim 116..156, physics 156..212, field offsets as in
Setup_Settings (new_schema_generated.rs:1088-1349), Simulation_Settings
(:1471-1761) and Physics_Settings (:1898-2333).

`load_state(path)` mirrors State::load (src/state.rs:583-706): vectors are
taken whole, p_count comes from the setup settings, min/max radius are taken
over the whole radii vector, and the grid comes from grid_capacity
(src/wgpu_prog.rs:698-717).  Settings that the file does not persist take the
defaults of Settings::new (src/settings.rs:257-439).
"""
import struct

import numpy as np

STATE_FIELDS = ["pos", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "radii", "fixity",
                "bonds", "contacts", "material_pointers", "materials", "groups", "scripts",
                "settings"]
INT_VECTORS = {"fixity", "bonds", "material_pointers", "groups"}
# contacts are a [float] vector whose int fields hold i32 bit patterns: read as raw words


def parse(buf):
    """Return a dict of the State table's fields (numpy arrays, str, raw settings bytes)."""
    b = bytes(buf)
    if len(b) < 8:
        raise ValueError("buffer too small for a FlatBuffer")
    root = struct.unpack_from("<I", b, 0)[0]
    if root + 4 > len(b):
        raise ValueError("root offset out of range")
    vt = root - struct.unpack_from("<i", b, root)[0]
    if vt < 0 or vt + 4 > len(b):
        raise ValueError("vtable offset out of range")
    vtlen, _objlen = struct.unpack_from("<HH", b, vt)
    nf = (vtlen - 4) // 2
    out = {}
    for i, name in enumerate(STATE_FIELDS):
        off = struct.unpack_from("<H", b, vt + 4 + 2 * i)[0] if i < nf else 0
        if off == 0:
            out[name] = None
            continue
        fo = root + off
        if name == "settings":
            if fo + 212 > len(b):
                raise ValueError("settings struct out of range")
            out[name] = b[fo:fo + 212]
            continue
        vo = fo + struct.unpack_from("<I", b, fo)[0]
        if vo + 4 > len(b):
            raise ValueError("vector offset out of range")
        ln = struct.unpack_from("<I", b, vo)[0]
        if name == "scripts":
            if vo + 4 + ln > len(b):
                raise ValueError("string out of range")
            out[name] = b[vo + 4:vo + 4 + ln].decode("utf-8")
            continue
        if vo + 4 + 4 * ln > len(b):
            raise ValueError("vector %s out of range" % name)
        dt = "<i4" if (name in INT_VECTORS or name == "contacts") else "<f4"
        out[name] = np.frombuffer(b, dtype=dt, count=ln, offset=vo + 4).copy()
    return out


def _f(b, o):
    return struct.unpack_from("<f", b, o)[0]


def _i(b, o):
    return struct.unpack_from("<i", b, o)[0]


def decode_settings(raw):
    """The persisted Settings struct -> dict of setup/sim/physics values."""
    su, sm, ph = raw[76:116], raw[116:156], raw[156:212]
    return {
        "particles": _i(su, 0), "max_radius": _f(su, 4), "variable_rad": bool(su[8]),
        "timestep": _f(sm, 0), "gen_per_frame": _i(sm, 4), "width": _f(sm, 12),
        "height": _f(sm, 16), "round_walls": bool(sm[21]), "wall_radius": _f(sm, 24),
        "x_timesteps": _i(sm, 32), "use_f64": bool(sm[36]),
        "gravity": bool(ph[0]), "g_force": _f(ph, 4), "planet_mode": bool(ph[8]),
        "mouse_gravity": bool(ph[9]), "collisions": bool(ph[10]),
        "collision_interval": _i(ph, 12), "friction_coef": _f(ph, 16), "bond": _i(ph, 20),
        "bond_tearing": bool(ph[24]), "bond_normal_stiffness": _f(ph, 28),
        "bond_shear_stiffness": _f(ph, 32), "bond_normal_strength": _f(ph, 36),
        "bond_shear_strength": _f(ph, 40), "moment_contribution_factor": _f(ph, 44),
        "local_damping": bool(ph[48]), "local_damping_alpha": _f(ph, 52),
    }


def uniform_from(st, particles):
    """collision_settings() (settings.rs:2086-2119) for a loaded file; non-persisted
    fields keep their Settings::new defaults (walls on, wall_friction 0,
    contact_damping 0.2, bond_damping 0.2, drag 1, mouse position 0)."""
    return {
        "walls": 1, "hor_bound": st["width"], "vert_bound": st["height"],
        "round_bounds": int(st["round_walls"]), "bound_radius": st["wall_radius"],
        "wall_friction": 0.0, "gravity": int(st["gravity"]), "planet_mode": int(st["planet_mode"]),
        "bonds": st["bond"], "collisions": int(st["collisions"]),
        "friction_coefficient": st["friction_coef"], "gravity_acc": st["g_force"],
        "bond_normal_stiffness": st["bond_normal_stiffness"], "bonds_tear": int(st["bond_tearing"]),
        "bond_normal_strength": st["bond_normal_strength"], "contact_damping": 0.2,
        "bond_damping": 0.2, "drag": 1.0, "bond_shear_strength": st["bond_shear_strength"],
        "dT": st["timestep"], "bond_shear_stiffness": st["bond_shear_stiffness"],
        "gravity_x": 0.0, "gravity_y": 0.0, "mouse_gravity": int(st["mouse_gravity"]),
        "moment_contribution_factor": st["moment_contribution_factor"],
        "collision_interval": st["collision_interval"], "local_damping": int(st["local_damping"]),
        "local_damping_alpha": st["local_damping_alpha"], "particles": int(particles),
    }


def grid_capacity(hor_bound, vert_bound, max_radius, min_radius, variable_rad, particles):
    """wgpu_prog.rs:698-717 in float32 arithmetic; Rust `as i32` saturates."""
    f = np.float32
    width = f(hor_bound) * f(2.0)
    height = f(vert_bound) * f(2.0)
    max_rad = f(max_radius) * f(2.0)
    min_rad = f(min_radius) if variable_rad else f(max_radius)

    def as_i32(x):
        x = float(x)
        if x != x:
            return 0
        return int(max(min(x, 2147483647.0), -2147483648.0))

    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        w = as_i32(np.ceil(width / max_rad))
        h = as_i32(np.ceil(height / max_rad))
        q = max_rad / min_rad + f(1.0)
        cap = as_i32(np.ceil(q * q))
    cap = min(cap, int(particles)) + 2
    return (float(max_rad), cap, w, h)


def load_state(path_or_bytes):
    """State::load (state.rs:583-706) -> (scene dict trimmed to p_count, uniform, info)."""
    buf = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    f = parse(buf)
    st = decode_settings(f["settings"])
    n = st["particles"]
    radii_all = f["radii"]
    rmin = float(radii_all.min()) if radii_all.size else 0.0
    rmax = float(radii_all.max()) if radii_all.size else 0.0
    grid = grid_capacity(st["width"], st["height"], rmax, rmin, rmin != rmax, n)

    def take(name, per, dtype):
        a = f[name]
        return np.ascontiguousarray(a[: per * n], dtype=dtype)

    scene = {
        "pos": take("pos", 2, np.float32), "radii": take("radii", 1, np.float32),
        "vel": take("vel", 2, np.float32), "acc": take("acc", 2, np.float32),
        "rot": take("rot", 1, np.float32), "rot_vel": take("rot_vel", 1, np.float32),
        "rot_acc": take("rot_acc", 1, np.float32), "forces": take("forces", 6, np.float32),
        "fixity": take("fixity", 6, np.int32),
        "contacts": take("contacts", 84, np.int32),
        "material_pointers": take("material_pointers", 1, np.int32),
        "materials": np.ascontiguousarray(f["materials"], dtype=np.float32),
        "bonds": np.ascontiguousarray(f["bonds"], dtype=np.int32),
        "data": np.zeros(7 * n, dtype=np.float32),
        "coll_cont": np.zeros(4, dtype=np.int32),
        "grid": grid,
    }
    # State::restore uploads vel into the del_pos binding and rot_vel into the
    # del_rot binding (wgpu_prog.rs:1247-1248)
    scene["del_pos"] = scene["vel"].copy()
    scene["del_rot"] = scene["rot_vel"].copy()
    info = dict(st)
    info["groups"] = f["groups"]
    info["scripts"] = f["scripts"]
    return scene, uniform_from(st, n), info
