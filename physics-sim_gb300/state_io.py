"""Saved states: the reference's FlatBuffers `State` files, read and written.

The host-side counterpart of State::save (src/state.rs:369-493), State::load
(src/state.rs:583-706) and restore's upload (src/wgpu_prog.rs:1235-1262), for
scenes in the reference's host layouts (the dicts that `dem.Context` takes).

Wire format.  `table State` of new_schema.fbs has 16 fields (ids 0-15: pos,
vel, acc, rot, rot_vel, rot_acc, forces, radii, fixity, bonds, contacts,
material_pointers, materials, groups, scripts, settings); the older
schema.fbs has the first 14 of them followed by settings (id 14) and no
scripts.  `settings` is an inline struct of four structs laid out by the
FlatBuffers rules (each scalar aligned to its size, structs to 4 bytes):
212 bytes in the new schema (view 0-76, setup 76-116, simulation 116-156,
physics 156-212) and 204 in the old one, whose Simulation_Settings lacks
use_f64 and whose Physics_Settings lacks bond_tearing.  `contacts` is a
[float] vector whose integer fields are i32 bit patterns, so it is moved as
raw 32-bit words.

`save_state` writes the new schema: a root offset, the vtable, the table
(soffset, 15 offsets, the settings struct), then the vectors and the scripts
string, every object 4-byte aligned and every offset pointing forward, which
is what the FlatBuffers verifier of the reference's loader accepts.
"""
import struct

import numpy as np

FIELDS_NEW = ["pos", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "radii", "fixity", "bonds",
              "contacts", "material_pointers", "materials", "groups", "scripts", "settings"]
FIELDS_OLD = FIELDS_NEW[:14] + ["settings"]
INT_VECTORS = {"fixity", "bonds", "material_pointers", "groups", "contacts"}

# (name, kind) in declaration order; kinds: b = bool, i = int32, f = float32
VIEW = [("circular_particles", "b"), ("render_rot", "b"), ("render_bonds", "b"), ("render_outline", "b"),
        ("render_bp_grid", "b"), ("color_code_rot", "b"), ("use_particle_color_outline", "b"),
        ("outline_color_r", "f"), ("outline_color_g", "f"), ("outline_color_b", "f"),
        ("background_color_r", "f"), ("background_color_g", "f"), ("background_color_b", "f"),
        ("color_source", "i"), ("dim_slow_particles", "b"), ("max_brightness_vel", "f"), ("crt_res", "i"),
        ("grain", "b"), ("grain_strength", "f"), ("grain_size", "i"), ("sobel", "b"), ("colored_sobel", "b"),
        ("invert", "b"), ("chrom_ab", "b"), ("abb_strength", "f"), ("bond_highlight_strength", "f"),
        ("render_unbonded_contacts", "b"), ("lighting", "b"), ("show_hit_tex", "b")]
SETUP = [("particles", "i"), ("max_radius", "f"), ("variable_rad", "b"), ("holeyness", "f"),
         ("max_h_velocity", "f"), ("min_h_velocity", "f"), ("max_v_velocity", "f"), ("min_v_velocity", "f"),
         ("grid_width", "f"), ("hex_grid", "b")]
SIM_OLD = [("timestep", "f"), ("gen_per_frame", "i"), ("auto_width", "b"), ("width", "f"), ("height", "f"),
           ("maintain_ar", "b"), ("round_walls", "b"), ("wall_radius", "f"), ("d3", "b"), ("x_timesteps", "i")]
SIM_NEW = SIM_OLD + [("use_f64", "b")]
PHYS_NEW = [("gravity", "b"), ("g_force", "f"), ("planet_mode", "b"), ("mouse_gravity", "b"), ("collisions", "b"),
            ("collision_interval", "i"), ("friction_coef", "f"), ("bond", "i"), ("bond_tearing", "b"),
            ("bond_normal_stiffness", "f"), ("bond_shear_stiffness", "f"), ("bond_normal_strength", "f"),
            ("bond_shear_strength", "f"), ("moment_contribution_factor", "f"), ("local_damping", "b"),
            ("local_damping_alpha", "f")]
PHYS_OLD = [f for f in PHYS_NEW if f[0] != "bond_tearing"]


def _layout(fields):
    """FlatBuffers struct layout: [(name, kind, offset)], size (4-byte aligned)."""
    out, off = [], 0
    for name, kind in fields:
        size = 1 if kind == "b" else 4
        off = (off + size - 1) // size * size
        out.append((name, kind, off))
        off += size
    return out, (off + 3) // 4 * 4


def _settings_layout(old):
    parts = [VIEW, SETUP, SIM_OLD if old else SIM_NEW, PHYS_OLD if old else PHYS_NEW]
    fields, base = [], 0
    for p in parts:
        lay, size = _layout(p)
        fields += [(n, k, base + o) for n, k, o in lay]
        base += size
    return fields, base


SETTINGS_NEW, SETTINGS_NEW_SIZE = _settings_layout(False)
SETTINGS_OLD, SETTINGS_OLD_SIZE = _settings_layout(True)
assert SETTINGS_NEW_SIZE == 212 and SETTINGS_OLD_SIZE == 204


def decode_settings(raw, old=False):
    """The persisted Settings struct -> dict of every field."""
    fields, size = (SETTINGS_OLD, SETTINGS_OLD_SIZE) if old else (SETTINGS_NEW, SETTINGS_NEW_SIZE)
    if len(raw) < size:
        raise ValueError("settings struct too short")
    out = {}
    for name, kind, off in fields:
        if kind == "b":
            out[name] = bool(raw[off])
        elif kind == "i":
            out[name] = struct.unpack_from("<i", raw, off)[0]
        else:
            out[name] = struct.unpack_from("<f", raw, off)[0]
    if old:
        out["use_f64"] = False      # absent from the old schema: the new schema's default
        out["bond_tearing"] = False
    return out


def encode_settings(values):
    """dict -> the new schema's 212-byte Settings struct (absent fields 0)."""
    raw = bytearray(SETTINGS_NEW_SIZE)
    for name, kind, off in SETTINGS_NEW:
        v = values.get(name, 0)
        if kind == "b":
            raw[off] = 1 if v else 0
        elif kind == "i":
            struct.pack_into("<i", raw, off, int(v))
        else:
            struct.pack_into("<f", raw, off, float(v))
    return bytes(raw)


def parse(buf):
    """Fields of the root State table: numpy arrays, the scripts string, the
    raw settings bytes, and which schema the file follows."""
    b = bytes(buf)
    if len(b) < 8:
        raise ValueError("buffer too small for a FlatBuffer")
    root = struct.unpack_from("<I", b, 0)[0]
    if root + 4 > len(b):
        raise ValueError("root offset out of range")
    vt = root - struct.unpack_from("<i", b, root)[0]
    if vt < 0 or vt + 4 > len(b):
        raise ValueError("vtable offset out of range")
    vtlen, _ = struct.unpack_from("<HH", b, vt)
    nf = (vtlen - 4) // 2
    old = nf <= len(FIELDS_OLD)
    names = FIELDS_OLD if old else FIELDS_NEW
    out = {"schema": "old" if old else "new"}
    for i, name in enumerate(names):
        off = struct.unpack_from("<H", b, vt + 4 + 2 * i)[0] if i < nf else 0
        if off == 0:
            out[name] = None
            continue
        fo = root + off
        if name == "settings":
            size = SETTINGS_OLD_SIZE if old else SETTINGS_NEW_SIZE
            if fo + size > len(b):
                raise ValueError("settings struct out of range")
            out[name] = b[fo:fo + size]
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
        dt = "<i4" if name in INT_VECTORS else "<f4"
        out[name] = np.frombuffer(b, dtype=dt, count=ln, offset=vo + 4).copy()
    if old:
        out["scripts"] = ""
    return out


def uniform_from(st, particles):
    """collision_settings() (settings.rs:2086-2119) for loaded settings; the
    fields a file does not persist keep their Settings::new defaults (walls
    on, wall_friction 0, contact_damping 0.2, bond_damping 0.2, drag 1, mouse
    position 0)."""
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


def settings_from_uniform(uniform, radii, base=None, use_f64=False):
    """Settings fields for save_state from a 29-word uniform dict: the
    persisted ones follow the uniform (and the radii for the setup fields);
    the rest come from `base` (decoded settings of a loaded file) or are 0."""
    v = dict(base or {})
    r = np.asarray(radii, np.float32)
    v.update({
        "particles": int(r.size), "max_radius": float(r.max()) if r.size else 0.0,
        "variable_rad": bool(r.size and r.min() != r.max()),
        "timestep": uniform["dT"], "width": uniform["hor_bound"], "height": uniform["vert_bound"],
        "round_walls": bool(uniform["round_bounds"]), "wall_radius": uniform["bound_radius"],
        "use_f64": bool(use_f64 or v.get("use_f64", False)),
        "gravity": bool(uniform["gravity"]), "g_force": uniform["gravity_acc"],
        "planet_mode": bool(uniform["planet_mode"]), "mouse_gravity": bool(uniform["mouse_gravity"]),
        "collisions": bool(uniform["collisions"]), "collision_interval": uniform["collision_interval"],
        "friction_coef": uniform["friction_coefficient"], "bond": uniform["bonds"],
        "bond_tearing": bool(uniform["bonds_tear"]), "bond_normal_stiffness": uniform["bond_normal_stiffness"],
        "bond_shear_stiffness": uniform["bond_shear_stiffness"],
        "bond_normal_strength": uniform["bond_normal_strength"],
        "bond_shear_strength": uniform["bond_shear_strength"],
        "moment_contribution_factor": uniform["moment_contribution_factor"],
        "local_damping": bool(uniform["local_damping"]), "local_damping_alpha": uniform["local_damping_alpha"],
    })
    v.setdefault("gen_per_frame", 105)
    return v


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
    """State::load (state.rs:583-706) -> (scene dict trimmed to p_count,
    uniform dict, info dict with every decoded setting, 'settings_raw',
    'schema', 'groups' and 'scripts')."""
    buf = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    f = parse(buf)
    if f["settings"] is None:
        raise ValueError("state has no settings")
    st = decode_settings(f["settings"], old=f["schema"] == "old")
    n = st["particles"]
    radii_all = f["radii"] if f["radii"] is not None else np.zeros(0, np.float32)
    rmin = float(radii_all.min()) if radii_all.size else 0.0
    rmax = float(radii_all.max()) if radii_all.size else 0.0
    grid = grid_capacity(st["width"], st["height"], rmax, rmin, rmin != rmax, n)

    def take(name, per, dtype):
        a = f[name] if f[name] is not None else np.zeros(0, dtype)
        if a.size < per * n:
            raise ValueError("%s holds fewer than %d particles" % (name, n))
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
        "bonds": np.ascontiguousarray(f["bonds"] if f["bonds"] is not None else np.full(1, -1), dtype=np.int32),
        "data": np.zeros(7 * n, dtype=np.float32),
        "coll_cont": np.zeros(4, dtype=np.int32),
        "grid": grid,
    }
    # State::restore uploads vel into the del_pos binding and rot_vel into the
    # del_rot binding (wgpu_prog.rs:1247-1248)
    scene["del_pos"] = scene["vel"].copy()
    scene["del_rot"] = scene["rot_vel"].copy()
    info = dict(st)
    info["settings_raw"] = bytes(f["settings"])
    info["schema"] = f["schema"]
    info["groups"] = f["groups"]
    info["scripts"] = f["scripts"]
    return scene, uniform_from(st, n), info


class _Builder:
    """Front-to-back FlatBuffer writer for one root table: objects are
    appended after the table, so every uoffset points forward."""

    def __init__(self):
        self.buf = bytearray()

    def align(self):
        self.buf += b"\0" * (-len(self.buf) % 4)

    def vector(self, arr):
        self.align()
        pos = len(self.buf)
        a = np.ascontiguousarray(arr)
        self.buf += struct.pack("<I", a.size)
        self.buf += a.astype("<i4" if a.dtype.kind in "iu" else "<f4").tobytes()
        return pos

    def string(self, s):
        self.align()
        pos = len(self.buf)
        data = s.encode("utf-8")
        self.buf += struct.pack("<I", len(data)) + data + b"\0"
        return pos


def save_state(scene, uniform, info=None, path=None, use_f64=False):
    """State::save (state.rs:369-493) of a scene dict: the new schema, the
    scene's arrays as they are, settings from the uniform (and, for the view
    and setup fields the uniform does not carry, from `info` of a loaded
    file).  Returns the bytes; writes them to `path` when given."""
    info = info or {}
    base = None
    if info.get("settings_raw") is not None:
        base = decode_settings(info["settings_raw"], old=info.get("schema") == "old")
    settings = encode_settings(settings_from_uniform(uniform, scene["radii"], base, use_f64))
    vectors = [("pos", np.float32), ("vel", np.float32), ("acc", np.float32), ("rot", np.float32),
               ("rot_vel", np.float32), ("rot_acc", np.float32), ("forces", np.float32), ("radii", np.float32),
               ("fixity", np.int32), ("bonds", np.int32), ("contacts", np.int32),
               ("material_pointers", np.int32), ("materials", np.float32)]
    groups = info.get("groups")
    groups = np.zeros(0, np.int32) if groups is None else np.asarray(groups, np.int32)
    scripts = info.get("scripts") or ""
    nfields = len(FIELDS_NEW)
    vt_size = 4 + 2 * nfields
    vt_pos = 4
    table_pos = (vt_pos + vt_size + 3) // 4 * 4
    # table: soffset, 15 uoffsets (ids 0-14), settings struct (id 15)
    table_size = 4 + 4 * (nfields - 1) + SETTINGS_NEW_SIZE
    b = _Builder()
    b.buf += struct.pack("<I", table_pos)
    vt = [vt_size, table_size] + [4 + 4 * i for i in range(nfields - 1)] + [4 + 4 * (nfields - 1)]
    b.buf += struct.pack("<%dH" % len(vt), *vt)
    b.align()
    assert len(b.buf) == table_pos
    b.buf += struct.pack("<i", table_pos - vt_pos)
    b.buf += b"\0" * (4 * (nfields - 1))
    b.buf += settings
    targets = [b.vector(np.asarray(scene[k], dt)) for k, dt in vectors]
    targets.append(b.vector(groups))
    targets.append(b.string(scripts))
    for i, t in enumerate(targets):
        fo = table_pos + 4 + 4 * i
        struct.pack_into("<I", b.buf, fo, t - fo)
    b.align()
    out = bytes(b.buf)
    if path is not None:
        with open(path, "wb") as fh:
            fh.write(out)
    return out
