"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE, never the product).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm
use this module.  It drives oracle/_build/liborc.so, a deterministic C
restatement of the reference's two WGSL physics passes
(src/shaders/physics/2D_LOM.wgsl:80-201 and 2D_Simulation.wgsl:108-478).

A scene is a dict of numpy arrays in the reference's host layouts
(src/state.rs:69-93):

    pos f32[2n], radii f32[n], vel f32[2n], acc f32[2n], rot f32[n],
    rot_vel f32[n], rot_acc f32[n], forces f32[6n], fixity i32[6n],
    del_pos f32[2n], del_rot f32[n], bonds i32[3B] (raw bits),
    contacts i32[84n] (raw bits, 14 records of 6 words per particle),
    material_pointers i32[n], materials f32[6M], data f32[7n],
    coll_cont i32[4], grid i32-or-f32 tuple (cell_size, cell_cap, w, h)

Settings are the 29-word uniform of settings.rs:2086-2119 as a dict.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

MAX_CONTACTS = 14
DATA_SIZE = 7

SETTINGS_FIELDS = [
    ("walls", C.c_int32), ("hor_bound", C.c_float), ("vert_bound", C.c_float),
    ("round_bounds", C.c_int32), ("bound_radius", C.c_float), ("wall_friction", C.c_float),
    ("gravity", C.c_int32), ("planet_mode", C.c_int32), ("bonds", C.c_int32),
    ("collisions", C.c_int32), ("friction_coefficient", C.c_float), ("gravity_acc", C.c_float),
    ("bond_normal_stiffness", C.c_float), ("bonds_tear", C.c_int32),
    ("bond_normal_strength", C.c_float), ("contact_damping", C.c_float),
    ("bond_damping", C.c_float), ("drag", C.c_float), ("bond_shear_strength", C.c_float),
    ("dT", C.c_float), ("bond_shear_stiffness", C.c_float), ("gravity_x", C.c_float),
    ("gravity_y", C.c_float), ("mouse_gravity", C.c_int32),
    ("moment_contribution_factor", C.c_float), ("collision_interval", C.c_int32),
    ("local_damping", C.c_int32), ("local_damping_alpha", C.c_float), ("particles", C.c_int32),
]


class Settings(C.Structure):
    _fields_ = SETTINGS_FIELDS


class Ext(C.Structure):
    _fields_ = [("use_f64", C.c_int32), ("bond_lambda", C.c_float),
                ("bond_sn", C.POINTER(C.c_float)), ("bond_ss", C.POINTER(C.c_float)),
                ("restitution", C.c_float)]


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)


class State(C.Structure):
    _fields_ = [("n", C.c_int32), ("n_bonds", C.c_int32), ("n_materials", C.c_int32),
                ("pos", _FP), ("radii", _FP), ("vel", _FP), ("acc", _FP), ("rot", _FP),
                ("rot_vel", _FP), ("rot_acc", _FP), ("forces", _FP), ("fixity", _IP),
                ("del_pos", _FP), ("del_rot", _FP), ("bonds", _IP), ("contacts", _IP),
                ("material_pointers", _IP), ("materials", _FP), ("data", _FP),
                ("coll_cont", C.c_int32 * 4), ("cell_size", C.c_float), ("cell_cap", C.c_int32),
                ("grid_w", C.c_int32), ("grid_h", C.c_int32)]


class StateD(C.Structure):
    _fields_ = [(k, _DP) for k in ("pos", "vel", "acc", "rot", "rot_vel", "rot_acc", "del_pos",
                                   "del_rot", "data", "slot_tf", "slot_btf", "slot_thb")]


class Break(C.Structure):
    _fields_ = [("step", C.c_int32), ("bond", C.c_int32), ("code", C.c_int32),
                ("a", C.c_int32), ("b", C.c_int32)]


BREAK_DTYPE = np.dtype([("step", "<i4"), ("bond", "<i4"), ("code", "<i4"), ("a", "<i4"), ("b", "<i4")])

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        L.orc_step_f32.argtypes = [C.POINTER(State), C.POINTER(Settings), C.POINTER(Ext), C.c_int,
                                   C.c_int, C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int64), C.c_int]
        L.orc_step_f32.restype = C.c_int
        L.orc_step_f64.argtypes = [C.POINTER(State), C.POINTER(Settings), C.POINTER(Ext), C.c_int,
                                   C.POINTER(StateD), C.c_int]
        L.orc_step_f64.restype = C.c_int
        L.orc_set_properties.argtypes = [C.POINTER(State), _IP, _IP]
        L.orc_set_properties.restype = None
        L.orc_grid_capacity.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                        _FP, _IP, _IP, _IP]
        L.orc_grid_capacity.restype = None
        L.orc_regen_bonds.argtypes = [C.c_int, _FP, _FP, C.c_int, _IP, _IP]
        L.orc_regen_bonds.restype = C.c_int
        _lib = L
    return _lib


F32_KEYS = ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "del_pos",
            "del_rot", "materials", "data")
I32_KEYS = ("fixity", "bonds", "contacts", "material_pointers", "coll_cont")


def _ptr(a, ty):
    return a.ctypes.data_as(ty)


def make_settings(d):
    s = Settings()
    for k, _ in SETTINGS_FIELDS:
        setattr(s, k, d[k])
    return s


def _check(scene):
    for k in F32_KEYS:
        a = scene[k]
        assert a.dtype == np.float32 and a.flags.c_contiguous, k
    for k in I32_KEYS:
        a = scene[k]
        assert a.dtype == np.int32 and a.flags.c_contiguous, k


def make_state(scene):
    _check(scene)
    n = int(scene["radii"].shape[0])
    st = State()
    st.n = n
    st.n_bonds = int(scene["bonds"].shape[0] // 3)
    st.n_materials = int(scene["materials"].shape[0] // 6)
    for k in ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "del_pos",
              "del_rot", "materials", "data"):
        setattr(st, k, _ptr(scene[k], _FP))
    for k in ("fixity", "bonds", "contacts", "material_pointers"):
        setattr(st, k, _ptr(scene[k], _IP))
    for i in range(4):
        st.coll_cont[i] = int(scene["coll_cont"][i])
    cs, cap, w, h = scene["grid"]
    st.cell_size = float(cs)
    st.cell_cap = int(cap)
    st.grid_w = int(w)
    st.grid_h = int(h)
    return st


def make_ext(use_f64=False, bond_lambda=0.5, bond_sn=None, bond_ss=None, keep=None, restitution=0.0):
    e = Ext()
    e.use_f64 = 1 if use_f64 else 0
    e.bond_lambda = bond_lambda
    e.restitution = restitution
    if bond_sn is not None:
        bond_sn = np.ascontiguousarray(bond_sn, dtype=np.float32)
        e.bond_sn = _ptr(bond_sn, _FP)
        if keep is not None:
            keep.append(bond_sn)
    if bond_ss is not None:
        bond_ss = np.ascontiguousarray(bond_ss, dtype=np.float32)
        e.bond_ss = _ptr(bond_ss, _FP)
        if keep is not None:
            keep.append(bond_ss)
    return e


def step(scene, settings, nsteps, *, use_f64=False, bond_lambda=0.5, bond_sn=None, bond_ss=None,
         step_base=0, threads=0, ev_cap=1 << 16, restitution=0.0):
    """Advance `scene` in place by nsteps; return (break events, stats[4]).
    restitution > 0 switches on the normal dashpot extension (not in the
    reference)."""
    keep = []
    st = make_state(scene)
    ext = make_ext(use_f64, bond_lambda, bond_sn, bond_ss, keep, restitution)
    s = make_settings(settings)
    ev = np.zeros(ev_cap, dtype=BREAK_DTYPE)
    nev = C.c_int(0)
    stats = np.zeros(4, dtype=np.int64)
    rc = lib().orc_step_f32(C.byref(st), C.byref(s), C.byref(ext), int(nsteps), int(step_base),
                            ev.ctypes.data, ev_cap, C.byref(nev), _ptr(stats, C.POINTER(C.c_int64)),
                            int(threads))
    if rc != 0:
        raise RuntimeError("oracle step rejected its input")
    scene["coll_cont"][:] = np.array(st.coll_cont[:], dtype=np.int32)
    return ev[: min(nev.value, ev_cap)].copy(), stats


def step_f64(scene, settings, nsteps=1, *, use_f64=False, bond_lambda=0.5, bond_sn=None,
             bond_ss=None, threads=0, restitution=0.0):
    """FP64 twin: evolve a copy of `scene` in double; return a dict of float64 arrays."""
    keep = []
    st = make_state(scene)
    ext = make_ext(use_f64, bond_lambda, bond_sn, bond_ss, keep, restitution)
    s = make_settings(settings)
    n = int(scene["radii"].shape[0])
    out = {"pos": np.zeros(2 * n), "vel": np.zeros(2 * n), "acc": np.zeros(2 * n),
           "rot": np.zeros(n), "rot_vel": np.zeros(n), "rot_acc": np.zeros(n),
           "del_pos": np.zeros(2 * n), "del_rot": np.zeros(n), "data": np.zeros(7 * n),
           "slot_tf": np.zeros(MAX_CONTACTS * n), "slot_btf": np.zeros(MAX_CONTACTS * n),
           "slot_thb": np.zeros(MAX_CONTACTS * n)}
    sd = StateD()
    for k, v in out.items():
        setattr(sd, k, _ptr(v, _DP))
    rc = lib().orc_step_f64(C.byref(st), C.byref(s), C.byref(ext), int(nsteps), C.byref(sd),
                            int(threads))
    if rc != 0:
        raise RuntimeError("oracle FP64 step rejected its input")
    return out


def set_properties(scene, selections, words):
    """Set_Properties event (Set_Properties.wgsl:68-90); words = 28 int32 words."""
    st = make_state(scene)
    sel = np.ascontiguousarray(selections, dtype=np.int32)
    w = np.ascontiguousarray(words, dtype=np.int32)
    assert w.shape == (28,)
    lib().orc_set_properties(C.byref(st), _ptr(sel, _IP), _ptr(w, _IP))
    scene["coll_cont"][:] = np.array(st.coll_cont[:], dtype=np.int32)
    return sel


def grid_capacity(hor_bound, vert_bound, max_radius, min_radius, variable_rad, particles):
    cs = C.c_float()
    cap = C.c_int32()
    w = C.c_int32()
    h = C.c_int32()
    lib().orc_grid_capacity(hor_bound, vert_bound, max_radius, min_radius, int(variable_rad),
                            int(particles), C.byref(cs), C.byref(cap), C.byref(w), C.byref(h))
    return (cs.value, cap.value, w.value, h.value)


def regen_bonds(pos, radii, max_bonds=6):
    """Bond generation of state.rs:291-367; returns (bonds i32[3B], contacts i32[84n])."""
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    n = radii.shape[0]
    bonds = np.full(3 * max_bonds * max(n, 1), -1, dtype=np.int32)
    contacts = np.full(6 * MAX_CONTACTS * n, -1, dtype=np.int32)
    nb = lib().orc_regen_bonds(n, _ptr(pos, _FP), _ptr(radii, _FP), max_bonds, _ptr(bonds, _IP),
                               _ptr(contacts, _IP))
    bonds = bonds[: 3 * nb].copy()
    if nb == 0:
        bonds = np.full(1, -1, dtype=np.int32)
    return bonds, contacts
