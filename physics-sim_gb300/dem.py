"""ctypes binding of libdemgb.so (include/dem.h, include/dem_debug.h).

The host-side mirror of the reference's compute program for Python callers:
`Context` plays WGPUComputeProg (src/wgpu_prog.rs): `step(n)` is `compute`
with gen_per_frame = n, `upload` is `restore`, `download` is `update_state`,
`set_properties` is the Set_Properties event.  Scenes are dicts of numpy
arrays in the reference's host layouts (src/state.rs:69-93):

    pos f32[2n], radii f32[n], vel f32[2n], acc f32[2n], rot f32[n],
    rot_vel f32[n], rot_acc f32[n], forces f32[6n], fixity i32[6n],
    del_pos f32[2n], del_rot f32[n], bonds i32[3B], contacts i32[84n],
    material_pointers i32[n], materials f32[6M], data f32[7n],
    coll_cont i32[4], grid (cell_size, cell_cap, w, h)

There is no fallback: if the CUDA library cannot be loaded, or no GPU is
present, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdemgb.so")

MAX_CONTACTS = 14
DATA_SIZE = 7

DEM_E = {0: "OK", -1: "INVALID", -2: "OOM", -3: "CUDA", -4: "TIMEOUT", -5: "STATE",
         -6: "UNSUPPORTED", -7: "CAPACITY"}

PARAM_FIELDS = [
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

_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)


class Params(C.Structure):
    _fields_ = PARAM_FIELDS


class GridInfo(C.Structure):
    _fields_ = [("cell_size", C.c_float), ("cell_cap", C.c_int32), ("w", C.c_int32), ("h", C.c_int32)]


class Ext(C.Structure):
    _fields_ = [("use_f64", C.c_int32), ("bond_lambda", C.c_float),
                ("bond_normal_strength", _FP), ("bond_shear_strength", _FP),
                ("diagnostics", C.c_int32), ("reorder_interval", C.c_int32),
                ("block_size", C.c_int32), ("search_cell_factor", C.c_float),
                ("event_capacity", C.c_int32), ("list_skin", C.c_float),
                ("plain_launches", C.c_int32), ("split_narrow", C.c_int32), ("unfused_lom", C.c_int32),
                ("host_copies", C.c_int32), ("reorder_every", C.c_int32), ("restitution", C.c_float)]


class Scene(C.Structure):
    # array fields are plain addresses (float* / int32_t* in dem.h): setting
    # an int is several times cheaper than building a ctypes pointer, which
    # matters when hundreds of scenes are marshalled per call
    _fields_ = [("n_particles", C.c_int32), ("n_bonds", C.c_int32), ("n_materials", C.c_int32),
                ("pos", C.c_void_p), ("radii", C.c_void_p), ("vel", C.c_void_p), ("acc", C.c_void_p),
                ("rot", C.c_void_p), ("rot_vel", C.c_void_p), ("rot_acc", C.c_void_p),
                ("forces", C.c_void_p), ("fixity", C.c_void_p), ("del_pos", C.c_void_p),
                ("del_rot", C.c_void_p), ("bonds", C.c_void_p), ("contacts", C.c_void_p),
                ("material_pointers", C.c_void_p), ("materials", C.c_void_p), ("data", C.c_void_p),
                ("coll_cont", C.c_int32 * 4), ("grid", GridInfo)]


class BreakEvent(C.Structure):
    _fields_ = [("scene", C.c_int32), ("step", C.c_int32), ("bond", C.c_int32),
                ("code", C.c_int32), ("a", C.c_int32), ("b", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("capped", C.c_int64), ("events", C.c_int64),
                ("events_dropped", C.c_int64), ("reorders", C.c_int64),
                ("device_error", C.c_int32), ("reserved", C.c_int32),
                ("kernel_launches", C.c_int64), ("list_overflows", C.c_int64)]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_int64), ("max_active_particles", C.c_int64),
                ("max_scenes", C.c_int32), ("cells_per_particle", C.c_float),
                ("bonds_per_particle", C.c_float), ("reserved", C.c_int32), ("ext", Ext)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("queued", "running", "completed", "active_particles",
                                         "particle_steps", "capacity_particles", "used_particles",
                                         "device_bytes", "steps", "waits_active", "waits_memory")]


class TuneResult(C.Structure):
    _fields_ = [("search_cell_factor", C.c_float), ("list_skin", C.c_float), ("block_size", C.c_int32),
                ("reorder_interval", C.c_int32), ("ms_per_step", C.c_double),
                ("default_ms_per_step", C.c_double), ("trials", C.c_int32), ("sample_scenes", C.c_int32),
                ("sample_particles", C.c_int64), ("seconds", C.c_double), ("split_narrow", C.c_int32),
                ("unfused_lom", C.c_int32), ("reserved", C.c_int32 * 6)]


EVENT_FIX, EVENT_DROP, EVENT_RELEASE = 1, 2, 3

BREAK_DTYPE = np.dtype([("scene", "<i4"), ("step", "<i4"), ("bond", "<i4"), ("code", "<i4"),
                        ("a", "<i4"), ("b", "<i4")])

# exported symbols of include/dem.h and include/dem_debug.h
SYMBOLS = ["dem_abi_version", "dem_ext_defaults", "dem_last_error", "dem_grid_capacity",
           "dem_create", "dem_destroy", "dem_upload", "dem_set_params", "dem_set_materials",
           "dem_set_control", "dem_get_control", "dem_step", "dem_synchronize", "dem_download",
           "dem_set_properties", "dem_break_events", "dem_get_stats", "dem_stream",
           "dem_debug_broad_phase", "dem_debug_search_grid", "dem_debug_kernel_timing",
           "dem_debug_kernel_time", "dem_broad_phase_noalloc", "dem_noalloc_last_error",
           "dem_batch_create", "dem_batch_destroy", "dem_batch_last_error", "dem_batch_scene_count",
           "dem_batch_step", "dem_batch_synchronize", "dem_batch_download", "dem_batch_upload",
           "dem_batch_set_params", "dem_batch_set_properties", "dem_batch_break_events",
           "dem_batch_get_stats", "dem_batch_stream", "dem_batch_kernel_timing",
           "dem_batch_kernel_time", "dem_server_config_defaults", "dem_server_create",
           "dem_server_destroy", "dem_server_last_error", "dem_server_submit", "dem_server_submit_borrowed",
           "dem_server_advance",
           "dem_server_poll", "dem_server_fetch", "dem_server_events", "dem_server_release",
           "dem_server_get_stats", "dem_server_stream", "dem_batch_autotune", "dem_tune_last_error",
           "dem_generate_bonds", "dem_bondgen_last_error", "dem_event", "dem_get_datum",
           "dem_batch_event", "dem_batch_get_datum", "dem_batch_upload_many", "dem_batch_download_many",
           "dem_record", "dem_batch_record",
           "dem_server_cancel"]

_lib = None


class DemError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("dem error %d (%s): %s" % (code, DEM_E.get(code, "?"), msg))
        self.code = code


def lib(path=None):
    """Load libdemgb.so (built by build_lib.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise OSError("libdemgb.so not built at %s (run __graft_entry__.build())" % path)
    L = C.CDLL(path)
    L.dem_abi_version.restype = C.c_int
    L.dem_ext_defaults.argtypes = [C.POINTER(Ext)]
    L.dem_last_error.argtypes = [C.c_void_p]
    L.dem_last_error.restype = C.c_char_p
    L.dem_grid_capacity.argtypes = [C.POINTER(Params), _FP, C.c_int32, C.c_int32, C.POINTER(GridInfo)]
    L.dem_create.argtypes = [C.POINTER(Scene), C.POINTER(Params), C.POINTER(Ext), C.c_int,
                             C.POINTER(C.c_void_p)]
    L.dem_destroy.argtypes = [C.c_void_p]
    L.dem_destroy.restype = None
    L.dem_upload.argtypes = [C.c_void_p, C.POINTER(Scene)]
    L.dem_set_params.argtypes = [C.c_void_p, C.POINTER(Params)]
    L.dem_set_materials.argtypes = [C.c_void_p, _FP, C.c_int32]
    L.dem_set_control.argtypes = [C.c_void_p, _IP]
    L.dem_get_control.argtypes = [C.c_void_p, _IP]
    L.dem_step.argtypes = [C.c_void_p, C.c_int32]
    L.dem_synchronize.argtypes = [C.c_void_p]
    L.dem_download.argtypes = [C.c_void_p, C.POINTER(Scene)]
    L.dem_set_properties.argtypes = [C.c_void_p, _IP, _IP]
    L.dem_break_events.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.dem_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.dem_stream.argtypes = [C.c_void_p]
    L.dem_stream.restype = C.c_void_p
    L.dem_debug_broad_phase.argtypes = [C.c_void_p, _IP, _IP, _IP, C.POINTER(C.c_int32)]
    L.dem_debug_search_grid.argtypes = [C.c_void_p, _FP, _FP, _FP, _IP, _IP]
    L.dem_debug_kernel_timing.argtypes = [C.c_void_p, C.c_int32]
    L.dem_debug_kernel_time.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double),
                                        C.POINTER(C.c_int64)]
    L.dem_broad_phase_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float,
                                          C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
    L.dem_noalloc_last_error.restype = C.c_char_p
    L.dem_batch_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int,
                                   C.POINTER(C.c_void_p)]
    L.dem_batch_destroy.argtypes = [C.c_void_p]
    L.dem_batch_destroy.restype = None
    L.dem_batch_last_error.argtypes = [C.c_void_p]
    L.dem_batch_last_error.restype = C.c_char_p
    L.dem_batch_scene_count.argtypes = [C.c_void_p]
    L.dem_batch_step.argtypes = [C.c_void_p, C.c_int32]
    L.dem_batch_synchronize.argtypes = [C.c_void_p]
    L.dem_batch_download.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Scene)]
    L.dem_batch_upload.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Scene)]
    L.dem_batch_upload_many.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.dem_batch_download_many.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    L.dem_batch_set_params.argtypes = [C.c_void_p, C.c_int32, C.POINTER(Params)]
    L.dem_batch_set_properties.argtypes = [C.c_void_p, C.c_int32, _IP, _IP]
    L.dem_batch_break_events.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.dem_batch_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.dem_batch_stream.argtypes = [C.c_void_p]
    L.dem_batch_stream.restype = C.c_void_p
    L.dem_server_config_defaults.argtypes = [C.POINTER(ServerConfig)]
    L.dem_server_config_defaults.restype = None
    L.dem_server_create.argtypes = [C.POINTER(ServerConfig), C.c_int, C.POINTER(C.c_void_p)]
    L.dem_server_destroy.argtypes = [C.c_void_p]
    L.dem_server_destroy.restype = None
    L.dem_server_last_error.argtypes = [C.c_void_p]
    L.dem_server_last_error.restype = C.c_char_p
    L.dem_tune_last_error.argtypes = []
    L.dem_tune_last_error.restype = C.c_char_p
    L.dem_event.argtypes = [C.c_void_p, C.c_int32, _IP, C.c_int32, C.c_float, C.c_float, C.c_int32]
    L.dem_get_datum.argtypes = [C.c_void_p, _IP, C.POINTER(C.c_double)]
    L.dem_batch_event.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _IP, C.c_int32, C.c_float, C.c_float,
                                  C.c_int32]
    L.dem_batch_get_datum.argtypes = [C.c_void_p, C.c_int32, _IP, C.POINTER(C.c_double)]
    L.dem_record.argtypes = [C.c_void_p, C.c_int32, _IP, C.POINTER(C.c_double)]
    L.dem_batch_record.argtypes = [C.c_void_p, C.c_int32, C.c_int32, _IP, C.POINTER(C.c_double)]
    L.dem_bondgen_last_error.argtypes = []
    L.dem_bondgen_last_error.restype = C.c_char_p
    L.dem_generate_bonds.argtypes = [_FP, _FP, C.c_int32, C.c_int32, C.c_int32, _IP, C.c_int64,
                                     C.POINTER(C.c_int64), _IP]
    L.dem_batch_autotune.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64,
                                     C.c_int32, C.POINTER(TuneResult)]
    L.dem_server_submit.argtypes = [C.c_void_p, C.POINTER(Scene), C.POINTER(Params), C.POINTER(Ext),
                                    C.c_int64, C.POINTER(C.c_int64)]
    L.dem_server_submit_borrowed.argtypes = L.dem_server_submit.argtypes
    L.dem_server_advance.argtypes = [C.c_void_p, C.c_int32]
    L.dem_server_poll.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_int32)]
    L.dem_server_fetch.argtypes = [C.c_void_p, C.c_int64, C.POINTER(Scene), C.POINTER(C.c_double)]
    L.dem_server_events.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.POINTER(C.c_int32)]
    L.dem_server_release.argtypes = [C.c_void_p, C.c_int64]
    L.dem_server_cancel.argtypes = [C.c_void_p, C.c_int64]
    L.dem_server_get_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    L.dem_server_stream.argtypes = [C.c_void_p]
    L.dem_server_stream.restype = C.c_void_p
    for name in SYMBOLS:
        if name not in ("dem_destroy", "dem_ext_defaults", "dem_last_error", "dem_stream",
                        "dem_abi_version", "dem_noalloc_last_error", "dem_batch_destroy",
                        "dem_batch_last_error", "dem_batch_stream", "dem_server_config_defaults",
                        "dem_server_destroy", "dem_server_last_error", "dem_server_stream",
                        "dem_tune_last_error", "dem_bondgen_last_error"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def make_params(d):
    p = Params()
    for k, _ in PARAM_FIELDS:
        setattr(p, k, d[k])
    return p


def make_ext(use_f64=False, bond_lambda=0.5, bond_sn=None, bond_ss=None, diagnostics=True,
             reorder_interval=0, block_size=0, search_cell_factor=0.0, event_capacity=0,
             list_skin=0.0, plain_launches=False, split_narrow=0, unfused_lom=0, host_copies=0, reorder_every=0,
             restitution=0.0, keep=None):
    e = Ext()
    lib().dem_ext_defaults(C.byref(e))
    e.use_f64 = 1 if use_f64 else 0
    e.bond_lambda = bond_lambda
    e.diagnostics = 1 if diagnostics else 0
    e.reorder_interval = reorder_interval
    e.block_size = block_size
    e.search_cell_factor = search_cell_factor
    e.event_capacity = event_capacity
    e.list_skin = list_skin
    e.plain_launches = 1 if plain_launches else 0
    e.split_narrow = 1 if split_narrow else 0
    e.unfused_lom = 1 if unfused_lom else 0
    e.host_copies = 1 if host_copies else 0
    e.reorder_every = int(reorder_every)
    e.restitution = float(restitution)
    for attr, arr in (("bond_normal_strength", bond_sn), ("bond_shear_strength", bond_ss)):
        if arr is not None:
            a = np.ascontiguousarray(arr, dtype=np.float32)
            setattr(e, attr, a.ctypes.data_as(_FP))
            if keep is not None:
                keep.append(a)
    return e


F32_KEYS = ("pos", "radii", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "del_pos",
            "del_rot", "materials", "data")
I32_KEYS = ("fixity", "bonds", "contacts", "material_pointers")
# words per particle of the per-particle arrays (state.rs:69-93)
_PER_PARTICLE = (("pos", 2), ("vel", 2), ("acc", 2), ("rot", 1), ("rot_vel", 1), ("rot_acc", 1),
                 ("forces", 6), ("fixity", 6), ("del_pos", 2), ("del_rot", 1), ("contacts", 84),
                 ("material_pointers", 1), ("data", 7))


# The data pointer of an ndarray is the first field after the object header
# (PyArrayObject_fields.data, which numpy's PyArray_DATA reads); on CPython
# reading it there costs a fifth of __array_interface__, which matters when
# hundreds of scenes are marshalled per call.  Checked once against numpy's
# own answer; anything else falls back to the interface.
_DATA_OFFSET = 2 * C.sizeof(C.c_void_p)


def _fast_data_probe():
    import platform
    if platform.python_implementation() != "CPython":
        return False
    a = np.zeros(3, dtype=np.float32)
    return C.c_void_p.from_address(id(a) + _DATA_OFFSET).value == a.ctypes.data


_FAST_DATA = _fast_data_probe()


def _addr(a):
    if _FAST_DATA:
        return C.c_void_p.from_address(id(a) + _DATA_OFFSET).value
    return a.__array_interface__["data"][0]


def make_scene(sc, s=None):
    """Scene struct (or the given one, filled) pointing into the numpy arrays of
    dict `sc` (kept alive by the caller)."""
    for k in F32_KEYS:
        a = sc[k]
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            raise TypeError("%s must be contiguous float32" % k)
    for k in I32_KEYS:
        a = sc[k]
        if a.dtype != np.int32 or not a.flags.c_contiguous:
            raise TypeError("%s must be contiguous int32" % k)
    n = int(sc["radii"].shape[0])
    for k, per in _PER_PARTICLE:
        a = sc.get(k)
        if a is None and k == "data":
            continue
        if a.size != per * n:
            raise ValueError("%s holds %d values, expected %d x %d particles" % (k, a.size, per, n))
    if s is None:
        s = Scene()
    s.n_particles = n
    s.n_bonds = int(sc["bonds"].shape[0] // 3)
    s.n_materials = int(sc["materials"].shape[0] // 6)
    for k in F32_KEYS:
        setattr(s, k, _addr(sc[k]))
    for k in I32_KEYS:
        setattr(s, k, _addr(sc[k]))
    s.coll_cont[:] = [int(v) for v in sc["coll_cont"]]
    cs, cap, w, h = sc["grid"]
    s.grid.cell_size = float(cs)
    s.grid.cell_cap = int(cap)
    s.grid.w = int(w)
    s.grid.h = int(h)
    return s


def empty_like_scene(sc):
    out = {k: np.zeros_like(sc[k]) for k in F32_KEYS + I32_KEYS}
    # a scene without bonds carries the placeholder record [-1] (state.rs:357-359)
    if sc["bonds"].shape[0] < 3:
        out["bonds"] = sc["bonds"].copy()
    out["coll_cont"] = np.zeros(4, dtype=np.int32)
    out["grid"] = sc["grid"]
    return out


def _check(L, ctx, rc):
    if rc != 0:
        raise DemError(rc, (L.dem_last_error(ctx) or b"").decode())


class Context:
    """One scene resident on one GPU (WGPUComputeProg's compute side)."""

    def __init__(self, scene, params, *, device=-1, **ext_kw):
        L = lib()
        self._keep = []
        self.params = dict(params)
        ext = make_ext(keep=self._keep, **ext_kw)
        self._template = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in scene.items()}
        st = make_scene(scene)
        p = make_params(self.params)
        h = C.c_void_p()
        rc = L.dem_create(C.byref(st), C.byref(p), C.byref(ext), device, C.byref(h))
        if rc != 0:
            raise DemError(rc, (L.dem_last_error(None) or b"").decode())
        self.h = h
        self.n = int(scene["radii"].shape[0])
        self.dt = np.float32(self.params["dT"])

    def close(self):
        if getattr(self, "h", None):
            lib().dem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, n=1):
        L = lib()
        _check(L, self.h, L.dem_step(self.h, int(n)))

    def synchronize(self):
        L = lib()
        _check(L, self.h, L.dem_synchronize(self.h))

    def download(self, out=None):
        """The scene in the reference's layouts (update_state); `out`, a scene
        dict from an earlier download, is filled in place instead of a new one."""
        L = lib()
        out = empty_like_scene(self._template) if out is None else out
        st = make_scene(out)
        _check(L, self.h, L.dem_download(self.h, C.byref(st)))
        out["coll_cont"] = np.array(st.coll_cont[:], dtype=np.int32)
        return out

    def upload(self, scene):
        L = lib()
        st = make_scene(scene)
        _check(L, self.h, L.dem_upload(self.h, C.byref(st)))

    def set_params(self, params):
        L = lib()
        self.params = dict(params)
        p = make_params(self.params)
        _check(L, self.h, L.dem_set_params(self.h, C.byref(p)))

    def set_properties(self, selections, words):
        L = lib()
        sel = np.ascontiguousarray(selections, dtype=np.int32).copy()
        w = np.ascontiguousarray(words, dtype=np.int32)
        _check(L, self.h, L.dem_set_properties(self.h, sel.ctypes.data_as(_IP), w.ctypes.data_as(_IP)))
        return sel

    def control(self):
        L = lib()
        cc = np.zeros(4, dtype=np.int32)
        _check(L, self.h, L.dem_get_control(self.h, cc.ctypes.data_as(_IP)))
        return cc

    def set_control(self, cc):
        L = lib()
        cc = np.ascontiguousarray(cc, dtype=np.int32)
        _check(L, self.h, L.dem_set_control(self.h, cc.ctypes.data_as(_IP)))

    def event(self, kind, selections, throw=False, del_x=0.0, del_y=0.0, ticks=1):
        """Fix / Drop / Release (EVENT_FIX, EVENT_DROP, EVENT_RELEASE) on the
        marked particles; `selections` (int32[n]) is updated in place."""
        L = lib()
        assert selections.dtype == np.int32 and selections.flags.c_contiguous
        _check(L, self.h, L.dem_event(self.h, kind, selections.ctypes.data_as(_IP), 1 if throw else 0,
                                      del_x, del_y, ticks))

    def datum(self, selections):
        """State::get_datum on the device state: 10 doubles, or None when
        nothing is selected."""
        L = lib()
        sel = np.ascontiguousarray(selections, dtype=np.int32)
        out = (C.c_double * 10)()
        rc = L.dem_get_datum(self.h, sel.ctypes.data_as(_IP), out)
        if rc < 0:
            _check(L, self.h, rc)
        return None if rc == 0 else np.array(out[:], np.float64)

    def record(self, n_steps, selections):
        """Advance with Record on: n_steps steps, each followed by the datum
        of the selected particles, gathered on the device and read back once
        (dem_record).  Returns an (n_steps, 10) float64 array, or None when
        nothing is selected (the steps still run)."""
        L = lib()
        sel = np.ascontiguousarray(selections, dtype=np.int32)
        rows = np.zeros((max(int(n_steps), 1), 10), np.float64)
        rc = L.dem_record(self.h, int(n_steps), sel.ctypes.data_as(_IP), rows.ctypes.data_as(C.POINTER(C.c_double)))
        if rc < 0:
            _check(L, self.h, rc)
        return None if rc == 0 else rows[: int(n_steps)]

    def break_events(self, cap=1 << 16):
        L = lib()
        buf = np.zeros(cap, dtype=BREAK_DTYPE)
        n = C.c_int32(0)
        _check(L, self.h, L.dem_break_events(self.h, buf.ctypes.data, cap, C.byref(n)))
        return buf[: n.value].copy()

    def stats(self):
        L = lib()
        s = Stats()
        _check(L, self.h, L.dem_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_ if k != "reserved"}

    def stream(self):
        return lib().dem_stream(self.h)

    def kernel_timing(self, on):
        L = lib()
        _check(L, self.h, L.dem_debug_kernel_timing(self.h, 1 if on else 0))

    def kernel_time(self, kernel):
        """(total device ms, launches) of a kernel since kernel timing was enabled."""
        L = lib()
        ms = C.c_double(0.0)
        n = C.c_int64(0)
        _check(L, self.h, L.dem_debug_kernel_time(self.h, kernel.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def broad_phase(self):
        """(keys per particle, particle order, cell_start) of the current positions."""
        L = lib()
        nc = C.c_int32(0)
        _check(L, self.h, L.dem_debug_broad_phase(self.h, None, None, None, C.byref(nc)))
        keys = np.zeros(self.n, dtype=np.int32)
        order = np.zeros(self.n, dtype=np.int32)
        cs = np.zeros(nc.value + 1, dtype=np.int32)
        _check(L, self.h, L.dem_debug_broad_phase(self.h, keys.ctypes.data_as(_IP),
                                                  order.ctypes.data_as(_IP), cs.ctypes.data_as(_IP),
                                                  C.byref(nc)))
        return keys, order, cs

    def search_grid(self):
        L = lib()
        x0, y0, inv = C.c_float(), C.c_float(), C.c_float()
        gw, gh = C.c_int32(), C.c_int32()
        _check(L, self.h, L.dem_debug_search_grid(self.h, C.byref(x0), C.byref(y0), C.byref(inv),
                                                  C.byref(gw), C.byref(gh)))
        return x0.value, y0.value, inv.value, gw.value, gh.value


def generate_bonds(pos, radii, max_bonds=6, device=-1):
    """dem_generate_bonds: regen_bonds (src/state.rs:291-367) on the GPU.
    Returns (bonds i32[3 nb] or [-1] when there are none, contacts i32[84 n]),
    the arrays State::regen_bonds leaves in the state."""
    L = lib()
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1)
    radii = np.ascontiguousarray(radii, dtype=np.float32)
    n = radii.size
    contacts = np.empty(6 * MAX_CONTACTS * n, np.int32)
    nb = C.c_int64(0)
    cap = max(n * max_bonds, 1)
    bonds = np.empty(3 * cap, np.int32)
    rc = L.dem_generate_bonds(pos.ctypes.data_as(_FP), radii.ctypes.data_as(_FP), n, max_bonds, device,
                              bonds.ctypes.data_as(_IP), cap, C.byref(nb), contacts.ctypes.data_as(_IP))
    if rc != 0:
        raise DemError(rc, (L.dem_bondgen_last_error() or b"").decode())
    if nb.value == 0:
        return np.full(1, -1, np.int32), contacts
    return bonds[:3 * nb.value].copy(), contacts


def autotune(items, *, device=-1, sample_particles=0, trial_steps=0, **world_kw):
    """dem_batch_autotune over (scene, params, ext) items: returns (ext keyword
    arguments to pass to Batch/Context, info dict).  The knobs it picks change
    speed only; results are the same for every choice."""
    L = lib()
    keep = []
    n = len(items)
    scenes = (Scene * n)()
    params = (Params * n)()
    exts = (Ext * n)()
    for k, (sc, p, ext) in enumerate(items):
        kw = dict(world_kw)
        kw.update(ext)
        scenes[k] = make_scene(sc)
        params[k] = make_params(p)
        exts[k] = make_ext(keep=keep, **kw)
    ptrs = (C.c_void_p * n)(*[C.addressof(scenes[k]) for k in range(n)])
    res = TuneResult()
    rc = L.dem_batch_autotune(ptrs, C.addressof(params), C.addressof(exts), n, device,
                              C.c_int64(sample_particles), trial_steps, C.byref(res))
    if rc != 0:
        raise DemError(rc, (L.dem_tune_last_error() or b"").decode())
    chosen = {"search_cell_factor": float(res.search_cell_factor), "list_skin": float(res.list_skin),
              "block_size": int(res.block_size), "reorder_interval": int(res.reorder_interval),
              "split_narrow": int(res.split_narrow), "unfused_lom": int(res.unfused_lom)}
    info = {"ms_per_step": res.ms_per_step, "default_ms_per_step": res.default_ms_per_step,
            "trials": int(res.trials), "sample_scenes": int(res.sample_scenes),
            "sample_particles": int(res.sample_particles), "seconds": res.seconds}
    return chosen, info


class SceneTable:
    """The dem_scene structs of [(scene index, scene dict), ...] in one array,
    as a C caller keeps them: pointers into the dicts' arrays, with the
    coll_cont and grid values of the moment it is built (build it again after
    replacing an array or changing those values).  Bulk calls accept it in
    place of the list, which spares re-marshalling hundreds of scenes."""

    def __init__(self, pairs):
        self.pairs = list(pairs)
        self.n = len(self.pairs)
        self.structs = (Scene * self.n)()
        for k, (_, sc) in enumerate(self.pairs):
            make_scene(sc, self.structs[k])
        self.idx = np.array([int(k) for k, _ in self.pairs], dtype=np.int32)
        self.ptrs = np.arange(self.n, dtype=np.uint64) * C.sizeof(Scene) + C.addressof(self.structs)

    def read_control(self):
        """coll_cont of every struct (written by a download) into its dict."""
        raw = np.frombuffer(self.structs, dtype=np.uint8).reshape(self.n, C.sizeof(Scene))
        off = Scene.coll_cont.offset
        cc = raw[:, off:off + 16].copy().view(np.int32)
        for k, (_, out) in enumerate(self.pairs):
            out["coll_cont"] = cc[k]


class Batch:
    """Many independent scenes resident on one GPU, stepped together
    (dem_batch_*).  `items` is a list of (scene, params, ext) triples as the
    dem_scenes builders return them; ext keys as for Context."""

    def __init__(self, items, *, device=-1, **world_kw):
        L = lib()
        self._keep = []
        n = len(items)
        scenes = (Scene * n)()
        params = (Params * n)()
        exts = (Ext * n)()
        self._templates = []
        for k, (sc, p, ext) in enumerate(items):
            kw = dict(world_kw)
            kw.update(ext)
            scenes[k] = make_scene(sc)
            params[k] = make_params(p)
            exts[k] = make_ext(keep=self._keep, **kw)
            self._templates.append({key: (v.copy() if hasattr(v, "copy") else v) for key, v in sc.items()
                                    if key in F32_KEYS + I32_KEYS + ("grid",)})
        self._keep.append((scenes, params, exts, [it[0] for it in items]))
        ptrs = (C.c_void_p * n)(*[C.addressof(scenes[k]) for k in range(n)])
        h = C.c_void_p()
        rc = L.dem_batch_create(ptrs, C.addressof(params), C.addressof(exts), n, device, C.byref(h))
        if rc != 0:
            raise DemError(rc, (L.dem_batch_last_error(None) or b"").decode())
        self.h = h
        self.n_scenes = n
        self.particles = [int(it[0]["radii"].shape[0]) for it in items]

    def close(self):
        if getattr(self, "h", None):
            lib().dem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise DemError(rc, (lib().dem_batch_last_error(self.h) or b"").decode())

    def step(self, n=1):
        self._check(lib().dem_batch_step(self.h, int(n)))

    def synchronize(self):
        self._check(lib().dem_batch_synchronize(self.h))

    def download(self, scene, out=None):
        out = empty_like_scene(self._templates[scene]) if out is None else out
        st = make_scene(out)
        self._check(lib().dem_batch_download(self.h, int(scene), C.byref(st)))
        out["coll_cont"] = np.array(st.coll_cont[:], dtype=np.int32)
        return out

    def upload(self, scene, sc):
        st = make_scene(sc)
        self._check(lib().dem_batch_upload(self.h, int(scene), C.byref(st)))

    def upload_many(self, pairs):
        """[(scene index, scene dict), ...] -- or a SceneTable of them -- in one
        call (dem_batch_upload_many)."""
        t = pairs if isinstance(pairs, SceneTable) else SceneTable(pairs)
        self._check(lib().dem_batch_upload_many(self.h, t.n, C.c_void_p(t.idx.ctypes.data),
                                                C.c_void_p(t.ptrs.ctypes.data)))

    def download_many(self, pairs):
        """[(scene index, scene dict to fill), ...] -- or a SceneTable of them --
        in one call (dem_batch_download_many)."""
        t = pairs if isinstance(pairs, SceneTable) else SceneTable(pairs)
        self._check(lib().dem_batch_download_many(self.h, t.n, C.c_void_p(t.idx.ctypes.data),
                                                  C.c_void_p(t.ptrs.ctypes.data)))
        t.read_control()

    def kernel_timing(self, on):
        """CUDA-event timing of every kernel kind (plain launches while on)."""
        L = lib()
        L.dem_batch_kernel_timing.argtypes = [C.c_void_p, C.c_int32]
        self._check(L.dem_batch_kernel_timing(self.h, 1 if on else 0))

    def kernel_time(self, kernel):
        """(total device ms, launches) of a kernel since kernel timing was enabled."""
        L = lib()
        L.dem_batch_kernel_time.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]
        ms = C.c_double(0.0)
        n = C.c_int64(0)
        self._check(L.dem_batch_kernel_time(self.h, kernel.encode(), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def record(self, scene, n_steps, selections):
        """dem_batch_record: Context.record for one scene (every scene steps)."""
        sel = np.ascontiguousarray(selections, dtype=np.int32)
        rows = np.zeros((max(int(n_steps), 1), 10), np.float64)
        rc = lib().dem_batch_record(self.h, int(scene), int(n_steps), sel.ctypes.data_as(_IP),
                                    rows.ctypes.data_as(C.POINTER(C.c_double)))
        if rc < 0:
            self._check(rc)
        return None if rc == 0 else rows[: int(n_steps)]

    def break_events(self, cap=1 << 18):
        buf = np.zeros(cap, dtype=BREAK_DTYPE)
        n = C.c_int32(0)
        self._check(lib().dem_batch_break_events(self.h, buf.ctypes.data, cap, C.byref(n)))
        return buf[: n.value].copy()

    def stats(self):
        s = Stats()
        self._check(lib().dem_batch_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_ if k != "reserved"}

    def stream(self):
        return lib().dem_batch_stream(self.h)


class Server:
    """Continuous batching of scene requests on one GPU (dem_server_*)."""

    def __init__(self, *, device=-1, memory_budget_bytes=None, max_active_particles=None,
                 max_scenes=None, cells_per_particle=None, bonds_per_particle=None, **ext_kw):
        L = lib()
        cfg = ServerConfig()
        L.dem_server_config_defaults(C.byref(cfg))
        if memory_budget_bytes is not None:
            cfg.memory_budget_bytes = int(memory_budget_bytes)
        if max_active_particles is not None:
            cfg.max_active_particles = int(max_active_particles)
        if max_scenes is not None:
            cfg.max_scenes = int(max_scenes)
        if cells_per_particle is not None:
            cfg.cells_per_particle = float(cells_per_particle)
        if bonds_per_particle is not None:
            cfg.bonds_per_particle = float(bonds_per_particle)
        self._keep = []
        cfg.ext = make_ext(keep=self._keep, **ext_kw)
        h = C.c_void_p()
        rc = L.dem_server_create(C.byref(cfg), device, C.byref(h))
        if rc != 0:
            raise DemError(rc, (L.dem_server_last_error(None) or b"").decode())
        self.h = h
        self._templates = {}

    def close(self):
        if getattr(self, "h", None):
            lib().dem_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise DemError(rc, (lib().dem_server_last_error(self.h) or b"").decode())

    def submit(self, scene, params, horizon, borrow=False, **ext_kw):
        """Queue a request; returns its id.  borrow=True (dem_server_submit_borrowed):
        the server refers to `scene`'s arrays instead of copying them, so they
        must stay unchanged until the request is polled done or cancelled."""
        keep = []
        st = make_scene(scene)
        p = make_params(params)
        e = make_ext(keep=keep, **ext_kw)
        rid = C.c_int64(0)
        fn = lib().dem_server_submit_borrowed if borrow else lib().dem_server_submit
        self._check(fn(self.h, C.byref(st), C.byref(p), C.byref(e), int(horizon), C.byref(rid)))
        if borrow:
            self._templates[rid.value] = scene   # the caller's arrays, also the result's shapes
        else:
            self._templates[rid.value] = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in scene.items()
                                          if k in F32_KEYS + I32_KEYS + ("grid",)}
        return rid.value

    def finish(self, rid):
        """Completion times (submit, admit, done) of a finished request, then
        release it without copying its result out."""
        times = (C.c_double * 3)()
        self._check(lib().dem_server_fetch(self.h, int(rid), None, times))
        self._check(lib().dem_server_release(self.h, int(rid)))
        self._templates.pop(rid, None)
        return times[0], times[1], times[2]

    def advance(self, n):
        self._check(lib().dem_server_advance(self.h, int(n)))

    def poll(self, cap=4096):
        ids = (C.c_int64 * cap)()
        n = C.c_int32(0)
        self._check(lib().dem_server_poll(self.h, ids, cap, C.byref(n)))
        return [ids[k] for k in range(n.value)]

    def fetch(self, rid, release=True):
        out = empty_like_scene(self._templates[rid])
        st = make_scene(out)
        times = (C.c_double * 3)()
        self._check(lib().dem_server_fetch(self.h, int(rid), C.byref(st), times))
        out["coll_cont"] = np.array(st.coll_cont[:], dtype=np.int32)
        ev = self.events(rid)
        if release:
            self._check(lib().dem_server_release(self.h, int(rid)))
            self._templates.pop(rid, None)
        return out, (times[0], times[1], times[2]), ev

    def cancel(self, rid):
        """Withdraw a queued, running or finished request (dem_server_cancel)."""
        self._check(lib().dem_server_cancel(self.h, int(rid)))
        self._templates.pop(rid, None)

    def release(self, rid):
        self._check(lib().dem_server_release(self.h, int(rid)))
        self._templates.pop(rid, None)

    def events(self, rid):
        n = C.c_int32(0)
        self._check(lib().dem_server_events(self.h, int(rid), None, 0, C.byref(n)))
        buf = np.zeros(max(n.value, 1), dtype=BREAK_DTYPE)
        self._check(lib().dem_server_events(self.h, int(rid), buf.ctypes.data, n.value, C.byref(n)))
        return buf[: n.value].copy()

    def stats(self):
        s = ServerStats()
        self._check(lib().dem_server_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def stream(self):
        return lib().dem_server_stream(self.h)


def grid_capacity(params, radii, particles):
    L = lib()
    r = np.ascontiguousarray(radii, dtype=np.float32)
    g = GridInfo()
    p = make_params(params)
    rc = L.dem_grid_capacity(C.byref(p), r.ctypes.data_as(_FP), int(r.shape[0]), int(particles),
                             C.byref(g))
    if rc != 0:
        raise DemError(rc, "grid_capacity")
    return (g.cell_size, g.cell_cap, g.w, g.h)
