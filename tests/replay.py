"""Replays the reference's experiment scripts to regenerate its exported traces.

Test infrastructure.  The experiment fixtures (tests/golden/*.bin) carry JSON
scripts (src/scripts.rs:20-347) that the reference's render loop executes;
their `Export` actions wrote the CSV traces in tests/golden/traces.npz.  This
module restates that loop closely enough to drive any backend (the CPU oracle
or the CUDA library) through the same action sequence:

  Client::render (client.rs:1106-1421): per frame, handle_events first
  (client.rs:829-908; `advance` at 931-960 when a script requested it), then the
  script threads (Thread::execute, scripts.rs:217-231, which run actions until a
  Wait), then `collect_data` at the end of the frame while recording
  (client.rs:1420-1421).
  advance() with gather_data: per tick one compute of one step, generation+1,
  collect_data; then one extra unrecorded compute (client.rs:944-952).
  collect_data: sim_time = timestep * generation in f32, then
  State::get_datum over the selected particles (state.rs:708-737).
  Backup = update_state + save (scripts.rs:318-321): pos, vel, acc, rot,
  rot_vel, rot_acc, forces, radii, fixity, bonds, contacts, material_pointers.
  Restore = State::load(init=false) + restore (scripts.rs:323-327,
  state.rs:583-706, wgpu_prog.rs:1235-1262): data and selections zeroed,
  del_pos <- vel, del_rot <- rot_vel; coll_cont is a device buffer and persists.
"""
import json

import numpy as np

PROP_NAMES = 14  # Boolean flags before the 10 floats, 3 fixity bools, 1 material


def prop_words(parameters):
    """Script Set_Properties parameters -> the 28-word uniform (scripts.rs:242-247, 828-836)."""
    w = np.zeros(28, dtype=np.int32)
    for i, p in enumerate(parameters):
        kind, (_, value) = next(iter(p.items()))
        if kind == "Boolean":
            w[i] = 1 if value else 0
        elif kind == "Integer":
            w[i] = int(value)
        elif kind == "Float":
            w[i] = np.array([value], dtype=np.float32).view(np.int32)[0]
        else:
            w[i] = np.array([-1.0], dtype=np.float32).view(np.int32)[0]
    return w


def datum(scene, selections):
    """State::get_datum (state.rs:708-737)."""
    sel = np.nonzero(selections)[0]
    if sel.size == 0:
        return None
    d = scene["data"].reshape(-1, 7).astype(np.float64)
    pos = scene["pos"].reshape(-1, 2).astype(np.float64)
    rot = scene["rot"].astype(np.float64)
    sums = np.zeros(10)
    for i in sel:
        sums += [pos[i, 0], pos[i, 1], d[i, 4], d[i, 5], rot[i], d[i, 6], abs(d[i, 0]),
                 d[i, 1], d[i, 2], d[i, 3]]
    for k in range(10):
        if k != 6:
            sums[k] /= sel.size
    return sums


BACKUP_KEYS = ("pos", "vel", "acc", "rot", "rot_vel", "rot_acc", "forces", "radii", "fixity",
               "bonds", "contacts", "material_pointers")


class Replayer:
    """Runs a fixture's auto-run script against a backend.

    backend API: download() -> scene dict; upload(scene); set_properties(sel, words);
    step(n); dt (float32 timestep).
    """

    def __init__(self, backend, scripts_json, n, long_wait_frames=1):
        self.b = backend
        self.scripts = json.loads(scripts_json)
        self.n = n
        self.long_wait_frames = long_wait_frames
        self.exports = {}

    def run(self, max_frames=100000):
        b = self.b
        scripts = self.scripts
        auto = [i for i, s in enumerate(scripts) if s.get("auto_run")]
        stack = [[auto[0], -1]] if auto else []
        selections = np.zeros(self.n, dtype=np.int32)
        generation = 0
        recording = False
        gather = False
        advance = None
        wait_frames = 0
        backup = None
        rows = []
        dt = np.float32(b.dt)

        def collect():
            nonlocal rows
            t = float(np.float32(dt * np.float32(generation)))
            dm = datum(b.download(), selections)
            if dm is None:
                rows = []
            else:
                rows.append([t] + list(dm))

        for _frame in range(max_frames):
            if not stack and advance is None:
                break
            advanced = False
            if advance is not None:
                ticks, advance = advance, None
                if gather and hasattr(b, "record"):
                    # the device record path: the same rows, read back once
                    data = b.record(ticks, selections)
                    if data is None:
                        rows = []
                    for j in range(ticks):
                        generation += 1
                        if data is not None:
                            rows.append([float(np.float32(dt * np.float32(generation)))] + list(data[j]))
                    b.step(1)
                elif gather:
                    for _ in range(ticks):
                        b.step(1)
                        generation += 1
                        collect()
                    b.step(1)
                else:
                    b.step(ticks)
                    generation += ticks
                advanced = True
            if wait_frames > 0:
                wait_frames -= 1
            while stack and wait_frames == 0:
                si, ai = stack[-1]
                acts = scripts[si]["actions"]
                if ai >= len(acts) - 1:
                    stack.pop()
                    continue
                ai += 1
                stack[-1][1] = ai
                if ai == len(acts) - 1:
                    stack.pop()
                act = acts[ai]
                name, params = act["name"], act["parameters"]
                val = [next(iter(p.values()))[1] for p in params]
                if name == "Backup":
                    sc = b.download()
                    backup = {k: sc[k].copy() for k in BACKUP_KEYS}
                elif name == "Restore":
                    sc = b.download()
                    for k in BACKUP_KEYS:
                        sc[k] = backup[k].copy()
                    sc["data"] = np.zeros_like(sc["data"])
                    sc["del_pos"] = sc["vel"].copy()
                    sc["del_rot"] = sc["rot_vel"].copy()
                    b.upload(sc)
                    selections = np.zeros(self.n, dtype=np.int32)
                    rows = []
                elif name == "Select":
                    lst = np.array(val[0], dtype=np.int32)
                    selections = np.zeros(self.n, dtype=np.int32)
                    selections[: min(self.n, lst.size)] = lst[: self.n]
                elif name == "Set_Properties":
                    selections = b.set_properties(selections, prop_words(params))
                elif name == "Call_Script":
                    stack.append([int(val[0]), -1])
                elif name == "Record":
                    recording = bool(val[0])
                    gather = bool(val[0])
                elif name == "Advance":
                    advance = int(val[0])
                elif name == "Wait":
                    wait_frames = 1 if float(val[0]) <= 0.01 else 1 + self.long_wait_frames
                    break
                elif name == "Export":
                    key = val[0].replace("\\", "/").split("/")[-1].rsplit(".", 1)[0]
                    self.exports[key] = np.array(rows, dtype=np.float64).reshape(-1, 11)
                elif name in ("None", "Select_All", "Simulate", "Goto"):
                    pass
                else:
                    raise NotImplementedError(name)
            if recording:
                collect()
            del advanced
        return self.exports


class OracleBackend:
    """Backend over the CPU oracle."""

    def __init__(self, scene, settings, use_f64):
        import oracle  # noqa: the oracle lives in oracle/, added to sys.path by conftest
        self.o = oracle
        self.scene = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in scene.items()}
        self.settings = dict(settings)
        self.use_f64 = use_f64
        self.dt = settings["dT"]
        self.events = []

    def download(self):
        return {k: (v.copy() if hasattr(v, "copy") else v) for k, v in self.scene.items()}

    def upload(self, scene):
        cc = self.scene["coll_cont"].copy()
        self.scene = {k: (v.copy() if hasattr(v, "copy") else v) for k, v in scene.items()}
        self.scene["coll_cont"] = cc

    def set_properties(self, selections, words):
        return self.o.set_properties(self.scene, selections, words)

    def step(self, n):
        ev, _ = self.o.step(self.scene, self.settings, n, use_f64=self.use_f64)
        if len(ev):
            self.events.append(ev)
