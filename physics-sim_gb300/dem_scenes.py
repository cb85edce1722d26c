"""Scene setup for the DEM pipeline (the role of src/setup.rs, src/particle_def.rs
and the scene-building half of src/state.rs), plus the seeded synthetic
workloads the benchmark runs.

Every builder returns (scene, params, ext) where `scene` is a dict of numpy
arrays in the reference's host layouts (see dem.py), `params` the 29-word
settings dict, and `ext` keyword arguments for dem.Context (extensions such as
per-bond strengths).  Synthetic inputs stand in for the reference's saved
scenes: shapes, sizes and value distributions follow the workload definitions
quoted in each docstring.
"""
import numpy as np

MAX_CONTACTS = 14


def reference_defaults(particles):
    """Settings::new (src/settings.rs:257-439) packed as collision_settings()."""
    vert = np.float32(2.0)
    return {
        "walls": 1, "hor_bound": float(vert * np.float32(1.333)), "vert_bound": float(vert),
        "round_bounds": 0, "bound_radius": 1.0, "wall_friction": 0.0, "gravity": 1,
        "planet_mode": 1, "bonds": 0, "collisions": 1, "friction_coefficient": 0.5,
        "gravity_acc": 1.0, "bond_normal_stiffness": 10.0, "bonds_tear": 0,
        "bond_normal_strength": 0.5, "contact_damping": 0.2, "bond_damping": 0.2, "drag": 1.0,
        "bond_shear_strength": 0.5, "dT": float(np.float32(1.0 / 12600.0)),
        "bond_shear_stiffness": 10.0, "gravity_x": 0.0, "gravity_y": 0.0, "mouse_gravity": 0,
        "moment_contribution_factor": 1.0, "collision_interval": 1, "local_damping": 0,
        "local_damping_alpha": 0.1, "particles": int(particles),
    }


def empty_scene(n, materials):
    """A scene with n particles at rest, no contacts and no bonds (state.rs:98-118)."""
    materials = np.ascontiguousarray(materials, dtype=np.float32).reshape(-1)
    return {
        "pos": np.zeros(2 * n, np.float32), "radii": np.zeros(n, np.float32),
        "vel": np.zeros(2 * n, np.float32), "acc": np.zeros(2 * n, np.float32),
        "rot": np.zeros(n, np.float32), "rot_vel": np.zeros(n, np.float32),
        "rot_acc": np.zeros(n, np.float32), "forces": np.zeros(6 * n, np.float32),
        "fixity": np.zeros(6 * n, np.int32), "del_pos": np.zeros(2 * n, np.float32),
        "del_rot": np.zeros(n, np.float32), "bonds": np.full(1, -1, np.int32),
        "contacts": np.full(6 * MAX_CONTACTS * n, -1, np.int32),
        "material_pointers": np.zeros(n, np.int32), "materials": materials,
        "data": np.zeros(7 * n, np.float32), "coll_cont": np.zeros(4, np.int32),
        "grid": (0.0, 0, 0, 0),
    }


def grid_capacity(hor_bound, vert_bound, radii, particles):
    """grid_capacity (wgpu_prog.rs:698-717) over the radii, float32 arithmetic."""
    f = np.float32
    rmax = f(radii.max()) if radii.size else f(0)
    rmin = f(radii.min()) if radii.size else f(0)
    variable = rmin != rmax
    max_rad = rmax * f(2.0)
    min_rad = rmin if variable else rmax
    w = int(np.ceil(f(hor_bound) * f(2.0) / max_rad))
    h = int(np.ceil(f(vert_bound) * f(2.0) / max_rad))
    with np.errstate(divide="ignore", over="ignore"):
        q = max_rad / min_rad + f(1.0)
        capf = np.ceil(q * q)
    cap = int(min(capf, 2147483647.0)) if np.isfinite(capf) else 2147483647
    return (float(max_rad), min(cap, int(particles)) + 2, w, h)


def _bond_record(dx, dy):
    """Bond triple of regen_bonds (state.rs:308-314): status 1, atan2 angle, length."""
    dx = np.float32(dx)
    dy = np.float32(dy)
    mag = np.float32(np.power(np.float32(dx * dx + dy * dy), np.float32(0.5)))
    ang = np.float32(np.arctan2(np.float32(dx / mag), np.float32(dy / mag)))
    return 1, int(np.array([ang], np.float32).view(np.int32)[0]), int(np.array([mag], np.float32).view(np.int32)[0])


def add_straight_chain_bonds(scene, starts, lengths):
    """Vectorised add_chain_bonds for chains of consecutive indices
    [start, start + length): the same bond records and slot assignment as
    regen_bonds (state.rs:291-367) gives such chains (bond to the previous
    member in slot 0, to the next member in the first free slot)."""
    pos = scene["pos"].reshape(-1, 2)
    starts = np.asarray(starts, np.int64)
    lengths = np.asarray(lengths, np.int64)
    i_list = np.concatenate([np.arange(s0, s0 + ln - 1) for s0, ln in zip(starts, lengths)]) \
        if len(starts) else np.zeros(0, np.int64)
    i_list = np.sort(i_list)
    j_list = i_list + 1
    nb = i_list.size
    if nb == 0:
        scene["bonds"] = np.full(1, -1, np.int32)
        return scene
    dx = (pos[j_list, 0] - pos[i_list, 0]).astype(np.float32)
    dy = (pos[j_list, 1] - pos[i_list, 1]).astype(np.float32)
    mag = np.power((dx * dx + dy * dy).astype(np.float32), np.float32(0.5)).astype(np.float32)
    ang = np.arctan2((dx / mag).astype(np.float32), (dy / mag).astype(np.float32)).astype(np.float32)
    bonds = np.empty((nb, 3), np.int32)
    bonds[:, 0] = 1
    bonds[:, 1] = ang.view(np.int32)
    bonds[:, 2] = mag.view(np.int32)
    contacts = scene["contacts"].reshape(-1, MAX_CONTACTS, 6)
    k = np.arange(nb, dtype=np.int32)
    is_first = np.zeros(pos.shape[0], bool)
    is_first[starts] = True
    slot_i = np.where(is_first[i_list], 0, 1)
    contacts[i_list, slot_i, 0] = i_list
    contacts[i_list, slot_i, 1] = j_list
    contacts[i_list, slot_i, 2:5] = 0
    contacts[i_list, slot_i, 5] = k
    contacts[j_list, 0, 0] = j_list
    contacts[j_list, 0, 1] = i_list
    contacts[j_list, 0, 2:5] = 0
    contacts[j_list, 0, 5] = k
    scene["bonds"] = bonds.reshape(-1).copy()
    scene["contacts"] = contacts.reshape(-1).copy()
    return scene


def c3_mix_scene(n, bond_fraction, seed):
    """One scene of the batched mix: n particles, a fraction `bond_fraction`
    of them in horizontal bonded chains (radius 1, spacing 2, parallel bonds
    with bond radius factor 0.8, k_n 1e5, k_s 5e4, strengths Weibull(8, 5e3)),
    the rest loose disks (radii U[0.8, 1.2]) on a jittered lattice below them;
    gravity on, walls, contacts and dt as in c0_settle."""
    rng = np.random.default_rng(seed)
    n_chain = int(round(n * bond_fraction))
    chain_len = 32
    n_chains = n_chain // chain_len
    n_chain = n_chains * chain_len
    n_loose = n - n_chain
    # box: ~8 units^2 per particle, aspect 1:2 (c0_settle's density)
    W = float(np.ceil(np.sqrt(8.0 * n / 2.0)))
    W = max(W, 2.0 * chain_len + 8.0)
    H = max(8.0 * n / W, 40.0)
    H = float(np.ceil(H))
    pos = np.zeros((n, 2), np.float64)
    radii = np.ones(n, np.float32)
    # loose lattice in the lower part
    if n_loose > 0:
        spacing = 2.75
        cols = max(int((W - 2.6) // spacing), 1)
        idx = np.arange(n_loose)
        pos[:n_loose, 0] = (idx % cols - (cols - 1) / 2.0) * spacing + rng.uniform(-0.1, 0.1, n_loose)
        pos[:n_loose, 1] = -H / 2.0 + 1.4 + (idx // cols) * spacing + rng.uniform(-0.1, 0.1, n_loose)
        radii[:n_loose] = rng.uniform(0.8, 1.2, n_loose).astype(np.float32)
    top_loose = (pos[:n_loose, 1].max() + 1.3) if n_loose > 0 else -H / 2.0
    # chains in rows above
    starts = []
    if n_chains > 0:
        per_row = max(int((W - 4.0) // (2.0 * chain_len + 4.0)), 1)
        for c in range(n_chains):
            row, col = divmod(c, per_row)
            x0 = -W / 2.0 + 3.0 + col * (2.0 * chain_len + 4.0)
            y = top_loose + 4.0 + row * 4.0
            b0 = n_loose + c * chain_len
            pos[b0:b0 + chain_len, 0] = x0 + 2.0 * np.arange(chain_len)
            pos[b0:b0 + chain_len, 1] = y
            starts.append(b0)
        # a taller box for the chains: everything moves down with the floor,
        # so the loose lattice still starts 1.4 above it and lands at once
        H_new = max(H, 2.0 * (pos[:, 1].max() + 2.0))
        pos[:, 1] -= (H_new - H) / 2.0
        H = H_new
    sc = empty_scene(n, [1, 1, 1, 1.0, 1e5, 5e4])
    sc["pos"] = pos.astype(np.float32).reshape(-1)
    sc["radii"] = radii
    # chains: exact float positions first, then bonds from those positions
    add_straight_chain_bonds(sc, starts, [chain_len] * len(starts))
    p = reference_defaults(n)
    p.update({"hor_bound": W, "vert_bound": H, "planet_mode": 0, "gravity": 1, "gravity_acc": 1.0,
              "friction_coefficient": 0.5, "dT": 1e-4, "bonds": 3 if n_chains else 0,
              "bonds_tear": 1, "bond_normal_stiffness": 1e5, "bond_shear_stiffness": 5e4,
              "bond_normal_strength": 5e3, "bond_shear_strength": 5e3})
    sc["grid"] = grid_capacity(W, H, sc["radii"], n)
    ext = {"bond_lambda": 0.8}
    nb = sc["bonds"].shape[0] // 3
    if nb > 0:
        st = (5e3 * rng.weibull(8.0, size=(2, nb))).astype(np.float32)
        ext["bond_sn"], ext["bond_ss"] = st[0], st[1]
    return sc, p, ext


def c3_batch(n_scenes=512, seed=0, n_min=1000, n_max=64000, indices=None):
    """The batched mix: n_scenes scenes with log-uniform particle counts in
    [n_min, n_max] and bond fractions uniform in [0, 0.5], each seeded.
    `indices` builds only those scenes of the mix (the same scenes the whole
    mix holds at those positions)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), n_scenes)).astype(int)
    fr = rng.uniform(0.0, 0.5, n_scenes)
    ks = range(n_scenes) if indices is None else indices
    return [c3_mix_scene(int(ns[k]), float(fr[k]), seed * 100003 + k) for k in ks]


def add_chain_bonds(scene, chains):
    """Bonds and bonded contact slots for particle chains whose consecutive
    members are within 1.05 (r_i + r_j) and whose other pairs are not: the
    output of regen_bonds (state.rs:291-367) for such a layout, built in
    O(n).  `chains` is a list of index arrays in ascending order."""
    pos = scene["pos"].reshape(-1, 2)
    contacts = scene["contacts"].reshape(-1, MAX_CONTACTS, 6)
    pairs = []
    for ch in chains:
        ch = np.asarray(ch)
        pairs.extend(zip(ch[:-1].tolist(), ch[1:].tolist()))
    pairs.sort()
    bonds = np.zeros(3 * max(len(pairs), 1), np.int32)
    nxt = np.zeros(pos.shape[0], np.int64)
    for k, (i, j) in enumerate(pairs):
        d = pos[j] - pos[i]
        bonds[3 * k:3 * k + 3] = _bond_record(d[0], d[1])
        for a, b in ((i, j), (j, i)):
            s = nxt[a]
            contacts[a, s] = [a, b, 0, 0, 0, k]
            nxt[a] += 1
    if not pairs:
        bonds = np.full(1, -1, np.int32)
    scene["bonds"] = bonds
    scene["contacts"] = contacts.reshape(-1).copy()
    return scene


def c0_settle(n=4096, seed=0, box=(128.0, 256.0), spacing=None):
    """Plain granular settle: n disks, radii U[0.8, 1.2] (r0 = 1), a jittered
    square lattice (jitter U[-0.1, 0.1]) filling a 128 x 256 box with walls,
    gravity -9.81 (planet mode off, gravity_acc 1), density 1, k_n = 1e5,
    k_t = 0.5 k_n, friction 0.5, dt = 1e-4.  Wall restitution is the
    reference's fixed 0.5 (2D_LOM.wgsl:110-126)."""
    rng = np.random.default_rng(seed)
    W, H = float(box[0]), float(box[1])
    if spacing is None:
        s0 = np.sqrt(W * H / n)
        cols = int(np.floor(W / s0))
        rows = int(np.ceil(n / cols))
        spacing = min((W - 2.6) / cols, (H - 2.6) / rows)
    else:
        cols = max(int(np.floor((W - 2.6) / spacing)), 1)
        rows = int(np.ceil(n / cols))
    idx = np.arange(n)
    cx = (idx % cols) - (cols - 1) / 2.0
    cy = (idx // cols) - (rows - 1) / 2.0
    pos = np.empty((n, 2), np.float64)
    pos[:, 0] = cx * spacing + rng.uniform(-0.1, 0.1, n)
    pos[:, 1] = cy * spacing + rng.uniform(-0.1, 0.1, n)
    radii = rng.uniform(0.8, 1.2, n).astype(np.float32)
    mats = [1, 1, 1, 1.0, 1e5, 5e4]
    sc = empty_scene(n, mats)
    sc["pos"] = pos.astype(np.float32).reshape(-1)
    sc["radii"] = radii
    p = reference_defaults(n)
    p.update({"hor_bound": W, "vert_bound": H, "planet_mode": 0, "gravity": 1, "gravity_acc": 1.0,
              "friction_coefficient": 0.5, "dT": 1e-4, "bonds": 0})
    sc["grid"] = grid_capacity(W, H, radii, n)
    return sc, p, {}


def c1_chains(chains=64, length=256, seed=0, pull_velocity=0.1):
    """Bonded chain tensile test: `chains` independent chains of `length` disks
    of radius 1 at spacing 2 (touching), joined by parallel bonds (bond radius
    factor 0.8, k_n = 1e5, k_s = 0.5 k_n, tensile and shear strengths Weibull
    shape 8 scale 5e3 per bond); particle 0 of each chain fully fixed, the last
    one pulled along x at 0.01 per 1e3 steps of dt = 1e-4 (velocity 0.1) with its
    x DOF fixed; contacts as in c0_settle (no gravity)."""
    rng = np.random.default_rng(seed)
    n = chains * length
    gap = 6.0  # > 2 search cells between chains
    L = 2.0 * (length - 1)
    pos = np.zeros((n, 2), np.float32)
    for c in range(chains):
        base = c * length
        pos[base:base + length, 0] = (np.arange(length, dtype=np.float32) * np.float32(2.0)
                                      - np.float32(L / 2.0))
        pos[base:base + length, 1] = np.float32((c - (chains - 1) / 2.0) * gap)
    sc = empty_scene(n, [1, 1, 1, 1.0, 1e5, 5e4])
    sc["pos"] = pos.reshape(-1)
    sc["radii"] = np.ones(n, np.float32)
    add_chain_bonds(sc, [np.arange(c * length, (c + 1) * length) for c in range(chains)])
    fix = sc["fixity"].reshape(-1, 6)
    vel = sc["vel"].reshape(-1, 2)
    for c in range(chains):
        first, last = c * length, (c + 1) * length - 1
        fix[first, :] = 1
        fix[last, 0] = 1
        fix[last, 3] = 1
        vel[last, 0] = pull_velocity
    W = L + 40.0
    Hb = chains * gap + 20.0
    nb = sc["bonds"].shape[0] // 3
    strength = (5e3 * rng.weibull(8.0, size=(2, nb))).astype(np.float32)
    p = reference_defaults(n)
    p.update({"hor_bound": float(W), "vert_bound": float(Hb), "gravity": 0, "planet_mode": 0,
              "bonds": 3, "bonds_tear": 1, "bond_normal_stiffness": 1e5,
              "bond_shear_stiffness": 5e4, "bond_normal_strength": 5e3,
              "bond_shear_strength": 5e3, "dT": 1e-4, "friction_coefficient": 0.5})
    sc["grid"] = grid_capacity(W, Hb, sc["radii"], n)
    ext = {"bond_lambda": 0.8, "bond_sn": strength[0], "bond_ss": strength[1]}
    return sc, p, ext


def c2_impact(cols=1024, rows=4096, seed=0, projectile_radius=40.0, projectile_speed=50.0,
              bonded_fraction=0.3, cluster_min=4, cluster_max=32, sigma=0.15, projectiles=1):
    """Single large impact scene: cols x rows disks on a square lattice of
    pitch 2 (the default 1024 x 4096 = 4,194,304 disks fill a 2048 x 8192
    bed), radii log-normal with median 1 and log-sigma `sigma` (so lattice
    neighbours overlap where r_i + r_j > 2 and push apart from the first
    step), walls at the bed's sides and bottom; about `bonded_fraction` of the
    disks in horizontal clusters of cluster_min..cluster_max lattice
    neighbours joined by parallel bonds (bond radius factor 0.8, k_n 1e5,
    k_s 5e4, strengths Weibull(8, 5e3) per bond); one projectile disk of
    radius `projectile_radius` resting 0.3 into the bed's top row, moving
    down at `projectile_speed`; gravity, friction 0.5, k_n 1e5, k_s 5e4,
    dt 5e-5.  The projectile is the last particle; with projectiles > 1 they
    are the last ones, side by side, each 0.2 into its neighbour."""
    rng = np.random.default_rng(seed)
    nb = cols * rows
    n = nb + projectiles
    W = 2.0 * cols
    bed_h = 2.0 * rows
    H = bed_h + 4.0 * projectile_radius + 20.0
    pos = np.zeros((n, 2), np.float64)
    col = np.arange(nb) % cols
    row = np.arange(nb) // cols
    pos[:nb, 0] = (col - (cols - 1) / 2.0) * 2.0
    pos[:nb, 1] = -H / 2.0 + 1.0 + row * 2.0
    radii = np.exp(rng.normal(0.0, sigma, n)).astype(np.float32)
    radii[:nb] = np.minimum(radii[:nb], np.float32(W / 4.0))
    radii[nb:] = np.float32(projectile_radius)
    pitch = 2.0 * projectile_radius - 0.2
    for j in range(projectiles):
        pos[nb + j] = ((j - (projectiles - 1) / 2.0) * pitch, pos[:nb, 1].max() + 1.0 + projectile_radius - 0.3)
    # bonded clusters: each row cut into runs of cluster_min..cluster_max
    # consecutive columns, each run bonded with probability bonded_fraction
    per_row = cols // cluster_min + 1
    L = rng.integers(cluster_min, cluster_max + 1, size=(rows, per_row))
    c0 = np.cumsum(L, axis=1) - L
    pick = rng.random((rows, per_row)) < bonded_fraction
    ln = np.minimum(L, cols - c0)
    ok = (c0 < cols) & (ln >= 2) & pick
    rr, kk = np.nonzero(ok)
    starts = (rr * cols + c0[rr, kk]).astype(np.int64)
    lengths = ln[rr, kk].astype(np.int64)
    sc = empty_scene(n, [1, 1, 1, 1.0, 1e5, 5e4])
    sc["pos"] = pos.astype(np.float32).reshape(-1)
    sc["radii"] = radii
    sc["vel"].reshape(-1, 2)[nb:, 1] = -projectile_speed
    add_straight_chain_bonds(sc, starts, lengths)
    p = reference_defaults(n)
    p.update({"hor_bound": W + 2.0, "vert_bound": H, "planet_mode": 0, "gravity": 1, "gravity_acc": 1.0,
              "friction_coefficient": 0.5, "dT": 5e-5, "bonds": 3 if len(starts) else 0,
              "bonds_tear": 1, "bond_normal_stiffness": 1e5, "bond_shear_stiffness": 5e4,
              "bond_normal_strength": 5e3, "bond_shear_strength": 5e3})
    sc["grid"] = grid_capacity(p["hor_bound"], H, sc["radii"], n)
    ext = {"bond_lambda": 0.8}
    nbnd = sc["bonds"].shape[0] // 3
    if len(starts) and nbnd > 0:
        st = (5e3 * rng.weibull(8.0, size=(2, nbnd))).astype(np.float32)
        ext["bond_sn"], ext["bond_ss"] = st[0], st[1]
    return sc, p, ext


def dense_bed(n, seed=0, spacing=2.05, aspect=1.0):
    """A packed bed for contact-heavy runs: the c0_settle particle and material
    model on a jittered square lattice of the given spacing (radii U[0.8, 1.2],
    so about half of the lattice neighbours overlap from the first step),
    walls just outside the lattice."""
    cols = max(int(np.sqrt(n * aspect)), 1)
    rows = int(np.ceil(n / cols))
    W = cols * spacing + 2.6
    H = rows * spacing + 2.6
    return c0_settle(n=n, seed=seed, box=(W, H), spacing=spacing)
