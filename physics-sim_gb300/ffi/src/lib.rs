//! Rust binding of libdemgb.so: the `extern "C"` block of include/dem.h and a
//! shim with the shape of the reference's `WGPUComputeProg` compute side
//! (src/wgpu_prog.rs:733-815 `new`, 1235-1262 `restore`, 1420-1473
//! `compute`; `State::update_state`, src/state.rs:264-289), so the
//! reference's `State` vectors (src/state.rs:69-93) and the 29-word
//! `Settings::collision_settings()` (src/settings.rs:2086-2119) pass through
//! unchanged.
//!
//! Every `#[repr(C)]` struct below lists the fields of its include/dem.h
//! counterpart in the same order with the same widths (checked against the
//! header by tests/test_ffi_crate.py).
#![allow(non_camel_case_types)]

use std::ffi::CStr;
use std::os::raw::{c_char, c_int, c_void};

pub const DEM_ABI_VERSION: c_int = 1;
pub const DEM_MAX_CONTACTS: usize = 14;
pub const DEM_DATA_SIZE: usize = 7;
pub const DEM_PROPS_WORDS: usize = 28;

pub const DEM_OK: c_int = 0;
pub const DEM_E_INVALID: c_int = -1;
pub const DEM_E_OOM: c_int = -2;
pub const DEM_E_CUDA: c_int = -3;
pub const DEM_E_TIMEOUT: c_int = -4;
pub const DEM_E_STATE: c_int = -5;
pub const DEM_E_UNSUPPORTED: c_int = -6;
pub const DEM_E_CAPACITY: c_int = -7;

pub const DEM_EVENT_FIX: i32 = 1;
pub const DEM_EVENT_DROP: i32 = 2;
pub const DEM_EVENT_RELEASE: i32 = 3;
pub const DEM_NOALLOC_MAX_CELLS: i32 = 262144;

/// The Settings uniform, 29 words in the order of collision_settings();
/// binary-identical to that `Vec<f32>`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_params {
    pub walls: i32,
    pub hor_bound: f32,
    pub vert_bound: f32,
    pub round_bounds: i32,
    pub bound_radius: f32,
    pub wall_friction: f32,
    pub gravity: i32,
    pub planet_mode: i32,
    pub bonds: i32,
    pub collisions: i32,
    pub friction_coefficient: f32,
    pub gravity_acc: f32,
    pub bond_normal_stiffness: f32,
    pub bonds_tear: i32,
    pub bond_normal_strength: f32,
    pub contact_damping: f32,
    pub bond_damping: f32,
    pub drag: f32,
    pub bond_shear_strength: f32,
    pub dT: f32,
    pub bond_shear_stiffness: f32,
    pub gravity_x: f32,
    pub gravity_y: f32,
    pub mouse_gravity: i32,
    pub moment_contribution_factor: f32,
    pub collision_interval: i32,
    pub local_damping: i32,
    pub local_damping_alpha: f32,
    pub particles: i32,
}

/// GridInfo of grid_info_buffer (wgpu_prog.rs:653-675).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_grid_info {
    pub cell_size: f32,
    pub cell_cap: i32,
    pub w: i32,
    pub h: i32,
}

/// Extensions; `dem_ext_defaults` gives the reference's behaviour.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct dem_ext {
    pub use_f64: i32,
    pub bond_lambda: f32,
    pub bond_normal_strength: *const f32,
    pub bond_shear_strength: *const f32,
    pub diagnostics: i32,
    pub reorder_interval: i32,
    pub block_size: i32,
    pub search_cell_factor: f32,
    pub event_capacity: i32,
    pub list_skin: f32,
    pub plain_launches: i32,
    pub split_narrow: i32,
    pub unfused_lom: i32,
    pub host_copies: i32,
    pub reorder_every: i32,
    pub restitution: f32,
}

/// One scene in the reference's host layouts.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct dem_scene {
    pub n_particles: i32,
    pub n_bonds: i32,
    pub n_materials: i32,
    pub pos: *mut f32,
    pub radii: *mut f32,
    pub vel: *mut f32,
    pub acc: *mut f32,
    pub rot: *mut f32,
    pub rot_vel: *mut f32,
    pub rot_acc: *mut f32,
    pub forces: *mut f32,
    pub fixity: *mut i32,
    pub del_pos: *mut f32,
    pub del_rot: *mut f32,
    pub bonds: *mut i32,
    pub contacts: *mut i32,
    pub material_pointers: *mut i32,
    pub materials: *mut f32,
    pub data: *mut f32,
    pub coll_cont: [i32; 4],
    pub grid: dem_grid_info,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_break_event {
    pub scene: i32,
    pub step: i32,
    pub bond: i32,
    pub code: i32,
    pub a: i32,
    pub b: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_stats {
    pub steps: i64,
    pub capped: i64,
    pub events: i64,
    pub events_dropped: i64,
    pub reorders: i64,
    pub device_error: i32,
    pub reserved: i32,
    pub kernel_launches: i64,
    pub list_overflows: i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_tune_result {
    pub search_cell_factor: f32,
    pub list_skin: f32,
    pub block_size: i32,
    pub reorder_interval: i32,
    pub ms_per_step: f64,
    pub default_ms_per_step: f64,
    pub trials: i32,
    pub sample_scenes: i32,
    pub sample_particles: i64,
    pub seconds: f64,
    pub split_narrow: i32,
    pub unfused_lom: i32,
    pub reserved: [i32; 6],
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct dem_server_config {
    pub memory_budget_bytes: i64,
    pub max_active_particles: i64,
    pub max_scenes: i32,
    pub cells_per_particle: f32,
    pub bonds_per_particle: f32,
    pub reserved: i32,
    pub ext: dem_ext,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct dem_server_stats {
    pub queued: i64,
    pub running: i64,
    pub completed: i64,
    pub active_particles: i64,
    pub particle_steps: i64,
    pub capacity_particles: i64,
    pub used_particles: i64,
    pub device_bytes: i64,
    pub steps: i64,
    pub waits_active: i64,
    pub waits_memory: i64,
}

/// Opaque handles.
#[repr(C)]
pub struct dem_ctx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct dem_batch {
    _p: [u8; 0],
}
#[repr(C)]
pub struct dem_server {
    _p: [u8; 0],
}

#[link(name = "demgb")]
extern "C" {
    pub fn dem_abi_version() -> c_int;
    pub fn dem_ext_defaults(ext: *mut dem_ext);
    pub fn dem_last_error(ctx: *const dem_ctx) -> *const c_char;
    pub fn dem_grid_capacity(p: *const dem_params, radii: *const f32, n_radii: i32, particles: i32,
                             out: *mut dem_grid_info) -> c_int;
    pub fn dem_create(scene: *const dem_scene, params: *const dem_params, ext: *const dem_ext, device: c_int,
                      out: *mut *mut dem_ctx) -> c_int;
    pub fn dem_destroy(ctx: *mut dem_ctx);
    pub fn dem_upload(ctx: *mut dem_ctx, scene: *const dem_scene) -> c_int;
    pub fn dem_set_params(ctx: *mut dem_ctx, params: *const dem_params) -> c_int;
    pub fn dem_set_materials(ctx: *mut dem_ctx, materials: *const f32, n_materials: i32) -> c_int;
    pub fn dem_set_control(ctx: *mut dem_ctx, coll_cont: *const i32) -> c_int;
    pub fn dem_get_control(ctx: *mut dem_ctx, coll_cont: *mut i32) -> c_int;
    pub fn dem_step(ctx: *mut dem_ctx, n_steps: i32) -> c_int;
    pub fn dem_synchronize(ctx: *mut dem_ctx) -> c_int;
    pub fn dem_download(ctx: *mut dem_ctx, out: *mut dem_scene) -> c_int;
    pub fn dem_set_properties(ctx: *mut dem_ctx, selections: *mut i32, props: *const i32) -> c_int;
    pub fn dem_break_events(ctx: *mut dem_ctx, buf: *mut dem_break_event, cap: i32, n: *mut i32) -> c_int;
    pub fn dem_get_stats(ctx: *mut dem_ctx, out: *mut dem_stats) -> c_int;
    pub fn dem_stream(ctx: *mut dem_ctx) -> *mut c_void;
    pub fn dem_event(ctx: *mut dem_ctx, kind: i32, selections: *mut i32, throw_particles: i32, del_x: f32,
                     del_y: f32, ticks: i32) -> c_int;
    pub fn dem_get_datum(ctx: *mut dem_ctx, selections: *const i32, out: *mut f64) -> c_int;
    pub fn dem_record(ctx: *mut dem_ctx, n_steps: i32, selections: *const i32, rows: *mut f64) -> c_int;

    pub fn dem_batch_create(scenes: *const *const dem_scene, params: *const dem_params, exts: *const dem_ext,
                            n_scenes: i32, device: c_int, out: *mut *mut dem_batch) -> c_int;
    pub fn dem_batch_destroy(b: *mut dem_batch);
    pub fn dem_batch_last_error(b: *const dem_batch) -> *const c_char;
    pub fn dem_batch_scene_count(b: *const dem_batch) -> c_int;
    pub fn dem_batch_step(b: *mut dem_batch, n_steps: i32) -> c_int;
    pub fn dem_batch_synchronize(b: *mut dem_batch) -> c_int;
    pub fn dem_batch_download(b: *mut dem_batch, scene: i32, out: *mut dem_scene) -> c_int;
    pub fn dem_batch_upload(b: *mut dem_batch, scene: i32, input: *const dem_scene) -> c_int;
    pub fn dem_batch_upload_many(b: *mut dem_batch, n: i32, idx: *const i32, input: *const *const dem_scene)
                                 -> c_int;
    pub fn dem_batch_download_many(b: *mut dem_batch, n: i32, idx: *const i32, out: *const *mut dem_scene)
                                   -> c_int;
    pub fn dem_batch_set_params(b: *mut dem_batch, scene: i32, params: *const dem_params) -> c_int;
    pub fn dem_batch_set_properties(b: *mut dem_batch, scene: i32, selections: *mut i32, props: *const i32)
                                    -> c_int;
    pub fn dem_batch_break_events(b: *mut dem_batch, buf: *mut dem_break_event, cap: i32, n: *mut i32) -> c_int;
    pub fn dem_batch_event(b: *mut dem_batch, scene: i32, kind: i32, selections: *mut i32, throw_particles: i32,
                           del_x: f32, del_y: f32, ticks: i32) -> c_int;
    pub fn dem_batch_get_datum(b: *mut dem_batch, scene: i32, selections: *const i32, out: *mut f64) -> c_int;
    pub fn dem_batch_record(b: *mut dem_batch, scene: i32, n_steps: i32, selections: *const i32, rows: *mut f64)
                            -> c_int;
    pub fn dem_batch_get_stats(b: *mut dem_batch, out: *mut dem_stats) -> c_int;
    pub fn dem_batch_stream(b: *mut dem_batch) -> *mut c_void;

    pub fn dem_batch_autotune(scenes: *const *const dem_scene, params: *const dem_params, exts: *const dem_ext,
                              n_scenes: i32, device: i32, sample_particles: i64, trial_steps: i32,
                              out: *mut dem_tune_result) -> c_int;
    pub fn dem_tune_last_error() -> *const c_char;

    pub fn dem_generate_bonds(pos: *const f32, radii: *const f32, n: i32, max_bonds: i32, device: i32,
                              bonds: *mut i32, bonds_cap: i64, n_bonds: *mut i64, contacts: *mut i32) -> c_int;
    pub fn dem_bondgen_last_error() -> *const c_char;

    pub fn dem_server_config_defaults(cfg: *mut dem_server_config);
    pub fn dem_server_create(cfg: *const dem_server_config, device: c_int, out: *mut *mut dem_server) -> c_int;
    pub fn dem_server_destroy(sv: *mut dem_server);
    pub fn dem_server_last_error(sv: *const dem_server) -> *const c_char;
    pub fn dem_server_submit(sv: *mut dem_server, scene: *const dem_scene, params: *const dem_params,
                             ext: *const dem_ext, horizon_steps: i64, request_id: *mut i64) -> c_int;
    pub fn dem_server_submit_borrowed(sv: *mut dem_server, scene: *const dem_scene, params: *const dem_params,
                                      ext: *const dem_ext, horizon_steps: i64, request_id: *mut i64) -> c_int;
    pub fn dem_server_advance(sv: *mut dem_server, n_steps: i32) -> c_int;
    pub fn dem_server_poll(sv: *mut dem_server, done_ids: *mut i64, cap: i32, n: *mut i32) -> c_int;
    pub fn dem_server_fetch(sv: *mut dem_server, id: i64, out: *mut dem_scene, times: *mut f64) -> c_int;
    pub fn dem_server_events(sv: *mut dem_server, id: i64, buf: *mut dem_break_event, cap: i32, n: *mut i32)
                             -> c_int;
    pub fn dem_server_release(sv: *mut dem_server, id: i64) -> c_int;
    pub fn dem_server_cancel(sv: *mut dem_server, id: i64) -> c_int;
    pub fn dem_server_get_stats(sv: *mut dem_server, out: *mut dem_server_stats) -> c_int;
    pub fn dem_server_stream(sv: *mut dem_server) -> *mut c_void;

    pub fn dem_broad_phase_noalloc(d_pos_radius: *const f32, n: i32, x0: f32, y0: f32, inv_cell: f32, gw: i32,
                                   gh: i32, d_keys: *mut i32, d_order: *mut i32, d_cell_start: *mut i32,
                                   stream: *mut c_void) -> c_int;
    pub fn dem_noalloc_last_error() -> *const c_char;
}

/// The reference's `State` arrays as the library reads and writes them.
/// Each slice keeps the reference's length (state.rs:69-93); `contacts` are
/// the f32 records viewed as their bit patterns.
pub struct StateArrays<'a> {
    pub pos: &'a mut [f32],
    pub radii: &'a mut [f32],
    pub vel: &'a mut [f32],
    pub acc: &'a mut [f32],
    pub rot: &'a mut [f32],
    pub rot_vel: &'a mut [f32],
    pub rot_acc: &'a mut [f32],
    pub forces: &'a mut [f32],
    pub fixity: &'a mut [i32],
    pub del_pos: &'a mut [f32],
    pub del_rot: &'a mut [f32],
    pub bonds: &'a mut [i32],
    pub contacts: &'a mut [f32],
    pub material_pointers: &'a mut [i32],
    pub materials: &'a mut [f32],
    pub data: &'a mut [f32],
    pub coll_cont: [i32; 4],
    pub grid: dem_grid_info,
}

impl<'a> StateArrays<'a> {
    /// The scene view of the arrays: plain pointers, the reference's layouts.
    pub fn scene(&mut self) -> dem_scene {
        let n = self.radii.len() as i32;
        dem_scene {
            n_particles: n,
            n_bonds: (self.bonds.len() / 3) as i32,
            n_materials: (self.materials.len() / 6) as i32,
            pos: self.pos.as_mut_ptr(),
            radii: self.radii.as_mut_ptr(),
            vel: self.vel.as_mut_ptr(),
            acc: self.acc.as_mut_ptr(),
            rot: self.rot.as_mut_ptr(),
            rot_vel: self.rot_vel.as_mut_ptr(),
            rot_acc: self.rot_acc.as_mut_ptr(),
            forces: self.forces.as_mut_ptr(),
            fixity: self.fixity.as_mut_ptr(),
            del_pos: self.del_pos.as_mut_ptr(),
            del_rot: self.del_rot.as_mut_ptr(),
            bonds: self.bonds.as_mut_ptr(),
            contacts: self.contacts.as_mut_ptr() as *mut i32,
            material_pointers: self.material_pointers.as_mut_ptr(),
            materials: self.materials.as_mut_ptr(),
            data: self.data.as_mut_ptr(),
            coll_cont: self.coll_cont,
            grid: self.grid,
        }
    }
}

/// A failed call: its DEM_E_* code and the library's message.
#[derive(Debug)]
pub struct DemError {
    pub code: c_int,
    pub message: String,
}

fn message(p: *const c_char) -> String {
    if p.is_null() {
        String::new()
    } else {
        unsafe { CStr::from_ptr(p) }.to_string_lossy().into_owned()
    }
}

/// The compute side of the reference's `WGPUComputeProg` on the GB300 path:
/// `new` creates the device state from `State` (WGPUComputeProg::new + the
/// buffer uploads), `restore` replaces it, `compute` enqueues one frame of
/// `gen_per_frame` LOM + Simulation steps and returns without waiting (like
/// `queue.submit`), `update_state` reads the whole state back into `State`'s
/// vectors.  `collision_settings` is `Settings::collision_settings()`: 29
/// words, passed as they are.
pub struct DemCompute {
    ctx: *mut dem_ctx,
}

impl DemCompute {
    pub fn new(state: &mut StateArrays, collision_settings: &[f32], device: i32) -> Result<DemCompute, DemError> {
        assert_eq!(collision_settings.len(), 29, "collision_settings() holds 29 words");
        let scene = state.scene();
        let mut ext = std::mem::MaybeUninit::<dem_ext>::uninit();
        let mut ctx: *mut dem_ctx = std::ptr::null_mut();
        let rc = unsafe {
            dem_ext_defaults(ext.as_mut_ptr());
            dem_create(&scene, collision_settings.as_ptr() as *const dem_params, ext.as_ptr(), device, &mut ctx)
        };
        if rc != DEM_OK {
            return Err(DemError { code: rc, message: message(unsafe { dem_last_error(std::ptr::null()) }) });
        }
        Ok(DemCompute { ctx })
    }

    fn check(&self, rc: c_int) -> Result<(), DemError> {
        if rc == DEM_OK {
            Ok(())
        } else {
            Err(DemError { code: rc, message: message(unsafe { dem_last_error(self.ctx) }) })
        }
    }

    /// WGPUComputeProg::compute (wgpu_prog.rs:1420-1473): re-upload the
    /// uniform when the settings changed, then gen_per_frame steps.
    pub fn compute(&mut self, collision_settings: &[f32], settings_changed: bool, gen_per_frame: i32)
                   -> Result<(), DemError> {
        if settings_changed {
            assert_eq!(collision_settings.len(), 29, "collision_settings() holds 29 words");
            self.check(unsafe { dem_set_params(self.ctx, collision_settings.as_ptr() as *const dem_params) })?;
        }
        self.check(unsafe { dem_step(self.ctx, gen_per_frame) })
    }

    /// WGPUComputeProg::restore (wgpu_prog.rs:1235-1262).
    pub fn restore(&mut self, state: &mut StateArrays) -> Result<(), DemError> {
        let scene = state.scene();
        self.check(unsafe { dem_upload(self.ctx, &scene) })
    }

    /// State::update_state (state.rs:264-289): waits for the enqueued steps.
    pub fn update_state(&mut self, state: &mut StateArrays) -> Result<(), DemError> {
        let mut scene = state.scene();
        self.check(unsafe { dem_download(self.ctx, &mut scene) })?;
        state.coll_cont = scene.coll_cont;
        Ok(())
    }

    /// The material buffer update (6 floats per material).
    pub fn set_materials(&mut self, materials: &[f32]) -> Result<(), DemError> {
        self.check(unsafe { dem_set_materials(self.ctx, materials.as_ptr(), (materials.len() / 6) as i32) })
    }

    /// Bond breaks since the last call, oldest first.
    pub fn break_events(&mut self) -> Result<Vec<dem_break_event>, DemError> {
        let mut buf = vec![dem_break_event::default(); 1 << 16];
        let mut n: i32 = 0;
        self.check(unsafe { dem_break_events(self.ctx, buf.as_mut_ptr(), buf.len() as i32, &mut n) })?;
        buf.truncate(n as usize);
        Ok(buf)
    }
}

impl Drop for DemCompute {
    fn drop(&mut self) {
        unsafe { dem_destroy(self.ctx) };
    }
}
