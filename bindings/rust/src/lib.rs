//! Rust binding of the wrach GB300 C ABI (`include/wrach.h`).
//!
//! `WrachAPI` keeps the method names and data of the reference's
//! `runners/api` surface (`new`, `tick`, `read_data`, `add_particles`,
//! `positions`, `velocities`) over the CUDA library.  Written against the
//! header; this repository's image has no Rust toolchain to build it.

use std::ffi::CStr;
use std::os::raw::{c_char, c_int, c_void};

pub const WRACH_MODE_REFERENCE: u32 = 0;
pub const WRACH_MODE_EXTENDED: u32 = 1;

/// The reference's 32-byte uniform (`runners/bevy/src/config_shader.rs`).
#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct WrachWorldSettings {
    pub view_dimensions: [f32; 2],
    pub view_anchor: [f32; 2],
    pub grid_dimensions: [u32; 2],
    pub cell_size: u32,
    pub particles_in_frame_count: u32,
}

/// `WrachConfig` of `include/wrach.h` (80 bytes).
#[repr(C)]
#[derive(Clone, Copy, Default, Debug)]
pub struct WrachConfigC {
    pub width: f32,
    pub height: f32,
    pub anchor_x: f32,
    pub anchor_y: f32,
    pub cell_size: u32,
    pub mode: u32,
    pub iterations: u32,
    pub gravity: f32,
    pub min_distance: f32,
    pub max_velocity: f32,
    pub cell_capacity: u32,
    pub capacity: u32,
    pub device: i32,
    pub rebin_blocks: u32,
    pub solve_block: u32,
    pub solve_per_thread: u32,
    pub reserved: [u32; 4],
}

#[repr(C)]
pub struct WrachContext {
    _private: [u8; 0],
}

extern "C" {
    fn wrach_config_default(config: *mut WrachConfigC) -> c_int;
    fn wrach_create(config: *const WrachConfigC, out: *mut *mut WrachContext) -> c_int;
    fn wrach_destroy(ctx: *mut WrachContext) -> c_int;
    fn wrach_add_particles(ctx: *mut WrachContext, world: u32, pos: *const f32, vel: *const f32,
                           n: u32) -> c_int;
    fn wrach_step(ctx: *mut WrachContext, nsteps: u32) -> c_int;
    fn wrach_read(ctx: *mut WrachContext, world: u32, positions: *mut f32, velocities: *mut f32,
                  indices: *mut u32, capacity: u32) -> c_int;
    fn wrach_get_settings(ctx: *mut WrachContext, world: u32, out: *mut WrachWorldSettings) -> c_int;
    fn wrach_capacity(ctx: *mut WrachContext, world: u32) -> u32;
    fn wrach_last_error(ctx: *mut WrachContext) -> *const c_char;
    fn wrach_stream(ctx: *mut WrachContext) -> *mut c_void;
}

/// A non-zero status of the C ABI with the context's message.
#[derive(Debug)]
pub struct WrachError {
    pub code: i32,
    pub message: String,
}

fn check(ctx: *mut WrachContext, rc: c_int) -> Result<(), WrachError> {
    if rc == 0 {
        return Ok(());
    }
    let message = if ctx.is_null() {
        String::new()
    } else {
        unsafe { CStr::from_ptr(wrach_last_error(ctx)).to_string_lossy().into_owned() }
    };
    Err(WrachError { code: rc, message })
}

/// `WrachConfig` of `runners/bevy/src/config_app.rs`, same defaults.
#[derive(Clone, Copy, Debug)]
pub struct WrachConfig {
    pub dimensions: (u16, u16),
    pub boundaries_as_dimensions: bool,
    pub cell_size: u16,
}

impl Default for WrachConfig {
    fn default() -> Self {
        Self { dimensions: (480, 352), boundaries_as_dimensions: false, cell_size: 3 }
    }
}

/// `Particle` of `runners/bevy/src/state.rs`.
#[derive(Clone, Copy, Debug, Default)]
pub struct Particle {
    pub position: (f32, f32),
    pub velocity: (f32, f32),
}

/// Drop-in for `runners/api`'s `WrachAPI`.
pub struct WrachAPI {
    ctx: *mut WrachContext,
    pub positions: Vec<(f32, f32)>,
    pub velocities: Vec<(f32, f32)>,
    pub indices: Vec<u32>,
}

impl WrachAPI {
    pub fn new(config: WrachConfig) -> Self {
        Self::try_new(config).expect("wrach_create")
    }

    pub fn try_new(config: WrachConfig) -> Result<Self, WrachError> {
        let mut c = WrachConfigC::default();
        let mut ctx = std::ptr::null_mut();
        unsafe {
            wrach_config_default(&mut c);
            c.width = f32::from(config.dimensions.0);
            c.height = f32::from(config.dimensions.1);
            c.cell_size = u32::from(config.cell_size);
            check(ctx, wrach_create(&c, &mut ctx))?;
        }
        Ok(Self { ctx, positions: Vec::new(), velocities: Vec::new(), indices: Vec::new() })
    }

    /// One frame, then the readback (`runners/api/src/lib.rs:49-52`).
    pub fn tick(&mut self) {
        unsafe { check(self.ctx, wrach_step(self.ctx, 1)).expect("wrach_step") };
        self.read_data();
    }

    /// Positions and velocities, capacity long, zero-padded, cell order.
    pub fn read_data(&mut self) {
        unsafe {
            let cap = wrach_capacity(self.ctx, 0) as usize;
            let mut s = WrachWorldSettings::default();
            check(self.ctx, wrach_get_settings(self.ctx, 0, &mut s)).expect("wrach_get_settings");
            let cells = (s.grid_dimensions[0] as usize) * (s.grid_dimensions[1] as usize);
            self.positions = vec![(0.0, 0.0); cap];
            self.velocities = vec![(0.0, 0.0); cap];
            self.indices = vec![0; cells + 2];
            check(self.ctx, wrach_read(self.ctx, 0, self.positions.as_mut_ptr() as *mut f32,
                                       self.velocities.as_mut_ptr() as *mut f32,
                                       self.indices.as_mut_ptr(), cap as u32))
                .expect("wrach_read");
        }
    }

    pub fn add_particles(&mut self, particles: Vec<Particle>) {
        let pos: Vec<(f32, f32)> = particles.iter().map(|p| p.position).collect();
        let vel: Vec<(f32, f32)> = particles.iter().map(|p| p.velocity).collect();
        unsafe {
            check(self.ctx, wrach_add_particles(self.ctx, 0, pos.as_ptr() as *const f32,
                                                vel.as_ptr() as *const f32, pos.len() as u32))
                .expect("wrach_add_particles");
        }
    }

    pub fn get_simulation_state(&self) -> WrachWorldSettings {
        let mut s = WrachWorldSettings::default();
        unsafe { check(self.ctx, wrach_get_settings(self.ctx, 0, &mut s)).expect("settings") };
        s
    }

    /// The CUDA stream the context runs on.
    pub fn stream(&self) -> *mut c_void {
        unsafe { wrach_stream(self.ctx) }
    }
}

impl Drop for WrachAPI {
    fn drop(&mut self) {
        unsafe {
            wrach_destroy(self.ctx);
        }
    }
}

#[cfg(test)]
mod tests {
    use super::*;

    // runners/api/src/lib.rs:101-126, needs a GB300 and the library
    #[test]
    fn api_returns_data() {
        let mut wrach = WrachAPI::new(WrachConfig { dimensions: (10, 10), cell_size: 3, ..Default::default() });
        wrach.add_particles(vec![Particle { position: (5.0, 5.0), velocity: (0.5, 0.5) }; 3]);
        for _ in 0..5 {
            wrach.tick();
        }
        assert_eq!(wrach.positions.len(), 164);
        assert_ne!(wrach.positions[0], (0.0, 0.0));
    }
}
