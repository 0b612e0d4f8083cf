//! Raw bindings to `liblightgarden_cuda.so`, the GB300 trace-and-accumulate path of
//! light_garden (`include/lg.h`, C ABI version 5).
//!
//! The reference crate calls this in place of `Tracer::trace_all` (src/light_garden/tracer.rs:276)
//! and the wgpu line pass (src/sub_render_pass.rs:43-101): flatten the objects and lights into
//! `lg_geo` / `lg_object` / `lg_light` arrays, `lg_scene_upload` them when the scene changes, then
//! `lg_render` a frame into the Rgba16Float upload buffer.  Every struct here is `#[repr(C)]` with
//! the field order, types and padding of the header; check `lg_abi_version() == LG_ABI_VERSION`
//! once after loading, since a library of another version lays its structs out differently.
#![allow(non_camel_case_types)]
#![no_std]

use core::ffi::{c_char, c_void};

pub const LG_ABI_VERSION: u32 = 5;

pub type lg_status = i32;
pub const LG_OK: lg_status = 0;
pub const LG_ERR_INVALID_ARGUMENT: lg_status = 1;
pub const LG_ERR_UNSUPPORTED: lg_status = 2;
pub const LG_ERR_OUT_OF_MEMORY: lg_status = 3;
pub const LG_ERR_CUDA: lg_status = 4;
pub const LG_ERR_NO_SCENE: lg_status = 5;
pub const LG_ERR_TRUNCATED: lg_status = 6;
pub const LG_ERR_TIMEOUT: lg_status = 7;
pub const LG_ERR_BUDGET: lg_status = 8;
pub const LG_ERR_NOT_READY: lg_status = 9;
pub const LG_ERR_NOT_FOUND: lg_status = 10;

// lg_geo_kind
pub const LG_GEO_CIRCLE: i32 = 0;
pub const LG_GEO_RECT: i32 = 1;
pub const LG_GEO_SEGMENT: i32 = 2;
pub const LG_GEO_CUBIC: i32 = 3;
pub const LG_GEO_LOGIC: i32 = 4;
pub const LG_GEO_POLYGON: i32 = 5;
pub const LG_GEO_ELLIPSE: i32 = 6;
pub const LG_GEO_VERTICES: i32 = 7;
// lg_logic_op
pub const LG_OP_AND: i32 = 0;
pub const LG_OP_OR: i32 = 1;
pub const LG_OP_AND_NOT: i32 = 2;
// lg_object_kind
pub const LG_OBJ_STRAIGHT_MIRROR: i32 = 0;
pub const LG_OBJ_CURVED_MIRROR: i32 = 1;
pub const LG_OBJ_CIRCLE: i32 = 2;
pub const LG_OBJ_RECT: i32 = 3;
pub const LG_OBJ_LENS: i32 = 4;
pub const LG_OBJ_CONVEX_POLYGON: i32 = 5;
pub const LG_OBJ_ELLIPSE: i32 = 6;
pub const LG_OBJ_GEO: i32 = 7;
// lg_light_kind
pub const LG_LIGHT_POINT: i32 = 0;
pub const LG_LIGHT_DIRECTIONAL: i32 = 1;
pub const LG_LIGHT_SPOT: i32 = 2;
// lg_blend_factor
pub const LG_BF_ZERO: i32 = 0;
pub const LG_BF_ONE: i32 = 1;
pub const LG_BF_SRC: i32 = 2;
pub const LG_BF_ONE_MINUS_SRC: i32 = 3;
pub const LG_BF_SRC_ALPHA: i32 = 4;
pub const LG_BF_ONE_MINUS_SRC_ALPHA: i32 = 5;
pub const LG_BF_DST: i32 = 6;
pub const LG_BF_ONE_MINUS_DST: i32 = 7;
pub const LG_BF_DST_ALPHA: i32 = 8;
pub const LG_BF_ONE_MINUS_DST_ALPHA: i32 = 9;
pub const LG_BF_SRC_ALPHA_SATURATED: i32 = 10;
pub const LG_BF_CONSTANT: i32 = 11;
pub const LG_BF_ONE_MINUS_CONSTANT: i32 = 12;
// lg_blend_op
pub const LG_BO_ADD: i32 = 0;
pub const LG_BO_SUBTRACT: i32 = 1;
pub const LG_BO_REVERSE_SUBTRACT: i32 = 2;
pub const LG_BO_MIN: i32 = 3;
pub const LG_BO_MAX: i32 = 4;
// lg_accum_mode
pub const LG_ACCUM_FIXED64: i32 = 0;
pub const LG_ACCUM_F32: i32 = 1;
// lg_string_mod_mode
pub const LG_SM_ADD: u32 = 0;
pub const LG_SM_MUL: u32 = 1;
pub const LG_SM_POW: u32 = 2;
pub const LG_SM_BASE: u32 = 3;
// lg_string_mod_curve
pub const LG_CURVE_CIRCLE: u32 = 0;
pub const LG_CURVE_COMPLEX_EXP: u32 = 1;
pub const LG_CURVE_HYPOTROCHOID: u32 = 2;
pub const LG_CURVE_LISSAJOUS: u32 = 3;
pub const LG_STRING_MOD_NESTED_MAX: u32 = 4096;
// lg_precision
pub const LG_PRECISION_EXACT: i32 = 0;
pub const LG_PRECISION_FAST: i32 = 1;
// lg_path_flags
pub const LG_PATH_NEAR_DEGENERATE: u8 = 1;
pub const LG_PATH_TIR: u8 = 2;
pub const LG_PATH_FALLBACK: u8 = 4;
pub const LG_PATH_ILL_CONDITIONED: u8 = 8;
// lg_path_source
pub const LG_SRC_TRACE: u32 = 0;
pub const LG_SRC_CONTROL_LINE: u32 = 1;
pub const LG_SRC_STRING_MOD: u32 = 2;
// lg_culling
pub const LG_CULL_AUTO: i32 = 0;
pub const LG_CULL_OFF: i32 = 1;
pub const LG_CULL_ON: i32 = 2;
pub const LG_CULL_AUTO_MIN: u32 = 16;
pub const LG_CULL_WALK_MIN: u32 = 96;

#[repr(C)]
pub struct lg_ctx {
    _p: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_geo {
    pub kind: i32,
    pub op: i32,
    pub a: i32,
    pub b: i32,
    pub origin: [f64; 2],
    pub rot: [f64; 2],
    pub v: [f64; 8],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_object {
    pub kind: i32,
    pub geo: i32,
    pub has_material: i32,
    pub _pad: i32,
    pub refractive_index: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_light {
    pub kind: i32,
    pub num_rays: u32,
    pub color: [f32; 4],
    pub origin: [f64; 2],
    pub v: [f64; 2],
    pub spot_angle: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_blend_component {
    pub src_factor: i32,
    pub dst_factor: i32,
    pub op: i32,
}

/// ModRemColor (src/light_garden/string_mod.rs:167-172).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_mod_color {
    pub modulo: u64,
    pub rem: u64,
    pub color: [f32; 4],
}

/// StringMod (src/light_garden/string_mod.rs:4-15); `colors` is read during lg_scene_upload.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct lg_string_mod {
    pub modulo: u64,
    pub num: u64,
    pub turns: u64,
    pub mode: u32,
    pub curve: u32,
    pub color: [f32; 4],
    pub curve_f: [f64; 2],
    pub curve_u: [u64; 3],
    pub n_colors: u32,
    pub _pad: u32,
    pub colors: *const lg_mod_color,
    /// StringMod::nested: NULL, or the mod drawn between the crossings of this one's lines.
    pub nested: *const lg_string_mod,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct lg_params {
    pub max_bounce: u32,
    pub width: u32,
    pub height: u32,
    pub cutoff_color: [f32; 4],
    pub clear_color: [f32; 4],
    pub blend_constant: [f32; 4],
    pub color_blend: lg_blend_component,
    pub alpha_blend: lg_blend_component,
    pub accum: i32,
    pub emit_control_lines: i32,
    pub record_paths: i32,
    pub precision: i32,
    pub string_mod: lg_string_mod,
    pub ray_stride: u32,
    pub ray_offset: u32,
}

/// Two (P2, Color) vertices of the reference's line list with one colour.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_segment {
    pub x0: f32,
    pub y0: f32,
    pub x1: f32,
    pub y1: f32,
    pub color: [f32; 4],
}

/// One string-mod line: two vertices with their own colours (string_mod.rs:118-119).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_chord {
    pub x0: f32,
    pub y0: f32,
    pub x1: f32,
    pub y1: f32,
    pub color0: [f32; 4],
    pub color1: [f32; 4],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_path_record {
    pub path: u64,
    pub primary: u32,
    pub light: u16,
    pub gen: u8,
    pub flags: u8,
    pub hit: i32,
    pub source: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_trace_stats {
    pub primary_rays: u64,
    pub ray_visits: u64,
    pub segments: u64,
    pub fp64_solves: u64,
    pub fp64_fallbacks: u64,
    pub near_degenerate: u64,
    pub pixels: u64,
    pub tile_refs: u64,
    pub bound_tests: u64,
    pub object_tests: u64,
    pub retries: u32,
    pub _pad: u32,
    pub trace_ms: f32,
    pub accumulate_ms: f32,
    pub resolve_ms: f32,
    pub total_ms: f32,
    pub bin_ms: f32,
    pub raster_ms: f32,
    pub scan_ms: f32,
    pub solve_ms: f32,
    pub bounce_ms: f32,
    pub _pad2: f32,
    pub ill_conditioned: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_device_opts {
    pub device: i32,
    pub raster_variant: i32,
    pub segment_capacity: u64,
    pub queue_capacity: u64,
    pub stream_segments: u64,
    pub culling: i32,
    pub grid_density: f32,
    pub wait_polls: i32,
    pub scan_pairs: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct lg_scene_desc {
    pub geos: *const lg_geo,
    pub objects: *const lg_object,
    pub lights: *const lg_light,
    pub params: *const lg_params,
    pub n_geo: u32,
    pub n_objects: u32,
    pub n_lights: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_serve_opts {
    pub hbm_budget_bytes: u64,
    pub max_slots: u32,
    pub _pad: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct lg_serve_step_stats {
    pub admitted: u32,
    pub finished: u32,
    pub in_flight: u32,
    pub pending: u32,
    pub rasterised: u32,
    pub restarted: u32,
    pub live_rays: u64,
    pub segments: u64,
    pub step_ms: f32,
    pub _pad: u32,
}

extern "C" {
    pub fn lg_abi_version() -> u32;
    pub fn lg_params_default(p: *mut lg_params);
    pub fn lg_create(out: *mut *mut lg_ctx, opts_or_null: *const lg_device_opts) -> lg_status;
    pub fn lg_destroy(ctx: *mut lg_ctx) -> lg_status;
    pub fn lg_last_error(ctx_or_null: *const lg_ctx) -> *const c_char;
    pub fn lg_scene_upload(ctx: *mut lg_ctx, geos: *const lg_geo, n_geo: u32, objects: *const lg_object,
                           n_objects: u32, lights: *const lg_light, n_lights: u32,
                           params: *const lg_params) -> lg_status;
    pub fn lg_trace(ctx: *mut lg_ctx, stats_or_null: *mut lg_trace_stats) -> lg_status;
    pub fn lg_accumulate(ctx: *mut lg_ctx, stats_or_null: *mut lg_trace_stats) -> lg_status;
    pub fn lg_accumulate_segments(ctx: *mut lg_ctx, segments: *const lg_segment, n: u64,
                                  stats_or_null: *mut lg_trace_stats) -> lg_status;
    pub fn lg_resolve_f16(ctx: *mut lg_ctx, dst: *mut u16, pitch_bytes: usize, dst_is_device: i32) -> lg_status;
    pub fn lg_resolve_rgba8(ctx: *mut lg_ctx, dst: *mut u8, pitch_bytes: usize, dst_is_device: i32) -> lg_status;
    pub fn lg_render(ctx: *mut lg_ctx, dst: *mut u16, pitch_bytes: usize, dst_is_device: i32,
                     stats_or_null: *mut lg_trace_stats) -> lg_status;
    pub fn lg_segments_download(ctx: *mut lg_ctx, out: *mut lg_segment, paths_or_null: *mut lg_path_record,
                                cap: u64, n_out: *mut u64) -> lg_status;
    pub fn lg_accum_download(ctx: *mut lg_ctx, out: *mut c_void, cap_bytes: u64) -> lg_status;
    pub fn lg_chords_download(ctx: *mut lg_ctx, out: *mut lg_chord, cap: u64, n_out: *mut u64) -> lg_status;
    pub fn lg_batch_upload(ctx: *mut lg_ctx, scenes: *const lg_scene_desc, k: u32) -> lg_status;
    pub fn lg_batch_render(ctx: *mut lg_ctx, dst: *mut u16, dst_bytes: u64, dst_is_device: i32,
                           stats_or_null: *mut lg_trace_stats) -> lg_status;
    pub fn lg_batch_image_offset(ctx: *const lg_ctx, scene: u32, px_offset: *mut u64) -> lg_status;
    pub fn lg_serve_begin(ctx: *mut lg_ctx, opts: *const lg_serve_opts) -> lg_status;
    pub fn lg_serve_submit(ctx: *mut lg_ctx, scene: *const lg_scene_desc, id_out: *mut u64) -> lg_status;
    pub fn lg_serve_step(ctx: *mut lg_ctx, stats_or_null: *mut lg_serve_step_stats) -> lg_status;
    pub fn lg_serve_poll(ctx: *mut lg_ctx, id: u64, dst: *mut u16, dst_bytes: u64, dst_is_device: i32) -> lg_status;
    pub fn lg_serve_end(ctx: *mut lg_ctx) -> lg_status;
    pub fn lg_accumulate_segments_noalloc(segments: *const lg_segment, n: u64, params: *const lg_params,
                                          accum: *mut c_void, stream: *mut c_void,
                                          pixels_out: *mut u64) -> lg_status;
}
