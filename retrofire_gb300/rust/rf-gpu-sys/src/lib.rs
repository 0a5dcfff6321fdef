//! Raw bindings of librfgpu's C ABI (include/rfgpu.h), for a Rust caller of
//! retrofire that renders on a GB300.  Every declaration mirrors the header
//! one for one; see the header for the meaning of each call.
//!
//! Not compiled here: neither this machine nor the GPU machine has a Rust
//! toolchain.  `tests/test_abi.py` checks that this file declares every
//! function the header declares.
#![allow(non_camel_case_types)]
#![no_std]

use core::ffi::{c_char, c_void};

pub type rf_status = i32;
pub type rf_mesh = u64;
pub type rf_texture = u64;
pub type rf_target = u64;

pub const RF_OK: rf_status = 0;
pub const RF_ERR_BAD_HANDLE: rf_status = 1;
pub const RF_ERR_BAD_ARG: rf_status = 2;
pub const RF_ERR_NON_POT_TEXTURE: rf_status = 3;
pub const RF_ERR_OOM: rf_status = 4;
pub const RF_ERR_OVER_BUDGET: rf_status = 5;
pub const RF_ERR_OVERFLOW: rf_status = 6;
pub const RF_ERR_TIMEOUT: rf_status = 7;
pub const RF_ERR_CUDA: rf_status = 8;
pub const RF_ERR_NO_DEVICE: rf_status = 9;

pub const RF_SHADER_FLAT: i32 = 0;
pub const RF_SHADER_GOURAUD: i32 = 1;
pub const RF_SHADER_TEXTURED: i32 = 2;
pub const RF_SHADER_TEX_GOURAUD: i32 = 3;
pub const RF_SHADER_GOURAUD_SRGB: i32 = 4;
pub const RF_SAMPLER_REPEAT_POT: u32 = 0;
pub const RF_SAMPLER_CLAMP: u32 = 1;
pub const RF_SAMPLER_ONCE: u32 = 2;
pub const RF_ARGB8888: i32 = 0;
pub const RF_XRGB8888: i32 = 1;
pub const RF_RGBA8888: i32 = 2;
pub const RF_BGRA8888: i32 = 3;
pub const RF_DEPTH_NONE: i32 = 0;
pub const RF_DEPTH_LESS: i32 = 1;
pub const RF_DEPTH_EQUAL: i32 = 2;
pub const RF_DEPTH_GREATER: i32 = 3;
pub const RF_CULL_NONE: i32 = 0;
pub const RF_CULL_BACK: i32 = 1;
pub const RF_CULL_FRONT: i32 = 2;
pub const RF_SORT_NONE: i32 = 0;
pub const RF_SORT_FRONT_TO_BACK: i32 = 1;
pub const RF_SORT_BACK_TO_FRONT: i32 = 2;
pub const RF_DRAW_CULL_BBOX: u32 = 1;
pub const RF_STAGE_N: usize = 5;
pub const RF_MAX_TARGET_DIM: u32 = 32768;
pub const RF_NOALLOC_MAX_TRIS: u32 = 1024;
pub const RF_NOALLOC_MAX_VERTS: u32 = 4096;
pub const RF_NOALLOC_MAX_W: u32 = 1024;
pub const RF_NOALLOC_MAX_H: u32 = 1024;
pub const RF_OBJ_POSITION: i32 = 0;
pub const RF_OBJ_NORMAL: i32 = 1;
pub const RF_OBJ_TEXCOORD: i32 = 2;
pub const RF_OBJ_NORMAL_TEXCOORD: i32 = 3;

#[repr(C)]
pub struct rf_ctx {
    _p: [u8; 0],
}
#[repr(C)]
pub struct rf_server {
    _p: [u8; 0],
}

#[repr(C)]
#[derive(Copy, Clone)]
pub struct rf_uniforms {
    pub mvp: [f32; 16],
    pub flat_rgba: u32,
    pub sampler: u32,
    pub texture: rf_texture,
}

#[repr(C)]
#[derive(Copy, Clone)]
pub struct rf_context_flags {
    pub depth_test: i32,
    pub color_write: i32,
    pub depth_write: i32,
    pub face_cull: i32,
    pub depth_sort: i32,
}

#[repr(C)]
#[derive(Copy, Clone, Default, Debug)]
pub struct rf_stats {
    pub calls: u64,
    pub prims_i: u64,
    pub prims_o: u64,
    pub verts_i: u64,
    pub verts_o: u64,
    pub frags_i: u64,
    pub frags_o: u64,
    pub oob: u64,
    pub objs_i: u64,
    pub objs_o: u64,
}

#[repr(C)]
#[derive(Copy, Clone)]
pub struct rf_draw {
    pub mesh: rf_mesh,
    pub shader: i32,
    pub flags: u32,
    pub uniforms: rf_uniforms,
}

#[repr(C)]
#[derive(Copy, Clone)]
pub struct rf_job {
    pub target: rf_target,
    pub ndraws: u32,
    pub draws: *const rf_draw,
    pub viewport: [f32; 16],
    pub flags: rf_context_flags,
}

#[repr(C)]
#[derive(Copy, Clone, Default)]
pub struct rf_server_config {
    pub hbm_budget_bytes: u64,
    pub max_batch: u32,
    pub inflight: u32,
    pub staging_bytes: u64,
    pub max_batch_tris: u64,
}

#[repr(C)]
#[derive(Copy, Clone)]
pub struct rf_request {
    pub ndraws: u32,
    pub draws: *const rf_draw,
    pub viewport: [f32; 16],
    pub flags: rf_context_flags,
    pub w: u32,
    pub h: u32,
    pub pixfmt: i32,
    pub has_depth: i32,
    pub clear_rgba: u32,
    pub depth_clear: f32,
    pub color_out: *mut u32,
    pub depth_out: *mut f32,
}

#[repr(C)]
#[derive(Copy, Clone, Default, Debug)]
pub struct rf_result {
    pub status: i32,
    pub batch_size: u32,
    pub batch_id: u64,
    pub queue_ms: f64,
    pub render_ms: f64,
    pub total_ms: f64,
    pub stats: rf_stats,
    pub gpu_start_ns: u64,
    pub gpu_end_ns: u64,
    pub pipeline: u32,
    pub reserved_: u32,
}

#[link(name = "rfgpu")]
extern "C" {
    // context
    pub fn rf_ctx_create(cuda_stream: *mut c_void, out: *mut *mut rf_ctx) -> rf_status;
    pub fn rf_ctx_destroy(ctx: *mut rf_ctx) -> rf_status;
    pub fn rf_ctx_device(ctx: *mut rf_ctx, device: *mut i32) -> rf_status;
    pub fn rf_ctx_sync(ctx: *mut rf_ctx) -> rf_status;
    pub fn rf_ctx_take_stats(ctx: *mut rf_ctx, out: *mut rf_stats) -> rf_status;
    pub fn rf_status_str(s: rf_status) -> *const c_char;
    pub fn rf_ctx_last_error(ctx: *const rf_ctx) -> *const c_char;
    pub fn rf_ctx_set_tiling(ctx: *mut rf_ctx, tile_w: u32, warps_per_block: u32) -> rf_status;
    pub fn rf_ctx_set_online_tuning(ctx: *mut rf_ctx, enable: i32) -> rf_status;
    pub fn rf_ctx_last_tiling(ctx: *mut rf_ctx, tile_w: *mut u32, warps: *mut u32) -> rf_status;
    pub fn rf_ctx_set_timing(ctx: *mut rf_ctx, enable: i32) -> rf_status;
    pub fn rf_ctx_stage_ms(ctx: *mut rf_ctx, out: *mut f64, frames: *mut u32) -> rf_status;
    pub fn rf_ctx_set_graphs(ctx: *mut rf_ctx, enable: i32) -> rf_status;
    pub fn rf_ctx_counts(
        ctx: *mut rf_ctx,
        kernels: *mut u64,
        graph_launches: *mut u64,
        graphs_cached: *mut u32,
    ) -> rf_status;
    pub fn rf_ctx_autotune(
        ctx: *mut rf_ctx,
        jobs: *const rf_job,
        njobs: u32,
        reps: u32,
        tile_w: *mut u32,
        warps: *mut u32,
        best_ms: *mut f32,
    ) -> rf_status;

    // resources
    pub fn rf_mesh_upload(
        ctx: *mut rf_ctx,
        verts: *const f32,
        nverts: u32,
        pos_dim: u32,
        nattr: u32,
        idx: *const u32,
        ntri: u32,
        out: *mut rf_mesh,
    ) -> rf_status;
    pub fn rf_mesh_update(ctx: *mut rf_ctx, mesh: rf_mesh, verts: *const f32, idx: *const u32) -> rf_status;
    pub fn rf_mesh_update_async(
        ctx: *mut rf_ctx,
        mesh: rf_mesh,
        verts: *const f32,
        idx: *const u32,
    ) -> rf_status;
    pub fn rf_mesh_info(
        ctx: *mut rf_ctx,
        mesh: rf_mesh,
        nverts: *mut u32,
        ntri: *mut u32,
        nattr: *mut u32,
    ) -> rf_status;
    pub fn rf_mesh_destroy(ctx: *mut rf_ctx, mesh: rf_mesh) -> rf_status;
    pub fn rf_texture_upload(
        ctx: *mut rf_ctx,
        rgba: *const u32,
        w: u32,
        h: u32,
        out: *mut rf_texture,
    ) -> rf_status;
    pub fn rf_texture_destroy(ctx: *mut rf_ctx, tex: rf_texture) -> rf_status;
    pub fn rf_target_create(
        ctx: *mut rf_ctx,
        w: u32,
        h: u32,
        pixfmt: i32,
        has_depth: i32,
        out: *mut rf_target,
    ) -> rf_status;
    pub fn rf_target_destroy(ctx: *mut rf_ctx, t: rf_target) -> rf_status;
    pub fn rf_target_clear(
        ctx: *mut rf_ctx,
        t: rf_target,
        clear_rgba: *const u32,
        depth_clear: *const f32,
    ) -> rf_status;
    pub fn rf_target_write(ctx: *mut rf_ctx, t: rf_target, color: *const u32, depth: *const f32) -> rf_status;
    pub fn rf_target_read(ctx: *mut rf_ctx, t: rf_target, color: *mut u32, depth: *mut f32) -> rf_status;
    pub fn rf_target_read_async(ctx: *mut rf_ctx, t: rf_target, color: *mut u32, depth: *mut f32) -> rf_status;

    // rendering
    pub fn rf_render(
        ctx: *mut rf_ctx,
        mesh: rf_mesh,
        shader: i32,
        uniforms: *const rf_uniforms,
        viewport: *const f32,
        target: rf_target,
        flags: *const rf_context_flags,
        stats: *mut rf_stats,
    ) -> rf_status;
    pub fn rf_render_draws(
        ctx: *mut rf_ctx,
        draws: *const rf_draw,
        ndraws: u32,
        viewport: *const f32,
        target: rf_target,
        flags: *const rf_context_flags,
        stats: *mut rf_stats,
    ) -> rf_status;
    pub fn rf_render_batch(ctx: *mut rf_ctx, jobs: *const rf_job, njobs: u32, stats: *mut rf_stats) -> rf_status;
    pub fn rf_lines_upload(
        ctx: *mut rf_ctx,
        verts: *const f32,
        nverts: u32,
        pos_dim: u32,
        nattr: u32,
        idx: *const u32,
        nlines: u32,
        out: *mut rf_mesh,
    ) -> rf_status;
    pub fn rf_render_lines(
        ctx: *mut rf_ctx,
        lines: rf_mesh,
        shader: i32,
        uniforms: *const rf_uniforms,
        viewport: *const f32,
        target: rf_target,
        flags: *const rf_context_flags,
        stats: *mut rf_stats,
    ) -> rf_status;
    pub fn rf_render_noalloc(
        verts: *const f32,
        nverts: u32,
        pos_dim: u32,
        nattr: u32,
        idx: *const u32,
        ntri: u32,
        shader: i32,
        mvp: *const f32,
        flat_rgba: u32,
        tex: *const u32,
        tw: u32,
        th: u32,
        sampler: u32,
        viewport: *const f32,
        color: *mut u32,
        depth: *mut f32,
        w: u32,
        h: u32,
        pixfmt: i32,
        flags: *const rf_context_flags,
        clear_rgba: *const u32,
        depth_clear: *const f32,
        cuda_stream: *mut c_void,
        stats: *mut rf_stats,
    ) -> rf_status;

    // OBJ ingestion (host only)
    pub fn rf_obj_parse(
        text: *const c_char,
        len: usize,
        attrs: i32,
        verts: *mut *mut f32,
        nverts: *mut u32,
        nattr: *mut u32,
        idx: *mut *mut u32,
        ntri: *mut u32,
        err: *mut c_char,
        err_len: usize,
    ) -> rf_status;
    pub fn rf_obj_free(p: *mut c_void);
    pub fn rf_mesh_load_obj(
        ctx: *mut rf_ctx,
        text: *const c_char,
        len: usize,
        attrs: i32,
        out: *mut rf_mesh,
    ) -> rf_status;

    // serving loop
    pub fn rf_server_create(
        ctx: *mut rf_ctx,
        cfg: *const rf_server_config,
        out: *mut *mut rf_server,
    ) -> rf_status;
    pub fn rf_server_submit(srv: *mut rf_server, req: *const rf_request, ticket: *mut u64) -> rf_status;
    pub fn rf_server_wait(srv: *mut rf_server, ticket: u64, timeout_ms: u32, out: *mut rf_result) -> rf_status;
    pub fn rf_server_counts(
        srv: *mut rf_server,
        batches: *mut u64,
        completed: *mut u64,
        queued: *mut u64,
    ) -> rf_status;
    pub fn rf_server_memory(
        srv: *mut rf_server,
        charged: *mut u64,
        peak_charged: *mut u64,
        peak_inflight: *mut u32,
    ) -> rf_status;
    pub fn rf_server_destroy(srv: *mut rf_server) -> rf_status;
}
