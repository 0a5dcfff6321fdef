/*
 * rfgpu.h — C ABI of the GB300 (sm_103a) triangle rendering library.
 *
 * Drop-in boundary for retrofire's rendering hot path.  The reference entry
 * point is the generic Rust function
 *
 *   pub fn render(prims, verts, shader: &Shd, uniform: Uni,
 *                 to_screen: Mat4<Ndc, Screen>, target: &mut impl Target,
 *                 ctx: &Context)                    core/src/render.rs:134-147
 *
 * which transforms vertices, clips against the view frustum, maps to the
 * viewport, culls, scan-converts and depth-tests into a Buf2 colour/depth
 * target on the CPU.  Here the same path runs as CUDA kernels on one GPU;
 * meshes, textures and targets are device-resident objects named by handle.
 * Results (coverage, depth, stats) are bit-identical to the reference; colour
 * is bit-identical except for RF_SHADER_GOURAUD_SRGB (powf, +-1 LSB).
 *
 * Threading: one rf_ctx per host thread; each rf_ctx is bound to one CUDA
 * stream and every call on it is ordered on that stream.  Nothing here traps
 * or panics on the device: out-of-range input is reported by status code or
 * counted in rf_stats.oob (the reference panics on those, buf.rs:444-449).
 */
#ifndef RFGPU_H
#define RFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t rf_status;
#define RF_OK 0
#define RF_ERR_BAD_HANDLE 1
#define RF_ERR_BAD_ARG 2
#define RF_ERR_NON_POT_TEXTURE 3 /* SamplerRepeatPot::new panics (tex.rs:227-233) */
#define RF_ERR_OOM 4
#define RF_ERR_OVER_BUDGET 5
#define RF_ERR_OVERFLOW 6
#define RF_ERR_TIMEOUT 7
#define RF_ERR_CUDA 8
#define RF_ERR_NO_DEVICE 9

typedef struct rf_ctx rf_ctx;
typedef uint64_t rf_mesh;
typedef uint64_t rf_texture;
typedef uint64_t rf_target;

/* Fixed shader family replacing the reference's closure shaders
 * (core/src/render/shader.rs:31-76).  Vertex side of every kind:
 * `vertex(mvp.apply(&v.pos), v.attrib)` (mat.rs:952-973), or the clip-space
 * passthrough `vertex(v.pos, v.attrib)` for meshes uploaded with pos_dim 4. */
enum {
    RF_SHADER_FLAT = 0,         /* attrib (): constant Color4 (benches/fill.rs:21-34) */
    RF_SHADER_GOURAUD = 1,      /* attrib Color3f: frag.var.to_color4() (color.rs:253-263) */
    RF_SHADER_TEXTURED = 2,     /* attrib TexCoord: sampler.sample(&tex, frag.var) (tex.rs) */
    RF_SHADER_TEX_GOURAUD = 3,  /* attrib (Color3f, TexCoord):
                                   (texel.to_rgb().to_color3f() * col).to_color4() */
    RF_SHADER_GOURAUD_SRGB = 4  /* attrib linear Color3f: frag.var.to_srgb().to_color4()
                                   (core/examples/hello_tri.rs:12-20) */
};
enum { RF_SAMPLER_REPEAT_POT = 0, RF_SAMPLER_CLAMP = 1, RF_SAMPLER_ONCE = 2 };
/* u32 colour formats, IntoPixel<u32, F> (util/pixfmt.rs:76-103). */
enum { RF_ARGB8888 = 0, RF_XRGB8888 = 1, RF_RGBA8888 = 2, RF_BGRA8888 = 3 };
/* Context::depth_test (ctx.rs:41-47): None, Some(Less), Some(Equal), Some(Greater). */
enum { RF_DEPTH_NONE = 0, RF_DEPTH_LESS = 1, RF_DEPTH_EQUAL = 2, RF_DEPTH_GREATER = 3 };
/* Context::face_cull (ctx.rs:21-27). */
enum { RF_CULL_NONE = 0, RF_CULL_BACK = 1, RF_CULL_FRONT = 2 };

/* The `uniform` argument of render() for the fixed shader family. */
typedef struct {
    float mvp[16];        /* ProjMat3<Model>, row-major like Matrix.0 (mat.rs:77-80) */
    uint32_t flat_rgba;   /* RF_SHADER_FLAT: Color4 bytes r,g,b,a, little-endian */
    uint32_t sampler;     /* RF_SAMPLER_* */
    rf_texture texture;   /* RF_SHADER_TEXTURED / RF_SHADER_TEX_GOURAUD */
} rf_uniforms;

/* Context::depth_sort (ctx.rs:39, render.rs:180-182, 209-219): None,
 * Some(FrontToBack), Some(BackToFront). */
enum { RF_SORT_NONE = 0, RF_SORT_FRONT_TO_BACK = 1, RF_SORT_BACK_TO_FRONT = 2 };

/* Context (ctx.rs:11-65) without the clears (rf_target_clear) and stats
 * (returned in rf_stats).  Context::default() == {LESS, 1, 1, BACK, NONE}.
 * depth_sort orders each render() call's clipped triangles by their mean
 * clip-space z (Render::depth, prim.rs:21-23) under f32::total_cmp before
 * setup, as depth_sort() does.  The reference sorts with sort_unstable_by,
 * whose order of equal keys is unspecified; here the sort is stable, so
 * triangles of equal depth keep their submission (and fan) order. */
typedef struct {
    int32_t depth_test;
    int32_t color_write;
    int32_t depth_write;
    int32_t face_cull;
    int32_t depth_sort;
} rf_context_flags;

/* Stats / Throughput (render/stats.rs:16-40).  oob counts scanlines that
 * left the target buffer (where the reference would panic).  objs_i /
 * objs_o: draws submitted with RF_DRAW_CULL_BBOX and those of them drawn
 * (Stats::objs as the per-object loop of demos/src/bin/crates.rs:114-133
 * keeps it). */
typedef struct {
    uint64_t calls, prims_i, prims_o, verts_i, verts_o, frags_i, frags_o, oob;
    uint64_t objs_i, objs_o;
} rf_stats;

/* One render() call for rf_render_draws (Batch::render, batch.rs:127-146).
 * flags: RF_DRAW_CULL_BBOX = object-level frustum culling of the
 * per-object loop (crates.rs:114-133): when the mesh's bounding box
 * (BBox::of its positions, render/scene.rs:37-39) is Hidden under the
 * draw's mvp (BBox::visibility, scene.rs:80-87: the 8 corners through the
 * vertex transform, their outcodes, view_frustum::status, clip.rs:245-267)
 * the draw is skipped like a render() call that was never made; every
 * other draw renders as without the flag.  Meshes with pos_dim 3 only. */
#define RF_DRAW_CULL_BBOX 1u
typedef struct {
    rf_mesh mesh;
    int32_t shader;
    uint32_t flags;
    rf_uniforms uniforms;
} rf_draw;

/* ---- context ---------------------------------------------------------- */
/* cuda_stream: a cudaStream_t to run on, or NULL for a new private stream.
 * Replaces the reference's implicit single thread (render.rs:134). */
rf_status rf_ctx_create(void *cuda_stream, rf_ctx **out);
rf_status rf_ctx_destroy(rf_ctx *ctx);
/* The CUDA device the context was created on (the caller's current device
 * at rf_ctx_create). */
rf_status rf_ctx_device(rf_ctx *ctx, int32_t *device);
/* Waits for all work queued on the context's streams (rendering and the
 * streaming copies). */
rf_status rf_ctx_sync(rf_ctx *ctx);
/* Adds the stats of every render since the last call into *out (and syncs). */
rf_status rf_ctx_take_stats(rf_ctx *ctx, rf_stats *out);
const char *rf_status_str(rf_status s);
/* The CUDA call and error message behind the context's last RF_ERR_CUDA or
 * RF_ERR_OOM ("" if none; "" for a NULL context).  Valid until the next call
 * on the context. */
const char *rf_ctx_last_error(const rf_ctx *ctx);
/* Tile raster tuning: tile width in pixels (8, 16, 32 or 64; tiles are 32
 * rows high) and rasteriser warps per block.  0 keeps the current value. */
rf_status rf_ctx_set_tiling(rf_ctx *ctx, uint32_t tile_w, uint32_t warps_per_block);
/* Online tiling (on by default until rf_ctx_set_tiling sets a tile width):
 * for each frame shape (draw, scene, vertex and triangle counts, target
 * pixels) the first frame is a warm-up, the next four run with tile widths
 * 8, 16, 32 and 64 while CUDA events time their GPU work, and every later
 * frame of that shape uses the fastest.  Results do not depend on the
 * width.  rf_ctx_last_tiling reports the last frame's width and warps. */
rf_status rf_ctx_set_online_tuning(rf_ctx *ctx, int32_t enable);
rf_status rf_ctx_last_tiling(rf_ctx *ctx, uint32_t *tile_w, uint32_t *warps);

/* Per-stage GPU timing (the device side of Stats::time, stats.rs:57-78).
 * When enabled, every render records CUDA events around its stages on the
 * context's stream; rf_ctx_stage_ms waits for the stream, adds the elapsed
 * milliseconds of every timed render since the last call into
 * out[0..RF_STAGE_N) and returns the number of renders timed in *frames. */
#define RF_STAGE_VERTEX 0
#define RF_STAGE_CLIP 1
#define RF_STAGE_SCAN 2
#define RF_STAGE_SETUP 3
#define RF_STAGE_RASTER 4
#define RF_STAGE_N 5
rf_status rf_ctx_set_timing(rf_ctx *ctx, int32_t enable);
rf_status rf_ctx_stage_ms(rf_ctx *ctx, double out[RF_STAGE_N], uint32_t *frames);

/* ---- resources (replace borrowed slices / Buf2s, render.rs:149-150) ---- */
/* verts: nverts * (pos_dim + nattr) floats, pos_dim 3 (Vertex3) or 4 (clip
 * space); idx: ntri * 3 u32 (Tri<usize>, geom/prim.rs:33). */
rf_status rf_mesh_upload(rf_ctx *ctx, const float *verts, uint32_t nverts, uint32_t pos_dim,
                         uint32_t nattr, const uint32_t *idx, uint32_t ntri, rf_mesh *out);
/* Replaces the contents of a mesh with arrays of the same sizes (an
 * animated or re-submitted mesh without reallocation). */
rf_status rf_mesh_update(rf_ctx *ctx, rf_mesh mesh, const float *verts, const uint32_t *idx);
/* Streaming variants: the copies run on the context's own upload / read-back
 * streams and return at once.  A render that reads the mesh waits for its
 * upload; an upload waits for every queued render that reads the mesh; a
 * read waits for every queued render into the target; the next render into
 * the target (or write, clear) waits for the read.  The host buffers must
 * stay valid (and, for a read, unread) until rf_ctx_sync; page-locked host
 * memory lets the copies overlap the rendering of other frames. */
rf_status rf_mesh_update_async(rf_ctx *ctx, rf_mesh mesh, const float *verts, const uint32_t *idx);
/* Sizes of a mesh; NULL pointers are skipped. */
rf_status rf_mesh_info(rf_ctx *ctx, rf_mesh mesh, uint32_t *nverts, uint32_t *ntri, uint32_t *nattr);
rf_status rf_mesh_destroy(rf_ctx *ctx, rf_mesh mesh);
/* rgba: w*h texels, Color4 bytes r,g,b,a little-endian, row-major
 * (Texture<Buf2<Color4>>, tex.rs:33-37). */
rf_status rf_texture_upload(rf_ctx *ctx, const uint32_t *rgba, uint32_t w, uint32_t h,
                            rf_texture *out);
rf_status rf_texture_destroy(rf_ctx *ctx, rf_texture tex);
/* Framebuf<Colorbuf<Buf2<u32>, pixfmt>, Buf2<f32>> (target.rs:35-44) when
 * has_depth, else a colour-only Colorbuf (target.rs:138-161).  Contents
 * start zeroed, like Buf2::new (buf.rs:155-161).  w, h <= RF_MAX_TARGET_DIM. */
#define RF_MAX_TARGET_DIM 32768u
rf_status rf_target_create(rf_ctx *ctx, uint32_t w, uint32_t h, int32_t pixfmt,
                           int32_t has_depth, rf_target *out);
rf_status rf_target_destroy(rf_ctx *ctx, rf_target t);
/* Frame::clear (front/src/lib.rs:103-120): colour <- into_pixel(*clear_rgba),
 * depth <- 1 / *depth_clear; NULL leaves that buffer alone.  The fill is
 * fused into the next render's tile loads. */
rf_status rf_target_clear(rf_ctx *ctx, rf_target t, const uint32_t *clear_rgba,
                          const float *depth_clear);
rf_status rf_target_write(rf_ctx *ctx, rf_target t, const uint32_t *color, const float *depth);
/* Copies the target to host memory (synchronous); NULL skips a buffer. */
rf_status rf_target_read(rf_ctx *ctx, rf_target t, uint32_t *color, float *depth);
/* See rf_mesh_update_async. */
rf_status rf_target_read_async(rf_ctx *ctx, rf_target t, uint32_t *color, float *depth);

/* ---- rendering -------------------------------------------------------- */
/* render(mesh.faces, mesh.verts, shader, uniforms, viewport, target, ctx)
 * (render.rs:134-207).  viewport: Mat4<Ndc, Screen>, row-major.  When stats
 * is non-NULL the call waits for the work queued before it and for its own,
 * and stores this call's stats alone (like `*ctx.stats.borrow_mut() +=
 * stats`, render.rs:206), which rf_ctx_take_stats then does not report
 * again; with NULL it only queues the work and the stats accumulate for
 * rf_ctx_take_stats. */
rf_status rf_render(rf_ctx *ctx, rf_mesh mesh, int32_t shader, const rf_uniforms *uniforms,
                    const float viewport[16], rf_target target, const rf_context_flags *flags,
                    rf_stats *stats);
/* ndraws consecutive render() calls into one target, in order, as one GPU
 * pass (the per-object submission idiom of demos/src/bin/crates.rs:114-133).
 * The result equals calling rf_render once per draw in order. */
rf_status rf_render_draws(rf_ctx *ctx, const rf_draw *draws, uint32_t ndraws,
                          const float viewport[16], rf_target target,
                          const rf_context_flags *flags, rf_stats *stats);

/* ---- line primitives ---------------------------------------------------
 * One render() call of Edge<usize> primitives (prim.rs:41-60): a line mesh
 * holds nlines vertex index pairs.  Lines are clipped like clip.rs:311-348,
 * never back-facing (face_cull FRONT drops them all, ctx.rs:95-101), drawn
 * one pixel per column or row by line() (raster.rs:115-173) with the first
 * vertex's depth and varyings, and counted like render() (render.rs:
 * 150-206).  A line longer than 2^22 pixels counts once in oob and is not
 * drawn.  Line meshes are rejected by the triangle entry points. */
rf_status rf_lines_upload(rf_ctx *ctx, const float *verts, uint32_t nverts, uint32_t pos_dim,
                          uint32_t nattr, const uint32_t *idx, uint32_t nlines, rf_mesh *out);
rf_status rf_render_lines(rf_ctx *ctx, rf_mesh lines, int32_t shader, const rf_uniforms *uniforms,
                          const float viewport[16], rf_target target, const rf_context_flags *flags,
                          rf_stats *stats);

/* ---- batched scenes ----------------------------------------------------
 * A scene = one target and the render() calls that draw into it, in order
 * (a frame of demos/src/bin/crates.rs:114-133).  rf_render_batch renders
 * njobs scenes as one pass of the pipeline: every stage runs once over the
 * triangles of all scenes and one persistent raster launch takes the tiles
 * of every target from a single queue.  The result for each scene equals
 * rf_render_draws on it alone.  A target may appear in at most one job of a
 * batch (RF_ERR_BAD_ARG otherwise).  stats: NULL queues the work (stats
 * accumulate for rf_ctx_take_stats), else njobs entries, one per scene,
 * stored after the batch completes. */
typedef struct {
    rf_target target;
    uint32_t ndraws;
    const rf_draw *draws;
    float viewport[16];       /* Mat4<Ndc, Screen> of the scene */
    rf_context_flags flags;
} rf_job;
rf_status rf_render_batch(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, rf_stats *stats);

/* CUDA-graph replay.  When enabled, the launch sequence of a frame is
 * captured once per frame shape (draw, job, vertex, triangle and tile
 * counts, tiling) and replayed with one graph launch when a frame of the
 * same shape comes again; the per-frame data (matrices, targets, clears)
 * are uploaded before the replay.  Stage timing (rf_ctx_set_timing) turns
 * replay off. */
rf_status rf_ctx_set_graphs(rf_ctx *ctx, int32_t enable);
/* Counters of the context so far: GPU kernels launched by the library
 * (directly or as graph nodes), graph launches, graphs cached.  NULL
 * pointers are skipped. */
rf_status rf_ctx_counts(rf_ctx *ctx, uint64_t *kernels, uint64_t *graph_launches,
                        uint32_t *graphs_cached);

/* Tiling autotuner: renders the batch with every tile width (8, 16, 32, 64)
 * and rasteriser warps per block (4, 8), reps timed runs each after a
 * warm-up, keeps the fastest on the context and returns it.  Every target
 * is snapshotted first and restored after each trial and at the end, and
 * the trials' stats are not reported, so the call leaves no trace but the
 * tiling. */
rf_status rf_ctx_autotune(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, uint32_t reps,
                          uint32_t *tile_w, uint32_t *warps, float *best_ms);

/* ---- rendering without device allocation ------------------------------
 * No counterpart in the reference: retrofire allocates freely on the CPU.
 * For callers that must not call cudaMalloc while rendering — a frame loop
 * held to a fixed, pre-reserved device-memory budget, or a plugin inside a
 * host application that owns every allocation and only lends the plugin the
 * buffers to read and fill.
 * One render() call like rf_render, but every buffer is the caller's device
 * memory (verts, idx, texture, colour, optional depth) and the temporaries
 * live in a fixed scratch area of RF_NOALLOC_SCRATCH_BYTES compiled into the
 * library, which every GPU that loads the library keeps until exit.  The
 * call allocates nothing.  Limits: ntri <= RF_NOALLOC_MAX_TRIS, nverts <=
 * RF_NOALLOC_MAX_VERTS, w <= RF_NOALLOC_MAX_W, h <= RF_NOALLOC_MAX_H;
 * larger inputs return RF_ERR_OVER_BUDGET.
 * The first call on a device looks up the scratch area's device address
 * (once per device, with that device current), so make that first call
 * before any stream capture; the address is kept until exit, so the call
 * must not be used on a device after cudaDeviceReset.  All calls share the
 * one area: calls whose GPU work overlaps race and give wrong results —
 * order them on one stream.  ntri > 0 with nverts == 0, and a depth_sort
 * other than RF_SORT_NONE, are RF_ERR_BAD_ARG.
 * clear_rgba / depth_clear (nullable) apply Frame::clear first.  stats,
 * when non-NULL, waits for the stream and receives this call's stats.
 * cuda_stream may be NULL (the legacy default stream). */
#define RF_NOALLOC_MAX_TRIS 1024u
#define RF_NOALLOC_MAX_VERTS 4096u
#define RF_NOALLOC_MAX_W 1024u
#define RF_NOALLOC_MAX_H 1024u
#define RF_NOALLOC_SCRATCH_BYTES (8u << 20)
rf_status rf_render_noalloc(const float *verts, uint32_t nverts, uint32_t pos_dim, uint32_t nattr,
                            const uint32_t *idx, uint32_t ntri, int32_t shader,
                            const float mvp[16], uint32_t flat_rgba, const uint32_t *tex,
                            uint32_t tw, uint32_t th, uint32_t sampler, const float viewport[16],
                            uint32_t *color, float *depth, uint32_t w, uint32_t h,
                            int32_t pixfmt, const rf_context_flags *flags,
                            const uint32_t *clear_rgba, const float *depth_clear,
                            void *cuda_stream, rf_stats *stats);

/* ---- mesh ingestion (Wavefront OBJ) -----------------------------------
 * retrofire's OBJ reader (geom/src/io.rs:106-370) as a host function: v,
 * vt, vn and f (triangles; quads split as [a,b,c], [a,c,d]); comments, g,
 * mtllib, usemtl and s skipped; any other item, a missing token, a bad
 * number, an out-of-range or zero index, a missing attribute kind or faces
 * that mix with and without normals/texcoords return RF_ERR_BAD_ARG with a
 * message in err.  Vertices are the distinct (position, texcoord, normal)
 * index triples in order of first use, like Mesh::new via the reader's
 * Builder.  attrs picks the vertex attributes: positions only (nattr 0),
 * normals (3), texcoords (2) or normal + texcoord (5).  *verts (nverts *
 * (3 + nattr) floats) and *idx (3 * ntri u32) are allocated by the library;
 * release them with rf_obj_free.  Needs no GPU. */
enum { RF_OBJ_POSITION = 0, RF_OBJ_NORMAL = 1, RF_OBJ_TEXCOORD = 2, RF_OBJ_NORMAL_TEXCOORD = 3 };
rf_status rf_obj_parse(const char *text, size_t len, int32_t attrs, float **verts, uint32_t *nverts,
                       uint32_t *nattr, uint32_t **idx, uint32_t *ntri, char *err, size_t err_len);
void rf_obj_free(void *p);
/* rf_obj_parse, then rf_mesh_upload of the result (positions in model
 * space, pos_dim 3). */
rf_status rf_mesh_load_obj(rf_ctx *ctx, const char *text, size_t len, int32_t attrs, rf_mesh *out);

/* ---- serving loop -----------------------------------------------------
 * No counterpart in the reference, which renders one frame per call on
 * the caller's thread (render.rs:134).  A server takes over an rf_ctx
 * whose meshes and textures are already uploaded.  Any thread submits
 * requests: a scene (draws on the context's meshes and textures, a
 * viewport, context flags), a target size and format, the Frame::clear
 * values and host buffers for the image.
 *
 * Continuous batching: the server runs `inflight` pipelines (default 2),
 * each a worker thread with its own CUDA stream, scratch arenas, pooled
 * targets and pre-sized page-locked staging, all reading the context's
 * meshes and textures.  Whenever a pipeline is free it takes, in arrival
 * order, the queued requests that fit what is left of the device-memory
 * budget (at most max_batch requests, max_batch_tris input triangles and
 * its staging room; the first always goes) and queues them as one
 * rf_render_batch, then their read-backs, on its stream; while it waits for
 * the GPU, the other pipelines admit the requests that arrived meanwhile,
 * so their work overlaps on the device.
 *
 * Admission: each request is charged an estimate of the device memory it
 * holds while in flight: its target, RF_SERVE_BYTES_PER_TRI per input
 * triangle and RF_SERVE_BYTES_PER_VERT per vertex of scratch, and its tile
 * masks (one bit per input triangle per 8x32-pixel tile).  A batch is
 * admitted while the charges of every batch in flight stay within the
 * budget; a request whose charge alone exceeds it is refused at submit
 * (RF_ERR_OVER_BUDGET).
 *
 * A request's image and stats equal rf_render_draws of its scene alone on a
 * cleared target, whatever batch or pipeline it lands in.  A request that
 * fails validation (bad handle, bad argument) fails alone.
 *
 * While a server runs, the context belongs to it: the caller makes no
 * other call on that context until rf_server_destroy, which drains the
 * queue, joins the workers and frees the pipelines (the context and its
 * meshes and textures stay the caller's). */
#define RF_SERVE_BYTES_PER_TRI 5632u
#define RF_SERVE_BYTES_PER_VERT 24u
typedef struct rf_server rf_server;
typedef struct {
    uint64_t hbm_budget_bytes; /* 0: 64 GiB */
    uint32_t max_batch;        /* requests per batch; 0: 256 */
    uint32_t inflight;         /* pipelines (batches in flight at once); 0: 2, at most 8 */
    uint64_t staging_bytes;    /* page-locked image staging per pipeline; 0: 256 MiB.  A
                                  request whose image is larger is read straight into
                                  its host buffers */
    uint64_t max_batch_tris;   /* input triangles per batch (the first request always
                                  goes); 0: 1,000,000 */
} rf_server_config;
typedef struct {
    uint32_t ndraws;
    const rf_draw *draws;      /* copied at submit */
    float viewport[16];
    rf_context_flags flags;
    uint32_t w, h;
    int32_t pixfmt;
    int32_t has_depth;
    uint32_t clear_rgba;       /* Color4 bytes r,g,b,a (Context::color_clear) */
    float depth_clear;         /* Context::depth_clear; the buffer gets 1/x */
    uint32_t *color_out;       /* host, w*h pixels, or NULL */
    float *depth_out;          /* host, w*h, or NULL (ignored without depth) */
} rf_request;
typedef struct {
    int32_t status;            /* the request's own status */
    uint32_t batch_size;       /* requests in the batch it was rendered in */
    uint64_t batch_id;
    double queue_ms;           /* submit -> its batch was admitted */
    double render_ms;          /* its batch on the GPU: gpu_end_ns - gpu_start_ns */
    double total_ms;           /* submit -> image in the host buffers */
    rf_stats stats;
    uint64_t gpu_start_ns;     /* GPU global timer when its batch's work began on the */
    uint64_t gpu_end_ns;       /* pipeline's stream, and when its rendering ended */
    uint32_t pipeline;         /* the pipeline that rendered it */
    uint32_t reserved_;
} rf_result;
rf_status rf_server_create(rf_ctx *ctx, const rf_server_config *cfg, rf_server **out);
/* Queues a request; *ticket identifies it for rf_server_wait.  The host
 * buffers must stay valid until the request completes. */
rf_status rf_server_submit(rf_server *srv, const rf_request *req, uint64_t *ticket);
/* Waits up to timeout_ms (UINT32_MAX: no limit) for a request; RF_OK and
 * its result, RF_ERR_TIMEOUT if still pending, RF_ERR_BAD_ARG for a ticket
 * that was never issued or was already collected. */
rf_status rf_server_wait(rf_server *srv, uint64_t ticket, uint32_t timeout_ms, rf_result *out);
/* Batches rendered, requests completed, requests queued right now. */
rf_status rf_server_counts(rf_server *srv, uint64_t *batches, uint64_t *completed, uint64_t *queued);
/* Admission charges of the batches in flight right now, the largest total
 * seen so far (never above the budget unless one request alone was), and
 * the most batches that were in flight at once.  NULL pointers are skipped. */
rf_status rf_server_memory(rf_server *srv, uint64_t *charged, uint64_t *peak_charged,
                           uint32_t *peak_inflight);
rf_status rf_server_destroy(rf_server *srv);

#ifdef __cplusplus
}
#endif
#endif
