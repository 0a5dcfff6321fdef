// rf_api.cu — the C ABI of include/rfgpu.h: handle tables, device arenas and
// the per-frame launch sequence of the render path.
//
// A frame = one or more "jobs" (a target plus its draws).  rf_render and
// rf_render_draws build one job; every draw is one reference render() call
// (core/src/render.rs:134-207) and the draws of a job are rendered in order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <unordered_map>
#include <vector>

#include "../../include/rfgpu.h"
#include "rf_ctx_internal.h"
#include "rf_internal.cuh"
#include "rf_kernels.cuh"

namespace {

struct Mesh {
    float *verts = nullptr;
    uint32_t *idx = nullptr;
    uint32_t nverts = 0, ntri = 0, pos_dim = 3, nattr = 0;  // ntri: lines of a line mesh
    bool lines = false;  // Edge<usize> primitives (index pairs), rf_render_lines
    // Device: BBox::of the positions (render/scene.rs:37-39), low x,y,z,
    // high x,y,z, computed after each upload; then the kernel's scratch
    // (RF_MESH_BBOX_FLOATS floats in all)
    float *bbox = nullptr;
    // Asynchronous updates (rf_mesh_update_async): `used` marks the last
    // render that read the mesh, `ready` the end of the last upload.
    bool async = false, ready_pending = false;
    cudaEvent_t used = nullptr, ready = nullptr;
};

// Every index below nverts (`vs[i]` panics past the vertices, prim.rs:17-19,
// 53-55).  A running maximum rather than an early exit, so the loop
// vectorises.
bool indices_ok(const uint32_t *idx, uint64_t n, uint32_t nverts) {
    uint32_t mx = 0;
    for (uint64_t i = 0; i < n; ++i) mx = idx[i] > mx ? idx[i] : mx;
    return n == 0 || mx < nverts;
}

struct Texture {
    uint32_t *texels = nullptr;
    uint32_t w = 0, h = 0;
};
struct Target {
    uint32_t *color = nullptr;
    float *depth = nullptr;
    uint32_t w = 0, h = 0;
    int32_t fmt = RF_ARGB8888;
    uint32_t clear_flags = 0;  // pending Frame::clear, fused into the next render
    uint32_t clear_px = 0;
    float clear_z = 0.0f;
    // Asynchronous reads (rf_target_read_async): `rendered` marks the last
    // work that wrote the target, `read_done` the end of the last read.
    bool async = false, read_pending = false;
    cudaEvent_t rendered = nullptr, read_done = nullptr;
};

// Mesh and texture tables by handle.
struct Resources {
    std::unordered_map<uint64_t, Mesh> meshes;
    std::unordered_map<uint64_t, Texture> textures;
};

// Grow-only device buffer.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

// An instantiated launch sequence and the frame shape it was captured for.
struct GraphKey {
    uint64_t v[13];
    bool operator==(const GraphKey &o) const { return memcmp(v, o.v, sizeof v) == 0; }
};
struct GraphEntry {
    GraphKey key;
    cudaGraphExec_t exec;
    uint64_t used;
};
constexpr size_t RF_GRAPH_CACHE = 8;

// Online tiling choice for one frame shape: one untimed warm-up frame, then
// one timed frame per tile width in RF_TUNE_TW, then the fastest width for
// every later frame of that shape.  All widths give identical results.
constexpr uint32_t RF_TUNE_TW[4] = {8, 16, 32, 64};
constexpr size_t RF_TUNE_CACHE = 512;  // frame shapes remembered (a per-frame loop over a few hundred scenes)
struct TuneState {
    uint64_t key[5];
    uint32_t next = 0;  // 0: warm-up, 1..4: timed RF_TUNE_TW[next-1], 5: decided
    int32_t tidx = -1;
    bool pending = false;
    float ms[4] = {0, 0, 0, 0};
    uint32_t best = 32;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

}  // namespace

struct rf_ctx {
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // Copy streams of the asynchronous uploads and read-backs (lazily made).
    cudaStream_t up = nullptr, down = nullptr;
    std::vector<Mesh *> async_meshes;  // async meshes of the frame being built
    int nsm = 1;
    int device = 0;
    uint32_t tile_w = 32, warps = 4;
    uint64_t next_handle = 1;
    // Meshes and textures: the context's own tables, or (a context made by
    // rfi_ctx_share for the serving loop) those of the context it shares
    // them with, read-only while shared.
    Resources own_res;
    Resources *res = &own_res;
    bool shared_res = false;
    std::unordered_map<uint64_t, Target> targets;
    // per-frame scratch
    DevBuf draws, jobs, cpos, coc, tcnt, toff, tpoly, pool, prims, mask, scan, counters, stats;
    DevBuf rowtot, rows, rprims, live, marks, items, jstats, clipq;
    DevBuf lrec, lmask;  // line pass
    // depth-sorted frames: sorted order, source triangles, per-draw counts,
    // sort scratch, the setup pass's draws / jobs, the raster's unit arrays
    DevBuf perm, ptri, nout, dsort, vdraws, vjobs, vtoff, vtcnt;
    uint32_t *nout_host = nullptr;  // pinned, grown with the draw count
    size_t nout_host_cap = 0;
    // CUDA graphs of the launch sequence, keyed by frame shape (graph mode).
    bool graphs = false;
    uint64_t gen = 0;  // bumped whenever a scratch buffer moves
    std::vector<GraphEntry> gcache;
    uint64_t gclock = 0, graph_launches = 0;
    uint64_t kernels = 0;  // kernels launched (directly or inside graphs)
    // Online tiling choice per frame shape (see tune_tile).
    bool tune_online = true;
    std::vector<TuneState> tunes;
    uint32_t last_tile_w = 0;
    // Row-record capacity (words): grown when a frame asked for more, which
    // the library learns from an asynchronous read-back of the total.
    uint64_t rows_cap = 0;
    unsigned long long *rows_need_host = nullptr;  // pinned
    cudaEvent_t rows_evt = nullptr;
    bool rows_evt_pending = false;
    // stats: host-side counts + device-accumulated counts, and what was
    // already handed out by rf_ctx_take_stats / rf_render
    rf_stats host_acc{};
    rf_stats taken{};
    char last_error[1024] = {0};  // the failing call (as written) and the CUDA message
    std::vector<DrawDev> hdraws;
    std::vector<JobDev> hjobs;
    // stage timing
    bool timing = false;
    std::vector<cudaEvent_t> ev_free;
    std::vector<std::vector<cudaEvent_t>> ev_pending;  // RF_STAGE_N + 1 events per render
    double stage_ms[RF_STAGE_N] = {0};
    uint32_t timed_frames = 0;
};

namespace {

rf_status cuda_fail(rf_ctx *c, cudaError_t e, const char *what) {
    if (c) snprintf(c->last_error, sizeof c->last_error, "%s: %s", what, cudaGetErrorString(e));
    // A failed call (an allocation, say) leaves the runtime's last-error
    // state set; the launches of a later call check that state, so clear it
    // here (a sticky error keeps failing every later call anyway).
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? RF_ERR_OOM : RF_ERR_CUDA;
}

#define CK(call)                                                  \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
    } while (0)

void graphs_drop(rf_ctx *ctx);

rf_status ensure(rf_ctx *ctx, DevBuf &b, size_t bytes) {
    if (bytes <= b.cap && b.p) return RF_OK;
    size_t cap = b.cap ? b.cap : 4096;
    while (cap < bytes) cap *= 2;
    // The old buffer may still be in use, and cached graphs point at it.
    CK(cudaStreamSynchronize(ctx->stream));
    graphs_drop(ctx);
    ctx->gen += 1;
    if (b.p) {
        CK(cudaFree(b.p));
        b.p = nullptr;
        b.cap = 0;
    }
    CK(cudaMalloc(&b.p, cap));
    b.cap = cap;
    return RF_OK;
}

rf_status copy_streams(rf_ctx *ctx) {
    if (!ctx->up) CK(cudaStreamCreateWithFlags(&ctx->up, cudaStreamNonBlocking));
    if (!ctx->down) CK(cudaStreamCreateWithFlags(&ctx->down, cudaStreamNonBlocking));
    return RF_OK;
}

// First asynchronous use of a mesh / target: its events, and a `used` /
// `rendered` mark covering every render queued so far.
rf_status make_async(rf_ctx *ctx, Mesh &m) {
    if (m.async) return RF_OK;
    CK(cudaEventCreateWithFlags(&m.used, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&m.ready, cudaEventDisableTiming));
    CK(cudaEventRecord(m.used, ctx->stream));
    m.async = true;
    return RF_OK;
}
rf_status make_async(rf_ctx *ctx, Target &t) {
    if (t.async) return RF_OK;
    CK(cudaEventCreateWithFlags(&t.rendered, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&t.read_done, cudaEventDisableTiming));
    CK(cudaEventRecord(t.rendered, ctx->stream));
    t.async = true;
    return RF_OK;
}
void drop_async(Mesh &m) {
    if (m.used) cudaEventDestroy(m.used);
    if (m.ready) cudaEventDestroy(m.ready);
    m.used = m.ready = nullptr;
}
void drop_async(Target &t) {
    if (t.rendered) cudaEventDestroy(t.rendered);
    if (t.read_done) cudaEventDestroy(t.read_done);
    t.rendered = t.read_done = nullptr;
}
// Work on the render stream that reads a mesh waits for its upload; work
// that writes a target waits for its read-back.
rf_status before_use(rf_ctx *ctx, Mesh &m) {
    if (m.ready_pending) {
        CK(cudaStreamWaitEvent(ctx->stream, m.ready, 0));
        m.ready_pending = false;
    }
    return RF_OK;
}
rf_status before_write(rf_ctx *ctx, Target &t) {
    if (t.read_pending) {
        CK(cudaStreamWaitEvent(ctx->stream, t.read_done, 0));
        t.read_pending = false;
    }
    return RF_OK;
}
rf_status sync_all(rf_ctx *ctx) {
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->up) CK(cudaStreamSynchronize(ctx->up));
    if (ctx->down) CK(cudaStreamSynchronize(ctx->down));
    return RF_OK;
}

template <class T>
T *P(DevBuf &b) {
    return reinterpret_cast<T *>(b.p);
}

bool is_pot(uint32_t x) { return x && !(x & (x - 1)); }

uint32_t nattr_for(int32_t shader) {
    switch (shader) {
        case RF_SHADER_FLAT: return 0;
        case RF_SHADER_TEXTURED: return 2;
        case RF_SHADER_TEX_GOURAUD: return 5;
        default: return 3;
    }
}

uint32_t pack_px(uint32_t c, int32_t fmt) {
    const uint32_t r = c & 0xFFu, g = (c >> 8) & 0xFFu, b = (c >> 16) & 0xFFu, a = c >> 24;
    switch (fmt) {
        case RF_ARGB8888: return (a << 24) | (r << 16) | (g << 8) | b;
        case RF_XRGB8888: return (r << 16) | (g << 8) | b;
        case RF_RGBA8888: return (r << 24) | (g << 16) | (b << 8) | a;
        default: return (b << 24) | (g << 16) | (r << 8) | a;
    }
}

void add_stats(rf_stats &a, const rf_stats &b) {
    a.calls += b.calls; a.prims_i += b.prims_i; a.prims_o += b.prims_o;
    a.verts_i += b.verts_i; a.verts_o += b.verts_o; a.frags_i += b.frags_i;
    a.frags_o += b.frags_o; a.oob += b.oob; a.objs_i += b.objs_i; a.objs_o += b.objs_o;
}

rf_stats sub_stats(const rf_stats &a, const rf_stats &b) {
    rf_stats d{};
    d.calls = a.calls - b.calls; d.prims_i = a.prims_i - b.prims_i; d.prims_o = a.prims_o - b.prims_o;
    d.verts_i = a.verts_i - b.verts_i; d.verts_o = a.verts_o - b.verts_o;
    d.frags_i = a.frags_i - b.frags_i; d.frags_o = a.frags_o - b.frags_o; d.oob = a.oob - b.oob;
    d.objs_i = a.objs_i - b.objs_i; d.objs_o = a.objs_o - b.objs_o;
    return d;
}

// Device stats + overflow counters + host counts = the running total.
rf_status read_totals(rf_ctx *ctx, rf_stats &tot) {
    StatsDev sd{};
    uint32_t cnt[RF_CNT_N] = {0};
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->stats.p) CK(cudaMemcpy(&sd, ctx->stats.p, sizeof sd, cudaMemcpyDeviceToHost));
    if (ctx->counters.p) CK(cudaMemcpy(cnt, ctx->counters.p, sizeof cnt, cudaMemcpyDeviceToHost));
    tot = ctx->host_acc;
    tot.prims_o += sd.prims_o;
    tot.verts_o += sd.verts_o;
    tot.frags_i += sd.frags_i;
    tot.frags_o += sd.frags_o;
    tot.oob += sd.oob + cnt[RF_CNT_POOLOVF] + cnt[RF_CNT_POLYOVF] + cnt[RF_CNT_BADIDX];
    // culled draws are render() calls that were not made
    tot.calls -= sd.cull_calls;
    tot.prims_i -= sd.cull_prims;
    tot.verts_i -= sd.cull_verts;
    tot.objs_i += sd.objs_i;
    tot.objs_o += sd.objs_o;
    return RF_OK;
}

rf_status init_stats(rf_ctx *ctx) {
    if (ctx->stats.p) return RF_OK;
    rf_status s = ensure(ctx, ctx->stats, sizeof(StatsDev));
    if (s) return s;
    s = ensure(ctx, ctx->counters, RF_CNT_N * 4);
    if (s) return s;
    CK(cudaMemsetAsync(ctx->stats.p, 0, sizeof(StatsDev), ctx->stream));
    CK(cudaMemsetAsync(ctx->counters.p, 0, RF_CNT_N * 4, ctx->stream));
    return RF_OK;
}

// One job of a frame: a target, its context flags and viewport, and the
// draws rendered into it in order.
struct JobIn {
    const rf_draw *draws = nullptr;
    uint32_t ndraws = 0;
    const float *vp = nullptr;
    Target *tg = nullptr;
    const rf_context_flags *fl = nullptr;
};

// Host-side counts of one job (render.rs:152-155) and its slot among the
// jobs that reach the GPU (-1: no triangles).
using JobHost = rfi_counts;

bool flags_ok(const rf_context_flags *fl) {
    return fl && fl->depth_test >= RF_DEPTH_NONE && fl->depth_test <= RF_DEPTH_GREATER &&
           fl->face_cull >= RF_CULL_NONE && fl->face_cull <= RF_CULL_FRONT &&
           fl->depth_sort >= RF_SORT_NONE && fl->depth_sort <= RF_SORT_BACK_TO_FRONT;
}

void graphs_drop(rf_ctx *ctx) {
    for (GraphEntry &g : ctx->gcache) cudaGraphExecDestroy(g.exec);
    ctx->gcache.clear();
}

// Word offsets of every job's tile masks and, after all of them, of the
// tiles' summary words (one bit per mask word); returns the words in all.
uint64_t layout_masks(std::vector<JobDev> &hj) {
    uint64_t w = 0;
    for (JobDev &J : hj) {
        J.mask_base = w;
        w += (uint64_t)J.tiles_x * J.tiles_y * J.mask_words;
    }
    for (JobDev &J : hj) {
        J.sum_words = (J.mask_words + 31) / 32;
        J.sum_base = w;
        w += (uint64_t)J.tiles_x * J.tiles_y * J.sum_words;
    }
    return w;
}

// Validates every draw of every job and fills ctx->hdraws / ctx->hjobs.
// Nothing is queued on the GPU and no state changes on failure.
rf_status build_jobs(rf_ctx *ctx, const JobIn *in, uint32_t nin, std::vector<JobHost> &host,
                     uint64_t &nv_out, uint64_t &nt_out) {
    auto &hd = ctx->hdraws;
    auto &hj = ctx->hjobs;
    hd.clear();
    hj.clear();
    ctx->async_meshes.clear();
    host.assign(nin, JobHost{});
    uint64_t nv = 0, nt = 0;
    uint64_t tiles = 0, mask_words = 0;
    const uint32_t TW = ctx->tile_w;
    for (uint32_t k = 0; k < nin; ++k) {
        const JobIn &ji = in[k];
        if (!ji.vp || !flags_ok(ji.fl) || !ji.tg || (ji.ndraws && !ji.draws)) return RF_ERR_BAD_ARG;
        const size_t d0 = hd.size();
        const uint64_t nt0 = nt, nv0 = nv;
        for (uint32_t i = 0; i < ji.ndraws; ++i) {
            const rf_draw &dr = ji.draws[i];
            auto mit = ctx->res->meshes.find(dr.mesh);
            if (mit == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
            Mesh &m = mit->second;
            if (m.lines) return RF_ERR_BAD_ARG;  // line meshes render with rf_render_lines
            if (m.async && !ctx->shared_res &&
                (ctx->async_meshes.empty() || ctx->async_meshes.back() != &m))
                ctx->async_meshes.push_back(&m);
            if (dr.shader < RF_SHADER_FLAT || dr.shader > RF_SHADER_GOURAUD_SRGB) return RF_ERR_BAD_ARG;
            if (m.nattr != nattr_for(dr.shader)) return RF_ERR_BAD_ARG;
            DrawDev d{};
            d.verts = m.verts;
            d.idx = m.idx;
            d.nverts = m.nverts;
            d.ntri = m.ntri;
            d.pos_dim = m.pos_dim;
            d.nattr = m.nattr;
            d.stride = m.pos_dim + m.nattr;
            d.shader = dr.shader;
            d.sampler = (int32_t)dr.uniforms.sampler;
            d.flat_rgba = dr.uniforms.flat_rgba;
            if (dr.shader == RF_SHADER_TEXTURED || dr.shader == RF_SHADER_TEX_GOURAUD) {
                auto tit = ctx->res->textures.find(dr.uniforms.texture);
                if (tit == ctx->res->textures.end()) return RF_ERR_BAD_HANDLE;
                if (d.sampler < RF_SAMPLER_REPEAT_POT || d.sampler > RF_SAMPLER_ONCE) return RF_ERR_BAD_ARG;
                if (d.sampler == RF_SAMPLER_REPEAT_POT && (!is_pot(tit->second.w) || !is_pot(tit->second.h)))
                    return RF_ERR_NON_POT_TEXTURE;
                d.tex = tit->second.texels;
                d.tw = tit->second.w;
                d.th = tit->second.h;
            }
            d.vert_base = (uint32_t)nv;
            d.tri_base = (uint32_t)nt;
            d.job = (uint32_t)hj.size();
            d.flags = dr.flags & RF_DRAW_CULL_BBOX;
            d.culled = 0;
            d.src_tri_base = (uint32_t)nt;
            d.bbox = m.bbox;
            memcpy(d.mvp, dr.uniforms.mvp, sizeof d.mvp);
            nv += m.nverts;
            nt += m.ntri;
            if (nv > 0xFFFFFFF0ull || nt > 0x7FFFFFF0ull) return RF_ERR_BAD_ARG;
            hd.push_back(d);
        }
        JobHost &h = host[k];
        h.calls = ji.ndraws;
        h.prims_i = nt - nt0;
        h.verts_i = nv - nv0;
        if (nt == nt0 || nv == nv0) {
            // Nothing to draw: a pending clear stays pending for the next read.
            hd.resize(d0);
            nt = nt0;
            nv = nv0;
            continue;
        }
        const Target &tg = *ji.tg;
        JobDev J{};
        J.color = tg.color;
        J.depth = tg.depth;
        J.w = tg.w;
        J.h = tg.h;
        J.pixfmt = tg.fmt;
        J.depth_test = ji.fl->depth_test;
        J.color_write = ji.fl->color_write;
        J.depth_write = ji.fl->depth_write;
        J.face_cull = ji.fl->face_cull;
        J.tiles_x = (tg.w + TW - 1) / TW;
        J.tiles_y = (tg.h + RF_TILE_H - 1) / RF_TILE_H;
        J.tile_base = (uint32_t)tiles;
        J.tri_base = (uint32_t)nt0;
        J.ntri = (uint32_t)(nt - nt0);
        J.mask_words = (J.ntri + 31) / 32;
        J.mask_base = mask_words;
        J.clear_flags = tg.clear_flags;
        J.clear_px = tg.clear_px;
        J.clear_z = tg.clear_z;
        J.depth_sort = ji.fl->depth_sort;
        memcpy(J.vp, ji.vp, sizeof J.vp);
        tiles += (uint64_t)J.tiles_x * J.tiles_y;
        mask_words += (uint64_t)J.tiles_x * J.tiles_y * J.mask_words;
        if (tiles > RF_MAX_TILES) return RF_ERR_BAD_ARG;
        h.slot = (int32_t)hj.size();
        hj.push_back(J);
    }
    layout_masks(hj);
    nv_out = nv;
    nt_out = nt;
    return RF_OK;
}

// Tile fields of every job for tile width TW (the jobs were built for
// another width).
rf_status retile(std::vector<JobDev> &hj, uint32_t TW) {
    uint64_t tiles = 0, mask_words = 0;
    for (JobDev &J : hj) {
        J.tiles_x = (J.w + TW - 1) / TW;
        J.tiles_y = (J.h + RF_TILE_H - 1) / RF_TILE_H;
        J.tile_base = (uint32_t)tiles;
        J.mask_base = mask_words;
        tiles += (uint64_t)J.tiles_x * J.tiles_y;
        mask_words += (uint64_t)J.tiles_x * J.tiles_y * J.mask_words;
        if (tiles > RF_MAX_TILES) return RF_ERR_BAD_ARG;
    }
    layout_masks(hj);
    return RF_OK;
}

// The tile width for this frame (online tuning) and, when the frame is a
// timed trial, the state whose events bracket its GPU work.
rf_status tune_tile(rf_ctx *ctx, const uint64_t key[5], uint32_t &TW, TuneState *&timed) {
    timed = nullptr;
    TW = ctx->tile_w;
    if (!ctx->tune_online) return RF_OK;
    TuneState *ts = nullptr;
    for (TuneState &t : ctx->tunes)
        if (memcmp(t.key, key, sizeof t.key) == 0) ts = &t;
    if (!ts) {
        if (ctx->tunes.size() >= RF_TUNE_CACHE) {
            CK(cudaStreamSynchronize(ctx->stream));
            for (TuneState &t : ctx->tunes) {
                if (t.e0) cudaEventDestroy(t.e0);
                if (t.e1) cudaEventDestroy(t.e1);
            }
            ctx->tunes.clear();
        }
        ctx->tunes.emplace_back();
        ts = &ctx->tunes.back();
        memcpy(ts->key, key, sizeof ts->key);
        CK(cudaEventCreate(&ts->e0));
        CK(cudaEventCreate(&ts->e1));
    }
    if (ts->pending) {
        CK(cudaEventSynchronize(ts->e1));
        float ms = 0.0f;
        CK(cudaEventElapsedTime(&ms, ts->e0, ts->e1));
        ts->ms[ts->tidx] = ms;
        ts->pending = false;
    }
    if (ts->next == 0) {
        TW = RF_TUNE_TW[0];
        ts->next = 1;
    } else if (ts->next <= 4) {
        ts->tidx = (int32_t)ts->next - 1;
        TW = RF_TUNE_TW[ts->tidx];
        ts->next += 1;
        timed = ts;
    } else {
        if (ts->next == 5) {
            uint32_t b = 0;
            for (uint32_t i = 1; i < 4; ++i)
                if (ts->ms[i] < ts->ms[b]) b = i;
            ts->best = RF_TUNE_TW[b];
            ts->next = 6;
        }
        TW = ts->best;
    }
    return RF_OK;
}

// One frame: the jobs of `in` (distinct targets), each with its draws in
// order, as one pass of the pipeline over all of them.  per_job: kernels
// count into per-job slots (ctx->jstats), folded into the running total at
// the end of the pass; otherwise (a single job) straight into the total.
rf_status run_jobs(rf_ctx *ctx, const JobIn *in, uint32_t nin, bool per_job,
                   std::vector<JobHost> &host) {
    rf_status st = init_stats(ctx);
    if (st) return st;
    uint64_t nv = 0, nt = 0;
    if ((st = build_jobs(ctx, in, nin, host, nv, nt))) return st;
    auto &hd = ctx->hdraws;
    auto &hj = ctx->hjobs;
    for (const JobHost &h : host) {
        ctx->host_acc.calls += h.calls;
        ctx->host_acc.prims_i += h.prims_i;
        ctx->host_acc.verts_i += h.verts_i;
    }
    if (hj.empty()) return RF_OK;
    const uint32_t nj = (uint32_t)hj.size();
    if (nj > 1) per_job = true;
    uint32_t TW = ctx->tile_w;
    TuneState *tuned = nullptr;
    {
        uint64_t px = 0;
        for (const JobDev &J : hj) px += (uint64_t)J.w * J.h;
        const uint64_t key[5] = {hd.size(), nj, nv, nt, px};
        if ((st = tune_tile(ctx, key, TW, tuned))) return st;
        if (TW != ctx->tile_w && (st = retile(hj, TW))) return st;
    }
    ctx->last_tile_w = TW;
    const JobDev &JL = hj.back();
    const uint32_t ntiles = JL.tile_base + JL.tiles_x * JL.tiles_y;
    const size_t mask_words = JL.sum_base + (size_t)JL.tiles_x * JL.tiles_y * JL.sum_words;  // masks + summaries
    const uint32_t ndraws = (uint32_t)hd.size();

    if ((st = ensure(ctx, ctx->draws, hd.size() * sizeof(DrawDev)))) return st;
    if ((st = ensure(ctx, ctx->jobs, hj.size() * sizeof(JobDev)))) return st;
    if (per_job && (st = ensure(ctx, ctx->jstats, hj.size() * sizeof(StatsDev)))) return st;
    if ((st = ensure(ctx, ctx->cpos, nv * sizeof(float4)))) return st;
    if ((st = ensure(ctx, ctx->coc, nv))) return st;
    if ((st = ensure(ctx, ctx->tcnt, nt * 4))) return st;
    if ((st = ensure(ctx, ctx->toff, nt * 4))) return st;
    if ((st = ensure(ctx, ctx->tpoly, nt * 4))) return st;
    if ((st = ensure(ctx, ctx->clipq, nt * 4))) return st;
    const uint32_t pool_cap = (uint32_t)nt;
    if ((st = ensure(ctx, ctx->pool, (size_t)pool_cap * RF_POLY_STORE * sizeof(PolyVert)))) return st;
    if ((st = ensure(ctx, ctx->prims, (size_t)nt * RF_MAX_FAN * sizeof(PrimRec)))) return st;
    if ((st = ensure(ctx, ctx->mask, mask_words * 4))) return st;
    if ((st = ensure(ctx, ctx->scan, rfk::scan_scratch_words((uint32_t)nt) * 4))) return st;
    if ((st = ensure(ctx, ctx->rowtot, 8))) return st;
    if ((st = ensure(ctx, ctx->rprims, (size_t)nt * RF_MAX_FAN * sizeof(RasterPrim)))) return st;
    if ((st = ensure(ctx, ctx->live, (size_t)nt * RF_MAX_FAN * 12))) return st;  // three lists
    if ((st = ensure(ctx, ctx->marks, 8))) return st;
    if ((st = ensure(ctx, ctx->items, (size_t)ntiles * (RF_SPLIT_K + 1) * 4))) return st;
    if (!ctx->rows_need_host) {
        CK(cudaMallocHost(&ctx->rows_need_host, sizeof(unsigned long long)));
        CK(cudaEventCreateWithFlags(&ctx->rows_evt, cudaEventDisableTiming));
    }
    if (ctx->rows_evt_pending && cudaEventQuery(ctx->rows_evt) == cudaSuccess) {
        const uint64_t need = *ctx->rows_need_host;
        if (need > ctx->rows_cap) ctx->rows_cap = need + need / 4;
        ctx->rows_evt_pending = false;
    }
    if (ctx->rows_cap == 0) ctx->rows_cap = std::max<uint64_t>((uint64_t)nt * 160u, 1u << 22);
    if (ctx->rows_cap > 0xFFFF0000ull) ctx->rows_cap = 0xFFFF0000ull;  // 32-bit record offsets
    if ((st = ensure(ctx, ctx->rows, ctx->rows_cap * 4))) return st;

    cudaStream_t s = ctx->stream;
    int kind = hd[0].shader;
    bool any_cull = false;
    for (const DrawDev &d : hd) {
        if (d.shader != kind) kind = RF_K_ANY;
        any_cull = any_cull || (d.flags & RF_DRAW_CULL_BBOX);
    }
    bool fast = true;
    for (const JobDev &J : hj)
        fast = fast && J.depth && J.depth_test == RF_DEPTH_LESS && J.color_write && J.depth_write;

    // Asynchronous uploads of the meshes read and read-backs of the targets
    // written must finish first.
    std::sort(ctx->async_meshes.begin(), ctx->async_meshes.end());
    ctx->async_meshes.erase(std::unique(ctx->async_meshes.begin(), ctx->async_meshes.end()),
                            ctx->async_meshes.end());
    for (Mesh *m : ctx->async_meshes)
        if ((st = before_use(ctx, *m))) return st;
    for (uint32_t k = 0; k < nin; ++k)
        if (host[k].slot >= 0 && (st = before_write(ctx, *in[k].tg))) return st;

    // Per-frame parameters travel as data (draws, jobs); the launch sequence
    // below depends only on the sizes, so it is replayed as a CUDA graph when
    // a frame of the same shape comes again.
    CK(cudaMemcpyAsync(ctx->draws.p, hd.data(), hd.size() * sizeof(DrawDev), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(ctx->jobs.p, hj.data(), hj.size() * sizeof(JobDev), cudaMemcpyHostToDevice, s));

    std::vector<cudaEvent_t> ev;
    if (ctx->timing) {
        for (int i = 0; i <= RF_STAGE_N; ++i) {
            cudaEvent_t e;
            if (!ctx->ev_free.empty()) {
                e = ctx->ev_free.back();
                ctx->ev_free.pop_back();
            } else {
                CK(cudaEventCreate(&e));
            }
            ev.push_back(e);
        }
    }
    uint32_t *counters = P<uint32_t>(ctx->counters);
    StatsDev *kst = per_job ? P<StatsDev>(ctx->jstats) : P<StatsDev>(ctx->stats);
    const DrawDev *dd = P<DrawDev>(ctx->draws);
    const JobDev *jd = P<JobDev>(ctx->jobs);
    auto enqueue = [&](bool marks) -> rf_status {
        auto mark = [&](int i) -> cudaError_t { return marks ? cudaEventRecord(ev[i], s) : cudaSuccess; };
        CK(cudaMemsetAsync(ctx->mask.p, 0, mask_words * 4, s));
        if (per_job) CK(cudaMemsetAsync(kst, 0, nj * sizeof(StatsDev), s));
        CK(mark(RF_STAGE_VERTEX));
        if (any_cull) CK(rfk::launch_cull(P<DrawDev>(ctx->draws), ndraws, kst, ctx->nsm, s));
        CK(rfk::launch_vertex(dd, ndraws, (uint32_t)nv, P<float4>(ctx->cpos), P<uint8_t>(ctx->coc),
                              counters, P<unsigned long long>(ctx->marks),
                              ctx->nsm, s));
        CK(mark(RF_STAGE_CLIP));
        // (each triangle's output slots placed by the clip kernels: no scan)
        CK(rfk::launch_clip(dd, ndraws, (uint32_t)nt, P<float4>(ctx->cpos), P<uint8_t>(ctx->coc),
                            P<uint32_t>(ctx->tcnt), P<uint32_t>(ctx->tpoly), P<uint32_t>(ctx->clipq),
                            P<PolyVert>(ctx->pool), pool_cap, counters, ctx->nsm, s,
                            P<uint32_t>(ctx->toff), true));
        CK(mark(RF_STAGE_SCAN));
        CK(mark(RF_STAGE_SETUP));
        CK(rfk::launch_setup(dd, ndraws, jd, (uint32_t)nt, TW, P<float4>(ctx->cpos),
                             P<uint32_t>(ctx->tcnt), P<uint32_t>(ctx->toff), P<uint32_t>(ctx->tpoly),
                             P<PolyVert>(ctx->pool), P<PrimRec>(ctx->prims), P<unsigned long long>(ctx->rowtot),
                             P<uint32_t>(ctx->rows), ctx->rows_cap, P<RasterPrim>(ctx->rprims),
                             P<uint32_t>(ctx->mask), P<uint32_t>(ctx->live), P<unsigned long long>(ctx->marks),
                             kst, counters, ctx->nsm, s, nullptr, nullptr, kind));
        CK(rfk::launch_items(jd, nj, P<uint32_t>(ctx->mask), ntiles, P<unsigned long long>(ctx->marks),
                             (uint32_t)ctx->nsm * 16u, P<uint32_t>(ctx->items), counters, s));
        CK(mark(RF_STAGE_RASTER));
        CK(rfk::launch_raster(TW, kind, fast, jd, nj, dd, P<PrimRec>(ctx->prims),
                              P<RasterPrim>(ctx->rprims), P<uint32_t>(ctx->rows), P<uint32_t>(ctx->tcnt),
                              P<uint32_t>(ctx->toff), P<uint32_t>(ctx->mask), ntiles, P<uint32_t>(ctx->items),
                              counters + RF_CNT_ITEMS, counters + RF_CNT_QUEUE, kst, ctx->warps, ctx->nsm, s));
        CK(mark(RF_STAGE_N));
        if (per_job) CK(rfk::launch_stats_fold(kst, nj, P<StatsDev>(ctx->stats), s));
        return RF_OK;
    };

    // A frame with depth-sorted jobs (render.rs:180-182): vertex, clip and
    // the scan as usual; then the clipped triangles' count per draw comes
    // back to the host (one wait), the triangles are sorted on the device
    // (rf_sort.cu), and setup, binning and the raster pass run over the
    // sorted order, every clipped triangle one unit of the tile masks.
    bool sorted = false;
    for (const JobDev &J : hj) sorted = sorted || J.depth_sort != RF_SORT_NONE;
    uint64_t sort_kernels = 0;
    auto enqueue_sorted = [&]() -> rf_status {
        auto mark = [&](int i) -> cudaError_t { return ctx->timing ? cudaEventRecord(ev[i], s) : cudaSuccess; };
        if (per_job) CK(cudaMemsetAsync(kst, 0, nj * sizeof(StatsDev), s));
        CK(mark(RF_STAGE_VERTEX));
        if (any_cull) CK(rfk::launch_cull(P<DrawDev>(ctx->draws), ndraws, kst, ctx->nsm, s));
        CK(rfk::launch_vertex(dd, ndraws, (uint32_t)nv, P<float4>(ctx->cpos), P<uint8_t>(ctx->coc),
                              counters, P<unsigned long long>(ctx->marks), ctx->nsm, s));
        CK(mark(RF_STAGE_CLIP));
        CK(rfk::launch_clip(dd, ndraws, (uint32_t)nt, P<float4>(ctx->cpos), P<uint8_t>(ctx->coc),
                            P<uint32_t>(ctx->tcnt), P<uint32_t>(ctx->tpoly), P<uint32_t>(ctx->toff),
                            P<PolyVert>(ctx->pool), pool_cap, counters, ctx->nsm, s,
                            P<uint32_t>(ctx->toff), false));
        CK(mark(RF_STAGE_SCAN));
        CK(rfk::launch_scan(P<uint32_t>(ctx->tcnt), P<uint32_t>(ctx->toff), (uint32_t)nt,
                            P<uint32_t>(ctx->scan), counters + RF_CNT_PRIMS, s));
        rf_status st2;
        if ((st2 = ensure(ctx, ctx->nout, (size_t)ndraws * 4))) return st2;
        CK(rfk::launch_draw_counts(dd, ndraws, (uint32_t)nt, P<uint32_t>(ctx->toff), counters,
                                   P<uint32_t>(ctx->nout), s));
        if (ctx->nout_host_cap < ndraws) {
            CK(cudaStreamSynchronize(s));
            if (ctx->nout_host) CK(cudaFreeHost(ctx->nout_host));
            ctx->nout_host = nullptr;
            ctx->nout_host_cap = 0;
            CK(cudaMallocHost(&ctx->nout_host, (size_t)ndraws * 4));
            ctx->nout_host_cap = ndraws;
        }
        CK(cudaMemcpyAsync(ctx->nout_host, ctx->nout.p, (size_t)ndraws * 4, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        // The setup pass's draws and jobs count clipped triangles, in the
        // sorted order (draw by draw, as the keys lead with the draw).
        std::vector<DrawDev> vd = hd;
        std::vector<JobDev> vj = hj;
        uint64_t np = 0;
        for (uint32_t d = 0; d < ndraws; ++d) {
            vd[d].tri_base = (uint32_t)np;
            vd[d].ntri = ctx->nout_host[d];
            np += ctx->nout_host[d];
        }
        if (np > 0x7FFFFFF0ull) return RF_ERR_BAD_ARG;
        for (JobDev &J : vj) {
            J.ntri = 0;
            J.tri_base = 0;
        }
        for (int64_t d = (int64_t)ndraws - 1; d >= 0; --d) {  // each job's first draw sets its base
            JobDev &J = vj[vd[d].job];
            J.tri_base = vd[d].tri_base;
            J.ntri += vd[d].ntri;
        }
        for (JobDev &J : vj) J.mask_words = (J.ntri + 31) / 32;
        layout_masks(vj);
        const size_t vmask = vj.back().sum_base + (size_t)vj.back().tiles_x * vj.back().tiles_y * vj.back().sum_words;
        const uint32_t n32 = (uint32_t)np;
        if ((st2 = ensure(ctx, ctx->mask, std::max<size_t>(vmask, 1) * 4))) return st2;
        if ((st2 = ensure(ctx, ctx->perm, (size_t)std::max<uint32_t>(n32, 1) * 4))) return st2;
        if ((st2 = ensure(ctx, ctx->ptri, (size_t)std::max<uint32_t>(n32, 1) * 4))) return st2;
        if ((st2 = ensure(ctx, ctx->dsort, rfk::dsort_scratch_bytes(n32)))) return st2;
        if ((st2 = ensure(ctx, ctx->scan,
                          rfk::scan_scratch_words(std::max<uint32_t>(rfk::dsort_scan_items(n32), (uint32_t)nt)) * 4)))
            return st2;
        if ((st2 = ensure(ctx, ctx->vtoff, (size_t)std::max<uint32_t>(n32, 1) * 4))) return st2;
        if ((st2 = ensure(ctx, ctx->vtcnt, (size_t)std::max<uint32_t>(n32, 1) * 4))) return st2;
        if ((st2 = ensure(ctx, ctx->vdraws, vd.size() * sizeof(DrawDev)))) return st2;
        if ((st2 = ensure(ctx, ctx->vjobs, vj.size() * sizeof(JobDev)))) return st2;
        CK(cudaMemcpyAsync(ctx->vdraws.p, vd.data(), vd.size() * sizeof(DrawDev), cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->vjobs.p, vj.data(), vj.size() * sizeof(JobDev), cudaMemcpyHostToDevice, s));
        const DrawDev *vdd = P<DrawDev>(ctx->vdraws);
        const JobDev *vjd = P<JobDev>(ctx->vjobs);
        CK(mark(RF_STAGE_SETUP));
        CK(rfk::launch_dsort(dd, ndraws, jd, (uint32_t)nt, n32, P<float4>(ctx->cpos), P<uint32_t>(ctx->tcnt),
                             P<uint32_t>(ctx->toff), P<uint32_t>(ctx->tpoly), P<PolyVert>(ctx->pool),
                             counters, P<uint32_t>(ctx->perm), P<uint32_t>(ctx->ptri), ctx->dsort.p,
                             P<uint32_t>(ctx->scan), s));
        CK(cudaMemsetAsync(ctx->mask.p, 0, vmask * 4, s));
        CK(rfk::launch_iota(P<uint32_t>(ctx->vtoff), P<uint32_t>(ctx->vtcnt), n32, s));
        CK(rfk::launch_setup(vdd, ndraws, vjd, n32, TW, P<float4>(ctx->cpos), P<uint32_t>(ctx->tcnt),
                             P<uint32_t>(ctx->toff), P<uint32_t>(ctx->tpoly), P<PolyVert>(ctx->pool),
                             P<PrimRec>(ctx->prims), P<unsigned long long>(ctx->rowtot),
                             P<uint32_t>(ctx->rows), ctx->rows_cap, P<RasterPrim>(ctx->rprims),
                             P<uint32_t>(ctx->mask), P<uint32_t>(ctx->live), P<unsigned long long>(ctx->marks),
                             kst, counters, ctx->nsm, s, P<uint32_t>(ctx->perm), P<uint32_t>(ctx->ptri), kind));
        CK(rfk::launch_items(vjd, nj, P<uint32_t>(ctx->mask), ntiles, P<unsigned long long>(ctx->marks),
                             (uint32_t)ctx->nsm * 16u, P<uint32_t>(ctx->items), counters, s));
        CK(mark(RF_STAGE_RASTER));
        CK(rfk::launch_raster(TW, kind, fast, vjd, nj, vdd, P<PrimRec>(ctx->prims), P<RasterPrim>(ctx->rprims),
                              P<uint32_t>(ctx->rows), P<uint32_t>(ctx->vtcnt), P<uint32_t>(ctx->vtoff),
                              P<uint32_t>(ctx->mask), ntiles, P<uint32_t>(ctx->items), counters + RF_CNT_ITEMS,
                              counters + RF_CNT_QUEUE, kst, ctx->warps, ctx->nsm, s));
        CK(mark(RF_STAGE_N));
        if (per_job) CK(rfk::launch_stats_fold(kst, nj, P<StatsDev>(ctx->stats), s));
        // draw counts, sort keys, per digit pass a histogram, a scan of 1 or 3
        // launches and a scatter, the unit arrays
        const uint32_t dpasses = 4 + (ndraws > 1 ? (ndraws > 256 ? (ndraws > 65536 ? 3 : 2) : 1) : 0);
        const uint32_t sitems = rfk::dsort_scan_items(n32);
        sort_kernels = 2 + (n32 ? 1 + dpasses * (2 + (sitems <= RF_SCAN_BLOCK_ITEMS ? 1 : 3)) + 1 : 0);
        return RF_OK;
    };

    if (tuned) CK(cudaEventRecord(tuned->e0, s));
    if (sorted) {
        if ((st = enqueue_sorted())) return st;
    } else if (ctx->graphs && !ctx->timing) {
        GraphKey key{};
        const uint64_t kv[] = {ctx->gen, ndraws, nj, nv, nt, ntiles, mask_words, TW, ctx->warps,
                               (uint64_t)(kind + 16) | (any_cull ? 0x100u : 0u), fast ? 1u : 0u,
                               per_job ? 1u : 0u, ctx->rows_cap};
        static_assert(sizeof kv == sizeof key.v, "graph key size");
        memcpy(key.v, kv, sizeof kv);
        GraphEntry *hit = nullptr;
        for (GraphEntry &g : ctx->gcache)
            if (g.key == key) hit = &g;
        if (!hit) {
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            st = enqueue(false);
            cudaError_t ce = cudaStreamEndCapture(s, &g);
            if (st) {
                if (g) cudaGraphDestroy(g);
                return st;
            }
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
            cudaGraphExec_t ex = nullptr;
            ce = cudaGraphInstantiate(&ex, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
            if (ctx->gcache.size() >= RF_GRAPH_CACHE) {
                size_t old = 0;
                for (size_t i = 1; i < ctx->gcache.size(); ++i)
                    if (ctx->gcache[i].used < ctx->gcache[old].used) old = i;
                cudaGraphExecDestroy(ctx->gcache[old].exec);  // stream-ordered launches finish first
                ctx->gcache.erase(ctx->gcache.begin() + old);
            }
            ctx->gcache.push_back(GraphEntry{key, ex, 0});
            hit = &ctx->gcache.back();
        }
        hit->used = ++ctx->gclock;
        CK(cudaGraphLaunch(hit->exec, s));
        ctx->graph_launches += 1;
    } else {
        if ((st = enqueue(ctx->timing))) return st;
    }
    if (tuned) {
        CK(cudaEventRecord(tuned->e1, s));
        tuned->pending = true;
    }
    // vertex, clip (2), setup, bin (3: 8- and 16-lane groups, then warps),
    // work list, raster (+ the stats fold; a depth-sorted frame adds the
    // scan of the fan counts, 3 launches or 1 for one block, and its sort)
    const uint64_t scan_kernels = sorted ? (nt <= RF_SCAN_BLOCK_ITEMS ? 1 : 3) : 0;
    ctx->kernels += 9 + scan_kernels + (per_job ? 1 : 0) + (any_cull ? 1 : 0) + sort_kernels;
    if (!ctx->rows_evt_pending) {
        CK(cudaMemcpyAsync(ctx->rows_need_host, ctx->rowtot.p, 8, cudaMemcpyDeviceToHost, s));
        CK(cudaEventRecord(ctx->rows_evt, s));
        ctx->rows_evt_pending = true;
    }
    if (ctx->timing) ctx->ev_pending.push_back(ev);
    for (uint32_t k = 0; k < nin; ++k)
        if (host[k].slot >= 0) in[k].tg->clear_flags = 0;  // the raster pass wrote the pending clear
    for (Mesh *m : ctx->async_meshes) CK(cudaEventRecord(m->used, s));
    for (uint32_t k = 0; k < nin; ++k)
        if (host[k].slot >= 0 && in[k].tg->async) CK(cudaEventRecord(in[k].tg->rendered, s));
    return RF_OK;
}

rf_status flush_clear(rf_ctx *ctx, Target &tg) {
    if (!tg.clear_flags) return RF_OK;
    rf_status st = before_write(ctx, tg);
    if (st) return st;
    CK(rfk::launch_fill(tg.color, tg.depth, (size_t)tg.w * tg.h, tg.clear_px, tg.clear_z,
                        tg.clear_flags, ctx->nsm, ctx->stream));
    if (tg.async) CK(cudaEventRecord(tg.rendered, ctx->stream));
    ctx->kernels += 1;
    tg.clear_flags = 0;
    return RF_OK;
}

// rf_mesh_upload (per = 3 indices per triangle) and rf_lines_upload (per =
// 2 per line).  A failed allocation or copy frees what was allocated.
rf_status upload_mesh(rf_ctx *ctx, const float *verts, uint32_t nverts, uint32_t pos_dim,
                      uint32_t nattr, const uint32_t *idx, uint32_t nprim, uint32_t per,
                      rf_mesh *out) {
    if (!ctx || !out || (pos_dim != 3 && pos_dim != 4) || nattr > RF_MAX_ATTR) return RF_ERR_BAD_ARG;
    if ((nverts && !verts) || (nprim && !idx)) return RF_ERR_BAD_ARG;
    if (!indices_ok(idx, (uint64_t)per * nprim, nverts)) return RF_ERR_BAD_ARG;
    Mesh m;
    m.nverts = nverts;
    m.ntri = nprim;
    m.pos_dim = pos_dim;
    m.nattr = nattr;
    m.lines = per == 2;
    const size_t vb = (size_t)nverts * (pos_dim + nattr) * 4, ib = (size_t)nprim * per * 4;
    cudaError_t e = cudaSuccess;
    if (vb) e = cudaMalloc(&m.verts, vb);
    if (e == cudaSuccess && ib) e = cudaMalloc(&m.idx, ib);
    if (e == cudaSuccess) e = cudaMalloc(&m.bbox, RF_MESH_BBOX_FLOATS * 4);
    if (e == cudaSuccess && vb) e = cudaMemcpyAsync(m.verts, verts, vb, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess && ib) e = cudaMemcpyAsync(m.idx, idx, ib, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = rfk::launch_mesh_bbox(m.verts, nverts, pos_dim + nattr, m.bbox, ctx->stream);
    ctx->kernels += 2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(m.verts);
        cudaFree(m.idx);
        cudaFree(m.bbox);
        return cuda_fail(ctx, e, per == 2 ? "rf_lines_upload" : "rf_mesh_upload");
    }
    const uint64_t h = ctx->next_handle++;
    ctx->res->meshes[h] = m;
    *out = h;
    return RF_OK;
}

// The jobs of a batch (distinct targets of this context) queued as one pass.
rf_status queue_batch(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, std::vector<JobHost> &host) {
    std::vector<JobIn> in(njobs);
    std::vector<rf_target> seen(njobs);
    for (uint32_t k = 0; k < njobs; ++k) {
        auto it = ctx->targets.find(jobs[k].target);
        if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
        in[k].draws = jobs[k].draws;
        in[k].ndraws = jobs[k].ndraws;
        in[k].vp = jobs[k].viewport;
        in[k].tg = &it->second;
        in[k].fl = &jobs[k].flags;
        seen[k] = jobs[k].target;
    }
    std::sort(seen.begin(), seen.end());
    if (std::adjacent_find(seen.begin(), seen.end()) != seen.end()) return RF_ERR_BAD_ARG;
    return run_jobs(ctx, in.data(), njobs, true, host);
}

// The stats of one call made with a stats pointer (render.rs:206 adds them
// into ctx.stats): the running totals just before and just after the
// call's work; they are then marked as handed out, so rf_ctx_take_stats
// does not report them again.
struct CallStats {
    rf_stats before{};
    bool on = false;
};
rf_status call_stats_begin(rf_ctx *ctx, const rf_stats *out, CallStats &cs) {
    if (!out) return RF_OK;
    rf_status st = init_stats(ctx);
    if (st) return st;
    if ((st = read_totals(ctx, cs.before))) return st;
    cs.on = true;
    return RF_OK;
}
rf_status call_stats_end(rf_ctx *ctx, rf_stats *out, const CallStats &cs) {
    if (!cs.on) return RF_OK;
    rf_stats after{};
    rf_status st = read_totals(ctx, after);
    if (st) return st;
    *out = sub_stats(after, cs.before);
    add_stats(ctx->taken, *out);
    return RF_OK;
}

rf_status finish_call(rf_ctx *ctx, rf_stats *out) {
    if (!out) return RF_OK;
    rf_stats tot{};
    rf_status st = read_totals(ctx, tot);
    if (st) return st;
    const rf_stats d = sub_stats(tot, ctx->taken);
    ctx->taken = tot;
    *out = d;
    return RF_OK;
}

}  // namespace

extern "C" {

const char *rf_status_str(rf_status s) {
    switch (s) {
        case RF_OK: return "ok";
        case RF_ERR_BAD_HANDLE: return "bad handle";
        case RF_ERR_BAD_ARG: return "bad argument";
        case RF_ERR_NON_POT_TEXTURE: return "texture dimensions must be powers of two";
        case RF_ERR_OOM: return "out of device memory";
        case RF_ERR_OVER_BUDGET: return "over memory budget";
        case RF_ERR_OVERFLOW: return "overflow";
        case RF_ERR_TIMEOUT: return "timeout";
        case RF_ERR_CUDA: return "cuda error";
        case RF_ERR_NO_DEVICE: return "no cuda device";
        default: return "unknown status";
    }
}

const char *rf_ctx_last_error(const rf_ctx *ctx) {
    return ctx ? ctx->last_error : "";
}

rf_status rf_ctx_create(void *cuda_stream, rf_ctx **out) {
    if (!out) return RF_ERR_BAD_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return RF_ERR_NO_DEVICE;
    }
    rf_ctx *ctx = new (std::nothrow) rf_ctx();
    if (!ctx) return RF_ERR_OOM;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
        delete ctx;
        return RF_ERR_CUDA;
    }
    ctx->device = dev;
    if (cuda_stream) {
        ctx->stream = (cudaStream_t)cuda_stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete ctx;
            return RF_ERR_CUDA;
        }
        ctx->own_stream = true;
    }
    *out = ctx;
    return RF_OK;
}

rf_status rf_ctx_destroy(rf_ctx *ctx) {
    if (!ctx) return RF_ERR_BAD_ARG;
    sync_all(ctx);
    if (!ctx->shared_res) {
        for (auto &kv : ctx->res->meshes) {
            cudaFree(kv.second.verts);
            cudaFree(kv.second.idx);
            cudaFree(kv.second.bbox);
            drop_async(kv.second);
        }
        for (auto &kv : ctx->res->textures) cudaFree(kv.second.texels);
    }
    for (auto &kv : ctx->targets) { cudaFree(kv.second.color); cudaFree(kv.second.depth); drop_async(kv.second); }
    if (ctx->up) cudaStreamDestroy(ctx->up);
    if (ctx->down) cudaStreamDestroy(ctx->down);
    graphs_drop(ctx);
    for (TuneState &t : ctx->tunes) {
        if (t.e0) cudaEventDestroy(t.e0);
        if (t.e1) cudaEventDestroy(t.e1);
    }
    DevBuf *bufs[] = {&ctx->draws, &ctx->jobs, &ctx->cpos, &ctx->coc, &ctx->tcnt, &ctx->toff,
                      &ctx->tpoly, &ctx->pool, &ctx->prims, &ctx->mask, &ctx->scan,
                      &ctx->counters, &ctx->stats,
                      &ctx->rowtot, &ctx->clipq, &ctx->rows, &ctx->rprims, &ctx->live, &ctx->marks, &ctx->items, &ctx->jstats, &ctx->lrec, &ctx->lmask,
                      &ctx->perm, &ctx->ptri, &ctx->nout, &ctx->dsort, &ctx->vdraws, &ctx->vjobs,
                      &ctx->vtoff, &ctx->vtcnt};
    if (ctx->nout_host) cudaFreeHost(ctx->nout_host);
    if (ctx->rows_need_host) cudaFreeHost(ctx->rows_need_host);
    if (ctx->rows_evt) cudaEventDestroy(ctx->rows_evt);
    for (DevBuf *b : bufs) cudaFree(b->p);
    for (auto &ev : ctx->ev_pending)
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->ev_free) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return RF_OK;
}

rf_status rf_ctx_device(rf_ctx *ctx, int32_t *device) {
    if (!ctx || !device) return RF_ERR_BAD_ARG;
    *device = ctx->device;
    return RF_OK;
}

rf_status rf_ctx_sync(rf_ctx *ctx) {
    if (!ctx) return RF_ERR_BAD_ARG;
    return sync_all(ctx);
}

rf_status rf_ctx_take_stats(rf_ctx *ctx, rf_stats *out) {
    if (!ctx || !out) return RF_ERR_BAD_ARG;
    rf_stats d{};
    rf_status st = finish_call(ctx, &d);
    if (st) return st;
    add_stats(*out, d);
    return RF_OK;
}

rf_status rf_ctx_set_timing(rf_ctx *ctx, int32_t enable) {
    if (!ctx) return RF_ERR_BAD_ARG;
    ctx->timing = enable != 0;
    return RF_OK;
}

rf_status rf_ctx_stage_ms(rf_ctx *ctx, double out[RF_STAGE_N], uint32_t *frames) {
    if (!ctx || !out) return RF_ERR_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    for (auto &ev : ctx->ev_pending) {
        for (int i = 0; i < RF_STAGE_N; ++i) {
            float ms = 0.0f;
            CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
            ctx->stage_ms[i] += ms;
        }
        for (cudaEvent_t e : ev) ctx->ev_free.push_back(e);
        ctx->timed_frames += 1;
    }
    ctx->ev_pending.clear();
    for (int i = 0; i < RF_STAGE_N; ++i) {
        out[i] += ctx->stage_ms[i];
        ctx->stage_ms[i] = 0.0;
    }
    if (frames) *frames = ctx->timed_frames;
    ctx->timed_frames = 0;
    return RF_OK;
}

rf_status rf_ctx_set_tiling(rf_ctx *ctx, uint32_t tile_w, uint32_t warps) {
    if (!ctx) return RF_ERR_BAD_ARG;
    if (tile_w && tile_w != 8 && tile_w != 16 && tile_w != 32 && tile_w != 64) return RF_ERR_BAD_ARG;
    if (warps && (warps > RF_RASTER_MAX_THREADS / 32)) return RF_ERR_BAD_ARG;
    if (tile_w) {
        ctx->tile_w = tile_w;
        ctx->tune_online = false;  // an explicit width is kept for every frame
    }
    if (warps) ctx->warps = warps;
    return RF_OK;
}

rf_status rf_ctx_set_online_tuning(rf_ctx *ctx, int32_t enable) {
    if (!ctx) return RF_ERR_BAD_ARG;
    ctx->tune_online = enable != 0;
    return RF_OK;
}

rf_status rf_ctx_last_tiling(rf_ctx *ctx, uint32_t *tile_w, uint32_t *warps) {
    if (!ctx) return RF_ERR_BAD_ARG;
    if (tile_w) *tile_w = ctx->last_tile_w;
    if (warps) *warps = ctx->warps;
    return RF_OK;
}

rf_status rf_mesh_upload(rf_ctx *ctx, const float *verts, uint32_t nverts, uint32_t pos_dim,
                         uint32_t nattr, const uint32_t *idx, uint32_t ntri, rf_mesh *out) {
    return upload_mesh(ctx, verts, nverts, pos_dim, nattr, idx, ntri, 3, out);
}

rf_status rf_lines_upload(rf_ctx *ctx, const float *verts, uint32_t nverts, uint32_t pos_dim,
                          uint32_t nattr, const uint32_t *idx, uint32_t nlines, rf_mesh *out) {
    return upload_mesh(ctx, verts, nverts, pos_dim, nattr, idx, nlines, 2, out);
}

rf_status rf_render_lines(rf_ctx *ctx, rf_mesh mesh, int32_t shader, const rf_uniforms *u,
                          const float viewport[16], rf_target target, const rf_context_flags *fl,
                          rf_stats *stats) {
    if (!ctx || !u || !viewport || !flags_ok(fl)) return RF_ERR_BAD_ARG;
    auto mit = ctx->res->meshes.find(mesh);
    if (mit == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
    auto tit = ctx->targets.find(target);
    if (tit == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    Mesh &m = mit->second;
    Target &tg = tit->second;
    if (!m.lines) return RF_ERR_BAD_ARG;
    if (shader < RF_SHADER_FLAT || shader > RF_SHADER_GOURAUD_SRGB || m.nattr != nattr_for(shader))
        return RF_ERR_BAD_ARG;
    rf_status st = init_stats(ctx);
    if (st) return st;
    CallStats cs;
    if ((st = call_stats_begin(ctx, stats, cs))) return st;
    DrawDev d{};
    d.verts = m.verts;
    d.idx = m.idx;
    d.bbox = m.bbox;
    d.nverts = m.nverts;
    d.ntri = m.ntri;
    d.pos_dim = m.pos_dim;
    d.nattr = m.nattr;
    d.stride = m.pos_dim + m.nattr;
    d.shader = shader;
    d.sampler = (int32_t)u->sampler;
    d.flat_rgba = u->flat_rgba;
    if (shader == RF_SHADER_TEXTURED || shader == RF_SHADER_TEX_GOURAUD) {
        auto xit = ctx->res->textures.find(u->texture);
        if (xit == ctx->res->textures.end()) return RF_ERR_BAD_HANDLE;
        if (d.sampler < RF_SAMPLER_REPEAT_POT || d.sampler > RF_SAMPLER_ONCE) return RF_ERR_BAD_ARG;
        if (d.sampler == RF_SAMPLER_REPEAT_POT && (!is_pot(xit->second.w) || !is_pot(xit->second.h)))
            return RF_ERR_NON_POT_TEXTURE;
        d.tex = xit->second.texels;
        d.tw = xit->second.w;
        d.th = xit->second.h;
    }
    memcpy(d.mvp, u->mvp, sizeof d.mvp);
    ctx->host_acc.calls += 1;  // render.rs:152-155
    ctx->host_acc.prims_i += m.ntri;
    ctx->host_acc.verts_i += m.nverts;
    if (m.ntri && m.nverts) {
        // The line pass writes the target directly: a pending clear first.
        if ((st = flush_clear(ctx, tg))) return st;
        if ((st = before_use(ctx, m))) return st;
        if ((st = before_write(ctx, tg))) return st;
        JobDev J{};
        J.color = tg.color;
        J.depth = tg.depth;
        J.w = tg.w;
        J.h = tg.h;
        J.pixfmt = tg.fmt;
        J.depth_test = fl->depth_test;
        J.color_write = fl->color_write;
        J.depth_write = fl->depth_write;
        J.face_cull = fl->face_cull;
        J.tiles_x = (tg.w + RF_TILE_H - 1) / RF_TILE_H;
        J.tiles_y = (tg.h + RF_TILE_H - 1) / RF_TILE_H;
        J.ntri = m.ntri;
        J.mask_words = (m.ntri + 31) / 32;
        memcpy(J.vp, viewport, sizeof J.vp);
        const uint32_t ntiles = J.tiles_x * J.tiles_y;
        const size_t mwords = (size_t)ntiles * J.mask_words;
        if ((st = ensure(ctx, ctx->draws, sizeof(DrawDev)))) return st;
        if ((st = ensure(ctx, ctx->jobs, sizeof(JobDev)))) return st;
        if ((st = ensure(ctx, ctx->cpos, (size_t)m.nverts * sizeof(float4)))) return st;
        if ((st = ensure(ctx, ctx->coc, m.nverts))) return st;
        if ((st = ensure(ctx, ctx->lrec, (size_t)m.ntri * sizeof(LineRec)))) return st;
        if ((st = ensure(ctx, ctx->lmask, mwords * 4))) return st;
        cudaStream_t s = ctx->stream;
        CK(cudaMemcpyAsync(ctx->draws.p, &d, sizeof d, cudaMemcpyHostToDevice, s));
        CK(cudaMemcpyAsync(ctx->jobs.p, &J, sizeof J, cudaMemcpyHostToDevice, s));
        uint32_t *counters = P<uint32_t>(ctx->counters);
        CK(cudaMemsetAsync(counters + RF_CNT_QUEUE, 0, 4, s));
        CK(cudaMemsetAsync(ctx->lmask.p, 0, mwords * 4, s));
        CK(rfk::launch_vertex(P<DrawDev>(ctx->draws), 1, m.nverts, P<float4>(ctx->cpos),
                              P<uint8_t>(ctx->coc), nullptr, nullptr, ctx->nsm, s));
        CK(rfk::launch_lines(P<DrawDev>(ctx->draws), P<JobDev>(ctx->jobs), m.ntri, P<float4>(ctx->cpos),
                             P<uint8_t>(ctx->coc), P<LineRec>(ctx->lrec), P<uint32_t>(ctx->lmask), ntiles,
                             counters + RF_CNT_QUEUE, P<StatsDev>(ctx->stats), ctx->nsm, s));
        ctx->kernels += 3;
        if (m.async) CK(cudaEventRecord(m.used, s));
        if (tg.async) CK(cudaEventRecord(tg.rendered, s));
    }
    return call_stats_end(ctx, stats, cs);
}

rf_status rf_mesh_update(rf_ctx *ctx, rf_mesh mesh, const float *verts, const uint32_t *idx) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->res->meshes.find(mesh);
    if (it == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
    Mesh &m = it->second;
    const uint32_t per = m.lines ? 2u : 3u;
    if (idx && !indices_ok(idx, (uint64_t)per * m.ntri, m.nverts)) return RF_ERR_BAD_ARG;
    const size_t vb = (size_t)m.nverts * (m.pos_dim + m.nattr) * 4, ib = (size_t)m.ntri * per * 4;
    rf_status st = before_use(ctx, m);  // an asynchronous upload still in flight
    if (st) return st;
    if (verts && vb) CK(cudaMemcpyAsync(m.verts, verts, vb, cudaMemcpyHostToDevice, ctx->stream));
    if (idx && ib) CK(cudaMemcpyAsync(m.idx, idx, ib, cudaMemcpyHostToDevice, ctx->stream));
    if (verts) {
        CK(rfk::launch_mesh_bbox(m.verts, m.nverts, m.pos_dim + m.nattr, m.bbox, ctx->stream));
        ctx->kernels += 2;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return RF_OK;
}

rf_status rf_mesh_update_async(rf_ctx *ctx, rf_mesh mesh, const float *verts, const uint32_t *idx) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->res->meshes.find(mesh);
    if (it == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
    Mesh &m = it->second;
    const uint32_t per = m.lines ? 2u : 3u;
    if (idx && !indices_ok(idx, (uint64_t)per * m.ntri, m.nverts)) return RF_ERR_BAD_ARG;
    rf_status st = copy_streams(ctx);
    if (st) return st;
    if ((st = make_async(ctx, m))) return st;
    const size_t vb = (size_t)m.nverts * (m.pos_dim + m.nattr) * 4, ib = (size_t)m.ntri * per * 4;
    // The copy waits for every queued render that reads the mesh.
    CK(cudaStreamWaitEvent(ctx->up, m.used, 0));
    if (verts && vb) CK(cudaMemcpyAsync(m.verts, verts, vb, cudaMemcpyHostToDevice, ctx->up));
    if (idx && ib) CK(cudaMemcpyAsync(m.idx, idx, ib, cudaMemcpyHostToDevice, ctx->up));
    if (verts) {
        CK(rfk::launch_mesh_bbox(m.verts, m.nverts, m.pos_dim + m.nattr, m.bbox, ctx->up));
        ctx->kernels += 2;
    }
    CK(cudaEventRecord(m.ready, ctx->up));
    m.ready_pending = true;
    return RF_OK;
}

rf_status rf_mesh_info(rf_ctx *ctx, rf_mesh mesh, uint32_t *nverts, uint32_t *ntri, uint32_t *nattr) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->res->meshes.find(mesh);
    if (it == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
    if (nverts) *nverts = it->second.nverts;
    if (ntri) *ntri = it->second.ntri;
    if (nattr) *nattr = it->second.nattr;
    return RF_OK;
}

rf_status rf_mesh_destroy(rf_ctx *ctx, rf_mesh mesh) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->res->meshes.find(mesh);
    if (it == ctx->res->meshes.end()) return RF_ERR_BAD_HANDLE;
    rf_status st = sync_all(ctx);
    if (st) return st;
    cudaFree(it->second.verts);
    cudaFree(it->second.idx);
    cudaFree(it->second.bbox);
    drop_async(it->second);
    ctx->res->meshes.erase(it);
    return RF_OK;
}

rf_status rf_texture_upload(rf_ctx *ctx, const uint32_t *rgba, uint32_t w, uint32_t h,
                            rf_texture *out) {
    if (!ctx || !out || !rgba || !w || !h) return RF_ERR_BAD_ARG;
    Texture t;
    t.w = w;
    t.h = h;
    const size_t b = (size_t)w * h * 4;
    cudaError_t e = cudaMalloc(&t.texels, b);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t.texels, rgba, b, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) {
        cudaFree(t.texels);
        return cuda_fail(ctx, e, "rf_texture_upload");
    }
    const uint64_t hd = ctx->next_handle++;
    ctx->res->textures[hd] = t;
    *out = hd;
    return RF_OK;
}

rf_status rf_texture_destroy(rf_ctx *ctx, rf_texture tex) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->res->textures.find(tex);
    if (it == ctx->res->textures.end()) return RF_ERR_BAD_HANDLE;
    CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(it->second.texels);
    ctx->res->textures.erase(it);
    return RF_OK;
}

rf_status rf_target_create(rf_ctx *ctx, uint32_t w, uint32_t h, int32_t pixfmt, int32_t has_depth,
                           rf_target *out) {
    if (!ctx || !out || !w || !h || w > RF_MAX_TARGET_DIM || h > RF_MAX_TARGET_DIM) return RF_ERR_BAD_ARG;
    if (pixfmt < RF_ARGB8888 || pixfmt > RF_BGRA8888) return RF_ERR_BAD_ARG;
    Target t;
    t.w = w;
    t.h = h;
    t.fmt = pixfmt;
    const size_t n = (size_t)w * h;
    cudaError_t e = cudaMalloc(&t.color, n * 4);
    if (e == cudaSuccess) e = cudaMemsetAsync(t.color, 0, n * 4, ctx->stream);
    if (e == cudaSuccess && has_depth) e = cudaMalloc(&t.depth, n * 4);
    if (e == cudaSuccess && has_depth) e = cudaMemsetAsync(t.depth, 0, n * 4, ctx->stream);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(t.color);
        cudaFree(t.depth);
        return cuda_fail(ctx, e, "rf_target_create");
    }
    const uint64_t hd = ctx->next_handle++;
    ctx->targets[hd] = t;
    *out = hd;
    return RF_OK;
}

rf_status rf_target_destroy(rf_ctx *ctx, rf_target t) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(t);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    rf_status st = sync_all(ctx);
    if (st) return st;
    cudaFree(it->second.color);
    cudaFree(it->second.depth);
    drop_async(it->second);
    ctx->targets.erase(it);
    return RF_OK;
}

rf_status rf_target_clear(rf_ctx *ctx, rf_target t, const uint32_t *clear_rgba,
                          const float *depth_clear) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(t);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    Target &tg = it->second;
    if (clear_rgba) {
        tg.clear_flags |= 1u;
        tg.clear_px = pack_px(*clear_rgba, tg.fmt);
    }
    if (depth_clear && tg.depth) {
        tg.clear_flags |= 2u;
        volatile float one = 1.0f;
        tg.clear_z = one / *depth_clear;  // f32::recip
    }
    return RF_OK;
}

rf_status rf_target_write(rf_ctx *ctx, rf_target t, const uint32_t *color, const float *depth) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(t);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    Target &tg = it->second;
    rf_status st = flush_clear(ctx, tg);
    if (st) return st;
    if ((st = before_write(ctx, tg))) return st;
    const size_t n = (size_t)tg.w * tg.h * 4;
    if (color) CK(cudaMemcpyAsync(tg.color, color, n, cudaMemcpyHostToDevice, ctx->stream));
    if (depth && tg.depth) CK(cudaMemcpyAsync(tg.depth, depth, n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return RF_OK;
}

rf_status rf_target_read(rf_ctx *ctx, rf_target t, uint32_t *color, float *depth) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(t);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    Target &tg = it->second;
    rf_status st = flush_clear(ctx, tg);
    if (st) return st;
    const size_t n = (size_t)tg.w * tg.h * 4;
    if (color) CK(cudaMemcpyAsync(color, tg.color, n, cudaMemcpyDeviceToHost, ctx->stream));
    if (depth && tg.depth) CK(cudaMemcpyAsync(depth, tg.depth, n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return RF_OK;
}

rf_status rf_target_read_async(rf_ctx *ctx, rf_target t, uint32_t *color, float *depth) {
    if (!ctx) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(t);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    Target &tg = it->second;
    rf_status st = copy_streams(ctx);
    if (st) return st;
    if ((st = make_async(ctx, tg))) return st;
    if ((st = flush_clear(ctx, tg))) return st;
    const size_t n = (size_t)tg.w * tg.h * 4;
    // The copy waits for every queued render into the target.
    CK(cudaStreamWaitEvent(ctx->down, tg.rendered, 0));
    if (color) CK(cudaMemcpyAsync(color, tg.color, n, cudaMemcpyDeviceToHost, ctx->down));
    if (depth && tg.depth) CK(cudaMemcpyAsync(depth, tg.depth, n, cudaMemcpyDeviceToHost, ctx->down));
    CK(cudaEventRecord(tg.read_done, ctx->down));
    tg.read_pending = true;
    return RF_OK;
}

rf_status rf_render(rf_ctx *ctx, rf_mesh mesh, int32_t shader, const rf_uniforms *uniforms,
                    const float viewport[16], rf_target target, const rf_context_flags *flags,
                    rf_stats *stats) {
    if (!ctx || !uniforms) return RF_ERR_BAD_ARG;
    rf_draw d;
    memset(&d, 0, sizeof d);
    d.mesh = mesh;
    d.shader = shader;
    d.uniforms = *uniforms;
    return rf_render_draws(ctx, &d, 1, viewport, target, flags, stats);
}

rf_status rf_render_draws(rf_ctx *ctx, const rf_draw *draws, uint32_t ndraws,
                          const float viewport[16], rf_target target,
                          const rf_context_flags *flags, rf_stats *stats) {
    if (!ctx || (ndraws && !draws)) return RF_ERR_BAD_ARG;
    auto it = ctx->targets.find(target);
    if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
    JobIn ji;
    ji.draws = draws;
    ji.ndraws = ndraws;
    ji.vp = viewport;
    ji.tg = &it->second;
    ji.fl = flags;
    CallStats cs;
    rf_status st = call_stats_begin(ctx, stats, cs);
    if (st) return st;
    std::vector<JobHost> host;
    if ((st = run_jobs(ctx, &ji, 1, false, host))) return st;
    return call_stats_end(ctx, stats, cs);
}

rf_status rf_render_batch(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, rf_stats *stats) {
    if (!ctx || (njobs && !jobs)) return RF_ERR_BAD_ARG;
    std::vector<JobHost> host;
    rf_status st = queue_batch(ctx, jobs, njobs, host);
    if (st) return st;
    if (!stats) return RF_OK;
    // Per-job stats: this batch's slots plus the host counts; the running
    // total already holds them (folded on the device), so they are marked
    // as handed out.
    std::vector<StatsDev> js(ctx->hjobs.size());
    CK(cudaStreamSynchronize(ctx->stream));
    if (!js.empty())
        CK(cudaMemcpy(js.data(), ctx->jstats.p, js.size() * sizeof(StatsDev), cudaMemcpyDeviceToHost));
    rfi_batch_stats(host, js.data(), stats);
    for (uint32_t k = 0; k < njobs; ++k) add_stats(ctx->taken, stats[k]);
    return RF_OK;
}

rf_status rf_ctx_set_graphs(rf_ctx *ctx, int32_t enable) {
    if (!ctx) return RF_ERR_BAD_ARG;
    ctx->graphs = enable != 0;
    if (!ctx->graphs) {
        CK(cudaStreamSynchronize(ctx->stream));
        graphs_drop(ctx);
    }
    return RF_OK;
}

rf_status rf_ctx_counts(rf_ctx *ctx, uint64_t *kernels, uint64_t *graph_launches,
                        uint32_t *graphs_cached) {
    if (!ctx) return RF_ERR_BAD_ARG;
    if (kernels) *kernels = ctx->kernels;
    if (graph_launches) *graph_launches = ctx->graph_launches;
    if (graphs_cached) *graphs_cached = (uint32_t)ctx->gcache.size();
    return RF_OK;
}

rf_status rf_ctx_autotune(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, uint32_t reps,
                          uint32_t *tile_w, uint32_t *warps, float *best_ms) {
    if (!ctx || !jobs || !njobs) return RF_ERR_BAD_ARG;
    if (reps == 0) reps = 3;
    // Snapshot every target (pixels and pending clear) so each trial starts
    // from the same state and the call leaves the targets as they were.
    struct Snap {
        Target *tg;
        uint32_t *color = nullptr;
        float *depth = nullptr;
        uint32_t clear_flags;
    };
    std::vector<Snap> snaps;
    std::vector<rf_target> handles;
    for (uint32_t k = 0; k < njobs; ++k) {
        auto it = ctx->targets.find(jobs[k].target);
        if (it == ctx->targets.end()) return RF_ERR_BAD_HANDLE;
        handles.push_back(jobs[k].target);
    }
    std::sort(handles.begin(), handles.end());
    if (std::adjacent_find(handles.begin(), handles.end()) != handles.end()) return RF_ERR_BAD_ARG;
    rf_stats before{};
    rf_status st = read_totals(ctx, before);
    if (st) return st;
    const uint32_t tw0 = ctx->tile_w, wp0 = ctx->warps;
    const bool timing0 = ctx->timing, online0 = ctx->tune_online;
    ctx->timing = false;
    ctx->tune_online = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        for (Snap &sn : snaps) {
            cudaFree(sn.color);
            cudaFree(sn.depth);
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        ctx->timing = timing0;
        ctx->tune_online = online0;
    };
    auto restore = [&]() -> cudaError_t {
        for (Snap &sn : snaps) {
            const size_t n = (size_t)sn.tg->w * sn.tg->h * 4;
            cudaError_t e = cudaMemcpyAsync(sn.tg->color, sn.color, n, cudaMemcpyDeviceToDevice, ctx->stream);
            if (e == cudaSuccess && sn.depth)
                e = cudaMemcpyAsync(sn.tg->depth, sn.depth, n, cudaMemcpyDeviceToDevice, ctx->stream);
            if (e != cudaSuccess) return e;
            sn.tg->clear_flags = sn.clear_flags;
        }
        return cudaSuccess;
    };
    cudaError_t ce = cudaSuccess;
    for (uint32_t k = 0; k < njobs && ce == cudaSuccess; ++k) {
        Snap sn;
        sn.tg = &ctx->targets.find(jobs[k].target)->second;
        sn.clear_flags = sn.tg->clear_flags;
        const size_t n = (size_t)sn.tg->w * sn.tg->h * 4;
        ce = cudaMalloc(&sn.color, n);
        if (ce == cudaSuccess && sn.tg->depth) ce = cudaMalloc(&sn.depth, n);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(sn.color, sn.tg->color, n, cudaMemcpyDeviceToDevice, ctx->stream);
        if (ce == cudaSuccess && sn.depth)
            ce = cudaMemcpyAsync(sn.depth, sn.tg->depth, n, cudaMemcpyDeviceToDevice, ctx->stream);
        snaps.push_back(sn);
    }
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) {
        cleanup();
        return cuda_fail(ctx, ce, "autotune setup");
    }
    static const uint32_t TWS[] = {8, 16, 32, 64};
    static const uint32_t WPS[] = {4, 8};
    float best = -1.0f;
    uint32_t btw = tw0, bwp = wp0;
    for (uint32_t tw : TWS) {
        for (uint32_t wp : WPS) {
            ctx->tile_w = tw;
            ctx->warps = wp;
            float tmin = -1.0f;
            for (uint32_t r = 0; r <= reps && st == RF_OK; ++r) {  // r == 0: warm-up
                if ((ce = restore()) != cudaSuccess) break;
                if ((ce = cudaEventRecord(e0, ctx->stream)) != cudaSuccess) break;
                st = rf_render_batch(ctx, jobs, njobs, nullptr);
                if (st) break;
                if ((ce = cudaEventRecord(e1, ctx->stream)) != cudaSuccess) break;
                if ((ce = cudaEventSynchronize(e1)) != cudaSuccess) break;
                float ms = 0.0f;
                if ((ce = cudaEventElapsedTime(&ms, e0, e1)) != cudaSuccess) break;
                if (r > 0 && (tmin < 0.0f || ms < tmin)) tmin = ms;
            }
            if (st || ce != cudaSuccess) break;
            if (best < 0.0f || tmin < best) {
                best = tmin;
                btw = tw;
                bwp = wp;
            }
        }
        if (st || ce != cudaSuccess) break;
    }
    if (ce == cudaSuccess && !st) ce = restore();
    if (ce == cudaSuccess && !st) ce = cudaStreamSynchronize(ctx->stream);
    rf_stats after{};
    if (ce == cudaSuccess && !st) st = read_totals(ctx, after);
    cleanup();
    if (ce != cudaSuccess) {
        ctx->tile_w = tw0;
        ctx->warps = wp0;
        return cuda_fail(ctx, ce, "autotune");
    }
    if (st) {
        ctx->tile_w = tw0;
        ctx->warps = wp0;
        return st;
    }
    // The trial renders are not the caller's: hide their stats.
    add_stats(ctx->taken, sub_stats(after, before));
    ctx->tile_w = btw;
    ctx->warps = bwp;
    ctx->tune_online = false;  // the chosen tiling is kept
    if (tile_w) *tile_w = btw;
    if (warps) *warps = bwp;
    if (best_ms) *best_ms = best;
    return RF_OK;
}

}  // extern "C"

// ---- internal interface of the serving loop (rf_ctx_internal.h) --------

void rfi_batch_stats(const std::vector<rfi_counts> &counts, const StatsDev *js, rf_stats *out) {
    for (size_t k = 0; k < counts.size(); ++k) {
        rf_stats o{};
        o.calls = counts[k].calls;
        o.prims_i = counts[k].prims_i;
        o.verts_i = counts[k].verts_i;
        if (counts[k].slot >= 0) {
            const StatsDev &d = js[counts[k].slot];
            o.prims_o = d.prims_o;
            o.verts_o = d.verts_o;
            o.frags_i = d.frags_i;
            o.frags_o = d.frags_o;
            o.oob = d.oob;
            o.calls -= d.cull_calls;
            o.prims_i -= d.cull_prims;
            o.verts_i -= d.cull_verts;
            o.objs_i = d.objs_i;
            o.objs_o = d.objs_o;
        }
        out[k] = o;
    }
}

rf_status rfi_ctx_share(rf_ctx *parent, rf_ctx **out) {
    if (!parent || !out) return RF_ERR_BAD_ARG;
    *out = nullptr;
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) {
        cudaGetLastError();
        return RF_ERR_CUDA;
    }
    if (prev != parent->device && cudaSetDevice(parent->device) != cudaSuccess) {
        cudaGetLastError();
        return RF_ERR_CUDA;
    }
    rf_ctx *ctx = nullptr;
    rf_status st = rf_ctx_create(nullptr, &ctx);
    if (prev != parent->device) cudaSetDevice(prev);
    if (st) return st;
    ctx->res = parent->res;
    ctx->shared_res = true;
    ctx->tile_w = parent->tile_w;
    ctx->warps = parent->warps;
    ctx->tune_online = parent->tune_online;
    *out = ctx;
    return RF_OK;
}

cudaStream_t rfi_ctx_stream(rf_ctx *ctx) { return ctx ? ctx->stream : nullptr; }

rf_status rfi_render_batch_async(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs, StatsDev *js_host,
                                 uint32_t js_cap, std::vector<rfi_counts> &counts) {
    if (!ctx || (njobs && !jobs) || njobs > js_cap || (njobs && !js_host)) return RF_ERR_BAD_ARG;
    rf_status st = queue_batch(ctx, jobs, njobs, counts);
    if (st) return st;
    const size_t n = ctx->hjobs.size();  // jobs that reached the GPU (this batch)
    bool any = false;
    for (const rfi_counts &c : counts) any = any || c.slot >= 0;
    if (any && n)
        CK(cudaMemcpyAsync(js_host, ctx->jstats.p, n * sizeof(StatsDev), cudaMemcpyDeviceToHost,
                           ctx->stream));
    return RF_OK;
}

rf_status rfi_stamp(rf_ctx *ctx, unsigned long long *dst) {
    if (!ctx || !dst) return RF_ERR_BAD_ARG;
    CK(rfk::launch_stamp(dst, ctx->stream));
    ctx->kernels += 1;
    return RF_OK;
}
