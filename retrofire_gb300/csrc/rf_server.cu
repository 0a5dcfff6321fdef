// rf_server.cu — the serving loop of include/rfgpu.h: continuous batching
// over several pipelines.  Host code only; the GPU work goes through the
// library's own batch path (rf_ctx_internal.h).
//
// A pipeline = one worker thread + one rf_ctx that shares the server
// context's meshes and textures (its own CUDA stream, scratch arenas and
// target pool) + page-locked staging for the images and the per-job
// counters.  A free pipeline takes the queued requests that fit the memory
// still unclaimed by the batches in flight, queues them as one batch and
// their read-backs on its stream, and waits for its stream only; meanwhile
// the other pipelines admit and queue what arrives, so batches overlap on
// the device and the GPU does not idle while one batch's images are copied
// out and its requests completed.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/rfgpu.h"
#include "rf_ctx_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t MAX_PIPES = 8;
constexpr uint64_t DEFAULT_STAGING = 256ull << 20;
constexpr uint64_t DEFAULT_BATCH_TRIS = 1000000ull;

struct Req {
    uint64_t ticket = 0;
    std::vector<rf_draw> draws;
    float vp[16];
    rf_context_flags flags;
    uint32_t w = 0, h = 0;
    int32_t fmt = RF_ARGB8888, has_depth = 0;
    uint32_t clear_rgba = 0;
    float depth_clear = 0.0f;
    uint32_t *color_out = nullptr;
    float *depth_out = nullptr;
    uint64_t est = 0;    // admission charge (bytes)
    uint64_t tris = 0;   // input triangles
    uint64_t img = 0;    // bytes read back
    Clock::time_point t_submit;
};

uint64_t target_bytes(uint32_t w, uint32_t h, int32_t has_depth) {
    return (uint64_t)w * h * 4u * (has_depth ? 2u : 1u);
}

uint64_t pool_key(uint32_t w, uint32_t h, int32_t fmt, int32_t depth) {
    return ((uint64_t)w << 32) | ((uint64_t)h << 8) | ((uint64_t)(fmt & 0x7F) << 1) | (depth ? 1u : 0u);
}

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Pipe {
    uint32_t id = 0;
    rf_ctx *ctx = nullptr;
    char *stage = nullptr;  // page-locked images
    size_t stage_cap = 0;
    StatsDev *js = nullptr;  // page-locked per-job counters, max_batch entries
    unsigned long long *stamps = nullptr;  // page-locked: batch start, end (GPU timer)
    std::unordered_map<uint64_t, std::vector<rf_target>> pool;  // free targets
    uint64_t pool_bytes = 0;  // pooled targets, free or in use
    std::thread th;
};

}  // namespace

struct rf_server {
    rf_ctx *ctx = nullptr;
    int device = 0;
    rf_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Req> queue;
    std::unordered_map<uint64_t, rf_result> done;
    std::unordered_set<uint64_t> live;  // issued and not yet collected
    uint64_t next_ticket = 1;
    bool stop = false;
    uint64_t batches = 0, completed = 0, next_batch = 0;
    uint64_t charged = 0, peak_charged = 0;  // admission charges in flight
    uint32_t inflight = 0, peak_inflight = 0;
    std::vector<Pipe *> pipes;
};

namespace {

rf_status acquire_target(Pipe *P, const Req &r, rf_target *out) {
    auto &fl = P->pool[pool_key(r.w, r.h, r.fmt, r.has_depth)];
    if (!fl.empty()) {
        *out = fl.back();
        fl.pop_back();
        return RF_OK;
    }
    rf_status st = rf_target_create(P->ctx, r.w, r.h, r.fmt, r.has_depth, out);
    if (st == RF_OK) P->pool_bytes += target_bytes(r.w, r.h, r.has_depth);
    return st;
}

// Keeps a pipeline's free targets within its share of half the budget
// (targets in use are charged to their requests).
void trim_pool(rf_server *S, Pipe *P) {
    const uint64_t cap = S->cfg.hbm_budget_bytes / 2 / S->pipes.size();
    for (auto &kv : P->pool) {
        const uint32_t w = (uint32_t)(kv.first >> 32), h = (uint32_t)((kv.first >> 8) & 0xFFFFFFu);
        const int32_t d = (int32_t)(kv.first & 1u);
        while (P->pool_bytes > cap && !kv.second.empty()) {
            rf_target_destroy(P->ctx, kv.second.back());
            kv.second.pop_back();
            P->pool_bytes -= target_bytes(w, h, d);
        }
    }
}

// Renders one admitted batch on pipeline P and completes its requests.
void serve(rf_server *S, Pipe *P, std::vector<Req> &batch, uint64_t batch_id,
           Clock::time_point t_admit) {
    const size_t n = batch.size();
    std::vector<rf_target> tg(n, 0);
    std::vector<rf_result> res(n);
    for (size_t i = 0; i < n; ++i) {
        res[i].status = acquire_target(P, batch[i], &tg[i]);
        if (res[i].status == RF_OK) {
            const float dc = batch[i].depth_clear;
            res[i].status = rf_target_clear(P->ctx, tg[i], &batch[i].clear_rgba, &dc);
        }
    }
    std::vector<rf_job> jobs;
    std::vector<size_t> of;  // job -> request
    for (size_t i = 0; i < n; ++i) {
        if (res[i].status != RF_OK) continue;
        rf_job j;
        memset(&j, 0, sizeof j);
        j.target = tg[i];
        j.ndraws = (uint32_t)batch[i].draws.size();
        j.draws = batch[i].draws.data();
        memcpy(j.viewport, batch[i].vp, sizeof j.viewport);
        j.flags = batch[i].flags;
        jobs.push_back(j);
        of.push_back(i);
    }
    P->stamps[0] = P->stamps[1] = 0;
    rf_status sst = rfi_stamp(P->ctx, &P->stamps[0]);
    std::vector<rf_stats> stats(jobs.size());
    std::vector<rfi_counts> counts;
    bool have_js = false;
    rf_status st = RF_OK;
    if (!jobs.empty()) {
        st = rfi_render_batch_async(P->ctx, jobs.data(), (uint32_t)jobs.size(), P->js,
                                    S->cfg.max_batch, counts);
        have_js = st == RF_OK;
    }
    if (st == RF_ERR_BAD_ARG || st == RF_ERR_BAD_HANDLE || st == RF_ERR_NON_POT_TEXTURE) {
        // Validation refused the batch before any GPU work: find the
        // offending requests by rendering each alone.
        for (size_t k = 0; k < jobs.size(); ++k)
            res[of[k]].status = rf_render_batch(P->ctx, &jobs[k], 1, &stats[k]);
    } else if (st != RF_OK) {
        for (size_t k = 0; k < jobs.size(); ++k) res[of[k]].status = st;
    }
    if (sst == RF_OK) sst = rfi_stamp(P->ctx, &P->stamps[1]);
    // Read-backs into the staging area (or straight into the caller's
    // buffers for an image larger than it), then one wait for the stream.
    std::vector<size_t> off(n, 0);
    std::vector<bool> staged(n, false);
    size_t used = 0;
    for (size_t k = 0; k < jobs.size(); ++k) {
        const size_t i = of[k];
        if (res[i].status != RF_OK) continue;
        const Req &r = batch[i];
        const size_t px = (size_t)r.w * r.h * 4;
        const bool dd = r.depth_out && r.has_depth;
        const size_t need = (r.color_out ? px : 0) + (dd ? px : 0);
        if (!need) continue;
        if (used + need <= P->stage_cap) {
            off[i] = used;
            used += need;
            staged[i] = true;
            uint32_t *c = r.color_out ? reinterpret_cast<uint32_t *>(P->stage + off[i]) : nullptr;
            float *d = dd ? reinterpret_cast<float *>(P->stage + off[i] + (c ? px : 0)) : nullptr;
            res[i].status = rf_target_read_async(P->ctx, tg[i], c, d);
        }
    }
    const rf_status ss = rf_ctx_sync(P->ctx);
    if (have_js && ss == RF_OK) rfi_batch_stats(counts, P->js, stats.data());
    for (size_t k = 0; k < jobs.size(); ++k) {
        const size_t i = of[k];
        if (res[i].status != RF_OK) continue;
        if (ss != RF_OK) {
            res[i].status = ss;
            continue;
        }
        const Req &r = batch[i];
        res[i].stats = stats[k];
        const size_t px = (size_t)r.w * r.h * 4;
        const bool dd = r.depth_out && r.has_depth;
        if (staged[i]) {
            if (r.color_out) memcpy(r.color_out, P->stage + off[i], px);
            if (dd) memcpy(r.depth_out, P->stage + off[i] + (r.color_out ? px : 0), px);
        } else if (r.color_out || dd) {
            res[i].status = rf_target_read(P->ctx, tg[i], r.color_out, dd ? r.depth_out : nullptr);
        }
    }
    const Clock::time_point t_done = Clock::now();
    const uint64_t g0 = sst == RF_OK ? P->stamps[0] : 0, g1 = sst == RF_OK ? P->stamps[1] : 0;
    for (size_t i = 0; i < n; ++i)
        if (tg[i]) P->pool[pool_key(batch[i].w, batch[i].h, batch[i].fmt, batch[i].has_depth)].push_back(tg[i]);
    trim_pool(S, P);
    uint64_t charge = 0;
    for (const Req &r : batch) charge += r.est;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (size_t i = 0; i < n; ++i) {
            rf_result &r = res[i];
            r.batch_size = (uint32_t)n;
            r.batch_id = batch_id;
            r.queue_ms = ms_between(batch[i].t_submit, t_admit);
            r.render_ms = g1 > g0 ? (double)(g1 - g0) * 1e-6 : 0.0;
            r.total_ms = ms_between(batch[i].t_submit, t_done);
            r.gpu_start_ns = g0;
            r.gpu_end_ns = g1;
            r.pipeline = P->id;
            S->done[batch[i].ticket] = r;
        }
        S->completed += n;
        S->batches += 1;
        S->charged -= charge;
        S->inflight -= 1;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();  // memory and a pipeline came free
}

// Whether the queue's first request may be admitted now.
bool can_admit(const rf_server *S) {
    if (S->queue.empty()) return false;
    return S->charged == 0 || S->charged + S->queue.front().est <= S->cfg.hbm_budget_bytes;
}

void worker_main(rf_server *S, Pipe *P) {
    cudaSetDevice(S->device);
    for (;;) {
        std::vector<Req> batch;
        uint64_t batch_id = 0;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return (S->stop && S->queue.empty()) || can_admit(S); });
            if (S->queue.empty()) break;  // stop requested and drained
            uint64_t sum = 0, tris = 0, img = 0;
            while (!S->queue.empty() && batch.size() < S->cfg.max_batch) {
                const Req &r = S->queue.front();
                if (!batch.empty()) {
                    if (S->charged + sum + r.est > S->cfg.hbm_budget_bytes) break;
                    if (tris + r.tris > S->cfg.max_batch_tris) break;
                    if (img + r.img > P->stage_cap) break;
                } else if (S->charged && S->charged + r.est > S->cfg.hbm_budget_bytes) {
                    break;
                }
                sum += r.est;
                tris += r.tris;
                img += r.img;
                batch.push_back(std::move(S->queue.front()));
                S->queue.pop_front();
            }
            if (batch.empty()) continue;
            S->charged += sum;
            S->peak_charged = std::max(S->peak_charged, S->charged);
            S->inflight += 1;
            S->peak_inflight = std::max(S->peak_inflight, S->inflight);
            batch_id = ++S->next_batch;
        }
        // Another pipeline may take what is left of the queue now.
        S->cv_work.notify_all();
        serve(S, P, batch, batch_id, Clock::now());
    }
}

void destroy_pipe(Pipe *P) {
    for (auto &kv : P->pool)
        for (rf_target t : kv.second) rf_target_destroy(P->ctx, t);
    if (P->ctx) rf_ctx_destroy(P->ctx);
    if (P->stage) cudaFreeHost(P->stage);
    if (P->js) cudaFreeHost(P->js);
    if (P->stamps) cudaFreeHost(P->stamps);
    delete P;
}

void destroy_server(rf_server *S) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(S->device);
    for (Pipe *P : S->pipes) destroy_pipe(P);
    S->pipes.clear();
    cudaSetDevice(prev);
    delete S;
}

}  // namespace

extern "C" {

rf_status rf_server_create(rf_ctx *ctx, const rf_server_config *cfg, rf_server **out) {
    if (!ctx || !out) return RF_ERR_BAD_ARG;
    *out = nullptr;
    int32_t dev = 0;
    rf_status st = rf_ctx_device(ctx, &dev);
    if (st) return st;
    rf_server *S = new (std::nothrow) rf_server();
    if (!S) return RF_ERR_OOM;
    S->ctx = ctx;
    S->device = dev;
    if (cfg) S->cfg = *cfg;
    if (S->cfg.hbm_budget_bytes == 0) S->cfg.hbm_budget_bytes = 64ull << 30;
    if (S->cfg.max_batch == 0) S->cfg.max_batch = 256;
    if (S->cfg.inflight == 0) S->cfg.inflight = 2;
    if (S->cfg.inflight > MAX_PIPES) {
        delete S;
        return RF_ERR_BAD_ARG;
    }
    if (S->cfg.staging_bytes == 0) S->cfg.staging_bytes = DEFAULT_STAGING;
    if (S->cfg.max_batch_tris == 0) S->cfg.max_batch_tris = DEFAULT_BATCH_TRIS;
    // The caller's queued work on the context finishes before the
    // pipelines read its meshes and textures.
    st = rf_ctx_sync(ctx);
    if (st) {
        delete S;
        return st;
    }
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(dev);
    for (uint32_t p = 0; p < S->cfg.inflight && st == RF_OK; ++p) {
        Pipe *P = new (std::nothrow) Pipe();
        if (!P) {
            st = RF_ERR_OOM;
            break;
        }
        P->id = p;
        S->pipes.push_back(P);
        st = rfi_ctx_share(ctx, &P->ctx);
        if (st) break;
        if (cudaHostAlloc(reinterpret_cast<void **>(&P->stage), S->cfg.staging_bytes, cudaHostAllocDefault) !=
                cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void **>(&P->js), (size_t)S->cfg.max_batch * sizeof(StatsDev),
                          cudaHostAllocDefault) != cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void **>(&P->stamps), 2 * sizeof(unsigned long long),
                          cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            st = RF_ERR_OOM;
            break;
        }
        P->stage_cap = S->cfg.staging_bytes;
    }
    cudaSetDevice(prev);
    if (st) {
        destroy_server(S);
        return st;
    }
    try {
        for (Pipe *P : S->pipes) P->th = std::thread(worker_main, S, P);
    } catch (...) {
        {
            std::lock_guard<std::mutex> lk(S->mu);
            S->stop = true;
        }
        S->cv_work.notify_all();
        for (Pipe *P : S->pipes)
            if (P->th.joinable()) P->th.join();
        destroy_server(S);
        return RF_ERR_OOM;
    }
    *out = S;
    return RF_OK;
}

rf_status rf_server_submit(rf_server *S, const rf_request *q, uint64_t *ticket) {
    if (!S || !q || !ticket || (q->ndraws && !q->draws)) return RF_ERR_BAD_ARG;
    if (!q->w || !q->h || q->w > RF_MAX_TARGET_DIM || q->h > RF_MAX_TARGET_DIM) return RF_ERR_BAD_ARG;
    if (q->pixfmt < RF_ARGB8888 || q->pixfmt > RF_BGRA8888) return RF_ERR_BAD_ARG;
    Req r;
    r.draws.assign(q->draws, q->draws + q->ndraws);
    memcpy(r.vp, q->viewport, sizeof r.vp);
    r.flags = q->flags;
    r.w = q->w;
    r.h = q->h;
    r.fmt = q->pixfmt;
    r.has_depth = q->has_depth ? 1 : 0;
    r.clear_rgba = q->clear_rgba;
    r.depth_clear = q->depth_clear;
    r.color_out = q->color_out;
    r.depth_out = q->depth_out;
    uint64_t est = target_bytes(q->w, q->h, r.has_depth), tris = 0;
    for (const rf_draw &d : r.draws) {
        // The meshes table is read-only while the server runs, so this
        // lookup may run beside the pipelines.
        uint32_t nv = 0, nt = 0;
        if (rf_mesh_info(S->ctx, d.mesh, &nv, &nt, nullptr) == RF_OK) {
            est += (uint64_t)nt * RF_SERVE_BYTES_PER_TRI + (uint64_t)nv * RF_SERVE_BYTES_PER_VERT;
            tris += nt;
        }
    }
    // Tile masks and their summary words at the narrowest tiling (8 x 32).
    const uint64_t tiles = (uint64_t)((q->w + 7) / 8) * ((q->h + 31) / 32);
    const uint64_t mw = (tris + 31) / 32;
    est += tiles * (mw + (mw + 31) / 32) * 4u;
    r.est = est;
    r.tris = tris;
    const uint64_t px = (uint64_t)q->w * q->h * 4u;
    r.img = (q->color_out ? px : 0) + (q->depth_out && r.has_depth ? px : 0);
    if (est > S->cfg.hbm_budget_bytes) return RF_ERR_OVER_BUDGET;
    r.t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return RF_ERR_BAD_ARG;
        r.ticket = S->next_ticket++;
        *ticket = r.ticket;
        S->live.insert(r.ticket);
        S->queue.push_back(std::move(r));
    }
    S->cv_work.notify_one();
    return RF_OK;
}

rf_status rf_server_wait(rf_server *S, uint64_t ticket, uint32_t timeout_ms, rf_result *out) {
    if (!S) return RF_ERR_BAD_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    if (!S->live.count(ticket)) return RF_ERR_BAD_ARG;
    auto ready = [&] { return S->done.count(ticket) != 0; };
    if (timeout_ms == UINT32_MAX) {
        S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return RF_ERR_TIMEOUT;
    }
    auto it = S->done.find(ticket);
    if (out) *out = it->second;
    S->done.erase(it);
    S->live.erase(ticket);
    return RF_OK;
}

rf_status rf_server_counts(rf_server *S, uint64_t *batches, uint64_t *completed, uint64_t *queued) {
    if (!S) return RF_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (batches) *batches = S->batches;
    if (completed) *completed = S->completed;
    if (queued) *queued = S->queue.size();
    return RF_OK;
}

rf_status rf_server_memory(rf_server *S, uint64_t *charged, uint64_t *peak_charged,
                           uint32_t *peak_inflight) {
    if (!S) return RF_ERR_BAD_ARG;
    std::lock_guard<std::mutex> lk(S->mu);
    if (charged) *charged = S->charged;
    if (peak_charged) *peak_charged = S->peak_charged;
    if (peak_inflight) *peak_inflight = S->peak_inflight;
    return RF_OK;
}

rf_status rf_server_destroy(rf_server *S) {
    if (!S) return RF_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (Pipe *P : S->pipes)
        if (P->th.joinable()) P->th.join();
    destroy_server(S);
    return RF_OK;
}

}  // extern "C"
