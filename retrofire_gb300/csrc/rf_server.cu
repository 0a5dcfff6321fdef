// rf_server.cu — the serving loop of include/rfgpu.h: a worker thread that
// owns one rf_ctx, admits queued requests against a device-memory budget
// and renders each admitted group as one rf_render_batch (continuous
// batching).  Host code only; every GPU step goes through the C ABI.
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

namespace {

using Clock = std::chrono::steady_clock;

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
    uint64_t est = 0;
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
    uint64_t batches = 0, completed = 0;
    std::thread worker;
    // Worker-only state: free targets by (w, h, format, depth).
    std::unordered_map<uint64_t, std::vector<rf_target>> pool;
    uint64_t pool_bytes = 0;  // all pooled targets, free or in use
    // Page-locked staging of a batch's images (grow-only): the read-backs
    // run at page-locked speed, then the host copies into the callers'
    // buffers.
    char *stage = nullptr;
    size_t stage_cap = 0;
};

namespace {

rf_status acquire_target(rf_server *S, const Req &r, rf_target *out) {
    auto &fl = S->pool[pool_key(r.w, r.h, r.fmt, r.has_depth)];
    if (!fl.empty()) {
        *out = fl.back();
        fl.pop_back();
        return RF_OK;
    }
    rf_status st = rf_target_create(S->ctx, r.w, r.h, r.fmt, r.has_depth, out);
    if (st == RF_OK) S->pool_bytes += target_bytes(r.w, r.h, r.has_depth);
    return st;
}

// Keeps the free targets within half the budget; the ones in use are
// counted in the admitted batch's estimate.
void trim_pool(rf_server *S) {
    const uint64_t cap = S->cfg.hbm_budget_bytes / 2;
    for (auto &kv : S->pool) {
        const uint32_t w = (uint32_t)(kv.first >> 32), h = (uint32_t)((kv.first >> 8) & 0xFFFFFFu);
        const int32_t d = (int32_t)(kv.first & 1u);
        while (S->pool_bytes > cap && !kv.second.empty()) {
            rf_target_destroy(S->ctx, kv.second.back());
            kv.second.pop_back();
            S->pool_bytes -= target_bytes(w, h, d);
        }
    }
}

void serve(rf_server *S, std::vector<Req> &batch, uint64_t batch_id) {
    const size_t n = batch.size();
    const Clock::time_point t_start = Clock::now();
    std::vector<rf_target> tg(n, 0);
    std::vector<rf_result> res(n);
    for (size_t i = 0; i < n; ++i) {
        res[i].status = acquire_target(S, batch[i], &tg[i]);
        if (res[i].status == RF_OK) {
            const float dc = batch[i].depth_clear;
            res[i].status = rf_target_clear(S->ctx, tg[i], &batch[i].clear_rgba, &dc);
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
    std::vector<rf_stats> stats(jobs.size());
    rf_status st = jobs.empty() ? RF_OK : rf_render_batch(S->ctx, jobs.data(), (uint32_t)jobs.size(), stats.data());
    if (st == RF_ERR_BAD_ARG || st == RF_ERR_BAD_HANDLE || st == RF_ERR_NON_POT_TEXTURE) {
        // Validation refused the batch before any GPU work: find the
        // offending requests by rendering each alone.
        for (size_t k = 0; k < jobs.size(); ++k)
            res[of[k]].status = rf_render_batch(S->ctx, &jobs[k], 1, &stats[k]);
    } else if (st != RF_OK) {
        for (size_t k = 0; k < jobs.size(); ++k) res[of[k]].status = st;
    }
    const Clock::time_point t_gpu = Clock::now();
    // Read-backs into the staging area, one wait, then host copies.
    size_t need = 0;
    std::vector<size_t> off(n, 0);
    for (size_t k = 0; k < jobs.size(); ++k) {
        const size_t i = of[k];
        if (res[i].status != RF_OK) continue;
        off[i] = need;
        const size_t px = (size_t)batch[i].w * batch[i].h * 4;
        if (batch[i].color_out) need += px;
        if (batch[i].depth_out && batch[i].has_depth) need += px;
    }
    bool staged = false;
    if (need > S->stage_cap) {
        if (S->stage) cudaFreeHost(S->stage);
        S->stage = nullptr;
        S->stage_cap = 0;
        const size_t cap = need + need / 2;
        if (cudaHostAlloc(reinterpret_cast<void **>(&S->stage), cap, cudaHostAllocDefault) == cudaSuccess) {
            S->stage_cap = cap;
        } else {
            S->stage = nullptr;
            cudaGetLastError();  // the direct reads below stand in; later launches must not see it
        }
    }
    if (S->stage && need <= S->stage_cap) {
        staged = true;
        for (size_t k = 0; k < jobs.size(); ++k) {
            const size_t i = of[k];
            if (res[i].status != RF_OK) continue;
            res[i].stats = stats[k];
            const size_t px = (size_t)batch[i].w * batch[i].h * 4;
            uint32_t *c = batch[i].color_out ? reinterpret_cast<uint32_t *>(S->stage + off[i]) : nullptr;
            float *d = (batch[i].depth_out && batch[i].has_depth)
                           ? reinterpret_cast<float *>(S->stage + off[i] + (c ? px : 0))
                           : nullptr;
            if (c || d) res[i].status = rf_target_read_async(S->ctx, tg[i], c, d);
        }
        const rf_status ss = rf_ctx_sync(S->ctx);
        for (size_t k = 0; k < jobs.size(); ++k) {
            const size_t i = of[k];
            if (res[i].status != RF_OK) continue;
            if (ss != RF_OK) {
                res[i].status = ss;
                continue;
            }
            const size_t px = (size_t)batch[i].w * batch[i].h * 4;
            if (batch[i].color_out) memcpy(batch[i].color_out, S->stage + off[i], px);
            if (batch[i].depth_out && batch[i].has_depth)
                memcpy(batch[i].depth_out, S->stage + off[i] + (batch[i].color_out ? px : 0), px);
        }
    }
    if (!staged) {  // no page-locked memory to be had: direct reads
        for (size_t k = 0; k < jobs.size(); ++k) {
            const size_t i = of[k];
            if (res[i].status != RF_OK) continue;
            res[i].stats = stats[k];
            if (batch[i].color_out || (batch[i].depth_out && batch[i].has_depth))
                res[i].status = rf_target_read(S->ctx, tg[i], batch[i].color_out,
                                               batch[i].has_depth ? batch[i].depth_out : nullptr);
        }
    }
    const Clock::time_point t_done = Clock::now();
    for (size_t i = 0; i < n; ++i)
        if (tg[i]) S->pool[pool_key(batch[i].w, batch[i].h, batch[i].fmt, batch[i].has_depth)].push_back(tg[i]);
    trim_pool(S);
    {
        std::lock_guard<std::mutex> lk(S->mu);
        for (size_t i = 0; i < n; ++i) {
            rf_result &r = res[i];
            r.batch_size = (uint32_t)n;
            r.batch_id = batch_id;
            r.queue_ms = ms_between(batch[i].t_submit, t_start);
            r.render_ms = ms_between(t_start, t_gpu);
            r.total_ms = ms_between(batch[i].t_submit, t_done);
            S->done[batch[i].ticket] = r;
        }
        S->completed += n;
        S->batches += 1;
    }
    S->cv_done.notify_all();
}

void worker_main(rf_server *S) {
    cudaSetDevice(S->device);
    uint64_t batch_id = 0;
    for (;;) {
        std::vector<Req> batch;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
            if (S->queue.empty()) break;  // stop requested and drained
            uint64_t sum = 0;
            while (!S->queue.empty() && batch.size() < S->cfg.max_batch) {
                Req &r = S->queue.front();
                if (!batch.empty() && sum + r.est > S->cfg.hbm_budget_bytes) break;
                sum += r.est;
                batch.push_back(std::move(r));
                S->queue.pop_front();
            }
        }
        serve(S, batch, ++batch_id);
    }
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
    // The caller's queued work on the context finishes before the worker
    // takes it over.
    st = rf_ctx_sync(ctx);
    if (st) {
        delete S;
        return st;
    }
    try {
        S->worker = std::thread(worker_main, S);
    } catch (...) {
        delete S;
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
    uint64_t est = target_bytes(q->w, q->h, r.has_depth);
    for (const rf_draw &d : r.draws) {
        // The meshes map is read-only while the server runs (the worker
        // creates targets only), so this lookup may run beside it.
        uint32_t nv = 0, nt = 0;
        if (rf_mesh_info(S->ctx, d.mesh, &nv, &nt, nullptr) == RF_OK)
            est += (uint64_t)nt * RF_SERVE_BYTES_PER_TRI + (uint64_t)nv * RF_SERVE_BYTES_PER_VERT;
    }
    r.est = est;
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

rf_status rf_server_destroy(rf_server *S) {
    if (!S) return RF_ERR_BAD_ARG;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    if (S->worker.joinable()) S->worker.join();
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(S->device);
    for (auto &kv : S->pool)
        for (rf_target t : kv.second) rf_target_destroy(S->ctx, t);
    if (S->stage) cudaFreeHost(S->stage);
    cudaSetDevice(prev);
    delete S;
    return RF_OK;
}

}  // extern "C"
