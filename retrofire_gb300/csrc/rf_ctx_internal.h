// rf_ctx_internal.h — the library-internal interface between the context
// code (rf_api.cu) and the serving loop (rf_server.cu).  Not part of the C
// ABI: nothing here is exported under a public name.
#ifndef RF_CTX_INTERNAL_H
#define RF_CTX_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/rfgpu.h"
#include "rf_internal.cuh"

// Host-side counts of one job of a batch (render.rs:152-155) and its slot
// among the jobs that reached the GPU (-1: it had no triangles).
struct rfi_counts {
    uint64_t calls = 0, prims_i = 0, verts_i = 0;
    int32_t slot = -1;
};

// A context on the same device as `parent` that reads the parent's meshes
// and textures (which must not change while it lives) and has its own
// stream, targets, scratch arenas and tuning state.  Destroying it frees
// only its own objects.
rf_status rfi_ctx_share(rf_ctx *parent, rf_ctx **out);

// The stream the context's rendering is ordered on.
cudaStream_t rfi_ctx_stream(rf_ctx *ctx);

// rf_render_batch without waiting: the batch is queued on the context's
// stream, followed by a copy of its per-job device counters into js_host
// (page-locked, room for js_cap entries; njobs <= js_cap).  After the
// stream has reached that point, rfi_batch_stats gives each job's stats.
rf_status rfi_render_batch_async(rf_ctx *ctx, const rf_job *jobs, uint32_t njobs,
                                 StatsDev *js_host, uint32_t js_cap,
                                 std::vector<rfi_counts> &counts);
void rfi_batch_stats(const std::vector<rfi_counts> &counts, const StatsDev *js_host,
                     rf_stats *out);

// Queues a write of the GPU's global nanosecond timer into *dst (device or
// page-locked host memory) on the context's stream.
rf_status rfi_stamp(rf_ctx *ctx, unsigned long long *dst);

#endif
