// prof.cu — CUDA-event timing on the context stream: a start/stop timer for
// whole regions and named profiling scopes aggregated per name.
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <string>

#include "rt_internal.h"

namespace rt {

static size_t take_event(rt_ctx *ctx) {
    Prof &p = ctx->prof;
    if (p.next == p.pool.size()) {
        cudaEvent_t e;
        RT_CUDA(cudaEventCreate(&e));
        p.pool.push_back(e);
    }
    return p.next++;
}

int prof_begin(rt_ctx *ctx, const char *name) {
    Prof &p = ctx->prof;
    if (!p.on) return -1;
    size_t a = take_event(ctx);
    RT_CUDA(cudaEventRecord(p.pool[a], ctx->stream));
    p.recs.push_back(Prof::Rec{name, a, a, 0.0});
    return (int)p.recs.size() - 1;
}

void prof_end(rt_ctx *ctx, int rec, double bytes) {
    Prof &p = ctx->prof;
    if (rec < 0 || !p.on) return;
    size_t b = take_event(ctx);
    cudaEventRecord(p.pool[b], ctx->stream);
    p.recs[rec].b = b;
    p.recs[rec].bytes = bytes;
}

}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_profile_enable(rt_ctx *ctx, int32_t on) {
    if (!ctx) return RT_EINVAL;
    ctx->prof.on = on != 0;
    return RT_OK;
}

rt_status rt_profile_report(rt_ctx *ctx, char *buf, int32_t len) {
    if (!ctx || !buf || len <= 0) return RT_EINVAL;
    try {
        RT_CUDA(cudaStreamSynchronize(ctx->stream));
        struct Agg { long long n = 0; double ms = 0.0, bytes = 0.0; };
        std::map<std::string, Agg> agg;
        for (const auto &r : ctx->prof.recs) {
            if (r.b == r.a) continue;
            float ms = 0.f;
            RT_CUDA(cudaEventElapsedTime(&ms, ctx->prof.pool[r.a], ctx->prof.pool[r.b]));
            Agg &g = agg[r.name];
            g.n++;
            g.ms += ms;
            g.bytes += r.bytes;
        }
        ctx->prof.recs.clear();
        ctx->prof.next = 0;
        std::string out;
        char line[256];
        for (auto &kv : agg) {
            snprintf(line, sizeof line, "%s %lld %.6f %.6e\n", kv.first.c_str(), kv.second.n, kv.second.ms,
                     kv.second.bytes);
            out += line;
        }
        int n = (int)std::min<size_t>(out.size(), (size_t)len - 1);
        memcpy(buf, out.data(), n);
        buf[n] = 0;
        return out.size() < (size_t)len ? RT_OK : RT_EINVAL;
    } catch (const Error &e) {
        ctx->lastError = e.msg;
        return e.status;
    }
}

rt_status rt_timer_start(rt_ctx *ctx) {
    if (!ctx) return RT_EINVAL;
    if (!ctx->tStart && cudaEventCreate(&ctx->tStart) != cudaSuccess) return RT_ECUDA;
    if (!ctx->tStop && cudaEventCreate(&ctx->tStop) != cudaSuccess) return RT_ECUDA;
    return cudaEventRecord(ctx->tStart, ctx->stream) == cudaSuccess ? RT_OK : RT_ECUDA;
}

rt_status rt_timer_stop(rt_ctx *ctx, double *ms) {
    if (!ctx || !ms || !ctx->tStart) return RT_EINVAL;
    if (cudaEventRecord(ctx->tStop, ctx->stream) != cudaSuccess) return RT_ECUDA;
    if (cudaEventSynchronize(ctx->tStop) != cudaSuccess) return RT_ECUDA;
    float f = 0.f;
    if (cudaEventElapsedTime(&f, ctx->tStart, ctx->tStop) != cudaSuccess) return RT_ECUDA;
    *ms = f;
    return RT_OK;
}

rt_status rt_kernel_count(rt_ctx *ctx, int64_t *n) {
    if (!ctx || !n) return RT_EINVAL;
    *n = ctx->kernelLaunches;
    return RT_OK;
}

}  // extern "C"
