// Render orchestration: first hits, integrator dispatch (megakernel, wavefront, BDPT), resolve,
// timing, and the wavefront autotuner.
#include "api_internal.h"
#include "adjoint.h"
#include "wavefront.h"

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>

namespace e8g {

namespace {

struct WfCounters { // mirrors the device Counters of wavefront.cu
    unsigned long long next_path;
    uint32_t shadow_n, ext_n, busy, pad[3];
};

// The split form of E8G_MODE_BDPT_POWER. Paths go in chunks (at most 2^26, and at most 32 GiB or
// half the free device memory for subpaths, connection lists and shadow queue; fewer when the
// memory limit refuses that: every chunk ends with a tail of walk bounces, and the 1280x720,
// 32-spp frame took 46.0 ms in two chunks of 16 GiB against 43.5 ms in one). Per
// chunk: the walk wavefront (a captured graph of two bounces, replayed until every slot is idle
// and the chunk's paths are taken), then the connection list in pieces of at most the shadow
// queue's length: evaluation, then the queue's shadow rays.
e8g_status run_bdpt_split(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb) {
    const uint32_t ml = std::min<uint32_t>(A.bdpt_max_len, 16);
    uint64_t chunk = std::min<uint64_t>({A.total_paths, kBdwMaxChunk});
    chunk = std::max<uint64_t>(chunk, 1);
    // the chunk's arrays from base (sizes only when base is null), each 256-byte aligned; the
    // shadow queue holds every entry of a chunk of up to 2^24 entries, 2^24 beyond
    auto carve = [&](char *base, uint64_t n, WfSlots *Q, uint64_t **range, size_t *bytes) {
        BdwChunk C{};
        size_t off = 0;
        auto take = [&](size_t sz) {
            char *r = base ? base + off : nullptr;
            off += (sz + 255) & ~size_t(255);
            return r;
        };
        const size_t entries = n * ml * (ml + 1);
        const size_t qlen = std::max<size_t>(std::min<size_t>(entries, size_t(1) << 24), 1);
        C.vtx = reinterpret_cast<float4 *>(take(n * ml * 6 * 16));
        C.info = reinterpret_cast<int4 *>(take(n * 16));
        C.o0 = reinterpret_cast<float4 *>(take(n * 16));
        C.conn = reinterpret_cast<uint64_t *>(take(entries * 8));
        C.conn_n = reinterpret_cast<uint32_t *>(take(16));
        C.max_len = ml;
        *Q = WfSlots{};
        Q->capacity = static_cast<uint32_t>(qlen);
        Q->sh_o = reinterpret_cast<float4 *>(take(qlen * 16));
        Q->sh_d = reinterpret_cast<float4 *>(take(qlen * 16));
        Q->sh_c = reinterpret_cast<float4 *>(take(qlen * 16));
        Q->counters = take(wf_counters_bytes());
        *range = reinterpret_cast<uint64_t *>(take(16));
        *bytes = off;
        return C;
    };
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        free_b = size_t(8) << 30;
    }
    const size_t budget = std::min<size_t>(size_t(32) << 30, (free_b + c->b_bdw.bytes) / 2);
    cudaError_t e = cudaErrorMemoryAllocation;
    size_t need = 0;
    WfSlots Q{};
    uint64_t *range = nullptr;
    while (true) {
        carve(nullptr, chunk, &Q, &range, &need);
        e = need <= budget || chunk <= 4096 ? c->b_bdw.reserve(need) : cudaErrorMemoryAllocation;
        if (e == cudaSuccess || chunk <= 4096)
            break;
        cudaGetLastError();
        chunk /= 2;
    }
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bidirectional subpath buffers");
    BdwChunk C = carve(static_cast<char *>(c->b_bdw.ptr), chunk, &Q, &range, &need);
    // the walk's slots
    const uint32_t slots = static_cast<uint32_t>(std::min<uint64_t>((chunk + 255) / 256 * 256, 1u << 23));
    e = c->b_wf.reserve(wf_total_bytes(slots));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bidirectional walk slots");
    WfSlots W = wf_carve(c->b_wf.ptr, slots);
    // refill threshold of the trace kernels (threshold 8 against 16: 42.3 against 43.0 ms per
    // 1280x720, 32-spp frame)
    const uint32_t threshold = c->dev.layout == 0 || c->dev.layout == 2 ? 8u : 0u;
    const int grid_walk = static_cast<int>(std::min<uint64_t>((slots + 255) / 256, static_cast<uint64_t>(c->num_sms) * 8));
    const int grid_eval = persistent_grid(c, bdpt_eval_blocks_per_sm());
    const int grid_trace = persistent_grid(c, wf_trace_blocks_per_sm(c->dev.layout, threshold));
    auto const *fh = static_cast<FirstHit const *>(c->b_fh.ptr);
    constexpr uint32_t kBounces = 2;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bidirectional walk capture");
    for (uint32_t k = 0; k < kBounces; k++) {
        wf_enqueue_reset(W, c->stream);
        launch_bdpt_walk(c->dev, A, fh, path_rgb, C, W, range, grid_walk, c->stream);
        wf_enqueue_trace(c->dev, A, W, nullptr, nullptr, grid_trace, threshold, c->stream);
    }
    e = cudaStreamEndCapture(c->stream, &graph);
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        return cuda_fail(c, e, "bidirectional walk graph");
    }
    auto *host = static_cast<WfCounters *>(c->host_pinned);
    auto *host_range = reinterpret_cast<uint64_t *>(static_cast<char *>(c->host_pinned) + 32);
    auto *host_conn = reinterpret_cast<uint32_t *>(static_cast<char *>(c->host_pinned) + 48);
    // a path takes at most 2 max_len + 2 walk bounces; slots refill continuously
    const uint64_t max_replays = ((chunk + slots - 1) / slots + 1) * (2 * ml + 4) / kBounces + 16;
    bool cancelled = false, stuck = false;
    for (uint64_t first = 0; first < A.total_paths && e == cudaSuccess; first += chunk) {
        if (take_cancel(c)) {
            cancelled = true;
            break;
        }
        C.first = first;
        C.count = static_cast<uint32_t>(std::min<uint64_t>(chunk, A.total_paths - first));
        host_range[0] = C.first;
        host_range[1] = C.count;
        e = cudaMemcpyAsync(range, host_range, 16, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess)
            e = wf_init(W, c->stream);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(C.conn_n, 0, sizeof(uint32_t), c->stream);
        uint64_t r = 0;
        for (; r < max_replays && e == cudaSuccess; r++) {
            e = cudaGraphLaunch(exec, c->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(host, W.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(host_conn, C.conn_n, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
            if (e == cudaSuccess)
                e = cudaStreamSynchronize(c->stream);
            c->launches += 4 * kBounces;
            if (e == cudaSuccess && host->busy == 0 && host->next_path >= C.count)
                break;
        }
        if (e != cudaSuccess)
            break;
        if (r == max_replays) {
            stuck = true;
            break;
        }
        const uint32_t n_conn = *host_conn;
        for (uint32_t q0 = 0; q0 < n_conn && e == cudaSuccess; q0 += Q.capacity) {
            const uint32_t n = std::min<uint32_t>(Q.capacity, n_conn - q0);
            e = cudaMemsetAsync(Q.counters, 0, wf_counters_bytes(), c->stream);
            if (e != cudaSuccess)
                break;
            launch_bdpt_eval(c->dev, accum, path_rgb, C, Q, q0, n, grid_eval, c->stream);
            wf_enqueue_trace(c->dev, A, Q, accum, path_rgb, grid_trace, threshold, c->stream);
            c->launches += 3;
            e = cudaGetLastError();
        }
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "bidirectional split run");
    if (cancelled)
        return fail(c, E8G_ERR_CANCELLED, "render cancelled");
    if (stuck)
        return fail(c, E8G_ERR_INTERNAL, "bidirectional walk did not drain");
    return E8G_OK;
}

e8g_status run_integrator(e8g_ctx *c, e8g_render_params const *p, RenderArgs const &A, float4 *accum, float *path_rgb,
                          unsigned long long *d_counts) {
    // the counted run traces the same rays one thread per path
    if (p->integrator == E8G_INTEGRATOR_WAVEFRONT && p->mode == E8G_MODE_BDPT_POWER && !d_counts)
        return run_bdpt_split(c, A, accum, path_rgb);
    if (p->integrator == E8G_INTEGRATOR_WAVEFRONT && p->mode == E8G_MODE_MIS && !d_counts)
        return c->wf_concurrent ? run_wavefront_concurrent(c, A, accum, path_rgb, c->wf_capacity, c->wf_bounces,
                                                           c->wf_threshold)
                                : run_wavefront(c, A, accum, path_rgb, c->wf_capacity, c->wf_bounces, c->wf_threshold);
    cudaError_t e = cudaMemsetAsync(c->b_work.ptr, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "work counter");
    auto *work = static_cast<unsigned long long *>(c->b_work.ptr);
    auto const *fh = static_cast<FirstHit const *>(c->b_fh.ptr);
    if (A.mode == E8G_MODE_REF_BDPT || A.mode == E8G_MODE_BDPT_POWER || A.mode == E8G_MODE_REF_LT2) {
        launch_bdpt(c->dev, A, fh, accum, path_rgb, work, persistent_grid(c, bdpt_blocks_per_sm()), c->stream,
                    d_counts);
    } else {
        int grid = persistent_grid(c, megakernel_blocks_per_sm());
        launch_megakernel(c->dev, A, fh, accum, path_rgb, work, d_counts, grid, c->stream,
                          p->integrator == E8G_INTEGRATOR_PLAIN);
    }
    c->launches++;
    return E8G_OK;
}

// The firefly clamp compares each pixel with its neighbours within one sample of the whole image
// (renderer.cpp:46-83), so samples are rendered in chunks of K per-sample images (sample-major
// per-path output, at most 1 GiB), each chunk clamped and added to the accumulator in sample
// order. The paths and their streams are those of the unclamped render.
e8g_status run_firefly(e8g_ctx *c, e8g_render_params const *p, RenderArgs const &A, float4 *accum,
                       unsigned long long *d_counts) {
    size_t npix = static_cast<size_t>(p->width) * p->height;
    size_t per_sample = npix * 3 * sizeof(float);
    uint32_t K = static_cast<uint32_t>(std::max<size_t>(1, std::min<size_t>(p->spp, (size_t(1) << 30) / per_sample)));
    cudaError_t e = c->b_ff.reserve(K * per_sample);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "firefly sample images");
    float *est = static_cast<float *>(c->b_ff.ptr);
    for (uint32_t s0 = 0; s0 < p->spp; s0 += K) {
        if (take_cancel(c))
            return fail(c, E8G_ERR_CANCELLED, "render cancelled");
        uint32_t k = std::min(K, p->spp - s0);
        RenderArgs B = A;
        B.spp = k;
        B.sample_offset = A.sample_offset + s0;
        B.total_paths = static_cast<uint64_t>(A.paths_per_sample) * k;
        B.sample_major = 1;
        e = cudaMemsetAsync(est, 0, k * per_sample, c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "firefly clear");
        e8g_status s = run_integrator(c, p, B, nullptr, est, d_counts);
        if (s != E8G_OK)
            return s;
        launch_firefly(est, k, p->width, p->height, accum, c->stream);
        c->launches++;
    }
    return E8G_OK;
}

} // namespace

e8g_status run_wavefront(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t capacity,
                         uint32_t bounces, uint32_t threshold, BatchDev const *B, FirstHit const *fh_all) {
    uint64_t total = B ? B->total_paths : A.total_paths;
    uint32_t layout = B ? 2u : c->dev.layout;
    if (B && threshold == 0)
        threshold = 16; // the many-scene form always traces with dynamic fetch
    uint64_t want = std::max<uint64_t>(total, 1024);
    uint32_t Q = static_cast<uint32_t>(std::min<uint64_t>(capacity, (want + 255) / 256 * 256));
    cudaError_t e = c->b_wf.reserve(wf_total_bytes(Q));
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront slots");
    WfSlots W = wf_carve(c->b_wf.ptr, Q);
    e = wf_init(W, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront init");
    uint32_t shade_variant = B ? 0u : c->wf_shade_variant;
    int shade_grid = wf_shade_grid(shade_variant, Q, c->num_sms);
    int trace_grid = persistent_grid(c, wf_trace_blocks_per_sm(layout, threshold));
    auto const *fh = B ? fh_all : static_cast<FirstHit const *>(c->b_fh.ptr);
    // capture `bounces` bounces once, replay until no slot is busy and no path is left
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool timed = c->kernel_timing;
    while (timed && c->kt_events.size() < 3 * static_cast<size_t>(bounces)) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreate(&ev);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "kernel timing events");
        c->kt_events.push_back(ev);
    }
    uint32_t traces_per_bounce = layout == 2 && threshold > 0 ? 1u : 2u;
    e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront capture");
    for (uint32_t k = 0; k < bounces; k++)
        wf_enqueue_bounce(c->dev, A, fh, W, accum, path_rgb, shade_grid, trace_grid, threshold, total, B, c->stream,
                          timed ? c->kt_events.data() + 3 * k : nullptr, shade_variant);
    e = cudaStreamEndCapture(c->stream, &graph);
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        return cuda_fail(c, e, "wavefront graph");
    }
    auto *host = static_cast<WfCounters *>(c->host_pinned);
    // every path needs at most kHardDepth + 2 bounces; slots refill continuously
    uint64_t max_replays = ((total + Q - 1) / Q + 1) * (kHardDepth + 2) / bounces + 16;
    uint64_t r = 0;
    bool cancelled = false;
    for (; r < max_replays; r++) {
        if (take_cancel(c)) {
            cancelled = true;
            break;
        }
        e = cudaGraphLaunch(exec, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(host, W.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess)
            break;
        c->launches += (layout == 2 && threshold > 0 ? 3 : 4) * bounces; // reset, shade, trace(s)
        if (timed) { // the replay has finished: read its bounces' event pairs
            for (uint32_t k = 0; k < bounces; k++) {
                float a = 0, b = 0;
                cudaEventElapsedTime(&a, c->kt_events[3 * k], c->kt_events[3 * k + 1]);
                cudaEventElapsedTime(&b, c->kt_events[3 * k + 1], c->kt_events[3 * k + 2]);
                c->kt_shade_ms += a;
                c->kt_trace_ms += b;
            }
            c->kt_trace_launches += traces_per_bounce * bounces;
        }
        if (host->busy == 0 && host->next_path >= total)
            break;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront run");
    if (cancelled)
        return fail(c, E8G_ERR_CANCELLED, "render cancelled");
    if (r == max_replays)
        return fail(c, E8G_ERR_INTERNAL, "wavefront did not drain");
    return E8G_OK;
}

// The concurrent wavefront: the slots split into two pools A and B with their own queues and
// counters (one path counter shared), captured on two streams in anti-phase — while A shades, B
// traces, then A traces while B shades — with a two-way event join after every phase. Each kernel
// is launched for half of the SM's residency, so a shading kernel (waiting on its scene gathers)
// and a trace kernel (issue-bound on the eight-box tests) share every SM. Pool B's last phase of a
// replay is a shading, so the run ends only when B's queues are empty too.
e8g_status run_wavefront_concurrent(e8g_ctx *c, RenderArgs const &A, float4 *accum, float *path_rgb, uint32_t capacity,
                                    uint32_t bounces, uint32_t threshold) {
    uint64_t total = A.total_paths;
    uint32_t layout = c->dev.layout;
    uint64_t want = std::max<uint64_t>(total, 2048);
    uint32_t Qh = static_cast<uint32_t>(std::min<uint64_t>(capacity / 2, (want / 2 + 255) / 256 * 256));
    Qh = std::max<uint32_t>(Qh, 256);
    size_t pool = (wf_total_bytes(Qh) + 255) & ~static_cast<size_t>(255);
    cudaError_t e = c->b_wf.reserve(2 * pool);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront slots");
    if (!c->stream2) {
        e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&c->ev_a, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&c->ev_b, cudaEventDisableTiming);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "second stream");
    }
    WfSlots WA = wf_carve(c->b_wf.ptr, Qh);
    WfSlots WB = wf_carve(static_cast<char *>(c->b_wf.ptr) + pool, Qh);
    WB.next_path = WA.next_path;
    e = wf_init(WA, c->stream);
    if (e == cudaSuccess)
        e = wf_init(WB, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront init");
    uint32_t v = c->wf_shade_variant;
    int shade_grid = c->num_sms * std::max(1, wf_shade_blocks(v) / 2);
    int trace_grid = c->num_sms * std::max(1, wf_trace_blocks_per_sm(layout, threshold) / 2);
    auto const *fh = static_cast<FirstHit const *>(c->b_fh.ptr);
    cudaStream_t s0 = c->stream, s1 = c->stream2;
    bool timed = c->kernel_timing;
    size_t nev = 8 * static_cast<size_t>(bounces); // start and end of each of the four kernels of a step
    while (timed && c->kt_events.size() < nev) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreate(&ev);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "kernel timing events");
        c->kt_events.push_back(ev);
    }
    auto mark = [&](size_t k, cudaStream_t st) {
        if (timed)
            cudaEventRecordWithFlags(c->kt_events[k], st, cudaEventRecordExternal);
    };
    auto join = [&]() {
        cudaEventRecord(c->ev_a, s0);
        cudaEventRecord(c->ev_b, s1);
        cudaStreamWaitEvent(s0, c->ev_b, 0);
        cudaStreamWaitEvent(s1, c->ev_a, 0);
    };
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    e = cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "wavefront capture");
    cudaEventRecord(c->ev_a, s0); // fork the second stream into the capture
    cudaStreamWaitEvent(s1, c->ev_a, 0);
    for (uint32_t k = 0; k < bounces; k++) {
        size_t t = 8 * static_cast<size_t>(k);
        mark(t, s0);
        wf_enqueue_shade(c->dev, A, fh, WA, accum, path_rgb, shade_grid, total, s0, v);
        mark(t + 1, s0);
        mark(t + 2, s1);
        wf_enqueue_trace(c->dev, A, WB, accum, path_rgb, trace_grid, threshold, s1);
        mark(t + 3, s1);
        join();
        mark(t + 4, s0);
        wf_enqueue_trace(c->dev, A, WA, accum, path_rgb, trace_grid, threshold, s0);
        mark(t + 5, s0);
        mark(t + 6, s1);
        wf_enqueue_shade(c->dev, A, fh, WB, accum, path_rgb, shade_grid, total, s1, v);
        mark(t + 7, s1);
        join();
    }
    e = cudaStreamEndCapture(s0, &graph);
    if (e == cudaSuccess)
        e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        if (graph)
            cudaGraphDestroy(graph);
        cudaGetLastError();
        return cuda_fail(c, e, "concurrent wavefront graph");
    }
    auto *host = static_cast<WfCounters *>(c->host_pinned); // [0]: pool A, [1]: pool B
    uint64_t max_replays = ((total + 2 * Qh - 1) / (2 * Qh) + 1) * (kHardDepth + 3) / bounces + 16;
    uint32_t traces_per_bounce = layout == 2 && threshold > 0 ? 1u : 2u;
    uint64_t r = 0;
    bool cancelled = false;
    for (; r < max_replays; r++) {
        if (take_cancel(c)) {
            cancelled = true;
            break;
        }
        e = cudaGraphLaunch(exec, s0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&host[0], WA.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, s0);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&host[1], WB.counters, sizeof(WfCounters), cudaMemcpyDeviceToHost, s0);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s0);
        if (e != cudaSuccess)
            break;
        c->launches += 2 * (2 + traces_per_bounce) * bounces;
        if (timed) {
            for (uint32_t k = 0; k < bounces; k++) {
                size_t t = 8 * static_cast<size_t>(k);
                float a = 0, b = 0, x = 0, y = 0;
                cudaEventElapsedTime(&a, c->kt_events[t], c->kt_events[t + 1]);
                cudaEventElapsedTime(&b, c->kt_events[t + 2], c->kt_events[t + 3]);
                cudaEventElapsedTime(&x, c->kt_events[t + 4], c->kt_events[t + 5]);
                cudaEventElapsedTime(&y, c->kt_events[t + 6], c->kt_events[t + 7]);
                c->kt_shade_ms += a + y;
                c->kt_trace_ms += b + x;
            }
            c->kt_trace_launches += 2 * traces_per_bounce * bounces;
        }
        if (host[0].busy == 0 && host[1].busy == 0 && host[1].shadow_n == 0 && host[1].ext_n == 0 &&
            host[0].next_path >= total)
            break;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "concurrent wavefront run");
    if (cancelled)
        return fail(c, E8G_ERR_CANCELLED, "render cancelled");
    if (r == max_replays)
        return fail(c, E8G_ERR_INTERNAL, "wavefront did not drain");
    return E8G_OK;
}

e8g_status render_image(e8g_ctx *c, e8g_render_params const *p, float *d_rgba, unsigned long long *counts,
                        uint64_t prior_spp) {
    if (counts && p->mode == E8G_MODE_REF_LT2)
        return fail(c, E8G_ERR_UNSUPPORTED, "traversal counters cover every integrator but bidirect_lt2");
    nvtx_range range("e8g render");
    if (take_cancel(c))
        return fail(c, E8G_ERR_CANCELLED, "render cancelled");
    c->launches = 0;
    size_t npix = static_cast<size_t>(p->width) * p->height;
    cudaError_t e = c->b_accum.reserve(npix * sizeof(float4));
    if (e == cudaSuccess && counts)
        e = c->b_counts.reserve(64);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render buffers");
    unsigned long long *d_counts = counts ? static_cast<unsigned long long *>(c->b_counts.ptr) : nullptr;
    cudaEventRecord(c->ev0, c->stream);
    e8g_status s = first_hits(c, p->width, p->height);
    if (s != E8G_OK)
        return s;
    if (prior_spp == 0) { // else the accumulator already holds prior_spp samples of these pixels
        c->prog_spp = 0;  // a fresh accumulator ends any progressive sequence
        e = cudaMemsetAsync(c->b_accum.ptr, 0, npix * sizeof(float4), c->stream);
    }
    if (e == cudaSuccess && d_counts)
        e = cudaMemsetAsync(d_counts, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render clear");
    RenderArgs A = make_args(p);
    c->kt_trace_ms = c->kt_shade_ms = 0;
    c->kt_trace_launches = 0;
    cudaEventRecord(c->ev2, c->stream);
    if (p->firefly)
        s = run_firefly(c, p, A, static_cast<float4 *>(c->b_accum.ptr), d_counts);
    else
        s = run_integrator(c, p, A, static_cast<float4 *>(c->b_accum.ptr), nullptr, d_counts);
    if (s != E8G_OK)
        return s;
    cudaEventRecord(c->ev3, c->stream);
    uint64_t total_spp = prior_spp + p->spp;
    launch_resolve(static_cast<float4 const *>(c->b_accum.ptr), static_cast<uint32_t>(npix),
                   total_spp ? 1.0f / static_cast<float>(total_spp) : 0.0f, d_rgba, c->stream);
    c->launches++;
    cudaEventRecord(c->ev1, c->stream);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render launch");
    if (counts) {
        e = cudaMemcpyAsync(counts, d_counts, 3 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "counter readback");
    }
    e = cudaEventSynchronize(c->ev1);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "render");
    float ms = 0, kms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaEventElapsedTime(&kms, c->ev2, c->ev3);
    c->stats.ms = ms;
    c->stats.kernel_ms = kms;
    c->stats.paths = npix * p->spp;
    c->stats.launches = c->launches;
    c->stats.counted = 0;
    c->stats.trace_ms = c->kt_trace_ms;
    c->stats.shade_ms = c->kt_shade_ms;
    c->stats.trace_launches = c->kt_trace_launches;
    return read_checks(c);
}

e8g_status render_list(e8g_ctx *c, e8g_render_params const *p, uint32_t const *d_pixel, uint32_t const *d_sample,
                       uint32_t n, float *d_rgb, bool first_hits_ready) {
    c->launches = 0;
    e8g_status s = first_hits_ready ? E8G_OK : first_hits(c, p->width, p->height);
    if (s != E8G_OK)
        return s;
    RenderArgs A = make_args(p);
    A.list_pixel = d_pixel;
    A.list_sample = d_sample;
    A.total_paths = n;
    if (p->integrator == E8G_INTEGRATOR_WAVEFRONT && p->mode == E8G_MODE_MIS) {
        cudaError_t e = cudaMemsetAsync(d_rgb, 0, static_cast<size_t>(n) * 3 * sizeof(float), c->stream);
        if (e != cudaSuccess)
            return cuda_fail(c, e, "path output clear");
    }
    s = run_integrator(c, p, A, nullptr, d_rgb, nullptr);
    if (s != E8G_OK)
        return s;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "render_paths launch");
}

} // namespace e8g

extern "C" {

e8g_status e8g_wavefront_tune(e8g_ctx *c, e8g_render_params const *params, e8g_tune_result *res) {
    using namespace e8g;
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, params);
    if (s != E8G_OK)
        return s;
    if (params->mode != E8G_MODE_MIS)
        return fail(c, E8G_ERR_INVALID_ARG, "the wavefront integrator runs E8G_MODE_MIS");
    nvtx_range range("e8g_wavefront_tune");
    // a tuner run that fails (or is cancelled) leaves the configuration it found
    const uint32_t keep_cap = c->wf_capacity, keep_b = c->wf_bounces, keep_th = c->wf_threshold,
                   keep_shade = c->wf_shade_variant;
    const bool keep_conc = c->wf_concurrent;
    c->wf_concurrent = false; // the grid below runs with one pool
    e8g_render_params p = *params;
    p.integrator = E8G_INTEGRATOR_WAVEFRONT;
    p.spp = std::max<uint32_t>(1, std::min<uint32_t>(p.spp, 8)); // long enough for slots to refill steadily
    size_t bytes = static_cast<size_t>(p.width) * p.height * 4 * sizeof(float);
    cudaError_t e = c->b_img.reserve(bytes);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "image buffer");
    const uint32_t caps[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23, 1u << 24};
    const uint32_t bnc[] = {2, 4};
    const uint32_t thr[] = {4, 8, 12, 16, 24};
    e8g_tune_result r{};
    double best = 1e300;
    for (uint32_t cap : caps)
        for (uint32_t b : bnc)
            for (uint32_t th : thr) {
            c->wf_capacity = cap;
            c->wf_bounces = b;
            c->wf_threshold = th;
            double ms = 1e300;
            for (int rep = 0; rep < 2; rep++) { // first run warms caches and builds nothing twice
                s = render_image(c, &p, static_cast<float *>(c->b_img.ptr), nullptr);
                if (s != E8G_OK) {
                    c->wf_capacity = keep_cap, c->wf_bounces = keep_b, c->wf_threshold = keep_th;
                    c->wf_concurrent = keep_conc;
                    return s;
                }
                ms = std::min(ms, c->stats.kernel_ms);
            }
            if (r.num_candidates < E8G_TUNE_MAX_CANDIDATES) {
                r.cand_capacity[r.num_candidates] = cap;
                r.cand_bounces[r.num_candidates] = b;
                r.cand_threshold[r.num_candidates] = th;
                r.cand_ms[r.num_candidates] = ms;
                r.num_candidates++;
            }
            if (ms < best) {
                best = ms;
                r.capacity = cap;
                r.bounces_per_graph = b;
                r.threshold = th;
            }
            }
    // Short renders favour small slot pools (the frame's tail weighs more in them, and larger
    // pools amortise every bounce's fixed cost over more rays only in long renders): each
    // capacity's fastest (bounces, threshold) pair is timed again on a render of up to 64 samples
    // per pixel, and the fastest of those is kept.
    uint32_t spp2 = std::max<uint32_t>(p.spp, std::min<uint32_t>(params->spp, 64));
    if (spp2 > p.spp) {
        e8g_render_params p2 = p;
        p2.spp = spp2;
        best = 1e300;
        for (uint32_t cap : caps) {
            int bi = -1;
            for (uint32_t i = 0; i < r.num_candidates; i++)
                if (r.cand_capacity[i] == cap && (bi < 0 || r.cand_ms[i] < r.cand_ms[bi]))
                    bi = static_cast<int>(i);
            if (bi < 0)
                continue;
            c->wf_capacity = cap;
            c->wf_bounces = r.cand_bounces[bi];
            c->wf_threshold = r.cand_threshold[bi];
            s = render_image(c, &p2, static_cast<float *>(c->b_img.ptr), nullptr);
            if (s != E8G_OK) {
                c->wf_capacity = keep_cap, c->wf_bounces = keep_b, c->wf_threshold = keep_th;
                c->wf_concurrent = keep_conc;
                return s;
            }
            double ms = c->stats.kernel_ms;
            if (ms < best) {
                best = ms;
                r.capacity = cap;
                r.bounces_per_graph = r.cand_bounces[bi];
                r.threshold = r.cand_threshold[bi];
            }
        }
    }
    c->wf_capacity = r.capacity;
    c->wf_bounces = r.bounces_per_graph;
    c->wf_threshold = r.threshold;
    // the shading kernel's block shape, on the longest render of the search
    {
        e8g_render_params p3 = p;
        p3.spp = spp2;
        double best_ms = 1e300;
        r.shade_variant = keep_shade;
        for (uint32_t v = 0; v < kWfShadeVariants; v++) {
            c->wf_shade_variant = v;
            double ms = 1e300;
            for (int rep = 0; rep < 2; rep++) {
                s = render_image(c, &p3, static_cast<float *>(c->b_img.ptr), nullptr);
                if (s != E8G_OK) {
                    c->wf_capacity = keep_cap, c->wf_bounces = keep_b, c->wf_threshold = keep_th;
                    c->wf_shade_variant = keep_shade;
                    c->wf_concurrent = keep_conc;
                    return s;
                }
                ms = std::min(ms, c->stats.kernel_ms);
            }
            r.shade_ms[v] = ms;
            if (ms < best_ms) {
                best_ms = ms;
                r.shade_variant = v;
            }
        }
        r.num_shade = kWfShadeVariants;
        c->wf_shade_variant = r.shade_variant;
        // one slot pool, or two interleaving on two streams
        r.concurrent_ms[0] = best_ms;
        c->wf_concurrent = true;
        double ms = 1e300;
        for (int rep = 0; rep < 2; rep++) {
            s = render_image(c, &p3, static_cast<float *>(c->b_img.ptr), nullptr);
            if (s != E8G_OK) {
                c->wf_capacity = keep_cap, c->wf_bounces = keep_b, c->wf_threshold = keep_th;
                c->wf_shade_variant = keep_shade;
                c->wf_concurrent = keep_conc;
                return s;
            }
            ms = std::min(ms, c->stats.kernel_ms);
        }
        r.concurrent_ms[1] = ms;
        r.concurrent = ms < best_ms ? 1u : 0u;
        c->wf_concurrent = r.concurrent != 0;
    }
    if (res)
        *res = r;
    return E8G_OK;
}

e8g_status e8g_wavefront_set(e8g_ctx *c, uint32_t capacity, uint32_t bounces, uint32_t threshold) {
    using namespace e8g;
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (capacity < 1024 || capacity > (1u << 26) || bounces < 1 || bounces > 16 || threshold > 32)
        return fail(c, E8G_ERR_INVALID_ARG, "wavefront configuration out of range");
    c->wf_capacity = capacity;
    c->wf_bounces = bounces;
    c->wf_threshold = threshold;
    return E8G_OK;
}

e8g_status e8g_wavefront_set_concurrent(e8g_ctx *c, int on) {
    if (!c)
        return E8G_ERR_INVALID_ARG;
    c->wf_concurrent = on != 0;
    return E8G_OK;
}

e8g_status e8g_wavefront_set_shade(e8g_ctx *c, uint32_t variant) {
    using namespace e8g;
    if (!c)
        return E8G_ERR_INVALID_ARG;
    if (variant >= kWfShadeVariants)
        return fail(c, E8G_ERR_INVALID_ARG, "unknown shading block shape");
    c->wf_shade_variant = variant;
    return E8G_OK;
}

namespace {

// One line of the tuning cache: "key": {"capacity": C, "bounces": B, "threshold": T, "shade": S, "ms": M}
struct tune_entry {
    uint32_t capacity = 0, bounces = 0, threshold = 0, shade = 0, concurrent = 0;
    double ms = 0;
};

uint32_t log2_bucket(uint64_t v) {
    uint32_t b = 0;
    while (v > 1) {
        v >>= 1;
        b++;
    }
    return b;
}

std::map<std::string, tune_entry> read_tune_cache(char const *path) {
    std::map<std::string, tune_entry> out;
    FILE *f = std::fopen(path, "r");
    if (!f)
        return out;
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
        char key[200];
        tune_entry t;
        if (std::sscanf(line, " \"%199[^\"]\": {\"capacity\": %u, \"bounces\": %u, \"threshold\": %u, \"shade\": %u, "
                              "\"concurrent\": %u, \"ms\": %lf",
                        key, &t.capacity, &t.bounces, &t.threshold, &t.shade, &t.concurrent, &t.ms) == 7 &&
            t.concurrent <= 1 &&
            t.capacity >= 1024 && t.capacity <= (1u << 26) && t.bounces >= 1 && t.bounces <= 16 &&
            t.threshold <= 32 && t.shade < e8g::kWfShadeVariants)
            out[key] = t;
    }
    std::fclose(f);
    return out;
}

bool write_tune_cache(char const *path, std::map<std::string, tune_entry> const &m) {
    std::string tmp = std::string(path) + ".tmp";
    FILE *f = std::fopen(tmp.c_str(), "w");
    if (!f)
        return false;
    std::fprintf(f, "{\n");
    size_t i = 0;
    for (auto const &kv : m) {
        std::fprintf(f,
                     "  \"%s\": {\"capacity\": %u, \"bounces\": %u, \"threshold\": %u, \"shade\": %u, "
                     "\"concurrent\": %u, \"ms\": %.4f}%s\n",
                     kv.first.c_str(), kv.second.capacity, kv.second.bounces, kv.second.threshold, kv.second.shade,
                     kv.second.concurrent, kv.second.ms, ++i < m.size() ? "," : "");
    }
    std::fprintf(f, "}\n");
    bool ok = std::fclose(f) == 0;
    return ok && std::rename(tmp.c_str(), path) == 0;
}

} // namespace

e8g_status e8g_wavefront_tune_cached(e8g_ctx *c, e8g_render_params const *params, char const *path,
                                     e8g_tune_result *res) {
    using namespace e8g;
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, params);
    if (s != E8G_OK)
        return s;
    if (!path || !*path)
        return fail(c, E8G_ERR_INVALID_ARG, "no cache path");
    char key[200];
    std::snprintf(key, sizeof(key), "layout%u/rng%u/tris2^%u/pixels2^%u/spp2^%u", c->pack.layout, params->rng,
                  log2_bucket(c->pack.nt), log2_bucket(static_cast<uint64_t>(params->width) * params->height),
                  log2_bucket(std::min<uint32_t>(std::max<uint32_t>(params->spp, 1), 64)));
    std::map<std::string, tune_entry> cache = read_tune_cache(path);
    auto it = cache.find(key);
    if (it != cache.end()) {
        c->wf_capacity = it->second.capacity;
        c->wf_bounces = it->second.bounces;
        c->wf_threshold = it->second.threshold;
        c->wf_shade_variant = it->second.shade;
        c->wf_concurrent = it->second.concurrent != 0;
        if (res) {
            *res = e8g_tune_result{};
            res->capacity = it->second.capacity;
            res->bounces_per_graph = it->second.bounces;
            res->threshold = it->second.threshold;
            res->shade_variant = it->second.shade;
            res->concurrent = it->second.concurrent;
            res->from_cache = 1;
        }
        return E8G_OK;
    }
    e8g_tune_result r{};
    s = e8g_wavefront_tune(c, params, &r);
    if (s != E8G_OK)
        return s;
    tune_entry t;
    t.capacity = r.capacity;
    t.bounces = r.bounces_per_graph;
    t.threshold = r.threshold;
    t.shade = r.shade_variant;
    t.concurrent = r.concurrent;
    t.ms = r.concurrent_ms[r.concurrent];
    cache[key] = t;
    if (!write_tune_cache(path, cache))
        return fail(c, E8G_ERR_INVALID_ARG, std::string("cannot write the tuning cache ") + path);
    if (res)
        *res = r;
    return E8G_OK;
}

e8g_status e8g_forward(e8g_ctx *c, e8g_render_params const *p, float *rgba_out) {
    using namespace e8g;
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    s = validate_params(c, p);
    if (s != E8G_OK)
        return s;
    if (p->mode != E8G_MODE_MIS || p->rng != E8G_RNG_PHILOX)
        return fail(c, E8G_ERR_INVALID_ARG, "the adjoint replays E8G_MODE_MIS paths from Philox streams");
    c->have_forward = false;
    s = e8g_render(c, p, rgba_out);
    if (s != E8G_OK)
        return s;
    c->fwd_params = *p;
    c->have_forward = true;
    return E8G_OK;
}

e8g_status e8g_backward(e8g_ctx *c, float const *dl_dimage, float *d_albedo, float *d_roughness) {
    using namespace e8g;
    e8g_status s = check_ready(c);
    if (s != E8G_OK)
        return s;
    if (!c->have_forward)
        return fail(c, E8G_ERR_INVALID_ARG, "e8g_backward needs a preceding e8g_forward");
    if (!dl_dimage || !d_albedo || !d_roughness)
        return fail(c, E8G_ERR_INVALID_ARG, "NULL buffers");
    e8g_render_params const &p = c->fwd_params;
    cudaSetDevice(c->device);
    size_t npix = static_cast<size_t>(p.width) * p.height, nm = c->pack.nmat;
    size_t gb = npix * 3 * sizeof(float), ab = nm * 3 * sizeof(float), rb = nm * sizeof(float);
    cudaError_t e = c->b_io0.reserve(gb);
    if (e == cudaSuccess)
        e = c->b_grad.reserve(ab + rb + 16);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "adjoint buffers");
    float *d_dl = static_cast<float *>(c->b_io0.ptr);
    float *d_a = static_cast<float *>(c->b_grad.ptr), *d_r = d_a + nm * 3;
    cudaEventRecord(c->ev0, c->stream);
    e = cudaMemcpyAsync(d_dl, dl_dimage, gb, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_a, 0, ab + rb, c->stream);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(c->b_work.ptr, 0, 64, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "adjoint upload");
    s = first_hits(c, p.width, p.height);
    if (s != E8G_OK)
        return s;
    RenderArgs A = make_args(&p);
    cudaEventRecord(c->ev2, c->stream);
    e = launch_adjoint(c->dev, A, static_cast<FirstHit const *>(c->b_fh.ptr), d_dl,
                       p.spp ? 1.0f / static_cast<float>(p.spp) : 0.0f, static_cast<unsigned long long *>(c->b_work.ptr),
                       d_a, d_r, nullptr, c->num_sms, c->stream);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "adjoint launch");
    cudaEventRecord(c->ev3, c->stream);
    e = cudaMemcpyAsync(d_albedo, d_a, ab, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_roughness, d_r, rb, cudaMemcpyDeviceToHost, c->stream);
    cudaEventRecord(c->ev1, c->stream);
    if (e == cudaSuccess)
        e = cudaEventSynchronize(c->ev1);
    if (e != cudaSuccess)
        return cuda_fail(c, e, "adjoint");
    float ms = 0, kms = 0;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    cudaEventElapsedTime(&kms, c->ev2, c->ev3);
    c->stats.ms = ms;
    c->stats.kernel_ms = kms;
    c->stats.paths = npix * p.spp;
    c->stats.launches = 2;
    c->stats.trace_ms = c->stats.shade_ms = 0;
    c->stats.trace_launches = 0;
    return read_checks(c);
}

e8g_status e8g_set_materials(e8g_ctx *c, e8g_material const *m, uint32_t n) {
    using namespace e8g;
    if (!c || !m)
        return E8G_ERR_INVALID_ARG;
    if (!c->uploaded)
        return fail(c, E8G_ERR_NO_SCENE, "no scene uploaded");
    if (n != c->pack.nmat)
        return fail(c, E8G_ERR_INVALID_ARG, "material count differs from the uploaded scene");
    for (uint32_t i = 0; i < n; i++) {
        if (m[i].type > E8G_MAT_MIXTURE)
            return fail(c, E8G_ERR_INVALID_ARG, "unknown material type");
        if (m[i].type == E8G_MAT_MIXTURE &&
            (m[i].mix0 < 0 || m[i].mix1 < 0 || static_cast<uint32_t>(m[i].mix0) >= n ||
             static_cast<uint32_t>(m[i].mix1) >= n || m[m[i].mix0].type == E8G_MAT_MIXTURE ||
             m[m[i].mix1].type == E8G_MAT_MIXTURE))
            return fail(c, E8G_ERR_INVALID_ARG, "bad mixture components");
    }
    cudaSetDevice(c->device);
    pack_materials(m, n, c->pack.mats);
    c->prog_spp = 0;
    c->materials.assign(m, m + n);
    cudaError_t e = cudaMemcpyAsync(c->b_mats.ptr, c->pack.mats.data(), c->pack.mats.size() * sizeof(DevMaterial),
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? E8G_OK : cuda_fail(c, e, "material upload");
}

} // extern "C"
