// Host-side renderer: the orchestration of Renderer::render and its passes
// (projects/WaveFrontPathTracer/Renderer/Renderer.cpp:124-199, 552-654), the
// ray buffers of RayBuffer (Ray/RayBuffer.cpp) and the traceSort sequence of
// Tracer (Tracer/Tracer.cpp:214-225).
//
// Differences by design:
//  - wavefront sizes stay on the device: raygen_path writes the compacted
//    count into a device counter that every later kernel of the bounce reads,
//    so a frame issues no host readback (the reference reads the path count
//    and the hit count back after every pass, RayGen.cpp:178-183 and
//    Renderer.cpp:85-88);
//  - the per-pass hit count (countRayHits) is taken by the reconstructSmooth
//    kernel that reads the same hit records just before the shadow pass,
//    instead of a separate kernel on the frame's critical stream;
//  - buffers are sized once per resolution (capacity = width*height rays per
//    wavefront) and the frame can be captured into one CUDA graph;
//  - ray statistics are read back once, after the frame.
#include <atomic>
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/wfpt.h"
#include "host.h"
#include "internal.h"
#include "stages.cuh"
#include "trace.cuh"

namespace {

constexpr int kMaxDepth = 8;                    // RENDERER_MAX_RECURSION_DEPTH
constexpr int kMaxSamples = 1024;               // RENDERER_MAX_SAMPLES
constexpr int kMaxBatch = 8 * 1024 * 1024;      // RENDERER_MAX_BATCH_SIZE
constexpr int kCountersPerPass = 32;
// Per-pass counter block: [0..7] path rays per bounce, [8..16] hits among
// the input rays of each shadow pass, [17..24] shadow rays of the batch in
// flight on each shadow slot.
constexpr int kCntPath = 0, kCntHits = 8, kCntBatch = 17;

// Shadow batch slots (knob "renderer.shadow_slots"): 0 = planned from free
// device memory, 1..kMaxSlots = that many (capped by the batches a pass can
// need).
constexpr int kMaxSlots = 8;
static std::atomic<int> g_shadow_slots{0};

// Fault injection (knob "debug.fail_alloc_after"): when >= 0, the renderer's
// allocation after that many more succeeds reports out of memory, without
// touching the device.  -1 = off.
static std::atomic<int> g_fail_alloc_after{-1};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t b) {
        if (b <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        int left = g_fail_alloc_after.load();
        while (left >= 0 && !g_fail_alloc_after.compare_exchange_weak(left, left - 1)) {
        }
        if (left == 0) return cudaErrorMemoryAllocation;
        cudaError_t e = wfpt::dev_malloc(&p, b);
        if (e == cudaSuccess) bytes = b;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const {
        return reinterpret_cast<T*>(p);
    }
};

// RayBuffer (Ray/RayBuffer.h:22-70): double-buffered rays and slot maps,
// one result buffer, Morton keys and sort indices.
struct RayBufferDev {
    DevBuf rays[2], s2i[2], i2s[2], results, keys, idx;
    bool swapped = false;
    wfpt_ray* rays_cur() const { return rays[swapped ? 1 : 0].as<wfpt_ray>(); }
    wfpt_ray* rays_out() const { return rays[swapped ? 0 : 1].as<wfpt_ray>(); }
    int32_t* s2i_cur() const { return s2i[swapped ? 1 : 0].as<int32_t>(); }
    int32_t* s2i_out() const { return s2i[swapped ? 0 : 1].as<int32_t>(); }
    int32_t* i2s_cur() const { return i2s[swapped ? 1 : 0].as<int32_t>(); }
    int32_t* i2s_out() const { return i2s[swapped ? 0 : 1].as<int32_t>(); }
    void swap() { swapped = !swapped; }
    cudaError_t ensure(size_t cap, bool sortable) {
        cudaError_t e;
        if ((e = rays[0].ensure(cap * 32)) != cudaSuccess) return e;
        if ((e = results.ensure(cap * 16)) != cudaSuccess) return e;
        if ((e = s2i[0].ensure(cap * 4)) != cudaSuccess) return e;
        if ((e = i2s[0].ensure(cap * 4)) != cudaSuccess) return e;
        if (sortable) {
            if ((e = rays[1].ensure(cap * 32)) != cudaSuccess) return e;
            if ((e = s2i[1].ensure(cap * 4)) != cudaSuccess) return e;
            if ((e = i2s[1].ensure(cap * 4)) != cudaSuccess) return e;
            if ((e = keys.ensure(cap * 8)) != cudaSuccess) return e;
            if ((e = idx.ensure(cap * 4)) != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    void release() {
        for (auto* b : {&rays[0], &rays[1], &s2i[0], &s2i[1], &i2s[0], &i2s[1], &results, &keys, &idx}) b->release();
    }
};

}  // namespace

struct wfpt_renderer {
    wfpt_renderer_config cfg{};
    const wfpt_scene* scene = nullptr;
    const wfpt_geometry* geoms = nullptr;
    float smin[3] = {0, 0, 0}, smax[3] = {0, 0, 0}, light[3] = {5, -2, 1}, bg[3] = {0, 0, 1};
    int frame_index = 1;

    int width = 0, height = 0;
    int alloc_samples = 0;
    DevBuf i2p, p2i, seeds, decreases, aux, sort_scratch, path_scratch, counters;
    // Work counters of this renderer's persistent traversal launches (all on
    // one stream, one after another), so that renderers running
    // concurrently never share one.
    DevBuf work;
    // Shadow-pass overlap (cfg.shadow_overlap): the batches of a pass's
    // shadow rays are generated, traced and reconstructed on the streams of
    // `slots` (batch b on slot b % slots.size()) while the next bounce runs
    // on the frame's stream; each slot has its own ray buffers, traversal
    // work counters and sort scratch, and the colour buffers alternate
    // between passes (aux2 with aux).  The batch boundaries are the
    // reference's (RENDERER_MAX_BATCH_SIZE / S, Renderer.cpp:136-147): they
    // decide which seed a shadow ray reads, so they stay fixed; the memory
    // planner (prepare) only decides how many batches run at once.  The
    // batches of one pass add into disjoint pixels, so running them
    // concurrently gives the sequential result bit for bit.
    struct ShadowSlot {
        RayBufferDev rb;
        DevBuf work, scratch;
        cudaStream_t stream = nullptr;
        cudaEvent_t ev_rg = nullptr, ev_done = nullptr;
    };
    std::vector<ShadowSlot> slots;
    DevBuf aux2;
    cudaEvent_t ev_fork = nullptr;
    int pending_slots = 0;  // slots the next shadow pass (or the frame's end) waits for
    int last_slots = 0;     // slots used by the last frame
    RayBufferDev primary, shadow, queue[2];
    DevBuf accum64;  // cfg.accumulate_fp64: the running mean, double4 per pixel
    uint32_t* host_counters = nullptr;  // pinned

    // Timing (cfg.timing, Application.mode "benchmark" with
    // Benchmark.printSortLogs): a directly launched frame records event
    // pairs around its stages; get_stats resolves them into the per-type
    // trace times and the sort logs.  A span counts into a trace-time total
    // (T_PRIMARY/T_SHADOW/T_PATH) and/or into one component of a sort log
    // (log 0..8: shadowSortLogs[log], 100 + b: pathSortLogs[b]).
    enum { T_NONE = -1, T_PRIMARY, T_SHADOW, T_PATH };
    enum { C_NONE = -1, C_MORTON, C_SORT, C_REORDER, C_TRACE_SORT, C_TRACE };
    struct Span {
        int a, b, total, comp, log;
    };
    std::vector<cudaEvent_t> tev;
    size_t tev_used = 0;
    std::vector<Span> spans;
    bool timing_on = false;   // the frame being recorded is timed
    bool last_timed = false;  // the last rendered frame was timed

    // Records the next pool event on s; *idx receives its index.
    cudaError_t mark(cudaStream_t s, int* idx) {
        if (tev_used == tev.size()) {
            cudaEvent_t ev;
            cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return e;
            tev.push_back(ev);
        }
        *idx = (int)tev_used++;
        return cudaEventRecord(tev[*idx], s);
    }
    int last_spp = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    bool stats_pending = false;
    float frame_ms = 0.0f;

    // Frame graph: captured once per (configuration, resolution, buffers)
    // on a private stream (the legacy default stream cannot be captured);
    // replayed on the caller's stream with the per-frame values in fp_dev.
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    wfpt::FrameParams* fp_dev = nullptr;
    uint64_t graph_kernels = 0;  // kernels per replay (for the launch count)
    struct GraphKey {
        wfpt_renderer_config cfg;
        int w, h;
        const void *pixels, *frame_pixels, *scene, *geoms;
        float light[3], bg[3], smin[3], smax[3];
        int slots;
    } graph_key{};
    bool graph_valid = false;

    GraphKey make_key(float* pixels, float* frame_pixels) const {
        GraphKey k;
        std::memset(&k, 0, sizeof(k));
        k.cfg = cfg;
        k.w = width;
        k.h = height;
        k.pixels = pixels;
        k.frame_pixels = frame_pixels;
        k.scene = scene;
        k.geoms = geoms;
        k.slots = nslots;
        for (int i = 0; i < 3; ++i) {
            k.light[i] = light[i];
            k.bg[i] = bg[i];
            k.smin[i] = smin[i];
            k.smax[i] = smax[i];
        }
        return k;
    }

    // Renders through the frame graph, capturing it first when needed.
    cudaError_t render_graph(const float* s2w, const float* eye, float zfar, float* pixels, float* frame_pixels,
                             cudaStream_t s) {
        cudaError_t e;
        if (!fp_dev && (e = wfpt::dev_malloc(reinterpret_cast<void**>(&fp_dev), sizeof(wfpt::FrameParams))) !=
                            cudaSuccess)
            return e;
        if (!capture_stream && (e = cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking)) != cudaSuccess)
            return e;
        if ((e = wfpt::sort_prepare()) != cudaSuccess) return e;
        if ((e = wfpt::trace_prepare()) != cudaSuccess) return e;
        GraphKey key = make_key(pixels, frame_pixels);
        if (!graph_valid || std::memcmp(&key, &graph_key, sizeof(key)) != 0) {
            if (graph_exec) cudaGraphExecDestroy(graph_exec);
            if (graph) cudaGraphDestroy(graph);
            graph_exec = nullptr;
            graph = nullptr;
            graph_valid = false;
            uint64_t k0 = wfpt::launch_count();
            const cudaStream_t cs = capture_stream;
            if ((e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
            cudaError_t fe = frame(s2w, eye, zfar, pixels, frame_pixels, cs, fp_dev);
            e = cudaStreamEndCapture(cs, &graph);
            if (fe != cudaSuccess) return fe;
            if (e != cudaSuccess) return e;
            graph_kernels = wfpt::launch_count() - k0;
            if ((e = cudaGraphInstantiate(&graph_exec, graph, 0)) != cudaSuccess) return e;
            graph_key = key;
            graph_valid = true;
        }
        // The parameter block is copied from pageable host memory, which is
        // staged before the call returns.
        wfpt::FrameParams hp;
        std::memset(&hp, 0, sizeof(hp));
        for (int i = 0; i < 16; ++i) hp.s2w[i] = s2w[i];
        for (int i = 0; i < 3; ++i) hp.eye[i] = eye[i];
        hp.zfar = zfar;
        hp.frame_index = frame_index;
        if ((e = cudaMemcpyAsync(fp_dev, &hp, sizeof(hp), cudaMemcpyHostToDevice, s)) != cudaSuccess) return e;
        if ((e = cudaGraphLaunch(graph_exec, s)) != cudaSuccess) return e;
        wfpt::count_launch((uint32_t)graph_kernels);
        return cudaSuccess;
    }

    ~wfpt_renderer() {
        if (graph_exec) cudaGraphExecDestroy(graph_exec);
        if (graph) cudaGraphDestroy(graph);
        if (fp_dev) cudaFree(fp_dev);
        if (capture_stream) cudaStreamDestroy(capture_stream);
        for (ShadowSlot& sl : slots) {
            if (sl.stream) cudaStreamDestroy(sl.stream);
            if (sl.ev_rg) cudaEventDestroy(sl.ev_rg);
            if (sl.ev_done) cudaEventDestroy(sl.ev_done);
            sl.rb.release();
            sl.work.release();
            sl.scratch.release();
        }
        if (ev_fork) cudaEventDestroy(ev_fork);
        for (auto* b : {&i2p, &p2i, &seeds, &decreases, &aux, &sort_scratch, &path_scratch, &counters, &work, &aux2})
            b->release();
        primary.release();
        shadow.release();
        queue[0].release();
        queue[1].release();
        if (host_counters) cudaFreeHost(host_counters);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (ev2) cudaEventDestroy(ev2);
        for (cudaEvent_t ev : tev) cudaEventDestroy(ev);
        accum64.release();
    }

    // Ray counts of the last frame from the counters read back to the host
    // (the caller has waited for that copy).
    void fill_stats(wfpt_render_stats* st) const {
        uint64_t n = (uint64_t)width * height;
        int S = cfg.num_shadow_samples;
        int rt = cfg.ray_type;
        for (int p = 0; p < last_spp; ++p) {
            const uint32_t* c = host_counters + p * kCountersPerPass;
            st->num_primary_rays += n;
            if (rt == WFPT_PRIMARY_RAYS) continue;
            int passes = rt == WFPT_PATH_RAYS ? cfg.recursion_depth + 1 : 1;
            for (int i = 0; i < passes; ++i) {
                st->num_shadow_rays += (uint64_t)S * c[kCntHits + i];
                st->shadow_hits_per_pass[i] += c[kCntHits + i];
            }
            if (rt == WFPT_PATH_RAYS)
                for (int b = 0; b < cfg.recursion_depth; ++b) {
                    st->num_path_rays += c[kCntPath + b];
                    st->path_rays_per_bounce[b] += c[kCntPath + b];
                }
        }
        for (int i = 0; i < 9; ++i) st->shadow_sort_logs[i].ray_count = (uint64_t)S * st->shadow_hits_per_pass[i];
        for (int b = 0; b < 8; ++b) st->path_sort_logs[b].ray_count = st->path_rays_per_bounce[b];
    }

    // Trace times and sort-log times of the last frame, when it was timed
    // (its events have completed: the caller waited for ev2).
    void fill_times(wfpt_render_stats* st) const {
        if (!last_timed) return;
        st->timed = 1;
        for (const Span& sp : spans) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, tev[sp.a], tev[sp.b]) != cudaSuccess) continue;
            if (sp.total == T_PRIMARY) st->primary_trace_ms += ms;
            if (sp.total == T_SHADOW) st->shadow_trace_ms += ms;
            if (sp.total == T_PATH) st->path_trace_ms += ms;
            if (sp.comp == C_NONE || sp.log < 0) continue;
            wfpt_sort_log& lg = sp.log >= 100 ? st->path_sort_logs[sp.log - 100] : st->shadow_sort_logs[sp.log];
            float* f[5] = {&lg.morton_ms, &lg.sort_ms, &lg.reorder_ms, &lg.trace_sort_ms, &lg.trace_ms};
            *f[sp.comp] += ms;
        }
    }

    // Launches `fn` on s between two timing events when the frame is timed.
    template <class F>
    cudaError_t timed(cudaStream_t s, int total, int comp, int log, F&& fn) {
        if (!timing_on) return fn();
        int a = 0, b = 0;
        cudaError_t e;
        if ((e = mark(s, &a)) != cudaSuccess) return e;
        if ((e = fn()) != cudaSuccess) return e;
        if ((e = mark(s, &b)) != cudaSuccess) return e;
        spans.push_back(Span{a, b, total, comp, log});
        return cudaSuccess;
    }

    int key_bits() const {
        switch (cfg.morton_kind) {
            case WFPT_MORTON_6D48: return 48;
            case WFPT_MORTON_6D64: return 63;
            default: return 32;
        }
    }

    uint32_t* cnt(int pass, int slot) const { return counters.as<uint32_t>() + pass * kCountersPerPass + slot; }

    int nslots = 1;  // shadow batch slots of the current plan

    // The memory planner's share for shadow batches: how many of a pass's
    // batches (at most ceil(n / (kMaxBatch / S))) run at once.  Each slot
    // holds one batch's rays (double-buffered), hits, slot maps, keys and
    // sort scratch; the plan takes as many as fit in half of the device
    // memory that is free before they are allocated (slots already held by
    // this renderer count as free), at least one.
    int plan_slots(size_t n, int S, size_t shadow_cap) const {
        const size_t batch_diff = (size_t)(kMaxBatch / S);
        const int batches = (int)std::min<size_t>(kMaxSlots, (n + batch_diff - 1) / batch_diff);
        int want = g_shadow_slots.load() > 0 ? std::min(g_shadow_slots.load(), batches) : batches;
        if (want <= 1) return 1;
        const size_t per_slot = shadow_cap * (2 * 32 + 16 + 4 * 4 + 8 + 4) + 64 +
                                (cfg.sort_shadow_rays ? wfpt::sort_scratch_bytes((uint32_t)shadow_cap, 64) : 0);
        if (g_shadow_slots.load() > 0) return want;
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return 1;
        size_t held = 0;
        for (const ShadowSlot& sl : slots) held += sl.rb.rays[0].bytes ? per_slot : 0;
        const size_t budget = (free_b + held) / 2;
        return (int)std::max<size_t>(1, std::min<size_t>((size_t)want, budget / per_slot));
    }

    cudaError_t prepare(int w, int h) {
        cudaError_t e;
        size_t n = (size_t)w * h;
        int S = cfg.num_shadow_samples;
        if (w != width || h != height) {
            std::vector<int32_t> a(n), b(n);
            wfpt::pixel_table(w, h, a.data(), b.data());
            if ((e = i2p.ensure(n * 4)) != cudaSuccess) return e;
            if ((e = p2i.ensure(n * 4)) != cudaSuccess) return e;
            if ((e = cudaMemcpy(i2p.p, a.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
            if ((e = cudaMemcpy(p2i.p, b.data(), n * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
            width = w;
            height = h;
        }
        if ((e = seeds.ensure(n * 4)) != cudaSuccess) return e;
        if ((e = decreases.ensure(n * 16)) != cudaSuccess) return e;
        if ((e = aux.ensure(n * 16)) != cudaSuccess) return e;
        if ((e = primary.ensure(n, false)) != cudaSuccess) return e;
        if ((e = queue[0].ensure(n, true)) != cudaSuccess) return e;
        if ((e = queue[1].ensure(n, true)) != cudaSuccess) return e;
        size_t batch_in = std::min<size_t>(n, (size_t)(kMaxBatch / S));
        size_t shadow_cap = std::max<size_t>(1, batch_in * S);
        const bool sequential_shadow = !cfg.shadow_overlap || cfg.timing;
        if (sequential_shadow && (e = shadow.ensure(shadow_cap, true)) != cudaSuccess) return e;
        size_t sort_n = std::max(n, sequential_shadow ? shadow_cap : (size_t)0);
        if ((e = sort_scratch.ensure(wfpt::sort_scratch_bytes((uint32_t)sort_n, 64))) != cudaSuccess) return e;
        if ((e = path_scratch.ensure(wfpt::raygen_path_scratch_bytes((uint32_t)n))) != cudaSuccess) return e;
        if ((e = counters.ensure((size_t)kMaxSamples * kCountersPerPass * 4)) != cudaSuccess) return e;
        if (cfg.accumulate_fp64 && (e = accum64.ensure(n * 32)) != cudaSuccess) return e;
        if (!work.p) {
            if ((e = work.ensure(16 * sizeof(uint32_t))) != cudaSuccess) return e;
            if ((e = cudaMemset(work.p, 0, work.bytes)) != cudaSuccess) return e;
        }
        if (cfg.shadow_overlap) {
            if ((e = aux2.ensure(n * 16)) != cudaSuccess) return e;
            if (!ev_fork && (e = cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming)) != cudaSuccess) return e;
            const int want = plan_slots(n, S, shadow_cap);
            if ((int)slots.size() < want) slots.resize(want);
            for (int k = 0; k < want; ++k) {
                ShadowSlot& sl = slots[k];
                if ((e = sl.rb.ensure(shadow_cap, true)) != cudaSuccess) return e;
                if (!sl.work.p) {
                    if ((e = sl.work.ensure(16 * sizeof(uint32_t))) != cudaSuccess) return e;
                    if ((e = cudaMemset(sl.work.p, 0, sl.work.bytes)) != cudaSuccess) return e;
                }
                if (cfg.sort_shadow_rays &&
                    (e = sl.scratch.ensure(wfpt::sort_scratch_bytes((uint32_t)shadow_cap, 64))) != cudaSuccess)
                    return e;
                if (!sl.stream && (e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess)
                    return e;
                if (!sl.ev_rg && (e = cudaEventCreateWithFlags(&sl.ev_rg, cudaEventDisableTiming)) != cudaSuccess)
                    return e;
                if (!sl.ev_done && (e = cudaEventCreateWithFlags(&sl.ev_done, cudaEventDisableTiming)) != cudaSuccess)
                    return e;
            }
            nslots = want;
        }
        if (!host_counters &&
            (e = wfpt::host_malloc(reinterpret_cast<void**>(&host_counters), (size_t)kMaxSamples * kCountersPerPass * 4)) !=
                cudaSuccess)
            return e;
        if (!ev0 && (e = cudaEventCreate(&ev0)) != cudaSuccess) return e;
        if (!ev1 && (e = cudaEventCreate(&ev1)) != cudaSuccess) return e;
        if (!ev2 && (e = cudaEventCreate(&ev2)) != cudaSuccess) return e;
        return cudaSuccess;
    }

    // Tracer::trace / Tracer::traceSort (Tracer.cpp:185-225).  wk / scratch:
    // the traversal work counters and sort scratch of the stream s (each
    // concurrently running branch has its own).  total / log: where a timed frame books the stages (T_SHADOW or T_PATH;
    // the sort log slot); a timed sorted pass first traces its rays
    // unsorted, for the log's trace time, as Renderer.cpp:259-264 and
    // :281-286 do (the sorted trace then overwrites those results).
    // keys_ready: rb.keys / rb.idx already hold the rays' Morton keys (written
    // by the path-ray generation), so the sort starts without the Morton kernel.
    cudaError_t trace_rays(RayBufferDev& rb, uint32_t n, const uint32_t* n_dev, bool sort, bool reorder, bool closest,
                           cudaStream_t s, uint32_t* wk, DevBuf& scratch, int kind, int total = T_NONE,
                           int log = -1, bool keys_ready = false) {
        const wfpt::SceneDevice& sc = *wfpt::scene_device(scene);
        cudaError_t e;
        auto plain = [&]() {
            return wfpt::launch_trace(sc, kind, rb.rays_cur(), rb.results.as<wfpt_hit>(), nullptr, n, n_dev,
                                      closest ? 1 : 0, s, wk);
        };
        if (!sort) return timed(s, total, C_NONE, -1, plain);
        if (timing_on && log >= 0 && (e = timed(s, T_NONE, C_TRACE, log, plain)) != cudaSuccess) return e;
        float size[3] = {smax[0] - smin[0], smax[1] - smin[1], smax[2] - smin[2]};
        if (!keys_ready && (e = timed(s, total, C_MORTON, log, [&]() {
                 return wfpt::launch_morton(rb.rays_cur(), n, n_dev, smin, size, cfg.morton_kind, rb.keys.p,
                                            rb.idx.as<uint32_t>(), s);
             })) != cudaSuccess)
            return e;
        if ((e = timed(s, total, C_SORT, log, [&]() {
                 return wfpt::launch_sort_pairs(rb.keys.p, rb.idx.as<uint32_t>(), n, n_dev, key_bits(), scratch.p,
                                                scratch.bytes, s);
             })) != cudaSuccess)
            return e;
        if (reorder) {
            if ((e = timed(s, total, C_REORDER, log, [&]() {
                     return wfpt::launch_reorder(rb.idx.as<uint32_t>(), rb.rays_cur(), rb.rays_out(), rb.s2i_cur(),
                                                 rb.s2i_out(), rb.i2s_out(), n, n_dev, s);
                 })) != cudaSuccess)
                return e;
            rb.swap();
        }
        return timed(s, total, C_TRACE_SORT, log, [&]() {
            return wfpt::launch_trace(sc, kind, rb.rays_cur(), rb.results.as<wfpt_hit>(),
                                      reorder ? nullptr : rb.idx.as<uint32_t>(), n, n_dev, closest ? 1 : 0, s, wk);
        });
    }

    int primary_kind() const { return cfg.primary_bvh_kind >= 0 ? cfg.primary_bvh_kind : cfg.bvh_kind; }

    // Makes stream s wait for the shadow batches forked last (if any).
    cudaError_t join_shadow(cudaStream_t s) {
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < pending_slots && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(s, slots[k].ev_done, 0);
        pending_slots = 0;
        return e;
    }

    // Renderer::shadowPass (Renderer.cpp:133-154) over input rays `in`
    // whose slot->pixel map is `in_s2i`; n_in is the capacity, n_in_dev the
    // device-side count (null when the host count is exact).  Batches of
    // batch_diff input rays, as the reference cuts them.
    //  - Overlapped (cfg.shadow_overlap, not timed): batch b is generated,
    //    traced and reconstructed on the stream of slot b % nslots, forked
    //    from s; s waits for the last batch generated on every slot before it
    //    goes on (raygenShadow reads the seeds that the next raygenPath
    //    rewrites), and join_shadow() makes the next shadow pass wait for
    //    all of them, which keeps the order of the additions into
    //    out_pixels.  A slot's batches run in order on its stream, so a
    //    slot's buffers are reused only after its previous batch is done.
    //  - Sequential: every batch on s, in the reference's order.
    cudaError_t shadow_pass(const wfpt_ray* in_rays, const wfpt_hit* in_res, const int32_t* in_s2i, uint32_t n_in,
                            const uint32_t* n_in_dev, float* in_pixels, float* out_pixels,
                            uint32_t* batch_counters, cudaStream_t s, int kind, int slot_log) {
        const int S = cfg.num_shadow_samples;
        const uint32_t batch_diff = (uint32_t)(kMaxBatch / S);
        cudaError_t e;
        if ((e = join_shadow(s)) != cudaSuccess) return e;
        if (cfg.shadow_overlap && !timing_on && nslots >= 1 && (int)slots.size() >= nslots) {
            if ((e = cudaEventRecord(ev_fork, s)) != cudaSuccess) return e;
            const uint32_t nb = (n_in + batch_diff - 1) / batch_diff;
            const int used = (int)std::min<uint32_t>((uint32_t)nslots, std::max(nb, 1u));
            for (int k = 0; k < used; ++k)
                if ((e = cudaStreamWaitEvent(slots[k].stream, ev_fork, 0)) != cudaSuccess) return e;
            for (uint32_t b = 0; b < nb; ++b) {
                ShadowSlot& sl = slots[b % used];
                const cudaStream_t ss = sl.stream;
                const uint32_t bb = b * batch_diff, bs = std::min(batch_diff, n_in - bb);
                const uint32_t* n_sh_dev = nullptr;
                if (n_in_dev) {
                    uint32_t* bc = batch_counters + (b % used);
                    if ((e = wfpt::launch_batch_count(n_in_dev, bb, bs, S, bc, ss)) != cudaSuccess) return e;
                    n_sh_dev = bc;
                }
                sl.rb.swapped = false;
                if ((e = wfpt::launch_raygen_shadow(seeds.as<uint32_t>(), in_rays, in_res, sl.rb.rays_cur(),
                                                    sl.rb.s2i_cur(), sl.rb.i2s_cur(), light, cfg.shadow_radius,
                                                    (int)bb, (int)bs, n_in_dev, S, ss)) != cudaSuccess)
                    return e;
                if ((e = cudaEventRecord(sl.ev_rg, ss)) != cudaSuccess) return e;
                if ((e = trace_rays(sl.rb, bs * (uint32_t)S, n_sh_dev, cfg.sort_shadow_rays != 0,
                                    cfg.reorder_shadow_rays != 0, false, ss, sl.work.as<uint32_t>(), sl.scratch,
                                    kind)) != cudaSuccess)
                    return e;
                if ((e = wfpt::launch_reconstruct_shadow(sl.rb.results.as<wfpt_hit>(), in_s2i, sl.rb.i2s_cur(),
                                                         in_pixels, out_pixels, (int)bb, (int)bs, n_in_dev, S, 0,
                                                         ss)) != cudaSuccess)
                    return e;
            }
            for (int k = 0; k < used; ++k) {
                if ((e = cudaEventRecord(slots[k].ev_done, slots[k].stream)) != cudaSuccess) return e;
                if ((e = cudaStreamWaitEvent(s, slots[k].ev_rg, 0)) != cudaSuccess) return e;
            }
            pending_slots = used;
            last_slots = std::max(last_slots, used);
            return cudaSuccess;
        }
        uint32_t bb = 0;
        do {
            uint32_t be = std::min(bb + batch_diff, n_in);
            uint32_t bs = be - bb;
            const uint32_t* n_sh_dev = nullptr;
            if (n_in_dev) {
                if ((e = wfpt::launch_batch_count(n_in_dev, bb, bs, S, batch_counters, s)) != cudaSuccess) return e;
                n_sh_dev = batch_counters;
            }
            shadow.swapped = false;
            if ((e = timed(s, T_SHADOW, C_NONE, -1, [&]() {
                     return wfpt::launch_raygen_shadow(seeds.as<uint32_t>(), in_rays, in_res, shadow.rays_cur(),
                                                       shadow.s2i_cur(), shadow.i2s_cur(), light, cfg.shadow_radius,
                                                       (int)bb, (int)bs, n_in_dev, S, s);
                 })) != cudaSuccess)
                return e;
            if ((e = trace_rays(shadow, bs * (uint32_t)S, n_sh_dev, cfg.sort_shadow_rays != 0,
                                cfg.reorder_shadow_rays != 0, false, s, work.as<uint32_t>(), sort_scratch, kind,
                                T_SHADOW, slot_log)) != cudaSuccess)
                return e;
            if ((e = wfpt::launch_reconstruct_shadow(shadow.results.as<wfpt_hit>(), in_s2i, shadow.i2s_cur(),
                                                     in_pixels, out_pixels, (int)bb, (int)bs, n_in_dev, S, 0, s)) !=
                cudaSuccess)
                return e;
            bb = be;
        } while (bb != n_in);
        last_slots = std::max(last_slots, 1);
        return cudaSuccess;
    }

    // Renderer::primaryPass (Renderer.cpp:124-131).
    // hit_counter (nullable): receives the number of primary hits (the
    // shadow pass's input count, countRayHits) from reconstructSmooth.
    // fresh: target is this pass's colour buffer, taken as cleared (its
    // pixels are written, not accumulated); otherwise reconstructSmooth adds
    // into it (the frame buffer of the primary-rays mode, over the samples).
    cudaError_t primary_pass(const float* s2w, const float* eye, float zfar, int pass, float* target, cudaStream_t s,
                             const wfpt::FrameParams* fp, uint32_t* hit_counter, bool fresh) {
        uint32_t n = (uint32_t)width * height;
        cudaError_t e;
        int sample_index = pass + cfg.num_primary_samples * (frame_index - 1);
        if ((e = timed(s, T_PRIMARY, C_NONE, -1, [&]() {
                 cudaError_t r = wfpt::launch_raygen_primary(s2w, i2p.as<int32_t>(), primary.rays_cur(), eye,
                                                             sample_index, width, height, zfar, s, fp, pass,
                                                             cfg.num_primary_samples);
                 if (r != cudaSuccess) return r;
                 return wfpt::launch_trace(*wfpt::scene_device(scene), primary_kind(), primary.rays_cur(),
                                           primary.results.as<wfpt_hit>(), nullptr, n, nullptr, 1, s,
                                           work.as<uint32_t>());
             })) != cudaSuccess)
            return e;
        const float one = 1.0f;
        uint32_t one_bits;
        std::memcpy(&one_bits, &one, 4);
        if ((e = wfpt::launch_fill_u32(decreases.p, one_bits, (size_t)n * 4, s)) != cudaSuccess) return e;
        return wfpt::launch_reconstruct_smooth(primary.rays_cur(), primary.results.as<wfpt_hit>(), i2p.as<int32_t>(),
                                               target, decreases.as<float>(), geoms, light, bg, n, nullptr,
                                               cfg.num_primary_samples, s, hit_counter, fresh);
    }

    // One frame.  fp (nullable): device-side frame parameters that replace
    // s2w/eye/zfar/frame_index, so that the same launches can be captured
    // once into a graph and replayed every frame.  (The reference also
    // clears `pixels` on frame 1; interpolateColors overwrites all of it on
    // frame 1, so that clear is not needed.)
    cudaError_t frame(const float* s2w, const float* eye, float zfar, float* pixels, float* frame_pixels,
                      cudaStream_t s, const wfpt::FrameParams* fp = nullptr) {
        uint32_t n = (uint32_t)width * height;
        cudaError_t e;
        tev_used = 0;
        spans.clear();
        last_slots = 0;
        primary.swapped = queue[0].swapped = queue[1].swapped = shadow.swapped = false;
        if ((e = cudaMemsetAsync(frame_pixels, 0, (size_t)n * 16, s)) != cudaSuccess) return e;
        if ((e = cudaMemsetAsync(counters.p, 0, (size_t)cfg.num_primary_samples * kCountersPerPass * 4, s)) !=
            cudaSuccess)
            return e;
        int rt = cfg.ray_type;
        if (rt == WFPT_PATH_RAYS || rt == WFPT_SHADOW_RAYS)
            if ((e = wfpt::launch_init_seeds(seeds.as<uint32_t>(), n, frame_index, s, fp)) != cudaSuccess) return e;
        for (int pass = 0; pass < cfg.num_primary_samples; ++pass) {
            if (rt == WFPT_PRIMARY_RAYS) {
                if ((e = primary_pass(s2w, eye, zfar, pass, frame_pixels, s, fp, nullptr, false)) != cudaSuccess)
                    return e;
                continue;
            }
            // renderShadow / renderPath (Renderer.cpp:168-199).  Colour
            // buffers alternate between passes when shadow passes overlap
            // the next bounce (one is still read by the pending shadow pass).
            float* auxb[2] = {aux.as<float>(), cfg.shadow_overlap ? aux2.as<float>() : aux.as<float>()};
            int ai = 0;
            if ((e = join_shadow(s)) != cudaSuccess) return e;
            // The colour buffers are not cleared (Renderer.cpp clears them per
            // pass): every pixel the shadow pass reads back was written by
            // this pass's reconstructSmooth in fresh mode.
            if ((e = primary_pass(s2w, eye, zfar, pass, auxb[ai], s, fp, cnt(pass, kCntHits + 0), true)) !=
                cudaSuccess)
                return e;
            if ((e = shadow_pass(primary.rays_cur(), primary.results.as<wfpt_hit>(), i2p.as<int32_t>(), n, nullptr,
                                 auxb[ai], frame_pixels, cnt(pass, kCntBatch), s, primary_kind(), 0)) != cudaSuccess)
                return e;
            if (rt != WFPT_PATH_RAYS) continue;
            int qsel = 0;  // PathQueue::swapBuffers
            for (int bounce = 0; bounce < cfg.recursion_depth; ++bounce) {
                ai ^= 1;
                RayBufferDev& out = queue[qsel ? 0 : 1];
                const wfpt_ray* in_rays;
                const wfpt_hit* in_res;
                const int32_t* in_s2i;
                const uint32_t* in_cnt;
                if (bounce == 0) {
                    in_rays = primary.rays_cur();
                    in_res = primary.results.as<wfpt_hit>();
                    in_s2i = i2p.as<int32_t>();
                    in_cnt = nullptr;
                } else {
                    RayBufferDev& in = queue[qsel ? 1 : 0];
                    in_rays = in.rays_cur();
                    in_res = in.results.as<wfpt_hit>();
                    in_s2i = in.s2i_cur();
                    in_cnt = cnt(pass, kCntPath + bounce - 1);
                }
                out.swapped = false;
                uint32_t* out_cnt = cnt(pass, kCntPath + bounce);
                const bool sort_b = cfg.sort_path_rays != 0 && ((cfg.path_sort_skip >> bounce) & 1) == 0;
                // A sorted bounce gets its Morton keys from the path-ray
                // generation (the same keys the Morton kernel would compute
                // from the written rays); a timed frame keeps the Morton
                // kernel, whose time the sort log reports.
                wfpt::MortonOut mo{};
                const bool fused_keys = sort_b && !timing_on;
                if (fused_keys) {
                    mo.kind = cfg.morton_kind;
                    mo.keys = out.keys.p;
                    mo.indices = out.idx.as<uint32_t>();
                    for (int k = 0; k < 3; ++k) {
                        mo.box.smin[k] = smin[k];
                        mo.box.ssize[k] = smax[k] - smin[k];
                    }
                }
                // Renderer::pathPass -> tracePathRays (Renderer.cpp:156-162, 277-297).
                if ((e = timed(s, T_PATH, C_NONE, -1, [&]() {
                         return wfpt::launch_raygen_path(seeds.as<uint32_t>(), geoms, in_rays, out.rays_cur(), in_s2i,
                                                         out.s2i_cur(), in_res, decreases.as<float>(), out_cnt, n,
                                                         in_cnt, cfg.albedo, path_scratch.p, s,
                                                         fused_keys ? &mo : nullptr);
                     })) != cudaSuccess)
                    return e;
                if ((e = trace_rays(out, n, out_cnt, sort_b, sort_b && cfg.reorder_path_rays != 0, true, s,
                                    work.as<uint32_t>(), sort_scratch, cfg.bvh_kind, T_PATH, 100 + bounce,
                                    fused_keys)) != cudaSuccess)
                    return e;
                if ((e = wfpt::launch_reconstruct_smooth(out.rays_cur(), out.results.as<wfpt_hit>(), out.s2i_cur(),
                                                         auxb[ai], decreases.as<float>(), geoms, light, bg, n,
                                                         out_cnt, cfg.num_primary_samples, s,
                                                         cnt(pass, kCntHits + bounce + 1), true)) != cudaSuccess)
                    return e;
                if ((e = shadow_pass(out.rays_cur(), out.results.as<wfpt_hit>(), out.s2i_cur(), n, out_cnt,
                                     auxb[ai], frame_pixels, cnt(pass, kCntBatch), s, cfg.bvh_kind, bounce + 1)) !=
                    cudaSuccess)
                    return e;
                qsel ^= 1;  // PathQueue::swap
            }
        }
        if ((e = join_shadow(s)) != cudaSuccess) return e;
        if (cfg.accumulate_fp64)
            return wfpt::launch_interpolate_colors_fp64(frame_pixels, pixels, accum64.as<double>(), n, frame_index,
                                                        cfg.key_value, cfg.white_point, s, fp);
        return wfpt::launch_interpolate_colors(frame_pixels, pixels, n, frame_index, cfg.key_value, cfg.white_point, s,
                                               fp);
    }
};

namespace wfpt {
void set_fail_alloc_after(int n) { g_fail_alloc_after = n < 0 ? -1 : n; }
int get_fail_alloc_after() { return g_fail_alloc_after; }
void set_shadow_slots(int n) { g_shadow_slots = n < 0 ? 0 : (n > kMaxSlots ? kMaxSlots : n); }
int get_shadow_slots() { return g_shadow_slots; }
}  // namespace wfpt

namespace {

wfpt_status check_config(const wfpt_renderer_config* c) {
    if (c->ray_type < WFPT_PRIMARY_RAYS || c->ray_type > WFPT_PATH_RAYS) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->num_primary_samples < 1 || c->num_primary_samples > kMaxSamples) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->num_shadow_samples < 1 || c->num_shadow_samples > kMaxSamples) return WFPT_ERR_INVALID_ARGUMENT;
    if (!(c->shadow_radius > 0.0f && c->shadow_radius <= 100.0f)) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->recursion_depth < 0 || c->recursion_depth > kMaxDepth) return WFPT_ERR_INVALID_ARGUMENT;
    if (!(c->key_value > 0.0f && c->key_value <= 2.0f)) return WFPT_ERR_INVALID_ARGUMENT;
    if (!(c->white_point > 0.0f && c->white_point <= 2.0f)) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->morton_kind < WFPT_MORTON_AILA32 || c->morton_kind > WFPT_MORTON_6D64) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->bvh_kind != WFPT_BVH2_FP32 && c->bvh_kind != WFPT_BVH8_Q8) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->path_sort_skip < 0 || c->path_sort_skip > 255) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->shadow_overlap < 0 || c->shadow_overlap > 1) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->primary_bvh_kind != -1 && c->primary_bvh_kind != WFPT_BVH2_FP32 && c->primary_bvh_kind != WFPT_BVH8_Q8)
        return WFPT_ERR_INVALID_ARGUMENT;
    if (c->timing < 0 || c->timing > 1) return WFPT_ERR_INVALID_ARGUMENT;
    if (c->accumulate_fp64 < 0 || c->accumulate_fp64 > 1) return WFPT_ERR_INVALID_ARGUMENT;
    return WFPT_OK;
}

}  // namespace

extern "C" {

// Defaults of Renderer::Renderer (Renderer.cpp:300-308) overridden by the
// registered option defaults (AppEnvironment.cpp:24-35), as Renderer::init
// applies them.
void wfpt_renderer_config_default(wfpt_renderer_config* c) {
    if (!c) return;
    c->ray_type = WFPT_PRIMARY_RAYS;
    c->num_primary_samples = 1;
    c->num_shadow_samples = 2;
    c->shadow_radius = 0.001f;
    c->recursion_depth = 1;
    c->key_value = 0.6f;
    c->white_point = 2.0f;
    c->russian_roulette = 0;
    c->sort_shadow_rays = 0;
    c->reorder_shadow_rays = 0;
    c->sort_path_rays = 0;
    c->reorder_path_rays = 0;
    c->morton_kind = WFPT_MORTON_AILA32;
    c->bvh_kind = WFPT_BVH2_FP32;
    c->albedo = 0.8f;
    c->use_graph = 0;
    c->path_sort_skip = 0;
    c->shadow_overlap = 1;
    c->primary_bvh_kind = -1;
    c->timing = 0;
    c->accumulate_fp64 = 0;
}

wfpt_status wfpt_renderer_create(const wfpt_renderer_config* config, wfpt_renderer** renderer) {
    if (!renderer) return WFPT_ERR_INVALID_ARGUMENT;
    *renderer = nullptr;
    wfpt_renderer_config c;
    if (config) {
        c = *config;
    } else {
        wfpt_renderer_config_default(&c);
    }
    if (check_config(&c) != WFPT_OK) {
        wfpt::set_error("renderer option out of range");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    wfpt_renderer* r = new (std::nothrow) wfpt_renderer();
    if (!r) return WFPT_ERR_OUT_OF_MEMORY;
    r->cfg = c;
    *renderer = r;
    return WFPT_OK;
}

void wfpt_renderer_destroy(wfpt_renderer* r) { delete r; }

wfpt_status wfpt_renderer_set_config(wfpt_renderer* r, const wfpt_renderer_config* config) {
    if (!r || !config) return WFPT_ERR_INVALID_ARGUMENT;
    if (check_config(config) != WFPT_OK) {
        wfpt::set_error("renderer option out of range");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    r->cfg = *config;
    r->frame_index = 1;  // every setter of the reference resets the frame index
    return WFPT_OK;
}

wfpt_status wfpt_renderer_set_scene(wfpt_renderer* r, const wfpt_scene* scene, const wfpt_geometry* geometries,
                                    const float scene_min[3], const float scene_max[3], const float light[3],
                                    const float background[3]) {
    if (!r || !scene || !geometries) return WFPT_ERR_INVALID_ARGUMENT;
    if (!wfpt::scene_has(scene, r->cfg.bvh_kind) || !wfpt::scene_has(scene, r->primary_kind())) {
        wfpt::set_error("scene was built without the renderer's BVH kind");
        return WFPT_ERR_UNSUPPORTED;
    }
    r->scene = scene;
    r->geoms = geometries;
    float mn[3], mx[3];
    wfpt::scene_bounds(scene, mn, mx);
    for (int k = 0; k < 3; ++k) {
        r->smin[k] = scene_min ? scene_min[k] : mn[k];
        r->smax[k] = scene_max ? scene_max[k] : mx[k];
        if (light) r->light[k] = light[k];
        if (background) r->bg[k] = background[k];
    }
    return WFPT_OK;
}

void wfpt_renderer_reset_frame_index(wfpt_renderer* r) {
    if (r) r->frame_index = 1;
}

wfpt_status wfpt_renderer_render(wfpt_renderer* r, const wfpt_camera* camera, int width, int height, float* pixels,
                                 float* frame_pixels, void* stream) {
    if (!r || !camera || !pixels || !frame_pixels) return WFPT_ERR_INVALID_ARGUMENT;
    if (!r->scene) {
        wfpt::set_error("renderer has no scene");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    if (!wfpt::scene_has(r->scene, r->cfg.bvh_kind) || !wfpt::scene_has(r->scene, r->primary_kind())) {
        wfpt::set_error("scene was built without the renderer's BVH kind");
        return WFPT_ERR_UNSUPPORTED;
    }
    if (width <= 0 || height <= 0 || (long long)width * height > (1ll << 28)) {
        wfpt::set_error("bad resolution");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = r->prepare(width, height);
    if (e != cudaSuccess) return wfpt::from_cuda(e);
    float s2w[16];
    if (!wfpt::camera_screen_to_world(camera->position, camera->rotation_deg, camera->fov_deg,
                                      (float)width / (float)height, camera->znear, camera->zfar, s2w)) {
        wfpt::set_error("bad camera");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    if ((e = cudaEventRecord(r->ev0, s)) != cudaSuccess) return wfpt::from_cuda(e);
    r->timing_on = r->cfg.timing != 0;
    r->last_timed = false;
    if (r->cfg.use_graph && !r->timing_on)
        e = r->render_graph(s2w, camera->position, camera->zfar, pixels, frame_pixels, s);
    else
        e = r->frame(s2w, camera->position, camera->zfar, pixels, frame_pixels, s);
    r->last_timed = r->timing_on && e == cudaSuccess;
    r->timing_on = false;
    if (e != cudaSuccess) return wfpt::from_cuda(e);
    if ((e = cudaEventRecord(r->ev1, s)) != cudaSuccess) return wfpt::from_cuda(e);
    size_t cbytes = (size_t)r->cfg.num_primary_samples * kCountersPerPass * 4;
    if ((e = cudaMemcpyAsync(r->host_counters, r->counters.p, cbytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return wfpt::from_cuda(e);
    if ((e = cudaEventRecord(r->ev2, s)) != cudaSuccess) return wfpt::from_cuda(e);
    r->last_spp = r->cfg.num_primary_samples;
    r->stats_pending = true;
    ++r->frame_index;
    return WFPT_OK;
}

wfpt_status wfpt_renderer_get_stats(wfpt_renderer* r, wfpt_render_stats* st) {
    if (!r || !st) return WFPT_ERR_INVALID_ARGUMENT;
    std::memset(st, 0, sizeof(*st));
    if (!r->stats_pending) return WFPT_OK;
    cudaError_t e = cudaEventSynchronize(r->ev2);
    if (e != cudaSuccess) return wfpt::from_cuda(e);
    cudaEventElapsedTime(&r->frame_ms, r->ev0, r->ev1);
    r->fill_stats(st);
    r->fill_times(st);
    st->frame_ms = r->frame_ms;
    st->shadow_batch_slots = r->last_slots;
    return WFPT_OK;
}

}  // extern "C"

// ------------------------------------------------------------ batches
// Each request gets its own renderer (buffers sized to its resolution,
// counters, traversal work counters); the batch graph records every
// renderer's frame plus the read-back of its counters, request i on branch
// i % streams.
struct wfpt_batch {
    std::vector<wfpt_request> reqs;
    std::vector<wfpt_renderer*> rs;
    std::vector<cudaStream_t> branches;  // [0] is the capture stream
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr, ev0 = nullptr, ev1 = nullptr;
    wfpt::FrameParams* fp_dev = nullptr;
    std::vector<wfpt::FrameParams> fp_host;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t graph_kernels = 0;
    bool pending = false;
    float ms = 0.0f;

    ~wfpt_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (fp_dev) cudaFree(fp_dev);
        for (cudaEvent_t ev : joins)
            if (ev) cudaEventDestroy(ev);
        for (cudaEvent_t ev : {fork, ev0, ev1})
            if (ev) cudaEventDestroy(ev);
        for (cudaStream_t s : branches)
            if (s) cudaStreamDestroy(s);
        for (wfpt_renderer* r : rs) delete r;
    }

    // Per-request frame parameters from the current cameras and frame indices.
    bool fill_params() {
        for (size_t i = 0; i < reqs.size(); ++i) {
            const wfpt_request& q = reqs[i];
            wfpt::FrameParams& p = fp_host[i];
            std::memset(&p, 0, sizeof(p));
            if (!wfpt::camera_screen_to_world(q.camera.position, q.camera.rotation_deg, q.camera.fov_deg,
                                              (float)q.width / (float)q.height, q.camera.znear, q.camera.zfar,
                                              p.s2w))
                return false;
            for (int k = 0; k < 3; ++k) p.eye[k] = q.camera.position[k];
            p.zfar = q.camera.zfar;
            p.frame_index = rs[i]->frame_index;
        }
        return true;
    }

    cudaError_t record() {
        const int K = (int)branches.size();
        const cudaStream_t cs = branches[0];
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return e;
        uint64_t k0 = wfpt::launch_count();
        cudaError_t fe = cudaEventRecord(fork, cs);
        for (int k = 1; k < K && fe == cudaSuccess; ++k) fe = cudaStreamWaitEvent(branches[k], fork, 0);
        for (size_t i = 0; i < reqs.size() && fe == cudaSuccess; ++i) {
            wfpt_renderer* r = rs[i];
            const wfpt_request& q = reqs[i];
            const cudaStream_t s = branches[i % K];
            const wfpt::FrameParams& p = fp_host[i];
            fe = r->frame(p.s2w, p.eye, p.zfar, q.pixels, q.frame_pixels, s, fp_dev + i);
            if (fe == cudaSuccess)
                fe = cudaMemcpyAsync(r->host_counters, r->counters.p,
                                     (size_t)r->cfg.num_primary_samples * kCountersPerPass * 4,
                                     cudaMemcpyDeviceToHost, s);
        }
        for (int k = 1; k < K && fe == cudaSuccess; ++k) {
            fe = cudaEventRecord(joins[k], branches[k]);
            if (fe == cudaSuccess) fe = cudaStreamWaitEvent(cs, joins[k], 0);
        }
        e = cudaStreamEndCapture(cs, &graph);
        if (fe != cudaSuccess) return fe;
        if (e != cudaSuccess) return e;
        graph_kernels = wfpt::launch_count() - k0;
        return cudaGraphInstantiate(&exec, graph, 0);
    }
};

extern "C" {

wfpt_status wfpt_batch_create(const wfpt_request* requests, uint32_t count, int streams, wfpt_batch** batch) {
    if (!batch) return WFPT_ERR_INVALID_ARGUMENT;
    *batch = nullptr;
    if (!requests || count == 0 || streams < 1 || streams > 16) {
        wfpt::set_error("need requests, count >= 1 and 1 <= streams <= 16");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    for (uint32_t i = 0; i < count; ++i) {
        const wfpt_request& q = requests[i];
        if (!q.scene || !q.geometries || !q.pixels || !q.frame_pixels) {
            wfpt::set_error("request with a null scene, geometry table or image");
            return WFPT_ERR_INVALID_ARGUMENT;
        }
        if (q.width <= 0 || q.height <= 0 || (long long)q.width * q.height > (1ll << 28)) {
            wfpt::set_error("request with a bad resolution");
            return WFPT_ERR_INVALID_ARGUMENT;
        }
        if (check_config(&q.config) != WFPT_OK) {
            wfpt::set_error("request option out of range");
            return WFPT_ERR_INVALID_ARGUMENT;
        }
        if (!wfpt::scene_has(q.scene, q.config.bvh_kind) ||
            (q.config.primary_bvh_kind >= 0 && !wfpt::scene_has(q.scene, q.config.primary_bvh_kind))) {
            wfpt::set_error("request scene was built without the request's BVH kind");
            return WFPT_ERR_UNSUPPORTED;
        }
    }
    wfpt_batch* b = new (std::nothrow) wfpt_batch();
    if (!b) return WFPT_ERR_OUT_OF_MEMORY;
    b->reqs.assign(requests, requests + count);
    b->fp_host.resize(count);
    cudaError_t e = cudaSuccess;
    for (uint32_t i = 0; i < count && e == cudaSuccess; ++i) {
        wfpt_renderer* r = new (std::nothrow) wfpt_renderer();
        if (!r) {
            delete b;
            return WFPT_ERR_OUT_OF_MEMORY;
        }
        b->rs.push_back(r);
        const wfpt_request& q = b->reqs[i];
        r->cfg = q.config;
        r->cfg.use_graph = 0;
        r->scene = q.scene;
        r->geoms = q.geometries;
        wfpt::scene_bounds(q.scene, r->smin, r->smax);
        for (int k = 0; k < 3; ++k) {
            r->light[k] = q.light[k];
            r->bg[k] = q.background[k];
        }
        e = r->prepare(q.width, q.height);
        r->last_spp = r->cfg.num_primary_samples;
    }
    b->branches.assign((size_t)streams, nullptr);
    b->joins.assign((size_t)streams, nullptr);
    for (int k = 0; k < streams && e == cudaSuccess; ++k) {
        e = cudaStreamCreateWithFlags(&b->branches[k], cudaStreamNonBlocking);
        if (e == cudaSuccess && k > 0) e = cudaEventCreateWithFlags(&b->joins[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess)
        e = wfpt::dev_malloc(reinterpret_cast<void**>(&b->fp_dev), (size_t)count * sizeof(wfpt::FrameParams));
    if (e == cudaSuccess) e = wfpt::sort_prepare();
    if (e == cudaSuccess) e = wfpt::trace_prepare();
    if (e == cudaSuccess && !b->fill_params()) {
        delete b;
        wfpt::set_error("request with a bad camera");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    if (e == cudaSuccess) e = b->record();
    if (e != cudaSuccess) {
        delete b;
        return wfpt::from_cuda(e);
    }
    *batch = b;
    return WFPT_OK;
}

void wfpt_batch_destroy(wfpt_batch* batch) { delete batch; }

wfpt_status wfpt_batch_render(wfpt_batch* b, const wfpt_camera* cameras, void* stream) {
    if (!b) return WFPT_ERR_INVALID_ARGUMENT;
    if (cameras)
        for (size_t i = 0; i < b->reqs.size(); ++i) b->reqs[i].camera = cameras[i];
    if (!b->fill_params()) {
        wfpt::set_error("bad camera");
        return WFPT_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e;
    if ((e = cudaEventRecord(b->ev0, s)) != cudaSuccess) return wfpt::from_cuda(e);
    // Pageable source: the copy is staged before the call returns.
    if ((e = cudaMemcpyAsync(b->fp_dev, b->fp_host.data(), b->fp_host.size() * sizeof(wfpt::FrameParams),
                             cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return wfpt::from_cuda(e);
    if ((e = cudaGraphLaunch(b->exec, s)) != cudaSuccess) return wfpt::from_cuda(e);
    if ((e = cudaEventRecord(b->ev1, s)) != cudaSuccess) return wfpt::from_cuda(e);
    wfpt::count_launch((uint32_t)b->graph_kernels);
    for (wfpt_renderer* r : b->rs) ++r->frame_index;
    b->pending = true;
    return WFPT_OK;
}

wfpt_status wfpt_batch_get_stats(wfpt_batch* b, uint32_t i, wfpt_render_stats* st) {
    if (!b || !st || i >= b->rs.size()) return WFPT_ERR_INVALID_ARGUMENT;
    std::memset(st, 0, sizeof(*st));
    if (!b->pending) return WFPT_OK;
    cudaError_t e = cudaEventSynchronize(b->ev1);
    if (e != cudaSuccess) return wfpt::from_cuda(e);
    cudaEventElapsedTime(&b->ms, b->ev0, b->ev1);
    b->rs[i]->fill_stats(st);
    st->frame_ms = b->ms;
    return WFPT_OK;
}

uint64_t wfpt_batch_kernels(const wfpt_batch* b) { return b ? b->graph_kernels : 0; }

void wfpt_batch_reset_frame_index(wfpt_batch* b) {
    if (!b) return;
    for (wfpt_renderer* r : b->rs) r->frame_index = 1;
}

}  // extern "C"
