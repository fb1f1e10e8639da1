// Exercises the C++ facade (include/wfpt.hpp) the way reference-side code
// would use it.  `facade_test host` needs no GPU: errors surface as
// wfpt_cxx::Error and a host-only scene builds.  `facade_test gpu` runs
// RayGen::primary, Tracer::trace and Tracer::traceSort (with and without
// reordering), a scene built on the device from device buffers, and
// RayGen::shadow on a seeded triangle soup, checking that traceSort and the
// device-built scene return the same hits as trace.  Prints "FACADE OK" on
// success.
#include <cstdio>
#include <cstring>
#include <vector>

#include "wfpt.hpp"

using namespace wfpt_cxx;

static int fail(const char* what) {
    std::printf("FAIL: %s\n", what);
    return 1;
}

static void soup(std::vector<float>& pos, std::vector<uint32_t>& idx, uint32_t ntri) {
    uint32_t nv = 0, nt = ntri;
    check(wfpt_generate_scene(0, 3, ntri, nullptr, nullptr, &nv, nullptr, &nt));
    pos.resize(3 * (size_t)nv);
    std::vector<float> nrm(3 * (size_t)nv);
    idx.resize(3 * (size_t)nt);
    check(wfpt_generate_scene(0, 3, ntri, pos.data(), nrm.data(), &nv, idx.data(), &nt));
}

static int host_mode() {
    bool threw = false;
    try {
        check(wfpt_sort_pairs(nullptr, nullptr, 10, nullptr, 0, nullptr, 0, nullptr));
    } catch (const Error& e) {
        threw = e.status == WFPT_ERR_INVALID_ARGUMENT && std::strstr(e.what(), "key_bits") != nullptr;
    }
    if (!threw) return fail("invalid sort arguments did not throw");
    threw = false;
    wfpt_renderer_config c;
    wfpt_renderer_config_default(&c);
    c.recursion_depth = 99;
    try {
        Renderer r(&c);
    } catch (const Error& e) {
        threw = e.status == WFPT_ERR_INVALID_ARGUMENT;
    }
    if (!threw) return fail("bad renderer config did not throw");
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    soup(pos, idx, 2000);
    Scene s(pos.data(), (uint32_t)(pos.size() / 3), idx.data(), 2000, nullptr, 0,
            (1 << WFPT_BVH2_FP32) | (1 << WFPT_BVH8_Q8) | WFPT_SCENE_HOST_ONLY);
    if (s.info().num_triangles != 2000 || s.info().bvh8_nodes == 0) return fail("host-only scene info");
    std::printf("FACADE OK\n");
    return 0;
}

template <typename T>
static std::vector<T> to_host(const T* d, size_t n) {
    std::vector<T> h(n);
    check_cuda(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
}

static int gpu_mode() {
    std::vector<float> pos;
    std::vector<uint32_t> idx;
    soup(pos, idx, 20000);
    Scene scene(pos.data(), (uint32_t)(pos.size() / 3), idx.data(), 20000);
    const wfpt_scene_info info = scene.info();
    wfpt_camera cam = {{0.5f, 0.5f, 2.2f}, {0.0f, 0.0f, 0.0f}, 45.0f, 0.001f, 10.0f};
    const int w = 160, h = 120, n = w * h;

    RayGen gen;
    gen.init();
    gen.initSeeds(n, 1);
    RayBuffer rays;
    gen.primary(rays, cam, w, h, 0);
    if (rays.getSize() != n) return fail("primary size");
    Tracer tracer;
    tracer.init();
    for (int kind : {WFPT_BVH2_FP32, WFPT_BVH8_Q8}) {
        tracer.setAccelerationStructure(scene, kind);
        rays.setClosestHit(true);
        if (tracer.trace(rays) < 0.0f) return fail("trace time");
        const std::vector<wfpt_hit> plain = to_host(rays.getResultBuffer(), (size_t)n);
        for (int morton : {WFPT_MORTON_AILA32, WFPT_MORTON_6D64}) {
            tracer.setMortonKind(morton);
            // Indirect: results land at each ray's own slot.
            std::array<float, 4> times;
            tracer.traceSort(rays, info.bounds_min, info.bounds_max, false, times);
            std::vector<wfpt_hit> ind = to_host(rays.getResultBuffer(), (size_t)n);
            if (std::memcmp(ind.data(), plain.data(), (size_t)n * sizeof(wfpt_hit)) != 0)
                return fail("indirect traceSort differs from trace");
            // Reordered: slot i holds the ray that sorted to position i.
            RayBuffer copy;
            copy.resize(n);
            check_cuda(cudaMemcpy(copy.getRayBuffer(), rays.getRayBuffer(), (size_t)n * sizeof(wfpt_ray),
                                  cudaMemcpyDeviceToDevice));
            check_cuda(cudaMemcpy(copy.getSlotToIndexBuffer(), rays.getSlotToIndexBuffer(), (size_t)n * 4,
                                  cudaMemcpyDeviceToDevice));
            copy.setClosestHit(true);
            tracer.traceSort(copy, info.bounds_min, info.bounds_max, true, times);
            if (times[2] <= 0.0f) return fail("reorder time");
            std::vector<wfpt_hit> re = to_host(copy.getResultBuffer(), (size_t)n);
            std::vector<uint32_t> order = to_host(copy.getIndexBuffer(), (size_t)n);
            for (int i = 0; i < n; ++i)
                if (std::memcmp(&re[i], &plain[order[i]], sizeof(wfpt_hit)) != 0)
                    return fail("reordered traceSort differs from trace");
        }
    }
    // The same mesh with both BVHs built on the GPU gives the same hits.
    {
        DeviceArray<float> dpos;
        DeviceArray<uint32_t> didx;
        dpos.resize(pos.size());
        didx.resize(idx.size());
        check_cuda(cudaMemcpy(dpos.get(), pos.data(), pos.size() * 4, cudaMemcpyHostToDevice));
        check_cuda(cudaMemcpy(didx.get(), idx.data(), idx.size() * 4, cudaMemcpyHostToDevice));
        Scene dscene = Scene::fromDevice(dpos.get(), (uint32_t)(pos.size() / 3), didx.get(), 20000);
        if (dscene.info().num_triangles != 20000) return fail("device-built scene info");
        tracer.setAccelerationStructure(scene, WFPT_BVH8_Q8);
        rays.setClosestHit(true);
        tracer.trace(rays);
        const std::vector<wfpt_hit> host_hits = to_host(rays.getResultBuffer(), (size_t)n);
        tracer.setAccelerationStructure(dscene, WFPT_BVH8_Q8);
        tracer.trace(rays);
        const std::vector<wfpt_hit> dev_hits = to_host(rays.getResultBuffer(), (size_t)n);
        // dscene ends with this block: the tracer must not keep it.
        tracer.setAccelerationStructure(scene, WFPT_BVH8_Q8);
        if (std::memcmp(host_hits.data(), dev_hits.data(), (size_t)n * sizeof(wfpt_hit)) != 0)
            return fail("device-built scene hits differ");
    }
    // Shadow rays of the primary hits, traced any-hit.
    RayBuffer shadow;
    const float light[3] = {0.5f, 1.6f, 0.5f};
    gen.shadow(shadow, rays, 0, n, 2, light, 0.1f);
    if (shadow.getSize() != 2 * n || shadow.getClosestHit()) return fail("shadow rays");
    tracer.trace(shadow);
    uint32_t flags = 0;
    check(wfpt_device_status(&flags));
    std::printf("FACADE OK\n");
    return 0;
}

int main(int argc, char** argv) {
    try {
        if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) return gpu_mode();
        return host_mode();
    } catch (const Error& e) {
        std::printf("FAIL: %s\n", e.what());
        return 1;
    }
}
