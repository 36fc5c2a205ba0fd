// C++ drop-in smoke test of the class surface, following the reference's driver
// (libCL/TEST/main.cpp): testRadixSort (:133-181), testFluid3D0 (:188-240) and
// testFluid3D1 with an EVT_INTEGRATE handler (:246-343), with fixed step counts instead of
// 7 seconds of wall clock, and with assertions the reference does not make; then the 2D
// model and the two BVH builds through their classes (the reference's driver has no test
// for them).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "gbFluid3D.hpp"

#define CHECK(c)                                                           \
    do {                                                                   \
        if (!(c)) {                                                        \
            std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);        \
            return 1;                                                      \
        }                                                                  \
    } while (0)

static unsigned lcg(unsigned& s) { return s = s * 1664525u + 1013904223u; }

static int testRadixSort(gbContext& ctx) {
    gbDevice& dev = ctx.getDevice(0);
    gbBuffer key(ctx, "bfKey"), val(ctx, "bfVal");
    CHECK(key.create<unsigned>(1024) && val.create<unsigned>(1024));
    key.map(gbBuffer::MAP_WRITE);
    val.map(gbBuffer::MAP_WRITE);
    unsigned s = 1;
    for (int i = 0; i < 1024; i++) {
        key.ptr<unsigned>()[i] = lcg(s) >> 1;
        val.ptr<unsigned>()[i] = i;
    }
    std::vector<unsigned> orig(key.ptr<unsigned>(), key.ptr<unsigned>() + 1024);
    key.unmap();
    val.unmap();
    gbRadixSort sort(ctx);
    CHECK(sort.compile());
    CHECK(sort.compute(dev, key, val, 0, 32));
    cudaDeviceSynchronize();
    key.map(gbBuffer::MAP_READ);
    val.map(gbBuffer::MAP_READ);
    for (int i = 1; i < 1024; i++) CHECK(key.ptr<unsigned>()[i - 1] <= key.ptr<unsigned>()[i]);
    for (int i = 0; i < 1024; i++) CHECK(orig[val.ptr<unsigned>()[i]] == key.ptr<unsigned>()[i]);
    CHECK(!sort.compute(dev, key, val, 0, 30));  // bit range must be a multiple of 4
    CHECK(gbStatus() == GBSPH_ERR_BIT_RANGE);
    std::printf("testRadixSort completed\n");
    return 0;
}

static int initParticles(gbFluid3D& fluid) {
    gbBuffer* b = fluid.getPositionBuffer();
    size_t n = fluid.getParticleCount();
    b->map(gbBuffer::MAP_WRITE);
    unsigned s = 7;
    for (size_t i = 0; i < n; i++) {
        float* p = b->ptr<float>() + 4 * i;
        p[0] = (float)(lcg(s) >> 8) / (1 << 24) - 0.5f;
        p[1] = (float)(lcg(s) >> 8) / (1 << 24) - 0.5f;
        p[2] = (float)(lcg(s) >> 8) / (1 << 24) - 0.5f;
        p[3] = 0;
    }
    return b->unmap() ? 0 : 1;
}

static int averagePosition(gbFluid3D& fluid, float avg[3]) {
    gbBuffer* b = fluid.getPositionBuffer();
    size_t n = fluid.getParticleCount();
    CHECK(b->map(gbBuffer::MAP_READ));
    avg[0] = avg[1] = avg[2] = 0;
    for (size_t i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            float v = b->ptr<float>()[4 * i + c];
            CHECK(std::isfinite(v));
            avg[c] += v / n;
        }
    return 0;
}

static int testFluid3D0(gbContext& ctx) {
    gbDevice& dev = ctx.getDevice(0);
    gbFluid3D fluid(ctx);
    CHECK(fluid.compile());
    CHECK(fluid.getParticleCount() == gbFluid3D::cLocalSize);
    fluid.setParticleCount(4096);
    CHECK(initParticles(fluid) == 0);
    for (int i = 0; i < 50; i++) CHECK(fluid.compute(dev));
    cudaDeviceSynchronize();
    float avg[3];
    CHECK(averagePosition(fluid, avg) == 0);
    CHECK(avg[2] < 0.0f);  // gravity (0,0,-9.8) pulled the cloud down
    gbBuffer& sp = fluid.getSortedPositionBuffer();
    CHECK(sp.map(gbBuffer::MAP_READ));
    for (size_t i = 0; i < fluid.getParticleCount(); i++) CHECK(sp.ptr<float>()[4 * i + 3] >= 1.0f);  // density
    std::printf("testFluid3D0: average particle position = %g %g %g\n", avg[0], avg[1], avg[2]);
    // a step from page-locked host state (computeHost) equals the same step on device buffers
    const size_t n = fluid.getParticleCount();
    float *in = nullptr, *out = nullptr;
    CHECK(cudaHostAlloc((void**)&in, 3 * n * 16, cudaHostAllocDefault) == cudaSuccess);
    CHECK(cudaHostAlloc((void**)&out, 3 * n * 16, cudaHostAllocDefault) == cudaSuccess);
    gbBuffer* bufs[3] = {fluid.getPositionBuffer(), fluid.getVelocityBuffer(), fluid.getForceBuffer()};
    for (int k = 0; k < 3; k++) {
        CHECK(bufs[k]->map(gbBuffer::MAP_READ));
        std::memcpy(in + 4 * n * k, bufs[k]->ptr<float>(), n * 16);
    }
    CHECK(fluid.computeHost(dev, in, in + 4 * n, in + 8 * n, out, out + 4 * n, out + 8 * n));
    cudaDeviceSynchronize();
    for (int k = 0; k < 3; k++) {  // back to the state before the step, then the device step
        CHECK(bufs[k]->map(gbBuffer::MAP_WRITE));
        std::memcpy(bufs[k]->ptr<float>(), in + 4 * n * k, n * 16);
        CHECK(bufs[k]->unmap());
    }
    CHECK(fluid.compute(dev));
    cudaDeviceSynchronize();
    for (int k = 0; k < 3; k++) {
        CHECK(bufs[k]->map(gbBuffer::MAP_READ));
        CHECK(std::memcmp(out + 4 * n * k, bufs[k]->ptr<float>(), n * 16) == 0);
    }
    cudaFreeHost(in);
    cudaFreeHost(out);
    return 0;
}

// libCL/TEST/main.cpp:280-314: the handler re-enqueues integrate-force, gravity and
// integrate-velocity and skips the clip box.
struct srtFluid : public srtEvent {
    int calls = 0;
    srtFluid() : srtEvent(gbFluid3D::EVT_INTEGRATE) {}
    bool operator()(gbFluid3D& f) override {
        calls++;
        return f.stage(GBSPH_STAGE_INTEGRATE_FORCE) && f.stage(GBSPH_STAGE_GRAVITY) &&
               f.stage(GBSPH_STAGE_INTEGRATE_VELOCITY);
    }
};

static int testFluid3D1(gbContext& ctx) {
    gbDevice& dev = ctx.getDevice(0);
    gbFluid3D fluid(ctx);
    CHECK(fluid.compile());
    fluid.setParticleCount(2048);
    CHECK(initParticles(fluid) == 0);
    srtFluid handler;
    fluid.addEventHandler(handler);
    for (int i = 0; i < 20; i++) CHECK(fluid.compute(dev));
    cudaDeviceSynchronize();
    CHECK(handler.calls == 20);
    float avg[3];
    CHECK(averagePosition(fluid, avg) == 0);
    std::printf("testFluid3D1: average particle position = %g %g %g\n", avg[0], avg[1], avg[2]);
    return 0;
}

// getParamBuffer (libCL/phys/oclFluid3D.cpp:198-201): the device copy of the parameters,
// read through the buffer's map() as a caller that binds it to its own kernels sees it; a
// host edit reaches it with the next compute().
static int testParamBuffer(gbContext& ctx) {
    typedef gbFluid3D::Params Params;
    gbDevice& dev = ctx.getDevice(0);
    gbFluid3D fluid(ctx);
    CHECK(fluid.compile());
    fluid.setParticleCount(1024);
    CHECK(initParticles(fluid) == 0);
    gbBuffer& pb = fluid.getParamBuffer();
    CHECK(pb.devicePtr() != nullptr && pb.bytes() == sizeof(Params));
    CHECK(pb.map(gbBuffer::MAP_READ));
    CHECK(std::memcmp(pb.ptr<Params>(), &fluid.getParameters(), sizeof(Params)) == 0);
    pb.unmap();
    fluid.getParameters().viscosity = 2.5f;
    CHECK(fluid.compute(dev));
    cudaDeviceSynchronize();
    CHECK(pb.map(gbBuffer::MAP_READ));  // the same device memory, not looked up again
    CHECK(pb.ptr<Params>()->viscosity == 2.5f);
    CHECK(std::memcmp(pb.ptr<Params>(), &fluid.getParameters(), sizeof(Params)) == 0);
    pb.unmap();
    std::printf("testParamBuffer completed\n");
    return 0;
}

// oclFluid2D: compile, a dam-break block of particles in the default container, a border
// image with a wall column, 20 steps; positions stay finite and inside the container.
static int testFluid2D(gbContext& ctx) {
    gbDevice& dev = ctx.getDevice(0);
    gbFluid2D fluid(ctx);
    CHECK(fluid.compile());
    fluid.setParticleCount(4096);
    gbFluid2D::Params& p = fluid.getParameters();
    gbBuffer* st = fluid.getStateBuffer();
    CHECK(st->count<gbFluid2D::Particle>() == 4096);
    CHECK(st->map(gbBuffer::MAP_WRITE));
    for (int i = 0; i < 4096; i++) {
        gbFluid2D::Particle& q = st->ptr<gbFluid2D::Particle>()[i];
        q.pos[0] = 1.0f + (i % 64) * 0.5f * p.h;  // a 64 x 64 block in the lower left of the container
        q.pos[1] = 1.0f + (i / 64) * 0.5f * p.h;
        q.vel[0] = q.vel[1] = 0.0f;
        q.mass = p.particleMass;
        q.unused = 0.0f;
    }
    CHECK(st->unmap());
    gbImage2D wall(ctx, "imBorder");
    CHECK(wall.create(256, 256));
    std::vector<float> img(256 * 256 * 4, 0.0f);
    for (int y = 0; y < 256; y++) img[4 * (y * 256 + 200) + 3] = 1.0f;  // a wall column at x = 200
    CHECK(wall.write(img.data()));
    fluid.computeBorder(&wall);
    CHECK(gbStatus() == GBSPH_OK);
    for (int i = 0; i < 20; i++) CHECK(fluid.compute(dev));
    cudaDeviceSynchronize();
    CHECK(st->map(gbBuffer::MAP_READ));
    for (int i = 0; i < 4096; i++) {
        const gbFluid2D::Particle& q = st->ptr<gbFluid2D::Particle>()[i];
        CHECK(std::isfinite(q.pos[0]) && std::isfinite(q.pos[1]));
    }
    std::printf("testFluid2D completed\n");
    return 0;
}

// oclBvhTrimesh and oclBvhLines: build over a few primitives; 2n - 1 nodes, a root among the
// internal nodes whose box contains every primitive.
static int testBvh(gbContext& ctx) {
    gbDevice& dev = ctx.getDevice(0);
    const int n = 64;
    gbBuffer vtx(ctx, "bfVertex"), idx(ctx, "bfIndex");
    CHECK(vtx.create<float>(4 * 3 * n) && idx.create<unsigned>(3 * n));
    vtx.map(gbBuffer::MAP_WRITE);
    idx.map(gbBuffer::MAP_WRITE);
    unsigned s = 3;
    for (int t = 0; t < n; t++) {
        const float cx = (float)(lcg(s) >> 8) / (1 << 24), cy = (float)(lcg(s) >> 8) / (1 << 24),
                    cz = (float)(lcg(s) >> 8) / (1 << 24);
        for (int k = 0; k < 3; k++) {
            float* v = vtx.ptr<float>() + 4 * (3 * t + k);
            v[0] = cx + 0.01f * k;
            v[1] = cy + 0.01f * (k == 1);
            v[2] = cz;
            v[3] = 1.0f;
            idx.ptr<unsigned>()[3 * t + k] = 3 * t + k;
        }
    }
    CHECK(vtx.unmap() && idx.unmap());
    gbBvhTrimesh tri(ctx);
    CHECK(tri.compute(dev, vtx, idx));
    CHECK(tri.getNodeCount() == 2 * n - 1);
    const uint32_t root = tri.getRootNode();
    CHECK(root < (uint32_t)(n - 1));
    gbBuffer& nodes = tri.getNodeBuffer();
    CHECK(nodes.count<gbBvhTrimesh::BVHNode>() == (size_t)(2 * n - 1));
    CHECK(nodes.map(gbBuffer::MAP_READ));
    const gbBvhTrimesh::BVHNode& r = nodes.ptr<gbBvhTrimesh::BVHNode>()[root];
    CHECK(r.trav == 2);
    vtx.map(gbBuffer::MAP_READ);
    for (int i = 0; i < 3 * n; i++)
        for (int c = 0; c < 3; c++) {
            const float v = vtx.ptr<float>()[4 * i + c];
            CHECK(v >= r.bbMin[c] && v <= r.bbMax[c]);
        }

    gbBuffer seg(ctx, "bfSegment");
    CHECK(seg.create<float>(2 * 2 * n));
    seg.map(gbBuffer::MAP_WRITE);
    for (int i = 0; i < n; i++) {
        float* v = seg.ptr<float>() + 4 * i;
        v[0] = (float)(lcg(s) >> 16);
        v[1] = (float)(lcg(s) >> 16);
        v[2] = v[0] + 3.0f;
        v[3] = v[1] + 5.0f;
    }
    CHECK(seg.unmap());
    gbBvhLines lines(ctx);
    CHECK(lines.compute(dev, seg));
    CHECK(lines.getNodeCount() == 2 * n - 1);
    const uint32_t lroot = lines.getRootNode();
    CHECK(lroot < (uint32_t)(n - 1));
    gbBuffer& lnodes = lines.getNodeBuffer();
    CHECK(lnodes.map(gbBuffer::MAP_READ));
    seg.map(gbBuffer::MAP_READ);
    const gbBvhLines::BVHNode& lr = lnodes.ptr<gbBvhLines::BVHNode>()[lroot];
    CHECK(lr.trav == 3);
    for (int i = 0; i < 2 * n; i++) {
        const float* v = seg.ptr<float>() + 2 * i;
        CHECK(v[0] >= lr.bbMin[0] && v[0] <= lr.bbMax[0] && v[1] >= lr.bbMin[1] && v[1] <= lr.bbMax[1]);
    }
    std::printf("testBvh completed\n");
    return 0;
}

int main() {
    gbContext ctx(0);
    if (testRadixSort(ctx) || testFluid3D0(ctx) || testFluid3D1(ctx) || testParamBuffer(ctx) || testFluid2D(ctx) || testBvh(ctx)) return 1;
    std::printf("OK\n");
    return 0;
}
