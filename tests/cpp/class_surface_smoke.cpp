// C++ drop-in smoke test of the class surface, following the reference's driver
// (libCL/TEST/main.cpp): testRadixSort (:133-181), testFluid3D0 (:188-240) and
// testFluid3D1 with an EVT_INTEGRATE handler (:246-343), with fixed step counts instead of
// 7 seconds of wall clock, and with assertions the reference does not make.
#include <cmath>
#include <cstdio>
#include <cstdlib>

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

int main() {
    gbContext ctx(0);
    if (testRadixSort(ctx) || testFluid3D0(ctx) || testFluid3D1(ctx)) return 1;
    std::printf("OK\n");
    return 0;
}
