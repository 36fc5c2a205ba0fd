// gbFluid3D.hpp -- header-only C++ class surface over the C ABI in gbsph.h.
//
// Mirrors the classes a libCL user calls for the SPH path (jochenstier/libcl):
//   oclContext / oclDevice   (libCL/oclContext.h:25-49, libCL/oclDevice.h:22-45) -> gbContext / gbDevice
//   oclBuffer                (libCL/oclBuffer.h:22-70, libCL/oclMem.h:22-60)      -> gbBuffer
//   oclRadixSort             (libCL/sort/oclRadixSort.h:22-49)                     -> gbRadixSort
//   oclFluid3D + srtEvent    (libCL/phys/oclFluid3D.h:21-123, libCL/oclProgram.h:104-116)
//                                                                                  -> gbFluid3D + srtEvent
//   oclImage2D               (libCL/oclImage2D.h, an RGBA float image)           -> gbImage2D
//   oclFluid2D               (libCL/phys/oclFluid2D.h:22-79)                      -> gbFluid2D
//   oclBvhTrimesh            (libCL/geom/oclBvhTrimesh.h:20-84)                   -> gbBvhTrimesh
//   oclBvhLines              (libCL/geom/oclBvhLines.h:20-77)                     -> gbBvhLines
// Same method names and meanings: construct, compile(), setParticleCount(), set/get buffers,
// getParameters(), addEventHandler(EVT_INTEGRATE), compute(device), map()/unmap() to read
// results. Methods return 1/true on success and 0/false on failure like the reference; the
// last status code is kept in gbStatus (the reference's sStatusCL, libCL/oclCommon.cpp:19).
#pragma once

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "gbsph.h"

inline int& gbStatus() {
    static thread_local int s = GBSPH_OK;
    return s;
}

class gbDevice {
   public:
    explicit gbDevice(int ordinal = 0, cudaStream_t stream = nullptr) : mOrdinal(ordinal), mStream(stream) {}
    cudaStream_t getQueue() const { return mStream; }
    operator cudaStream_t() const { return mStream; }
    int ordinal() const { return mOrdinal; }
    void setQueue(cudaStream_t s) { mStream = s; }

   private:
    int mOrdinal;
    cudaStream_t mStream;
};

class gbContext {
   public:
    explicit gbContext(int device = 0) : mDevice(device) { cudaSetDevice(device); }
    gbDevice& getDevice(int) { return mDevice; }

   private:
    gbDevice mDevice;
};

// Device buffer with an owner tag; map()/unmap() stage a host copy (the reference maps
// ALLOC_HOST_PTR buffers, libCL/oclBuffer.cpp:26-45, libCL/oclMem.cpp:64-84).
class gbBuffer {
   public:
    enum { MAP_READ = 1, MAP_WRITE = 2 };
    gbBuffer(gbContext&, const char* name) : mName(name) {}
    ~gbBuffer() { release(); }
    gbBuffer(const gbBuffer&) = delete;
    gbBuffer& operator=(const gbBuffer&) = delete;

    template <class T>
    bool create(size_t count) {
        release();
        gbStatus() = cudaMalloc(&mPtr, count * sizeof(T)) == cudaSuccess ? GBSPH_OK : GBSPH_ERR_OUT_OF_MEMORY;
        if (gbStatus() != GBSPH_OK) return false;
        cudaMemset(mPtr, 0, count * sizeof(T));
        mBytes = count * sizeof(T);
        mOwned = true;
        return true;
    }
    // Wraps memory owned elsewhere (a fluid's internal buffer); never freed by this object.
    void wrap(void* device_ptr, size_t bytes) {
        release();
        mPtr = device_ptr;
        mBytes = bytes;
        mOwned = false;
    }
    template <class T>
    size_t count() const { return mBytes / sizeof(T); }
    size_t bytes() const { return mBytes; }
    void* devicePtr() const { return mPtr; }
    const std::string& getName() const { return mName; }
    template <class T>
    T* ptr() { return reinterpret_cast<T*>(mHost.data()); }
    bool map(int flags) {
        mHost.resize(mBytes);
        mMapFlags = flags;
        if (flags & MAP_READ) return cudaMemcpy(mHost.data(), mPtr, mBytes, cudaMemcpyDeviceToHost) == cudaSuccess;
        return true;
    }
    bool unmap() {
        bool ok = true;
        if (mMapFlags & MAP_WRITE) ok = cudaMemcpy(mPtr, mHost.data(), mBytes, cudaMemcpyHostToDevice) == cudaSuccess;
        mMapFlags = 0;
        return ok;
    }
    void setOwner(const void* owner) { mOwner = owner; }
    const void* getOwner() const { return mOwner; }

   private:
    void release() {
        if (mOwned && mPtr) cudaFree(mPtr);
        mPtr = nullptr;
        mBytes = 0;
        mOwned = false;
    }
    std::string mName;
    void* mPtr = nullptr;
    size_t mBytes = 0;
    bool mOwned = false;
    int mMapFlags = 0;
    const void* mOwner = nullptr;
    std::vector<unsigned char> mHost;
};

class gbRadixSort {
   public:
    explicit gbRadixSort(gbContext&) { gbStatus() = gbsph_radix_sort_create(&mH); }
    ~gbRadixSort() {
        if (mH) gbsph_radix_sort_destroy(mH);
    }
    int compile() { return mH != nullptr; }
    // oclRadixSort::compute(oclDevice&, oclBuffer& key, oclBuffer& val, int startBit, int endBit)
    int compute(gbDevice& dev, gbBuffer& key, gbBuffer& val, int startBit, int endBit) {
        gbStatus() = gbsph_radix_sort_compute(mH, (uint32_t*)key.devicePtr(), (uint32_t*)val.devicePtr(),
                                              key.count<uint32_t>(), val.count<uint32_t>(), startBit, endBit,
                                              dev.getQueue());
        return gbStatus() == GBSPH_OK;
    }
    const char* lastError() const { return gbsph_radix_sort_last_error(mH); }

   private:
    gbsph_radix_sort_t mH = nullptr;
};

class gbFluid3D;

// Event handler (srtEvent, libCL/oclProgram.h:104-116): called by compute() in place of the
// clip/integrate stages when registered for EVT_INTEGRATE.
struct srtEvent {
    explicit srtEvent(const char* name, void* data = nullptr) : mName(name), mData(data) {}
    virtual ~srtEvent() = default;
    virtual bool operator()(gbFluid3D& fluid) = 0;
    const char* mName;
    void* mData;
};

class gbFluid3D {
   public:
    typedef gbsph_fluid3d_params Params;
    static constexpr const char* EVT_INTEGRATE = "OnIntegrate";
    static constexpr size_t cLocalSize = 256;
    static constexpr size_t cBucketCount = 262144;

    explicit gbFluid3D(gbContext& ctx)
        : mPosition(ctx, "bfPosition"), mVelocity(ctx, "bfVelocity"), mForce(ctx, "bfForce"),
          mSortedPosition(ctx, "bfSortedPosition"), mSortedVelocity(ctx, "bfSortedVelocity"),
          mIndex(ctx, "bfIndex"), mParams(ctx, "bfParams") {
        gbStatus() = gbsph_fluid3d_create(&mH);
        rewrap();
    }
    ~gbFluid3D() {
        if (mH) gbsph_fluid3d_destroy(mH);
    }
    gbFluid3D(const gbFluid3D&) = delete;
    gbFluid3D& operator=(const gbFluid3D&) = delete;

    int compile() { return ok(gbsph_fluid3d_compile(mH)); }
    int compute(gbDevice& dev) {
        mDevice = &dev;
        return ok(gbsph_fluid3d_compute(mH, dev.getQueue()));
    }
    // One step on host-resident float4 state (page-locked memory for the overlapped path):
    // the inputs are uploaded, the step runs, the outputs (may be the inputs) are downloaded;
    // asynchronous on dev's queue.
    int computeHost(gbDevice& dev, const float* pos, const float* vel, const float* force, float* posOut,
                    float* velOut, float* forceOut) {
        mDevice = &dev;
        return ok(gbsph_fluid3d_compute_host(mH, pos, vel, force, posOut, velOut, forceOut, dev.getQueue()));
    }
    // One reference stage (GBSPH_STAGE_*), e.g. from an EVT_INTEGRATE handler.
    int stage(int which) { return ok(gbsph_fluid3d_stage(mH, which, mDevice ? mDevice->getQueue() : nullptr)); }

    void setParticleCount(size_t n) {
        ok(gbsph_fluid3d_set_particle_count(mH, n));
        rewrap();
    }
    size_t getParticleCount() { return gbsph_fluid3d_get_particle_count(mH); }

    int setPositionBuffer(gbBuffer* b) { return setBuffer(GBSPH_BUF_POSITION, b); }
    int setVelocityBuffer(gbBuffer* b) { return setBuffer(GBSPH_BUF_VELOCITY, b); }
    int setForceBuffer(gbBuffer* b) { return setBuffer(GBSPH_BUF_FORCE, b); }

    gbBuffer* getPositionBuffer() { return mUser[0] ? mUser[0] : &mPosition; }
    gbBuffer* getVelocityBuffer() { return mUser[1] ? mUser[1] : &mVelocity; }
    gbBuffer* getForceBuffer() { return mUser[2] ? mUser[2] : &mForce; }
    gbBuffer& getSortedPositionBuffer() { return mSortedPosition; }
    gbBuffer& getSortedVelocityBuffer() { return mSortedVelocity; }
    gbBuffer& getIndexBuffer() { return mIndex; }
    // getParamBuffer (libCL/phys/oclFluid3D.cpp:198-201): the device copy of getParameters()
    // (one Params record; its first 13 fields are the kernels' System block), brought up to
    // date by this call and by every compute() whose parameters changed.
    gbBuffer& getParamBuffer() {
        size_t count = 0;
        void* p = mH ? gbsph_fluid3d_get_buffer(mH, GBSPH_BUF_PARAMS, &count) : nullptr;
        mParams.wrap(p, count * sizeof(Params));
        mParams.setOwner(this);
        return mParams;
    }

    Params& getParameters() { return *gbsph_fluid3d_get_params(mH); }

    void addEventHandler(srtEvent& e) {
        if (std::strcmp(e.mName, EVT_INTEGRATE) != 0) return;
        mHandler = &e;
        gbsph_fluid3d_set_integrate_hook(mH, &gbFluid3D::hookTrampoline, this);
    }
    const char* lastError() const { return gbsph_fluid3d_last_error(mH); }
    gbsph_fluid3d_t handle() const { return mH; }

   private:
    static int hookTrampoline(gbsph_fluid3d_t, void* stream, void* user) {
        gbFluid3D* self = static_cast<gbFluid3D*>(user);
        if (self->mDevice) self->mDevice->setQueue((cudaStream_t)stream);
        return (*self->mHandler)(*self) ? 0 : 1;
    }
    int ok(int status) {
        gbStatus() = status;
        return status == GBSPH_OK;
    }
    int setBuffer(int which, gbBuffer* b) {
        const int r = ok(gbsph_fluid3d_set_buffer(mH, which, b->devicePtr(), b->count<float>() / 4));
        if (r) mUser[which] = b;
        return r;
    }
    void rewrap() {
        gbBuffer* own[6] = {&mPosition, &mVelocity, &mForce, &mSortedPosition, &mSortedVelocity, &mIndex};
        const int which[6] = {GBSPH_BUF_POSITION, GBSPH_BUF_VELOCITY, GBSPH_BUF_FORCE,
                              GBSPH_BUF_SORTED_POSITION, GBSPH_BUF_SORTED_VELOCITY, GBSPH_BUF_INDEX};
        for (int i = 0; i < 6; i++) {
            size_t count = 0;
            void* p = mH ? gbsph_fluid3d_get_buffer(mH, which[i], &count) : nullptr;
            own[i]->wrap(p, count * (which[i] == GBSPH_BUF_INDEX ? 4 : 16));
            own[i]->setOwner(this);
        }
    }

    gbsph_fluid3d_t mH = nullptr;
    gbBuffer mPosition, mVelocity, mForce, mSortedPosition, mSortedVelocity, mIndex, mParams;
    gbBuffer* mUser[3] = {nullptr, nullptr, nullptr};
    srtEvent* mHandler = nullptr;
    gbDevice* mDevice = nullptr;
};

// A device RGBA float image (the wall mask oclFluid2D::computeBorder reads).
class gbImage2D {
   public:
    gbImage2D(gbContext&, const char* name) : mName(name) {}
    ~gbImage2D() {
        if (mPtr) cudaFree(mPtr);
    }
    gbImage2D(const gbImage2D&) = delete;
    gbImage2D& operator=(const gbImage2D&) = delete;
    bool create(int width, int height) {
        if (mPtr) cudaFree(mPtr);
        mPtr = nullptr;
        gbStatus() = cudaMalloc(&mPtr, (size_t)width * height * 16) == cudaSuccess ? GBSPH_OK : GBSPH_ERR_OUT_OF_MEMORY;
        if (gbStatus() != GBSPH_OK) return false;
        cudaMemset(mPtr, 0, (size_t)width * height * 16);
        mW = width;
        mH = height;
        return true;
    }
    // Uploads width * height RGBA float pixels.
    bool write(const float* rgba) {
        return cudaMemcpy(mPtr, rgba, (size_t)mW * mH * 16, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    int getImageWidth() const { return mW; }
    int getImageHeight() const { return mH; }
    const float* devicePtr() const { return mPtr; }

   private:
    std::string mName;
    float* mPtr = nullptr;
    int mW = 0, mH = 0;
};

// oclFluid2D: the 2D relaxation model. Same calls: compile(), setParticleCount(),
// setStateBuffer() / getStateBuffer() (Particle records, 24 bytes), computeBorder(image),
// getParameters(), compute(device).
class gbFluid2D {
   public:
    typedef gbsph_fluid2d_params Params;
    typedef gbsph_particle2d Particle;
    static constexpr size_t cLocalSize = 256;

    explicit gbFluid2D(gbContext& ctx) : mState(ctx, "bfParticle") {
        gbStatus() = gbsph_fluid2d_create(&mH);
        rewrap();
    }
    ~gbFluid2D() {
        if (mH) gbsph_fluid2d_destroy(mH);
    }
    gbFluid2D(const gbFluid2D&) = delete;
    gbFluid2D& operator=(const gbFluid2D&) = delete;

    int compile() { return ok(gbsph_fluid2d_compile(mH)); }
    int compute(gbDevice& dev) { return ok(gbsph_fluid2d_compute(mH, dev.getQueue())); }
    void setParticleCount(size_t n) {
        ok(gbsph_fluid2d_set_particle_count(mH, n));
        mUser = nullptr;
        rewrap();
    }
    size_t getParticleCount() { return gbsph_fluid2d_get_particle_count(mH); }
    int setStateBuffer(gbBuffer* b) {
        const int r = ok(gbsph_fluid2d_set_state_buffer(mH, b->devicePtr(), b->count<Particle>()));
        if (r) mUser = b;
        return r;
    }
    gbBuffer* getStateBuffer() { return mUser ? mUser : &mState; }
    void computeBorder(gbImage2D* image) {
        ok(gbsph_fluid2d_compute_border(mH, image->devicePtr(), image->getImageWidth(), image->getImageHeight(),
                                        nullptr));
    }
    Params& getParameters() { return *gbsph_fluid2d_get_params(mH); }
    const char* lastError() const { return gbsph_fluid2d_last_error(mH); }
    gbsph_fluid2d_t handle() const { return mH; }

   private:
    int ok(int status) {
        gbStatus() = status;
        return status == GBSPH_OK;
    }
    void rewrap() {
        size_t count = 0;
        void* p = mH ? gbsph_fluid2d_get_buffer(mH, GBSPH2D_BUF_STATE, &count) : nullptr;
        mState.wrap(p, count * sizeof(Particle));
        mState.setOwner(this);
    }
    gbsph_fluid2d_t mH = nullptr;
    gbBuffer mState;
    gbBuffer* mUser = nullptr;
};

// oclBvhTrimesh: compute(device, vertex float4 buffer, index uint buffer), then the node
// buffer (BVHNode records, 48 bytes), node count and root.
class gbBvhTrimesh {
   public:
    typedef gbsph_bvh_node BVHNode;
    explicit gbBvhTrimesh(gbContext& ctx) : mNodes(ctx, "bfBvhNode") { gbStatus() = gbsph_bvh_create(&mH); }
    ~gbBvhTrimesh() {
        if (mH) gbsph_bvh_destroy(mH);
    }
    gbBvhTrimesh(const gbBvhTrimesh&) = delete;
    gbBvhTrimesh& operator=(const gbBvhTrimesh&) = delete;
    int compute(gbDevice& dev, gbBuffer& vertex, gbBuffer& index) {
        mDevice = &dev;
        gbStatus() = gbsph_bvh_compute(mH, (const float*)vertex.devicePtr(), vertex.count<float>() / 4,
                                       (const uint32_t*)index.devicePtr(), index.count<uint32_t>(), dev.getQueue());
        size_t count = 0;
        void* p = gbsph_bvh_get_node_buffer(mH, &count);
        mNodes.wrap(p, count * sizeof(BVHNode));
        mNodes.setOwner(this);
        return gbStatus() == GBSPH_OK;
    }
    gbBuffer& getNodeBuffer() { return mNodes; }
    uint32_t getNodeCount() { return (uint32_t)gbsph_bvh_get_node_count(mH); }
    uint32_t getRootNode() {
        uint32_t r = 0;
        gbStatus() = gbsph_bvh_get_root_node(mH, &r, mDevice ? mDevice->getQueue() : nullptr);
        return r;
    }
    const char* lastError() const { return gbsph_bvh_last_error(mH); }
    gbsph_bvh_t handle() const { return mH; }

   private:
    gbsph_bvh_t mH = nullptr;
    gbBuffer mNodes;
    gbDevice* mDevice = nullptr;
};

// oclBvhLines: compute(device, vertex float2 buffer, two vertices per segment), then the node
// buffer (BVHNode records, 32 bytes), node count and root.
class gbBvhLines {
   public:
    typedef gbsph_bvh2d_node BVHNode;
    explicit gbBvhLines(gbContext& ctx) : mNodes(ctx, "bfBvhNode") { gbStatus() = gbsph_bvh_lines_create(&mH); }
    ~gbBvhLines() {
        if (mH) gbsph_bvh_lines_destroy(mH);
    }
    gbBvhLines(const gbBvhLines&) = delete;
    gbBvhLines& operator=(const gbBvhLines&) = delete;
    int compute(gbDevice& dev, gbBuffer& vertex) {
        mDevice = &dev;
        gbStatus() = gbsph_bvh_lines_compute(mH, (const float*)vertex.devicePtr(), vertex.count<float>() / 2,
                                             dev.getQueue());
        size_t count = 0;
        void* p = gbsph_bvh_lines_get_node_buffer(mH, &count);
        mNodes.wrap(p, count * sizeof(BVHNode));
        mNodes.setOwner(this);
        return gbStatus() == GBSPH_OK;
    }
    gbBuffer& getNodeBuffer() { return mNodes; }
    uint32_t getNodeCount() { return (uint32_t)gbsph_bvh_lines_get_node_count(mH); }
    uint32_t getRootNode() {
        uint32_t r = 0;
        gbStatus() = gbsph_bvh_lines_get_root_node(mH, &r, mDevice ? mDevice->getQueue() : nullptr);
        return r;
    }
    const char* lastError() const { return gbsph_bvh_lines_last_error(mH); }

   private:
    gbsph_bvh_lines_t mH = nullptr;
    gbBuffer mNodes;
    gbDevice* mDevice = nullptr;
};

