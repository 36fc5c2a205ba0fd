// clshim.h -- a small OpenCL C 1.1 environment for C++20, so that the reference's own
// kernel sources (libCL/phys/oclFluid3D.cl, libCL/phys/oclFluid2D.cl,
// libCL/sort/oclRadixSort.cl, libCL/geom/oclBvhTrimesh.cl, libCL/geom/oclBvhLines.cl) compile
// and run on the host cores.
//
// TEST INFRASTRUCTURE ONLY: it exists to execute the reference's kernels as the checker of
// the oracle restatement (and, through it, of the CUDA library). Nothing in the product
// library includes or links it.
//
// What it provides (all in namespace clc; the kernel text is compiled inside a namespace
// nested in clc, so unqualified names resolve here before the C library's):
//   * the vector types float2/float4/int2/int4/uint2/uint4 with OpenCL's layout (size and
//     alignment 8 or 16 bytes), .x/.y/.z/.w lanes, the .xy/.zw swizzles (also as lvalues),
//     component-wise arithmetic between vectors and with scalars (the scalar is converted
//     to the element type first, OpenCL C 1.1 section 6.3), and scalar broadcast on
//     initialisation and assignment;
//   * work-item functions (get_global_id, get_local_id, get_group_id, get_global_size,
//     get_local_size, get_num_groups) backed by a per-thread work-item record;
//   * the math, common and geometric built-ins the kernels call, with the conventions that
//     OpenCL leaves to the implementation fixed as follows:
//       fast_length(v)  = sqrtf(x*x + y*y + z*z + w*w), summed left to right;
//       length(v)       = sqrtf of the same sum (float2: x*x + y*y);
//       dot(a, b)       = a.x*b.x + a.y*b.y (+ a.z*b.z + a.w*b.w), left to right;
//       normalize(v)    = v / length(v) (each lane divided by the correctly rounded length);
//       cross(a, b)     = (a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x, 0);
//       pow(x, y)       = the C library's powf, except that in POW_INTEGER_CUBE mode
//                         pow(x, 3.0f) = x*x*x (what compilers that expand a literal small
//                         integral exponent produce); see clc::set_pow_mode;
//       `/` and sqrt    = IEEE correctly rounded (the unit is built with -ffp-contract=off);
//       min/max         = OpenCL's definitions (max(x, y) = x < y ? y : x; min(x, y) =
//                         y < x ? y : x), component-wise for vectors;
//   * 2D images: RGBA half-float or float texels, read_imagef with the nearest filter on
//     integer coordinates and the bilinear filter on normalised coordinates exactly as the
//     OpenCL C 1.1 specification's filtering section writes it (u = s*W - 0.5,
//     i0 = floor(u), a = u - floor(u), CLK_ADDRESS_CLAMP_TO_EDGE clamps the texel indices,
//     T = (1-a)(1-b)T00 + a(1-b)T10 + (1-a)bT01 + abT11 summed left to right), and
//     write_imagef rounding to half precision to nearest even;
//   * atom_cmpxchg on int and uint words (a sequentially consistent compare-and-swap);
//   * barrier(): kernels that call it are compiled as C++20 coroutines (the source rewrite
//     turns barrier(...) into `co_await clc::barrier_point{}` and `return;` into
//     `co_return;`); run_groups_coro() runs a work-group's work-items in local-id order up
//     to each barrier in turn, which is what the barrier requires of a work-group. __local
//     arrays declared in a kernel body live in per-host-thread storage (local_array), shared
//     by the work-group the thread is running.
// Work-groups of one launch run on OpenMP threads where the reference's kernels write disjoint
// locations per work-item, so that the results do not depend on the schedule; the runners'
// PAR = false runs a launch's work-groups one after another on the calling thread (for the
// kernels whose work-items meet through atomics).
#pragma once

#include <cmath>
#include <coroutine>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <atomic>
#include <exception>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

// OpenCL address-space and access qualifiers: no meaning on the host. (`__local` is
// handled by the source rewrite because its meaning depends on where it appears.)
#define __kernel
#define __global
#define __private
#define __read_only
#define __write_only
#define CLK_LOCAL_MEM_FENCE 1u
#define CLK_GLOBAL_MEM_FENCE 2u
// OpenCL C's predefined float constants (the float nearest to pi; the largest finite float).
#define M_PI_F 3.14159274101257f
#define MAXFLOAT 3.40282346638528859811704183484516925e+38F

namespace clc {

typedef unsigned int uint;
typedef unsigned char uchar;
typedef unsigned short ushort;

// ------------------------------------------------------------------------------------
// Vector types
// ------------------------------------------------------------------------------------
template <class T>
struct vec2;
template <class T>
struct vec4;

// Two lanes (A, B) of an N-lane vector, usable as an rvalue vec2 and as an lvalue.
template <class T, int N, int A, int B>
struct swz2 {
    T v[N];
    operator vec2<T>() const;
    swz2& operator=(const vec2<T>& r);
};

template <class T>
struct alignas(2 * sizeof(T)) vec2 {
    union {
        struct {
            T x, y;
        };
        T v[2];
        swz2<T, 2, 0, 1> xy;
    };
    vec2() = default;
    vec2(T s) {
        x = s;
        y = s;
    }
    template <class S, class = std::enable_if_t<std::is_arithmetic_v<S> && !std::is_same_v<S, T>>>
    vec2(S s) : vec2((T)s) {}
    vec2(T a, T b) {
        x = a;
        y = b;
    }
    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
};

template <class T>
struct alignas(4 * sizeof(T)) vec4 {
    union {
        struct {
            T x, y, z, w;
        };
        T v[4];
        swz2<T, 4, 0, 1> xy;
        swz2<T, 4, 2, 3> zw;
    };
    vec4() = default;
    vec4(T s) {
        x = s;
        y = s;
        z = s;
        w = s;
    }
    template <class S, class = std::enable_if_t<std::is_arithmetic_v<S> && !std::is_same_v<S, T>>>
    vec4(S s) : vec4((T)s) {}
    vec4(T a, T b, T c, T d) {
        x = a;
        y = b;
        z = c;
        w = d;
    }
    T& operator[](int i) { return v[i]; }
    const T& operator[](int i) const { return v[i]; }
};

template <class T, int N, int A, int B>
swz2<T, N, A, B>::operator vec2<T>() const {
    return vec2<T>(v[A], v[B]);
}
template <class T, int N, int A, int B>
swz2<T, N, A, B>& swz2<T, N, A, B>::operator=(const vec2<T>& r) {
    v[A] = r.x;
    v[B] = r.y;
    return *this;
}

typedef vec2<float> float2;
typedef vec4<float> float4;
typedef vec2<int> int2;
typedef vec4<int> int4;
typedef vec2<uint> uint2;
typedef vec4<uint> uint4;
static_assert(sizeof(float2) == 8 && alignof(float2) == 8, "float2 layout");
static_assert(sizeof(float4) == 16 && alignof(float4) == 16, "float4 layout");
static_assert(sizeof(uint4) == 16, "uint4 layout");

// Trait machinery: what counts as a vector operand, its element type and its value.
template <class X>
struct vtraits {
    static constexpr bool is_vec = false;
};
template <class T>
struct vtraits<vec2<T>> {
    static constexpr bool is_vec = true;
    typedef T elem;
    typedef vec2<T> type;
};
template <class T>
struct vtraits<vec4<T>> {
    static constexpr bool is_vec = true;
    typedef T elem;
    typedef vec4<T> type;
};
template <class T, int N, int A, int B>
struct vtraits<swz2<T, N, A, B>> {
    static constexpr bool is_vec = true;
    typedef T elem;
    typedef vec2<T> type;
};
template <class X>
using vdecay = std::remove_cv_t<std::remove_reference_t<X>>;
template <class X>
constexpr bool is_vec_v = vtraits<vdecay<X>>::is_vec;

template <class X>
inline auto vval(const X& x) {
    if constexpr (is_vec_v<X>)
        return typename vtraits<vdecay<X>>::type(x);
    else
        return x;
}

template <class T, class F>
inline vec2<T> vmap(const vec2<T>& a, const vec2<T>& b, F f) {
    return vec2<T>(f(a.x, b.x), f(a.y, b.y));
}
template <class T, class F>
inline vec4<T> vmap(const vec4<T>& a, const vec4<T>& b, F f) {
    return vec4<T>(f(a.x, b.x), f(a.y, b.y), f(a.z, b.z), f(a.w, b.w));
}

// Binary operator on (vector, vector), (vector, scalar) or (scalar, vector). The scalar is
// converted to the vector's element type before the operation.
template <class A, class B, class F>
inline auto vbin(const A& a0, const B& b0, F f) {
    if constexpr (is_vec_v<A> && is_vec_v<B>) {
        return vmap(vval(a0), vval(b0), f);
    } else if constexpr (is_vec_v<A>) {
        typedef typename vtraits<vdecay<A>>::type V;
        typedef typename vtraits<vdecay<A>>::elem T;
        return vmap(vval(a0), V((T)b0), f);
    } else {
        typedef typename vtraits<vdecay<B>>::type V;
        typedef typename vtraits<vdecay<B>>::elem T;
        return vmap(V((T)a0), vval(b0), f);
    }
}

#define CLC_VEC_OP(op)                                                                          \
    template <class A, class B, class = std::enable_if_t<is_vec_v<A> || is_vec_v<B>>>          \
    inline auto operator op(const A& a, const B& b) {                                           \
        return vbin(a, b, [](auto x, auto y) { return x op y; });                               \
    }
CLC_VEC_OP(+)
CLC_VEC_OP(-)
CLC_VEC_OP(*)
CLC_VEC_OP(/)
#undef CLC_VEC_OP

#define CLC_VEC_CAOP(op, bop)                                                                   \
    template <class V, class B, class = std::enable_if_t<is_vec_v<V>>>                          \
    inline V& operator op(V& a, const B& b) {                                                   \
        a = vbin(a, b, [](auto x, auto y) { return x bop y; });                                 \
        return a;                                                                               \
    }
CLC_VEC_CAOP(+=, +)
CLC_VEC_CAOP(-=, -)
CLC_VEC_CAOP(*=, *)
CLC_VEC_CAOP(/=, /)
#undef CLC_VEC_CAOP

template <class T>
inline vec2<T> operator-(const vec2<T>& a) {
    return vec2<T>(-a.x, -a.y);
}
template <class T>
inline vec4<T> operator-(const vec4<T>& a) {
    return vec4<T>(-a.x, -a.y, -a.z, -a.w);
}

// Vector literal (T)(a, b, ...): scalars and vectors concatenated lane by lane, or a single
// scalar broadcast (the source rewrite turns `(float4)(` into `clc::make<clc::float4>(`).
template <class V>
struct lanes;
template <class T>
struct lanes<vec2<T>> {
    static constexpr int n = 2;
};
template <class T>
struct lanes<vec4<T>> {
    static constexpr int n = 4;
};
template <class V, class E>
inline void put_lanes(V& out, int& k, const E& e) {
    typedef typename vtraits<V>::elem T;
    if constexpr (is_vec_v<E>) {
        auto ev = vval(e);
        for (int i = 0; i < lanes<decltype(ev)>::n; i++) out[k++] = (T)ev[i];
    } else {
        out[k++] = (T)e;
    }
}
template <class V, class... E>
inline V make(const E&... e) {
    if constexpr (sizeof...(E) == 1 && (!is_vec_v<E> && ...)) {
        typedef typename vtraits<V>::elem T;
        return V((T)(e, ...));
    } else {
        V out;
        int k = 0;
        (put_lanes(out, k, e), ...);
        return out;
    }
}

// ------------------------------------------------------------------------------------
// Work-items
// ------------------------------------------------------------------------------------
struct work_item {
    size_t gid[3], lid[3], grp[3], gsize[3], lsize[3], ngroups[3];
    uint dims;
};
inline thread_local work_item wi;

inline size_t get_global_id(uint d) { return d < wi.dims ? wi.gid[d] : 0; }
inline size_t get_local_id(uint d) { return d < wi.dims ? wi.lid[d] : 0; }
inline size_t get_group_id(uint d) { return d < wi.dims ? wi.grp[d] : 0; }
inline size_t get_global_size(uint d) { return d < wi.dims ? wi.gsize[d] : 1; }
inline size_t get_local_size(uint d) { return d < wi.dims ? wi.lsize[d] : 1; }
inline size_t get_num_groups(uint d) { return d < wi.dims ? wi.ngroups[d] : 1; }
inline uint get_work_dim() { return wi.dims; }

// The calling thread's work-item record set to the first item of 1D work-group `group`
// (one thread-local lookup; the caller then steps lid/gid through the group).
inline work_item& enter_group_1d(size_t global, size_t local, size_t group) {
    work_item& w = wi;
    w.dims = 1;
    w.gsize[0] = global;
    w.lsize[0] = local;
    w.ngroups[0] = global / local;
    w.grp[0] = group;
    w.lid[0] = 0;
    w.gid[0] = group * local;
    return w;
}
inline void set_local_id(work_item& w, size_t l) {
    w.lid[0] = l;
    w.gid[0] = w.grp[0] * w.lsize[0] + l;
}

// A kernel without barriers: every work-item of a 1D range, groups on OpenMP threads (PAR) or
// in order on the calling thread. `global` must be a multiple of `local` (the reference's
// OpenCL 1.x launches are).
template <bool PAR = true, class F>
inline void run_groups(size_t global, size_t local, F&& f) {
    const long long groups = (long long)(global / local);
#pragma omp parallel for schedule(dynamic, 4) if (PAR)
    for (long long g = 0; g < groups; g++) {
        work_item& w = enter_group_1d(global, local, (size_t)g);
        for (size_t l = 0; l < local; l++) {
            set_local_id(w, l);
            f();
        }
    }
}

// A kernel without barriers over a 2D range (each work-item its own group).
template <class F>
inline void run_items_2d(size_t gx, size_t gy, F&& f) {
#pragma omp parallel for schedule(dynamic, 4)
    for (long long y = 0; y < (long long)gy; y++)
        for (size_t x = 0; x < gx; x++) {
            wi.dims = 2;
            wi.gsize[0] = gx;
            wi.gsize[1] = gy;
            wi.lsize[0] = wi.lsize[1] = 1;
            wi.ngroups[0] = gx;
            wi.ngroups[1] = gy;
            wi.grp[0] = wi.gid[0] = x;
            wi.grp[1] = wi.gid[1] = (size_t)y;
            wi.lid[0] = wi.lid[1] = 0;
            f();
        }
}

// Storage of one `__local T name[N]` declaration site for the work-group the calling host
// thread is running (the source rewrite binds a reference to it once per work-item).
template <class T, size_t N, int SITE>
inline T (&local_array())[N] {
    static thread_local T storage[N];
    return storage;
}

// Coroutine work-items for kernels with barriers. Their frames come from a per-thread pool
// (a work-group's items are created and destroyed together, thousands of times per launch).
struct frame_pool {
    std::vector<void*> free_blocks;
    size_t block = 0;
    ~frame_pool() {
        for (void* p : free_blocks) ::operator delete(p);
    }
};
inline thread_local frame_pool g_frames;

struct wi_task {
    struct promise_type {
        static void* operator new(size_t sz) {
            frame_pool& fp = g_frames;
            if (sz != fp.block) {  // a kernel with another frame size: start a new pool
                for (void* p : fp.free_blocks) ::operator delete(p);
                fp.free_blocks.clear();
                fp.block = sz;
            }
            if (fp.free_blocks.empty()) return ::operator new(sz);
            void* p = fp.free_blocks.back();
            fp.free_blocks.pop_back();
            return p;
        }
        static void operator delete(void* p, size_t sz) {
            frame_pool& fp = g_frames;
            if (sz == fp.block)
                fp.free_blocks.push_back(p);
            else
                ::operator delete(p);
        }
        wi_task get_return_object() { return wi_task{std::coroutine_handle<promise_type>::from_promise(*this)}; }
        std::suspend_never initial_suspend() noexcept { return {}; }
        std::suspend_always final_suspend() noexcept { return {}; }
        void return_void() noexcept {}
        void unhandled_exception() noexcept { std::terminate(); }
    };
    std::coroutine_handle<promise_type> h;
};

struct barrier_point {
    bool await_ready() const noexcept { return false; }
    void await_suspend(std::coroutine_handle<>) const noexcept {}
    void await_resume() const noexcept {}
};

// A kernel with barriers: each work-group's items start in local-id order and run to their
// first barrier, then are resumed in the same order, one barrier interval at a time.
// `local_mem(bytes)` returns the group's __local argument buffers (sized by the caller).
template <bool PAR = true, class F>
inline void run_groups_coro(size_t global, size_t local, F&& f) {
    const long long groups = (long long)(global / local);
#pragma omp parallel for schedule(dynamic, 4) if (PAR)
    for (long long g = 0; g < groups; g++) {
        std::vector<wi_task> items(local);
        work_item& w = enter_group_1d(global, local, (size_t)g);
        for (size_t l = 0; l < local; l++) {
            set_local_id(w, l);
            items[l] = f();
        }
        for (bool live = true; live;) {
            live = false;
            for (size_t l = 0; l < local; l++) {
                if (items[l].h.done()) continue;
                set_local_id(w, l);
                items[l].h.resume();
                live = true;
            }
        }
        for (auto& t : items) t.h.destroy();
    }
}

// ------------------------------------------------------------------------------------
// Atomics
// ------------------------------------------------------------------------------------
// atom_cmpxchg(p, cmp, val): stores val if *p == cmp; returns the old *p.
template <class T, class = std::enable_if_t<std::is_same_v<T, int> || std::is_same_v<T, uint>>>
inline T atom_cmpxchg(T* p, T cmp, T val) {
    std::atomic_ref<T> a(*p);
    a.compare_exchange_strong(cmp, val);
    return cmp;
}
template <class T, class C, class V, class = std::enable_if_t<std::is_same_v<T, int> || std::is_same_v<T, uint>>>
inline T atom_cmpxchg(T* p, C cmp, V val) {
    return atom_cmpxchg<T>(p, (T)cmp, (T)val);
}

// ------------------------------------------------------------------------------------
// Math, common and geometric built-ins
// ------------------------------------------------------------------------------------
enum pow_mode_t { POW_LIBM = 0, POW_INTEGER_CUBE = 1 };
inline int g_pow_mode = POW_INTEGER_CUBE;
inline void set_pow_mode(int m) { g_pow_mode = m; }

inline float pow(float x, float y) {
    if (g_pow_mode == POW_INTEGER_CUBE && y == 3.0f) return x * x * x;
    return ::powf(x, y);
}
inline float floor(float x) { return ::floorf(x); }
inline double floor(double x) { return ::floor(x); }
inline float fabs(float x) { return ::fabsf(x); }
inline float sqrt(float x) { return ::sqrtf(x); }

inline float max(float x, float y) { return x < y ? y : x; }
inline float min(float x, float y) { return y < x ? y : x; }
inline int max(int x, int y) { return x < y ? y : x; }
inline int min(int x, int y) { return y < x ? y : x; }
inline uint max(uint x, uint y) { return x < y ? y : x; }
inline uint min(uint x, uint y) { return y < x ? y : x; }
template <class A, class B, class = std::enable_if_t<is_vec_v<A> || is_vec_v<B>>>
inline auto max(const A& a, const B& b) {
    return vbin(a, b, [](auto x, auto y) { return x < y ? y : x; });
}
template <class A, class B, class = std::enable_if_t<is_vec_v<A> || is_vec_v<B>>>
inline auto min(const A& a, const B& b) {
    return vbin(a, b, [](auto x, auto y) { return y < x ? y : x; });
}

inline float dot(const float2& a, const float2& b) { return a.x * b.x + a.y * b.y; }
inline float dot(const float4& a, const float4& b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
inline float length(const float2& v) { return ::sqrtf(v.x * v.x + v.y * v.y); }
inline float length(const float4& v) { return ::sqrtf(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w); }
inline float fast_length(const float2& v) { return length(v); }
inline float fast_length(const float4& v) { return length(v); }
inline float2 normalize(const float2& v) {
    const float l = length(v);
    return float2(v.x / l, v.y / l);
}
inline float4 normalize(const float4& v) {
    const float l = length(v);
    return float4(v.x / l, v.y / l, v.z / l, v.w / l);
}
inline float4 cross(const float4& a, const float4& b) {
    return float4(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x, 0.0f);
}
// Swizzle arguments of the geometric built-ins.
template <class T, int N, int A, int B>
inline float length(const swz2<T, N, A, B>& v) {
    return length(float2(v));
}
template <class T, int N, int A, int B, class U>
inline float dot(const swz2<T, N, A, B>& a, const U& b) {
    return dot(float2(a), float2(vval(b)));
}

// ------------------------------------------------------------------------------------
// Images
// ------------------------------------------------------------------------------------
enum { IMG_HALF_RGBA = 0, IMG_FLOAT_RGBA = 1 };
struct image {
    int width, height, format;
    void* data;  // RGBA texels, row-major: _Float16[4 * w * h] or float[4 * w * h]
};
typedef image* image2d_t;
typedef uint sampler_t;
enum : uint {
    CLK_NORMALIZED_COORDS_FALSE = 0u,
    CLK_NORMALIZED_COORDS_TRUE = 1u,
    CLK_ADDRESS_NONE = 0u,
    CLK_ADDRESS_CLAMP_TO_EDGE = 2u,
    CLK_ADDRESS_CLAMP = 4u,
    CLK_ADDRESS_REPEAT = 6u,
    CLK_FILTER_NEAREST = 0u,
    CLK_FILTER_LINEAR = 16u,
};

inline float4 texel(const image* im, int i, int j) {
    const size_t o = 4 * ((size_t)j * (size_t)im->width + (size_t)i);
    if (im->format == IMG_HALF_RGBA) {
        const _Float16* p = (const _Float16*)im->data + o;
        return float4((float)p[0], (float)p[1], (float)p[2], (float)p[3]);
    }
    const float* p = (const float*)im->data + o;
    return float4(p[0], p[1], p[2], p[3]);
}

inline int clamp_edge(int i, int n) { return i < 0 ? 0 : (i > n - 1 ? n - 1 : i); }

// read_imagef(image, sampler, int2): nearest texel, unnormalised coordinates.
inline float4 read_imagef(image2d_t im, sampler_t s, const int2& c) {
    (void)s;
    return texel(im, clamp_edge(c.x, im->width), clamp_edge(c.y, im->height));
}

// read_imagef(image, sampler, float2) with normalised coordinates: the specification's
// nearest or bilinear filter with clamp-to-edge addressing.
inline float4 read_imagef(image2d_t im, sampler_t s, const float2& c) {
    const int W = im->width, H = im->height;
    float u = c.x, v = c.y;
    if (s & CLK_NORMALIZED_COORDS_TRUE) {
        u = u * (float)W;
        v = v * (float)H;
    }
    if (!(s & CLK_FILTER_LINEAR)) {
        return texel(im, clamp_edge((int)::floorf(u), W), clamp_edge((int)::floorf(v), H));
    }
    const float uu = u - 0.5f, vv = v - 0.5f;
    const float fu = ::floorf(uu), fv = ::floorf(vv);
    const int i0 = clamp_edge((int)fu, W), j0 = clamp_edge((int)fv, H);
    const int i1 = clamp_edge((int)fu + 1, W), j1 = clamp_edge((int)fv + 1, H);
    const float a = uu - fu, b = vv - fv;
    const float4 t00 = texel(im, i0, j0), t10 = texel(im, i1, j0);
    const float4 t01 = texel(im, i0, j1), t11 = texel(im, i1, j1);
    float4 r;
    for (int k = 0; k < 4; k++)
        r[k] = (1 - a) * (1 - b) * t00[k] + a * (1 - b) * t10[k] + (1 - a) * b * t01[k] + a * b * t11[k];
    return r;
}

inline void write_imagef(image2d_t im, const int2& c, const float4& v) {
    const size_t o = 4 * ((size_t)c.y * (size_t)im->width + (size_t)c.x);
    if (im->format == IMG_HALF_RGBA) {
        _Float16* p = (_Float16*)im->data + o;
        for (int k = 0; k < 4; k++) p[k] = (_Float16)v[k];
    } else {
        float* p = (float*)im->data + o;
        for (int k = 0; k < 4; k++) p[k] = v[k];
    }
}

}  // namespace clc
