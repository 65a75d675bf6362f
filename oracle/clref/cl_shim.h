// cl_shim.h -- OpenCL C, as CLImage's demosaic.cl uses it, for compiling that kernel file as
// C++ on the CPU (TEST INFRASTRUCTURE ONLY: it lets the reference's own kernel source run as
// a checker of the oracle's restatement; nothing in the product includes it).
//
// What it provides, under the conventions the oracle and the CUDA kernels share
// (climage_gb300/csrc/gls_clmath.h):
//   * vector types int2..int4, float2..float4, half2..half4 with component access, the
//     .xyz / .yz / .xy swizzles (read as values; .xyz / .yz written through a proxy), literals flattened
//     from scalars and vectors, component-wise arithmetic, comparisons (true = -1) and
//     && / ||, any / all; a vector used as a condition must agree in every component
//     (C++ cannot select per component there): otherwise the run is reported as failed;
//   * built-ins (half-precision mix and smoothstep round every operation to binary16, as an
//     fp16 ALU does): sqrt, fabs, fmin/fmax, mix, clamp, smoothstep, step, length, dot, atan2pi,
//     tanh, pow/powr, native_powr(x, 0.5) = sqrt(x), copysign, convert_float2..4, and
//     min / max / abs with the selects of the kernel file's own macros, applied per
//     component to vectors;
//   * images: read_imagef / read_imageh without a sampler (clamp to the edge), with the
//     linear sampler (normalised coordinates, clamp to the edge, fractions quantised to 8
//     bits, the four texels blended in the order w00, w10, w01, w11), write_imagef /
//     write_imageh, get_image_dim; 1-, 2- and 4-channel images; UNORM16 reads divide by 65535;
//   * get_global_id, set per work item by the driver.
// The kernel file is compiled with -fsingle-precision-constant (the reference builds it with
// -cl-single-precision-constant) and -ffp-contract=off.
#ifndef CL_SHIM_H
#define CL_SHIM_H

#include <cstddef>
#include <cstdint>
#include <type_traits>

#include "../../climage_gb300/csrc/gls_clmath.h"

typedef _Float16 half;

namespace clshim {
inline thread_local int gid[2];
// set when a vector condition (?: or if) had components that disagree: C++ cannot select
// per component there, so such a run is reported as failed instead of picking one side
inline thread_local bool mixed_condition = false;
template <class S>
constexpr bool scalar_v = std::is_arithmetic_v<S> || std::is_same_v<S, _Float16>;
}  // namespace clshim

inline size_t get_global_id(int d) { return (size_t)clshim::gid[d]; }

template <class T, int N>
struct V;
template <class T, int N, int K>
struct Swz;

template <class A>
struct ncomp {
    static constexpr int value = 1;
};
template <class T, int N>
struct ncomp<V<T, N>> {
    static constexpr int value = N;
};

template <class T, class A>
inline void vput(T* c, int& i, const A& a) {
    if constexpr (clshim::scalar_v<A>) {
        c[i++] = (T)a;
    } else {
        for (int k = 0; k < ncomp<A>::value; k++) c[i++] = (T)a.c[k];
    }
}

#define CLSHIM_VEC_BODY(N)                                                                         \
    V() = default;                                                                                 \
    template <class S, class = std::enable_if_t<clshim::scalar_v<S>>>                              \
    V(S s) {                                                                                       \
        for (int k = 0; k < N; k++) c[k] = (T)s;                                                   \
    }                                                                                              \
    explicit operator bool() const {                                                               \
        for (int k = 1; k < N; k++)                                                                \
            if ((c[k] != 0) != (c[0] != 0)) clshim::mixed_condition = true;                        \
        return c[0] != 0;                                                                          \
    }                                                                                              \
    template <class A, class B, class... R>                                                        \
    V(const A& a, const B& b, const R&... r) {                                                     \
        static_assert(ncomp<A>::value + ncomp<B>::value + (0 + ... + ncomp<R>::value) == N,        \
                      "vector literal component count");                                          \
        int i = 0;                                                                                 \
        vput(c, i, a);                                                                             \
        vput(c, i, b);                                                                             \
        (vput(c, i, r), ...);                                                                      \
    }

template <class T>
struct V<T, 2> {
    union {
        struct {
            T x, y;
        };
        T c[2];
    };
    CLSHIM_VEC_BODY(2)
};
template <class T>
struct V<T, 3> {
    union {
        struct {
            T x, y, z;
        };
        T c[3];
    };
    CLSHIM_VEC_BODY(3)
    V<T, 3> xyz() const { return V<T, 3>(x, y, z); }
    V<T, 2> yz() const { return V<T, 2>(y, z); }
    V<T, 2> xy() const { return V<T, 2>(x, y); }
    Swz<T, 3, 3> xyz_ref() { return Swz<T, 3, 3>{*this, 0}; }
    Swz<T, 3, 2> yz_ref() { return Swz<T, 3, 2>{*this, 1}; }
};
template <class T>
struct V<T, 4> {
    union {
        struct {
            T x, y, z, w;
        };
        T c[4];
    };
    CLSHIM_VEC_BODY(4)
    V<T, 3> xyz() const { return V<T, 3>(x, y, z); }
    V<T, 2> yz() const { return V<T, 2>(y, z); }
    V<T, 2> xy() const { return V<T, 2>(x, y); }
    Swz<T, 4, 3> xyz_ref() { return Swz<T, 4, 3>{*this, 0}; }
    Swz<T, 4, 2> yz_ref() { return Swz<T, 4, 2>{*this, 1}; }
};

// A swizzle written through (lab[0].yz *= chratio): a proxy over the vector's components.
template <class T, int N, int K>
struct Swz {
    V<T, N>& v;
    int i0;
    operator V<T, K>() const {
        V<T, K> r;
        for (int k = 0; k < K; k++) r.c[k] = v.c[i0 + k];
        return r;
    }
    Swz& operator=(const V<T, K>& b) {
        for (int k = 0; k < K; k++) v.c[i0 + k] = b.c[k];
        return *this;
    }
    template <class S>
    Swz& operator*=(const S& s) {
        for (int k = 0; k < K; k++) v.c[i0 + k] = v.c[i0 + k] * (T)s;
        return *this;
    }
    template <class S>
    Swz& operator+=(const S& s) {
        for (int k = 0; k < K; k++) v.c[i0 + k] = v.c[i0 + k] + (T)s;
        return *this;
    }
};

typedef V<int, 2> int2;
typedef V<int, 3> int3;
typedef V<int, 4> int4;
typedef V<float, 2> float2;
typedef V<float, 3> float3;
typedef V<float, 4> float4;
typedef V<half, 2> half2;
typedef V<half, 3> half3;
typedef V<half, 4> half4;

// ---- component-wise arithmetic ----
#define CLSHIM_BINOP(op)                                                                          \
    template <class T, int N>                                                                     \
    inline V<T, N> operator op(const V<T, N>& a, const V<T, N>& b) {                              \
        V<T, N> r;                                                                                \
        for (int k = 0; k < N; k++) r.c[k] = a.c[k] op b.c[k];                                    \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class S, class = std::enable_if_t<clshim::scalar_v<S>>>             \
    inline V<T, N> operator op(const V<T, N>& a, S s) {                                           \
        V<T, N> r;                                                                                \
        for (int k = 0; k < N; k++) r.c[k] = a.c[k] op(T) s;                                      \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class S, class = std::enable_if_t<clshim::scalar_v<S>>>             \
    inline V<T, N> operator op(S s, const V<T, N>& a) {                                           \
        V<T, N> r;                                                                                \
        for (int k = 0; k < N; k++) r.c[k] = (T)s op a.c[k];                                      \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class B>                                                            \
    inline V<T, N>& operator op##=(V<T, N>& a, const B& b) {                                      \
        a = a op b;                                                                               \
        return a;                                                                                 \
    }
CLSHIM_BINOP(+)
CLSHIM_BINOP(-)
CLSHIM_BINOP(*)
CLSHIM_BINOP(/)

template <class T, int N>
inline V<T, N> operator-(const V<T, N>& a) {
    V<T, N> r;
    for (int k = 0; k < N; k++) r.c[k] = -a.c[k];
    return r;
}

#define CLSHIM_CMP(op)                                                                            \
    template <class T, int N>                                                                     \
    inline V<int, N> operator op(const V<T, N>& a, const V<T, N>& b) {                            \
        V<int, N> r;                                                                              \
        for (int k = 0; k < N; k++) r.c[k] = a.c[k] op b.c[k] ? -1 : 0;                           \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class S, class = std::enable_if_t<clshim::scalar_v<S>>>             \
    inline V<int, N> operator op(const V<T, N>& a, S s) {                                         \
        V<int, N> r;                                                                              \
        for (int k = 0; k < N; k++) r.c[k] = a.c[k] op(T) s ? -1 : 0;                             \
        return r;                                                                                 \
    }
CLSHIM_CMP(<)
CLSHIM_CMP(>)
CLSHIM_CMP(<=)
CLSHIM_CMP(>=)
CLSHIM_CMP(==)
CLSHIM_CMP(!=)

// && / || per component (true = -1)
template <int N>
inline V<int, N> operator&&(const V<int, N>& a, const V<int, N>& b) {
    V<int, N> r;
    for (int k = 0; k < N; k++) r.c[k] = (a.c[k] && b.c[k]) ? -1 : 0;
    return r;
}
template <int N>
inline V<int, N> operator||(const V<int, N>& a, const V<int, N>& b) {
    V<int, N> r;
    for (int k = 0; k < N; k++) r.c[k] = (a.c[k] || b.c[k]) ? -1 : 0;
    return r;
}

template <int N>
inline int any(const V<int, N>& a) {
    for (int k = 0; k < N; k++)
        if (a.c[k] < 0) return 1;
    return 0;
}
template <int N>
inline int all(const V<int, N>& a) {
    for (int k = 0; k < N; k++)
        if (a.c[k] >= 0) return 0;
    return 1;
}

// ---- built-ins: float scalars through the shared conventions (half through float); any
// mix of scalars and vectors applies them per component, scalars broadcast ----
inline float clf(half v) { return (float)v; }
inline float clf(float v) { return v; }
inline float clf(double v) { return (float)v; }
inline float clf(int v) { return (float)v; }

template <class... A>
struct first_vec {
    using type = void;
};
template <class A, class... R>
struct first_vec<A, R...> {
    using type = std::conditional_t<!clshim::scalar_v<A>, A, typename first_vec<R...>::type>;
};
template <class X>
inline float cget(const X& x, int k) {
    if constexpr (clshim::scalar_v<X>) return clf(x);
    else return clf(x.c[k]);
}

#define CLSHIM_F1(name, expr)                                                                     \
    inline float name(float x) { return expr; }                                                   \
    inline half name(half hx) {                                                                   \
        const float x = (float)hx;                                                                \
        return (half)(expr);                                                                      \
    }                                                                                             \
    template <class T, int N>                                                                     \
    inline V<T, N> name(const V<T, N>& a) {                                                       \
        V<T, N> r;                                                                                \
        for (int k = 0; k < N; k++) r.c[k] = (T)name(clf(a.c[k]));                                \
        return r;                                                                                 \
    }
CLSHIM_F1(sqrt, glsm::sqrt_(x))
CLSHIM_F1(fabs, glsm::fabs_(x))
CLSHIM_F1(tanh, glsm::tanh_(x))
CLSHIM_F1(ceil, -glsm::floor_(-x))
CLSHIM_F1(exp, glsm::exp2_(x * 1.44269504088896341f))
CLSHIM_F1(native_exp, glsm::exp2_(x * 1.44269504088896341f))

inline float fmax(float a, float b) { return glsm::fmax_(a, b); }
inline float fmin(float a, float b) { return glsm::fmin_(a, b); }
inline float step(float e, float x) { return glsm::step_(e, x); }
inline float atan2pi(float y, float x) { return glsm::atan2pi_(y, x); }
inline float pow(float x, float y) { return glsm::pow_(x, y); }
inline float powr(float x, float y) { return glsm::powr_(x, y); }
inline float native_powr(float x, float y) { return y == 0.5f ? glsm::sqrt_(x) : glsm::powr_(x, y); }
inline float copysign(float x, float s) { return glsm::copysign_(x, s); }
inline float mix(float a, float b, float t) { return glsm::mix_(a, b, t); }
// half arithmetic: every operation rounded to binary16, as an fp16 ALU computes it
inline float hr(float v) { return glsm::round_half(v); }
inline half mix(half x, half y, half t) {
    return (half)hr((float)x + hr(hr((float)y - (float)x) * (float)t));
}
inline half smoothstep(half e0, half e1, half x) {
    const float u = glsm::clamp_(hr(glsm::div_(hr((float)x - (float)e0), hr((float)e1 - (float)e0))), 0.0f, 1.0f);
    return (half)hr(hr(u * u) * hr(3.0f - hr(2.0f * u)));
}
inline float clamp(float x, float lo, float hi) { return glsm::clamp_(x, lo, hi); }
inline float smoothstep(float e0, float e1, float x) { return glsm::smoothstep_ref(e0, e1, x); }

#define CLSHIM_E2(name)                                                                           \
    template <class A, class B, class Vt = typename first_vec<A, B>::type,                        \
              class = std::enable_if_t<!std::is_void_v<Vt>>>                                      \
    inline Vt name(const A& a, const B& b) {                                                      \
        Vt r;                                                                                     \
        for (int k = 0; k < ncomp<Vt>::value; k++) r.c[k] = name(cget(a, k), cget(b, k));        \
        return r;                                                                                 \
    }
#define CLSHIM_E3(name)                                                                           \
    template <class A, class B, class C, class Vt = typename first_vec<A, B, C>::type,            \
              class = std::enable_if_t<!std::is_void_v<Vt>>>                                      \
    inline Vt name(const A& a, const B& b, const C& c) {                                          \
        Vt r;                                                                                     \
        for (int k = 0; k < ncomp<Vt>::value; k++) r.c[k] = name(cget(a, k), cget(b, k), cget(c, k)); \
        return r;                                                                                 \
    }
CLSHIM_E2(fmax)
CLSHIM_E2(fmin)
CLSHIM_E2(step)
CLSHIM_E2(atan2pi)
CLSHIM_E2(pow)
CLSHIM_E2(powr)
CLSHIM_E2(native_powr)
CLSHIM_E2(copysign)
CLSHIM_E3(mix)
CLSHIM_E3(clamp)
CLSHIM_E3(smoothstep)

template <class T, int N>
inline T dot(const V<T, N>& a, const V<T, N>& b) {
    T s = a.c[0] * b.c[0];
    for (int k = 1; k < N; k++) s = s + a.c[k] * b.c[k];
    return s;
}
inline float length(const float2& a) { return glsm::length2_(a.x, a.y); }
inline float length(const float3& a) { return glsm::length3_(a.x, a.y, a.z); }
inline float length(const float4& a) { return glsm::length4_(a.x, a.y, a.z, a.w); }

inline float2 convert_float2(const int2& a) { return float2((float)a.x, (float)a.y); }
inline float3 convert_float3(const int3& a) { return float3((float)a.x, (float)a.y, (float)a.z); }
inline float4 convert_float4(const int4& a) { return float4((float)a.x, (float)a.y, (float)a.z, (float)a.w); }

// cond ? a : b with OpenCL's semantics: a vector condition selects per component (true = the
// sign bit set), a scalar one picks a side
template <class A, class B, class Cd>
inline A clref_select(const A& a, const B& b, const Cd& cond) {
    if constexpr (clshim::scalar_v<Cd> || std::is_same_v<Cd, bool>) {
        return cond ? a : (A)b;
    } else {
        A r;
        for (int k = 0; k < ncomp<Cd>::value; k++) {
            decltype(r.c[0] + 0) ak, bk;
            if constexpr (clshim::scalar_v<A>) ak = a; else ak = a.c[k];
            if constexpr (clshim::scalar_v<B>) bk = b; else bk = b.c[k];
            r.c[k] = cond.c[k] < 0 ? ak : bk;
        }
        return r;
    }
}

// min / max / abs: the kernel file's own macros (plain selects), per component on vectors;
// the macros are redirected here so that they still expand before name lookup.
template <class A, class B>
inline A clref_min(const A& a, const B& b) {
    if constexpr (clshim::scalar_v<A>) {
        const A bb = (A)b;
        return a < bb ? a : bb;
    } else {
        A r;
        for (int k = 0; k < ncomp<A>::value; k++) {
            decltype(r.c[0] + 0) bk;
            if constexpr (clshim::scalar_v<B>) bk = b; else bk = b.c[k];
            r.c[k] = a.c[k] < bk ? a.c[k] : bk;
        }
        return r;
    }
}
template <class A, class B>
inline A clref_max(const A& a, const B& b) {
    if constexpr (clshim::scalar_v<A>) {
        const A bb = (A)b;
        return a > bb ? a : bb;
    } else {
        A r;
        for (int k = 0; k < ncomp<A>::value; k++) {
            decltype(r.c[0] + 0) bk;
            if constexpr (clshim::scalar_v<B>) bk = b; else bk = b.c[k];
            r.c[k] = a.c[k] > bk ? a.c[k] : bk;
        }
        return r;
    }
}
template <class A>
inline A clref_abs(const A& a) {
    if constexpr (clshim::scalar_v<A>) {
        return a > 0 ? a : -a;
    } else {
        A r;
        for (int k = 0; k < ncomp<A>::value; k++) r.c[k] = a.c[k] > 0 ? a.c[k] : -a.c[k];
        return r;
    }
}

// ---- images ----
enum { CLSHIM_U16 = 0, CLSHIM_F32 = 1, CLSHIM_F16 = 2, CLSHIM_U8 = 3 };
struct cl_image {
    int w, h, ch, kind;
    void* p;
};
typedef cl_image* image2d_t;
typedef int sampler_t;

inline float clshim_get(const cl_image* im, int x, int y, int k) {
    x = x < 0 ? 0 : (x >= im->w ? im->w - 1 : x);
    y = y < 0 ? 0 : (y >= im->h ? im->h - 1 : y);
    const size_t i = ((size_t)y * im->w + x) * im->ch + k;
    switch (im->kind) {
        case CLSHIM_U16: return glsm::from_unorm16(((const uint16_t*)im->p)[i]);
        case CLSHIM_F32: return ((const float*)im->p)[i];
        case CLSHIM_F16: return (float)((const half*)im->p)[i];
        default: return glsm::div_((float)((const uint8_t*)im->p)[i], 255.0f);
    }
}

inline float4 read_imagef(image2d_t im, int2 pos) {
    if (im->ch == 1) return float4(clshim_get(im, pos.x, pos.y, 0), 0.0f, 0.0f, 1.0f);
    if (im->ch == 2) return float4(clshim_get(im, pos.x, pos.y, 0), clshim_get(im, pos.x, pos.y, 1), 0.0f, 1.0f);
    return float4(clshim_get(im, pos.x, pos.y, 0), clshim_get(im, pos.x, pos.y, 1), clshim_get(im, pos.x, pos.y, 2),
                  clshim_get(im, pos.x, pos.y, 3));
}
inline half4 read_imageh(image2d_t im, int2 pos) {
    const float4 v = read_imagef(im, pos);
    return half4((half)v.x, (half)v.y, (half)v.z, (half)v.w);
}
inline float4 read_imagef(image2d_t im, sampler_t, float2 pos) {
    const float fu = pos.x * (float)im->w - 0.5f, fv = pos.y * (float)im->h - 0.5f;
    const float i0f = glsm::floor_(fu), j0f = glsm::floor_(fv);
    float a = fu - i0f, b = fv - j0f;
    a = glsm::floor_(a * 256.0f + 0.5f) / 256.0f;
    b = glsm::floor_(b * 256.0f + 0.5f) / 256.0f;
    const int i0 = (int)i0f, j0 = (int)j0f;
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float o[4] = {0.0f, 0.0f, 0.0f, 1.0f};
    for (int k = 0; k < im->ch; k++)
        o[k] = w00 * clshim_get(im, i0, j0, k) + w10 * clshim_get(im, i0 + 1, j0, k) +
               w01 * clshim_get(im, i0, j0 + 1, k) + w11 * clshim_get(im, i0 + 1, j0 + 1, k);
    return float4(o[0], o[1], o[2], o[3]);
}

inline void clshim_put(image2d_t im, int x, int y, int k, float v) {
    if (x < 0 || y < 0 || x >= im->w || y >= im->h) return;  // out-of-range writes are dropped
    const size_t i = ((size_t)y * im->w + x) * im->ch + k;
    switch (im->kind) {
        case CLSHIM_F32: ((float*)im->p)[i] = v; break;
        case CLSHIM_F16: ((half*)im->p)[i] = (half)glsm::round_half(v); break;
        case CLSHIM_U8: ((uint8_t*)im->p)[i] = glsm::to_unorm8(v); break;
        default: break;
    }
}
inline void write_imagef(image2d_t im, int2 pos, float4 v) {
    for (int k = 0; k < im->ch; k++) clshim_put(im, pos.x, pos.y, k, v.c[k]);
}
inline void write_imageh(image2d_t im, int2 pos, half4 v) {
    for (int k = 0; k < im->ch; k++) clshim_put(im, pos.x, pos.y, k, (float)v.c[k]);
}
inline int2 get_image_dim(image2d_t im) { return int2(im->w, im->h); }
inline int get_image_width(image2d_t im) { return im->w; }
inline int get_image_height(image2d_t im) { return im->h; }

// ---- qualifiers and constants ----
#define kernel
#define __kernel
#define read_only
#define write_only
#define __read_only
#define __write_only
#define constant
#define __constant
#define global
#define __global
#define CLK_NORMALIZED_COORDS_TRUE 1
#define CLK_ADDRESS_CLAMP_TO_EDGE 2
#define CLK_FILTER_LINEAR 4
#define M_SQRT2_F 1.41421356237309504880f
#define M_PI_F 3.14159265358979323846f

#endif  // CL_SHIM_H
