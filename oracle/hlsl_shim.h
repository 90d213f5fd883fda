/*
 * hlsl_shim.h -- TEST INFRASTRUCTURE ONLY (oracle pinning).
 *
 * The C++ stand-ins for HLSL's built-in types and intrinsics that let the reference's own
 * shader math (its .hlsl files, mechanically edited by oracle/ref_build.py) compile with g++
 * on the CPU, so that the oracle's restatement can be compared with the reference's code on
 * the same inputs. Vectors with swizzles, 3x3 matrices, the elementwise intrinsics, bit
 * casts, and the resource types the shader math reads (textures sampled with an FP32
 * bilinear/trilinear LINEAR_CLAMP filter, structured buffers). Nothing in the product path
 * includes this file.
 *
 * Deliberate choices: lerp(a, b, t) = a + t * (b - a); normalize(v) = v * (1 / sqrt(dot(v, v)));
 * rsqrt(x) = 1 / sqrt(x); round() rounds half to even; texture filtering weights are FP32
 * (a GPU's texture unit uses 8-bit weights, which no CPU code reproduces).
 */
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>

// The namespace is chosen by the includer, so that one program can hold the shader code twice,
// compiled with different defines (hlsl by default).
#ifndef HLSL_SHIM_NS
#define HLSL_SHIM_NS hlsl
#endif
namespace HLSL_SHIM_NS
{
typedef unsigned int uint;
typedef float half;
typedef uint32_t dword;

template <class T, int N> struct vec;

// A swizzle: a view of components I... of its host vector's storage (a union member).
template <class T, int N, int... I> struct swz
{
    T s[N];
    using V = vec<T, (int)sizeof...(I)>;
    operator V() const
    {
        V r;
        int k = 0;
        ((r.v[k++] = s[I]), ...);
        return r;
    }
    swz& operator=(const V& o)
    {
        T tmp[sizeof...(I)];
        for (int k = 0; k < (int)sizeof...(I); ++k) tmp[k] = o.v[k];
        int k = 0;
        ((s[I] = tmp[k++]), ...);
        return *this;
    }
    swz& operator=(const swz& o) { return *this = V(o); }
    template <class X> swz& operator+=(const X& o) { return *this = V(*this) + o; }
    template <class X> swz& operator-=(const X& o) { return *this = V(*this) - o; }
    template <class X> swz& operator*=(const X& o) { return *this = V(*this) * o; }
    template <class X> swz& operator/=(const X& o) { return *this = V(*this) / o; }
};

#define HLSL_VEC_COMMON(N_)                                                                                     \
    vec() = default;                                                                                            \
    vec(const vec& o) { std::memcpy(v, o.v, sizeof(v)); }                                                      \
    vec& operator=(const vec& o)                                                                                \
    {                                                                                                           \
        std::memcpy(v, o.v, sizeof(v));                                                                         \
        return *this;                                                                                           \
    }                                                                                                           \
    template <class S, typename std::enable_if<std::is_arithmetic<S>::value, int>::type = 0> vec(S s)           \
    {                                                                                                           \
        for (int k = 0; k < N_; ++k) v[k] = (T)s;                                                               \
    }                                                                                                           \
    template <class U, int M, typename std::enable_if<(M >= N_), int>::type = 0> vec(const vec<U, M>& o)         \
    {                                                                                                           \
        for (int k = 0; k < N_; ++k) v[k] = (T)o.v[k];                                                          \
    }                                                                                                           \
    template <class U, int M, int... J, typename std::enable_if<(sizeof...(J) >= N_), int>::type = 0>           \
    vec(const swz<U, M, J...>& o)                                                                               \
    {                                                                                                           \
        const U src[] = {o.s[J]...};                                                                            \
        for (int k = 0; k < N_; ++k) v[k] = (T)src[k];                                                          \
    }                                                                                                           \
    T& operator[](int k) { return v[k]; }                                                                       \
    const T& operator[](int k) const { return v[k]; }                                                           \
    template <class X> vec& operator+=(const X& o) { return *this = *this + o; }                                \
    template <class X> vec& operator-=(const X& o) { return *this = *this - o; }                                \
    template <class X> vec& operator*=(const X& o) { return *this = *this * o; }                                \
    template <class X> vec& operator/=(const X& o) { return *this = *this / o; }                                \
    template <class X> vec& operator%=(const X& o) { return *this = *this % o; }                                \
    template <class X> vec& operator&=(const X& o) { return *this = *this & o; }                                \
    template <class X> vec& operator|=(const X& o) { return *this = *this | o; }                                \
    template <class X> vec& operator^=(const X& o) { return *this = *this ^ o; }

template <class T> struct vec<T, 2>
{
    union
    {
        struct { T x, y; };
        T v[2];
        swz<T, 2, 0, 0> xx;
        swz<T, 2, 0, 1> xy;
        swz<T, 2, 1, 0> yx;
        swz<T, 2, 1, 1> yy;
        swz<T, 2, 0, 0, 0> xxx;
        swz<T, 2, 0, 0, 1> xxy;
        swz<T, 2, 0, 1, 0> xyx;
        swz<T, 2, 0, 1, 1> xyy;
        swz<T, 2, 1, 0, 0> yxx;
        swz<T, 2, 1, 0, 1> yxy;
        swz<T, 2, 1, 1, 0> yyx;
        swz<T, 2, 1, 1, 1> yyy;
        swz<T, 2, 0, 1> rg;
    };
    HLSL_VEC_COMMON(2)
    vec(T a, T b) { v[0] = a; v[1] = b; }
};

template <class T> struct vec<T, 3>
{
    union
    {
        struct { T x, y, z; };
        struct { T r, g, b; };
        T v[3];
        swz<T, 3, 0, 0> xx;
        swz<T, 3, 0, 1> xy;
        swz<T, 3, 0, 2> xz;
        swz<T, 3, 1, 0> yx;
        swz<T, 3, 1, 1> yy;
        swz<T, 3, 1, 2> yz;
        swz<T, 3, 2, 0> zx;
        swz<T, 3, 2, 1> zy;
        swz<T, 3, 2, 2> zz;
        swz<T, 3, 0, 0, 0> xxx;
        swz<T, 3, 0, 0, 1> xxy;
        swz<T, 3, 0, 0, 2> xxz;
        swz<T, 3, 0, 1, 0> xyx;
        swz<T, 3, 0, 1, 1> xyy;
        swz<T, 3, 0, 1, 2> xyz;
        swz<T, 3, 0, 2, 0> xzx;
        swz<T, 3, 0, 2, 1> xzy;
        swz<T, 3, 0, 2, 2> xzz;
        swz<T, 3, 1, 0, 0> yxx;
        swz<T, 3, 1, 0, 1> yxy;
        swz<T, 3, 1, 0, 2> yxz;
        swz<T, 3, 1, 1, 0> yyx;
        swz<T, 3, 1, 1, 1> yyy;
        swz<T, 3, 1, 1, 2> yyz;
        swz<T, 3, 1, 2, 0> yzx;
        swz<T, 3, 1, 2, 1> yzy;
        swz<T, 3, 1, 2, 2> yzz;
        swz<T, 3, 2, 0, 0> zxx;
        swz<T, 3, 2, 0, 1> zxy;
        swz<T, 3, 2, 0, 2> zxz;
        swz<T, 3, 2, 1, 0> zyx;
        swz<T, 3, 2, 1, 1> zyy;
        swz<T, 3, 2, 1, 2> zyz;
        swz<T, 3, 2, 2, 0> zzx;
        swz<T, 3, 2, 2, 1> zzy;
        swz<T, 3, 2, 2, 2> zzz;
        swz<T, 3, 0, 1, 2> rgb;
        swz<T, 3, 0, 1> rg;
    };
    HLSL_VEC_COMMON(3)
    vec(T a, T b, T c) { v[0] = a; v[1] = b; v[2] = c; }
    vec(const vec<T, 2>& a, T c) { v[0] = a.v[0]; v[1] = a.v[1]; v[2] = c; }
    vec(T a, const vec<T, 2>& b) { v[0] = a; v[1] = b.v[0]; v[2] = b.v[1]; }
};

template <class T> struct vec<T, 4>
{
    union
    {
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
        T v[4];
        swz<T, 4, 0, 0> xx;
        swz<T, 4, 0, 1> xy;
        swz<T, 4, 0, 2> xz;
        swz<T, 4, 0, 3> xw;
        swz<T, 4, 1, 0> yx;
        swz<T, 4, 1, 1> yy;
        swz<T, 4, 1, 2> yz;
        swz<T, 4, 1, 3> yw;
        swz<T, 4, 2, 0> zx;
        swz<T, 4, 2, 1> zy;
        swz<T, 4, 2, 2> zz;
        swz<T, 4, 2, 3> zw;
        swz<T, 4, 3, 0> wx;
        swz<T, 4, 3, 1> wy;
        swz<T, 4, 3, 2> wz;
        swz<T, 4, 3, 3> ww;
        swz<T, 4, 0, 0, 0> xxx;
        swz<T, 4, 0, 0, 1> xxy;
        swz<T, 4, 0, 0, 2> xxz;
        swz<T, 4, 0, 0, 3> xxw;
        swz<T, 4, 0, 1, 0> xyx;
        swz<T, 4, 0, 1, 1> xyy;
        swz<T, 4, 0, 1, 2> xyz;
        swz<T, 4, 0, 1, 3> xyw;
        swz<T, 4, 0, 2, 0> xzx;
        swz<T, 4, 0, 2, 1> xzy;
        swz<T, 4, 0, 2, 2> xzz;
        swz<T, 4, 0, 2, 3> xzw;
        swz<T, 4, 0, 3, 0> xwx;
        swz<T, 4, 0, 3, 1> xwy;
        swz<T, 4, 0, 3, 2> xwz;
        swz<T, 4, 0, 3, 3> xww;
        swz<T, 4, 1, 0, 0> yxx;
        swz<T, 4, 1, 0, 1> yxy;
        swz<T, 4, 1, 0, 2> yxz;
        swz<T, 4, 1, 0, 3> yxw;
        swz<T, 4, 1, 1, 0> yyx;
        swz<T, 4, 1, 1, 1> yyy;
        swz<T, 4, 1, 1, 2> yyz;
        swz<T, 4, 1, 1, 3> yyw;
        swz<T, 4, 1, 2, 0> yzx;
        swz<T, 4, 1, 2, 1> yzy;
        swz<T, 4, 1, 2, 2> yzz;
        swz<T, 4, 1, 2, 3> yzw;
        swz<T, 4, 1, 3, 0> ywx;
        swz<T, 4, 1, 3, 1> ywy;
        swz<T, 4, 1, 3, 2> ywz;
        swz<T, 4, 1, 3, 3> yww;
        swz<T, 4, 2, 0, 0> zxx;
        swz<T, 4, 2, 0, 1> zxy;
        swz<T, 4, 2, 0, 2> zxz;
        swz<T, 4, 2, 0, 3> zxw;
        swz<T, 4, 2, 1, 0> zyx;
        swz<T, 4, 2, 1, 1> zyy;
        swz<T, 4, 2, 1, 2> zyz;
        swz<T, 4, 2, 1, 3> zyw;
        swz<T, 4, 2, 2, 0> zzx;
        swz<T, 4, 2, 2, 1> zzy;
        swz<T, 4, 2, 2, 2> zzz;
        swz<T, 4, 2, 2, 3> zzw;
        swz<T, 4, 2, 3, 0> zwx;
        swz<T, 4, 2, 3, 1> zwy;
        swz<T, 4, 2, 3, 2> zwz;
        swz<T, 4, 2, 3, 3> zww;
        swz<T, 4, 3, 0, 0> wxx;
        swz<T, 4, 3, 0, 1> wxy;
        swz<T, 4, 3, 0, 2> wxz;
        swz<T, 4, 3, 0, 3> wxw;
        swz<T, 4, 3, 1, 0> wyx;
        swz<T, 4, 3, 1, 1> wyy;
        swz<T, 4, 3, 1, 2> wyz;
        swz<T, 4, 3, 1, 3> wyw;
        swz<T, 4, 3, 2, 0> wzx;
        swz<T, 4, 3, 2, 1> wzy;
        swz<T, 4, 3, 2, 2> wzz;
        swz<T, 4, 3, 2, 3> wzw;
        swz<T, 4, 3, 3, 0> wwx;
        swz<T, 4, 3, 3, 1> wwy;
        swz<T, 4, 3, 3, 2> wwz;
        swz<T, 4, 3, 3, 3> www;
        swz<T, 4, 0, 1, 2, 3> xyzw;
        swz<T, 4, 0, 1, 2> rgb;
        swz<T, 4, 0, 1> rg;
        swz<T, 4, 0, 1, 2, 3> rgba;
    };
    HLSL_VEC_COMMON(4)
    vec(T a, T b, T c, T d) { v[0] = a; v[1] = b; v[2] = c; v[3] = d; }
    vec(const vec<T, 3>& a, T d) { v[0] = a.v[0]; v[1] = a.v[1]; v[2] = a.v[2]; v[3] = d; }
    vec(T a, const vec<T, 3>& b) { v[0] = a; v[1] = b.v[0]; v[2] = b.v[1]; v[3] = b.v[2]; }
    vec(const vec<T, 2>& a, const vec<T, 2>& b) { v[0] = a.v[0]; v[1] = a.v[1]; v[2] = b.v[0]; v[3] = b.v[1]; }
    vec(const vec<T, 2>& a, T c, T d) { v[0] = a.v[0]; v[1] = a.v[1]; v[2] = c; v[3] = d; }
};
#undef HLSL_VEC_COMMON

typedef vec<float, 2> float2;
typedef vec<float, 3> float3;
typedef vec<float, 4> float4;
typedef vec<int, 2> int2;
typedef vec<int, 3> int3;
typedef vec<int, 4> int4;
typedef vec<uint, 2> uint2;
typedef vec<uint, 3> uint3;
typedef vec<uint, 4> uint4;
typedef vec<bool, 2> bool2;
typedef vec<bool, 3> bool3;
typedef vec<bool, 4> bool4;
typedef vec<float, 2> half2;
typedef vec<float, 3> half3;
typedef vec<float, 4> half4;

// ---- vector traits and normalisation (swizzles become vectors, scalars stay scalars)
template <class X> struct vt
{
    static constexpr bool is = false;
    typedef X elem;
    static constexpr int n = 1;
};
template <class T, int N> struct vt<vec<T, N>>
{
    static constexpr bool is = true;
    typedef T elem;
    static constexpr int n = N;
};
template <class T, int N, int... I> struct vt<swz<T, N, I...>>
{
    static constexpr bool is = true;
    typedef T elem;
    static constexpr int n = (int)sizeof...(I);
};
template <class X> auto nv(const X& x)
{
    if constexpr (vt<X>::is) return vec<typename vt<X>::elem, vt<X>::n>(x);
    else return x;
}
template <class X> using enable_vec = typename std::enable_if<vt<X>::is, int>::type;

template <class A, class B, class F> auto zipv(const A& a, const B& b, F f)
{
    typedef A NA;
    typedef B NB;
    constexpr int n = vt<NA>::n > vt<NB>::n ? vt<NA>::n : vt<NB>::n;
    typedef decltype(f(typename vt<NA>::elem(), typename vt<NB>::elem())) R;
    vec<R, n> r;
    for (int k = 0; k < n; ++k)
    {
        typename vt<NA>::elem ea;
        typename vt<NB>::elem eb;
        if constexpr (vt<NA>::is) ea = a.v[vt<NA>::n == 1 ? 0 : k]; else ea = a;
        if constexpr (vt<NB>::is) eb = b.v[vt<NB>::n == 1 ? 0 : k]; else eb = b;
        r.v[k] = f(ea, eb);
    }
    return r;
}
template <class A, class B, class F> auto zip(const A& a0, const B& b0, F f)
{
    auto a = nv(a0);
    auto b = nv(b0);
    if constexpr (!vt<decltype(a)>::is && !vt<decltype(b)>::is) return f(a, b);
    else return zipv(a, b, f);
}
template <class A, class F> auto each(const A& a0, F f)
{
    auto a = nv(a0);
    if constexpr (vt<decltype(a)>::is)
    {
        typedef decltype(f(a.v[0])) R;
        vec<R, vt<decltype(a)>::n> r;
        for (int k = 0; k < vt<decltype(a)>::n; ++k) r.v[k] = f(a.v[k]);
        return r;
    }
    else return f(a);
}

#define HLSL_BINOP(OP)                                                                                          \
    template <class A, class B, typename std::enable_if<vt<A>::is || vt<B>::is, int>::type = 0>                 \
    auto operator OP(const A& a, const B& b)                                                                    \
    {                                                                                                           \
        return zip(a, b, [](auto p, auto q) { return p OP q; });                                               \
    }
HLSL_BINOP(+)
HLSL_BINOP(-)
HLSL_BINOP(*)
HLSL_BINOP(/)
HLSL_BINOP(%)
HLSL_BINOP(&)
HLSL_BINOP(|)
HLSL_BINOP(^)
HLSL_BINOP(<<)
HLSL_BINOP(>>)
HLSL_BINOP(<)
HLSL_BINOP(>)
HLSL_BINOP(<=)
HLSL_BINOP(>=)
HLSL_BINOP(==)
HLSL_BINOP(!=)
HLSL_BINOP(&&)
HLSL_BINOP(||)
#undef HLSL_BINOP
template <class A, enable_vec<A> = 0> auto operator-(const A& a) { return each(a, [](auto p) { return -p; }); }
template <class A, enable_vec<A> = 0> auto operator!(const A& a) { return each(a, [](auto p) { return !p; }); }
template <class A, enable_vec<A> = 0> auto operator~(const A& a) { return each(a, [](auto p) { return ~p; }); }

// ---- elementwise intrinsics
#define HLSL_UNARY(NAME, EXPR)                                                                                  \
    template <class A> auto NAME(const A& a)                                                                    \
    {                                                                                                           \
        return each(a, [](auto x) { return EXPR; });                                                            \
    }
HLSL_UNARY(abs, (x < 0 ? -x : x))
HLSL_UNARY(sqrt, std::sqrt((float)x))
HLSL_UNARY(rsqrt, 1.0f / std::sqrt((float)x))
HLSL_UNARY(rcp, 1.0f / (float)x)
HLSL_UNARY(exp, std::exp((float)x))
HLSL_UNARY(exp2, std::exp2((float)x))
HLSL_UNARY(log, std::log((float)x))
HLSL_UNARY(log2, std::log2((float)x))
HLSL_UNARY(log10, std::log10((float)x))
HLSL_UNARY(cos, std::cos((float)x))
HLSL_UNARY(sin, std::sin((float)x))
HLSL_UNARY(tan, std::tan((float)x))
HLSL_UNARY(acos, std::acos((float)x))
HLSL_UNARY(asin, std::asin((float)x))
HLSL_UNARY(atan, std::atan((float)x))
HLSL_UNARY(cosh, std::cosh((float)x))
HLSL_UNARY(sinh, std::sinh((float)x))
HLSL_UNARY(tanh, std::tanh((float)x))
HLSL_UNARY(floor, std::floor((float)x))
HLSL_UNARY(ceil, std::ceil((float)x))
HLSL_UNARY(trunc, std::trunc((float)x))
HLSL_UNARY(round, std::nearbyint((float)x))
HLSL_UNARY(frac, (float)x - std::floor((float)x))
HLSL_UNARY(saturate, std::fmin(std::fmax((float)x, 0.0f), 1.0f))
HLSL_UNARY(sign, (int)((x > 0) - (x < 0)))
HLSL_UNARY(isnan, std::isnan((float)x))
HLSL_UNARY(isinf, std::isinf((float)x))
HLSL_UNARY(isfinite, std::isfinite((float)x))
HLSL_UNARY(radians, (float)x * 0.0174532924f)
HLSL_UNARY(degrees, (float)x * 57.2957764f)
#undef HLSL_UNARY

template <class A, class B> auto min(const A& a, const B& b)
{
    return zip(a, b, [](auto p, auto q) {
        typedef decltype(p + q) R;
        if constexpr (std::is_floating_point<R>::value) return (R)std::fmin((R)p, (R)q);
        else return (R)(q < p ? q : p);
    });
}
template <class A, class B> auto max(const A& a, const B& b)
{
    return zip(a, b, [](auto p, auto q) {
        typedef decltype(p + q) R;
        if constexpr (std::is_floating_point<R>::value) return (R)std::fmax((R)p, (R)q);
        else return (R)(p < q ? q : p);
    });
}
template <class A, class B> auto pow(const A& a, const B& b)
{
    return zip(a, b, [](auto p, auto q) { return std::pow((float)p, (float)q); });
}
template <class A, class B> auto atan2(const A& a, const B& b)
{
    return zip(a, b, [](auto p, auto q) { return std::atan2((float)p, (float)q); });
}
template <class A, class B> auto fmod(const A& a, const B& b)
{
    return zip(a, b, [](auto p, auto q) { return std::fmod((float)p, (float)q); });
}
template <class A, class B> auto step(const A& e, const B& x)
{
    return zip(e, x, [](auto p, auto q) { return q >= p ? 1.0f : 0.0f; });
}
template <class X, class L, class H> auto clamp(const X& x, const L& lo, const H& hi) { return min(max(x, lo), hi); }
template <class A, class B, class C> auto lerp(const A& a, const B& b, const C& t)
{
    auto d = nv(b) - nv(a);
    return nv(a) + nv(t) * d;
}
template <class A, class B, class X> auto smoothstep(const A& a, const B& b, const X& x)
{
    auto t = saturate((nv(x) - nv(a)) / (nv(b) - nv(a)));
    return t * t * (3.0f - 2.0f * t);
}
template <class A, class B> auto dot(const A& a0, const B& b0)
{
    auto a = nv(a0);
    auto b = nv(b0);
    auto s = a.v[0] * b.v[0];
    for (int k = 1; k < vt<decltype(a)>::n; ++k) s = s + a.v[k] * b.v[k];
    return s;
}
template <class A, class B> auto cross(const A& a0, const B& b0)
{
    auto a = nv(a0);
    auto b = nv(b0);
    typedef typename vt<decltype(a)>::elem T;
    return vec<T, 3>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class A> auto length(const A& a) { return std::sqrt((float)dot(a, a)); }
template <class A, class B> auto distance(const A& a, const B& b) { return length(nv(a) - nv(b)); }
// the shape of DXC's lowering, x * rsqrt(dot(x, x)), with a correctly rounded reciprocal root
template <class A> auto normalize(const A& a0)
{
    auto a = nv(a0);
    return a * (1.0f / std::sqrt((float)dot(a, a)));
}
template <class I, class N> auto reflect(const I& i, const N& n) { return nv(i) - 2.0f * dot(n, i) * nv(n); }
template <class I, class N> auto refract(const I& i0, const N& n0, float eta)
{
    auto i = nv(i0);
    auto n = nv(n0);
    float c = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - c * c);
    if (k < 0.0f) return decltype(i)(0.0f);
    return eta * i - (eta * c + std::sqrt(k)) * n;
}
template <class A> bool any(const A& a0)
{
    auto a = nv(a0);
    if constexpr (vt<decltype(a)>::is)
    {
        for (int k = 0; k < vt<decltype(a)>::n; ++k)
            if (a.v[k]) return true;
        return false;
    }
    else return a != 0;
}
template <class A> bool all(const A& a0)
{
    auto a = nv(a0);
    if constexpr (vt<decltype(a)>::is)
    {
        for (int k = 0; k < vt<decltype(a)>::n; ++k)
            if (!a.v[k]) return false;
        return true;
    }
    else return a != 0;
}
template <class C, class A, class B> auto select(const C& c, const A& a, const B& b)
{
    auto cc = nv(c);
    if constexpr (vt<decltype(cc)>::is)
        return zip(zip(cc, a, [](auto p, auto q) { return p ? q : decltype(q)(0); }), zip(cc, b, [](auto p, auto q) {
                       return p ? decltype(q)(0) : q;
                   }), [](auto p, auto q) { return p + q; });
    else return cc ? nv(a) : decltype(nv(a))(nv(b));
}
template <class A, class S, class C> void sincos(const A& x, S& s, C& c)
{
    s = sin(x);
    c = cos(x);
}

// ---- bit casts and integer intrinsics
inline float asfloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float asfloat(int u) { float f; std::memcpy(&f, &u, 4); return f; }
inline float asfloat(float f) { return f; }
template <class A, enable_vec<A> = 0> auto asfloat(const A& a) { return each(a, [](auto x) { return asfloat(x); }); }
inline uint asuint(float f) { uint u; std::memcpy(&u, &f, 4); return u; }
inline uint asuint(int i) { return (uint)i; }
inline uint asuint(uint u) { return u; }
template <class A, enable_vec<A> = 0> auto asuint(const A& a) { return each(a, [](auto x) { return asuint(x); }); }
inline int asint(float f) { int u; std::memcpy(&u, &f, 4); return u; }
inline int asint(uint u) { return (int)u; }
template <class A, enable_vec<A> = 0> auto asint(const A& a) { return each(a, [](auto x) { return asint(x); }); }
inline uint reversebits(uint v)
{
    uint r = 0;
    for (int k = 0; k < 32; ++k) r |= ((v >> k) & 1u) << (31 - k);
    return r;
}
inline uint countbits(uint v) { return (uint)__builtin_popcount(v); }
inline int firstbithigh(uint v) { return v ? 31 - __builtin_clz(v) : -1; }
inline int firstbitlow(uint v) { return v ? __builtin_ctz(v) : -1; }
inline float f16tof32(uint h)
{
    uint s = (h >> 15) & 1u, e = (h >> 10) & 31u, m = h & 1023u;
    float v;
    if (e == 0) v = std::ldexp((float)m, -24);
    else if (e == 31) v = m ? std::numeric_limits<float>::quiet_NaN() : std::numeric_limits<float>::infinity();
    else v = std::ldexp((float)(m | 1024u), (int)e - 25);
    return s ? -v : v;
}
inline uint f32tof16(float f) // round to nearest even
{
    uint u = asuint(f), s = (u >> 16) & 0x8000u;
    float a = std::fabs(f);
    if (std::isnan(f)) return s | 0x7e00u;
    if (a >= 65520.0f) return s | 0x7c00u;
    if (a < 6.103515625e-05f) return s | (uint)std::nearbyint(a * 16777216.0f);
    int e;
    float m = std::frexp(a, &e); // a = m * 2^e, m in [0.5, 1)
    uint mant = (uint)std::nearbyint(m * 2048.0f); // 11 significant bits
    if (mant == 2048u) { mant = 1024u; ++e; }
    return s | ((uint)(e + 14) << 10) | (mant & 1023u);
}
template <class T> T NonUniformResourceIndex(T i) { return i; }

// ---- 3x3 matrices (row-major as HLSL's float3x3(r0, r1, r2))
struct float3x3
{
    float3 m[3];
    float3x3() = default;
    float3x3(const float3& a, const float3& b, const float3& c) { m[0] = a; m[1] = b; m[2] = c; }
    float3x3(float a, float b, float c, float d, float e, float f, float g, float h, float i)
    {
        m[0] = float3(a, b, c); m[1] = float3(d, e, f); m[2] = float3(g, h, i);
    }
    float3& operator[](int r) { return m[r]; }
    const float3& operator[](int r) const { return m[r]; }
};
inline float3 mul(const float3x3& M, const float3& v) { return float3(dot(M.m[0], v), dot(M.m[1], v), dot(M.m[2], v)); }
inline float3 mul(const float3& v, const float3x3& M)
{
    return float3(v.x * M.m[0].x + v.y * M.m[1].x + v.z * M.m[2].x, v.x * M.m[0].y + v.y * M.m[1].y + v.z * M.m[2].y,
                  v.x * M.m[0].z + v.y * M.m[1].z + v.z * M.m[2].z);
}
inline float3x3 transpose(const float3x3& M)
{
    return float3x3(M.m[0].x, M.m[1].x, M.m[2].x, M.m[0].y, M.m[1].y, M.m[2].y, M.m[0].z, M.m[1].z, M.m[2].z);
}
template <class A, enable_vec<A> = 0> float3 mul(const float3x3& M, const A& v) { return mul(M, float3(v)); }
template <class A, enable_vec<A> = 0> float3 mul(const A& v, const float3x3& M) { return mul(float3(v), M); }

// other matrix shapes (row-major rows of C floats); mul(M, v) and mul(v, M)
template <int R, int C> struct fmat
{
    vec<float, C> m[R];
    fmat() = default;
    template <class... Rows, typename std::enable_if<sizeof...(Rows) == R, int>::type = 0> fmat(const Rows&... rows)
    {
        int k = 0;
        ((m[k++] = vec<float, C>(rows)), ...);
    }
    vec<float, C>& operator[](int r) { return m[r]; }
    const vec<float, C>& operator[](int r) const { return m[r]; }
};
typedef fmat<4, 4> float4x4;
typedef fmat<3, 4> float3x4;
typedef fmat<4, 3> float4x3;
template <int R, int C> vec<float, R> mul(const fmat<R, C>& M, const vec<float, C>& v)
{
    vec<float, R> r;
    for (int i = 0; i < R; ++i) r.v[i] = dot(M.m[i], v);
    return r;
}
template <int R, int C> vec<float, C> mul(const vec<float, R>& v, const fmat<R, C>& M)
{
    vec<float, C> r;
    for (int j = 0; j < C; ++j)
    {
        float s = v.v[0] * M.m[0].v[j];
        for (int i = 1; i < R; ++i) s = s + v.v[i] * M.m[i].v[j];
        r.v[j] = s;
    }
    return r;
}

// ---- resources read by the shader math
struct SamplerState
{
};
// Filtered reads: texel centres at (i + 0.5) / size, clamp to edge, FP32 weights.
inline void texAxis(float u, int n, int& i0, int& i1, float& t)
{
    float x = u * (float)n - 0.5f;
    float f = std::floor(x);
    t = x - f;
    i0 = std::min(std::max((int)f, 0), n - 1);
    i1 = std::min(std::max((int)f + 1, 0), n - 1);
}
struct Texture1D
{
    const float4* texels = nullptr;
    int w = 0;
    float4 SampleLevel(const SamplerState&, float u, float) const
    {
        int i0, i1;
        float t;
        texAxis(u, w, i0, i1, t);
        return texels[i0] + t * (texels[i1] - texels[i0]);
    }
    float4 Load(int2 c) const { return texels[c.x]; }
    void GetDimensions(float& ow) const { ow = (float)w; }
    void GetDimensions(uint& ow) const { ow = (uint)w; }
};
struct Texture2D
{
    const float4* texels = nullptr;
    int w = 0, h = 0;
    float4 at(int x, int y) const { return texels[y * w + x]; }
    float4 SampleLevel(const SamplerState&, float2 uv, float) const
    {
        int x0, x1, y0, y1;
        float tx, ty;
        texAxis(uv.x, w, x0, x1, tx);
        texAxis(uv.y, h, y0, y1, ty);
        float4 a = at(x0, y0) + tx * (at(x1, y0) - at(x0, y0));
        float4 b = at(x0, y1) + tx * (at(x1, y1) - at(x0, y1));
        return a + ty * (b - a);
    }
    float4 Load(int3 c) const { return at(c.x, c.y); }
    void GetDimensions(uint& ow, uint& oh) const { ow = (uint)w; oh = (uint)h; }
    void GetDimensions(float& ow, float& oh) const { ow = (float)w; oh = (float)h; }
};
struct Texture3D
{
    const float4* texels = nullptr;
    int w = 0, h = 0, d = 0;
    float4 at(int x, int y, int z) const { return texels[(z * h + y) * w + x]; }
    float4 SampleLevel(const SamplerState&, float3 uvw, float) const
    {
        int x0, x1, y0, y1, z0, z1;
        float tx, ty, tz;
        texAxis(uvw.x, w, x0, x1, tx);
        texAxis(uvw.y, h, y0, y1, ty);
        texAxis(uvw.z, d, z0, z1, tz);
        auto plane = [&](int z) {
            float4 a = at(x0, y0, z) + tx * (at(x1, y0, z) - at(x0, y0, z));
            float4 b = at(x0, y1, z) + tx * (at(x1, y1, z) - at(x0, y1, z));
            return a + ty * (b - a);
        };
        float4 p0 = plane(z0), p1 = plane(z1);
        return p0 + tz * (p1 - p0);
    }
    void GetDimensions(float& ow, float& oh, float& od) const { ow = (float)w; oh = (float)h; od = (float)d; }
    void GetDimensions(uint& ow, uint& oh, uint& od) const { ow = (uint)w; oh = (uint)h; od = (uint)d; }
};
struct TextureCube
{
    float4 SampleLevel(const SamplerState&, float3, float) const { return float4(0.0f); }
};
template <class T> struct StructuredBuffer
{
    const T* data = nullptr;
    const T& operator[](uint i) const { return data[i]; }
};
template <class T> struct RWStructuredBuffer
{
    T* data = nullptr;
    T& operator[](uint i) const { return data[i]; }
};
// Raw buffer; reads past the end return 0, as DX12 does for a bound buffer.
struct ByteAddressBuffer
{
    const uint8_t* data = nullptr;
    uint bytes = 0;
    uint Load(uint a) const
    {
        if ((uint64_t)a + 4 > bytes) return 0u;
        uint v;
        std::memcpy(&v, data + a, 4);
        return v;
    }
    uint2 Load2(uint a) const { return uint2(Load(a), Load(a + 4)); }
    uint3 Load3(uint a) const { return uint3(Load(a), Load(a + 4), Load(a + 8)); }
    uint4 Load4(uint a) const { return uint4(Load(a), Load(a + 4), Load(a + 8), Load(a + 12)); }
};
template <class T> struct ConstantBuffer : T
{
};
} // namespace HLSL_SHIM_NS
