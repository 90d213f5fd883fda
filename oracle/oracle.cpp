// CPU oracle: scalar C++ restatement of YAPT's uni / NEE integrator shaders.
// TEST INFRASTRUCTURE ONLY (see oracle.h). Templated on the scalar type T:
//   T = float : the same operation sequence as the reference shaders in FP32, for
//               per-sample parity; transcendental functions from yapt_fmath.h so that
//               every platform computes the same bits.
//   T = double: the FP64 reference used to judge converged images (relMSE).
// Reference files followed (paths inside the YAPT tree, Source/Renderer/shaders/):
//   raytracing/rayGenPrimaryRays.hlsl, rayHitDefault.hlsl, rayMissEnvironment.hlsl,
//   payload.hlsl, hitShadersCommon.hlsl, raytraceCommonResources.hlsl, lightSampling.hlsl,
//   materialSample.hlsl, scatteringSample.hlsl, spectralDistribution.hlsl,
//   materials/materialsCommon.hlsl, materialLayers.hlsl,
//   common/bsdfSample.hlsl, ggx.hlsl, fresnel.hlsl, multiScatter.hlsl, miscBrdf.hlsl,
//   commonMath.hlsl, common.hlsl, random.hlsl, randomSampler.hlsl, surfaceParameters.hlsl;
// host: RaytraceCommonResources.cpp:325-547 (light pdfs, alias table),
//   BindlessMaterialManager.cpp:73-98 (material clamps), Tools/generate_sobol_matrices.py.
#include "oracle.h"

#include "../include/yapt_fmath.h"
#include "../yapt_gb300/csrc/yg_tables.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <limits>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace orc
{

// ------------------------------------------------------------------ math traits
template <typename T>
struct Mth;
template <>
struct Mth<float>
{
    static float sqrt(float x) { return std::sqrt(x); }
    static void sincos(float x, float& s, float& c) { ygm_sincosf(x, &s, &c); }
    static float cos(float x) { return ygm_cosf(x); }
    static float exp(float x) { return ygm_expf(x); }
    static float log(float x) { return ygm_logf(x); }
    static float pow(float x, float y) { return ygm_powf(x, y); }
};
template <>
struct Mth<double>
{
    static double sqrt(double x) { return std::sqrt(x); }
    static void sincos(double x, double& s, double& c)
    {
        s = std::sin(x);
        c = std::cos(x);
    }
    static double cos(double x) { return std::cos(x); }
    static double exp(double x) { return std::exp(x); }
    static double log(double x) { return std::log(x); }
    static double pow(double x, double y) { return std::pow(x, y); }
};

template <typename T>
struct V3
{
    T x, y, z;
};
template <typename T> V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <typename T> V3<T> operator+(V3<T> a, V3<T> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> V3<T> operator-(V3<T> a, V3<T> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> V3<T> operator-(V3<T> a) { return v3(-a.x, -a.y, -a.z); }
template <typename T> V3<T> operator*(V3<T> a, T s) { return v3(a.x * s, a.y * s, a.z * s); }
template <typename T> V3<T> operator/(V3<T> a, T s) { return v3(a.x / s, a.y / s, a.z / s); }
template <typename T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename T> V3<T> cross(V3<T> a, V3<T> b)
{
    return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <typename T> T len(V3<T> v) { return Mth<T>::sqrt(dot(v, v)); }
template <typename T> V3<T> normalize(V3<T> v)
{
    T inv = T(1) / Mth<T>::sqrt(dot(v, v));
    return v * inv;
}
template <typename T> bool isZero(V3<T> v) { return v.x == 0 && v.y == 0 && v.z == 0; }

// SpectralSamples: four hero-wavelength lanes (spectralDistribution.hlsl:85-403)
template <typename T>
struct S4
{
    T v[4];
    T& operator[](int i) { return v[i]; }
    T operator[](int i) const { return v[i]; }
};
template <typename T> S4<T> sp(T a) { return S4<T>{{a, a, a, a}}; }
template <typename T> S4<T> operator+(const S4<T>& a, const S4<T>& b) { S4<T> r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] + b.v[i]; return r; }
template <typename T> S4<T> operator*(const S4<T>& a, const S4<T>& b) { S4<T> r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * b.v[i]; return r; }
template <typename T> S4<T> operator*(const S4<T>& a, T s) { S4<T> r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] * s; return r; }
template <typename T> S4<T> operator/(const S4<T>& a, T s) { S4<T> r; for (int i = 0; i < 4; ++i) r.v[i] = a.v[i] / s; return r; }
template <typename T> bool allEq(const S4<T>& a, T s) { return a.v[0] == s && a.v[1] == s && a.v[2] == s && a.v[3] == s; }

template <typename T> T sqr(T x) { return x * x; }
template <typename T> T tmin(T a, T b) { return std::fmin(a, b); }
template <typename T> T tmax(T a, T b) { return std::fmax(a, b); }
template <typename T> T saturate(T x) { return tmin(tmax(x, T(0)), T(1)); }
template <typename T> T clampT(T x, T lo, T hi) { return tmin(tmax(x, lo), hi); }
template <typename T> T lerpT(T a, T b, T t) { return a + t * (b - a); }
template <typename T> T safeDiv(T n, T d) { return d == T(0) ? T(0) : n / d; }

template <typename T> struct C
{
    static constexpr T PI = T(3.14159265f);
    static constexpr T INVPI = T(0.31830988f);
    static constexpr T PI_OVER_2 = T(1.57079633f);
    static constexpr T PI_OVER_4 = T(0.785398163f);
};

// HLSL reflect / refract
template <typename T> V3<T> reflect(V3<T> i, V3<T> n) { return i - n * (T(2) * dot(n, i)); }
template <typename T> V3<T> refract(V3<T> i, V3<T> n, T eta)
{
    T ni = dot(n, i);
    T k = T(1) - eta * eta * (T(1) - ni * ni);
    if (k < T(0)) return v3<T>(0, 0, 0);
    return i * eta - n * (eta * ni + Mth<T>::sqrt(k));
}

// float3x3(t, n, b) rows (constructBasisTransform, commonMath.hlsl:128-133)
// IEEE binary32 -> binary16, round to nearest, ties to even (HLSL f32tof16); subnormal
// halves kept, overflow to infinity.
inline uint16_t halfFromFloat(float f)
{
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    x &= 0x7fffffffu;
    if (x >= 0x7f800000u) return (uint16_t)(sign | (x > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (x >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u); // >= 65520 rounds past the largest half
    if (x >= 0x38800000u)                                   // normal half
    {
        uint32_t h = (((x >> 23) - 112u) << 10) | ((x & 0x7fffffu) >> 13);
        const uint32_t rem = x & 0x1fffu;
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
        return (uint16_t)(sign | h);
    }
    if (x < 0x33000000u) return (uint16_t)sign; // below half of the smallest subnormal
    const uint32_t e = x >> 23, mant = (x & 0x7fffffu) | 0x800000u, shift = 126u - e;
    uint32_t h = mant >> shift;
    const uint32_t rem = mant & ((1u << shift) - 1u), halfway = 1u << (shift - 1u);
    if (rem > halfway || (rem == halfway && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

inline float floatFromHalf(uint16_t h)
{
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t x;
    if (e == 0x1fu)
        x = sign | 0x7f800000u | (m << 13);
    else if (e != 0)
        x = sign | ((e + 112u) << 23) | (m << 13);
    else if (m == 0)
        x = sign;
    else
    {
        // subnormal: m * 2^-24, exact in binary32
        float v = (float)m * 5.9604644775390625e-08f;
        std::memcpy(&x, &v, 4);
        x |= sign;
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

template <typename T>
struct Basis
{
    V3<T> t, n, b;
};
template <typename T> Basis<T> basis(V3<T> n, V3<T> t)
{
    Basis<T> B;
    B.t = normalize(t - n * dot(n, t));
    B.n = n;
    B.b = cross(B.t, n);
    return B;
}
template <typename T> V3<T> mulMv(const Basis<T>& B, V3<T> v) { return v3(dot(B.t, v), dot(B.n, v), dot(B.b, v)); }
template <typename T> V3<T> mulvM(V3<T> v, const Basis<T>& B)
{
    return v3(v.x * B.t.x + v.y * B.n.x + v.z * B.b.x, v.x * B.t.y + v.y * B.n.y + v.z * B.b.y,
              v.x * B.t.z + v.y * B.n.z + v.z * B.b.z);
}
template <typename T> V3<T> xPoint(const float* m, V3<T> p)
{
    return v3(T(m[0]) * p.x + T(m[1]) * p.y + T(m[2]) * p.z + T(m[3]), T(m[4]) * p.x + T(m[5]) * p.y + T(m[6]) * p.z + T(m[7]),
              T(m[8]) * p.x + T(m[9]) * p.y + T(m[10]) * p.z + T(m[11]));
}
template <typename T> V3<T> xVec(const float* m, V3<T> v)
{
    return v3(T(m[0]) * v.x + T(m[1]) * v.y + T(m[2]) * v.z, T(m[4]) * v.x + T(m[5]) * v.y + T(m[6]) * v.z,
              T(m[8]) * v.x + T(m[9]) * v.y + T(m[10]) * v.z);
}
template <typename T> V3<T> xVecT(const float* m, V3<T> v)
{
    return v3(v.x * T(m[0]) + v.y * T(m[4]) + v.z * T(m[8]), v.x * T(m[1]) + v.y * T(m[5]) + v.z * T(m[9]),
              v.x * T(m[2]) + v.y * T(m[6]) + v.z * T(m[10]));
}
template <typename T> void mul44(const float* m, const T* v, T* o)
{
    for (int r = 0; r < 4; ++r) o[r] = T(m[4 * r]) * v[0] + T(m[4 * r + 1]) * v[1] + T(m[4 * r + 2]) * v[2] + T(m[4 * r + 3]) * v[3];
}

// ------------------------------------------------------------------ sampler (random.hlsl, randomSampler.hlsl)
inline uint32_t reverseBits(uint32_t v)
{
    uint32_t r = 0;
    for (int i = 0; i < 32; ++i)
    {
        r = (r << 1) | (v & 1u);
        v >>= 1;
    }
    return r;
}
inline uint32_t murmurFinal(uint32_t x)
{
    x ^= x >> 16;
    x *= 0x85ebca6bu;
    x ^= x >> 13;
    x *= 0xc2b2ae35u;
    x ^= x >> 16;
    return x;
}
inline uint32_t hashAB(uint32_t a, uint32_t b) { return murmurFinal(((a + b) * (a + b + 1u)) / (2u + b)); }
inline uint32_t owenFast(uint32_t v, uint32_t seed)
{
    v = reverseBits(v);
    v ^= v * 0x3d20adeau;
    v += seed;
    v *= (seed >> 16) | 1u;
    v ^= v * 0x05526c56u;
    v ^= v * 0x53a22864u;
    return reverseBits(v);
}
inline float toFloat01(uint32_t r) { return std::fmin((float)r * 0x1p-32f, 0x1.fffffep-1f); }

struct Sampler
{
    const uint32_t* point; // 256 Sobol values for this sample index
    uint32_t dim;
    uint32_t seed;
    float get(uint32_t d) const
    {
        uint32_t s = d < 256u ? point[d] : 0u; // out-of-range reads are 0 on DX12
        return toFloat01(owenFast(s, hashAB(seed, d)));
    }
    float r1() { float v = get(dim); dim += 1; return v; }
};

// ------------------------------------------------------------------ tables
struct Tables
{
    std::vector<double> cie; // 471 x 4
    std::vector<uint32_t> sobol;
    int lmin, lmax;
    double ySum, d65Sum;
};

bool loadCie(const std::string& dir, std::vector<double>& cie)
{
    std::ifstream f(dir + "/cie1931_2deg_d65_1nm.txt");
    if (!f) return false;
    std::string line;
    while (std::getline(f, line))
    {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        double l, x, y, z, d;
        if (is >> l >> x >> y >> z >> d)
        {
            cie.push_back(x);
            cie.push_back(y);
            cie.push_back(z);
            cie.push_back(d);
        }
    }
    return cie.size() == 471 * 4;
}

// Sobol generator matrices, Tools/generate_sobol_matrices.py:37-90
bool sobolMatrices(const std::string& dir, std::vector<uint32_t>& m)
{
    std::ifstream f(dir + "/joe_kuo_6_21201_first256.txt");
    if (!f) return false;
    m.assign(256 * 32, 0);
    for (int j = 0; j < 32; ++j) m[j] = 1u << (31 - j);
    std::string line;
    int dim = 1;
    while (dim < 256 && std::getline(f, line))
    {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        int d, s, a;
        if (!(is >> d >> s >> a)) continue;
        std::vector<uint32_t> mi(s);
        for (int i = 0; i < s; ++i) is >> mi[i];
        uint32_t V[32];
        for (int i = 0; i < 32; ++i)
        {
            if (i < s) V[i] = mi[i] << (31 - i);
            else
            {
                V[i] = V[i - s] ^ (V[i - s] >> s);
                for (int k = 1; k < s; ++k)
                    if ((a >> (s - 1 - k)) & 1) V[i] ^= V[i - k];
            }
        }
        std::memcpy(&m[dim * 32], V, sizeof(V));
        ++dim;
    }
    return dim == 256;
}
inline uint32_t sobolUint(const std::vector<uint32_t>& m, uint32_t index, uint32_t dim)
{
    uint32_t v = 0;
    for (uint32_t i = dim * 32; index != 0; index >>= 1, ++i)
        if (index & 1) v ^= m[i];
    return v;
}

// ------------------------------------------------------------------ the integrator (templated)
template <typename T>
struct Ctx
{
    const oracle_scene* sc;
    const Tables* tb;
    std::vector<T> cieT; // per nm in [lmin, lmax]: x y z d65
    T ySumInv, d65SumInv;
    T lmin, lmax;
    // lights
    struct Light
    {
        uint32_t inst;
        float pdf, thr;
        uint32_t alias;
        // punctual lights (type != 0): their own table over the punctual lights alone
        uint32_t type;
        float ppdf, pthr;
        uint32_t palias;
        float pos[3], dir[3], inten[3], cosIn, cosOut;
    };
    uint32_t nPunctual = 0;
    std::vector<Light> lights;
    // textures decoded to linear float RGBA (yg_upload_texture)
    std::vector<std::vector<float>> tex;
    std::vector<uint32_t> texW, texH;
    std::vector<float> instLightPdf;
    // world triangles and BVH
    struct Tri
    {
        V3<float> v0, e1, e2;
        uint32_t inst, prim;
    };
    std::vector<Tri> tris;
    struct Node
    {
        float lo[3], hi[3];
        int left, right; // child nodes, or -1
        int first, count; // leaf range
    };
    std::vector<Node> nodes;
    std::vector<uint32_t> triIdx;
    float wlo[3] = {INFINITY, INFINITY, INFINITY}, whi[3] = {-INFINITY, -INFINITY, -INFINITY}; // world bounds
};

// LUT read with the texel-centre remap of sampleLUT (materialsCommonResources.hlsl:132-169):
// coordinate u addresses texel u*(dim-1), linear filtering, clamped.
template <typename T> void lutIdx(T u, int dim, int& i, T& t)
{
    T x = clampT(u * T(dim - 1), T(0), T(dim - 1));
    int k = (int)x;
    if (k > dim - 2) k = dim - 2;
    i = k;
    t = x - T(k);
}
template <typename T> T lut1(const float* L, int d, T u)
{
    int i; T t;
    lutIdx(u, d, i, t);
    return lerpT(T(L[i]), T(L[i + 1]), t);
}
template <typename T> T lut2(const float* L, int d, T u, T v)
{
    int i, j; T tx, ty;
    lutIdx(u, d, i, tx);
    lutIdx(v, d, j, ty);
    T a = lerpT(T(L[j * d + i]), T(L[j * d + i + 1]), tx);
    T b = lerpT(T(L[(j + 1) * d + i]), T(L[(j + 1) * d + i + 1]), tx);
    return lerpT(a, b, ty);
}
template <typename T> T lut3(const float* L, int d, T u, T v, T w)
{
    int k; T tz;
    lutIdx(w, d, k, tz);
    T a = lut2(L + k * d * d, d, u, v);
    T b = lut2(L + (k + 1) * d * d, d, u, v);
    return lerpT(a, b, tz);
}

template <typename T>
struct Spec
{
    T hero;
    T lam[4];
};

template <typename T> void cieAt(const Ctx<T>& c, T lambda, T out[4])
{
    T u = (lambda - c.lmin) / (c.lmax - c.lmin);
    int n = (int)(c.cieT.size() / 4);
    int i; T t;
    lutIdx(u, n, i, t);
    for (int k = 0; k < 4; ++k) out[k] = lerpT(c.cieT[4 * i + k], c.cieT[4 * (i + 1) + k], t);
}

template <typename T> T sigmoid(T x)
{
    if (std::isinf(x)) return x > 0 ? T(1) : T(0);
    return T(0.5f) * x / Mth<T>::sqrt(T(1) + x * x) + T(0.5f);
}
template <typename T> T sigmoidInv(T x)
{
    if (x == T(1)) return std::numeric_limits<T>::infinity();
    if (x == T(0)) return -std::numeric_limits<T>::infinity();
    return (x - T(0.5f)) / Mth<T>::sqrt(x * (T(1) - x));
}
template <typename T> S4<T> withCoeffs(const Ctx<T>& c, const Spec<T>& s, V3<T> k)
{
    S4<T> r;
    for (int i = 0; i < 4; ++i)
    {
        T l = (s.lam[i] - c.lmin) / (c.lmax - c.lmin);
        T poly = k.x * l * l + k.y * l + k.z;
        r[i] = sigmoid(poly);
    }
    return r;
}
template <typename T> V3<T> rgbCoeffs(const Ctx<T>& c, V3<T> rgb)
{
    const int R = 64;
    const float* L = c.sc->rgb_to_spd;
    int i, j, k; T tx, ty, tz;
    lutIdx(rgb.x, R, i, tx);
    lutIdx(rgb.y, R, j, ty);
    lutIdx(rgb.z, R, k, tz);
    T o[3];
    for (int ch = 0; ch < 3; ++ch)
    {
        auto at = [&](int x, int y, int z) { return T(L[((size_t)((z * R + y) * R + x)) * 3 + ch]); };
        T a = lerpT(lerpT(at(i, j, k), at(i + 1, j, k), tx), lerpT(at(i, j + 1, k), at(i + 1, j + 1, k), tx), ty);
        T b = lerpT(lerpT(at(i, j, k + 1), at(i + 1, j, k + 1), tx), lerpT(at(i, j + 1, k + 1), at(i + 1, j + 1, k + 1), tx), ty);
        o[ch] = lerpT(a, b, tz);
    }
    return v3(o[0], o[1], o[2]);
}
// setFromRGB (spectralDistribution.hlsl:183-202)
template <typename T> S4<T> setFromRGB(const Ctx<T>& c, const Spec<T>& s, V3<T> v)
{
    V3<T> k;
    if (v.x == v.y && v.x == v.z) k = v3(T(0), T(0), sigmoidInv(v.x));
    else k = rgbCoeffs(c, v);
    return withCoeffs(c, s, k);
}
template <typename T> S4<T> setFromRGBUnboundedNoIllum(const Ctx<T>& c, const Spec<T>& s, V3<T> v)
{
    T m = tmax(tmax(v.x, v.y), v.z);
    T scale = T(2) * m;
    V3<T> d = scale == T(0) ? v3(T(0), T(0), T(0)) : v / scale;
    return setFromRGB(c, s, d) * scale;
}
template <typename T> S4<T> setFromRGBUnbounded(const Ctx<T>& c, const Spec<T>& s, V3<T> v)
{
    S4<T> r = setFromRGBUnboundedNoIllum(c, s, v);
    for (int i = 0; i < 4; ++i)
    {
        T cc[4];
        cieAt(c, s.lam[i], cc);
        r[i] = r[i] * (cc[3] * c.d65SumInv * T(100));
    }
    return r;
}
template <typename T> S4<T> curve(const Ctx<T>& c, const Spec<T>& s, int id)
{
    const float* cv = c.sc->spectra + (size_t)id * c.sc->spec_points;
    S4<T> r;
    for (int i = 0; i < 4; ++i)
    {
        T u = (s.lam[i] - T(c.sc->spec_lmin)) / (T(c.sc->spec_lmax) - T(c.sc->spec_lmin));
        int k; T t;
        lutIdx(u, (int)c.sc->spec_points, k, t);
        r[i] = lerpT(T(cv[k]), T(cv[k + 1]), t);
    }
    return r;
}
template <typename T> S4<T> reflectance(const Ctx<T>& c, const Spec<T>& s, const float* rgb, int id)
{
    if (id >= 0) return curve(c, s, id);
    return setFromRGB(c, s, v3(T(rgb[0]), T(rgb[1]), T(rgb[2])));
}
template <typename T> S4<T> emission(const Ctx<T>& c, const Spec<T>& s, const float* rgb, int id)
{
    if (id >= 0) return curve(c, s, id) * T(std::fmax(std::fmax(rgb[0], rgb[1]), rgb[2]));
    if (rgb[0] == 0 && rgb[1] == 0 && rgb[2] == 0) return sp(T(0));
    return setFromRGBUnbounded(c, s, v3(T(rgb[0]), T(rgb[1]), T(rgb[2])));
}

// ToXYZ (spectralDistribution.hlsl:345-365)
template <typename T> V3<T> toXYZ(const Ctx<T>& c, const Spec<T>& s, const S4<T>& L)
{
    T pdf = T(1) / (c.lmax - c.lmin);
    T k = safeDiv(c.ySumInv, pdf);
    V3<T> acc = v3(T(0), T(0), T(0));
    for (int i = 0; i < 4; ++i)
    {
        T cc[4];
        cieAt(c, s.lam[i], cc);
        acc = acc + v3(L[i] * cc[0], L[i] * cc[1], L[i] * cc[2]) * k;
    }
    return acc / T(4);
}

// ------------------------------------------------------------------ BSDF pieces
template <typename T> T jRefl(V3<T> wi, V3<T> wm) { return safeDiv(T(1), T(4) * saturate(dot(wi, wm))); }
template <typename T> T jRefr(T eta, V3<T> wo, V3<T> wm, V3<T> wi)
{
    T mo = dot(wo, wm), mi = dot(wi, wm);
    return safeDiv(std::fabs(mi), sqr(mo / eta + mi));
}
template <typename T> bool sameHemi(V3<T> r, V3<T> d) { return r.y * d.y >= T(0); }
template <typename T> V3<T> forceHemi(V3<T> r, V3<T> d) { return sameHemi(r, d) ? d : -d; }
template <typename T> void concentricDisk(T ux, T uy, T& ox, T& oy)
{
    T sx = T(2) * ux - T(1), sy = T(2) * uy - T(1);
    if (sx == 0 && sy == 0)
    {
        ox = oy = 0;
        return;
    }
    T theta, r;
    if (std::fabs(sx) > std::fabs(sy))
    {
        r = sx;
        theta = C<T>::PI_OVER_4 * (sy / sx);
    }
    else
    {
        r = sy;
        theta = C<T>::PI_OVER_2 - C<T>::PI_OVER_4 * (sx / sy);
    }
    T s, co;
    Mth<T>::sincos(theta, s, co);
    ox = r * co;
    oy = r * s;
}
template <typename T> V3<T> cosHemi(T rx, T ry)
{
    T y = Mth<T>::sqrt(T(1) - rx), r = Mth<T>::sqrt(rx), phi = T(2) * C<T>::PI * ry, s, co;
    Mth<T>::sincos(phi, s, co);
    return v3(r * co, y, r * s);
}
template <typename T> T pdfCosHemi(T d) { return saturate(d) * C<T>::INVPI; }
template <typename T> T emissionProfile(T d, T e)
{
    T p = e > T(0) ? Mth<T>::pow(std::fabs(d), e) : T(1);
    return (e + T(2)) * T(0.5f) * p;
}
template <typename T> T glSheen(T x, T a, T b, T c, T d, T e) { return (a / (T(1) + b * Mth<T>::pow(x, c))) + d * x + e; }
template <typename T> T glambdaSheen(T r, T ct)
{
    T t = T(1) - r;
    t *= t;
    T a = lerpT(T(21.5473f), T(25.3245f), t), b = lerpT(T(3.82987f), T(3.32435f), t), c = lerpT(T(0.19823f), T(0.16801f), t);
    T d = lerpT(T(-1.97760f), T(-1.27393f), t), e = lerpT(T(-4.32054f), T(-4.85967f), t);
    T ex = ct < T(0.5f) ? glSheen(ct, a, b, c, d, e) : T(2) * glSheen(T(0.5f), a, b, c, d, e) - glSheen(T(1) - ct, a, b, c, d, e);
    return Mth<T>::exp(ex);
}
template <typename T> T DSheen(V3<T> wm, T r)
{
    T ri = T(1) / r;
    T s2 = tmax(T(1) - wm.y * wm.y, T(0.0001f));
    return (T(2) + ri) * Mth<T>::pow(s2, ri * T(0.5f)) / (T(2) * C<T>::PI);
}
template <typename T> T GSheen(V3<T> wo, V3<T> wi, T r) { return T(1) / (T(1) + glambdaSheen(r, wi.y) + glambdaSheen(r, wo.y)); }
template <typename T> T lambdaGGX(V3<T> d, T ax, T ay)
{
    T s = T(1) + (d.x * d.x * (ax * ax) + d.z * d.z * (ay * ay)) / (d.y * d.y);
    return (Mth<T>::sqrt(s) - T(1)) * T(0.5f);
}
template <typename T> T G1(V3<T> wo, V3<T> wm, T ax, T ay) { return (dot(wo, wm) >= T(0) ? T(1) : T(0)) / (T(1) + lambdaGGX(wo, ax, ay)); }
template <typename T> T G2(V3<T> wo, V3<T> wi, V3<T> wm, T ax, T ay)
{
    T li = lambdaGGX(wi, ax, ay), lo = lambdaGGX(wo, ax, ay);
    return T(1) / (T(1) + li + lo);
}
template <typename T> T DGGX(V3<T> wm, T ax, T ay)
{
    T d = sqr(wm.x / ax) + sqr(wm.z / ay) + sqr(wm.y);
    d *= d;
    d *= ax * ay * C<T>::PI;
    return safeDiv(T(1), d);
}
template <typename T> V3<T> vndf(V3<T> wo, T ax, T ay, T u1, T u2)
{
    V3<T> Vh = normalize(v3(ax * wo.x, ay * wo.z, wo.y));
    T lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    V3<T> T1 = lensq > 0 ? v3(-Vh.y, Vh.x, T(0)) * (T(1) / Mth<T>::sqrt(lensq)) : v3(T(1), T(0), T(0));
    V3<T> T2 = cross(Vh, T1);
    T r = Mth<T>::sqrt(u1), phi = T(2) * C<T>::PI * u2, s, co;
    Mth<T>::sincos(phi, s, co);
    T t1 = r * co, t2 = r * s;
    T sh = T(0.5f) * (T(1) + Vh.z);
    t2 = (T(1) - sh) * Mth<T>::sqrt(T(1) - t1 * t1) + sh * t2;
    V3<T> Nh = T1 * t1 + T2 * t2 + Vh * Mth<T>::sqrt(tmax(T(0), T(1) - t1 * t1 - t2 * t2));
    return normalize(v3(ax * Nh.x, tmax(T(0), Nh.z), ay * Nh.y));
}
template <typename T> T DV(V3<T> wo, V3<T> wm, T ax, T ay)
{
    T D = DGGX(wm, ax, ay), g1 = G1(wo, wm, ax, ay);
    return safeDiv(g1 * std::fabs(dot(wo, wm)) * D, std::fabs(wo.y));
}
template <typename T> V3<T> sampleWM(V3<T> wo, T ax, T ay, T u1, T u2)
{
    bool flip = wo.y < 0;
    wo.y = std::fabs(wo.y);
    V3<T> wh = vndf(wo, ax, ay, u1, u2);
    if (flip)
    {
        wo.y = -wo.y;
        wh.y = -wh.y;
    }
    return forceHemi(wo, wh);
}
// fresnel.hlsl
template <typename T> void conductorNK2(T r, T g, T& n, T& k2)
{
    T rc = clampT(r, T(0), T(0.99f));
    T sq = Mth<T>::sqrt(rc);
    n = g * ((T(1) - rc) / (T(1) + rc)) + (T(1) - g) * ((T(1) + sq) / (T(1) - sq));
    T nr = (n + T(1)) * (n + T(1)) * rc - (n - T(1)) * (n - T(1));
    k2 = nr / (T(1) - rc);
}
template <typename T> T fresnelDC(T er, T ei, T ct)
{
    T c2 = ct * ct, s2 = T(1) - c2, er2 = er * er, ei2 = ei * ei;
    T t0 = er2 - ei2 - s2;
    T a2b2 = Mth<T>::sqrt(er2 * ei2 * T(4) + t0 * t0);
    T t1 = a2b2 + c2;
    T a = Mth<T>::sqrt((a2b2 + t0) * T(0.5f));
    T t2 = a * c2 * T(2);
    T rs = (t1 - t2) / (t1 + t2);
    T t3 = a2b2 + s2 * s2 * c2;
    T t4 = t2 * s2;
    T rp = rs * (t3 - t4) / (t3 + t4);
    return (rp + rs) * T(0.5f);
}
template <typename T> T fresnelDD(T eta, T ct)
{
    T c = saturate(ct);
    T temp = eta * eta + c * c - T(1);
    if (temp < T(0)) return T(1);
    T g = Mth<T>::sqrt(temp);
    return T(0.5f) * sqr((g - c) / tmax(g + c, T(0.00001f))) * (T(1) + sqr(((g + c) * c - T(1)) / ((g - c) * c + T(1))));
}
template <typename T> bool deltaGGX(T ax, T ay) { return tmax(ax, ay) < T(0.002f); }
template <typename T> bool deltaGGX1(T r) { return r < T(0.002f); }
template <typename T> bool deltaSheen(T r) { return r < T(0.01f); }
template <typename T> void roughParams(T r, T aniso, T& ax, T& ay)
{
    T a2 = r * r;
    ax = clampT(a2 * (T(1) + aniso), T(0), T(1));
    ay = clampT(a2 * (T(1) - aniso), T(0), T(1));
}

template <typename T>
struct LutSet
{
    const float* L[9];
    T ssNoF(T c, T r) const { return lut2(L[0], 32, c, r); }
    T ssms(T eta, T c, T r) const { return lut3(L[2], 16, c, r, saturate((eta - T(1)) * T(0.333333f))); }
    T trL(T eta, T c, T r) const { return lut3(L[5], 16, c, r, saturate((eta - T(0.3f)) * (T(1) / T(0.69f)))); }
    T trD(T eta, T c, T r) const { return lut3(L[4], 16, c, r, saturate((eta - T(1)) * T(0.333333f))); }
    T sheen(T c, T r) const { return lut2(L[8], 16, c, saturate(r - T(0.07f))); }
    T ssAvg(T r) const { return lut1(L[1], 32, r); }
    T trAvgL(T eta, T r) const { return lut2(L[7], 16, r, saturate((eta - T(0.3f)) * (T(1) / T(0.69f)))); }
    T trAvgD(T eta, T r) const { return lut2(L[6], 16, r, saturate((eta - T(1)) * T(0.333333f))); }
};
// multiScatter.hlsl (Turquin variant: RECIPROCAL_MULTISCATTER is off for uni/NEE)
template <typename T> T dirAlbedoTrans(const LutSet<T>& L, T eta, T d, T lr)
{
    return eta < T(1) ? L.trL(eta, std::fabs(d), lr) : L.trD(eta, std::fabs(d), lr);
}
template <typename T> T energyComp(const LutSet<T>& L, T fms, T dWo, T dWi, T lr, T ss)
{
    T dw = L.ssNoF(std::fabs(std::fabs(dWo)), lr);
    T comp = fms * (T(1) - dw) / dw;
    return ss * comp;
}
template <typename T> T energyAfterSpec(const LutSet<T>& L, T eta, T dWo, T lr, T amount)
{
    return T(1) - L.ssms(eta, std::fabs(dWo), lr) * amount;
}
template <typename T> T energyCompTrans(const LutSet<T>& L, T eta, T dWo, T lr, T ss)
{
    T d = tmax(dirAlbedoTrans(L, eta, std::fabs(dWo), lr), T(0.1f));
    return (ss / d) - ss;
}
// Kulla-Conty variant (RECIPROCAL_MULTISCATTER, which BDPTCommon.hlsl:6 switches on):
// getAvgFresnel, getAverageAlbedoTranslucent, getMsTransmissionRatio,
// getEnergyCompensationKulla, getEnergyCompensationTranslucentKulla (multiScatter.hlsl:93-213)
template <typename T> T avgFresnel(T eta)
{
    if (eta < T(1)) return T(0.997118f) + T(0.1014f) * eta - T(0.965241f) * eta * eta - T(0.130607f) * eta * eta * eta;
    return (eta - T(1)) / (T(4.08567f) + T(1.00071f) * eta);
}
template <typename T> T avgAlbedoTrans(const LutSet<T>& L, T eta, T lr) { return eta < T(1) ? L.trAvgL(eta, lr) : L.trAvgD(eta, lr); }
template <typename T> T msTransRatio(const LutSet<T>& L, T eta, T lr)
{
    T etaOut = tmax(eta, T(1) / eta);
    T tOut = T(1) - avgFresnel(etaOut);
    if (eta >= T(1)) return tOut;
    T eOut = avgAlbedoTrans(L, etaOut, lr);
    T eIn = avgAlbedoTrans(L, eta, lr);
    return saturate(safeDiv(tOut * (T(1) - eOut), etaOut * etaOut * (T(1) - eIn)));
}
template <typename T> T energyCompKulla(const LutSet<T>& L, T fms, T dWo, T dWi, T lr)
{
    T aWo = L.ssNoF(std::fabs(dWo), lr);
    T aWi = L.ssNoF(std::fabs(dWi), lr);
    T eAvg = L.ssAvg(lr);
    T ems = safeDiv((T(1) - aWo) * (T(1) - aWi), (T(1) - eAvg) * C<T>::PI);
    return fms * ems;
}
template <typename T> T energyCompTransKulla(const LutSet<T>& L, T eta, T dWo, T dWi, T lr)
{
    bool transmission = dWo * dWi < T(0);
    T ratioT = msTransRatio(L, eta, lr);
    T aWo, aWi, eAvg, ratio;
    if (transmission)
    {
        T inv = T(1) / eta;
        aWo = dirAlbedoTrans(L, eta, dWo, lr);
        aWi = dirAlbedoTrans(L, inv, dWi, lr);
        eAvg = avgAlbedoTrans(L, inv, lr);
        ratio = ratioT;
    }
    else
    {
        aWo = dirAlbedoTrans(L, eta, dWo, lr);
        aWi = dirAlbedoTrans(L, eta, dWi, lr);
        eAvg = avgAlbedoTrans(L, eta, lr);
        ratio = T(1) - ratioT;
    }
    return ratio * safeDiv((T(1) - aWo) * (T(1) - aWi), (T(1) - eAvg) * C<T>::PI);
}
// getEnergyCompensation / getFmsDielectric / getEnergyCompensationTranslucent of either model
template <typename T, bool R> T energyCompM(const LutSet<T>& L, T fms, T dWo, T dWi, T lr, T ss)
{
    if (R) return energyCompKulla(L, fms, std::fabs(dWo), std::fabs(dWi), lr);
    return energyComp(L, fms, dWo, dWi, lr, ss);
}
template <typename T, bool R> T fmsDielM(const LutSet<T>& L, T eta, T lr, T cosT)
{
    if (R)
    {
        T fAvg = avgFresnel(eta);
        T eAvg = L.ssAvg(lr);
        return fAvg * eAvg / (T(1) - fAvg * (T(1) - eAvg));
    }
    return fresnelDD(eta, cosT);
}
template <typename T, bool R> T energyCompTransM(const LutSet<T>& L, T eta, T dWo, T dWi, T lr, T ss)
{
    if (R) return energyCompTransKulla(L, eta, dWo, dWi, lr);
    return energyCompTrans(L, eta, dWo, lr, ss);
}

// bsdfSample.hlsl lobes
template <typename T> V3<T> sampleCondRefl(T ax, T ay, V3<T> wo, T s0, T s1)
{
    V3<T> wm = deltaGGX(ax, ay) ? v3(T(0), T(1), T(0)) : sampleWM(wo, ax, ay, s0, s1);
    V3<T> wi = reflect(-wo, wm);
    return wi.y < T(0) ? v3(T(0), T(0), T(0)) : wi;
}
template <typename T> T pdfCondRefl(V3<T> wo, V3<T> wi, T ax, T ay)
{
    V3<T> wm = normalize(wo + wi);
    if (dot(wm, wo) < T(0)) return T(0);
    if (deltaGGX(ax, ay)) return T(1);
    return DV(wo, wm, ax, ay) * jRefl(wo, wm);
}
template <typename T> V3<T> sampleDielRefl(T ax, T ay, V3<T> wo, T s0, T s1)
{
    V3<T> wm = deltaGGX(ax, ay) ? v3(T(0), T(1), T(0)) : sampleWM(wo, ax, ay, s0, s1);
    V3<T> wi = reflect(-wo, wm);
    return !sameHemi(wo, wi) ? v3(T(0), T(0), T(0)) : wi;
}
template <typename T> T pdfDielRefl(V3<T> wo, V3<T> wi, T ax, T ay)
{
    if (!sameHemi(wo, wi)) return T(0);
    if (deltaGGX(ax, ay)) return T(1);
    V3<T> wm = normalize(wo + wi);
    return DV(wo, wm, ax, ay) * jRefl(wo, wm);
}
template <typename T> T evalDielRefl(T eta, T ax, T ay, V3<T> wo, V3<T> wi)
{
    V3<T> wm = normalize(wo + wi);
    if (!sameHemi(wo, wi)) return T(0);
    if (dot(wi, wm) > T(0) && dot(wo, wm) > T(0))
    {
        T F = fresnelDD(eta, dot(wo, wm));
        if (deltaGGX(ax, ay)) return F / std::fabs(wi.y);
        T D = DGGX(wm, ax, ay), g2 = G2(wo, wi, wm, ax, ay);
        return F * g2 * D / tmax(T(4) * wo.y * wi.y, T(0.00001f));
    }
    return T(0);
}
template <typename T> V3<T> wmTrans(V3<T> wo, V3<T> wi, T eta)
{
    if (sameHemi(wo, wi)) return normalize(wo + wi);
    if (eta == T(1)) eta = T(1.001f);
    return forceHemi(wo, normalize(wo + wi * eta));
}
template <typename T> T pdfTrans(T eta, V3<T> wo, V3<T> wi, T ax, T ay)
{
    if (eta == T(1)) eta = T(1.001f);
    V3<T> wm = wmTrans(wo, wi, eta);
    if (sameHemi(wo, wi)) return T(0);
    if (deltaGGX(ax, ay)) return T(1);
    T pdf = DV(wo, wm, ax, ay);
    if (dot(wo, wm) <= T(0) || dot(wi, wm) >= T(0)) return T(0);
    return pdf * jRefr(eta, wo, wm, wi);
}
template <typename T> T evalTrans(T eta, T ax, T ay, V3<T> wo, V3<T> wi)
{
    if (eta == T(1)) eta = T(1.001f);
    V3<T> wm = wmTrans(wo, wi, eta);
    if (sameHemi(wo, wi)) return T(0);
    if (dot(wo, wm) <= T(0) || dot(wi, wm) >= T(0)) return T(0);
    T vh = std::fabs(dot(wo, wm));
    T F = fresnelDD(eta, vh);
    if (deltaGGX(ax, ay)) return (T(1) - F) / std::fabs(wi.y);
    T g2 = G2(wo, wi, wm, ax, ay), D = DGGX(wm, ax, ay);
    T denom = std::fabs(wo.y * wi.y);
    return safeDiv((T(1) - F) * g2 * D * vh * jRefr(eta, wo, wm, wi), denom);
}
template <typename T> void reflRefrProb(T eta, V3<T> wo, V3<T> wm, bool aR, bool aT, T& pr, T& pt)
{
    T vh = saturate(dot(wo, wm));
    T r = fresnelDD(eta, vh), t = T(1) - r;
    if (!aR) r = 0;
    if (!aT) t = 0;
    if (r == 0 && t == 0)
    {
        pr = pt = 0;
        return;
    }
    T sum = r + t;
    pr = safeDiv(r, sum);
    pt = safeDiv(t, sum);
}
template <typename T> V3<T> sampleDiel(T eta, T ax, T ay, V3<T> wo, T s0, T s1, T sc, bool aR, bool aT)
{
    V3<T> wm = deltaGGX(ax, ay) ? (wo.y < 0 ? v3(T(0), T(-1), T(0)) : v3(T(0), T(1), T(0))) : sampleWM(wo, ax, ay, s0, s1);
    if (dot(wo, wm) < T(0)) return v3(T(0), T(0), T(0));
    if (eta == T(1)) eta = T(1.001f);
    T pr, pt;
    reflRefrProb(eta, wo, wm, aR, aT, pr, pt);
    if (pr == 0 && pt == 0) return v3(T(0), T(0), T(0));
    if (sc < pr || pt == 0)
    {
        V3<T> wi = reflect(-wo, wm);
        return !sameHemi(wo, wi) ? v3(T(0), T(0), T(0)) : wi;
    }
    V3<T> wi = refract(-wo, wm, T(1) / eta);
    return sameHemi(wo, wi) ? v3(T(0), T(0), T(0)) : wi;
}
template <typename T> T pdfDiel(T eta, V3<T> wo, V3<T> wi, T ax, T ay, bool aR, bool aT)
{
    V3<T> wm = wmTrans(wo, wi, eta);
    T pr, pt;
    reflRefrProb(eta, wo, wm, aR, aT, pr, pt);
    if (sameHemi(wo, wi)) return pdfDielRefl(wo, wi, ax, ay) * pr;
    return pdfTrans(eta, wo, wi, ax, ay) * pt;
}
template <typename T> S4<T> evalSheen(const S4<T>& col, T r, V3<T> wo, V3<T> wi)
{
    if (wi.y < T(0)) return sp(T(0));
    V3<T> wm = normalize(wo + wi);
    if (dot(wi, wm) > T(0) && dot(wo, wm) > T(0))
    {
        if (deltaSheen(r))
        {
            T d = std::fabs(wi.y);
            return d == T(0) ? sp(T(0)) : col / d;
        }
        T DG = std::fabs(safeDiv(DSheen(wm, r) * GSheen(wo, wi, r), T(4) * wo.y * wi.y));
        return col * DG;
    }
    return sp(T(0));
}

// SpecularLayer (materialLayers.hlsl:297-405)
template <typename T>
struct SpecLayer
{
    T ax, ay, lr, eta;
    bool aR, aT;
};
template <typename T, bool R = false> T specEval(const LutSet<T>& L, const SpecLayer<T>& l, V3<T> wo, V3<T> wi)
{
    if (sameHemi(wo, wi))
    {
        T w = evalDielRefl(l.eta, l.ax, l.ay, wo, wi);
        T ms;
        if (l.aR && l.aT) ms = energyCompTransM<T, R>(L, l.eta, wo.y, wi.y, l.lr, w);
        else
        {
            V3<T> wm = normalize(wo + wi);
            T fms = fmsDielM<T, R>(L, l.eta, l.lr, std::fabs(dot(wo, wm)));
            ms = energyCompM<T, R>(L, fms, std::fabs(wo.y), std::fabs(wi.y), l.lr, w);
        }
        w += ms;
        w *= std::fabs(wi.y);
        return w;
    }
    T w = evalTrans(l.eta, l.ax, l.ay, wo, wi);
    w += energyCompTransM<T, R>(L, l.eta, wo.y, wi.y, l.lr, w);
    w *= std::fabs(wi.y);
    return w;
}
// getMsSamplingProbability / getMsRefractionSelectionProbability (materialLayers.hlsl:327-344)
template <typename T, bool R> T specMsProb(const LutSet<T>& L, const SpecLayer<T>& l, V3<T> wo)
{
    if (!R || !l.aT || deltaGGX(l.ax, l.ay)) return T(0);
    return saturate(T(1) - dirAlbedoTrans(L, l.eta, wo.y, l.lr));
}
template <typename T, bool R> T specPdf(const LutSet<T>& L, const SpecLayer<T>& l, V3<T> wo, V3<T> wi)
{
    T pdfSS = pdfDiel(l.eta, wo, wi, l.ax, l.ay, l.aR, l.aT);
    T msProb = specMsProb<T, R>(L, l, wo);
    if (msProb == T(0)) return pdfSS;
    T refrSel = l.aR ? msTransRatio(L, l.eta, l.lr) : T(1);
    T pdfMS = pdfCosHemi(std::fabs(wi.y)) * (sameHemi(wo, wi) ? T(1) - refrSel : refrSel);
    return lerpT(pdfSS, pdfMS, msProb);
}

// surface (SurfaceDefinition, hitShadersCommon.hlsl:13-47)
template <typename T>
struct Surf
{
    S4<T> specular, albedo, absorption, emissive, sheenColor;
    V3<T> coatN, baseN, geoN, tangent;
    T transparency, metalness, ior, roughness, cauchyA, cauchyB, specAmount, ccAmount, ccIOR, ccRough;
    T aniso, anisoRot, thinFilm, sheenRough, sheenAmount, focus, sssAmount;
    T diffOcc = T(1), specOcc = T(1); // unpackOcclusion of the ORM texture's occlusion
    uint32_t flags;
    S4<T> sssRadius; // subsurface radius per lane (setFromRGBUnboundedNoIlluminant), when sssAmount > 0
};
template <typename T>
struct SCtx
{
    Basis<T> coatB, baseB;
    V3<T> woB, woC;
    T fromIOR, toIOR, ax, ay;
    bool exiting;
    T probs[6];
};
template <typename T> T cauchy(const Surf<T>& s, T lam)
{
    T um = lam * T(0.001f);
    return s.cauchyA + (s.cauchyB / (um * um));
}
// makeSurfaceSamplingContext (materialSample.hlsl:564-611, 89-127)
template <typename T> void makeCtx(const Surf<T>& s, T cur, T prev, V3<T> woOS, bool front, SCtx<T>& c)
{
    roughParams(s.roughness, s.aniso, c.ax, c.ay);
    c.exiting = !front;
    c.fromIOR = cur;
    c.toIOR = c.exiting ? prev : s.ior;
    c.coatB = basis(s.coatN, s.tangent);
    c.baseB = basis(s.baseN, s.tangent);
    c.woC = normalize(mulMv(c.coatB, woOS));
    c.woB = normalize(mulMv(c.baseB, woOS));
    T inside = c.woB.y < T(0) ? T(0) : T(1);
    T diel = T(1) - s.metalness, opaque = diel * (T(1) - s.transparency);
    T sum = 0;
    c.probs[0] = s.ccAmount * inside; sum += c.probs[0];
    c.probs[1] = s.sheenAmount * inside; sum += c.probs[1];
    c.probs[2] = s.metalness * inside; sum += c.probs[2];
    c.probs[3] = diel * (s.specAmount + s.transparency); sum += c.probs[3];
    c.probs[4] = opaque * (T(1) - s.sssAmount) * inside; sum += c.probs[4];
    c.probs[5] = opaque * s.sssAmount * inside; sum += c.probs[5];
    sum = tmax(T(0.000001f), sum);
    for (int i = 0; i < 6; ++i) c.probs[i] /= sum;
}
template <typename T> bool isDeltaDistr(const SCtx<T>& c, const Surf<T>& s)
{
    if (s.metalness == T(1) || s.transparency == T(1))
    {
        bool coatRough = (s.ccAmount > 0 && !deltaGGX1(s.ccRough)) || (s.sheenAmount > 0 && !deltaSheen(s.sheenRough));
        return !coatRough && deltaGGX(c.ax, c.ay);
    }
    return false;
}

template <typename T>
struct EvalR
{
    S4<T> w;
    T pdf;
    uint32_t trans;
};

template <typename T> void thinFilm(const T lam[4], const S4<T>& A1, S4<T>& A2, T nF, T etaTop, T phase, T cosI, T thick)
{
    if (allEq(A1, T(0))) return;
    if (allEq(A2, T(0)))
    {
        A2 = A1;
        return;
    }
    T m[4];
    if (thick > T(1200))
    {
        for (int i = 0; i < 4; ++i) m[i] = 0;
    }
    else
    {
        T cr2 = T(1) - (T(1) - cosI * cosI) / (etaTop * etaTop);
        T opd = cr2 < T(0) ? T(0) : T(2) * nF * thick * Mth<T>::sqrt(cr2);
        T f = tmax(T(0), thick - T(1200) + T(200)) * (T(1) / T(200));
        for (int i = 0; i < 4; ++i)
        {
            T mm = opd / lam[i] + phase;
            m[i] = Mth<T>::cos(T(2) * mm * C<T>::PI);
            m[i] = m[i] + (T(0) - m[i]) * f;
        }
    }
    for (int i = 0; i < 4; ++i)
        A2[i] = tmax(T(0), A1[i] + A2[i] + T(2) * Mth<T>::sqrt(tmax(T(0), A1[i] * A2[i])) * m[i]);
}

// evaluateSurface (materialSample.hlsl:264-562). R selects the Kulla-Conty multiple-scattering
// model of the bidirectional integrator. Flags as EVALUATE_FLAGS_* (materialSample.hlsl:57-61):
// EV_LIGHT_PATH adds the shading-normal compensation of light subpaths (compensateForShadingNormal,
// :259-262) and drops the camera-side 1/eta^2 solid-angle compression of refraction.
constexpr uint32_t EV_NONE = 1, EV_PDF_ONLY = 2, EV_LIGHT_PATH = 4, EV_TREAT_AS_DELTA = 8;
template <typename T, bool R> EvalR<T> evalSurfaceF(const LutSet<T>& L, const Surf<T>& s, const SCtx<T>& c, V3<T> wo,
                                                    V3<T> wi, uint32_t flags, const Spec<T>& sp4)
{
    EvalR<T> r;
    r.trans = 0;
    const bool treatAsDelta = (flags & EV_TREAT_AS_DELTA) != 0;
    const bool lightPath = (flags & EV_LIGHT_PATH) != 0;
    T ccx, ccy;
    roughParams(s.ccRough, T(0), ccx, ccy);
    T fromIOR = c.fromIOR, toIOR = c.toIOR;
    S4<T> ws = sp(T(0));
    T pdfSum = 0;
    V3<T> wiC = normalize(mulMv(c.coatB, wi)), wiB = normalize(mulMv(c.baseB, wi));
    V3<T> woC = c.woC, woB = c.woB;
    T dWoG = dot(wo, s.geoN), dWiG = dot(wi, s.geoN);
    bool bRefl = dWoG * dWiG > T(0), bRefr = dWoG * dWiG < T(0);
    const T compC = lightPath ? (std::fabs(woC.y) * std::fabs(dWiG)) / (std::fabs(dWoG) * std::fabs(wiC.y)) : T(1);
    const T compB = lightPath ? (std::fabs(woB.y) * std::fabs(dWiG)) / (std::fabs(dWoG) * std::fabs(wiB.y)) : T(1);
    T eLeft = 1, eLayer = 1;
    T diel = T(1) - s.metalness, specAmount = diel * s.specAmount;
    bool infer = s.thinFilm > 0 && s.ccAmount > 0 && (s.metalness > 0 || specAmount > 0);
    infer = infer && (deltaGGX(ccx, ccy) == deltaGGX(c.ax, c.ay));
    S4<T> coatAmp = sp(T(0));
    if (s.ccAmount > 0)
    {
        T eta = s.ccIOR / fromIOR;
        if (deltaGGX(ccx, ccy) == treatAsDelta)
        {
            T pdf = sameHemi(woC, wiC) ? pdfDielRefl(woC, wiC, ccx, ccy) : T(0);
            bool cRefl = dot(wo, s.geoN) * dot(wi, s.geoN) > T(0);
            if (pdf > 0 && cRefl)
            {
                T w = 0;
                if (sameHemi(woC, wiC))
                {
                    w = evalDielRefl(eta, ccx, ccy, woC, wiC);
                    w *= std::fabs(wiC.y);
                    V3<T> wm = normalize(woC + wiC);
                    T fms = fmsDielM<T, R>(L, eta, s.ccRough, std::fabs(dot(woC, wm)));
                    w += energyCompM<T, R>(L, fms, std::fabs(woC.y), std::fabs(wiC.y), s.ccRough, w);
                }
                S4<T> weight = sp(w) * (s.ccAmount * eLeft) * compC * s.specOcc;
                if (infer) coatAmp = weight;
                else ws = ws + weight;
                pdfSum += c.probs[0] * pdf;
            }
        }
        eLayer *= energyAfterSpec(L, eta, woC.y, s.ccRough, s.ccAmount);
    }
    if (s.sheenAmount > 0)
    {
        if (deltaSheen(s.sheenRough) == treatAsDelta)
        {
            T pdf = 0;
            if (sameHemi(woB, wiB) && wiB.y >= T(0)) pdf = deltaSheen(s.sheenRough) ? T(1) : pdfCosHemi(wiB.y);
            if (pdf > 0 && bRefl)
            {
                S4<T> w = sameHemi(woB, wiB) ? evalSheen(s.sheenColor, s.sheenRough, woB, wiB) * std::fabs(wiB.y) : sp(T(0));
                ws = ws + w * (s.sheenAmount * eLeft) * compB * s.specOcc;
                pdfSum += c.probs[1] * pdf;
            }
        }
        eLayer *= T(1) - L.sheen(std::fabs(woB.y), s.sheenRough) * s.sheenAmount;
    }
    eLeft *= eLayer;
    eLayer = 1;
    if (s.metalness > 0)
    {
        if (deltaGGX(c.ax, c.ay) == treatAsDelta)
        {
            T pdf = sameHemi(woB, wiB) ? pdfCondRefl(woB, wiB, c.ax, c.ay) : T(0);
            if (pdf > 0 && bRefl)
            {
                S4<T> w = sp(T(0));
                if (sameHemi(woB, wiB))
                {
                    V3<T> wm = normalize(woB + wiB);
                    bool delta = deltaGGX(c.ax, c.ay);
                    T g2 = 0, D = 0, den = 1;
                    if (!delta)
                    {
                        g2 = G2(woB, wiB, wm, c.ax, c.ay);
                        D = DGGX(wm, c.ax, c.ay);
                        den = tmax(T(4) * woB.y * wiB.y, T(0.00001f));
                    }
                    T dOM = dot(woB, wm);
                    T dw = L.ssNoF(std::fabs(woB.y), s.roughness);
                    for (int i = 0; i < 4; ++i)
                    {
                        T n, k2;
                        conductorNK2(s.albedo[i], s.specular[i], n, k2);
                        T er = n / fromIOR, ek = Mth<T>::sqrt(k2) / fromIOR;
                        T F = fresnelDC(er, ek, dOM);
                        T ss = delta ? F / std::fabs(wiB.y) : F * g2 * D / den;
                        T fms = fresnelDC(er, ek, dOM);
                        T ms = R ? energyCompKulla(L, fms, std::fabs(woB.y), std::fabs(wiB.y), s.roughness)
                                 : ss * (fms * (T(1) - dw) / dw);
                        w[i] = (ss + ms) * std::fabs(wiB.y);
                    }
                }
                S4<T> weight = w * (s.metalness * eLeft) * compB * s.specOcc;
                if (infer)
                {
                    T etaC = s.ccIOR / fromIOR;
                    V3<T> wm = normalize(woC + wiC);
                    T phase = etaC > T(1) ? T(0) : T(0.5f);
                    thinFilm(sp4.lam, coatAmp, weight, s.ccIOR, etaC, phase, dot(woC, wm), s.thinFilm);
                }
                ws = ws + weight;
                pdfSum += c.probs[2] * pdf;
            }
        }
        eLayer *= (T(1) - s.metalness);
    }
    if (specAmount > 0 && bRefl)
    {
        if (s.flags & YG_MATERIAL_DISPERSION)
        {
            if (c.exiting) fromIOR = cauchy(s, sp4.hero);
            else toIOR = cauchy(s, sp4.hero);
        }
        SpecLayer<T> sl{c.ax, c.ay, s.roughness, toIOR / fromIOR, s.specAmount > 0, s.transparency > 0};
        if (deltaGGX(c.ax, c.ay) == treatAsDelta)
        {
            T pdf = specPdf<T, R>(L, sl, woB, wiB);
            if (pdf > 0)
            {
                S4<T> weight = sp(specEval<T, R>(L, sl, woB, wiB)) * (specAmount * eLeft) * compB * s.specOcc;
                if (infer)
                {
                    T etaC = s.ccIOR / fromIOR;
                    V3<T> wm = normalize(woC + wiC);
                    T phase = ((etaC > T(1)) != (toIOR > s.ccIOR)) ? T(0.5f) : T(0);
                    thinFilm(sp4.lam, coatAmp, weight, s.ccIOR, etaC, phase, dot(woC, wm), s.thinFilm);
                }
                ws = ws + weight;
                pdfSum += c.probs[3] * pdf;
            }
        }
        eLayer *= sameHemi(woB, wiB) ? energyAfterSpec(L, sl.eta, woB.y, sl.lr, specAmount) : T(0);
    }
    eLeft *= eLayer;
    T diffAmount = (T(1) - s.transparency) * diel * (T(1) - s.sssAmount);
    if (diffAmount > 0 && !treatAsDelta)
    {
        T pdf = (sameHemi(woB, wiB) && wiB.y >= T(0)) ? pdfCosHemi(wiB.y) : T(0);
        if (pdf > 0 && bRefl)
        {
            S4<T> alb = s.albedo / C<T>::PI;
            S4<T> w = sameHemi(woB, wiB) ? alb * std::fabs(wiB.y) : sp(T(0));
            ws = ws + w * (diffAmount * eLeft) * compB * s.diffOcc;
            pdfSum += c.probs[4] * pdf;
        }
    }
    T transAmount = s.transparency * diel;
    if (transAmount > 0 && bRefr && (deltaGGX(c.ax, c.ay) == treatAsDelta))
    {
        if (s.flags & YG_MATERIAL_DISPERSION)
        {
            if (c.exiting) fromIOR = cauchy(s, sp4.hero);
            else toIOR = cauchy(s, sp4.hero);
            r.trans |= 4;
        }
        SpecLayer<T> sl{c.ax, c.ay, s.roughness, toIOR / fromIOR, s.specAmount > 0, s.transparency > 0};
        T pdf = specPdf<T, R>(L, sl, woB, wiB);
        if (pdf > 0)
        {
            pdfSum += c.probs[3] * pdf;
            bool two = (s.flags & YG_MATERIAL_TWO_SIDED) != 0;
            T comp = 1;
            if (!two)
            {
                if (!lightPath) comp *= sqr(T(1) / sl.eta);
                r.trans |= c.exiting ? 2u : 1u;
            }
            else r.trans |= 3u;
            ws = ws + sp(specEval<T, R>(L, sl, woB, wiB)) * (transAmount * eLeft) * comp * compB * s.specOcc;
        }
    }
    r.pdf = pdfSum;
    r.w = ws;
    return r;
}
// the unidirectional integrators' evaluation (Turquin model, camera path)
template <typename T> EvalR<T> evalSurface(const LutSet<T>& L, const Surf<T>& s, const SCtx<T>& c, V3<T> wo, V3<T> wi,
                                           bool treatAsDelta, const Spec<T>& sp4)
{
    return evalSurfaceF<T, false>(L, s, c, wo, wi, treatAsDelta ? EV_TREAT_AS_DELTA : EV_NONE, sp4);
}

// getSampleDirectionOSForLayer (materialSample.hlsl:147-257); with R the dielectric layer also
// samples the multiple-scattering cosine lobe (SpecularLayer::sampleWi, materialLayers.hlsl:346-360)
template <typename T, bool R = false>
V3<T> sampleLayer(const LutSet<T>* L, const Surf<T>& s, const SCtx<T>& c, int layer, T sel, T r0, T r1, T hero, bool& diffuse,
                  bool& delta)
{
    V3<T> wi = v3(T(0), T(0), T(0));
    bool allowT = s.transparency > 0;
    T fromIOR = c.fromIOR, toIOR = c.toIOR;
    diffuse = delta = false;
    if (layer == 0)
    {
        if (c.woC.y > 0)
        {
            T cx, cy;
            roughParams(s.ccRough, T(0), cx, cy);
            wi = mulvM(sampleDielRefl(cx, cy, c.woC, r0, r1), c.coatB);
            diffuse = tmin(cx, cy) > T(0.05f);
            delta = deltaGGX(cx, cy);
        }
    }
    else if (layer == 1)
    {
        if (c.woB.y > 0)
        {
            V3<T> w = deltaSheen(s.sheenRough) ? reflect(-c.woB, v3(T(0), T(1), T(0))) : cosHemi(r0, r1);
            if (w.y < T(0)) w = v3(T(0), T(0), T(0));
            wi = mulvM(w, c.baseB);
            diffuse = s.sheenRough > T(0.15f);
            delta = deltaSheen(s.sheenRough);
        }
    }
    else if (layer == 2)
    {
        if (c.woB.y > 0)
        {
            wi = mulvM(sampleCondRefl(c.ax, c.ay, c.woB, r0, r1), c.baseB);
            diffuse = tmin(c.ax, c.ay) > T(0.05f);
            delta = deltaGGX(c.ax, c.ay);
        }
    }
    else if (layer == 3)
    {
        if (s.flags & YG_MATERIAL_DISPERSION)
        {
            if (c.exiting) fromIOR = cauchy(s, hero);
            else toIOR = cauchy(s, hero);
        }
        T eta = toIOR / fromIOR;
        SpecLayer<T> sl{c.ax, c.ay, s.roughness, eta, s.specAmount > 0, s.transparency > 0};
        T msProb = R ? specMsProb<T, R>(*L, sl, c.woB) : T(0);
        if (sel < msProb)
        {
            T sc = sel / msProb;
            V3<T> w = cosHemi(r0, r1);
            T refrSel = sl.aR ? msTransRatio(*L, sl.eta, sl.lr) : T(1);
            bool msRefract = sc < refrSel;
            w.y = ((c.woB.y < T(0)) != msRefract) ? -w.y : w.y;
            wi = mulvM(w, c.baseB);
        }
        else
        {
            T fsel = (sel - msProb) / (T(1) - msProb);
            wi = mulvM(sampleDiel(eta, c.ax, c.ay, c.woB, r0, r1, fsel, s.specAmount > 0, s.transparency > 0), c.baseB);
        }
        diffuse = tmin(c.ax, c.ay) > T(0.05f);
        delta = deltaGGX(c.ax, c.ay);
    }
    else if (layer == 4)
    {
        if (c.woB.y > 0)
        {
            V3<T> w = cosHemi(r0, r1);
            if (w.y < T(0)) w = v3(T(0), T(0), T(0));
            wi = mulvM(w, c.baseB);
            diffuse = true;
        }
    }
    if (!allowT && dot(s.geoN, wi) < T(0)) wi = v3(T(0), T(0), T(0));
    if (allowT && layer == 3 && !isZero(wi))
    {
        V3<T> woOS = mulvM(c.woB, c.baseB);
        bool tg = dot(woOS, s.geoN) * dot(wi, s.geoN) < T(0);
        bool ts = c.woB.y * dot(wi, c.baseB.n) < T(0);
        if (tg != ts) wi = v3(T(0), T(0), T(0));
    }
    return wi;
}

// ---------------------------------------------------------------- traversal (independent BVH)
template <typename T>
struct TriHit
{
    float t, b1, b2;
    uint32_t inst, prim;
    bool front, found;
};
inline bool keyLess(uint32_t ia, uint32_t pa, uint32_t ib, uint32_t pb) { return ia < ib || (ia == ib && pa < pb); }

template <typename T> void buildBvh(Ctx<T>& c)
{
    size_t n = c.tris.size();
    c.triIdx.resize(n);
    std::vector<std::array<float, 6>> box(n);
    std::vector<std::array<float, 3>> cen(n);
    for (size_t i = 0; i < n; ++i)
    {
        c.triIdx[i] = (uint32_t)i;
        const auto& t = c.tris[i];
        V3<float> v1 = t.v0 + t.e1, v2 = t.v0 + t.e2;
        float p[3][3] = {{t.v0.x, t.v0.y, t.v0.z}, {v1.x, v1.y, v1.z}, {v2.x, v2.y, v2.z}};
        for (int a = 0; a < 3; ++a)
        {
            box[i][a] = std::min(p[0][a], std::min(p[1][a], p[2][a]));
            box[i][3 + a] = std::max(p[0][a], std::max(p[1][a], p[2][a]));
            box[i][a] -= 4e-7f * std::max(1.0f, std::fabs(box[i][a]));
            box[i][3 + a] += 4e-7f * std::max(1.0f, std::fabs(box[i][3 + a]));
            cen[i][a] = 0.5f * (box[i][a] + box[i][3 + a]);
        }
    }
    c.nodes.clear();
    struct Job
    {
        int node, first, count;
    };
    std::vector<Job> st;
    c.nodes.push_back({});
    st.push_back({0, 0, (int)n});
    while (!st.empty())
    {
        Job j = st.back();
        st.pop_back();
        typename Ctx<T>::Node nd;
        for (int a = 0; a < 3; ++a)
        {
            nd.lo[a] = std::numeric_limits<float>::infinity();
            nd.hi[a] = -std::numeric_limits<float>::infinity();
        }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = j.first; i < j.first + j.count; ++i)
        {
            uint32_t t = c.triIdx[i];
            for (int a = 0; a < 3; ++a)
            {
                nd.lo[a] = std::min(nd.lo[a], box[t][a]);
                nd.hi[a] = std::max(nd.hi[a], box[t][3 + a]);
                clo[a] = std::min(clo[a], cen[t][a]);
                chi[a] = std::max(chi[a], cen[t][a]);
            }
        }
        nd.left = nd.right = -1;
        nd.first = j.first;
        nd.count = j.count;
        int axis = 0;
        for (int a = 1; a < 3; ++a)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        if (j.count > 4 && chi[axis] > clo[axis])
        {
            int mid = j.first + j.count / 2;
            std::nth_element(c.triIdx.begin() + j.first, c.triIdx.begin() + mid, c.triIdx.begin() + j.first + j.count,
                             [&](uint32_t a, uint32_t b) { return cen[a][axis] < cen[b][axis]; });
            nd.left = (int)c.nodes.size();
            c.nodes.push_back({});
            nd.right = (int)c.nodes.size();
            c.nodes.push_back({});
            nd.count = 0;
            st.push_back({nd.left, j.first, mid - j.first});
            st.push_back({nd.right, mid, j.first + j.count - mid});
        }
        c.nodes[j.node] = nd;
    }
}

// Texture2D.SampleLevel(LINEAR_REPEAT, uv, 0) restated: bilinear between the four nearest
// texel centres with wrapped coordinates, in the same arithmetic order as the device
template <typename T> void bilinearTexels(const float* tx, int W, int H, T u0, T v0, T out[4])
{
    T u = u0 - std::floor(u0), v = v0 - std::floor(v0);
    T x = u * T(W) - T(0.5f), y = v * T(H) - T(0.5f);
    T fx = std::floor(x), fy = std::floor(y);
    T ax = x - fx, ay = y - fy;
    int x0 = (int)fx, y0 = (int)fy;
    x0 = x0 < 0 ? x0 + W : (x0 >= W ? x0 - W : x0);
    y0 = y0 < 0 ? y0 + H : (y0 >= H ? y0 - H : y0);
    const int x1 = x0 + 1 == W ? 0 : x0 + 1, y1 = y0 + 1 == H ? 0 : y0 + 1;
    const float* c00 = &tx[4 * ((size_t)y0 * W + x0)];
    const float* c10 = &tx[4 * ((size_t)y0 * W + x1)];
    const float* c01 = &tx[4 * ((size_t)y1 * W + x0)];
    const float* c11 = &tx[4 * ((size_t)y1 * W + x1)];
    const T sx = T(1) - ax, sy = T(1) - ay;
    for (int k = 0; k < 4; ++k)
        out[k] = (T(c00[k]) * sx + T(c10[k]) * ax) * sy + (T(c01[k]) * sx + T(c11[k]) * ax) * ay;
}

// alphaTestPasses (hitShadersCommon.hlsl:162-183): a hit on an instance whose material has an
// alpha cutoff above 0 and an albedo texture, on a mesh with texture coordinates, counts only
// where the albedo alpha at its uv (times the albedo uv scale) reaches the cutoff. FP32 for
// both oracle precisions, like the traversal itself.
template <typename T> bool cutoutPasses(const Ctx<T>& c, uint32_t inst, uint32_t prim, float b1, float b2)
{
    const oracle_scene* sc = c.sc;
    const oracle_instance& I = sc->instances[inst];
    const yg_material& M = sc->materials[I.material];
    if (!(M.alpha_cutoff > 0.0f) || !M.albedo_texture || !I.has_uvs || !sc->uvs) return true;
    uint32_t id[3];
    for (int k = 0; k < 3; ++k) id[k] = sc->indices[I.first_index + 3 * prim + k] + I.vertex_base;
    const float* U = sc->uvs;
    const float b0 = 1.0f - b1 - b2;
    const float u = U[2 * id[0]] * b0 + U[2 * id[1]] * b1 + U[2 * id[2]] * b2;
    const float v = U[2 * id[0] + 1] * b0 + U[2 * id[1] + 1] * b1 + U[2 * id[2] + 1] * b2;
    const int t = (int)M.albedo_texture - 1;
    float a[4];
    bilinearTexels(c.tex[t].data(), (int)c.texW[t], (int)c.texH[t], u * M.albedo_uv_scale[0], v * M.albedo_uv_scale[1], a);
    return a[3] >= M.alpha_cutoff;
}

// Moller-Trumbore in the same operation order as the device kernel; a candidate that would
// become the closest hit must also pass the cutout test
template <typename Cut>
inline void triTest(const V3<float>& o, const V3<float>& d, float tminv, const V3<float>& v0, const V3<float>& e1,
                    const V3<float>& e2, uint32_t inst, uint32_t prim, TriHit<float>& h, Cut&& cut)
{
    V3<float> pvec = cross(d, e2);
    float det = dot(e1, pvec);
    if (det == 0.0f) return;
    float inv = 1.0f / det;
    V3<float> tvec = o - v0;
    float u = dot(tvec, pvec) * inv;
    if (u < 0.0f || u > 1.0f) return;
    V3<float> q = cross(tvec, e1);
    float v = dot(d, q) * inv;
    if (v < 0.0f || u + v > 1.0f) return;
    float t = dot(e2, q) * inv;
    if (!(t > tminv)) return;
    if (t < h.t || (t == h.t && h.found && keyLess(inst, prim, h.inst, h.prim)))
    {
        if (!cut(u, v)) return;
        h.t = t;
        h.b1 = u;
        h.b2 = v;
        h.inst = inst;
        h.prim = prim;
        h.front = det > 0.0f;
        h.found = true;
    }
}

// Closest hit. The FP64 oracle traces in FP32 geometry too (the scene is FP32 data);
// only shading runs in T.
// onlyInst restricts the hits to one instance (the subsurface probe rays)
template <typename T>
bool trace(const Ctx<T>& c, V3<T> oT, V3<T> dT, float tminv, float tmaxv, TriHit<float>& h, uint32_t onlyInst = 0xffffffffu)
{
    V3<float> o = v3((float)oT.x, (float)oT.y, (float)oT.z), d = v3((float)dT.x, (float)dT.y, (float)dT.z);
    h.t = tmaxv;
    h.found = false;
    double inv[3] = {1.0 / d.x, 1.0 / d.y, 1.0 / d.z};
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp)
    {
        const auto& nd = c.nodes[stack[--sp]];
        double t0 = tminv, t1 = h.t;
        bool miss = false;
        double oo[3] = {o.x, o.y, o.z};
        for (int a = 0; a < 3 && !miss; ++a)
        {
            double ta = (nd.lo[a] - oo[a]) * inv[a], tb = (nd.hi[a] - oo[a]) * inv[a];
            if (std::isnan(ta) || std::isnan(tb)) continue; // ray parallel and on the slab plane
            if (ta > tb) std::swap(ta, tb);
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb * (1 + 1e-6));
            if (t0 > t1) miss = true;
        }
        if (miss) continue;
        if (nd.left < 0)
        {
            for (int i = nd.first; i < nd.first + nd.count; ++i)
            {
                const auto& t = c.tris[c.triIdx[i]];
                if (onlyInst != 0xffffffffu && t.inst != onlyInst) continue;
                triTest(o, d, tminv, t.v0, t.e1, t.e2, t.inst, t.prim, h,
                        [&](float b1, float b2) { return cutoutPasses(c, t.inst, t.prim, b1, b2); });
            }
        }
        else
        {
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
    }
    return h.found;
}

// ---------------------------------------------------------------- scene setup
template <typename T> bool setup(Ctx<T>& c, const oracle_scene* sc, const Tables* tb, T lmin, T lmax)
{
    c.sc = sc;
    c.tb = tb;
    c.lmin = lmin;
    c.lmax = lmax;
    // textures as yg_upload_texture decodes them (8-bit: v / 255, or the sRGB transfer function
    // of IEC 61966-2-1 in double on RGB)
    for (uint32_t t = 0; t < sc->n_textures; ++t)
    {
        const oracle_texture& X = sc->textures[t];
        const size_t n = (size_t)X.width * X.height;
        std::vector<float> v(4 * n);
        if (X.format == YG_TEXTURE_RGBA32_FLOAT)
            std::memcpy(v.data(), X.data, 4 * n * sizeof(float));
        else
        {
            float lut[256];
            for (int k = 0; k < 256; ++k)
            {
                double x = k / 255.0;
                lut[k] = X.format == YG_TEXTURE_RGBA8_SRGB ? (float)(x <= 0.04045 ? x / 12.92 : std::pow((x + 0.055) / 1.055, 2.4))
                                                           : (float)x;
            }
            const uint8_t* b = static_cast<const uint8_t*>(X.data);
            for (size_t i = 0; i < n; ++i)
            {
                for (int k = 0; k < 3; ++k) v[4 * i + k] = lut[b[4 * i + k]];
                v[4 * i + 3] = (float)(b[4 * i + 3] / 255.0);
            }
        }
        c.tex.push_back(std::move(v));
        c.texW.push_back(X.width);
        c.texH.push_back(X.height);
    }
    // the environment texture must exist, and a cube map is six square faces stacked (the
    // checks yg_set_environment_texture / yg_set_environment_cube make)
    if (sc->env_texture > sc->n_textures) return false;
    if (sc->env_cube && sc->env_texture && c.texH[sc->env_texture - 1] != 6 * c.texW[sc->env_texture - 1]) return false;
    int a = (int)lmin, b = (int)lmax;
    double ys = 0, ds = 0;
    for (int l = a; l <= b; ++l)
    {
        int s = l - 360;
        for (int k = 0; k < 4; ++k) c.cieT.push_back(std::is_same<T, float>::value ? T((float)tb->cie[4 * s + k]) : T(tb->cie[4 * s + k]));
        ys += tb->cie[4 * s + 1];
        ds += tb->cie[4 * s + 3];
    }
    c.ySumInv = std::is_same<T, float>::value ? T((float)(1.0 / ys)) : T(1.0 / ys);
    c.d65SumInv = std::is_same<T, float>::value ? T((float)(1.0 / ds)) : T(1.0 / ds);
    // flatten instances to world triangles (same float transform as the device scene build)
    std::vector<float> power;
    std::vector<uint32_t> lightInst;
    c.instLightPdf.assign(sc->n_instances, 0.f);
    for (uint32_t i = 0; i < sc->n_instances; ++i)
    {
        const oracle_instance& I = sc->instances[i];
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t p = 0; p < I.prim_count; ++p)
        {
            V3<float> w[3];
            for (int k = 0; k < 3; ++k)
            {
                uint32_t vi = sc->indices[I.first_index + 3 * p + k] + I.vertex_base;
                V3<float> ob = v3(sc->positions[3 * vi], sc->positions[3 * vi + 1], sc->positions[3 * vi + 2]);
                w[k] = xPoint<float>(I.o2w, ob);
                lo[0] = std::min(lo[0], w[k].x); lo[1] = std::min(lo[1], w[k].y); lo[2] = std::min(lo[2], w[k].z);
                hi[0] = std::max(hi[0], w[k].x); hi[1] = std::max(hi[1], w[k].y); hi[2] = std::max(hi[2], w[k].z);
                c.wlo[0] = std::min(c.wlo[0], w[k].x); c.wlo[1] = std::min(c.wlo[1], w[k].y); c.wlo[2] = std::min(c.wlo[2], w[k].z);
                c.whi[0] = std::max(c.whi[0], w[k].x); c.whi[1] = std::max(c.whi[1], w[k].y); c.whi[2] = std::max(c.whi[2], w[k].z);
            }
            typename Ctx<T>::Tri t;
            t.v0 = w[0];
            t.e1 = w[1] - w[0];
            t.e2 = w[2] - w[0];
            t.inst = i;
            t.prim = p;
            c.tris.push_back(t);
        }
        const yg_material& M = sc->materials[I.material];
        if (M.emissive[0] + M.emissive[1] + M.emissive[2] > 0.0f && I.prim_count > 0)
        {
            // estimateMeshLightPower (RaytraceCommonResources.cpp:385-404) over the instance bounds
            float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
            float area = ex * ey + ey * ez + ez * ex;
            float e = 0.2126f * M.emissive[0] + 0.7152f * M.emissive[1] + 0.0722f * M.emissive[2];
            if (e <= 0.f) e = 1.f;
            float sides = (M.material_mask & YG_MATERIAL_TWO_SIDED) ? 2.f : 1.f;
            power.push_back(3.14159274f * e * area * sides);
            lightInst.push_back(i);
        }
    }
    if (c.tris.empty())
        for (int k = 0; k < 3; ++k) c.wlo[k] = c.whi[k] = 0.0f;
    // punctual lights after the mesh lights (uploadLightData, RaytraceCommonResources.cpp:426-543),
    // power of estimatePunctualLightPower (:407-424)
    std::vector<float> pun;
    for (uint32_t i = 0; i < sc->n_punctual; ++i)
    {
        const yg_punctual_light& L = sc->punctual[i];
        float in = 0.2126f * L.intensity[0] + 0.7152f * L.intensity[1] + 0.0722f * L.intensity[2];
        const float pi = 3.14159274f;
        float pw;
        if (L.type == YG_LIGHT_POINT)
            pw = 4.f * pi * in;
        else if (L.type == YG_LIGHT_SPOT)
            pw = 2.f * pi * (1.f - 0.5f * (L.cos_inner + L.cos_outer)) * in;
        else
        {
            float ex = (c.whi[0] - c.wlo[0]) * 0.5f, ey = (c.whi[1] - c.wlo[1]) * 0.5f, ez = (c.whi[2] - c.wlo[2]) * 0.5f;
            pw = pi * (ex * ex + ey * ey + ez * ez) * in;
        }
        pun.push_back(pw);
        power.push_back(pw);
    }
    // calculateSelectionPDFs + buildAliasTable (RaytraceCommonResources.cpp:325-383)
    auto table = [](std::vector<float>& pw, std::vector<float>& thr, std::vector<uint32_t>& alias) {
        size_t cnt = pw.size();
        double total = 0;
        for (float w : pw) total += w;
        float share = total > 0 ? 0.1f : 1.f;
        for (float& w : pw) w = (1.f - share) * (total > 0 ? float(w / total) : 0.f) + share / cnt;
        std::vector<float> scaled(cnt);
        thr.assign(cnt, 0.f);
        alias.assign(cnt, 0);
        std::vector<uint32_t> small, large;
        for (size_t i = 0; i < cnt; ++i)
        {
            scaled[i] = pw[i] * cnt;
            (scaled[i] < 1.f ? small : large).push_back((uint32_t)i);
        }
        while (!small.empty() && !large.empty())
        {
            uint32_t s = small.back();
            small.pop_back();
            uint32_t l = large.back();
            large.pop_back();
            thr[s] = scaled[s];
            alias[s] = l;
            scaled[l] = (scaled[l] + scaled[s]) - 1.f;
            (scaled[l] < 1.f ? small : large).push_back(l);
        }
        for (uint32_t i : large) { thr[i] = 1.f; alias[i] = i; }
        for (uint32_t i : small) { thr[i] = 1.f; alias[i] = i; }
    };
    std::vector<float> thr, pthr;
    std::vector<uint32_t> alias, palias;
    if (!power.empty()) table(power, thr, alias);
    if (!pun.empty()) table(pun, pthr, palias);
    const size_t nMesh = lightInst.size();
    for (size_t l = 0; l < power.size(); ++l)
    {
        typename Ctx<T>::Light e{};
        e.pdf = power[l];
        e.thr = thr[l];
        e.alias = alias[l];
        if (l < nMesh)
        {
            e.inst = lightInst[l];
            c.instLightPdf[lightInst[l]] = power[l];
        }
        else
        {
            const size_t i = l - nMesh;
            yg_punctual_light L = sc->punctual[i];
            if (L.type != YG_LIGHT_POINT)
            {
                // normalised as yg_set_punctual_lights does
                float d = std::sqrt(L.direction[0] * L.direction[0] + L.direction[1] * L.direction[1] + L.direction[2] * L.direction[2]);
                for (int k = 0; k < 3; ++k) L.direction[k] = L.direction[k] / d;
            }
            e.inst = 0xffffffffu;
            e.type = L.type;
            e.ppdf = pun[i];
            e.pthr = pthr[i];
            e.palias = palias[i];
            for (int k = 0; k < 3; ++k)
            {
                e.pos[k] = L.position[k];
                e.dir[k] = L.direction[k];
                e.inten[k] = L.intensity[k];
            }
            e.cosIn = L.cos_inner;
            e.cosOut = L.cos_outer;
        }
        c.lights.push_back(e);
    }
    c.nPunctual = sc->n_punctual;

    buildBvh(c);
    return true;
}

// ---------------------------------------------------------------- one path
template <typename T>
struct Path
{
    S4<T> thr, total;
    V3<T> o, d;
    T pdfRay;
    uint32_t flags, len, nVol;
    T volIOR[4];
    S4<T> volAbs[4];
    uint32_t volMat[4];
};

template <typename T> void enterVol(Path<T>& p, T ior, const S4<T>& ab, uint32_t mat)
{
    p.nVol = std::min(p.nVol + 1, 4u);
    p.volIOR[p.nVol - 1] = ior;
    p.volAbs[p.nVol - 1] = ab;
    p.volMat[p.nVol - 1] = mat;
}
template <typename T> void exitVol(Path<T>& p, uint32_t mat)
{
    if (p.nVol == 0) return;
    int idx = -1;
    for (int i = (int)p.nVol - 1; i >= 0; --i)
        if (p.volMat[i] == mat)
        {
            idx = i;
            break;
        }
    if (idx < 0) idx = (int)p.nVol - 1;
    for (uint32_t i = (uint32_t)idx; i + 1 < p.nVol; ++i)
    {
        p.volIOR[i] = p.volIOR[i + 1];
        p.volAbs[i] = p.volAbs[i + 1];
        p.volMat[i] = p.volMat[i + 1];
    }
    --p.nVol;
}

// spawnRayOrigin (hitShadersCommon.hlsl:147-160) on FP32 positions
inline float spawnC(float p, float n, int oi)
{
    int so = p < 0.0f ? -oi : oi;
    int bits;
    std::memcpy(&bits, &p, 4);
    bits += so;
    float off;
    std::memcpy(&off, &bits, 4);
    return std::fabs(p) < (1.0f / 32.0f) ? p + (1.0f / 65536.0f) * n : off;
}
template <typename T> V3<T> spawn(V3<T> pT, V3<T> gnT, V3<T> dT)
{
    V3<float> p = v3((float)pT.x, (float)pT.y, (float)pT.z), gn = v3((float)gnT.x, (float)gnT.y, (float)gnT.z),
              d = v3((float)dT.x, (float)dT.y, (float)dT.z);
    V3<float> n = dot(d, gn) < 0.0f ? -gn : gn;
    int ox = (int)(256.0f * n.x), oy = (int)(256.0f * n.y), oz = (int)(256.0f * n.z);
    return v3(T(spawnC(p.x, n.x, ox)), T(spawnC(p.y, n.y, oy)), T(spawnC(p.z, n.z, oz)));
}
template <typename T> T misW(T a, T b)
{
    T a2 = a * a, b2 = b * b;
    return a2 / (a2 + b2);
}
template <typename T> T area2solid(V3<T> v, V3<T> n)
{
    T invD2 = T(1) / dot(v, v);
    T ad = std::fabs(dot(n, v * Mth<T>::sqrt(invD2)));
    return T(1) / (ad * invD2);
}
template <typename T> void triPositions(const Ctx<T>& c, const oracle_instance& I, uint32_t prim, V3<T> p[3], uint32_t idx[3])
{
    for (int k = 0; k < 3; ++k)
    {
        idx[k] = c.sc->indices[I.first_index + 3 * prim + k] + I.vertex_base;
        p[k] = v3(T(c.sc->positions[3 * idx[k]]), T(c.sc->positions[3 * idx[k] + 1]), T(c.sc->positions[3 * idx[k] + 2]));
    }
}
template <typename T> T regularizeR(T lr, bool sq)
{
    T r = sq ? lr * lr : lr;
    if (r < T(0.3f))
    {
        r = clampT(r * T(2), T(0.1f), T(0.3f));
        return sq ? Mth<T>::sqrt(r) : r;
    }
    return lr;
}

// a scene texture, sampled as bilinearTexels does
template <typename T> void sampleTex(const Ctx<T>& c, int id, T u0, T v0, T out[4])
{
    bilinearTexels(c.tex[id].data(), (int)c.texW[id], (int)c.texH[id], u0, v0, out);
}

// fetchMeshUV or (0.5, 0.5) without texture coordinates
template <typename T> void meshUV(const oracle_scene* sc, const oracle_instance& I, const uint32_t id[3], T b0, T b1, T b2,
                                  T& u, T& v)
{
    if (!I.has_uvs || !sc->uvs)
    {
        u = v = T(0.5f);
        return;
    }
    const float* U = sc->uvs;
    u = T(U[2 * id[0]]) * b0 + T(U[2 * id[1]]) * b1 + T(U[2 * id[2]]) * b2;
    v = T(U[2 * id[0] + 1]) * b0 + T(U[2 * id[1] + 1]) * b1 + T(U[2 * id[2] + 1]) * b2;
}

// getSkyBoxColor (materialsCommonResources.hlsl:181-224) times the intensity scale
// TextureCube.SampleLevel(LINEAR, dir, 0) restated: the Vulkan cube map face selection (major
// axis; sc, tc, ma per face, faces stacked +X, -X, +Y, -Y, +Z, -Z), then bilinear between texel
// centres clamped to the face's edge texels, in the device's operation order
template <typename T> void sampleCube(const Ctx<T>& c, int id, V3<T> d, T out[4])
{
    const T ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int face;
    T sc, tc, ma;
    if (ax >= ay && ax >= az)
    {
        face = d.x >= T(0) ? 0 : 1;
        sc = d.x >= T(0) ? -d.z : d.z;
        tc = -d.y;
        ma = ax;
    }
    else if (ay >= az)
    {
        face = d.y >= T(0) ? 2 : 3;
        sc = d.x;
        tc = d.y >= T(0) ? d.z : -d.z;
        ma = ay;
    }
    else
    {
        face = d.z >= T(0) ? 4 : 5;
        sc = d.z >= T(0) ? d.x : -d.x;
        tc = -d.y;
        ma = az;
    }
    const T s = T(0.5f) * (sc / ma + T(1)), t = T(0.5f) * (tc / ma + T(1));
    const int W = (int)c.texW[id];
    const T x = s * T(W) - T(0.5f), y = t * T(W) - T(0.5f);
    const T fx = std::floor(x), fy = std::floor(y);
    const T ax2 = x - fx, ay2 = y - fy;
    const int xi = (int)fx, yi = (int)fy;
    const int x0 = std::min(std::max(xi, 0), W - 1), x1 = std::min(std::max(xi + 1, 0), W - 1);
    const int y0 = std::min(std::max(yi, 0), W - 1), y1 = std::min(std::max(yi + 1, 0), W - 1);
    const float* F = c.tex[id].data() + 4 * (size_t)face * W * W;
    const float* c00 = &F[4 * ((size_t)y0 * W + x0)];
    const float* c10 = &F[4 * ((size_t)y0 * W + x1)];
    const float* c01 = &F[4 * ((size_t)y1 * W + x0)];
    const float* c11 = &F[4 * ((size_t)y1 * W + x1)];
    const T sx = T(1) - ax2, sy = T(1) - ay2;
    for (int k = 0; k < 4; ++k)
        out[k] = (T(c00[k]) * sx + T(c10[k]) * ax2) * sy + (T(c01[k]) * sx + T(c11[k]) * ax2) * ay2;
}

template <typename T> V3<T> skyColor(const Ctx<T>& c, V3<T> d, T scale)
{
    if (!c.sc->env_texture) return v3(std::fabs(d.x) * scale, std::fabs(d.y) * scale, std::fabs(d.z) * scale);
    V3<T> v = normalize(d);
    if (c.sc->env_cube)
    {
        T t[4];
        sampleCube(c, (int)c.sc->env_texture - 1, v, t);
        return v3(t[0] * scale, t[1] * scale, t[2] * scale);
    }
    T theta = std::atan2(v.z, v.x), phi = std::acos(clampT(v.y, T(-1), T(1)));
    T t[4];
    sampleTex(c, (int)c.sc->env_texture - 1, theta * C<T>::INVPI * T(0.5f) + T(0.5f), phi * C<T>::INVPI, t);
    return v3(t[0] * scale, t[1] * scale, t[2] * scale);
}

// fetch + fetchSurfaceMaterialParameters (with the BindlessMaterialManager clamps) +
// handleTwoSidedMaterialOrientation (when orient) + setupSurfaceOrientation + regularisation (when
// regularize) + convertSurfaceDefinitionFromRGB (rayHitDefault.hlsl:470-520, hitShadersCommon.hlsl:51-91)
template <typename T> void fillSurf(const Ctx<T>& c, const Spec<T>& s4, uint32_t inst, uint32_t prim, T b1, T b2, V3<T> rd,
                                    bool orient, bool regularize, Surf<T>& s)
{
    const oracle_scene* sc = c.sc;
    const oracle_instance& I = sc->instances[inst];
    const yg_material& M = sc->materials[I.material];
    V3<T> p[3];
    uint32_t id[3];
    triPositions(c, I, prim, p, id);
    T b0 = T(1) - b1 - b2;

    V3<T> gn = normalize(cross(p[1] - p[0], p[2] - p[0]));
    auto nv = [&](uint32_t k) { return v3(T(sc->normals[3 * k]), T(sc->normals[3 * k + 1]), T(sc->normals[3 * k + 2])); };
    V3<T> nrm = normalize(nv(id[0]) * b0 + nv(id[1]) * b1 + nv(id[2]) * b2);
    V3<T> tan = v3(T(1), T(0), T(0));
    if (I.has_tangents)
    {
        auto tv = [&](uint32_t k) {
            const float* t = sc->tangents + 4 * k;
            return v3(T(t[0] * t[3]), T(t[1] * t[3]), T(t[2] * t[3]));
        };
        tan = normalize(tv(id[0]) * b0 + tv(id[1]) * b1 + tv(id[2]) * b2);
    }
    // fetchSurfaceMaterialParameters with BindlessMaterialManager clamps
    auto sat = [](float x) { return std::min(std::max(x, 0.0f), 1.0f); };
    s.transparency = T(M.transparency);
    s.metalness = T(M.metalness);
    s.ior = T(std::min(std::max(M.dielectric_ior, 0.3f), 3.0f));
    s.roughness = T(sat(M.roughness));
    s.focus = T(M.emission_focus);
    s.specAmount = T(sat(M.specular_amount));
    s.ccAmount = T(sat(M.clear_coat_amount));
    s.ccIOR = T(M.clear_coat_ior);
    s.ccRough = T(sat(M.clear_coat_roughness));
    s.cauchyA = T(M.cauchy[0]);
    s.cauchyB = T(M.cauchy[1]);
    s.aniso = T(sat(M.anisotropy));
    s.anisoRot = T(M.anisotropy_rotation);
    s.thinFilm = T(M.thin_film_thickness_nm);
    s.flags = M.material_mask;
    s.sheenRough = T(std::fmax(M.sheen_roughness, 0.07f));
    s.sheenAmount = T(M.sheen_amount);
    s.sssAmount = T(sat(M.subsurface_amount));
    s.coatN = nrm;
    s.baseN = nrm;
    s.geoN = gn;
    s.tangent = tan;
    if (orient && s.transparency == T(0) && (s.flags & YG_MATERIAL_TWO_SIDED))
    {
        V3<T> wo = -rd;
        if (dot(wo, s.baseN) < T(0)) s.baseN = -s.baseN;
        if (dot(wo, s.coatN) < T(0)) s.coatN = -s.coatN;
        if (dot(wo, s.geoN) < T(0)) s.geoN = -s.geoN;
    }
    if (s.anisoRot > T(0))
    {
        T ang = s.anisoRot * T(2) * C<T>::PI, sa, ca;
        Mth<T>::sincos(ang, sa, ca);
        V3<T> t = s.tangent;
        s.tangent = v3(ca * t.x + T(0) * t.y + sa * t.z, T(0) * t.x + T(1) * t.y + T(0) * t.z, -sa * t.x + T(0) * t.y + ca * t.z);
    }
    // modifySurfaceMaterialParametersWithTextures (materialsCommon.hlsl:354-397)
    float alb[3] = {M.albedo[0], M.albedo[1], M.albedo[2]}, emi[3] = {M.emissive[0], M.emissive[1], M.emissive[2]};
    s.diffOcc = s.specOcc = T(1);
    if (M.albedo_texture || M.normal_texture || M.orm_texture || M.emissive_texture)
    {
        T u, v, t[4];
        meshUV(sc, I, id, b0, b1, b2, u, v);
        if (M.albedo_texture)
        {
            sampleTex(c, (int)M.albedo_texture - 1, u * T(M.albedo_uv_scale[0]), v * T(M.albedo_uv_scale[1]), t);
            for (int k = 0; k < 3; ++k) alb[k] = (float)(T(M.albedo[k]) * t[k]);
            if (s.flags & YG_MATERIAL_ALPHA_BLEND) s.transparency = T(1) - t[3] * (T(1) - s.transparency);
        }
        if (M.normal_texture)
        {
            sampleTex(c, (int)M.normal_texture - 1, u * T(M.normal_uv_scale[0]), v * T(M.normal_uv_scale[1]), t);
            V3<T> nn = normalize(v3(t[0] * T(2) - T(1), t[1] * T(2) - T(1), t[2] * T(2) - T(1)));
            s.baseN = mulvM(v3(nn.x, nn.z, nn.y), basis(s.baseN, s.tangent));
        }
        if (M.orm_texture)
        {
            sampleTex(c, (int)M.orm_texture - 1, u * T(M.orm_uv_scale[0]), v * T(M.orm_uv_scale[1]), t);
            T occ = T(floatFromHalf(halfFromFloat((float)t[0]))); // packOcclusion: a half
            s.diffOcc = s.specOcc = occ;
            s.roughness = s.roughness * t[1];
            s.metalness = s.metalness * t[2];
        }
        if (M.emissive_texture)
        {
            sampleTex(c, (int)M.emissive_texture - 1, u * T(M.emissive_uv_scale[0]), v * T(M.emissive_uv_scale[1]), t);
            for (int k = 0; k < 3; ++k) emi[k] = (float)(T(M.emissive[k]) * t[k]);
        }
    }
    if (regularize)
    {
        s.roughness = regularizeR(s.roughness, true);
        s.sheenRough = regularizeR(s.sheenRough, false);
        s.ccRough = regularizeR(s.ccRough, true);
    }
    s.specular = reflectance(c, s4, M.specular, M.specular_spectrum);
    s.albedo = reflectance(c, s4, alb, M.albedo_spectrum);
    bool absZero = M.absorption[0] == 0 && M.absorption[1] == 0 && M.absorption[2] == 0;
    s.absorption = absZero ? sp(T(0)) : setFromRGBUnboundedNoIllum(c, s4, v3(T(M.absorption[0]), T(M.absorption[1]), T(M.absorption[2])));
    s.emissive = emission(c, s4, emi, M.emission_spectrum);
    s.sheenColor = s.sheenAmount > T(0) ? setFromRGB(c, s4, v3(T(M.sheen_tint[0]), T(M.sheen_tint[1]), T(M.sheen_tint[2]))) : sp(T(0));
    // subsurfaceRadiusAmount.xyz = radius * scale, in FP32 as the material packing computes it
    const float sr[3] = {M.subsurface_radius[0] * M.subsurface_radius_scale, M.subsurface_radius[1] * M.subsurface_radius_scale,
                         M.subsurface_radius[2] * M.subsurface_radius_scale};
    s.sssRadius = s.sssAmount > T(0) ? setFromRGBUnboundedNoIllum(c, s4, v3(T(sr[0]), T(sr[1]), T(sr[2]))) : sp(T(0));
}

// ---------------------------------------------------------------- subsurface (subsurface.hlsl)
// The Christensen-Burley profile as a separable BSSRDF (subsurface.hlsl:88-394): profile, radius
// sampling, probe frame, exit density, the energy that reaches the diffuse base, the exit lobe.
template <typename T> T burleyScale(T albedo)
{
    T x = std::fabs(albedo - T(0.8f));
    return T(1.85f) - albedo + T(7) * x * x * x;
}
template <typename T> T burleyD(T radius, T albedo) { return tmax(radius, T(1e-6f)) / burleyScale(albedo); }
template <typename T> T burleyRMax(T d) { return T(20.7232658f) * d; }
template <typename T> T burleyProfileArea(T r, T d)
{
    r = tmax(r, d * T(1e-4f));
    return (Mth<T>::exp(-r / d) + Mth<T>::exp(-r / (T(3) * d))) / (T(8) * C<T>::PI * d * r);
}
template <typename T> T burleySampleRadius(T u, T d)
{
    T scale = d;
    if (u < T(0.25f)) u *= T(4);
    else
    {
        u = (u - T(0.25f)) / T(0.75f);
        scale = T(3) * d;
    }
    return -scale * Mth<T>::log(tmax(T(1) - u, T(1e-7f)));
}
template <typename T> S4<T> subsurfaceRd(const Surf<T>& s, T dist)
{
    S4<T> rd;
    for (int l = 0; l < 4; ++l) rd[l] = s.albedo[l] * burleyProfileArea(dist, burleyD(s.sssRadius[l], s.albedo[l]));
    return rd;
}
// constructVectorBase (commonMath.hlsl:84-90)
template <typename T> void vectorBase(V3<T> v, V3<T>& v2, V3<T>& v3o)
{
    if (std::fabs(v.x) > std::fabs(v.y)) v2 = v3(-v.z, T(0), v.x) / Mth<T>::sqrt(v.x * v.x + v.z * v.z);
    else v2 = v3(T(0), v.z, -v.y) / Mth<T>::sqrt(v.y * v.y + v.z * v.z);
    v3o = cross(v, v2);
}
template <typename T> void probeFrame(V3<T> n, uint32_t k, V3<T>& axis, V3<T>& u, V3<T>& v)
{
    V3<T> t, b;
    vectorBase(n, t, b);
    if (k == 0) { axis = n; u = t; v = b; }
    else if (k == 1) { axis = t; u = b; v = n; }
    else { axis = b; u = n; v = t; }
}
template <typename T> T pdfSssExit(const Surf<T>& s, V3<T> fromP, V3<T> fromN, V3<T> toP, V3<T> toN)
{
    V3<T> d = toP - fromP;
    T pdf = 0;
    for (uint32_t k = 0; k < 3; ++k)
    {
        V3<T> axis, pu, pv;
        probeFrame(fromN, k, axis, pu, pv);
        T du = dot(d, pu), dv = dot(d, pv);
        T rProj = Mth<T>::sqrt(du * du + dv * dv);
        T axisPdf = 0;
        for (int l = 0; l < 4; ++l)
        {
            T dl = burleyD(s.sssRadius[l], s.albedo[l]);
            if (rProj < burleyRMax(dl)) axisPdf += burleyProfileArea(rProj, dl);
        }
        pdf += (k == 0 ? T(0.5f) : T(0.25f)) * (T(1) / T(4)) * axisPdf * std::fabs(dot(toN, axis));
    }
    return pdf;
}
// getSubsurfaceEntryFactor (subsurface.hlsl:25-85)
template <typename T> T sssEntryFactor(const LutSet<T>& L, const Surf<T>& s, const SCtx<T>& c, T hero)
{
    T left = 1;
    T fromIOR = c.fromIOR, toIOR = c.toIOR;
    if (s.ccAmount > T(0)) left *= energyAfterSpec(L, s.ccIOR / fromIOR, c.woC.y, s.ccRough, s.ccAmount);
    if (s.sheenAmount > T(0)) left *= T(1) - L.sheen(std::fabs(c.woB.y), s.sheenRough) * s.sheenAmount;
    if (s.metalness > T(0)) left *= T(1) - s.metalness;
    T specAmount = (T(1) - s.metalness) * s.specAmount;
    if (specAmount > T(0))
    {
        if (s.flags & YG_MATERIAL_DISPERSION)
        {
            if (c.exiting) fromIOR = cauchy(s, hero);
            else toIOR = cauchy(s, hero);
        }
        left *= energyAfterSpec(L, toIOR / fromIOR, c.woB.y, s.roughness, specAmount);
    }
    T layer = (T(1) - s.metalness) * (T(1) - s.transparency) * s.sssAmount;
    return layer * left * s.diffOcc;
}
// sampleSubsurfaceExitLobe / evaluateSubsurfaceExitLobe (subsurface.hlsl:340-392)
template <typename T> V3<T> exitLobeSample(const Surf<T>& s, const SCtx<T>& c, V3<T> wo, T r0, T r1)
{
    V3<T> wi = mulvM(cosHemi(r0, r1), c.baseB);
    if (dot(wi, s.geoN) * dot(wo, s.geoN) <= T(0)) return v3(T(0), T(0), T(0));
    return wi;
}
template <typename T> void exitLobeEval(const Surf<T>& s, const SCtx<T>& c, V3<T> wo, V3<T> wi, uint32_t flags, S4<T>& w, T& pdf)
{
    w = sp(T(0));
    pdf = 0;
    T dWo = dot(wo, s.geoN), dWi = dot(wi, s.geoN);
    if (dWo * dWi <= T(0)) return;
    V3<T> wiB = normalize(mulMv(c.baseB, wi));
    if (wiB.y <= T(0)) return;
    pdf = pdfCosHemi(wiB.y);
    if ((flags & EV_PDF_ONLY) == 0)
    {
        T cosine = (flags & EV_LIGHT_PATH) ? std::fabs(dWi) : wiB.y;
        w = sp(C<T>::INVPI * cosine);
    }
}

// sampleSubsurfaceExit (subsurface.hlsl:212-337): an exit point for the entry point ep (normal en
// on the side the path arrived from) of instance inst, by up to eight probe rays along one axis of
// the entry frame at a radius drawn from one spectral lane's profile, one hit kept in proportion
// to the profile; the exit normal faces out of the geometry, the exit keeps the entry's face
template <typename T>
struct SssExit
{
    V3<T> pos, normal;
    TriHit<float> hit; // the probe hit (its face flag is the probe's)
    bool front;        // the exit's face flag: the entry's
    S4<T> w;  // Rd / (area density * probe-hit selection probability)
    T pdfPos; // area density of the exit point
};
template <typename T> bool sssSampleExit(const Ctx<T>& c, const Surf<T>& s, const oracle_instance& I, uint32_t inst, bool entryFront,
                                         V3<T> ep, V3<T> en, T r1, T r2, T r3, SssExit<T>& out, uint64_t& rays)
{
    T u = r1;
    uint32_t axisIndex;
    if (u < T(0.5f)) { axisIndex = 0; u *= T(2); }
    else if (u < T(0.75f)) { axisIndex = 1; u = (u - T(0.5f)) * T(4); }
    else { axisIndex = 2; u = (u - T(0.75f)) * T(4); }
    uint32_t lane = std::min((uint32_t)(u * T(4)), 3u);
    T uSel = saturate(u * T(4) - T(lane));
    const T dLane = burleyD(s.sssRadius[lane], s.albedo[lane]);
    const T rMax = burleyRMax(dLane);
    const T r = burleySampleRadius(r2, dLane);
    out.pdfPos = 0;
    out.w = sp(T(0));
    out.front = entryFront;
    TriHit<float>& sel = out.hit;
    sel.t = sel.b1 = sel.b2 = 0.f;
    sel.inst = inst;
    sel.prim = 0;
    sel.front = false;
    sel.found = false;
    if (!(r < rMax)) return false;
    V3<T> axis, pu, pv;
    probeFrame(en, axisIndex, axis, pu, pv);
    T sinPhi, cosPhi;
    Mth<T>::sincos(T(2) * C<T>::PI * r3, sinPhi, cosPhi);
    const T maxCoord = tmax(tmax(std::fabs(ep.x), std::fabs(ep.y)), std::fabs(ep.z));
    const T halfLength = tmax(Mth<T>::sqrt(rMax * rMax - r * r), T(1e-3f) + T(1e-5f) * maxCoord);
    const V3<T> po = ep + (pu * cosPhi + pv * sinPhi) * r - axis * halfLength;
    T wSum = 0, selW = 0;
    S4<T> selRd = sp(T(0));
    float tMin = 0.f;
    for (int k = 0; k < 8; ++k)
    {
        TriHit<float> th;
        rays++;
        if (!trace(c, po, axis, tMin, (float)(T(2) * halfLength), th, inst)) break;
        const S4<T> rd = subsurfaceRd(s, len(po + axis * T(th.t) - ep));
        const T w = rd[0] + rd[1] + rd[2] + rd[3];
        wSum += w;
        const T keep = wSum > T(0) ? w / wSum : T(0);
        if (keep >= T(1) || uSel < keep)
        {
            uSel = keep >= T(1) ? uSel : uSel / keep;
            selW = w;
            selRd = rd;
            sel = th;
        }
        else
        {
            uSel = (uSel - keep) / (T(1) - keep);
        }
        tMin = th.t + 5e-4f;
    }
    if (!(selW > T(0))) return false;
    V3<T> q[3];
    uint32_t qi[3];
    triPositions(c, I, sel.prim, q, qi);
    const V3<T> nOS = normalize(cross(q[1] - q[0], q[2] - q[0]));
    const V3<T> nW = normalize(xVecT<T>(I.w2o, nOS));
    const V3<T> frontN = ((dot(nW, axis) < T(0)) == sel.front) ? nW : -nW;
    out.pos = po + axis * T(sel.t);
    out.normal = entryFront ? frontN : -frontN;
    out.pdfPos = pdfSssExit(s, ep, en, out.pos, out.normal);
    if (!(out.pdfPos > T(0))) return false;
    out.w = selRd / (out.pdfPos * (selW / wSum));
    return true;
}

// spotFalloff / punctualLightAngularFalloff (lightSampling.hlsl:228-246) towards dirFromLight
template <typename T> T spotFalloff(V3<T> dirFromLight, const float* axis, float cosIn, float cosOut)
{
    T ct = dot(dirFromLight, v3(T(axis[0]), T(axis[1]), T(axis[2])));
    T ci = T(cosIn), co = T(cosOut);
    if (ci <= co) return ct >= co ? T(1) : T(0);
    T t = saturate((ct - co) / (ci - co));
    return t * t * (T(3) - T(2) * t);
}

// The hero wavelength and camera ray of a sample (rayGenPrimaryRays.hlsl:13-37,
// generateCameraRay in raytraceCommonResources.hlsl:113-137); rs starts at dimension 2.
template <typename T> void cameraSample(const Ctx<T>& c, const yg_render_params& P, uint32_t px, uint32_t py, Sampler& rs,
                                        Spec<T>& s4, V3<T>& rayO, V3<T>& rayD)
{
    const oracle_scene* sc = c.sc;
    s4.hero = c.lmin + T(rs.r1()) * (c.lmax - c.lmin);
    {
        // getSpectralSampleLambdas (spectralDistribution.hlsl:21-43)
        T step = (c.lmax - c.lmin) / T(4);
        T prev = s4.hero;
        s4.lam[0] = prev;
        for (int i = 1; i < 4; ++i)
        {
            T l = prev + step;
            if (l > c.lmax) l = c.lmin + (l - c.lmax);
            prev = l;
            s4.lam[i] = prev;
        }
    }
    // generateCameraRay (raytraceCommonResources.hlsl:113-137)
    const yg_camera& cam = *sc->camera;
    T invW = T(1) / T(P.width), invH = T(1) / T(P.height);
    T u = T(px) * invW + T(0.5f) * invW, v = T(py) * invH + T(0.5f) * invH;
    T tx = T(rs.get(0)), ty = T(rs.get(1));
    T lx = T(rs.r1()), ly = T(rs.r1());
    T ox = 0, oy = 0;
    if ((P.flags & YG_FLAG_DISABLE_TEXEL_JITTER) == 0)
    {
        ox = tx - T(0.5f);
        oy = ty - T(0.5f);
    }
    ox = ox * invW;
    oy = oy * invH;
    T pn0[4] = {u + ox, v + oy, T(0), T(1)}, pn[4];
    mul44(cam.uv_to_view, pn0, pn);
    T w = pn[3];
    for (int k = 0; k < 4; ++k) pn[k] = pn[k] / w;
    V3<T> pin = v3(pn[0], pn[1], pn[2]);
    V3<T> fp = pin * safeDiv(T(cam.focus_distance), std::fabs(pin.z));
    T dx, dy;
    concentricDisk(lx, ly, dx, dy);
    V3<T> lp = v3(dx * T(cam.aperture_radius), dy * T(cam.aperture_radius), T(0));
    T o4[4] = {lp.x, lp.y, lp.z, T(1)}, d4[4] = {fp.x - lp.x, fp.y - lp.y, fp.z - lp.z, T(0)}, ow[4], dw[4];
    mul44(cam.view_to_world, o4, ow);
    mul44(cam.view_to_world, d4, dw);
    rayO = v3(ow[0], ow[1], ow[2]);
    rayD = normalize(v3(dw[0], dw[1], dw[2]));
}

template <typename T> void tracePath(const Ctx<T>& c, const yg_render_params& P, const uint32_t* point, uint32_t px, uint32_t py,
                                     float* rec, V3<T>& xyzOut, uint64_t& rays)
{
    const oracle_scene* sc = c.sc;
    LutSet<T> L{{sc->luts[0], sc->luts[1], sc->luts[2], sc->luts[3], sc->luts[4], sc->luts[5], sc->luts[6], sc->luts[7], sc->luts[8]}};
    uint32_t rayIndex = py * P.width + px;
    uint32_t seed = rayIndex ^ (P.seed * 0x9E3779B9u);
    Sampler rs{point, 2u, seed};
    Spec<T> s4;
    Path<T> ps;
    cameraSample(c, P, px, py, rs, s4, ps.o, ps.d);
    ps.thr = sp(T(1));
    ps.total = sp(T(0));
    ps.pdfRay = 0;
    ps.flags = 0;
    ps.len = 0;
    ps.nVol = 0;
    bool alive = true;
    const uint32_t F_SEC = 1, F_REG = 2, F_DELTA = 4;
    for (uint32_t bounce = 0; bounce < P.max_depth; ++bounce)
    {
        if (!alive) break;
        TriHit<float> h;
        rays++;
        bool found = trace(c, ps.o, ps.d, 5e-4f, INFINITY, h);
        if (!found)
        {
            // rayMissEnvironment (rayMissEnvironment.hlsl:13-31)
            T sc4 = T(P.env_intensity_scale);
            V3<T> col = skyColor(c, ps.d, sc4);
            S4<T> Le = isZero(col) ? sp(T(0)) : setFromRGBUnbounded(c, s4, col);
            ps.total = ps.total + ps.thr * Le;
            alive = false;
        }
        else
        {
            const oracle_instance& I = sc->instances[h.inst];
            V3<T> rd = normalize(xVec<T>(I.w2o, ps.d));
            if (P.regularize_enable && ps.len >= P.regularize_after_vertices) ps.flags |= F_REG;
            Surf<T> s;
            fillSurf(c, s4, h.inst, h.prim, T(h.b1), T(h.b2), rd, true, P.regularize_enable && (ps.flags & F_REG), s);
            V3<T> hitPos = ps.o + ps.d * T(h.t);
            if (dot(rd, s.geoN) > T(0) && ps.nVol == 0 && !(s.flags & YG_MATERIAL_TWO_SIDED)) enterVol(ps, s.ior, s.absorption, I.material);
            S4<T> ab = ps.nVol ? ps.volAbs[ps.nVol - 1] : sp(T(0));
            if (!allEq(ab, T(0)))
                for (int k = 0; k < 4; ++k) ps.thr[k] = ps.thr[k] * Mth<T>::exp(-ab[k] * T(h.t));
            if (!allEq(s.emissive, T(0)))
            {
                T wMIS = 1;
                if (P.integrator == YG_INTEGRATOR_NEE && !c.lights.empty() && ps.pdfRay > T(0) && !(ps.flags & F_DELTA))
                {
                    V3<T> q[3];
                    uint32_t qi[3];
                    triPositions(c, I, h.prim, q, qi);
                    V3<T> p1 = xPoint<T>(I.o2w, q[0]), p2 = xPoint<T>(I.o2w, q[1]), p3 = xPoint<T>(I.o2w, q[2]);
                    V3<T> g = cross(p2 - p1, p3 - p1);
                    T gl = len(g);
                    g = g / gl;
                    T area = gl * T(0.5f);
                    T posPdf = T(1) / (T(I.prim_count) * area);
                    T lpdf = posPdf * T(c.instLightPdf[h.inst]) * area2solid(hitPos - ps.o, g);
                    wMIS = misW(ps.pdfRay, lpdf);
                }
                T side = dot(s.geoN, -rd) < T(0) ? T(0) : T(1);
                T prof = 1;
                if (s.focus > T(0))
                {
                    V3<T> gw = normalize(xVecT<T>(I.w2o, s.geoN));
                    prof = emissionProfile(dot(gw, -normalize(ps.d)), s.focus);
                }
                ps.total = ps.total + ps.thr * s.emissive * wMIS * side * prof;
                alive = false;
            }
            else
            {
                T rB[4];
                for (int k = 0; k < 4; ++k) rB[k] = T(rs.r1());
                V3<T> wo = -rd;
                SCtx<T> sctx;
                T cur = ps.nVol ? ps.volIOR[ps.nVol - 1] : T(1), prev = ps.nVol > 1 ? ps.volIOR[ps.nVol - 2] : T(1);
                makeCtx(s, cur, prev, wo, h.front, sctx);
                V3<T> nWS = normalize(xVecT<T>(I.w2o, s.geoN));
                const bool nee = P.integrator == YG_INTEGRATOR_NEE;
                // connectToExplicitLight (rayHitDefault.hlsl:204-257) from a vertex; at a subsurface exit
                // point (exitLobe) the light is weighed by the exit lobe instead of the BSDF
                auto connectLight = [&](const Surf<T>& s, const SCtx<T>& sctx, V3<T> wo, V3<T> hitPos, V3<T> nWS,
                                        const oracle_instance& I, bool exitLobe) {
                    auto evalToLight = [&](V3<T> toLOS) {
                        if (!exitLobe) return evalSurface(L, s, sctx, wo, toLOS, false, s4);
                        EvalR<T> e;
                        exitLobeEval(s, sctx, wo, toLOS, EV_NONE, e.w, e.pdf);
                        e.trans = 0;
                        return e;
                    };
                    // connectToExplicitLight (rayHitDefault.hlsl:204-257)
                    T rl[4];
                    for (int k = 0; k < 4; ++k) rl[k] = T(rs.r1());
                    // sampleLightIndex / samplePunctualLightIndex (lightSampling.hlsl:31-53)
                    uint32_t nL = (uint32_t)c.lights.size(), li;
                    float pick;
                    if (nee)
                    {
                        float scaled = (float)rl[3] * (float)nL;
                        if (!std::is_same<T, float>::value) scaled = (float)(rl[3] * T(nL));
                        li = std::min((uint32_t)scaled, nL - 1);
                        li = (scaled - (float)li) < c.lights[li].thr ? li : c.lights[li].alias;
                        pick = c.lights[li].pdf;
                    }
                    else
                    {
                        uint32_t nP = c.nPunctual, first = nL - nP;
                        float scaled = (float)rl[3] * (float)nP;
                        if (!std::is_same<T, float>::value) scaled = (float)(rl[3] * T(nP));
                        uint32_t idx = std::min((uint32_t)scaled, nP - 1);
                        const auto& E = c.lights[first + idx];
                        li = first + ((scaled - (float)idx) < E.pthr ? idx : E.palias);
                        pick = c.lights[li].ppdf;
                    }
                    const auto& Lt = c.lights[li];
                    if (Lt.type != 0)
                    {
                        // evaluatePunctualLightIncidence (lightSampling.hlsl:255-275)
                        V3<T> toL, I3;
                        T dist;
                        if (Lt.type == YG_LIGHT_DIRECTIONAL)
                        {
                            toL = v3(-T(Lt.dir[0]), -T(Lt.dir[1]), -T(Lt.dir[2]));
                            dist = T(INFINITY);
                            I3 = v3(T(Lt.inten[0]), T(Lt.inten[1]), T(Lt.inten[2]));
                        }
                        else
                        {
                            V3<T> v = v3(T(Lt.pos[0]), T(Lt.pos[1]), T(Lt.pos[2])) - hitPos;
                            T d2 = std::fmax(dot(v, v), T(1e-10f));
                            dist = Mth<T>::sqrt(d2);
                            toL = v / dist;
                            T fall = Lt.type == YG_LIGHT_SPOT ? spotFalloff(-toL, Lt.dir, Lt.cosIn, Lt.cosOut) : T(1);
                            T f = fall / d2;
                            I3 = v3(T(Lt.inten[0]) * f, T(Lt.inten[1]) * f, T(Lt.inten[2]) * f);
                        }
                        S4<T> emis = isZero(I3) ? sp(T(0)) : setFromRGBUnbounded(c, s4, I3);
                        if (!allEq(emis, T(0)) && T(pick) > T(0))
                        {
                            V3<T> toLOS = normalize(xVec<T>(I.w2o, toL));
                            EvalR<T> ev = evalToLight(toLOS);
                            S4<T> wl = ev.w;
                            if ((ev.trans & 4) && !(ps.flags & F_SEC))
                            {
                                wl[0] *= T(4);
                                wl[1] = wl[2] = wl[3] = 0;
                            }
                            if (!allEq(wl, T(0)))
                            {
                                V3<T> st = spawn(hitPos, nWS, toL);
                                TriHit<float> sh;
                                rays++;
                                // checkUnoccluded (rayHitDefault.hlsl:114-133)
                                bool any = trace(c, st, toL, 5e-4f, (float)dist - 5e-4f, sh);
                                if (!any)
                                {
                                    wl = (wl / T(pick)) * T(1);
                                    ps.total = ps.total + ps.thr * wl * emis;
                                }
                            }
                        }
                    }
                    else
                    {
                    const oracle_instance& LI = sc->instances[Lt.inst];
                    const yg_material& LM = sc->materials[LI.material];
                    uint32_t pc = LI.prim_count;
                    uint32_t prim = (uint32_t)std::fmin((float)pc * (float)rl[2], (float)(pc - 1));
                    if (!std::is_same<T, float>::value) prim = (uint32_t)std::fmin(T(pc) * rl[2], T(pc - 1));
                    T bx = rl[0], by = rl[1];
                    if (bx + by > T(1))
                    {
                        bx = T(1) - bx;
                        by = T(1) - by;
                    }
                    T lb0 = T(1) - bx - by;
                    V3<T> q[3];
                    uint32_t qi[3];
                    triPositions(c, LI, prim, q, qi);
                    V3<T> p1 = xPoint<T>(LI.o2w, q[0]), p2 = xPoint<T>(LI.o2w, q[1]), p3 = xPoint<T>(LI.o2w, q[2]);
                    V3<T> g = cross(p2 - p1, p3 - p1);
                    T gl = len(g);
                    g = g / gl;
                    T area = gl * T(0.5f);
                    V3<T> lpos = p1 * lb0 + p2 * bx + p3 * by;
                    float lem[3] = {LM.emissive[0], LM.emissive[1], LM.emissive[2]};
                    if (LM.emissive_texture)
                    {
                        // modifySurfaceEmissionWithTexture at the sampled point
                        T u, v, t[4];
                        meshUV(sc, LI, qi, lb0, bx, by, u, v);
                        sampleTex(c, (int)LM.emissive_texture - 1, u * T(LM.emissive_uv_scale[0]), v * T(LM.emissive_uv_scale[1]), t);
                        for (int k = 0; k < 3; ++k) lem[k] = (float)(T(LM.emissive[k]) * t[k]);
                    }
                    S4<T> rad = emission(c, s4, lem, LM.emission_spectrum);
                    T pdfPos = T(1) / (T(pc) * area);
                    bool two = (LM.material_mask & YG_MATERIAL_TWO_SIDED) != 0;
                    V3<T> toL = lpos - hitPos;
                    T dist = len(toL);
                    T cosE = -dot(g, toL / dist);
                    S4<T> emis = rad * emissionProfile(cosE, T(LM.emission_focus));
                    T lpdf = T(pick) * pdfPos * area2solid(toL, g);
                    V3<T> toLWS = toL / dist;
                    if (!two && dot(toL, g) >= T(0))
                    {
                        emis = sp(T(0));
                        lpdf = 0;
                    }
                    if (!allEq(emis, T(0)) && lpdf > T(0))
                    {
                        V3<T> toLOS = normalize(xVec<T>(I.w2o, toLWS));
                        EvalR<T> ev = evalToLight(toLOS);
                        S4<T> wl = ev.w;
                        if ((ev.trans & 4) && !(ps.flags & F_SEC))
                        {
                            wl[0] *= T(4);
                            wl[1] = wl[2] = wl[3] = 0;
                        }
                        if (!allEq(wl, T(0)))
                        {
                            V3<T> st = spawn(hitPos, nWS, toLWS);
                            TriHit<float> sh;
                            rays++;
                            bool any = trace(c, st, toLWS, 5e-4f, (float)dist + 5e-4f, sh);
                            bool vis = any && sh.inst == Lt.inst && sh.prim == prim;
                            T wm = misW(lpdf, ev.pdf);
                            if (vis)
                            {
                                wl = (wl / lpdf) * wm;
                                ps.total = ps.total + ps.thr * wl * emis;
                            }
                        }
                    }
                    }
                                };
                // hasExplicitlySampledLights (rayHitDefault.hlsl:26-34): without NEE only the punctual lights
                if ((nee ? !c.lights.empty() : c.nPunctual > 0) && !isDeltaDistr(sctx, s))
                    connectLight(s, sctx, wo, hitPos, nWS, I, false);
                // sampleScatteringEvent (scatteringSample.hlsl:30-65)
                T r = tmax(T(0), rB[0] + T(0.00001f));
                int layer;
                for (layer = 0; layer < 6; ++layer)
                {
                    if (r < sctx.probs[layer] && sctx.probs[layer] > T(0)) break;
                    r -= sctx.probs[layer];
                }
                if (layer == 5)
                {
                    // the subsurface event (scatteringSample.hlsl:45-54; rayHitDefault.hlsl:261-320, 349-355);
                    // the entry vertex's light connection was added above
                    alive = false;
                    const V3<T> ep = hitPos;
                    const V3<T> en = dot(-ps.d, nWS) < T(0) ? -nWS : nWS; // orientToSameSide
                    SssExit<T> ex;
                    bool ok = sssSampleExit(c, s, I, h.inst, h.front, ep, en, rB[1], rB[2], rB[3], ex, rays);
                    const V3<T> exitPos = ex.pos, exitN = ex.normal;
                    const S4<T> exitW = ex.w;
                    const T pdfPos = ex.pdfPos;
                    const TriHit<float>& sel = ex.hit;
                    if (!ok)
                    {
                        // no exit point: the event has no direction, the path ends
                        ps.pdfRay = 0;
                        ps.flags &= ~F_DELTA;
                        ps.thr = ps.thr * sp(T(0));
                    }
                    else
                    {
                        // evaluateSubsurfaceEntry, then continueFromSubsurfaceExit
                        S4<T> entryW = exitW * (sssEntryFactor(L, s, sctx, s4.hero) * pdfPos);
                        T pdfFwd = sctx.probs[5] * pdfPos;
                        ps.thr = ps.thr * entryW * safeDiv(T(1), pdfFwd);
                        V3<T> xrd = normalize(xVec<T>(I.w2o, -exitN));
                        Surf<T> xs;
                        fillSurf(c, s4, h.inst, sel.prim, T(sel.b1), T(sel.b2), xrd, true,
                                 P.regularize_enable && (ps.flags & F_REG), xs);
                        V3<T> xwo = -xrd;
                        SCtx<T> xc;
                        makeCtx(xs, cur, prev, xwo, h.front, xc);
                        if (nee ? !c.lights.empty() : c.nPunctual > 0) connectLight(xs, xc, xwo, exitPos, exitN, I, true);
                        T rX[4];
                        for (int k = 0; k < 4; ++k) rX[k] = T(rs.r1());
                        V3<T> xwi = exitLobeSample(xs, xc, xwo, rX[2], rX[3]);
                        S4<T> xw = sp(T(0));
                        T xpdf = 0;
                        bool dirSet = false;
                        if (!isZero(xwi))
                        {
                            exitLobeEval(xs, xc, xwo, xwi, EV_NONE, xw, xpdf);
                            if (xpdf > T(0))
                            {
                                xw = xw / xpdf;
                                V3<T> dW = normalize(xVec<T>(I.o2w, xwi));
                                ps.o = spawn(exitPos, exitN, dW);
                                ps.d = dW;
                                dirSet = true;
                            }
                            else xw = sp(T(0));
                        }
                        ps.flags |= F_REG;
                        ps.flags &= ~F_DELTA;
                        ps.pdfRay = xpdf;
                        ps.thr = ps.thr * xw;
                        alive = dirSet && xpdf != T(0);
                    }
                }
                else
                {
                    V3<T> wi = v3(T(0), T(0), T(0));
                    bool diff = false, delta = false;
                    if (layer < 5) wi = sampleLayer<T, false>(&L, s, sctx, layer, rB[1], rB[2], rB[3], s4.hero, diff, delta);
                    EvalR<T> ev;
                    ev.w = sp(T(0));
                    ev.pdf = 0;
                    ev.trans = 0;
                    if (!isZero(wi))
                    {
                        ev = evalSurface(L, s, sctx, wo, wi, delta, s4);
                        if (diff) ps.flags |= F_REG;
                    }
                    ps.pdfRay = ev.pdf;
                    if (delta) ps.flags |= F_DELTA;
                    else ps.flags &= ~F_DELTA;
                    if (ev.pdf > T(0))
                    {
                        if (ev.trans)
                        {
                            if (ev.trans & 4)
                            {
                                if (!(ps.flags & F_SEC))
                                {
                                    ev.w[0] *= T(4);
                                    ev.w[1] = ev.w[2] = ev.w[3] = 0;
                                }
                                ps.flags |= F_SEC;
                            }
                            bool en = (ev.trans & 1) != 0, ex = (ev.trans & 2) != 0;
                            if (en != ex)
                            {
                                if (ex) exitVol(ps, I.material);
                                else enterVol(ps, s.ior, s.absorption, I.material);
                            }
                        }
                        ev.w = ev.w / ev.pdf;
                    }
                    ps.thr = ps.thr * ev.w;
                    if (isZero(wi) || ps.pdfRay == T(0)) alive = false;
                    else
                    {
                        V3<T> nW = normalize(xVec<T>(I.o2w, s.geoN));
                        V3<T> dW = normalize(xVec<T>(I.o2w, wi));
                        ps.o = spawn(hitPos, nW, dW);
                        ps.d = dW;
                    }
                }
            }
        }
        ps.len += 1;
        // applyRussianRoulette (spectralDistribution.hlsl:124-138)
        T rr = T(rs.r1());
        T pmax = tmax(tmax(tmax(ps.thr[0], ps.thr[1]), ps.thr[2]), ps.thr[3]) / T(1);
        pmax = clampT(pmax, T(0.05f), T(1));
        if (rr > pmax)
        {
            alive = false;
            break;
        }
        ps.thr = ps.thr * (T(1) / pmax);
    }
    V3<T> X = toXYZ(c, s4, ps.total);
    xyzOut = X;
    if (rec)
    {
        rec[0] = (float)s4.hero;
        for (int k = 0; k < 4; ++k) rec[1 + k] = (float)ps.total[k];
        rec[5] = (float)X.x;
        rec[6] = (float)X.y;
        rec[7] = (float)X.z;
    }
}

// whether a render converts RGB colours to spectra, and so needs the scene's rgb_to_spd table
inline bool needsRgbTable(const oracle_scene* sc, const yg_render_params* P)
{
    auto nonGrey = [](const float* v) { return !(v[0] == v[1] && v[1] == v[2]); };
    auto nonZero = [](const float* v) { return v[0] != 0.0f || v[1] != 0.0f || v[2] != 0.0f; };
    if (P->env_intensity_scale > 0.0f) return true;
    for (uint32_t i = 0; i < sc->n_materials; ++i)
    {
        const yg_material& m = sc->materials[i];
        if ((m.albedo_spectrum < 0 && nonGrey(m.albedo)) || (m.specular_spectrum < 0 && nonGrey(m.specular)) ||
            (m.emission_spectrum < 0 && nonGrey(m.emissive)) || (nonZero(m.absorption) && nonGrey(m.absorption)) ||
            (m.sheen_amount > 0.0f && nonGrey(m.sheen_tint)) || (m.subsurface_amount > 0.0f && nonGrey(m.subsurface_radius)) ||
            m.albedo_texture || m.emissive_texture)
            return true;
    }
    for (uint32_t i = 0; i < sc->n_punctual; ++i)
        if (nonGrey(sc->punctual[i].intensity)) return true;
    return false;
}

// `stride` > 1 renders every stride-th pixel of the crop in x and y (a strided subsample of
// the request, each pixel with its own sample indices); records and film are then laid out
// over the ceil(crop_w / stride) x ceil(crop_h / stride) subsampled pixels.
template <typename T> int run(const oracle_scene* sc, const yg_render_params* P, int threads, float* records, double* film,
                              oracle_stats* stats, uint32_t stride = 1)
{
    Tables tb;
    if (!loadCie(sc->data_dir, tb.cie) || !sobolMatrices(sc->data_dir, tb.sobol)) return -5;
    float lminf = P->lambda_min, lmaxf = P->lambda_max;
    if (lminf == 0 && lmaxf == 0)
    {
        lminf = 380;
        lmaxf = 700;
    }
    Ctx<T> c;
    if (!setup(c, sc, &tb, T(lminf), T(lmaxf))) return -7; // a bad environment texture reference
    uint32_t cx = P->crop_x, cy = P->crop_y, cw = P->crop_w, ch = P->crop_h;
    if (cw == 0 || ch == 0)
    {
        cx = cy = 0;
        cw = P->width;
        ch = P->height;
    }
    const uint32_t px0 = cx, py0 = cy;
    cw = (cw + stride - 1) / stride;
    ch = (ch + stride - 1) / stride;
    std::vector<uint32_t> pts((size_t)P->spp_count * 256);
    for (uint32_t s = 0; s < P->spp_count; ++s)
        for (uint32_t d = 0; d < 256; ++d) pts[(size_t)s * 256 + d] = sobolUint(tb.sobol, P->spp_start + s, d);
    const uint32_t tile = 16;
    uint32_t tx = (cw + tile - 1) / tile, ty = (ch + tile - 1) / tile;
    std::atomic<uint32_t> next{0};
    std::atomic<uint64_t> rayTotal{0};
    uint64_t npix = (uint64_t)cw * ch;
    auto t0 = std::chrono::steady_clock::now();
    auto worker = [&]() {
        uint64_t rays = 0;
        for (uint32_t t = next++; t < tx * ty; t = next++)
        {
            uint32_t x0 = (t % tx) * tile, y0 = (t / tx) * tile;
            for (uint32_t y = y0; y < std::min(y0 + tile, ch); ++y)
                for (uint32_t x = x0; x < std::min(x0 + tile, cw); ++x)
                {
                    double acc[3] = {0, 0, 0};
                    for (uint32_t s = 0; s < P->spp_count; ++s)
                    {
                        uint64_t idx = (uint64_t)s * npix + (uint64_t)y * cw + x;
                        V3<T> X;
                        tracePath(c, *P, &pts[(size_t)s * 256], px0 + x * stride, py0 + y * stride,
                                  records ? records + idx * 8 : nullptr, X, rays);
                        acc[0] += (double)X.x;
                        acc[1] += (double)X.y;
                        acc[2] += (double)X.z;
                    }
                    if (film)
                        for (int k = 0; k < 3; ++k) film[((uint64_t)y * cw + x) * 3 + k] = acc[k] / P->spp_count;
                }
        }
        rayTotal += rays;
    };
    int nt = std::max(1, threads);
    std::vector<std::thread> th;
    for (int i = 0; i < nt; ++i) th.emplace_back(worker);
    for (auto& t : th) t.join();
    if (stats)
    {
        stats->rays = rayTotal;
        stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    return 0;
}

#include "oracle_bdpt.inc"
#include "oracle_atrous.inc"

} // namespace orc

extern "C" {

int oracle_render(const oracle_scene* sc, const yg_render_params* P, int precision, int threads, float* records, double* film,
                  oracle_stats* stats)
{
    if (!sc || !P) return -1;
    if (P->integrator > YG_INTEGRATOR_BDPT) return -1;
    if (!sc->rgb_to_spd && orc::needsRgbTable(sc, P)) return -6; // the RGB -> spectrum table was not given
    if (P->integrator == YG_INTEGRATOR_BDPT)
    {
        if (precision == 64) return orc::runBdpt<double>(sc, P, threads, records, film, stats);
        return orc::runBdpt<float>(sc, P, threads, records, film, stats);
    }
    if (precision == 64) return orc::run<double>(sc, P, threads, records, film, stats);
    return orc::run<float>(sc, P, threads, records, film, stats);
}

int oracle_needs_rgb_table(const oracle_scene* sc, const yg_render_params* P)
{
    if (!sc || !P) return -1;
    return orc::needsRgbTable(sc, P) ? 1 : 0;
}

int oracle_render_strided(const oracle_scene* sc, const yg_render_params* P, uint32_t stride, int precision, int threads,
                          double* film, oracle_stats* stats)
{
    if (!sc || !P || stride == 0) return -1;
    if (P->integrator > YG_INTEGRATOR_NEE) return -1; // uni and NEE (BDPT couples pixels through its light paths)
    if (!sc->rgb_to_spd && orc::needsRgbTable(sc, P)) return -6;
    if (precision == 64) return orc::run<double>(sc, P, threads, nullptr, film, stats, stride);
    return orc::run<float>(sc, P, threads, nullptr, film, stats, stride);
}

int oracle_atrous_moments(const oracle_scene* sc, const yg_render_params* P, int threads, float* moments)
{
    if (!sc || !P || !moments) return -1;
    if (!sc->rgb_to_spd && orc::needsRgbTable(sc, P)) return -6;
    return orc::gatherMoments(sc, P, threads, moments);
}

int oracle_atrous(uint32_t width, uint32_t height, const float* film_sum, const float* odd_sum, const float* moments,
                  const yg_camera* camera, const yg_atrous_params* params, int threads, float* out_xyzw, float* out_variance,
                  uint32_t* features)
{
    if (!film_sum || !odd_sum || !moments || !camera || !params || !out_xyzw || !out_variance || !width || !height) return -1;
    orc::ASettings A{params->depth_sigma_scale, params->normal_sigma, params->material_sigma, params->color_sigma,
                     params->feature_variance_scale, params->prefilter != 0, params->passes};
    orc::atrousFilter(width, height, film_sum, odd_sum, moments, *camera, A, threads, out_xyzw, out_variance, features);
    return 0;
}

int oracle_sobol_matrices(const char* dir, uint32_t* out)
{
    std::vector<uint32_t> m;
    if (!orc::sobolMatrices(dir, m)) return -5;
    std::memcpy(out, m.data(), m.size() * 4);
    return 0;
}

int oracle_host_table(const char* data_dir, int which, int lmin, int lmax, void* out, size_t capacity, size_t* count)
{
    if (!data_dir || !count) return -1;
    std::string dir(data_dir), err;
    std::vector<uint32_t> u;
    std::vector<float> f;
    std::vector<double> cie;
    if (which == YG_TABLE_SOBOL_MATRICES)
    {
        if (!yg::buildSobolMatrices(dir + "/joe_kuo_6_21201_first256.txt", u, err)) return -5;
    }
    else if (which >= YG_TABLE_LUT_SS_NOFRESNEL && which <= YG_TABLE_LUT_SHEEN)
    {
        static std::mutex m;
        static yg::MsLuts cache;
        static bool built = false;
        std::lock_guard<std::mutex> g(m);
        if (!built)
        {
            yg::buildMsLuts(cache);
            built = true;
        }
        const std::vector<float>* L[9] = {&cache.ss, &cache.ssAvg, &cache.ssms, &cache.ssmsAvg, &cache.transDenser,
                                          &cache.transLighter, &cache.transAvgDenser, &cache.transAvgLighter, &cache.sheen};
        f = *L[which - YG_TABLE_LUT_SS_NOFRESNEL];
    }
    else if (which == YG_TABLE_RGB_TO_SPD)
    {
        if (!yg::loadCie(dir + "/cie1931_2deg_d65_1nm.txt", cie, err)) return -5;
        if (lmin < 360 || lmax > 830 || lmax <= lmin) return -1;
        yg::buildRgbToSpd(cie, lmin, lmax, f);
    }
    else
    {
        return -1;
    }
    size_t n = u.empty() ? f.size() : u.size();
    *count = n;
    if (!out) return 0;
    if (capacity < n) return -1;
    if (u.empty()) std::memcpy(out, f.data(), n * sizeof(float));
    else std::memcpy(out, u.data(), n * sizeof(uint32_t));
    return 0;
}
}
