// Host-side table generation shared by every consumer of the tracer's tables:
//  * Sobol generator matrices from the Joe & Kuo direction numbers, following the
//    recurrence of Tools/generate_sobol_matrices.py:37-53 (dimension 0 = the
//    bit-reversal identity, :85-90); the per-frame point is sobolUint
//    (Source/Common/inc/Math/RandUtility.inl:34-46).
//  * CIE 1931 / D65 tables resampled to the render's spectral range, and the sums
//    CIE_Y_SUM / CIE_D65_SUM over it (spectralConstants.h:19-26).
//  * Multiple-scattering albedo LUTs (MultipleScatterLUT.cpp:76-489 with the
//    integrands of MultipleScatterLUTUtility.h:200-438 and Common/inc/Math/GGX.h).
//    The reference shuffles the Halton digits of the translucent LUTs with an
//    unseeded RNG, so its tables are not reproducible; these use the plain
//    radical inverse, which makes every build produce identical tables.
//  * The sRGB -> sigmoid-polynomial 64^3 fit (SpectralUtility.cpp:253-609),
//    FP64 Gauss-Newton with CIELAB residuals, generated on first use.
#include "yg_tables.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>

namespace yg
{

// ------------------------------------------------------------------ Sobol
bool buildSobolMatrices(const std::string& joeKuoPath, std::vector<uint32_t>& out, std::string& err)
{
    std::ifstream f(joeKuoPath);
    if (!f)
    {
        err = "cannot open " + joeKuoPath;
        return false;
    }
    out.assign(256 * 32, 0u);
    for (int j = 0; j < 32; ++j) out[j] = 1u << (31 - j);
    std::string line;
    int dim = 1;
    while (dim < 256 && std::getline(f, line))
    {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        long d, s, a;
        if (!(is >> d >> s >> a)) continue;
        std::vector<uint32_t> m(s);
        for (long i = 0; i < s; ++i) is >> m[i];
        uint32_t V[32];
        const int L = 32;
        if (L <= s)
        {
            for (int i = 0; i < L; ++i) V[i] = m[i] << (L - 1 - i);
        }
        else
        {
            for (int i = 0; i < s; ++i) V[i] = m[i] << (L - 1 - i);
            for (int i = (int)s; i < L; ++i)
            {
                V[i] = V[i - s] ^ (V[i - s] >> s);
                for (int k = 1; k < s; ++k)
                    if ((a >> (s - 1 - k)) & 1) V[i] ^= V[i - k];
            }
        }
        for (int j = 0; j < 32; ++j) out[dim * 32 + j] = V[j];
        ++dim;
    }
    if (dim != 256)
    {
        err = "Joe-Kuo file has too few dimensions";
        return false;
    }
    return true;
}

uint32_t sobolUint(const uint32_t* matrices, uint32_t index, uint32_t dim)
{
    uint32_t v = 0;
    for (uint32_t i = dim * 32; index != 0; index >>= 1, ++i)
        if (index & 1) v ^= matrices[i];
    return v;
}

// ------------------------------------------------------------------ CIE
bool loadCie(const std::string& path, std::vector<double>& cie471x4, std::string& err)
{
    std::ifstream f(path);
    if (!f)
    {
        err = "cannot open " + path;
        return false;
    }
    cie471x4.clear();
    std::string line;
    while (std::getline(f, line))
    {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        double l, x, y, z, d;
        if (!(is >> l >> x >> y >> z >> d)) continue;
        cie471x4.push_back(x);
        cie471x4.push_back(y);
        cie471x4.push_back(z);
        cie471x4.push_back(d);
    }
    if (cie471x4.size() != 471 * 4)
    {
        err = "CIE table must have 471 rows";
        return false;
    }
    return true;
}

bool cieForRange(const std::vector<double>& cie, int lmin, int lmax, std::vector<float>& out4, float& ySumInv,
                 float& d65SumInv)
{
    if (lmin < 360 || lmax > 830 || lmax <= lmin) return false;
    int n = lmax - lmin + 1;
    out4.resize((size_t)n * 4);
    double ySum = 0.0, dSum = 0.0;
    for (int i = 0; i < n; ++i)
    {
        int src = lmin - 360 + i;
        for (int c = 0; c < 4; ++c) out4[i * 4 + c] = (float)cie[src * 4 + c];
        ySum += cie[src * 4 + 1];
        dSum += cie[src * 4 + 3];
    }
    ySumInv = (float)(1.0 / ySum);
    d65SumInv = (float)(1.0 / dSum);
    return true;
}

// ------------------------------------------------------------------ MS LUTs (CPU GGX math)
namespace
{
struct V3
{
    float x, y, z;
};
inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
inline float dotp(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 crossp(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 norm(V3 a) { return a * (1.0f / std::sqrt(dotp(a, a))); }
inline float sqrf(float x) { return x * x; }
inline float sat(float x) { return std::min(std::max(x, 0.0f), 1.0f); }
inline float sdiv(float a, float b) { return b == 0.0f ? 0.0f : a / b; }
inline V3 reflectp(V3 i, V3 n) { return i - n * (2.0f * dotp(n, i)); }
inline V3 refractp(V3 i, V3 n, float eta)
{
    float ni = dotp(n, i);
    float k = 1.0f - eta * eta * (1.0f - ni * ni);
    if (k < 0.0f) return v3(0, 0, 0);
    return i * eta - n * (eta * ni + std::sqrt(k));
}
const float PI_F = 3.14159265f;

float smithLambda(V3 d, float ax, float ay)
{
    float s = 1.0f + (d.x * d.x * ax * ax + d.z * d.z * ay * ay) / (d.y * d.y);
    return (std::sqrt(s) - 1.0f) * 0.5f;
}
float G1(V3 wo, V3 wm, float ax, float ay) { return (dotp(wo, wm) >= 0.f ? 1.f : 0.f) / (1.0f + smithLambda(wo, ax, ay)); }
float G2(V3 wo, V3 wi, V3 wm, float ax, float ay)
{
    float nom = dotp(wo, wm) >= 0.f ? 1.f : 0.f;
    return nom / (1.f + smithLambda(wi, ax, ay) + smithLambda(wo, ax, ay));
}
float DG(V3 wm, float ax, float ay)
{
    ax = std::max(ax, 0.000001f);
    ay = std::max(ay, 0.000001f);
    float d = sqrf(sdiv(wm.x, ax)) + sqrf(sdiv(wm.z, ay)) + sqrf(wm.y);
    d *= d;
    d *= ax * ay * PI_F;
    return sdiv(1.0f, d);
}
float DV(V3 wo, V3 wm, float ax, float ay) { return sdiv(G1(wo, wm, ax, ay) * std::fabs(dotp(wo, wm)) * DG(wm, ax, ay), std::fabs(wo.y)); }
V3 sampleVNDF(V3 wo, float ax, float ay, float u1, float u2)
{
    V3 Vh = norm(v3(ax * wo.x, ay * wo.z, wo.y));
    float lensq = Vh.x * Vh.x + Vh.y * Vh.y;
    V3 T1 = lensq > 0 ? v3(-Vh.y, Vh.x, 0) * (1.f / std::sqrt(lensq)) : v3(1, 0, 0);
    V3 T2 = crossp(Vh, T1);
    float r = std::sqrt(u1);
    float phi = 2.0f * PI_F * u2;
    float t1 = r * std::cos(phi), t2 = r * std::sin(phi);
    float s = 0.5f * (1.0f + Vh.z);
    t2 = (1.0f - s) * std::sqrt(1.0f - t1 * t1) + s * t2;
    V3 Nh = T1 * t1 + T2 * t2 + Vh * std::sqrt(std::max(0.f, 1.f - t1 * t1 - t2 * t2));
    return norm(v3(ax * Nh.x, std::max(0.0f, Nh.z), ay * Nh.y));
}
V3 sampleWM(V3 wo, float ax, float ay, float u1, float u2)
{
    V3 wh = sampleVNDF(wo, ax, ay, u1, u2);
    if (wo.y * wh.y < 0) wh = -wh;
    return wh;
}
float jRefl(V3 wi, V3 wm) { return sdiv(1.f, 4 * sat(dotp(wi, wm))); }
float jRefr(float eta, V3 wo, V3 wm, V3 wi)
{
    float mo = dotp(wo, wm), mi = std::fabs(dotp(wi, wm));
    return sdiv(sqrf(eta) * mi, sqrf(mo + eta * mi));
}
float fresnelDD(float eta, float cosTheta)
{
    float c = sat(cosTheta);
    float temp = eta * eta + c * c - 1.f;
    if (temp < 0.f) return 1.f;
    float g = std::sqrt(temp);
    return 0.5f * sqrf((g - c) / std::max(g + c, 0.000001f)) * (1 + sqrf(((g + c) * c - 1.f) / ((g - c) * c + 1.f)));
}
float ensureValidEta(float e) { return e > 1 ? std::max(e, 1.01f) : std::min(e, 0.99f); }
float vdc(uint32_t i)
{
    i = (i << 16) | (i >> 16);
    i = ((i & 0x55555555u) << 1) | ((i & 0xAAAAAAAAu) >> 1);
    i = ((i & 0x33333333u) << 2) | ((i & 0xCCCCCCCCu) >> 2);
    i = ((i & 0x0F0F0F0Fu) << 4) | ((i & 0xF0F0F0F0u) >> 4);
    i = ((i & 0x00FF00FFu) << 8) | ((i & 0xFF00FF00u) >> 8);
    return float(i) * (float)(1.0 / 4294967295.0);
}
float radicalInverse(uint32_t base, uint32_t i)
{
    double inv = 1.0 / base, f = inv, r = 0.0;
    while (i > 0)
    {
        r += f * (i % base);
        i /= base;
        f *= inv;
    }
    return (float)std::min(r, 0.99999994039535522);
}
float lutSample2(V3 uv, const float* lut, int dim) // sampleLut 2D (MultipleScatterLUTUtility.h:44-67), uv.x/uv.y
{
    float u = sat(uv.x), v = sat(uv.y);
    float vx = std::min(u * dim, float(dim - 1)), vy = std::min(v * dim, float(dim - 1));
    auto at = [&](float x, float y) { return lut[size_t(y * dim + x)]; };
    float a = at(std::floor(vx), std::floor(vy)), b = at(std::ceil(vx), std::floor(vy));
    float c = at(std::floor(vx), std::ceil(vy)), d = at(std::ceil(vx), std::ceil(vy));
    float tx = vx - std::floor(vx), ty = vy - std::floor(vy);
    float ab = (1.f - tx) * a + tx * b, cd = (1.f - tx) * c + tx * d;
    return (1.f - ty) * ab + ty * cd;
}
float lutSample1(float u, const float* lut, int dim)
{
    u = sat(u);
    float v = std::min(u * dim, float(dim - 1));
    float a = lut[(uint32_t)std::floor(v)], b = lut[(uint32_t)std::ceil(v)];
    float t = v - std::floor(v);
    return (1.f - t) * a + t * b;
}
float integrateAverageAlbedo(const float* A, int dim)
{
    float h = 1.f / float(dim - 1), avg = 0.f;
    for (int x = 0; x + 1 < dim; ++x)
    {
        float a = float(x) * h, b = float(x + 1) * h;
        avg += h * (A[x] * (2.f * a + b) + A[x + 1] * (a + 2.f * b)) / 6.f;
    }
    return 2.f * avg;
}

float ssNoFresnel(float roughness, float cosTheta)
{
    const uint32_t N = 256;
    float acc = 0;
    roughness = std::max(0.01f, roughness);
    float a = roughness * roughness;
    V3 wo = v3(std::sqrt(1.f - sqrf(cosTheta)), cosTheta, 0);
    for (uint32_t i = 0; i < N; ++i)
    {
        V3 wm = sampleWM(wo, a, a, vdc(i), float(i) / float(N));
        V3 wi = reflectp(-wo, wm);
        if (wi.y <= 0.0f || dotp(wi, wm) <= 0.f || dotp(wo, wm) <= 0.f) continue;
        float w = G2(wo, wi, wm, a, a) * DG(wm, a, a) / std::max(4.f * wo.y * wi.y, 0.000001f);
        float pdf = DV(wo, wm, a, a) * jRefl(wo, wm);
        if (pdf > 0.f) acc += w * std::fabs(wi.y) / pdf;
    }
    return acc / N;
}
float ssmsAlbedo(float roughness, float cosTheta, float etaR, const float* ss, const float* ssAvg)
{
    const uint32_t N = 256;
    float acc = 0;
    roughness = std::max(0.01f, roughness);
    float a = roughness * roughness;
    etaR = ensureValidEta(etaR);
    V3 wo = v3(std::sqrt(1.f - sqrf(cosTheta)), cosTheta, 0);
    for (uint32_t i = 0; i < N; ++i)
    {
        V3 wm = sampleWM(wo, a, a, vdc(i), float(i) / float(N));
        V3 wi = reflectp(-wo, wm);
        if (wi.y < 0.0f || dotp(wi, wm) < 0.f || dotp(wo, wm) < 0.f) continue;
        float F = fresnelDD(etaR, dotp(wo, wm));
        float w = F * G2(wo, wi, wm, a, a) * DG(wm, a, a) / std::max(4.f * wo.y * wi.y, 0.000001f);
        float pdf = DV(wo, wm, a, a) * jRefl(wo, wm);
        // Kulla-Conty compensation (getEnergyCompensationKulla, MultipleScatterLUTUtility.h:97-110)
        float dWo = sat(cosTheta), dWi = sat(wi.y);
        float eo = 1.f - lutSample2(v3(dWo, roughness, 0), ss, kLutSS);
        float ei = 1.f - lutSample2(v3(dWi, roughness, 0), ss, kLutSS);
        float eAvg = lutSample1(roughness, ssAvg, kLutSS);
        float ems = eo * ei / std::max(0.0001f, (1.f - eAvg) * PI_F);
        w += F * ems;
        if (pdf > 0.f) acc += w * std::fabs(wi.y) / pdf;
    }
    return acc / N;
}
V3 wmTranslucent(V3 wo, V3 wi, float etaR)
{
    if (wi.y >= 0.f) return norm(wo + wi);
    if (etaR == 1.f) etaR = 1.0001f;
    V3 wm = norm(wo + wi * etaR);
    if (wo.y * wm.y < 0) wm = wm * -1.f;
    return wm;
}
float translucentAlbedo(float etaR, float roughness, float cosTheta)
{
    const uint32_t N = 1024;
    float acc = 0;
    etaR = ensureValidEta(etaR);
    roughness = std::max(0.01f, roughness);
    float a = roughness * roughness;
    V3 wo = v3(std::sqrt(1.f - sqrf(cosTheta)), cosTheta, 0);
    for (uint32_t i = 0; i < N; ++i)
    {
        float sx = radicalInverse(2, i), sy = radicalInverse(3, i), sz = radicalInverse(5, i);
        // sampleGGXDielectricTranslucent (GGX.h:195-236)
        V3 wm = sampleWM(wo, a, a, sx, sy);
        float e = etaR == 1.f ? 1.0001f : etaR;
        float F = fresnelDD(e, dotp(wo, wm));
        if (dotp(wo, wm) < 0.f) continue;
        V3 wi;
        if (sz < F)
        {
            wi = reflectp(-wo, wm);
            if (wi.y <= 0.f) continue;
        }
        else
        {
            wi = refractp(-wo, wm, 1.f / e);
            if (wi.y > 0) continue;
        }
        if (dotp(wi, wi) == 0.f) continue;
        // pdfGGXDielectricTranslucent (GGX.h:238-263)
        bool refl = wi.y >= 0.f;
        V3 wmp = wmTranslucent(wo, wi, etaR);
        if (dotp(wo, wmp) <= 0.f) continue;
        float Fp = fresnelDD(etaR, dotp(wo, wmp));
        float pdf = DV(wo, wmp, a, a) * (refl ? Fp * jRefl(wo, wmp) : (1.f - Fp) * jRefr(etaR, wo, wmp, wi));
        // evaluateGGXDielectricTranslucent (GGX.h:265-292)
        float VdotH = sat(dotp(wo, wmp));
        float Fe = fresnelDD(etaR, VdotH);
        float g2 = G2(wo, wi, wmp, a, a), d = DG(wmp, a, a), w;
        if (refl) w = Fe * g2 * d / (4.f * wo.y * wi.y);
        else
        {
            if (dotp(wo, wmp) * dotp(wi, wmp) > 0) continue;
            w = sdiv((1.f - Fe) * g2 * d * VdotH * jRefr(etaR, wo, wmp, wi), std::fabs(wo.y * wi.y));
        }
        if (pdf > 0.f) acc += w * std::fabs(wi.y) / pdf;
    }
    return acc / N;
}
float sheenAlbedo(float roughness, float cosTheta)
{
    const uint32_t N = 256;
    float acc = 0;
    roughness = std::max(0.01f, roughness);
    float a = std::max(roughness, 0.07f);
    V3 wo = v3(std::sqrt(1.f - sqrf(cosTheta)), cosTheta, 0);
    auto GL = [](float x, float A, float B, float C, float D, float E) { return (A / (1 + B * std::pow(x, C))) + D * x + E; };
    auto GLambda = [&](float r, float c) {
        float t = (1.f - r) * (1.f - r);
        float A = 21.5473f + t * (25.3245f - 21.5473f), B = 3.82987f + t * (3.32435f - 3.82987f);
        float C = 0.19823f + t * (0.16801f - 0.19823f), D = -1.97760f + t * (-1.27393f + 1.97760f);
        float E = -4.32054f + t * (-4.85967f + 4.32054f);
        float ex = c < 0.5f ? GL(c, A, B, C, D, E) : 2.f * GL(0.5f, A, B, C, D, E) - GL(1.f - c, A, B, C, D, E);
        return std::exp(ex);
    };
    for (uint32_t i = 0; i < N; ++i)
    {
        float sx = vdc(i), sy = float(i) / float(N);
        float z = sx, r = std::sqrt(1.f - z * z), phi = 2.f * PI_F * sy;
        V3 wi = v3(r * std::cos(phi), z, r * std::sin(phi));
        V3 wm = norm(wi + wo);
        if (wi.y <= 0.0f) continue;
        float G = 1.f / (1.f + GLambda(a, wi.y) + GLambda(a, wo.y));
        float rInv = 1.f / a;
        float D = (2.f + rInv) * std::pow(1.f - wm.y * wm.y, rInv * 0.5f) / (2.f * PI_F);
        float pdf = 1.f / (2.f * PI_F);
        float w = G * D / std::max(4.f * wo.y * wi.y, 0.000001f);
        acc += w * std::fabs(wi.y) / pdf;
    }
    return acc / N;
}

template <typename F>
void parallelFor(int n, F&& fn)
{
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int nt = (int)std::min<unsigned>(hw, (unsigned)n);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
        th.emplace_back([&, t]() {
            for (int i = t; i < n; i += nt) fn(i);
        });
    for (auto& x : th) x.join();
}
} // namespace

void buildMsLuts(MsLuts& L)
{
    const int S = kLutSS, M = kLutSSMS, T = kLutTrans, H = kLutSheen;
    const float minCos = 0.001f;
    L.ss.assign(S * S, 0.f);
    L.ssAvg.assign(S, 0.f);
    parallelFor(S, [&](int y) {
        for (int x = 0; x < S; ++x)
        {
            float c = float(x) / (S - 1), r = float(y) / (S - 1);
            L.ss[y * S + x] = ssNoFresnel(r, std::max(c, minCos));
        }
        L.ssAvg[y] = integrateAverageAlbedo(&L.ss[y * S], S);
    });
    L.ssms.assign(M * M * M, 0.f);
    L.ssmsAvg.assign(M * M, 0.f);
    parallelFor(M, [&](int z) {
        for (int y = 0; y < M; ++y)
        {
            float r = float(y) / (M - 1);
            for (int x = 0; x < M; ++x)
            {
                float c = float(x) / (M - 1);
                float eta = 1.f + (float(z) / (M - 1)) * 3.f;
                eta = std::max(eta, 1.01f);
                L.ssms[(z * M + y) * M + x] = ssmsAlbedo(r, std::max(c, minCos), eta, L.ss.data(), L.ssAvg.data());
            }
            L.ssmsAvg[z * M + y] = integrateAverageAlbedo(&L.ssms[(z * M + y) * M], M);
        }
    });
    L.transDenser.assign(T * T * T, 0.f);
    L.transLighter.assign(T * T * T, 0.f);
    L.transAvgDenser.assign(T * T, 0.f);
    L.transAvgLighter.assign(T * T, 0.f);
    parallelFor(2 * T, [&](int job) {
        bool dense = job < T;
        int z = dense ? job : job - T;
        float scale = dense ? 3.f : 0.69f, bias = dense ? 1.f : 0.3f;
        float emin = dense ? 1.0001f : 0.3f, emax = dense ? 4.0f : 0.99f;
        std::vector<float>& D = dense ? L.transDenser : L.transLighter;
        std::vector<float>& A = dense ? L.transAvgDenser : L.transAvgLighter;
        for (int y = 0; y < T; ++y)
        {
            float r = float(y) / (T - 1);
            for (int x = 0; x < T; ++x)
            {
                float c = float(x) / (T - 1);
                float eta = std::min(std::max(scale * (float(z) / (T - 1)) + bias, emin), emax);
                D[(z * T + y) * T + x] = translucentAlbedo(eta, r, std::max(c, minCos));
            }
            A[z * T + y] = integrateAverageAlbedo(&D[(z * T + y) * T], T);
        }
    });
    L.sheen.assign(H * H, 0.f);
    parallelFor(H, [&](int y) {
        for (int x = 0; x < H; ++x)
        {
            float c = float(x) / (H - 1), r = float(y) / (H - 1);
            L.sheen[y * H + x] = sheenAlbedo(r, std::max(c, minCos));
        }
    });
}

// ------------------------------------------------------------------ RGB -> SPD (SpectralUtility.cpp:253-609)
namespace
{
struct D3
{
    double v[3];
};
const double kSrgbXYZToRGB[9] = {3.2406, -1.5372, -0.4986, -0.9689, 1.8758, 0.0415, 0.0557, -0.2040, 1.0570};
const double kSrgbRGBToXYZ[9] = {0.4124, 0.3576, 0.1805, 0.2126, 0.7152, 0.0722, 0.0193, 0.1192, 0.9505};

D3 mat3(const double* m, const D3& x)
{
    D3 r;
    for (int i = 0; i < 3; ++i) r.v[i] = m[i * 3] * x.v[0] + m[i * 3 + 1] * x.v[1] + m[i * 3 + 2] * x.v[2];
    return r;
}
D3 toLab(const D3& rgb)
{
    const double Xn = 95.047f, Yn = 100.0, Zn = 108.883f; // float constants, as in the reference
    const double delta = (double)(float)(6.0 / 29.0);
    const double delta3 = (double)(float)(delta * delta * delta);
    D3 xyz = mat3(kSrgbRGBToXYZ, rgb);
    double n[3] = {xyz.v[0] / Xn, xyz.v[1] / Yn, xyz.v[2] / Zn}, ft[3];
    for (int i = 0; i < 3; ++i) ft[i] = n[i] > delta3 ? std::pow(n[i], 1.0 / 3.0) : n[i] / (3.0 * delta * delta) + 4.0 / 29.0;
    return D3{{116.0 * ft[1] - 16, 500 * (ft[0] - ft[1]), 200 * (ft[1] - ft[2])}};
}
D3 residual(const D3& expected, const D3& coeffs, const std::vector<D3>& toRGB)
{
    D3 est{{0, 0, 0}};
    size_t n = toRGB.size();
    for (size_t i = 0; i < n; ++i)
    {
        double lam = double(i) / double(n - 1);
        double poly = 0;
        for (int k = 0; k < 3; ++k) poly = poly * lam + coeffs.v[k];
        double s = 0.5 * poly / std::sqrt(1.0 + poly * poly) + 0.5;
        for (int c = 0; c < 3; ++c) est.v[c] += s * toRGB[i].v[c];
    }
    D3 a = toLab(expected), b = toLab(est);
    return D3{{a.v[0] - b.v[0], a.v[1] - b.v[1], a.v[2] - b.v[2]}};
}
bool inverse3(const double J[3][3], double inv[3][3])
{
    double det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) - J[1][0] * (J[0][1] * J[2][2] - J[2][1] * J[0][2]) +
                 J[2][0] * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
    if (det == 0.0) return false;
    double id = 1.0 / det;
    // inverse of the matrix with entries J[row][col]
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) * id;
    inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
    inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    return true;
}
} // namespace

void buildRgbToSpd(const std::vector<double>& cie, int lmin, int lmax, std::vector<float>& out)
{
    const int R = kRgbLutRes;
    int n = lmax - lmin + 1;
    std::vector<D3> toRGB(n);
    double d65YSum = 0.0;
    for (int i = 0; i < n; ++i)
    {
        int s = lmin - 360 + i;
        d65YSum += cie[s * 4 + 1] * cie[s * 4 + 3];
    }
    for (int i = 0; i < n; ++i)
    {
        int s = lmin - 360 + i;
        D3 xyz{{cie[s * 4] * cie[s * 4 + 3] / d65YSum, cie[s * 4 + 1] * cie[s * 4 + 3] / d65YSum,
                cie[s * 4 + 2] * cie[s * 4 + 3] / d65YSum}};
        toRGB[i] = mat3(kSrgbXYZToRGB, xyz);
    }
    out.assign((size_t)R * R * R * 3, 0.f);
    parallelFor(R, [&](int z) {
        for (int y = 0; y < R; ++y)
            for (int x = 0; x < R; ++x)
            {
                D3 rgb{{double(x) / (R - 1), double(y) / (R - 1), double(z) / (R - 1)}};
                D3 c{{0, 0, 0}};
                for (int it = 0; it < 16; ++it)
                {
                    D3 r = residual(rgb, c, toRGB);
                    double J[3][3]; // J[row = residual comp][col = coefficient]
                    for (int k = 0; k < 3; ++k)
                    {
                        D3 cm = c, cp = c;
                        cm.v[k] -= 1e-4;
                        cp.v[k] += 1e-4;
                        D3 r0 = residual(rgb, cm, toRGB), r1 = residual(rgb, cp, toRGB);
                        for (int q = 0; q < 3; ++q) J[q][k] = (r1.v[q] - r0.v[q]) / (2.0 * 1e-4);
                    }
                    double inv[3][3];
                    if (!inverse3(J, inv)) break;
                    for (int q = 0; q < 3; ++q) c.v[q] -= inv[q][0] * r.v[0] + inv[q][1] * r.v[1] + inv[q][2] * r.v[2];
                    double err = r.v[0] * r.v[0] + r.v[1] * r.v[1] + r.v[2] * r.v[2];
                    if (err < 1e-6) break;
                    double mx = std::max(std::max(c.v[0], c.v[1]), c.v[2]);
                    if (mx > 200)
                        for (int q = 0; q < 3; ++q) c.v[q] *= 200 / mx;
                }
                size_t o = ((size_t)(z * R + y) * R + x) * 3;
                out[o] = (float)c.v[0];
                out[o + 1] = (float)c.v[1];
                out[o + 2] = (float)c.v[2];
            }
    });
}

} // namespace yg
