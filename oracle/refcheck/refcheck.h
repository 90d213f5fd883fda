// TEST INFRASTRUCTURE ONLY: the functions compared between the reference's shader math
// (hlsl_side.cpp, prefix ref_) and the oracle's restatement (oracle_side.cpp, prefix orc_),
// with plain arguments so that neither side sees the other's types.
#pragma once
#include <cstdint>

namespace refcheck
{
// tables both sides read: the nine multiple-scattering / sheen LUTs (single channel), the
// CIE x, y, z, D65 table for 380..700 nm at 1 nm (321 x 4), the sRGB -> sigmoid fit (64^3 x 3)
struct Tables
{
    const float* lut[9];
    const float* cie321x4;
    const float* rgb64;
    const uint32_t* sobolPoint; // 256 dimensions of one sample index
};

// the fields of SurfaceDefinition (hitShadersCommon.hlsl:13-47), spectral values at the
// four wavelengths of the sample
struct Surface
{
    float specular[4], albedo[4], absorption[4], emissive[4], sheenColor[4];
    float coatN[3], baseN[3], geoN[3], tangent[3];
    float transparency, metalness, ior, roughness, cauchyA, cauchyB, specAmount, ccAmount, ccIOR, ccRough;
    float aniso, anisoRot, thinFilm, sheenRough, sheenAmount, focus, sssAmount;
    float diffOcc, specOcc;
    uint32_t flags;
    float sssRadius[4]; // subsurfaceRadius per lane
};
struct Eval
{
    float w[4];
    float pdf;
    uint32_t trans;
};

#define REFCHECK_API(P)                                                                                          \
    void P##setup(const Tables& t);                                                                              \
    uint32_t P##hash2(uint32_t a, uint32_t b);                                                                   \
    uint32_t P##owen(uint32_t v, uint32_t seed);                                                                 \
    float P##u01(uint32_t v);                                                                                    \
    void P##sampler(uint32_t pixelSeed, uint32_t n, float* out); /* getTexelOffset, then n x getRandom1 */      \
    void P##lambdas(float u, float out[4]);                                                                      \
    float P##sigmoid(float x);                                                                                   \
    void P##rgb_spectrum(int mode, const float rgb[3], float hero, float out[4]);                                \
    void P##to_xyz(float hero, const float L[4], float out[3]);                                                  \
    int P##roulette(const float w[4], float rand, float norm, float out[4]);                                     \
    float P##lambda_ggx(const float d[3], float ax, float ay);                                                    \
    float P##g1(const float wo[3], const float wm[3], float ax, float ay);                                       \
    float P##g2(const float wo[3], const float wi[3], const float wm[3], float ax, float ay);                     \
    float P##dggx(const float wm[3], float ax, float ay);                                                        \
    float P##dv(const float wo[3], const float wm[3], float ax, float ay);                                       \
    void P##sample_wm(const float wo[3], float ax, float ay, float u1, float u2, float out[3]);                  \
    void P##conductor_nk(float r, float g, float out[2]);                                                        \
    float P##fresnel_dc(float er, float ei, float c);                                                            \
    float P##fresnel_dd(float eta, float c);                                                                     \
    float P##dsheen(const float wm[3], float r);                                                                 \
    float P##gsheen(const float wo[3], const float wi[3], float r);                                              \
    float P##emission_profile(float d, float e);                                                                 \
    void P##concentric_disk(float u0, float u1, float out[2]);                                                   \
    void P##sample_lobe(int lobe, float eta, float ax, float ay, const float wo[3], float s0, float s1, float sc, \
                        int aR, int aT, float out[3]);                                                          \
    float P##pdf_lobe(int lobe, float eta, float ax, float ay, const float wo[3], const float wi[3], int aR,     \
                      int aT);                                                                                   \
    float P##eval_lobe(int lobe, float eta, float k, float ax, float ay, const float wo[3], const float wi[3]);   \
    float P##ms(int fn, float eta, float dWo, float dWi, float lr, float x);                                     \
    void P##layer_probs(const Surface& s, float cur, float prev, const float wo[3], int front, float out[6]);    \
    Eval P##eval_surface(const Surface& s, float hero, float cur, float prev, const float wo[3], int front,      \
                         const float wi[3], uint32_t flags);                                                     \
    void P##sample_layer(const Surface& s, float hero, float cur, float prev, const float wo[3], int front,      \
                         int layer, float sel, float r0, float r1, float out[3], int* diffuse, int* delta);        \
    float P##sss(int fn, float a, float b);                                                                      \
    float P##sss_pdf(const Surface& s, const float fromP[3], const float fromN[3], const float toP[3],          \
                     const float toN[3]);                                                                        \
    float P##sss_entry(const Surface& s, float hero, float cur, float prev, const float wo[3], int front);      \
    void P##sss_exit_lobe(const Surface& s, float cur, float prev, const float wo[3], int front, float r0,      \
                          float r1, const float wi[3], uint32_t flags, float out[8]);

REFCHECK_API(ref_)
REFCHECK_API(refK_)
REFCHECK_API(orc_)
// the oracle's bidirectional-integrator model (Kulla-Conty, evalSurfaceF<T, true>)
Eval orcK_eval_surface(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, const float wi[3],
                       uint32_t flags);
void orcK_sample_layer(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, int layer,
                       float sel, float r0, float r1, float out[3], int* diffuse, int* delta);
} // namespace refcheck
