// TEST INFRASTRUCTURE ONLY: the oracle's restatement (oracle.cpp, compiled into this
// translation unit) behind the plain functions of refcheck.h (prefix orc_), for the
// comparison with the reference's own shader math.
#include "../oracle.cpp"

#include "refcheck.h"

namespace refcheck
{
using namespace orc;

namespace
{
Tables g_t;
orc::Tables g_tb;
oracle_scene g_scene;
yg_camera g_cam;
Ctx<float> g_ctx;
LutSet<float> g_luts;

V3<float> v(const float* p) { return v3(p[0], p[1], p[2]); }
void put(V3<float> a, float* o) { o[0] = a.x; o[1] = a.y; o[2] = a.z; }
S4<float> s4(const float* p) { return S4<float>{{p[0], p[1], p[2], p[3]}}; }
Spec<float> specOf(float hero)
{
    Spec<float> s;
    s.hero = hero;
    float step = (g_ctx.lmax - g_ctx.lmin) / 4.0f, prev = hero;
    s.lam[0] = prev;
    for (int i = 1; i < 4; ++i)
    {
        float l = prev + step;
        if (l > g_ctx.lmax) l = g_ctx.lmin + (l - g_ctx.lmax);
        prev = l;
        s.lam[i] = prev;
    }
    return s;
}
Surf<float> surfOf(const Surface& x)
{
    Surf<float> s;
    s.specular = s4(x.specular);
    s.albedo = s4(x.albedo);
    s.absorption = s4(x.absorption);
    s.emissive = s4(x.emissive);
    s.sheenColor = s4(x.sheenColor);
    s.coatN = v(x.coatN);
    s.baseN = v(x.baseN);
    s.geoN = v(x.geoN);
    s.tangent = v(x.tangent);
    s.transparency = x.transparency;
    s.metalness = x.metalness;
    s.ior = x.ior;
    s.roughness = x.roughness;
    s.cauchyA = x.cauchyA;
    s.cauchyB = x.cauchyB;
    s.specAmount = x.specAmount;
    s.ccAmount = x.ccAmount;
    s.ccIOR = x.ccIOR;
    s.ccRough = x.ccRough;
    s.aniso = x.aniso;
    s.anisoRot = x.anisoRot;
    s.thinFilm = x.thinFilm;
    s.sheenRough = x.sheenRough;
    s.sheenAmount = x.sheenAmount;
    s.focus = x.focus;
    s.sssAmount = x.sssAmount;
    // the occlusion factors travel packed as halves (packOcclusion, materialsCommon.hlsl:302-311)
    s.diffOcc = floatFromHalf(halfFromFloat(x.diffOcc));
    s.specOcc = floatFromHalf(halfFromFloat(x.specOcc));
    s.flags = x.flags;
    s.sssRadius = s4(x.sssRadius);
    return s;
}
} // namespace

void orc_setup(const Tables& t)
{
    g_t = t;
    static std::string dir;
    const char* d = std::getenv("YAPT_DATA_DIR");
    dir = d ? d : "yapt_gb300/data";
    loadCie(dir, g_tb.cie);
    std::memset(&g_scene, 0, sizeof(g_scene));
    std::memset(&g_cam, 0, sizeof(g_cam));
    g_scene.camera = &g_cam;
    for (int i = 0; i < 9; ++i) g_scene.luts[i] = t.lut[i];
    g_scene.rgb_to_spd = t.rgb64;
    g_scene.data_dir = dir.c_str();
    setup(g_ctx, &g_scene, &g_tb, 380.0f, 700.0f);
    for (int i = 0; i < 9; ++i) g_luts.L[i] = t.lut[i];
}

uint32_t orc_hash2(uint32_t a, uint32_t b) { return hashAB(a, b); }
uint32_t orc_owen(uint32_t x, uint32_t seed) { return owenFast(x, seed); }
float orc_u01(uint32_t x) { return toFloat01(x); }
void orc_sampler(uint32_t pixelSeed, uint32_t n, float* out)
{
    Sampler rs{g_t.sobolPoint, 2u, pixelSeed};
    out[0] = rs.get(0);
    out[1] = rs.get(1);
    for (uint32_t i = 0; i < n; ++i) out[2 + i] = rs.r1();
}
void orc_lambdas(float u, float out[4])
{
    Spec<float> s = specOf(g_ctx.lmin + u * (g_ctx.lmax - g_ctx.lmin));
    for (int k = 0; k < 4; ++k) out[k] = s.lam[k];
}
float orc_sigmoid(float x) { return sigmoid(x); }
void orc_rgb_spectrum(int mode, const float rgb[3], float hero, float out[4])
{
    Spec<float> s = specOf(hero);
    S4<float> r = mode == 0 ? setFromRGB(g_ctx, s, v(rgb))
                            : (mode == 1 ? setFromRGBUnbounded(g_ctx, s, v(rgb)) : setFromRGBUnboundedNoIllum(g_ctx, s, v(rgb)));
    for (int k = 0; k < 4; ++k) out[k] = r[k];
}
void orc_to_xyz(float hero, const float L[4], float out[3]) { put(toXYZ(g_ctx, specOf(hero), s4(L)), out); }
int orc_roulette(const float w[4], float rand, float norm, float out[4])
{
    // as in the oracle's bounce loop (applyRussianRoulette)
    S4<float> t = s4(w);
    float pmax = tmax(tmax(tmax(t[0], t[1]), t[2]), t[3]) / norm;
    pmax = clampT(pmax, 0.05f, 1.0f);
    if (rand > pmax)
    {
        for (int k = 0; k < 4; ++k) out[k] = t[k];
        return 1;
    }
    t = t * (1.0f / pmax);
    for (int k = 0; k < 4; ++k) out[k] = t[k];
    return 0;
}
float orc_lambda_ggx(const float d[3], float ax, float ay) { return lambdaGGX(v(d), ax, ay); }
float orc_g1(const float wo[3], const float wm[3], float ax, float ay) { return G1(v(wo), v(wm), ax, ay); }
float orc_g2(const float wo[3], const float wi[3], const float wm[3], float ax, float ay) { return G2(v(wo), v(wi), v(wm), ax, ay); }
float orc_dggx(const float wm[3], float ax, float ay) { return DGGX(v(wm), ax, ay); }
float orc_dv(const float wo[3], const float wm[3], float ax, float ay) { return DV(v(wo), v(wm), ax, ay); }
void orc_sample_wm(const float wo[3], float ax, float ay, float u1, float u2, float out[3]) { put(sampleWM(v(wo), ax, ay, u1, u2), out); }
void orc_conductor_nk(float r, float g, float out[2]) { conductorNK2(r, g, out[0], out[1]); }
float orc_fresnel_dc(float er, float ei, float c) { return fresnelDC(er, ei, c); }
float orc_fresnel_dd(float eta, float c) { return fresnelDD(eta, c); }
float orc_dsheen(const float wm[3], float r) { return DSheen(v(wm), r); }
float orc_gsheen(const float wo[3], const float wi[3], float r) { return GSheen(v(wo), v(wi), r); }
float orc_emission_profile(float d, float e) { return emissionProfile(d, e); }
void orc_concentric_disk(float u0, float u1, float out[2]) { concentricDisk(u0, u1, out[0], out[1]); }
void orc_sample_lobe(int lobe, float eta, float ax, float ay, const float wo[3], float s0, float s1, float sc, int aR, int aT,
                     float out[3])
{
    V3<float> w = v(wo), r = v3(0.0f, 0.0f, 0.0f);
    switch (lobe)
    {
    case 0: r = sampleCondRefl(ax, ay, w, s0, s1); break;
    case 1: r = sampleDielRefl(ax, ay, w, s0, s1); break;
    case 2: r = sampleDiel(eta, ax, ay, w, s0, s1, 1.0f, false, true); break;
    case 3: r = sampleDiel(eta, ax, ay, w, s0, s1, sc, aR != 0, aT != 0); break;
    case 4: r = cosHemi(s0, s1); break;
    case 5: r = deltaSheen(ax) ? reflect(-w, v3(0.0f, 1.0f, 0.0f)) : cosHemi(s0, s1); break;
    }
    if ((lobe == 4 || lobe == 5) && r.y < 0.0f) r = v3(0.0f, 0.0f, 0.0f);
    put(r, out);
}
float orc_pdf_lobe(int lobe, float eta, float ax, float ay, const float wo[3], const float wi[3], int aR, int aT)
{
    V3<float> o = v(wo), i = v(wi);
    switch (lobe)
    {
    case 0: return pdfCondRefl(o, i, ax, ay);
    case 1: return pdfDielRefl(o, i, ax, ay);
    case 2: return pdfTrans(eta, o, i, ax, ay);
    case 3: return pdfDiel(eta, o, i, ax, ay, aR != 0, aT != 0);
    case 4: return pdfCosHemi(i.y);
    case 5: return i.y < 0.0f ? 0.0f : (deltaSheen(ax) ? 1.0f : pdfCosHemi(i.y));
    }
    return 0.0f;
}
// the conductor and Lambertian lobes are evaluated inside evalSurfaceF (compared there)
float orc_eval_lobe(int lobe, float eta, float k, float ax, float ay, const float wo[3], const float wi[3])
{
    (void)k;
    V3<float> o = v(wo), i = v(wi);
    switch (lobe)
    {
    case 1: return evalDielRefl(eta, ax, ay, o, i);
    case 2: return evalTrans(eta, ax, ay, o, i);
    case 5: return evalSheen(sp(eta), ax, o, i)[0];
    }
    return 0.0f;
}
// multiple scattering: 0 Turquin, 1 Kulla, 2 energy after the specular layer, 3 after sheen,
// 4 translucent Turquin, 5 translucent Kulla, 6 average Fresnel, 7 transmission ratio,
// 8 Fms of a dielectric (Turquin model), 9 sheen albedo, 10 translucent directional albedo,
// 11 translucent average albedo
float orc_ms(int fn, float a, float dWo, float dWi, float lr, float x)
{
    switch (fn)
    {
    case 0: return energyComp(g_luts, a, std::fabs(dWo), std::fabs(dWi), lr, x);
    case 1: return energyCompKulla(g_luts, a, dWo, dWi, lr);
    case 2: return energyAfterSpec(g_luts, a, dWo, lr, x);
    case 3: return 1.0f - g_luts.sheen(std::fabs(dWo), lr) * x;
    case 4: return energyCompTrans(g_luts, a, dWo, lr, x);
    case 5: return energyCompTransKulla(g_luts, a, dWo, dWi, lr);
    case 6: return avgFresnel(a);
    case 7: return msTransRatio(g_luts, a, lr);
    case 8: return fmsDielM<float, false>(g_luts, a, lr, dWo);
    case 9: return g_luts.sheen(dWo, lr);
    case 10: return dirAlbedoTrans(g_luts, a, dWo, lr);
    case 11: return avgAlbedoTrans(g_luts, a, lr);
    }
    return 0.0f;
}
void orc_layer_probs(const Surface& s, float cur, float prev, const float wo[3], int front, float out[6])
{
    SCtx<float> c;
    makeCtx(surfOf(s), cur, prev, v(wo), front != 0, c);
    for (int k = 0; k < 6; ++k) out[k] = c.probs[k];
}
template <bool R>
Eval evalSurfaceOf(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, const float wi[3],
                   uint32_t flags)
{
    Surf<float> sf = surfOf(s);
    SCtx<float> c;
    makeCtx(sf, cur, prev, v(wo), front != 0, c);
    EvalR<float> e = evalSurfaceF<float, R>(g_luts, sf, c, v(wo), v(wi), flags, specOf(hero));
    Eval r;
    for (int k = 0; k < 4; ++k) r.w[k] = e.w[k];
    r.pdf = e.pdf;
    r.trans = e.trans;
    return r;
}
template <bool R>
void sampleLayerOf(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, int layer, float sel,
                   float r0, float r1, float out[3], int* diffuse, int* delta)
{
    Surf<float> sf = surfOf(s);
    SCtx<float> c;
    makeCtx(sf, cur, prev, v(wo), front != 0, c);
    bool d = false, dl = false;
    put(sampleLayer<float, R>(&g_luts, sf, c, layer, sel, r0, r1, hero, d, dl), out);
    *diffuse = d ? 1 : 0;
    *delta = dl ? 1 : 0;
}
Eval orc_eval_surface(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, const float wi[3],
                      uint32_t flags)
{
    return evalSurfaceOf<false>(s, hero, cur, prev, wo, front, wi, flags);
}
Eval orcK_eval_surface(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, const float wi[3],
                       uint32_t flags)
{
    return evalSurfaceOf<true>(s, hero, cur, prev, wo, front, wi, flags);
}
void orc_sample_layer(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, int layer, float sel,
                      float r0, float r1, float out[3], int* diffuse, int* delta)
{
    sampleLayerOf<false>(s, hero, cur, prev, wo, front, layer, sel, r0, r1, out, diffuse, delta);
}
void orcK_sample_layer(const Surface& s, float hero, float cur, float prev, const float wo[3], int front, int layer, float sel,
                       float r0, float r1, float out[3], int* diffuse, int* delta)
{
    sampleLayerOf<true>(s, hero, cur, prev, wo, front, layer, sel, r0, r1, out, diffuse, delta);
}
float orc_sss(int fn, float a, float b)
{
    switch (fn)
    {
    case 0: return burleyProfileArea(a, b);
    case 1: return burleySampleRadius(a, b);
    case 2: return burleyD(a, b);
    }
    return 0.0f;
}
float orc_sss_pdf(const Surface& s, const float fromP[3], const float fromN[3], const float toP[3], const float toN[3])
{
    return pdfSssExit(surfOf(s), v(fromP), v(fromN), v(toP), v(toN));
}
float orc_sss_entry(const Surface& s, float hero, float cur, float prev, const float wo[3], int front)
{
    Surf<float> sf = surfOf(s);
    SCtx<float> c;
    makeCtx(sf, cur, prev, v(wo), front != 0, c);
    return sssEntryFactor(g_luts, sf, c, hero);
}
void orc_sss_exit_lobe(const Surface& s, float cur, float prev, const float wo[3], int front, float r0, float r1,
                       const float wi[3], uint32_t flags, float out[8])
{
    Surf<float> sf = surfOf(s);
    SCtx<float> c;
    makeCtx(sf, cur, prev, v(wo), front != 0, c);
    put(exitLobeSample(sf, c, v(wo), r0, r1), out);
    S4<float> w;
    float pdf = 0.0f;
    exitLobeEval(sf, c, v(wo), v(wi), flags, w, pdf);
    for (int k = 0; k < 4; ++k) out[3 + k] = w[k];
    out[7] = pdf;
}
} // namespace refcheck
