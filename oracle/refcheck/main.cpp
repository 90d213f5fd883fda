// TEST INFRASTRUCTURE ONLY: runs the reference's shader math (ref_*) and the oracle's
// restatement (orc_*) on the same seeded random inputs and reports, per function, how many
// results agree within the tolerance. Prints one JSON object; exit status 1 when a check
// falls below its bound.
//
//   refcheck <data dir> [samples per check]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../yapt_gb300/csrc/yg_tables.h"
#include "refcheck.h"

using namespace refcheck;

namespace
{
struct Rng
{
    uint64_t s;
    uint64_t next()
    {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    uint32_t u32() { return (uint32_t)(next() >> 32); }
    float uni() { return (float)((next() >> 40) * (1.0 / 16777216.0)); }
    float range(float a, float b) { return a + (b - a) * uni(); }
    void dir(float* d)
    {
        float z = range(-1.f, 1.f), phi = range(0.f, 6.2831853f), r = std::sqrt(std::fmax(0.f, 1.f - z * z));
        d[0] = r * std::cos(phi);
        d[1] = z;
        d[2] = r * std::sin(phi);
    }
    void hemi(float* d)
    {
        dir(d);
        d[1] = std::fabs(d[1]);
    }
    float rough()
    {
        float u = uni();
        if (u < 0.1f) return 0.0f;
        if (u < 0.2f) return range(0.0f, 0.02f);
        if (u < 0.5f) return range(0.02f, 0.3f);
        return uni();
    }
};

struct Check
{
    std::string name;
    double tol;
    bool exact;
    double minWithin;
    uint64_t n = 0, bad = 0;
    double maxRel = 0;
};
std::vector<Check> g_checks;

Check& check(const char* name, double tol, double minWithin = 0.999, bool exact = false)
{
    for (auto& c : g_checks)
        if (c.name == name) return c;
    g_checks.push_back(Check{name, tol, exact, minWithin});
    return g_checks.back();
}
// one sample: the components of a (the reference) and b (the oracle), relative to the
// reference's largest magnitude (floor 1e-6)
void compare(Check& c, const float* a, const float* b, int n)
{
    double scale = 1e-6;
    for (int k = 0; k < n; ++k) scale = std::fmax(scale, std::fabs((double)a[k]));
    double rel = 0;
    bool nanMismatch = false;
    for (int k = 0; k < n; ++k)
    {
        if (std::isnan(a[k]) || std::isnan(b[k]))
        {
            nanMismatch |= std::isnan(a[k]) != std::isnan(b[k]);
            continue;
        }
        if (c.exact && std::memcmp(&a[k], &b[k], 4) != 0) rel = INFINITY;
        else rel = std::fmax(rel, std::fabs((double)a[k] - (double)b[k]) / scale);
    }
    if (nanMismatch) rel = INFINITY;
    c.n++;
    if (!(rel <= c.tol)) c.bad++;
    if (std::isfinite(rel)) c.maxRel = std::fmax(c.maxRel, rel);
    else c.maxRel = INFINITY;
}
void compare1(Check& c, float a, float b) { compare(c, &a, &b, 1); }

Surface randomSurface(Rng& r)
{
    Surface s;
    std::memset(&s, 0, sizeof(s));
    for (int k = 0; k < 4; ++k)
    {
        s.specular[k] = r.uni();
        s.albedo[k] = r.uni();
        s.absorption[k] = r.range(0.f, 0.2f);
        s.emissive[k] = 0.f;
        s.sheenColor[k] = r.uni();
    }
    float g[3];
    r.dir(g);
    auto near = [&](float* out, float amount) {
        float p[3];
        r.dir(p);
        float l = 0;
        for (int k = 0; k < 3; ++k)
        {
            out[k] = g[k] + amount * p[k];
            l += out[k] * out[k];
        }
        l = std::sqrt(l);
        for (int k = 0; k < 3; ++k) out[k] /= l;
    };
    for (int k = 0; k < 3; ++k) s.geoN[k] = g[k];
    near(s.baseN, r.uni() < 0.5f ? 0.0f : 0.3f);
    near(s.coatN, r.uni() < 0.5f ? 0.0f : 0.3f);
    float t[3];
    r.dir(t);
    s.tangent[0] = s.baseN[1] * t[2] - s.baseN[2] * t[1];
    s.tangent[1] = s.baseN[2] * t[0] - s.baseN[0] * t[2];
    s.tangent[2] = s.baseN[0] * t[1] - s.baseN[1] * t[0];
    auto pick = [&](float zeroP, float oneP) {
        float u = r.uni();
        if (u < zeroP) return 0.0f;
        if (u < zeroP + oneP) return 1.0f;
        return r.uni();
    };
    s.transparency = pick(0.5f, 0.25f);
    s.metalness = pick(0.5f, 0.25f);
    s.ior = r.range(1.05f, 2.5f);
    s.roughness = r.rough();
    s.cauchyA = r.range(1.3f, 1.8f);
    s.cauchyB = r.range(0.0f, 0.01f);
    s.specAmount = pick(0.2f, 0.5f);
    s.ccAmount = pick(0.6f, 0.1f);
    s.ccIOR = r.range(1.2f, 2.0f);
    s.ccRough = r.rough();
    s.aniso = r.uni() < 0.5f ? 0.0f : r.range(-0.9f, 0.9f);
    s.anisoRot = r.uni();
    s.thinFilm = r.uni() < 0.7f ? 0.0f : r.range(100.f, 1000.f);
    s.sheenRough = r.rough();
    s.sheenAmount = pick(0.6f, 0.1f);
    s.focus = 0.0f;
    s.sssAmount = pick(0.6f, 0.2f);
    for (int k = 0; k < 4; ++k) s.sssRadius[k] = r.range(0.002f, 0.3f);
    s.diffOcc = r.uni() < 0.7f ? 1.0f : r.range(0.3f, 1.0f);
    s.specOcc = r.uni() < 0.7f ? 1.0f : r.range(0.3f, 1.0f);
    s.flags = (r.uni() < 0.5f ? 1u : 0u) | (r.uni() < 0.3f ? 2u : 0u);
    return s;
}

std::vector<float> table(const char* dir, int which)
{
    std::vector<float> out;
    std::string err;
    return out;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc < 2)
    {
        std::fprintf(stderr, "usage: refcheck <data dir> [samples]\n");
        return 2;
    }
    const std::string dir = argv[1];
    const int N = argc > 2 ? std::atoi(argv[2]) : 20000;
    setenv("YAPT_DATA_DIR", dir.c_str(), 1);
    // the tables both sides read (the shared generator)
    yg::MsLuts L;
    yg::buildMsLuts(L);
    std::vector<double> cie;
    std::string err;
    if (!yg::loadCie(dir + "/cie1931_2deg_d65_1nm.txt", cie, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 2;
    }
    std::vector<float> cie321(321 * 4), rgb;
    for (int i = 0; i < 321; ++i)
        for (int k = 0; k < 4; ++k) cie321[4 * i + k] = (float)cie[4 * (i + 20) + k];
    yg::buildRgbToSpd(cie, 380, 700, rgb);
    std::vector<uint32_t> mats;
    if (!yg::buildSobolMatrices(dir + "/joe_kuo_6_21201_first256.txt", mats, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 2;
    }
    uint32_t point[256];
    for (int d = 0; d < 256; ++d) point[d] = yg::sobolUint(mats.data(), 12345u, (uint32_t)d);
    Tables T;
    const std::vector<float>* luts[9] = {&L.ss, &L.ssAvg, &L.ssms, &L.ssmsAvg, &L.transDenser, &L.transLighter,
                                         &L.transAvgDenser, &L.transAvgLighter, &L.sheen};
    for (int i = 0; i < 9; ++i) T.lut[i] = luts[i]->data();
    T.cie321x4 = cie321.data();
    T.rgb64 = rgb.data();
    T.sobolPoint = point;
    ref_setup(T);
    refK_setup(T);
    orc_setup(T);

    Rng r{0x5eed};
    for (int i = 0; i < N; ++i)
    {
        // sampler (random.hlsl, randomSampler.hlsl): bit for bit
        uint32_t a = r.u32(), b = r.u32() & 0xffff;
        uint32_t h1 = ref_hash2(a, b), h2 = orc_hash2(a, b);
        compare1(check("hash(a,b)", 0, 1.0, true), *(float*)&h1, *(float*)&h2);
        uint32_t o1 = ref_owen(a, b * 2654435761u), o2 = orc_owen(a, b * 2654435761u);
        compare1(check("owenScrambleBase2Fast", 0, 1.0, true), *(float*)&o1, *(float*)&o2);
        compare1(check("uintToFloat01", 0, 1.0, true), ref_u01(a), orc_u01(a));
        if (i < 2000)
        {
            float s1[42], s2[42];
            ref_sampler(r.u32(), 40, s1);
            orc_sampler(r.u32() * 0 + 0, 0, s2); // warm (no-op)
            uint32_t seed = r.u32();
            ref_sampler(seed, 40, s1);
            orc_sampler(seed, 40, s2);
            compare(check("RandomSampler (texel offset, 40 dimensions)", 0, 1.0, true), s1, s2, 42);
        }
        // spectral (spectralDistribution.hlsl)
        float u = r.uni(), l1[4], l2[4];
        ref_lambdas(u, l1);
        orc_lambdas(u, l2);
        compare(check("getSpectralSampleLambdas", 1e-6), l1, l2, 4);
        float x = r.range(-20.f, 20.f);
        compare1(check("sigmoid", 1e-6), ref_sigmoid(x), orc_sigmoid(x));
        float rgbv[3] = {r.uni(), r.uni(), r.uni()};
        if (r.uni() < 0.1f) rgbv[1] = rgbv[2] = rgbv[0];
        float hero = 380.f + 320.f * r.uni(), sp1[4], sp2[4];
        for (int mode = 0; mode < 3; ++mode)
        {
            float sc = mode == 0 ? 1.0f : r.range(0.f, 20.f);
            float c3[3] = {rgbv[0] * sc, rgbv[1] * sc, rgbv[2] * sc};
            ref_rgb_spectrum(mode, c3, hero, sp1);
            orc_rgb_spectrum(mode, c3, hero, sp2);
            const char* nm[3] = {"setFromRGB", "setFromRGBUnbounded", "setFromRGBUnboundedNoIlluminant"};
            compare(check(nm[mode], 1e-4), sp1, sp2, 4);
        }
        float Ls[4] = {r.uni(), r.uni(), r.uni(), r.uni()}, X1[3], X2[3];
        ref_to_xyz(hero, Ls, X1);
        orc_to_xyz(hero, Ls, X2);
        compare(check("ToXYZ", 1e-4), X1, X2, 3);
        float w4[4] = {r.uni(), r.uni(), r.uni(), r.uni()}, q1[5], q2[5];
        float rr = r.uni(), norm = r.range(0.5f, 2.f);
        q1[4] = (float)ref_roulette(w4, rr, norm, q1);
        q2[4] = (float)orc_roulette(w4, rr, norm, q2);
        compare(check("applyRussianRoulette", 1e-6), q1, q2, 5);
        // GGX, Fresnel, sheen (ggx.hlsl, fresnel.hlsl, miscBrdf.hlsl)
        float wo[3], wi[3], wm[3];
        r.hemi(wo);
        r.dir(wi);
        r.hemi(wm);
        float ax = std::fmax(r.rough(), 1e-3f), ay = r.uni() < 0.5f ? ax : std::fmax(r.rough(), 1e-3f);
        compare1(check("smithLambdaGGX", 1e-4), ref_lambda_ggx(wo, ax, ay), orc_lambda_ggx(wo, ax, ay));
        compare1(check("G1GGX", 1e-4), ref_g1(wo, wm, ax, ay), orc_g1(wo, wm, ax, ay));
        compare1(check("G2GGX", 1e-4), ref_g2(wo, wi, wm, ax, ay), orc_g2(wo, wi, wm, ax, ay));
        compare1(check("DGGX", 1e-4), ref_dggx(wm, ax, ay), orc_dggx(wm, ax, ay));
        compare1(check("DVGGX", 1e-4), ref_dv(wo, wm, ax, ay), orc_dv(wo, wm, ax, ay));
        float u1 = r.uni(), u2 = r.uni(), m1[3], m2[3];
        float wos[3] = {wo[0], r.uni() < 0.3f ? -wo[1] : wo[1], wo[2]};
        ref_sample_wm(wos, ax, ay, u1, u2, m1);
        orc_sample_wm(wos, ax, ay, u1, u2, m2);
        compare(check("sampleWMGGX (visible normals)", 1e-4), m1, m2, 3);
        float cr = r.uni(), cg = r.uni(), nk1[2], nk2[2];
        ref_conductor_nk(cr, cg, nk1);
        orc_conductor_nk(cr, cg, nk2);
        compare(check("getConductorRefractiveIndexAndExtinction", 1e-4), nk1, nk2, 2);
        float ct = r.uni(), er = r.range(0.2f, 4.f), ei = r.range(0.f, 8.f);
        compare1(check("fresnelDielectricConductor", 1e-4), ref_fresnel_dc(er, ei, ct), orc_fresnel_dc(er, ei, ct));
        float eta = r.uni() < 0.1f ? 1.0f : r.range(0.3f, 3.0f);
        float ctd = r.range(-0.2f, 1.f);
        compare1(check("fresnelDielectricDielectric2", 1e-4), ref_fresnel_dd(eta, ctd), orc_fresnel_dd(eta, ctd));
        float sr = r.range(0.01f, 1.f);
        compare1(check("DSheen", 1e-4), ref_dsheen(wm, sr), orc_dsheen(wm, sr));
        compare1(check("GSheen", 1e-4), ref_gsheen(wo, wm, sr), orc_gsheen(wo, wm, sr));
        float ed = r.range(-1.f, 1.f), ee = r.uni() < 0.3f ? 0.f : r.range(0.f, 64.f);
        compare1(check("evaluateEmissionProfile", 1e-4), ref_emission_profile(ed, ee), orc_emission_profile(ed, ee));
        float dk1[2], dk2[2], du0 = r.uni(), du1 = r.uni();
        ref_concentric_disk(du0, du1, dk1);
        orc_concentric_disk(du0, du1, dk2);
        compare(check("sampleConcentricDisk", 1e-4), dk1, dk2, 2);
        // lobes (bsdfSample.hlsl)
        // (sampleGGXTransmitted belongs to TransmittedLayer, which no integrator uses: not compared)
        const char* sn[6] = {"sampleGGXReflectionConductor", "sampleGGXReflectionDielectric", nullptr,
                             "sampleDielectric", "sampleDiffuseLambertian", "sampleSheen"};
        const char* pn[6] = {"pdfGGXReflectionConductor", "pdfGGXReflectionDielectric", "pdfGGXTransmitted", "pdfDielectric",
                             "pdfDiffuseLambertian", "pdfSheen"};
        const char* en[6] = {nullptr, "evaluateGGXReflectionDielectric", "evaluateGGXTransmitted", nullptr, nullptr,
                             "evaluateSheen"};
        for (int lobe = 0; lobe < 6; ++lobe)
        {
            float lax = lobe == 5 ? r.range(0.f, 1.f) : r.rough(), lay = r.uni() < 0.5f ? lax : r.rough();
            float lwo[3];
            r.dir(lwo);
            if (lobe != 3 && lobe != 2) lwo[1] = std::fabs(lwo[1]);
            float s0 = r.uni(), s1 = r.uni(), scs = r.uni();
            int aR = r.uni() < 0.8f, aT = r.uni() < 0.8f;
            float d1[3], d2[3];
            ref_sample_lobe(lobe, eta, lax, lay, lwo, s0, s1, scs, aR, aT, d1);
            orc_sample_lobe(lobe, eta, lax, lay, lwo, s0, s1, scs, aR, aT, d2);
            if (sn[lobe]) compare(check(sn[lobe], 1e-4), d1, d2, 3);
            float lwi[3];
            if (r.uni() < 0.5f && (d1[0] != 0 || d1[1] != 0 || d1[2] != 0)) std::memcpy(lwi, d1, sizeof(lwi));
            else r.dir(lwi);
            compare1(check(pn[lobe], 1e-4), ref_pdf_lobe(lobe, eta, lax, lay, lwo, lwi, aR, aT),
                     orc_pdf_lobe(lobe, eta, lax, lay, lwo, lwi, aR, aT));
            if (en[lobe])
            {
                float ev = lobe == 5 ? r.uni() : eta;
                compare1(check(en[lobe], 1e-4), ref_eval_lobe(lobe, ev, 0.f, lax, lay, lwo, lwi),
                         orc_eval_lobe(lobe, ev, 0.f, lax, lay, lwo, lwi));
            }
        }
        // multiple scattering (multiScatter.hlsl, with the LUTs as textures)
        const char* mn[12] = {"getEnergyCompensationTurquin", "getEnergyCompensationKulla", "getEnergyRemainingAfterSpecular",
                              "getEnergyRemainingAfterSheen", "getEnergyCompensationTranslucentTurquin",
                              "getEnergyCompensationTranslucentKulla", "getAvgFresnel", "getMsTransmissionRatio",
                              "getFmsDielectric", "getSheenDirectionalAlbedo", "getDirectionalAlbedoTranslucent",
                              "getAverageAlbedoTranslucent"};
        for (int fn = 0; fn < 12; ++fn)
        {
            float aa = (fn == 0 || fn == 1) ? r.uni() : r.range(0.35f, 2.9f);
            float dWo = r.range(-1.f, 1.f), dWi = r.range(-1.f, 1.f), lr = r.uni(), xx = r.uni();
            if (fn == 8 || fn == 9) dWo = std::fabs(dWo);
            compare1(check(mn[fn], 1e-4), ref_ms(fn, aa, dWo, dWi, lr, xx), orc_ms(fn, aa, dWo, dWi, lr, xx));
        }
        // layered surface (materialSample.hlsl, materialLayers.hlsl)
        Surface S = randomSurface(r);
        float swo[3];
        r.dir(swo);
        int front = r.uni() < 0.8f;
        float cur = front ? 1.0f : S.ior, prev = 1.0f;
        float p1[6], p2[6];
        ref_layer_probs(S, cur, prev, swo, front, p1);
        orc_layer_probs(S, cur, prev, swo, front, p2);
        compare(check("calculateNormalizedMaterialLayerSamplingProbabilities", 1e-5), p1, p2, 6);
        int layer = (int)(r.uni() * 5.0f);
        float sel = r.uni(), r0 = r.uni(), r1 = r.uni(), sd1[5], sd2[5];
        int df1, dl1, df2, dl2;
        float shero = 380.f + 320.f * r.uni();
        ref_sample_layer(S, shero, cur, prev, swo, front, layer, sel, r0, r1, sd1, &df1, &dl1);
        orc_sample_layer(S, shero, cur, prev, swo, front, layer, sel, r0, r1, sd2, &df2, &dl2);
        sd1[3] = (float)df1, sd1[4] = (float)dl1;
        sd2[3] = (float)df2, sd2[4] = (float)dl2;
        compare(check("getSampleDirectionOSForLayer", 1e-4), sd1, sd2, 5);
        float swi[3];
        if (r.uni() < 0.5f && (sd1[0] != 0 || sd1[1] != 0 || sd1[2] != 0)) std::memcpy(swi, sd1, sizeof(swi));
        else r.dir(swi);
        const uint32_t flagSets[4] = {1u, 8u, 4u, 2u};
        uint32_t fl = flagSets[(int)(r.uni() * 4.0f) & 3];
        Eval e1 = ref_eval_surface(S, shero, cur, prev, swo, front, swi, fl);
        Eval e2 = orc_eval_surface(S, shero, cur, prev, swo, front, swi, fl);
        float ev1[6] = {e1.w[0], e1.w[1], e1.w[2], e1.w[3], e1.pdf, (float)e1.trans};
        float ev2[6] = {e2.w[0], e2.w[1], e2.w[2], e2.w[3], e2.pdf, (float)e2.trans};
        {
            Check& cw = check("evaluateSurface (weight)", 1e-4);
            uint64_t before = cw.bad;
            if (fl != 2u) compare(cw, ev1, ev2, 4); // EVALUATE_FLAGS_PDF_ONLY: the weight is not computed
            static int shown = 0;
            if (cw.bad != before && std::getenv("REFCHECK_DEBUG") && shown++ < 12)
                std::fprintf(stderr,
                             "eval mismatch fl=%u front=%d w ref (%g %g %g %g) orc (%g %g %g %g) pdf %g %g | tr=%g met=%g "
                             "rough=%g ior=%g spec=%g cc=%g ccR=%g sheen=%g sheenR=%g tf=%g aniso=%g flags=%u occ=%g/%g "
                             "wo.y=%g wi.y=%g\n",
                             fl, front, ev1[0], ev1[1], ev1[2], ev1[3], ev2[0], ev2[1], ev2[2], ev2[3], ev1[4], ev2[4],
                             S.transparency, S.metalness, S.roughness, S.ior, S.specAmount, S.ccAmount, S.ccRough,
                             S.sheenAmount, S.sheenRough, S.thinFilm, S.aniso, S.flags, S.diffOcc, S.specOcc, swo[1], swi[1]);
        }
        compare1(check("evaluateSurface (pdf)", 1e-4), ev1[4], ev2[4]);
        compare1(check("evaluateSurface (transmission type)", 0, 0.999, true), ev1[5], ev2[5]);
        // subsurface (subsurface.hlsl): the Burley profile, radius sampling, the exit density, the
        // entry factor and the exit lobe
        {
            float dd = r.range(1e-4f, 0.2f), rr = r.range(0.f, 2.f) * dd, uu = r.uni();
            compare1(check("burleyProfileArea", 1e-4), ref_sss(0, rr, dd), orc_sss(0, rr, dd));
            compare1(check("burleySampleRadius", 1e-4), ref_sss(1, uu, dd), orc_sss(1, uu, dd));
            float rad = r.range(0.f, 0.3f), alb = r.uni();
            compare1(check("burleyD", 1e-5), ref_sss(2, rad, alb), orc_sss(2, rad, alb));
            float fp[3], fnrm[3], tp[3], tn[3], off[3];
            r.dir(fnrm);
            r.dir(tn);
            r.dir(off);
            float dist = r.range(0.f, 0.5f);
            for (int k = 0; k < 3; ++k)
            {
                fp[k] = r.range(-2.f, 2.f);
                tp[k] = fp[k] + dist * off[k];
            }
            compare1(check("pdfSubsurfaceExit", 1e-4), ref_sss_pdf(S, fp, fnrm, tp, tn), orc_sss_pdf(S, fp, fnrm, tp, tn));
            compare1(check("getSubsurfaceEntryFactor", 1e-4), ref_sss_entry(S, shero, cur, prev, swo, front),
                     orc_sss_entry(S, shero, cur, prev, swo, front));
            float xo1[8], xo2[8], xr0 = r.uni(), xr1 = r.uni();
            uint32_t xfl = r.uni() < 0.5f ? 1u : 4u;
            ref_sss_exit_lobe(S, cur, prev, swo, front, xr0, xr1, swi, xfl, xo1);
            orc_sss_exit_lobe(S, cur, prev, swo, front, xr0, xr1, swi, xfl, xo2);
            compare(check("sampleSubsurfaceExitLobe", 1e-4), xo1, xo2, 3);
            compare(check("evaluateSubsurfaceExitLobe", 1e-4), xo1 + 3, xo2 + 3, 5);
        }
        // the bidirectional integrator's model (RECIPROCAL_MULTISCATTER): layer sampling with the
        // multiple-scattering lobe, and evaluation on camera and light paths
        refK_sample_layer(S, shero, cur, prev, swo, front, layer, sel, r0, r1, sd1, &df1, &dl1);
        orcK_sample_layer(S, shero, cur, prev, swo, front, layer, sel, r0, r1, sd2, &df2, &dl2);
        sd1[3] = (float)df1, sd1[4] = (float)dl1;
        sd2[3] = (float)df2, sd2[4] = (float)dl2;
        compare(check("getSampleDirectionOSForLayer (RECIPROCAL_MULTISCATTER)", 1e-4), sd1, sd2, 5);
        const uint32_t flagSetsK[4] = {1u, 8u, 4u, 12u};
        uint32_t flK = flagSetsK[(int)(r.uni() * 4.0f) & 3];
        Eval k1 = refK_eval_surface(S, shero, cur, prev, swo, front, swi, flK);
        Eval k2 = orcK_eval_surface(S, shero, cur, prev, swo, front, swi, flK);
        float kv1[6] = {k1.w[0], k1.w[1], k1.w[2], k1.w[3], k1.pdf, (float)k1.trans};
        float kv2[6] = {k2.w[0], k2.w[1], k2.w[2], k2.w[3], k2.pdf, (float)k2.trans};
        compare(check("evaluateSurface (RECIPROCAL_MULTISCATTER, weight)", 1e-4), kv1, kv2, 4);
        compare1(check("evaluateSurface (RECIPROCAL_MULTISCATTER, pdf)", 1e-4), kv1[4], kv2[4]);
        compare1(check("evaluateSurface (RECIPROCAL_MULTISCATTER, transmission type)", 0, 0.999, true), kv1[5], kv2[5]);
    }
    bool ok = true;
    std::printf("{\"samples\": %d, \"checks\": [", N);
    for (size_t i = 0; i < g_checks.size(); ++i)
    {
        const Check& c = g_checks[i];
        double within = c.n ? 1.0 - (double)c.bad / (double)c.n : 0.0;
        bool pass = within >= c.minWithin;
        ok = ok && pass;
        std::printf("%s\n {\"name\": \"%s\", \"n\": %llu, \"within\": %.6f, \"tol\": %g, \"exact\": %s, \"max_rel\": %.3g, "
                    "\"pass\": %s}",
                    i ? "," : "", c.name.c_str(), (unsigned long long)c.n, within, c.tol, c.exact ? "true" : "false",
                    std::isfinite(c.maxRel) ? c.maxRel : 1e300, pass ? "true" : "false");
    }
    std::printf("\n], \"ok\": %s}\n", ok ? "true" : "false");
    return ok ? 0 : 1;
}
