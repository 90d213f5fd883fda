// TEST INFRASTRUCTURE ONLY: known-answer and consistency checks of the oracle's BSDF lobes
// (the functions of oracle.cpp behind the plain orc_* interface of refcheck.h). Each check
// prints one JSON object per line; tests/test_oracle_kat.py judges them.
//
//   kat fresnel           dielectric Fresnel at normal incidence against ((eta - 1)/(eta + 1))^2
//   kat lobe <id> <eta> <ax> <ay> <cos wo> <samples> <seed>
//       samples the lobe (sampleCondRefl, sampleDielRefl, sampleDiel, cosHemi; ids as in
//       orc_sample_lobe) from the outgoing direction at the given cosine, histograms the
//       directions over (cos theta, phi) cells of the sphere, and integrates the lobe's pdf
//       (orc_pdf_lobe) over each cell; a sample returned as the zero vector (rejected below
//       the horizon) falls in an extra cell whose expectation is the pdf's mass outside the
//       lobe's domain.
//       Prints counts against expectations as a chi-square statistic and the pdf's integral.
//   kat albedo <id> <eta> <ax> <ay> <cos wo> <samples> <seed>
//       the lobe's directional albedo by its own importance sampling and by quadrature
//   kat layered <preset> <cos wo> <samples> <seed> <data dir>
//       the full layered BSDF's sampling against the mixture pdf of evaluateSurface
//   kat reciprocity <id> <pairs> <seed>
//       f(wo, wi) against f(wi, wo) for a reflection lobe
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../yapt_gb300/csrc/yg_tables.h"
#include "../refcheck/refcheck.h"

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
    float uni() { return (float)((next() >> 40) * (1.0 / 16777216.0)); }
};

int fresnel()
{
    const float etas[] = {1.1f, 1.33f, 1.5f, 1.8f, 2.4f, 1.0f / 1.5f, 1.0f / 1.33f};
    for (float eta : etas)
    {
        const double want = std::pow((eta - 1.0) / (eta + 1.0), 2.0);
        const double got = orc_fresnel_dd(eta, 1.0f);
        std::printf("{\"check\": \"fresnel_normal\", \"eta\": %.6f, \"want\": %.9g, \"got\": %.9g}\n", eta, want, got);
    }
    return 0;
}

constexpr int kCosBins = 24, kPhiBins = 48, kSub = 16, kFine = 256;
constexpr double kPi = 3.14159265358979323846;

void dirOf(double c, double phi, float out[3])
{
    const double s = std::sqrt(std::fmax(0.0, 1.0 - c * c));
    out[0] = (float)(s * std::cos(phi));
    out[1] = (float)c;
    out[2] = (float)(s * std::sin(phi));
}

int lobe(int id, float eta, float ax, float ay, float cosWo, long samples, uint64_t seed)
{
    float wo[3];
    dirOf(cosWo, 0.3, wo);
    const int aR = 1, aT = 1;
    std::vector<double> count(kCosBins * kPhiBins + 1, 0.0), expect(kCosBins * kPhiBins + 1, 0.0);
    Rng rng{seed};
    for (long n = 0; n < samples; ++n)
    {
        float wi[3];
        const float s0 = rng.uni(), s1 = rng.uni(), sc = rng.uni();
        orc_sample_lobe(id, eta, ax, ay, wo, s0, s1, sc, aR, aT, wi);
        if (wi[0] == 0.0f && wi[1] == 0.0f && wi[2] == 0.0f)
        {
            count[kCosBins * kPhiBins] += 1.0;
            continue;
        }
        const double len = std::sqrt((double)wi[0] * wi[0] + (double)wi[1] * wi[1] + (double)wi[2] * wi[2]);
        const double c = std::fmin(1.0, std::fmax(-1.0, wi[1] / len));
        double phi = std::atan2((double)wi[2], (double)wi[0]);
        if (phi < 0.0) phi += 2.0 * kPi;
        const int ic = std::min(kCosBins - 1, (int)((c + 1.0) * 0.5 * kCosBins));
        const int ip = std::min(kPhiBins - 1, (int)(phi / (2.0 * kPi) * kPhiBins));
        count[ic * kPhiBins + ip] += 1.0;
    }
    // the pdf (per solid angle) integrated over each cell of the lobe's domain (the upper
    // hemisphere for the reflection lobes 0, 1, 4, 5, the lower one for transmission 2, the
    // sphere for the dielectric lobe 3, with the outgoing direction above): midpoint rule on
    // kSub x kSub sub-cells, d(omega) = d(cos theta) d(phi). Outside its domain a lobe's pdf
    // is not evaluated by the integrator, and samples there are rejected by the sampler.
    const bool upper = id != 2, lower = id == 2 || id == 3;
    double integral = 0.0;
    const double dc = 2.0 / kCosBins, dp = 2.0 * kPi / kPhiBins;
    // a cell that the edge of the pdf's support crosses (some sub-cells zero, some not) is
    // integrated again on a kFine x kFine grid: the midpoint rule converges slowly there
    auto cellMass = [&](int ic, int ip, int sub, bool& edge) {
        double m = 0.0;
        bool zero = false, nonzero = false;
        for (int a = 0; a < sub; ++a)
            for (int b = 0; b < sub; ++b)
            {
                const double c = -1.0 + (ic + (a + 0.5) / sub) * dc;
                if ((c > 0.0 && !upper) || (c < 0.0 && !lower)) continue;
                const double phi = (ip + (b + 0.5) / sub) * dp;
                float wi[3];
                dirOf(c, phi, wi);
                const double p = orc_pdf_lobe(id, eta, ax, ay, wo, wi, aR, aT);
                m += p;
                (p > 0.0 ? nonzero : zero) = true;
            }
        edge = zero && nonzero;
        return m * dc * dp / ((double)sub * sub);
    };
    for (int ic = 0; ic < kCosBins; ++ic)
        for (int ip = 0; ip < kPhiBins; ++ip)
        {
            bool edge = false;
            double m = cellMass(ic, ip, kSub, edge);
            if (edge) m = cellMass(ic, ip, kFine, edge);
            expect[ic * kPhiBins + ip] = m * samples;
            integral += m;
        }
    // the rejected samples' cell, for the samplers that reject (0, 1, 3): the mass of the pdf
    // outside its domain; the others must put all their mass inside (pdf_integral = 1, up to
    // the quadrature's error, which would dominate an empty cell's expectation)
    const bool rejects = id == 0 || id == 1 || id == 3;
    expect[kCosBins * kPhiBins] = rejects ? std::fmax(0.0, 1.0 - integral) * samples : 0.0;
    // chi-square over the cells expecting at least 5 samples; the rest are pooled into one
    double chi2 = 0.0, poolE = 0.0, poolC = 0.0, worst = 0.0;
    int dof = -1;
    for (size_t k = 0; k < count.size(); ++k)
    {
        if (k == count.size() - 1 && !rejects) continue; // reported as "rejected" (must be 0)
        if (expect[k] >= 5.0)
        {
            const double d = count[k] - expect[k];
            chi2 += d * d / expect[k];
            worst = std::fmax(worst, std::fabs(d) / std::sqrt(expect[k]));
            ++dof;
        }
        else
        {
            poolE += expect[k];
            poolC += count[k];
        }
    }
    if (poolE >= 5.0)
    {
        const double d = poolC - poolE;
        chi2 += d * d / poolE;
        ++dof;
    }
    std::printf("{\"check\": \"lobe\", \"lobe\": %d, \"eta\": %.4f, \"ax\": %.4f, \"ay\": %.4f, \"cos_wo\": %.4f, "
                "\"samples\": %ld, \"chi2\": %.4f, \"dof\": %d, \"worst_z\": %.3f, \"pdf_integral\": %.6f, "
                "\"rejected\": %.0f, \"pooled_expect\": %.3f, \"pooled_count\": %.0f}\n",
                id, eta, ax, ay, cosWo, samples, chi2, dof, worst, integral, count[kCosBins * kPhiBins], poolE, poolC);
    return 0;
}
// Directional albedo of an evaluated lobe (orc_eval_lobe: 1 dielectric reflection, 2
// transmission, 5 sheen) two ways: the estimator an integrator uses, the mean of
// f(wo, wi) |cos wi| / pdf(wo, wi) over the lobe's own samples (a rejected sample counts 0),
// and a quadrature of f |cos wi| over the sphere. Equal within the estimator's standard error
// only if sampling, pdf and evaluation agree.
int albedo(int id, float eta, float ax, float ay, float cosWo, long samples, uint64_t seed)
{
    float wo[3];
    dirOf(cosWo, 0.3, wo);
    Rng rng{seed};
    double sum = 0.0, sum2 = 0.0;
    for (long n = 0; n < samples; ++n)
    {
        float wi[3];
        const float s0 = rng.uni(), s1 = rng.uni(), sc = rng.uni();
        orc_sample_lobe(id, eta, ax, ay, wo, s0, s1, sc, 1, 1, wi);
        double w = 0.0;
        if (wi[0] != 0.0f || wi[1] != 0.0f || wi[2] != 0.0f)
        {
            const double pdf = orc_pdf_lobe(id, eta, ax, ay, wo, wi, 1, 1);
            if (pdf > 0.0) w = orc_eval_lobe(id, eta, 0.0f, ax, ay, wo, wi) * std::fabs((double)wi[1]) / pdf;
        }
        sum += w;
        sum2 += w * w;
    }
    const double mean = sum / samples, se = std::sqrt(std::fmax(0.0, sum2 / samples - mean * mean) / samples);
    constexpr int nc = 1024, np = 1024;
    double quad = 0.0;
    for (int a = 0; a < nc; ++a)
    {
        const double c = -1.0 + (a + 0.5) * 2.0 / nc;
        for (int b = 0; b < np; ++b)
        {
            float wi[3];
            dirOf(c, (b + 0.5) * 2.0 * kPi / np, wi);
            quad += orc_eval_lobe(id, eta, 0.0f, ax, ay, wo, wi) * std::fabs(c);
        }
    }
    quad *= (2.0 / nc) * (2.0 * kPi / np);
    std::printf("{\"check\": \"albedo\", \"lobe\": %d, \"eta\": %.4f, \"ax\": %.4f, \"ay\": %.4f, \"cos_wo\": %.4f, "
                "\"samples\": %ld, \"estimate\": %.7f, \"stderr\": %.7f, \"quadrature\": %.7f}\n",
                id, eta, ax, ay, cosWo, samples, mean, se, quad);
    return 0;
}
// Helmholtz reciprocity of the reflection lobes with an evaluation (1 dielectric reflection,
// 5 sheen): f(wo, wi) = f(wi, wo) for random direction pairs above the surface and random
// roughness; prints the largest relative asymmetry.
int reciprocity(int id, long pairs, uint64_t seed)
{
    Rng rng{seed};
    double worst = 0.0;
    long n = 0;
    for (long k = 0; k < pairs; ++k)
    {
        float wo[3], wi[3];
        dirOf(rng.uni(), 2.0 * kPi * rng.uni(), wo);
        dirOf(rng.uni(), 2.0 * kPi * rng.uni(), wi);
        const float ax = 0.05f + 0.9f * rng.uni(), ay = 0.05f + 0.9f * rng.uni(), eta = 1.1f + rng.uni();
        const double a = orc_eval_lobe(id, eta, 0.0f, ax, ay, wo, wi), b = orc_eval_lobe(id, eta, 0.0f, ax, ay, wi, wo);
        if (a > 1e-6 || b > 1e-6)
        {
            ++n;
            worst = std::fmax(worst, std::fabs(a - b) / std::fmax(a, b));
        }
    }
    std::printf("{\"check\": \"reciprocity\", \"lobe\": %d, \"pairs\": %ld, \"worst_rel\": %.4g}\n", id, n, worst);
    return 0;
}
// The full layered BSDF as the integrators sample it (closestHit: a layer chosen with the
// probabilities of calculateNormalizedMaterialLayerSamplingProbabilities, then that layer's
// getSampleDirectionOSForLayer) against the mixture pdf evaluateSurface reports (the sum of the
// layers' pdfs weighted by the same probabilities). Presets: 0 clear coat + sheen + 30 % metal
// over a diffuse base; 1 rough glass (reflection and transmission); 2 rough plastic (specular
// layer over a diffuse base); 3 anisotropic metal under a rough coat. Needs the LUTs
// (multiple scattering, sheen) of the shared table generator.
int setupTables(const char* dataDir)
{
    static yg::MsLuts L;
    static std::vector<double> cie;
    static std::vector<float> cie321(321 * 4), rgb;
    static uint32_t point[256] = {};
    std::string err;
    yg::buildMsLuts(L);
    if (!yg::loadCie(std::string(dataDir) + "/cie1931_2deg_d65_1nm.txt", cie, err))
    {
        std::fprintf(stderr, "%s\n", err.c_str());
        return 2;
    }
    for (int i = 0; i < 321; ++i)
        for (int k = 0; k < 4; ++k) cie321[4 * i + k] = (float)cie[4 * (i + 20) + k];
    yg::buildRgbToSpd(cie, 380, 700, rgb);
    Tables T;
    const std::vector<float>* luts[9] = {&L.ss, &L.ssAvg, &L.ssms, &L.ssmsAvg, &L.transDenser, &L.transLighter,
                                         &L.transAvgDenser, &L.transAvgLighter, &L.sheen};
    for (int i = 0; i < 9; ++i) T.lut[i] = luts[i]->data();
    T.cie321x4 = cie321.data();
    T.rgb64 = rgb.data();
    T.sobolPoint = point;
    orc_setup(T);
    return 0;
}

Surface preset(int which)
{
    Surface s;
    std::memset(&s, 0, sizeof(s));
    for (int k = 0; k < 4; ++k)
    {
        s.specular[k] = 0.9f - 0.1f * k;
        s.albedo[k] = 0.6f + 0.05f * k;
        s.sheenColor[k] = 0.7f;
    }
    for (float* n : {s.geoN, s.baseN, s.coatN}) n[0] = 0.0f, n[1] = 1.0f, n[2] = 0.0f;
    s.tangent[0] = 1.0f;
    s.ior = 1.5f;
    s.cauchyA = 1.5f;
    s.diffOcc = s.specOcc = 1.0f;
    s.ccIOR = 1.5f;
    switch (which)
    {
    case 0:
        s.ccAmount = 0.5f, s.ccRough = 0.3f, s.sheenAmount = 0.4f, s.sheenRough = 0.5f, s.metalness = 0.3f;
        s.roughness = 0.5f, s.specAmount = 1.0f;
        break;
    case 1: s.transparency = 1.0f, s.roughness = 0.4f, s.specAmount = 1.0f; break;
    case 2: s.roughness = 0.45f, s.specAmount = 1.0f; break;
    default: s.metalness = 1.0f, s.roughness = 0.5f, s.aniso = 0.6f, s.ccAmount = 0.6f, s.ccRough = 0.25f; break;
    }
    return s;
}

int layered(int which, float cosWo, long samples, uint64_t seed, const char* dataDir)
{
    if (int r = setupTables(dataDir)) return r;
    const Surface S = preset(which);
    float wo[3];
    dirOf(cosWo, 0.3, wo);
    const float cur = 1.0f, prev = 1.0f, hero = 550.0f;
    const int front = 1;
    float probs[6];
    orc_layer_probs(S, cur, prev, wo, front, probs);
    std::vector<double> count(kCosBins * kPhiBins + 1, 0.0), expect(kCosBins * kPhiBins + 1, 0.0);
    Rng rng{seed};
    long deltas = 0;
    for (long n = 0; n < samples; ++n)
    {
        float u = rng.uni();
        int layer = 0;
        for (; layer < 5; ++layer)
        {
            if (u < probs[layer] && probs[layer] > 0.0f) break;
            u -= probs[layer];
        }
        const float sel = rng.uni(), r0 = rng.uni(), r1 = rng.uni();
        float wi[3];
        int diffuse = 0, delta = 0;
        orc_sample_layer(S, hero, cur, prev, wo, front, layer, sel, r0, r1, wi, &diffuse, &delta);
        deltas += delta;
        if (wi[0] == 0.0f && wi[1] == 0.0f && wi[2] == 0.0f)
        {
            count[kCosBins * kPhiBins] += 1.0;
            continue;
        }
        const double len = std::sqrt((double)wi[0] * wi[0] + (double)wi[1] * wi[1] + (double)wi[2] * wi[2]);
        const double c = std::fmin(1.0, std::fmax(-1.0, wi[1] / len));
        double phi = std::atan2((double)wi[2], (double)wi[0]);
        if (phi < 0.0) phi += 2.0 * kPi;
        const int ic = std::min(kCosBins - 1, (int)((c + 1.0) * 0.5 * kCosBins));
        const int ip = std::min(kPhiBins - 1, (int)(phi / (2.0 * kPi) * kPhiBins));
        count[ic * kPhiBins + ip] += 1.0;
    }
    const double dc = 2.0 / kCosBins, dp = 2.0 * kPi / kPhiBins;
    auto cellMass = [&](int ic, int ip, int sub, bool& edge) {
        double m = 0.0;
        bool zero = false, nonzero = false;
        for (int a = 0; a < sub; ++a)
            for (int b = 0; b < sub; ++b)
            {
                float wi[3];
                dirOf(-1.0 + (ic + (a + 0.5) / sub) * dc, (ip + (b + 0.5) / sub) * dp, wi);
                const double p = orc_eval_surface(S, hero, cur, prev, wo, front, wi, 2u /* pdf only */).pdf;
                m += p;
                (p > 0.0 ? nonzero : zero) = true;
            }
        edge = zero && nonzero;
        return m * dc * dp / ((double)sub * sub);
    };
    double integral = 0.0;
    for (int ic = 0; ic < kCosBins; ++ic)
        for (int ip = 0; ip < kPhiBins; ++ip)
        {
            bool edge = false;
            double m = cellMass(ic, ip, kSub, edge);
            if (edge) m = cellMass(ic, ip, kFine, edge);
            expect[ic * kPhiBins + ip] = m * samples;
            integral += m;
        }
    expect[kCosBins * kPhiBins] = std::fmax(0.0, 1.0 - integral) * samples;
    double chi2 = 0.0, poolE = 0.0, poolC = 0.0, worst = 0.0;
    int dof = -1;
    for (size_t k = 0; k < count.size(); ++k)
    {
        if (expect[k] >= 5.0)
        {
            const double d = count[k] - expect[k];
            chi2 += d * d / expect[k];
            worst = std::fmax(worst, std::fabs(d) / std::sqrt(expect[k]));
            ++dof;
        }
        else
        {
            poolE += expect[k];
            poolC += count[k];
        }
    }
    if (poolE >= 5.0)
    {
        const double d = poolC - poolE;
        chi2 += d * d / poolE;
        ++dof;
    }
    std::printf("{\"check\": \"layered\", \"preset\": %d, \"cos_wo\": %.4f, \"samples\": %ld, \"chi2\": %.4f, "
                "\"dof\": %d, \"worst_z\": %.3f, \"pdf_integral\": %.6f, \"rejected\": %.0f, \"deltas\": %ld, "
                "\"probs\": [%.4f, %.4f, %.4f, %.4f, %.4f, %.4f]}\n",
                which, cosWo, samples, chi2, dof, worst, integral, count[kCosBins * kPhiBins], deltas, probs[0], probs[1],
                probs[2], probs[3], probs[4], probs[5]);
    return 0;
}
} // namespace

int main(int argc, char** argv)
{
    if (argc >= 2 && std::strcmp(argv[1], "fresnel") == 0) return fresnel();
    if (argc >= 9 && std::strcmp(argv[1], "lobe") == 0)
        return lobe(std::atoi(argv[2]), (float)std::atof(argv[3]), (float)std::atof(argv[4]), (float)std::atof(argv[5]),
                    (float)std::atof(argv[6]), std::atol(argv[7]), (uint64_t)std::strtoull(argv[8], nullptr, 10));
    if (argc >= 9 && std::strcmp(argv[1], "albedo") == 0)
        return albedo(std::atoi(argv[2]), (float)std::atof(argv[3]), (float)std::atof(argv[4]), (float)std::atof(argv[5]),
                      (float)std::atof(argv[6]), std::atol(argv[7]), (uint64_t)std::strtoull(argv[8], nullptr, 10));
    if (argc >= 7 && std::strcmp(argv[1], "layered") == 0)
        return layered(std::atoi(argv[2]), (float)std::atof(argv[3]), std::atol(argv[4]),
                       (uint64_t)std::strtoull(argv[5], nullptr, 10), argv[6]);
    if (argc >= 5 && std::strcmp(argv[1], "reciprocity") == 0)
        return reciprocity(std::atoi(argv[2]), std::atol(argv[3]), (uint64_t)std::strtoull(argv[4], nullptr, 10));
    std::fprintf(stderr, "usage: kat fresnel | kat lobe|albedo <id> <eta> <ax> <ay> <cos wo> <samples> <seed> | "
                         "kat reciprocity <id> <pairs> <seed>\n");
    return 2;
}
