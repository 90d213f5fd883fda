// C-ABI runtime: context, scene ingest, acceleration structure, light tables, render
// submission and film readback. Mirrors the host side of YAPT's path tracer
// (RaytraceCommonResources.cpp, BindlessMaterialManager.cpp, LightManager.cpp,
// PathTraceStage.cpp) on one CUDA stream.
#include "yg_internal.h"
#include "yg_nvtx.h"
#include "yg_vec.cuh"

#include <algorithm>
#include <functional>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

// paths per wavefront wave of yg_render (log2); the path state takes wavefrontBytesPerSlot()
// bytes per path
#ifndef YG_WAVE_CAPACITY_LOG2
#define YG_WAVE_CAPACITY_LOG2 24
#endif

namespace ygi
{
thread_local std::string g_lastError;

int fail(int code, const std::string& msg)
{
    g_lastError = msg;
    return code;
}

float saturatef(float x) { return std::min(std::max(x, 0.0f), 1.0f); }

// BindlessMaterialManager.cpp:73-98
yg::GpuMaterial packMaterial(const yg_material& m)
{
    yg::GpuMaterial g{};
    g.specAmount_ccAmount_ccIOR_ccRough = make_float4(saturatef(m.specular_amount), saturatef(m.clear_coat_amount),
                                                      m.clear_coat_ior, saturatef(m.clear_coat_roughness));
    g.albedo_transparency = make_float4(m.albedo[0], m.albedo[1], m.albedo[2], m.transparency);
    g.specular_metalness = make_float4(m.specular[0], m.specular[1], m.specular[2], m.metalness);
    g.absorption_ior = make_float4(m.absorption[0], m.absorption[1], m.absorption[2],
                                   std::min(std::max(m.dielectric_ior, 0.3f), 3.0f));
    g.emissive_roughness = make_float4(m.emissive[0], m.emissive[1], m.emissive[2], saturatef(m.roughness));
    g.anisotropy = saturatef(m.anisotropy);
    g.anisotropyRotation = m.anisotropy_rotation;
    g.mask = m.material_mask;
    g.thinFilmNM = m.thin_film_thickness_nm;
    g.cauchyA = m.cauchy[0];
    g.cauchyB = m.cauchy[1];
    g.sheenAmount = m.sheen_amount;
    g.emissionFocus = m.emission_focus;
    g.sheenColor_roughness = make_float4(m.sheen_tint[0], m.sheen_tint[1], m.sheen_tint[2], m.sheen_roughness);
    g.subsurfaceRadius_amount =
        make_float4(m.subsurface_radius[0] * m.subsurface_radius_scale, m.subsurface_radius[1] * m.subsurface_radius_scale,
                    m.subsurface_radius[2] * m.subsurface_radius_scale, saturatef(m.subsurface_amount));
    g.albedoSpectrum = m.albedo_spectrum;
    g.specularSpectrum = m.specular_spectrum;
    g.emissionSpectrum = m.emission_spectrum;
    g.textures = make_int4((int)m.albedo_texture - 1, (int)m.normal_texture - 1, (int)m.orm_texture - 1,
                           (int)m.emissive_texture - 1);
    if (m.albedo_texture || m.normal_texture || m.orm_texture || m.emissive_texture) g.mask |= yg::kMaterialTextured;
    g.albedoNormalScale = make_float4(m.albedo_uv_scale[0], m.albedo_uv_scale[1], m.normal_uv_scale[0], m.normal_uv_scale[1]);
    g.ormEmissiveScale = make_float4(m.orm_uv_scale[0], m.orm_uv_scale[1], m.emissive_uv_scale[0], m.emissive_uv_scale[1]);
    return g;
}

bool isGreyOrZero(const float* c) { return c[0] == c[1] && c[0] == c[2]; }

// estimatePunctualLightPower (RaytraceCommonResources.cpp:407-424); directional lights cover
// the world bounds' half diagonal
float punctualPower(const yg_context* ctx, const yg_punctual_light& L)
{
    float intensity = 0.2126f * L.intensity[0] + 0.7152f * L.intensity[1] + 0.0722f * L.intensity[2];
    const float pi = 3.14159274f;
    if (L.type == YG_LIGHT_POINT) return 4.f * pi * intensity;
    if (L.type == YG_LIGHT_SPOT) return 2.f * pi * (1.f - 0.5f * (L.cos_inner + L.cos_outer)) * intensity;
    float ex = (ctx->worldHi[0] - ctx->worldLo[0]) * 0.5f, ey = (ctx->worldHi[1] - ctx->worldLo[1]) * 0.5f,
          ez = (ctx->worldHi[2] - ctx->worldLo[2]) * 0.5f;
    return pi * (ex * ex + ey * ey + ez * ez) * intensity;
}

// Vose alias table (RaytraceCommonResources.cpp:325-383)
void selectionPdfs(std::vector<float>& w)
{
    const float kUniform = 0.1f;
    size_t count = w.size();
    double total = 0;
    for (float x : w) total += x;
    float share = total > 0 ? kUniform : 1.f;
    for (float& x : w)
    {
        float ps = total > 0 ? float(x / total) : 0.f;
        x = (1.f - share) * ps + share / count;
    }
}
void aliasTable(const std::vector<float>& pdfs, std::vector<float>& thr, std::vector<uint32_t>& alias)
{
    size_t count = pdfs.size();
    thr.assign(count, 0.f);
    alias.assign(count, 0);
    std::vector<float> scaled(count);
    std::vector<uint32_t> small, large;
    for (size_t i = 0; i < count; ++i)
    {
        scaled[i] = pdfs[i] * count;
        (scaled[i] < 1.f ? small : large).push_back(uint32_t(i));
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
    for (uint32_t i : large)
    {
        thr[i] = 1.f;
        alias[i] = i;
    }
    for (uint32_t i : small)
    {
        thr[i] = 1.f;
        alias[i] = i;
    }
}

// uploadLightData (RaytraceCommonResources.cpp:426-543): selection pdfs and alias tables over
// the mesh lights then the punctual lights, and over the punctual lights alone; the
// instances' light pdfs are rewritten to match
int uploadLightTable(yg_context* ctx)
{
    const size_t nMesh = ctx->meshLightInst.size(), nP = ctx->punctual.size(), n = nMesh + nP;
    std::vector<float> all(ctx->meshLightPower), pun(nP);
    for (size_t i = 0; i < nP; ++i)
    {
        pun[i] = punctualPower(ctx, ctx->punctual[i]);
        all.push_back(pun[i]);
    }
    std::vector<yg::GpuLight> lights(std::max<size_t>(n, 1));
    std::memset(lights.data(), 0, lights.size() * sizeof(yg::GpuLight));
    for (yg::GpuInstance& G : ctx->hostInst) G.lightPdf = 0.0f;
    std::vector<float> thr, pthr;
    std::vector<uint32_t> alias, palias;
    if (n)
    {
        selectionPdfs(all);
        aliasTable(all, thr, alias);
    }
    if (nP)
    {
        selectionPdfs(pun);
        aliasTable(pun, pthr, palias);
    }
    for (size_t l = 0; l < n; ++l)
    {
        yg::GpuLight& G = lights[l];
        G.selectionPdf = all[l];
        G.aliasThreshold = thr[l];
        G.aliasIndex = alias[l];
        if (l < nMesh)
        {
            G.instance = ctx->meshLightInst[l];
            G.type = yg::kLightMesh;
            ctx->hostInst[G.instance].lightPdf = all[l];
            continue;
        }
        const size_t i = l - nMesh;
        const yg_punctual_light& P = ctx->punctual[i];
        G.instance = 0xffffffffu;
        G.type = P.type;
        G.punctualSelectionPdf = pun[i];
        G.punctualAliasThreshold = pthr[i];
        G.punctualAliasIndex = palias[i];
        G.positionCosInner = make_float4(P.position[0], P.position[1], P.position[2], P.cos_inner);
        G.directionCosOuter = make_float4(P.direction[0], P.direction[1], P.direction[2], P.cos_outer);
        G.intensity = make_float4(P.intensity[0], P.intensity[1], P.intensity[2], 0.0f);
    }
    int r;
    if ((r = upload(ctx, ctx->dLights, lights.data(), lights.size()))) return r;
    if (!ctx->hostInst.empty() && (r = upload(ctx, ctx->dInst, ctx->hostInst.data(), ctx->hostInst.size()))) return r;
    ctx->nLights = (uint32_t)n;
    ctx->nPunctual = (uint32_t)nP;
    return YG_OK;
}

int ensureCie(yg_context* c, int lmin, int lmax)
{
    if (c->cieLmin == lmin && c->cieLmax == lmax) return YG_OK;
    std::vector<float> t;
    float yInv, dInv;
    if (!yg::cieForRange(c->cie471, lmin, lmax, t, yInv, dInv))
        return fail(YG_ERR_INVALID_ARGUMENT, "spectral range must be integer nm within [360, 830]");
    int r = upload(c, c->dCie, t.data(), t.size());
    if (r) return r;
    c->cieLmin = lmin;
    c->cieLmax = lmax;
    c->cieN = (uint32_t)(lmax - lmin + 1);
    c->cieYSumInv = yInv;
    c->d65SumInv = dInv;
    return YG_OK;
}

bool sceneNeedsRgbLut(const yg_context* c, float envScale)
{
    if (envScale > 0.0f) return true;
    for (const yg_material& m : c->materials)
    {
        if (m.albedo_spectrum < 0 && !isGreyOrZero(m.albedo)) return true;
        if (m.specular_spectrum < 0 && !isGreyOrZero(m.specular)) return true;
        if (m.emission_spectrum < 0 && !isGreyOrZero(m.emissive)) return true;
        if (!isGreyOrZero(m.absorption)) return true;
        if (m.sheen_amount > 0.0f && !isGreyOrZero(m.sheen_tint)) return true;
        if (m.subsurface_amount > 0.0f && !isGreyOrZero(m.subsurface_radius)) return true;
    }
    for (const yg_punctual_light& L : c->punctual)
        if (!isGreyOrZero(L.intensity)) return true;
    for (const yg_material& m : c->materials)
        if (m.albedo_texture || m.emissive_texture) return true; // texels may be coloured
    return false;
}

int ensureRgbLut(yg_context* c, int lmin, int lmax)
{
    if (!c->rgbToSpd.empty() && c->rgbLmin == lmin && c->rgbLmax == lmax) return YG_OK;
    yg::buildRgbToSpd(c->cie471, lmin, lmax, c->rgbToSpd);
    c->rgbLmin = lmin;
    c->rgbLmax = lmax;
    return upload(c, c->dRgb, c->rgbToSpd.data(), c->rgbToSpd.size());
}

// fixed pseudo-random permutation of a crop's pixels for the BDPT camera groups (the texel
// remap of BidirectionalPathIntegratorSubStage.cpp:549-591, from a seeded splitmix64 generator)
void pixelPermutation(uint32_t cw, uint32_t ch, std::vector<uint32_t>& perm)
{
    const uint64_t npix = (uint64_t)cw * ch;
    perm.resize(npix);
    for (uint64_t i = 0; i < npix; ++i) perm[i] = (uint32_t)i;
    uint64_t state = 0x9E3779B97F4A7C15ull ^ ((uint64_t)cw << 32 | ch);
    for (uint64_t i = npix - 1; i > 0; --i)
    {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        std::swap(perm[i], perm[z % (i + 1)]);
    }
}

void fillSceneView(const yg_context* ctx, float lminf, float lmaxf, bool needRgb, yg::SceneView& S)
{
    S = yg::SceneView{};
    S.tris = ctx->dTris.as<float4>();
    S.nodes = ctx->dNodes.as<float4>();
    S.instances = ctx->dInst.as<yg::GpuInstance>();
    S.materials = ctx->dMat.as<yg::GpuMaterial>();
    S.lights = ctx->dLights.as<yg::GpuLight>();
    S.positions = ctx->dPos.as<float>();
    S.normals = ctx->dNrm.as<float>();
    S.tangents = ctx->dTan.as<float4>();
    S.uvs = ctx->dUV.as<float2>();
    S.textures = ctx->dTexTable.as<yg::GpuTexture>();
    S.instPrimStart = ctx->dPrimStart.as<uint32_t>();
    S.triOfPrim = ctx->dTriOfPrim.as<uint32_t>();
    S.nNodes = (uint32_t)ctx->nNodes;
    S.nTris = (uint32_t)ctx->nTris;
    S.boundsErrors = ctx->dBoundsErr.as<unsigned int>();
    S.envTexture = ctx->envTexture;
    S.envCube = ctx->envCube ? 1u : 0u;
    S.indices = ctx->dIdx.as<uint32_t>();
    S.spectra = ctx->dSpec.as<float>();
    S.lutSS = ctx->dLut[0].as<float>();
    S.lutSSAvg = ctx->dLut[1].as<float>();
    S.lutSSMS = ctx->dLut[2].as<float>();
    S.lutSSMSAvg = ctx->dLut[3].as<float>();
    S.lutTransDenser = ctx->dLut[4].as<float>();
    S.lutTransLighter = ctx->dLut[5].as<float>();
    S.lutTransAvgDenser = ctx->dLut[6].as<float>();
    S.lutTransAvgLighter = ctx->dLut[7].as<float>();
    S.lutSheen = ctx->dLut[8].as<float>();
    S.cie = ctx->dCie.as<float4>();
    S.rgbToSpd = needRgb ? ctx->dRgb.as<float>() : nullptr;
    S.cam = ctx->camera;
    S.nLights = ctx->nLights;
    S.nPunctual = ctx->nPunctual;
    S.nInstances = (uint32_t)ctx->instances.size();
    S.specPoints = ctx->specPoints;
    S.specLmin = ctx->specLmin;
    S.specLmax = ctx->specLmax;
    S.cieN = ctx->cieN;
    S.lambdaMin = lminf;
    S.lambdaMax = lmaxf;
    S.cieYSumInv = ctx->cieYSumInv;
    S.d65SumInv = ctx->d65SumInv;
}

int checkMaterialTextures(const yg_context* c, const char* what)
{
    const size_t nTex = c->texTable.size();
    for (const yg_material& m : c->materials)
        if (m.albedo_texture > nTex || m.normal_texture > nTex || m.orm_texture > nTex || m.emissive_texture > nTex)
            return fail(YG_ERR_INVALID_ARGUMENT,
                        std::string(what) + ": a material refers to a texture that was not uploaded (or was cleared)");
    return YG_OK;
}
} // namespace ygi

using namespace ygi;

extern "C" {

YG_API const char* yg_last_error(void) { return g_lastError.c_str(); }
YG_API int yg_version(void) { return 1; }

YG_API int yg_create(const char* data_dir, int device, yg_context** out)
{
    if (!out || !data_dir) return fail(YG_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    int n = 0;
    YG_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(YG_ERR_INVALID_ARGUMENT, "no such CUDA device");
    YG_CUDA(cudaSetDevice(device));
    yg_context* c = new yg_context();
    c->device = device;
    c->dataDir = data_dir;
    cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, device);
    std::string err;
    if (!yg::buildSobolMatrices(c->dataDir + "/joe_kuo_6_21201_first256.txt", c->sobolMatrices, err) ||
        !yg::loadCie(c->dataDir + "/cie1931_2deg_d65_1nm.txt", c->cie471, err))
    {
        delete c;
        return fail(YG_ERR_IO, err);
    }
    yg::buildMsLuts(c->luts);
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evStart);
    if (e == cudaSuccess) e = cudaEventCreate(&c->evStop);
    if (e != cudaSuccess)
    {
        delete c;
        return fail(YG_ERR_CUDA, cudaGetErrorString(e));
    }
    const std::vector<float>* L[9] = {&c->luts.ss, &c->luts.ssAvg, &c->luts.ssms, &c->luts.ssmsAvg, &c->luts.transDenser,
                                      &c->luts.transLighter, &c->luts.transAvgDenser, &c->luts.transAvgLighter,
                                      &c->luts.sheen};
    for (int i = 0; i < 9; ++i)
    {
        int r = upload(c, c->dLut[i], L[i]->data(), L[i]->size());
        if (r)
        {
            delete c;
            return r;
        }
    }
    int r = ensureCie(c, 380, 700);
    if (r)
    {
        delete c;
        return r;
    }
    YG_CUDA(cudaStreamSynchronize(c->stream));
    *out = c;
    return YG_OK;
}

YG_API int yg_destroy(yg_context* ctx)
{
    if (!ctx) return YG_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    delete ctx;
    return YG_OK;
}

YG_API int yg_synchronize(yg_context* ctx)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API int yg_get_table(yg_context* ctx, int which, void* out, size_t capacity, size_t* count)
{
    if (!ctx || !count) return fail(YG_ERR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    const void* src = nullptr;
    size_t n = 0, elem = 4;
    std::vector<float> tmp;
    const std::vector<float>* L[9] = {&ctx->luts.ss, &ctx->luts.ssAvg, &ctx->luts.ssms, &ctx->luts.ssmsAvg,
                                      &ctx->luts.transDenser, &ctx->luts.transLighter, &ctx->luts.transAvgDenser,
                                      &ctx->luts.transAvgLighter, &ctx->luts.sheen};
    if (which == YG_TABLE_SOBOL_MATRICES)
    {
        src = ctx->sobolMatrices.data();
        n = ctx->sobolMatrices.size();
    }
    else if (which >= YG_TABLE_LUT_SS_NOFRESNEL && which <= YG_TABLE_LUT_SHEEN)
    {
        src = L[which - 1]->data();
        n = L[which - 1]->size();
    }
    else if (which == YG_TABLE_CIE_1NM)
    {
        tmp.assign(ctx->cie471.begin(), ctx->cie471.end());
        src = tmp.data();
        n = tmp.size();
    }
    else if (which == YG_TABLE_RGB_TO_SPD)
    {
        int lmin = ctx->cieLmin, lmax = ctx->cieLmax;
        if (ctx->rgbToSpd.empty() || ctx->rgbLmin != lmin || ctx->rgbLmax != lmax)
        {
            int r = ensureRgbLut(ctx, lmin, lmax);
            if (r) return r;
        }
        src = ctx->rgbToSpd.data();
        n = ctx->rgbToSpd.size();
    }
    else
    {
        return fail(YG_ERR_INVALID_ARGUMENT, "unknown table");
    }
    *count = n;
    if (out)
    {
        if (capacity < n) return fail(YG_ERR_INVALID_ARGUMENT, "table buffer too small");
        std::memcpy(out, src, n * elem);
    }
    return YG_OK;
}

YG_API int yg_host_table(const char* data_dir, int which, int lmin, int lmax, void* out, size_t capacity, size_t* count)
{
    if (!data_dir || !count) return fail(YG_ERR_INVALID_ARGUMENT, "null argument");
    std::string dir(data_dir), err;
    std::vector<uint32_t> u;
    std::vector<float> f;
    std::vector<double> cie;
    if (which == YG_TABLE_SOBOL_MATRICES)
    {
        if (!yg::buildSobolMatrices(dir + "/joe_kuo_6_21201_first256.txt", u, err)) return fail(YG_ERR_IO, err);
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
        f = *L[which - 1];
    }
    else if (which == YG_TABLE_CIE_1NM || which == YG_TABLE_RGB_TO_SPD)
    {
        if (!yg::loadCie(dir + "/cie1931_2deg_d65_1nm.txt", cie, err)) return fail(YG_ERR_IO, err);
        if (which == YG_TABLE_CIE_1NM) f.assign(cie.begin(), cie.end());
        else
        {
            if (lmin < 360 || lmax > 830 || lmax <= lmin) return fail(YG_ERR_INVALID_ARGUMENT, "bad spectral range");
            yg::buildRgbToSpd(cie, lmin, lmax, f);
        }
    }
    else
    {
        return fail(YG_ERR_INVALID_ARGUMENT, "unknown table");
    }
    size_t n = u.empty() ? f.size() : u.size();
    *count = n;
    if (out)
    {
        if (capacity < n) return fail(YG_ERR_INVALID_ARGUMENT, "table buffer too small");
        std::memcpy(out, u.empty() ? (const void*)f.data() : (const void*)u.data(), n * 4);
    }
    return YG_OK;
}

YG_API int yg_upload_mesh(yg_context* ctx, const yg_mesh_desc* d, uint32_t* mesh_id)
{
    if (!ctx || !d || !mesh_id || !d->positions || !d->normals || !d->indices)
        return fail(YG_ERR_INVALID_ARGUMENT, "mesh: null argument");
    if (d->index_bits != 16 && d->index_bits != 32) return fail(YG_ERR_INVALID_ARGUMENT, "mesh: index_bits must be 16 or 32");
    if (d->index_count % 3 != 0) return fail(YG_ERR_INVALID_ARGUMENT, "mesh: index_count must be a multiple of 3");
    std::lock_guard<std::mutex> g(ctx->lock);
    Mesh m;
    m.vertexBase = (uint32_t)(ctx->positions.size() / 3);
    m.vertexCount = d->vertex_count;
    m.indexBase = (uint32_t)ctx->indices.size();
    m.indexCount = d->index_count;
    m.tangents = d->tangents != nullptr;
    m.uvs = d->uvs != nullptr;
    for (uint32_t i = 0; i < d->index_count; ++i)
    {
        uint32_t v = d->index_bits == 16 ? ((const uint16_t*)d->indices)[i] : ((const uint32_t*)d->indices)[i];
        if (v >= d->vertex_count) return fail(YG_ERR_INVALID_ARGUMENT, "mesh: index out of range");
    }
    if (d->submesh_count == 0 || !d->submesh_ranges)
    {
        m.submeshes.push_back({0u, d->index_count});
    }
    else
    {
        for (uint32_t s = 0; s < d->submesh_count; ++s)
        {
            uint32_t first = d->submesh_ranges[2 * s], cnt = d->submesh_ranges[2 * s + 1];
            if (first % 3 || cnt % 3 || (uint64_t)first + cnt > d->index_count)
                return fail(YG_ERR_INVALID_ARGUMENT, "mesh: invalid submesh range");
            m.submeshes.push_back({first, cnt});
        }
    }
    ctx->positions.insert(ctx->positions.end(), d->positions, d->positions + 3 * (size_t)d->vertex_count);
    ctx->normals.insert(ctx->normals.end(), d->normals, d->normals + 3 * (size_t)d->vertex_count);
    for (uint32_t i = 0; i < d->vertex_count; ++i)
    {
        ctx->tangents.push_back(d->tangents ? make_float4(d->tangents[4 * i], d->tangents[4 * i + 1], d->tangents[4 * i + 2],
                                                          d->tangents[4 * i + 3])
                                            : make_float4(1.f, 0.f, 0.f, 1.f));
        ctx->uvs.push_back(d->uvs ? d->uvs[2 * i] : 0.5f);
        ctx->uvs.push_back(d->uvs ? d->uvs[2 * i + 1] : 0.5f);
    }
    for (uint32_t i = 0; i < d->index_count; ++i)
        ctx->indices.push_back(d->index_bits == 16 ? ((const uint16_t*)d->indices)[i] : ((const uint32_t*)d->indices)[i]);
    *mesh_id = (uint32_t)ctx->meshes.size();
    ctx->meshes.push_back(m);
    ctx->sceneBuilt = false;
    return YG_OK;
}

YG_API int yg_clear_meshes(yg_context* ctx)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    ctx->positions.clear();
    ctx->normals.clear();
    ctx->tangents.clear();
    ctx->uvs.clear();
    ctx->indices.clear();
    ctx->meshes.clear();
    ctx->sceneBuilt = false;
    return YG_OK;
}

YG_API int yg_upload_materials(yg_context* ctx, const yg_material* mats, uint32_t count)
{
    if (!ctx || (!mats && count)) return fail(YG_ERR_INVALID_ARGUMENT, "materials: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    ctx->materials.assign(mats, mats + count);
    ctx->gpuMaterials.resize(count);
    for (uint32_t i = 0; i < count; ++i) ctx->gpuMaterials[i] = packMaterial(mats[i]);
    ctx->sceneBuilt = false;
    return upload(ctx, ctx->dMat, ctx->gpuMaterials.data(), ctx->gpuMaterials.size());
}

// sRGB electro-optical transfer function (IEC 61966-2-1), in double
static double srgbToLinear(double c) { return c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4); }

YG_API int yg_upload_texture(yg_context* ctx, uint32_t width, uint32_t height, uint32_t format, const void* data,
                             uint32_t* texture_id)
{
    if (!ctx || !data || !texture_id) return fail(YG_ERR_INVALID_ARGUMENT, "texture: null argument");
    if (width == 0 || height == 0 || width > 32768 || height > 32768) return fail(YG_ERR_INVALID_ARGUMENT, "texture: bad size");
    if (format > YG_TEXTURE_RGBA32_FLOAT) return fail(YG_ERR_INVALID_ARGUMENT, "texture: unknown format");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t n = (size_t)width * height;
    std::vector<float4> texels(n);
    if (format == YG_TEXTURE_RGBA32_FLOAT)
    {
        const float* f = static_cast<const float*>(data);
        for (size_t i = 0; i < 4 * n; ++i)
            if (!std::isfinite(f[i])) return fail(YG_ERR_INVALID_ARGUMENT, "texture: non-finite texel");
        std::memcpy(texels.data(), f, n * sizeof(float4));
    }
    else
    {
        float lut[256];
        for (int v = 0; v < 256; ++v)
            lut[v] = format == YG_TEXTURE_RGBA8_SRGB ? (float)srgbToLinear(v / 255.0) : (float)(v / 255.0);
        const uint8_t* b = static_cast<const uint8_t*>(data);
        for (size_t i = 0; i < n; ++i)
            texels[i] = make_float4(lut[b[4 * i]], lut[b[4 * i + 1]], lut[b[4 * i + 2]], (float)(b[4 * i + 3] / 255.0));
    }
    cudaSetDevice(ctx->device);
    DevBuf buf;
    int r = upload(ctx, buf, texels.data(), n);
    if (r) return r;
    ctx->texBufs.push_back(buf);
    ctx->texTable.push_back(yg::GpuTexture{buf.as<float4>(), width, height});
    if ((r = upload(ctx, ctx->dTexTable, ctx->texTable.data(), ctx->texTable.size()))) return r;
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    *texture_id = (uint32_t)ctx->texTable.size() - 1;
    return YG_OK;
}

YG_API int yg_clear_textures(yg_context* ctx)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "textures: null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    cudaSetDevice(ctx->device);
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (DevBuf& b : ctx->texBufs) b.release();
    // the cutout records of a built scene refer to texture memory: the scene is built again
    if (ctx->nAlphaInstances) ctx->sceneBuilt = false;
    ctx->texBufs.clear();
    ctx->texTable.clear();
    ctx->envTexture = -1;
    ctx->envCube = false;
    return YG_OK;
}

YG_API int yg_set_environment_texture(yg_context* ctx, uint32_t texture)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "environment: null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (texture > ctx->texTable.size()) return fail(YG_ERR_INVALID_ARGUMENT, "environment: unknown texture");
    ctx->envTexture = (int)texture - 1;
    ctx->envCube = false;
    return YG_OK;
}

YG_API int yg_set_environment_cube(yg_context* ctx, uint32_t texture)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "environment: null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (texture == 0 || texture > ctx->texTable.size()) return fail(YG_ERR_INVALID_ARGUMENT, "environment: unknown texture");
    const yg::GpuTexture& T = ctx->texTable[texture - 1];
    if (T.height != 6 * T.width)
        return fail(YG_ERR_INVALID_ARGUMENT, "environment: a cube map is six square faces stacked (height = 6 x width)");
    ctx->envTexture = (int)texture - 1;
    ctx->envCube = true;
    return YG_OK;
}

YG_API int yg_upload_spectra(yg_context* ctx, const float* values, uint32_t n_curves, uint32_t n_points, float lmin,
                             float lmax)
{
    if (!ctx || (!values && n_curves)) return fail(YG_ERR_INVALID_ARGUMENT, "spectra: null argument");
    if (n_curves && (n_points < 2 || !(lmax > lmin))) return fail(YG_ERR_INVALID_ARGUMENT, "spectra: need >= 2 points and lmax > lmin");
    std::lock_guard<std::mutex> g(ctx->lock);
    ctx->spectra.assign(values, values + (size_t)n_curves * n_points);
    ctx->specPoints = n_points;
    ctx->specLmin = lmin;
    ctx->specLmax = lmax;
    return upload(ctx, ctx->dSpec, ctx->spectra.data(), ctx->spectra.size());
}

YG_API int yg_set_instances(yg_context* ctx, const yg_instance* inst, uint32_t count)
{
    if (!ctx || (!inst && count)) return fail(YG_ERR_INVALID_ARGUMENT, "instances: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    ctx->instances.assign(inst, inst + count);
    ctx->sceneBuilt = false;
    return YG_OK;
}

YG_API int yg_set_camera(yg_context* ctx, const yg_camera* cam)
{
    if (!ctx || !cam) return fail(YG_ERR_INVALID_ARGUMENT, "camera: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    std::memcpy(ctx->camera.uvToView, cam->uv_to_view, 64);
    std::memcpy(ctx->camera.viewToUV, cam->view_to_uv, 64);
    std::memcpy(ctx->camera.worldToView, cam->world_to_view, 64);
    std::memcpy(ctx->camera.viewToWorld, cam->view_to_world, 64);
    ctx->camera.apertureRadius = std::max(0.0f, cam->aperture_radius);
    ctx->camera.focusDistance = std::max(1e-4f, cam->focus_distance);
    ctx->camera.forwardZSign = cam->view_forward_z_sign;
    ctx->cameraSet = true;
    return YG_OK;
}

extern "C++"
{
namespace
{
struct WideNodeHost
{
    float p[3];
    uint32_t e[3], imask, childBase, triBase, meta[8], qlo[3][8], qhi[3][8];
};

WideNodeHost decodeWide(const float4* n)
{
    auto u = [](float f) {
        uint32_t v;
        std::memcpy(&v, &f, 4);
        return v;
    };
    WideNodeHost w;
    w.p[0] = n[0].x, w.p[1] = n[0].y, w.p[2] = n[0].z;
    uint32_t pk = u(n[0].w);
    w.e[0] = pk & 0xffu, w.e[1] = (pk >> 8) & 0xffu, w.e[2] = (pk >> 16) & 0xffu, w.imask = pk >> 24;
    w.childBase = u(n[1].x), w.triBase = u(n[1].y);
    const uint32_t words[10] = {u(n[1].z), u(n[1].w), u(n[2].x), u(n[2].y), u(n[2].z), u(n[2].w), u(n[3].x), u(n[3].y),
                                u(n[3].z), u(n[3].w)};
    const uint32_t words2[4] = {u(n[4].x), u(n[4].y), u(n[4].z), u(n[4].w)};
    auto byteAt = [](uint32_t a, uint32_t b, int i) { return ((i < 4 ? a : b) >> (8 * (i & 3))) & 0xffu; };
    for (int i = 0; i < 8; ++i)
    {
        w.meta[i] = byteAt(words[0], words[1], i);
        w.qlo[0][i] = byteAt(words[2], words[3], i);
        w.qlo[1][i] = byteAt(words[4], words[5], i);
        w.qlo[2][i] = byteAt(words[6], words[7], i);
        w.qhi[0][i] = byteAt(words[8], words[9], i);
        w.qhi[1][i] = byteAt(words2[0], words2[1], i);
        w.qhi[2][i] = byteAt(words2[2], words2[3], i);
    }
    return w;
}
} // namespace

// Walks the wide tree from the root: every inner child index in range and reached once,
// every triangle slot in range and referenced once, depth within the traversal stack.
int ygi::checkWideBvhStructure(yg_context* ctx)
{
    std::vector<float4> nodes((size_t)ctx->nNodes * 5);
    YG_CUDA(cudaMemcpyAsync(nodes.data(), ctx->dNodes.p, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    std::vector<uint8_t> seen(ctx->nNodes, 0), triSeen(ctx->nTris, 0);
    std::vector<std::pair<uint32_t, uint32_t>> todo{{0u, 1u}};
    seen[0] = 1;
    uint64_t nodeCount = 0, triCount = 0;
    while (!todo.empty())
    {
        auto [idx, depth] = todo.back();
        todo.pop_back();
        ++nodeCount;
        if (depth > (uint32_t)yg::kWideMaxDepth) return fail(YG_ERR_CUDA, "bvh check: tree too deep");
        WideNodeHost w = decodeWide(&nodes[5 * (size_t)idx]);
        uint32_t rank = 0;
        for (int i = 0; i < 8; ++i)
        {
            if (w.imask & (1u << i))
            {
                uint64_t c = (uint64_t)w.childBase + rank++;
                if (c >= ctx->nNodes || seen[c]) return fail(YG_ERR_CUDA, "bvh check: bad inner child reference");
                seen[c] = 1;
                todo.push_back({(uint32_t)c, depth + 1});
            }
            else if (w.meta[i])
            {
                uint32_t cnt = w.meta[i] >> 5, off = w.meta[i] & 31u;
                if (cnt == 0 || cnt > (uint32_t)yg::kMaxLeafTris || off + cnt > 24)
                    return fail(YG_ERR_CUDA, "bvh check: bad leaf slot");
                for (uint32_t k = 0; k < cnt; ++k)
                {
                    uint64_t t = (uint64_t)w.triBase + off + k;
                    if (t >= ctx->nTris || triSeen[t]) return fail(YG_ERR_CUDA, "bvh check: bad triangle reference");
                    triSeen[t] = 1;
                    ++triCount;
                }
            }
        }
    }
    if (nodeCount != ctx->nNodes || triCount != ctx->nTris)
        return fail(YG_ERR_CUDA, "bvh check: " + std::to_string(nodeCount) + " nodes / " + std::to_string(triCount) +
                                     " triangles reachable of " + std::to_string(ctx->nNodes) + " / " +
                                     std::to_string(ctx->nTris));
    return YG_OK;
}

} // extern "C++"

YG_API int yg_bvh_check(yg_context* ctx, uint64_t* n_nodes, uint64_t* depth, uint64_t* violations)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (!ctx->sceneBuilt) return fail(YG_ERR_NOT_READY, "bvh check: no scene built");
    int r;
    if ((r = checkWideBvhStructure(ctx))) return r;
    std::vector<float4> nodes((size_t)ctx->nNodes * 5), tris((size_t)ctx->nTris * 3);
    YG_CUDA(cudaMemcpy(nodes.data(), ctx->dNodes.p, nodes.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    if (!tris.empty()) YG_CUDA(cudaMemcpy(tris.data(), ctx->dTris.p, tris.size() * sizeof(float4), cudaMemcpyDeviceToHost));
    // bounds (double) of the triangles under each slot must lie in the slot's dequantised box
    uint64_t bad = 0;
    struct Box
    {
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        void grow(const Box& b)
        {
            for (int a = 0; a < 3; ++a) lo[a] = std::min(lo[a], b.lo[a]), hi[a] = std::max(hi[a], b.hi[a]);
        }
    };
    auto triBox = [&](uint64_t t) {
        Box b;
        const float4 *v = &tris[3 * t], *e1 = v + 1, *e2 = v + 2;
        const double p0[3] = {v->x, v->y, v->z};
        const double p1[3] = {p0[0] + e1->x, p0[1] + e1->y, p0[2] + e1->z};
        const double p2[3] = {p0[0] + e2->x, p0[1] + e2->y, p0[2] + e2->z};
        for (int a = 0; a < 3; ++a)
        {
            b.lo[a] = std::min({p0[a], p1[a], p2[a]});
            b.hi[a] = std::max({p0[a], p1[a], p2[a]});
        }
        return b;
    };
    uint64_t maxDepth = 0;
    std::function<Box(uint32_t, uint64_t)> visit = [&](uint32_t idx, uint64_t d) -> Box {
        maxDepth = std::max(maxDepth, d);
        WideNodeHost w = decodeWide(&nodes[5 * (size_t)idx]);
        Box all;
        uint32_t rank = 0;
        for (int i = 0; i < 8; ++i)
        {
            Box cb;
            if (w.imask & (1u << i)) cb = visit(w.childBase + rank++, d + 1);
            else if (w.meta[i])
                for (uint32_t k = 0; k < (w.meta[i] >> 5); ++k) cb.grow(triBox((uint64_t)w.triBase + (w.meta[i] & 31u) + k));
            else continue;
            for (int a = 0; a < 3; ++a)
            {
                double scale = std::ldexp(1.0, (int)w.e[a] - 127);
                double lo = (double)w.p[a] + scale * w.qlo[a][i], hi = (double)w.p[a] + scale * w.qhi[a][i];
                if (!(cb.lo[a] >= lo && cb.hi[a] <= hi)) ++bad;
            }
            all.grow(cb);
        }
        return all;
    };
    if (ctx->nTris) visit(0, 1);
    if (n_nodes) *n_nodes = ctx->nNodes;
    if (depth) *depth = maxDepth;
    if (violations) *violations = bad;
    return YG_OK;
}

YG_API int yg_build_scene(yg_context* ctx)
{
    yg::NvtxRange range("yg_build_scene");
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    cudaSetDevice(ctx->device);
    const uint32_t nCurves = ctx->specPoints ? (uint32_t)(ctx->spectra.size() / ctx->specPoints) : 0u;
    for (const yg_material& m : ctx->materials)
    {
        const int32_t ids[3] = {m.albedo_spectrum, m.specular_spectrum, m.emission_spectrum};
        for (int32_t id : ids)
            if (id >= 0 && (uint32_t)id >= nCurves)
                return fail(YG_ERR_INVALID_ARGUMENT, "material references a spectrum that was not uploaded");
    }
    const size_t nInst = ctx->instances.size();
    std::vector<yg::GpuInstance> gi(nInst);
    std::vector<float> power;
    std::vector<uint32_t> lightInst;
    std::vector<uint32_t> primStart(nInst + 1, 0);
    std::vector<yg::GpuAlphaSource> alphaSrc;
    for (size_t i = 0; i < nInst; ++i)
    {
        const yg_instance& I = ctx->instances[i];
        if (I.mesh >= ctx->meshes.size()) return fail(YG_ERR_INVALID_ARGUMENT, "instance: bad mesh id");
        const Mesh& m = ctx->meshes[I.mesh];
        if (I.submesh >= m.submeshes.size()) return fail(YG_ERR_INVALID_ARGUMENT, "instance: bad submesh");
        if (I.material >= ctx->materials.size()) return fail(YG_ERR_INVALID_ARGUMENT, "instance: bad material id");
        yg::GpuInstance& G = gi[i];
        for (int r = 0; r < 3; ++r)
        {
            G.o2w[r] = make_float4(I.obj_to_world[4 * r], I.obj_to_world[4 * r + 1], I.obj_to_world[4 * r + 2], I.obj_to_world[4 * r + 3]);
            G.w2o[r] = make_float4(I.world_to_obj[4 * r], I.world_to_obj[4 * r + 1], I.world_to_obj[4 * r + 2], I.world_to_obj[4 * r + 3]);
        }
        G.firstIndex = m.indexBase + m.submeshes[I.submesh].first;
        G.primCount = m.submeshes[I.submesh].second / 3;
        G.vertexBase = m.vertexBase;
        G.material = I.material;
        G.lightPdf = 0.0f;
        G.hasTangents = m.tangents ? 1u : 0u;
        G.hasUVs = m.uvs ? 1u : 0u;
        G.alphaSource = 0;
        // alpha-tested: a cutoff above 0, an albedo texture and texture coordinates
        // (alphaTestPasses, hitShadersCommon.hlsl:162-175); the texture must be uploaded first
        const yg_material& AM = ctx->materials[I.material];
        if (AM.alpha_cutoff > 0.0f && AM.albedo_texture && m.uvs)
        {
            if (AM.albedo_texture > ctx->texTable.size())
                return fail(YG_ERR_INVALID_ARGUMENT, "an alpha-tested material's albedo texture is not uploaded");
            const yg::GpuTexture& T = ctx->texTable[AM.albedo_texture - 1];
            yg::GpuAlphaSource A{};
            A.texels = T.texels;
            A.size = T.width | T.height << 16;
            A.cutoff = AM.alpha_cutoff;
            A.su = AM.albedo_uv_scale[0];
            A.sv = AM.albedo_uv_scale[1];
            alphaSrc.push_back(A);
            G.alphaSource = (uint32_t)alphaSrc.size();
        }
        if ((uint64_t)primStart[i] + G.primCount > 0xffffffffull) return fail(YG_ERR_INVALID_ARGUMENT, "scene: too many triangles");
        primStart[i + 1] = primStart[i] + G.primCount;
        // mesh lights: emissive materials (LightManager.cpp:145), power estimate of
        // estimateMeshLightPower (RaytraceCommonResources.cpp:385-404) over the instance's
        // world-space bounds
        const yg_material& M = ctx->materials[I.material];
        if (M.emissive[0] + M.emissive[1] + M.emissive[2] > 0.0f && G.primCount > 0)
        {
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (uint32_t p = 0; p < G.primCount; ++p)
                for (int k = 0; k < 3; ++k)
                {
                    uint32_t vi = ctx->indices[G.firstIndex + 3 * p + k] + G.vertexBase;
                    float3 ob = yg::mk3(ctx->positions[3 * vi], ctx->positions[3 * vi + 1], ctx->positions[3 * vi + 2]);
                    float3 w = yg::xformPoint(G.o2w, ob);
                    lo[0] = std::min(lo[0], w.x); lo[1] = std::min(lo[1], w.y); lo[2] = std::min(lo[2], w.z);
                    hi[0] = std::max(hi[0], w.x); hi[1] = std::max(hi[1], w.y); hi[2] = std::max(hi[2], w.z);
                }
            float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
            float area = ex * ey + ey * ez + ez * ex;
            float e = 0.2126f * M.emissive[0] + 0.7152f * M.emissive[1] + 0.0722f * M.emissive[2];
            if (e <= 0.f) e = 1.f;
            float sides = (M.material_mask & YG_MATERIAL_TWO_SIDED) ? 2.f : 1.f;
            power.push_back(3.14159274f * e * area * sides);
            lightInst.push_back((uint32_t)i);
        }
    }
    ctx->meshLightInst = lightInst;
    ctx->meshLightPower = power;
    int r;
    if ((r = upload(ctx, ctx->dInst, gi.data(), gi.size()))) return r;
    if ((r = upload(ctx, ctx->dPos, ctx->positions.data(), ctx->positions.size()))) return r;
    if ((r = upload(ctx, ctx->dNrm, ctx->normals.data(), ctx->normals.size()))) return r;
    if ((r = upload(ctx, ctx->dTan, ctx->tangents.data(), ctx->tangents.size()))) return r;
    if ((r = upload(ctx, ctx->dUV, ctx->uvs.data(), ctx->uvs.size()))) return r;
    if ((r = upload(ctx, ctx->dIdx, ctx->indices.data(), ctx->indices.size()))) return r;
    if (ctx->dSpec.p == nullptr)
    {
        float z[4] = {0, 0, 0, 0};
        if ((r = upload(ctx, ctx->dSpec, z, 4))) return r;
    }
    // the acceleration structure, built on the device
    DevBuf dAlpha;
    if (!alphaSrc.empty() && (r = upload(ctx, dAlpha, alphaSrc.data(), alphaSrc.size()))) return r;
    yg::WideBvhInput bin{ctx->dInst.as<yg::GpuInstance>(), (uint32_t)nInst, primStart, ctx->dPos.as<float>(),
                         ctx->dIdx.as<uint32_t>(), primStart[nInst], ctx->dUV.as<float2>(),
                         alphaSrc.empty() ? nullptr : dAlpha.as<yg::GpuAlphaSource>()};
    yg::WideBvhOutput bout{};
    std::string berr;
    const int built = yg::buildWideBvh(bin, bout, ctx->stream, berr);
    const cudaError_t synced = cudaStreamSynchronize(ctx->stream); // the build reads the cutout sources
    dAlpha.release();
    if (built != 0) return fail(YG_ERR_CUDA, berr);
    YG_CUDA(synced);
    ctx->dTris.adopt(bout.tris, 3 * sizeof(float4) * std::max<uint32_t>(primStart[nInst], 1) *
                                    (alphaSrc.empty() || primStart[nInst] == 0 ? 1 : 2));
    ctx->nAlphaInstances = (uint32_t)alphaSrc.size();
    ctx->dNodes.adopt(bout.nodes, 5 * sizeof(float4) * (size_t)bout.nNodes);
    ctx->nTris = primStart[nInst];
    ctx->nNodes = bout.nNodes;
    // each primitive's position in the triangle array, for visibility tests that intersect
    // their target triangle before traversing
    if ((r = upload(ctx, ctx->dPrimStart, primStart.data(), primStart.size()))) return r;
    if (!ctx->dBoundsErr.p)
    {
        YG_CUDA(ctx->dBoundsErr.ensure(16));
        YG_CUDA(cudaMemsetAsync(ctx->dBoundsErr.p, 0, 16, ctx->stream));
    }
    YG_CUDA(ctx->dTriOfPrim.ensure(4 * (size_t)std::max<uint32_t>(primStart[nInst], 1)));
    YG_CUDA((cudaError_t)yg::indexTrianglesByPrim(bout.tris, primStart[nInst], ctx->dPrimStart.as<uint32_t>(),
                                                    ctx->dTriOfPrim.as<uint32_t>(), ctx->stream));
    ctx->bvhDepth = bout.depth;
    ctx->hostInst = gi;
    // every inner node reachable exactly once and every triangle referenced exactly once,
    // checked before any ray can traverse the tree
    if ((r = checkWideBvhStructure(ctx))) return r;
    // world bounds of all triangles (RaytraceCommonResources.cpp:560-600 unions the object bounds)
    float ext2 = 0.0f;
    for (int k = 0; k < 3; ++k)
    {
        ctx->worldCenter[k] = (bout.hi[k] + bout.lo[k]) * 0.5f;
        float e = bout.hi[k] - ctx->worldCenter[k];
        ext2 += e * e;
    }
    ctx->worldRadiusSqr = ext2;
    for (int k = 0; k < 3; ++k)
    {
        ctx->worldLo[k] = bout.lo[k];
        ctx->worldHi[k] = bout.hi[k];
    }
    if ((r = uploadLightTable(ctx))) return r;
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->sceneBuilt = true;
    return YG_OK;
}

YG_API int yg_set_punctual_lights(yg_context* ctx, const yg_punctual_light* lights, uint32_t count)
{
    if (!ctx || (!lights && count)) return fail(YG_ERR_INVALID_ARGUMENT, "punctual lights: null argument");
    std::vector<yg_punctual_light> v(lights, lights + count);
    for (yg_punctual_light& L : v)
    {
        if (L.type < YG_LIGHT_POINT || L.type > YG_LIGHT_DIRECTIONAL)
            return fail(YG_ERR_INVALID_ARGUMENT, "punctual lights: unknown type");
        const float* f = &L.position[0];
        for (int k = 0; k < 11; ++k)
            if (!std::isfinite(f[k])) return fail(YG_ERR_INVALID_ARGUMENT, "punctual lights: non-finite parameter");
        if (L.intensity[0] < 0.f || L.intensity[1] < 0.f || L.intensity[2] < 0.f)
            return fail(YG_ERR_INVALID_ARGUMENT, "punctual lights: negative intensity");
        if (L.type != YG_LIGHT_POINT)
        {
            float d = std::sqrt(L.direction[0] * L.direction[0] + L.direction[1] * L.direction[1] + L.direction[2] * L.direction[2]);
            if (!(d > 0.0f)) return fail(YG_ERR_INVALID_ARGUMENT, "punctual lights: zero direction");
            for (int k = 0; k < 3; ++k) L.direction[k] = L.direction[k] / d;
        }
    }
    std::lock_guard<std::mutex> g(ctx->lock);
    ctx->punctual = v;
    if (!ctx->sceneBuilt) return YG_OK;
    cudaSetDevice(ctx->device);
    int r = uploadLightTable(ctx);
    if (r) return r;
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API int yg_scene_info(yg_context* ctx, uint64_t* nt, uint64_t* nn, uint64_t* nl, uint64_t* bytes)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    if (nt) *nt = ctx->nTris;
    if (nn) *nn = ctx->nNodes;
    if (nl) *nl = ctx->nLights;
    if (bytes)
    {
        const DevBuf* all[] = {&ctx->dTris, &ctx->dNodes, &ctx->dInst, &ctx->dMat, &ctx->dLights, &ctx->dPos, &ctx->dNrm,
                               &ctx->dTan, &ctx->dUV, &ctx->dIdx, &ctx->dSpec};
        uint64_t s = 0;
        for (const DevBuf* b : all) s += b->bytes;
        *bytes = s;
    }
    return YG_OK;
}

YG_API int yg_film_clear(yg_context* ctx, uint32_t w, uint32_t h)
{
    if (!ctx || w == 0 || h == 0) return fail(YG_ERR_INVALID_ARGUMENT, "film: bad size");
    std::lock_guard<std::mutex> g(ctx->lock);
    cudaSetDevice(ctx->device);
    size_t bytes = (size_t)w * h * sizeof(float4);
    YG_CUDA(ctx->dFilmSum.ensure(bytes));
    YG_CUDA(ctx->dFilmComp.ensure(bytes));
    YG_CUDA(ctx->dAccA.ensure(bytes));
    YG_CUDA(ctx->dAccN.ensure(bytes));
    YG_CUDA(cudaMemsetAsync(ctx->dFilmSum.p, 0, bytes, ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->dFilmComp.p, 0, bytes, ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->dAccA.p, 0, bytes, ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->dAccN.p, 0, bytes, ctx->stream));
    ctx->filmW = w;
    ctx->filmH = h;
    ctx->atrousState = 0;
    return YG_OK;
}

YG_API int yg_render(yg_context* ctx, const yg_render_params* p, yg_sample_record* dump)
{
    if (!ctx || !p) return fail(YG_ERR_INVALID_ARGUMENT, "render: null argument");
    static const char* const kRangeNames[3] = {"yg_render uni", "yg_render nee", "yg_render bdpt"};
    yg::NvtxRange range(kRangeNames[p->integrator <= YG_INTEGRATOR_BDPT ? p->integrator : 0]);
    std::lock_guard<std::mutex> g(ctx->lock);
    if (!ctx->sceneBuilt) return fail(YG_ERR_NOT_READY, "render: call yg_build_scene first");
    if (!ctx->cameraSet) return fail(YG_ERR_NOT_READY, "render: camera not set");
    if (p->integrator > YG_INTEGRATOR_BDPT) return fail(YG_ERR_INVALID_ARGUMENT, "render: unknown integrator");
    if (p->width == 0 || p->height == 0 || p->spp_count == 0) return fail(YG_ERR_INVALID_ARGUMENT, "render: empty request");
    uint32_t cx = p->crop_x, cy = p->crop_y, cw = p->crop_w, ch = p->crop_h;
    if (cw == 0 || ch == 0)
    {
        cx = cy = 0;
        cw = p->width;
        ch = p->height;
    }
    if ((uint64_t)cx + cw > p->width || (uint64_t)cy + ch > p->height) return fail(YG_ERR_INVALID_ARGUMENT, "render: crop outside image");
    bool film = (p->flags & YG_FLAG_NO_FILM) == 0;
    if (film && (ctx->filmW != p->width || ctx->filmH != p->height))
        return fail(YG_ERR_NOT_READY, "render: film size differs, call yg_film_clear");
    float lminf = p->lambda_min, lmaxf = p->lambda_max;
    if (lminf == 0.0f && lmaxf == 0.0f)
    {
        lminf = 380.f;
        lmaxf = 700.f;
    }
    int lmin = (int)lminf, lmax = (int)lmaxf;
    if ((float)lmin != lminf || (float)lmax != lmaxf) return fail(YG_ERR_INVALID_ARGUMENT, "render: spectral range must be whole nm");
    cudaSetDevice(ctx->device);
    int r = ensureCie(ctx, lmin, lmax);
    if (r) return r;
    bool needRgb = sceneNeedsRgbLut(ctx, p->env_intensity_scale);
    if (needRgb && (r = ensureRgbLut(ctx, lmin, lmax))) return r;
    if ((r = checkMaterialTextures(ctx, "render"))) return r;

    const uint64_t npix = (uint64_t)cw * ch;
    const bool bdpt = p->integrator == YG_INTEGRATOR_BDPT;
    const uint64_t maxSamplesPerChunk = bdpt ? (1ull << 24) : (1ull << 26);
    uint32_t chunkSpp = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(p->spp_count, maxSamplesPerChunk / npix));
    if (bdpt && (p->flags & YG_FLAG_MEGAKERNEL)) return fail(YG_ERR_INVALID_ARGUMENT, "render: BDPT has no megakernel variant");
    const uint32_t lightVerts = p->bdpt_light_vertices ? p->bdpt_light_vertices : yg::kBdptMaxLightVertices;
    if (bdpt && (lightVerts < 2 || lightVerts > yg::kBdptMaxLightVertices))
        return fail(YG_ERR_INVALID_ARGUMENT, "render: bdpt_light_vertices must be 2..16");
    const uint32_t lightPaths = p->bdpt_light_paths ? p->bdpt_light_paths : ((cw + 7) / 8) * ((ch + 7) / 8);
    if (bdpt)
    {
        YG_CUDA(ctx->dArena.ensure(yg::bdptArenaBytes(chunkSpp, lightPaths, lightVerts, npix)));
        if (ctx->permW != cw || ctx->permH != ch)
        {
            std::vector<uint32_t> perm;
            pixelPermutation(cw, ch, perm);
            if ((r = upload(ctx, ctx->dPerm, perm.data(), perm.size()))) return r;
            ctx->permW = cw;
            ctx->permH = ch;
        }
    }
    bool feats = (p->flags & YG_FLAG_FEATURES) != 0;
    const bool atrous = (p->flags & YG_FLAG_ATROUS_FEATURES) != 0;
    if (atrous && !film) return fail(YG_ERR_INVALID_ARGUMENT, "render: YG_FLAG_ATROUS_FEATURES needs the film");
    if (film)
    {
        const size_t plane = (size_t)p->width * p->height;
        if (atrous)
        {
            YG_CUDA(ctx->dAtrousMom.ensure(4 * plane * sizeof(float4)));
            YG_CUDA(ctx->dAtrousOdd.ensure(plane * sizeof(float4)));
            if (ctx->atrousState == 0)
            {
                YG_CUDA(cudaMemsetAsync(ctx->dAtrousMom.p, 0, 4 * plane * sizeof(float4), ctx->stream));
                YG_CUDA(cudaMemsetAsync(ctx->dAtrousOdd.p, 0, plane * sizeof(float4), ctx->stream));
            }
        }
        const int st = atrous ? 1 : 2;
        ctx->atrousState = (ctx->atrousState == 0 || ctx->atrousState == st) ? st : 3;
    }
    YG_CUDA(ctx->dSamples.ensure(npix * chunkSpp * sizeof(float4)));
    if (feats)
    {
        YG_CUDA(ctx->dFeatA.ensure(npix * chunkSpp * sizeof(float4)));
        YG_CUDA(ctx->dFeatN.ensure(npix * chunkSpp * sizeof(float4)));
    }
    if (dump) YG_CUDA(ctx->dDump.ensure(npix * chunkSpp * 8 * sizeof(float)));
    const bool mega = (p->flags & YG_FLAG_MEGAKERNEL) != 0;
    uint32_t waveCap = (uint32_t)std::min<uint64_t>(npix * chunkSpp, 1ull << YG_WAVE_CAPACITY_LOG2);
    if (!mega && !bdpt) YG_CUDA(ctx->dArena.ensure(waveCap * yg::wavefrontBytesPerSlot() + (64u << 10)));
    const size_t counterBytes = 8 * (1 + yg::kTraversalCounters);
    YG_CUDA(ctx->dRayCount.ensure(counterBytes));
    YG_CUDA(cudaMemsetAsync(ctx->dRayCount.p, 0, counterBytes, ctx->stream));
    yg::KernelTimer timer{nullptr, nullptr, 0, 0};
    const bool timeKernels = (p->flags & YG_FLAG_TIME_KERNELS) != 0 && !mega;
    if (timeKernels)
    {
        // events for every timed launch of the render: 4 kinds per bounce, per wave (BDPT: 5
        // kinds per bounce of waves sized by the BDPT arena, bounded here by 8192 launches)
        uint64_t waves = (npix * (uint64_t)p->spp_count + waveCap - 1) / waveCap;
        size_t want = bdpt ? (size_t)1 << 13 : (size_t)std::min<uint64_t>(waves * p->max_depth * 4, 1u << 14);
        while (ctx->kernelKinds.size() < want)
        {
            cudaEvent_t a = nullptr, b = nullptr;
            YG_CUDA(cudaEventCreate(&a));
            YG_CUDA(cudaEventCreate(&b));
            ctx->kernelEvents.push_back(a);
            ctx->kernelEvents.push_back(b);
            ctx->kernelKinds.push_back(0);
        }
        timer = yg::KernelTimer{ctx->kernelEvents.data(), ctx->kernelKinds.data(), (uint32_t)ctx->kernelKinds.size(), 0};
    }
    ctx->kernelTimed = 0;
    // Sobol points of every sample index of the request (RaytraceCommonResources.cpp:623-627),
    // generated on the device from the generator matrices
    if (!ctx->dSobolMat.p)
        if ((r = upload(ctx, ctx->dSobolMat, ctx->sobolMatrices.data(), ctx->sobolMatrices.size()))) return r;
    YG_CUDA(ctx->dSobol.ensure((size_t)p->spp_count * yg::kSobolDims * 4));
    yg::launchSobolPoints(ctx->dSobolMat.as<uint32_t>(), p->spp_start, p->spp_count, ctx->dSobol.as<uint32_t>(), ctx->smCount,
                          ctx->stream);

    yg::SceneView S;
    fillSceneView(ctx, lminf, lmaxf, needRgb, S);

    yg::LaunchParams L{};
    L.integrator = p->integrator;
    L.width = p->width;
    L.height = p->height;
    L.cropX = cx;
    L.cropY = cy;
    L.cropW = cw;
    L.cropH = ch;
    L.maxDepth = p->max_depth;
    L.regularizeAfter = p->regularize_after_vertices;
    L.regularizeEnable = p->regularize_enable;
    L.envScale = p->env_intensity_scale;
    L.seed = p->seed;
    L.flags = p->flags;
    L.rayCounter = ctx->dRayCount.as<unsigned long long>();
    L.traversalCounter = (p->flags & YG_FLAG_COUNT_TRAVERSAL) ? ctx->dRayCount.as<unsigned long long>() + 1 : nullptr;

    uint32_t launches = 0;
    YG_CUDA(cudaEventRecord(ctx->evStart, ctx->stream));
    for (uint32_t s0 = 0; s0 < p->spp_count; s0 += chunkSpp)
    {
        uint32_t ns = std::min(chunkSpp, p->spp_count - s0);
        S.sobol = ctx->dSobol.as<uint32_t>() + (size_t)s0 * yg::kSobolDims;
        L.sppStart = p->spp_start + s0;
        L.sppCount = ns;
        L.nSamples = npix * ns;
        L.sampleXYZ = ctx->dSamples.as<float4>();
        L.dump = dump ? ctx->dDump.as<float>() : nullptr;
        L.featAlbedo = feats ? ctx->dFeatA.as<float4>() : nullptr;
        L.featNormalDepth = feats ? ctx->dFeatN.as<float4>() : nullptr;
        if (bdpt)
            launches += yg::launchBdpt(S, L, ctx->dArena.p, ctx->dPerm.as<uint32_t>(), lightPaths, lightVerts,
                                       yg::mk3(ctx->worldCenter[0], ctx->worldCenter[1], ctx->worldCenter[2]),
                                       ctx->worldRadiusSqr, ctx->smCount, ctx->stream, timeKernels ? &timer : nullptr);
        else if (mega) launches += yg::launchPathKernel(S, L, ctx->smCount, ctx->stream);
        else launches += yg::launchWavefront(S, L, ctx->dArena.p, waveCap, ctx->smCount, ctx->stream,
                                             timeKernels ? &timer : nullptr);
        if (film)
            launches += yg::launchFilm(ctx->dFilmSum.as<float4>(), ctx->dFilmComp.as<float4>(), L.sampleXYZ, p->width, cx,
                                       cy, cw, ch, ns, ctx->smCount, ctx->stream);
        if (film && atrous)
            launches += yg::launchAtrousGather(S, L, ctx->dAtrousMom.as<float4>(), ctx->dAtrousOdd.as<float4>(), L.sampleXYZ, ns,
                                               ctx->smCount, ctx->stream);
        if (film && feats)
            launches += yg::launchFeatures(ctx->dAccA.as<float4>(), ctx->dAccN.as<float4>(), L.featAlbedo, L.featNormalDepth,
                                           p->width, cx, cy, cw, ch, ns, ctx->smCount, ctx->stream);
        if (dump)
        {
            YG_CUDA(cudaMemcpyAsync(dump + (size_t)s0 * npix, ctx->dDump.p, npix * ns * 8 * sizeof(float),
                                    cudaMemcpyDeviceToHost, ctx->stream));
        }
    }
    YG_CUDA(cudaGetLastError());
    YG_CUDA(cudaEventRecord(ctx->evStop, ctx->stream));
    ctx->lastLaunches = launches;
    ctx->kernelTimed = timer.used;
    if (dump)
    {
        YG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
    return YG_OK;
}

YG_API int yg_last_render_stats(yg_context* ctx, float* ms, uint64_t* rays, uint32_t* launches)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    YG_CUDA(cudaEventSynchronize(ctx->evStop));
    float t = 0;
    YG_CUDA(cudaEventElapsedTime(&t, ctx->evStart, ctx->evStop));
    unsigned long long rc = 0;
    if (ctx->dRayCount.p) YG_CUDA(cudaMemcpy(&rc, ctx->dRayCount.p, 8, cudaMemcpyDeviceToHost));
    if (ms) *ms = t;
    if (rays) *rays = rc;
    if (launches) *launches = ctx->lastLaunches;
    return YG_OK;
}

YG_API int yg_last_traversal_counts(yg_context* ctx, uint64_t* nodes, uint64_t* tris)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "null context");
    unsigned long long c[1 + yg::kTraversalCounters] = {};
    if (ctx->dRayCount.p)
    {
        YG_CUDA(cudaStreamSynchronize(ctx->stream));
        YG_CUDA(cudaMemcpy(c, ctx->dRayCount.p, sizeof(c), cudaMemcpyDeviceToHost));
    }
    if (nodes) *nodes = c[1] + c[3];
    if (tris) *tris = c[2] + c[4];
    return YG_OK;
}

static_assert(YG_KERNEL_TRACE == yg::kKernelTrace && YG_KERNEL_REGROUP == yg::kKernelRegroup &&
                  YG_KERNEL_SHADE == yg::kKernelShade && YG_KERNEL_SHADOW == yg::kKernelShadow,
              "kernel kinds");

YG_API int yg_last_kernel_profile(yg_context* ctx, yg_kernel_profile* out)
{
    if (!ctx || !out) return fail(YG_ERR_INVALID_ARGUMENT, "kernel profile: null argument");
    std::memset(out, 0, sizeof(*out));
    YG_CUDA(cudaEventSynchronize(ctx->evStop));
    for (uint32_t k = 0; k < ctx->kernelTimed; ++k)
    {
        float t = 0;
        YG_CUDA(cudaEventElapsedTime(&t, ctx->kernelEvents[2 * k], ctx->kernelEvents[2 * k + 1]));
        uint8_t kind = ctx->kernelKinds[k];
        if (kind == yg::kKernelConnect)
        {
            out->connect_ms += t;
            out->connect_launches += 1;
            continue;
        }
        out->ms[kind] += t;
        out->launches[kind] += 1;
    }
    out->connection_record_bytes = yg::bdptConnectionRecordBytes();
    unsigned long long c[1 + yg::kTraversalCounters] = {};
    if (ctx->dRayCount.p) YG_CUDA(cudaMemcpy(c, ctx->dRayCount.p, sizeof(c), cudaMemcpyDeviceToHost));
    out->closest_nodes = c[1];
    out->closest_triangles = c[2];
    out->shadow_nodes = c[3];
    out->shadow_triangles = c[4];
    out->closest_rays = c[5];
    out->shadow_rays = c[6];
    return YG_OK;
}

YG_API int yg_film_read(yg_context* ctx, float* xyz, float* counts)
{
    if (!ctx || !xyz) return fail(YG_ERR_INVALID_ARGUMENT, "film: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    std::vector<float4> s(n);
    YG_CUDA(cudaMemcpyAsync(s.data(), ctx->dFilmSum.p, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < n; ++i)
    {
        float c = s[i].w;
        float inv = c > 0.0f ? 1.0f / c : 0.0f;
        xyz[3 * i] = s[i].x * inv;
        xyz[3 * i + 1] = s[i].y * inv;
        xyz[3 * i + 2] = s[i].z * inv;
        if (counts) counts[i] = c;
    }
    return YG_OK;
}

namespace
{
// film checkpoint layout: header, then the planes (float4 per pixel) in this order
struct FilmStateHeader
{
    uint64_t magic;
    uint32_t version, width, height, atrousState, atrousPlanes, reserved;
};
constexpr uint64_t kFilmMagic = 0x4D4C4946475930ull; // "0YGFILM"
constexpr uint32_t kFilmPlanes = 4;                  // sums, compensation, albedo and normal accumulators
uint32_t atrousPlanesOf(const yg_context* c)
{
    const size_t plane = (size_t)c->filmW * c->filmH * sizeof(float4);
    // the moments exist once an a-trous render has gathered into this film (states 1 and 3)
    return ((c->atrousState & 1) != 0 && c->dAtrousMom.bytes >= 4 * plane && c->dAtrousOdd.bytes >= plane) ? 5u : 0u;
}
size_t filmStateBytes(const yg_context* c)
{
    return sizeof(FilmStateHeader) + (size_t)(kFilmPlanes + atrousPlanesOf(c)) * c->filmW * c->filmH * sizeof(float4);
}
} // namespace

YG_API int yg_debug_bounds_errors(yg_context* ctx, uint32_t* count)
{
    if (!ctx || !count) return fail(YG_ERR_INVALID_ARGUMENT, "bounds errors: null argument");
#ifndef YG_DEBUG_BOUNDS
    return fail(YG_ERR_NOT_READY, "bounds errors: the library was built without YG_DEBUG_BOUNDS");
#else
    std::lock_guard<std::mutex> g(ctx->lock);
    *count = 0;
    if (!ctx->dBoundsErr.p) return YG_OK;
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    YG_CUDA(cudaMemcpy(count, ctx->dBoundsErr.p, 4, cudaMemcpyDeviceToHost));
    return YG_OK;
#endif
}

YG_API int yg_film_state_size(yg_context* ctx, size_t* bytes)
{
    if (!ctx || !bytes) return fail(YG_ERR_INVALID_ARGUMENT, "film state: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (ctx->filmW == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    *bytes = filmStateBytes(ctx);
    return YG_OK;
}

YG_API int yg_film_save(yg_context* ctx, void* host, size_t bytes)
{
    if (!ctx || !host) return fail(YG_ERR_INVALID_ARGUMENT, "film save: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (ctx->filmW == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    if (bytes < filmStateBytes(ctx)) return fail(YG_ERR_INVALID_ARGUMENT, "film save: buffer smaller than yg_film_state_size");
    YG_CUDA(cudaSetDevice(ctx->device));
    FilmStateHeader h{kFilmMagic, 1u, ctx->filmW, ctx->filmH, (uint32_t)ctx->atrousState, atrousPlanesOf(ctx), 0u};
    std::memcpy(host, &h, sizeof(h));
    char* dst = static_cast<char*>(host) + sizeof(h);
    const size_t plane = (size_t)ctx->filmW * ctx->filmH * sizeof(float4);
    const DevBuf* planes[4] = {&ctx->dFilmSum, &ctx->dFilmComp, &ctx->dAccA, &ctx->dAccN};
    for (const DevBuf* b : planes)
    {
        YG_CUDA(cudaMemcpyAsync(dst, b->p, plane, cudaMemcpyDeviceToHost, ctx->stream));
        dst += plane;
    }
    if (h.atrousPlanes)
    {
        YG_CUDA(cudaMemcpyAsync(dst, ctx->dAtrousMom.p, 4 * plane, cudaMemcpyDeviceToHost, ctx->stream));
        YG_CUDA(cudaMemcpyAsync(dst + 4 * plane, ctx->dAtrousOdd.p, plane, cudaMemcpyDeviceToHost, ctx->stream));
    }
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API int yg_film_restore(yg_context* ctx, const void* host, size_t bytes)
{
    if (!ctx || !host) return fail(YG_ERR_INVALID_ARGUMENT, "film restore: null argument");
    if (bytes < sizeof(FilmStateHeader)) return fail(YG_ERR_INVALID_ARGUMENT, "film restore: not a film state");
    FilmStateHeader h;
    std::memcpy(&h, host, sizeof(h));
    if (h.magic != kFilmMagic || h.version != 1u || h.width == 0 || h.height == 0 || (h.atrousPlanes != 0 && h.atrousPlanes != 5) ||
        h.atrousState > 3)
        return fail(YG_ERR_INVALID_ARGUMENT, "film restore: not a film state");
    // a corrupt header must not wrap the size arithmetic below (9 planes at most)
    if ((size_t)h.width * h.height > (SIZE_MAX - sizeof(h)) / (9 * sizeof(float4)))
        return fail(YG_ERR_INVALID_ARGUMENT, "film restore: film size out of range");
    const size_t plane = (size_t)h.width * h.height * sizeof(float4);
    if (bytes < sizeof(h) + (kFilmPlanes + h.atrousPlanes) * plane)
        return fail(YG_ERR_INVALID_ARGUMENT, "film restore: buffer shorter than its state");
    int r = yg_film_clear(ctx, h.width, h.height);
    if (r) return r;
    std::lock_guard<std::mutex> g(ctx->lock);
    YG_CUDA(cudaSetDevice(ctx->device));
    const char* src = static_cast<const char*>(host) + sizeof(h);
    DevBuf* planes[4] = {&ctx->dFilmSum, &ctx->dFilmComp, &ctx->dAccA, &ctx->dAccN};
    for (DevBuf* b : planes)
    {
        YG_CUDA(cudaMemcpyAsync(b->p, src, plane, cudaMemcpyHostToDevice, ctx->stream));
        src += plane;
    }
    if (h.atrousPlanes)
    {
        YG_CUDA(ctx->dAtrousMom.ensure(4 * plane));
        YG_CUDA(ctx->dAtrousOdd.ensure(plane));
        YG_CUDA(cudaMemcpyAsync(ctx->dAtrousMom.p, src, 4 * plane, cudaMemcpyHostToDevice, ctx->stream));
        YG_CUDA(cudaMemcpyAsync(ctx->dAtrousOdd.p, src + 4 * plane, plane, cudaMemcpyHostToDevice, ctx->stream));
    }
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->atrousState = (int)h.atrousState;
    return YG_OK;
}

YG_API int yg_film_resolve_device(yg_context* ctx, float* xyz, float* albedo, float* normal, float* depth)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "film resolve: null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    if ((albedo || normal || depth) && !ctx->dAccA.p)
        return fail(YG_ERR_NOT_READY, "film resolve: no feature accumulators");
    yg::launchFilmResolve(ctx->dFilmSum.as<float4>(), ctx->dAccA.as<float4>(), ctx->dAccN.as<float4>(), n, xyz, albedo, normal,
                          depth, ctx->smCount, ctx->stream);
    YG_CUDA(cudaGetLastError());
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API void yg_atrous_default_params(yg_atrous_params* p)
{
    if (!p) return;
    p->depth_sigma_scale = 0.02f;
    p->normal_sigma = 0.06f;
    p->material_sigma = 0.05f;
    p->color_sigma = 3.0f;
    p->feature_variance_scale = 1.0f;
    p->prefilter = 1;
    p->passes = 5;
    p->reserved = 0;
}

extern "C++"
{
namespace
{
int atrousSettings(const yg_atrous_params* p, yg::AtrousSettings& A)
{
    if (!p) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: null parameters");
    const float v[5] = {p->depth_sigma_scale, p->normal_sigma, p->material_sigma, p->color_sigma, p->feature_variance_scale};
    for (int i = 0; i < 5; ++i)
        if (!(v[i] >= 0.0f) || !std::isfinite(v[i])) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: sigmas must be finite and >= 0");
    if (p->passes > 12) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: at most 12 passes");
    A = yg::AtrousSettings{p->depth_sigma_scale, p->normal_sigma, p->material_sigma, p->color_sigma, p->feature_variance_scale,
                           p->prefilter ? 1u : 0u, p->passes};
    return YG_OK;
}

void atrousCamera(const float* uvToView, const float* viewToWorld, uint32_t w, uint32_t h, yg::AtrousBuffers& B)
{
    B.width = w;
    B.height = h;
    B.invW = 1.0f / (float)w;
    B.invH = 1.0f / (float)h;
    std::memcpy(B.uvToView, uvToView, sizeof(B.uvToView));
    std::memcpy(B.viewToWorld, viewToWorld, sizeof(B.viewToWorld));
}
} // namespace
}

YG_API int yg_atrous_denoise(yg_context* ctx, const yg_atrous_params* params, float* out_xyzw, float* out_variance)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: null context");
    yg::AtrousSettings A;
    int r = atrousSettings(params, A);
    if (r) return r;
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "a-trous: film not allocated");
    if (ctx->atrousState != 1)
        return fail(YG_ERR_NOT_READY, "a-trous: every film render since yg_film_clear needs YG_FLAG_ATROUS_FEATURES");
    if (!ctx->cameraSet) return fail(YG_ERR_NOT_READY, "a-trous: camera not set");
    cudaSetDevice(ctx->device);
    // planes: colour and variance ping-pong [0], [1] and the kept output [2]
    YG_CUDA(ctx->dAtrousFeat.ensure(2 * n * sizeof(uint4)));
    YG_CUDA(ctx->dAtrousCol.ensure(3 * n * sizeof(float4)));
    YG_CUDA(ctx->dAtrousVar.ensure(3 * n * sizeof(float)));
    yg::AtrousBuffers B;
    atrousCamera(ctx->camera.uvToView, ctx->camera.viewToWorld, ctx->filmW, ctx->filmH, B);
    B.film = ctx->dFilmSum.as<float4>();
    B.odd = ctx->dAtrousOdd.as<float4>();
    B.moments = ctx->dAtrousMom.as<float4>();
    B.feat0 = ctx->dAtrousFeat.as<uint4>();
    B.feat1 = B.feat0 + n;
    B.colour[0] = ctx->dAtrousCol.as<float4>();
    B.colour[1] = B.colour[0] + n;
    B.variance[0] = ctx->dAtrousVar.as<float>();
    B.variance[1] = B.variance[0] + n;
    float4* oc = out_xyzw ? reinterpret_cast<float4*>(out_xyzw) : B.colour[0] + 2 * n;
    float* ov = out_variance ? out_variance : B.variance[0] + 2 * n;
    yg::launchAtrous(B, A, oc, ov, ctx->stream);
    YG_CUDA(cudaGetLastError());
    if (out_xyzw && !out_variance)
    {
        // keep the context's copy complete for yg_atrous_read
        YG_CUDA(cudaMemcpyAsync(B.colour[0] + 2 * n, oc, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    else if (out_xyzw)
    {
        YG_CUDA(cudaMemcpyAsync(B.colour[0] + 2 * n, oc, n * sizeof(float4), cudaMemcpyDeviceToDevice, ctx->stream));
        YG_CUDA(cudaMemcpyAsync(B.variance[0] + 2 * n, ov, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    else if (out_variance)
    {
        YG_CUDA(cudaMemcpyAsync(B.variance[0] + 2 * n, ov, n * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    }
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API void yg_tonemap_default_params(yg_tonemap_params* p)
{
    if (!p) return;
    p->enable = 1;
    p->auto_exposure = 1;
    p->manual_exposure = 1.0f;
    p->exposure_compensation = 0.0f;
    p->eye_adaptation_speed = 1.0f;
    p->delta_time = 0.0f;
    p->reset = 0;
    p->source = 0;
}

YG_API int yg_tonemap(yg_context* ctx, const yg_tonemap_params* p, uint8_t* rgba8, float* exposure)
{
    if (!ctx || !p || !rgba8) return fail(YG_ERR_INVALID_ARGUMENT, "tonemap: null argument");
    if (!std::isfinite(p->manual_exposure) || !std::isfinite(p->exposure_compensation) || !std::isfinite(p->delta_time) ||
        !std::isfinite(p->eye_adaptation_speed) || p->delta_time < 0.0f || p->eye_adaptation_speed < 0.0f)
        return fail(YG_ERR_INVALID_ARGUMENT, "tonemap: non-finite or negative parameter");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "tonemap: film not allocated");
    if (p->source == 1 && ctx->dAtrousCol.bytes < 3 * n * sizeof(float4))
        return fail(YG_ERR_NOT_READY, "tonemap: no a-trous output (call yg_atrous_denoise first)");
    cudaSetDevice(ctx->device);
    const bool fresh = ctx->dDisplay.p == nullptr;
    YG_CUDA(ctx->dDisplay.ensure(128 * sizeof(uint32_t) + 4 * sizeof(float)));
    YG_CUDA(ctx->dDisplayOut.ensure(n * sizeof(uint32_t)));
    yg::DisplayArgs A{};
    A.width = ctx->filmW;
    A.height = ctx->filmH;
    A.film = ctx->dFilmSum.as<float4>();
    A.atrous = p->source == 1 ? ctx->dAtrousCol.as<float4>() + 2 * n : nullptr;
    A.histogram = ctx->dDisplay.as<uint32_t>();
    A.exposure = reinterpret_cast<float*>(A.histogram + 128);
    A.stats = A.exposure + 1;
    A.out = ctx->dDisplayOut.as<uint32_t>();
    A.tonemap = p->enable ? 1u : 0u;
    A.autoExposure = p->auto_exposure ? 1u : 0u;
    A.init = (p->reset || fresh) ? 1u : 0u;
    A.exposureParam = p->auto_exposure ? p->exposure_compensation : p->manual_exposure;
    A.deltaTime = p->delta_time;
    A.adaptSpeed = p->eye_adaptation_speed;
    yg::launchDisplay(A, ctx->smCount, ctx->stream);
    YG_CUDA(cudaGetLastError());
    YG_CUDA(cudaMemcpyAsync(rgba8, A.out, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (exposure) YG_CUDA(cudaMemcpyAsync(exposure, A.exposure, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API int yg_atrous_read(yg_context* ctx, float* xyzw, float* variance, float* film_sum, float* odd_sum, float* moments,
                          uint32_t* features)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous read: null context");
    std::lock_guard<std::mutex> g(ctx->lock);
    const size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "a-trous read: film not allocated");
    if ((moments || odd_sum) && ctx->atrousState != 1)
        return fail(YG_ERR_NOT_READY, "a-trous read: no complete gather since yg_film_clear");
    if ((xyzw || variance || features) && ctx->dAtrousCol.bytes < 3 * n * sizeof(float4))
        return fail(YG_ERR_NOT_READY, "a-trous read: call yg_atrous_denoise first");
    cudaSetDevice(ctx->device);
    auto d2h = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    };
    if (xyzw) YG_CUDA(d2h(xyzw, ctx->dAtrousCol.as<float4>() + 2 * n, n * sizeof(float4)));
    if (variance) YG_CUDA(d2h(variance, ctx->dAtrousVar.as<float>() + 2 * n, n * sizeof(float)));
    if (film_sum) YG_CUDA(d2h(film_sum, ctx->dFilmSum.p, n * sizeof(float4)));
    if (moments) YG_CUDA(d2h(moments, ctx->dAtrousMom.p, 4 * n * sizeof(float4)));
    if (odd_sum) YG_CUDA(d2h(odd_sum, ctx->dAtrousOdd.p, n * sizeof(float4)));
    if (features) YG_CUDA(d2h(features, ctx->dAtrousFeat.p, 2 * n * sizeof(uint4)));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    return YG_OK;
}

YG_API int yg_atrous_run(uint32_t width, uint32_t height, const float* film_sum, const float* odd_sum, const float* moments,
                         const yg_camera* camera, const yg_atrous_params* params, float* out_xyzw, float* out_variance,
                         uint32_t* features_out)
{
    if (!film_sum || !odd_sum || !moments || !camera || !out_xyzw || !out_variance)
        return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: null argument");
    if (width == 0 || height == 0) return fail(YG_ERR_INVALID_ARGUMENT, "a-trous: empty image");
    yg::AtrousSettings A;
    int r = atrousSettings(params, A);
    if (r) return r;
    const size_t n = (size_t)width * height;
    yg::AtrousBuffers B;
    atrousCamera(camera->uv_to_view, camera->view_to_world, width, height, B);
    // device layout: film, odd, 4 moment planes, 3 colour planes (float4); 2 feature planes
    // (uint4); 3 variance planes (float)
    const size_t f4 = n * sizeof(float4);
    void* mem = nullptr;
    YG_CUDA(cudaMalloc(&mem, 9 * f4 + 2 * n * sizeof(uint4) + 3 * n * sizeof(float)));
    float4* base = static_cast<float4*>(mem);
    cudaError_t e = cudaMemcpy(base, film_sum, f4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(base + n, odd_sum, f4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(base + 2 * n, moments, 4 * f4, cudaMemcpyHostToDevice);
    B.film = base;
    B.odd = base + n;
    B.moments = base + 2 * n;
    B.colour[0] = base + 6 * n;
    B.colour[1] = base + 7 * n;
    float4* oc = base + 8 * n;
    B.feat0 = reinterpret_cast<uint4*>(base + 9 * n);
    B.feat1 = B.feat0 + n;
    B.variance[0] = reinterpret_cast<float*>(B.feat1 + n);
    B.variance[1] = B.variance[0] + n;
    float* ov = B.variance[1] + n;
    if (e == cudaSuccess)
    {
        yg::launchAtrous(B, A, oc, ov, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out_xyzw, oc, f4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(out_variance, ov, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && features_out) e = cudaMemcpy(features_out, B.feat0, 2 * n * sizeof(uint4), cudaMemcpyDeviceToHost);
    cudaFree(mem);
    if (e != cudaSuccess) return fail(YG_ERR_CUDA, std::string("a-trous: ") + cudaGetErrorString(e));
    return YG_OK;
}

YG_API int yg_features_read(yg_context* ctx, float* albedo, float* normal, float* depth)
{
    if (!ctx) return fail(YG_ERR_INVALID_ARGUMENT, "features: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    std::vector<float4> a(n), nd(n), s(n);
    YG_CUDA(cudaMemcpyAsync(a.data(), ctx->dAccA.p, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaMemcpyAsync(nd.data(), ctx->dAccN.p, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaMemcpyAsync(s.data(), ctx->dFilmSum.p, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    for (size_t i = 0; i < n; ++i)
    {
        float c = s[i].w > 0.f ? 1.0f / s[i].w : 0.f;
        if (albedo)
        {
            albedo[3 * i] = a[i].x * c;
            albedo[3 * i + 1] = a[i].y * c;
            albedo[3 * i + 2] = a[i].z * c;
        }
        if (normal)
        {
            normal[3 * i] = nd[i].x * c;
            normal[3 * i + 1] = nd[i].y * c;
            normal[3 * i + 2] = nd[i].z * c;
        }
        if (depth) depth[i] = nd[i].w * c;
    }
    return YG_OK;
}

YG_API int yg_film_relmse(yg_context* ctx, const float* ref, double eps, double* out)
{
    if (!ctx || !ref || !out) return fail(YG_ERR_INVALID_ARGUMENT, "relmse: null argument");
    std::lock_guard<std::mutex> g(ctx->lock);
    size_t n = (size_t)ctx->filmW * ctx->filmH;
    if (n == 0) return fail(YG_ERR_NOT_READY, "film: not allocated");
    YG_CUDA(ctx->dRef.ensure(n * 3 * sizeof(float)));
    YG_CUDA(ctx->dRelmse.ensure(sizeof(double)));
    YG_CUDA(cudaMemcpyAsync(ctx->dRef.p, ref, n * 3 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->dRelmse.p, 0, sizeof(double), ctx->stream));
    yg::launchRelmse(ctx->dFilmSum.as<float4>(), ctx->dRef.as<float>(), (uint32_t)n, eps, ctx->dRelmse.as<double>(),
                     ctx->smCount, ctx->stream);
    double s = 0;
    YG_CUDA(cudaMemcpyAsync(&s, ctx->dRelmse.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    *out = s / (3.0 * (double)n);
    return YG_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------
// Render entry point that allocates nothing.
//
// Some callers cannot allocate device memory while rendering: a serving process whose
// admission controller reserves the device budget up front, or a host application that
// must not hit cudaMalloc's implicit device synchronisation in the middle of a frame.
// yg_render_samples_noalloc renders with the wavefront kernels like yg_render, but its
// scratch (path-state arena, Sobol points, generator matrices) is the file-scope device
// array below, kNoAllocScratchBytes = 256 KB of Sobol points + 32 KB of generator matrices
// + 16384 paths x 416 B + 64 KB of slack, about 7 MB, that every GPU loading this library
// holds until exit. The caller passes the scene (already built in the context) and the
// output buffer.
namespace
{
constexpr uint32_t kNoAllocWaveCapacity = 16384; // paths in flight per wave
constexpr uint32_t kNoAllocMaxSpp = 256;         // sample indices per call
constexpr size_t kNoAllocBytesPerSlot = 416;     // >= wavefrontBytesPerSlot(), checked at set-up
constexpr size_t kNoAllocSobolBytes = (size_t)kNoAllocMaxSpp * yg::kSobolDims * sizeof(uint32_t);
constexpr size_t kNoAllocMatrixBytes = (size_t)yg::kSobolDims * 32 * sizeof(uint32_t);
constexpr size_t kNoAllocArenaBytes = (size_t)kNoAllocWaveCapacity * kNoAllocBytesPerSlot + (64u << 10);
constexpr size_t kNoAllocScratchBytes = kNoAllocSobolBytes + kNoAllocMatrixBytes + kNoAllocArenaBytes;

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

std::mutex g_noallocMutex;
void* g_noallocDevicePtr[256] = {};

// Device address of the scratch array on `device` (which must be current). The host
// symbol is only a stand-in, so the address is looked up once per device and cached. The
// same one-time set-up copies the Sobol generator matrices (a constant table, identical in
// every context) into their part of the array with a synchronous copy; later calls only
// launch kernels.
int noallocScratchAddress(int device, const std::vector<uint32_t>& sobolMatrices, void** out)
{
    if (device < 0 || device >= 256) return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: device ordinal out of range");
    if (yg::wavefrontBytesPerSlot() > kNoAllocBytesPerSlot)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: scratch layout is smaller than the wavefront state");
    if (sobolMatrices.size() * sizeof(uint32_t) != kNoAllocMatrixBytes)
        return fail(YG_ERR_NOT_READY, "no-alloc render: Sobol generator matrices are not loaded");
    std::lock_guard<std::mutex> g(g_noallocMutex);
    if (!g_noallocDevicePtr[device])
    {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess || !p)
            return fail(YG_ERR_CUDA, std::string("no-alloc render: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        e = cudaMemcpy(static_cast<char*>(p) + kNoAllocSobolBytes, sobolMatrices.data(), kNoAllocMatrixBytes,
                       cudaMemcpyHostToDevice);
        if (e != cudaSuccess)
            return fail(YG_ERR_CUDA, std::string("no-alloc render: generator matrix upload: ") + cudaGetErrorString(e));
        g_noallocDevicePtr[device] = p;
    }
    *out = g_noallocDevicePtr[device];
    return YG_OK;
}

// Sobol points for sample indices [start, start + count), all 256 dimensions
__global__ void noallocSobolPoints(const uint32_t* __restrict__ matrices, uint32_t start, uint32_t count,
                                   uint32_t* __restrict__ out)
{
    const uint32_t n = count * (uint32_t)yg::kSobolDims;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        uint32_t s = i / yg::kSobolDims, d = i % yg::kSobolDims;
        uint32_t index = start + s, v = 0;
        for (uint32_t k = d * 32; index != 0; index >>= 1, ++k)
            if (index & 1u) v ^= matrices[k];
        out[i] = v;
    }
}
} // namespace

extern "C" {

YG_API int yg_render_samples_noalloc(yg_context* ctx, const yg_render_params* p, float* device_sample_xyz)
{
    if (!ctx || !p || !device_sample_xyz) return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: null argument");
    if (((uintptr_t)device_sample_xyz & 15u) != 0)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: output must be 16-byte aligned device memory");
    std::lock_guard<std::mutex> g(ctx->lock);
    if (!ctx->sceneBuilt) return fail(YG_ERR_NOT_READY, "no-alloc render: call yg_build_scene first");
    if (!ctx->cameraSet) return fail(YG_ERR_NOT_READY, "no-alloc render: camera not set");
    if (p->integrator > YG_INTEGRATOR_NEE)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: only the uni and NEE integrators are available");
    if (p->width == 0 || p->height == 0 || p->spp_count == 0)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: empty request");
    if (p->spp_count > kNoAllocMaxSpp)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: spp_count " + std::to_string(p->spp_count) +
                                                 " exceeds the maximum of " + std::to_string(kNoAllocMaxSpp) +
                                                 " sample indices per call");
    uint32_t cx = p->crop_x, cy = p->crop_y, cw = p->crop_w, ch = p->crop_h;
    if (cw == 0 || ch == 0)
    {
        cx = cy = 0;
        cw = p->width;
        ch = p->height;
    }
    if ((uint64_t)cx + cw > p->width || (uint64_t)cy + ch > p->height)
        return fail(YG_ERR_INVALID_ARGUMENT, "no-alloc render: crop outside image");
    float lminf = p->lambda_min, lmaxf = p->lambda_max;
    if (lminf == 0.0f && lmaxf == 0.0f)
    {
        lminf = 380.f;
        lmaxf = 700.f;
    }
    if ((float)ctx->cieLmin != lminf || (float)ctx->cieLmax != lmaxf)
        return fail(YG_ERR_NOT_READY, "no-alloc render: spectral range differs from the context's current range "
                                      "(render once with yg_render at this range first)");
    bool needRgb = sceneNeedsRgbLut(ctx, p->env_intensity_scale);
    if (needRgb && (ctx->rgbToSpd.empty() || ctx->rgbLmin != ctx->cieLmin || ctx->rgbLmax != ctx->cieLmax || !ctx->dRgb.p))
        return fail(YG_ERR_NOT_READY, "no-alloc render: the RGB spectral fit is not resident "
                                      "(render once with yg_render at this range first)");
    int r = checkMaterialTextures(ctx, "no-alloc render");
    if (r) return r;
    YG_CUDA(cudaSetDevice(ctx->device));
    void* scratch = nullptr;
    if ((r = noallocScratchAddress(ctx->device, ctx->sobolMatrices, &scratch))) return r;
    char* base = static_cast<char*>(scratch);
    uint32_t* sobolPts = reinterpret_cast<uint32_t*>(base);
    const uint32_t* matrices = reinterpret_cast<const uint32_t*>(base + kNoAllocSobolBytes);
    void* arena = base + kNoAllocSobolBytes + kNoAllocMatrixBytes;
    noallocSobolPoints<<<ctx->smCount, 256, 0, ctx->stream>>>(matrices, p->spp_start, p->spp_count, sobolPts);

    yg::SceneView S;
    fillSceneView(ctx, lminf, lmaxf, needRgb, S);
    S.sobol = sobolPts;

    yg::LaunchParams L{};
    L.integrator = p->integrator;
    L.width = p->width;
    L.height = p->height;
    L.cropX = cx;
    L.cropY = cy;
    L.cropW = cw;
    L.cropH = ch;
    L.sppStart = p->spp_start;
    L.sppCount = p->spp_count;
    L.maxDepth = p->max_depth;
    L.regularizeAfter = p->regularize_after_vertices;
    L.regularizeEnable = p->regularize_enable;
    L.envScale = p->env_intensity_scale;
    L.seed = p->seed;
    L.flags = p->flags;
    L.nSamples = (uint64_t)cw * ch * p->spp_count;
    L.sampleXYZ = reinterpret_cast<float4*>(device_sample_xyz);
    yg::launchWavefront(S, L, arena, kNoAllocWaveCapacity, ctx->smCount, ctx->stream);
    YG_CUDA(cudaGetLastError());
    return YG_OK;
}

} // extern "C"
