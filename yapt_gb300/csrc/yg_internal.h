// Internal host-side declarations shared by the C-ABI translation units (context state,
// device buffers, table set-up, request resolution). Not part of the public interface.
#pragma once
#include "../../include/yapt_gpu.h"
#include "yg_kernels.h"
#include "yg_tables.h"
#include "yg_types.h"

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

namespace ygi
{
// records msg as the calling thread's last error and returns code
int fail(int code, const std::string& msg);

#define YG_CUDA(call)                                                                                              \
    do                                                                                                             \
    {                                                                                                              \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess)                                                                                     \
            return fail(e_ == cudaErrorMemoryAllocation ? YG_ERR_OUT_OF_MEMORY : YG_ERR_CUDA,                      \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                                       \
    } while (0)

struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n)
    {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    // takes ownership of a cudaMalloc'd block
    void adopt(void* q, size_t n)
    {
        release();
        p = q;
        bytes = n;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

struct Mesh
{
    uint32_t vertexBase, vertexCount, indexBase, indexCount;
    bool tangents, uvs;
    std::vector<std::pair<uint32_t, uint32_t>> submeshes;
};
} // namespace ygi


using ygi::DevBuf;
using ygi::Mesh;

struct yg_context
{
    std::mutex lock;
    int device = 0;
    int smCount = 152;
    cudaStream_t stream = nullptr;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    std::vector<cudaEvent_t> kernelEvents; // YG_FLAG_TIME_KERNELS: pairs around timed launches
    std::vector<uint8_t> kernelKinds;
    uint32_t kernelTimed = 0;
    std::string dataDir;
    // tables
    std::vector<uint32_t> sobolMatrices;
    std::vector<double> cie471;
    yg::MsLuts luts;
    std::vector<float> rgbToSpd;
    int rgbLmin = 0, rgbLmax = 0;
    // scene (host)
    std::vector<float> positions, normals, uvs;
    std::vector<float4> tangents;
    std::vector<uint32_t> indices;
    std::vector<Mesh> meshes;
    std::vector<yg_material> materials;
    std::vector<yg::GpuMaterial> gpuMaterials;
    std::vector<float> spectra;
    uint32_t specPoints = 0;
    float specLmin = 380.f, specLmax = 780.f;
    std::vector<yg_instance> instances;
    yg::GpuCamera camera{};
    bool cameraSet = false;
    bool sceneBuilt = false;
    uint32_t nAlphaInstances = 0; // alpha-tested instances of the built scene (their cutout
                                  // records point into texture memory)
    uint64_t nTris = 0, nNodes = 0;
    uint32_t bvhDepth = 0;
    // device
    DevBuf dTris, dNodes, dInst, dMat, dLights, dPos, dNrm, dTan, dUV, dIdx, dSpec;
    DevBuf dLut[9];
    DevBuf dCie, dRgb, dSobol, dSobolMat, dSamples, dDump, dFeatA, dFeatN, dRelmse, dRef, dRayCount;
    DevBuf dFilmSum, dFilmComp, dAccA, dAccN, dArena, dPerm;
    DevBuf dPrimStart, dTriOfPrim; // first primitive of each instance; each primitive's triangle slot
    DevBuf dBoundsErr;             // debug build: out-of-range accesses the kernels refused
    DevBuf dAtrousMom, dAtrousOdd, dAtrousFeat, dAtrousCol, dAtrousVar; // a-trous denoiser state
    std::vector<DevBuf> texBufs;          // decoded texels of each texture
    std::vector<yg::GpuTexture> texTable; // device pointers and sizes, mirrored in dTexTable
    DevBuf dTexTable;
    DevBuf dDisplay, dDisplayOut; // tonemap histogram, exposure state, RGBA8 image
    int envTexture = -1;
    bool envCube = false;
    uint32_t nLights = 0;   // mesh and punctual
    uint32_t nPunctual = 0;
    std::vector<yg_punctual_light> punctual;
    std::vector<yg::GpuInstance> hostInst;  // as uploaded; lightPdf rewritten with the light table
    std::vector<uint32_t> meshLightInst;    // emissive instances and their power estimates
    std::vector<float> meshLightPower;
    float worldLo[3] = {0, 0, 0}, worldHi[3] = {0, 0, 0};
    float worldCenter[3] = {0, 0, 0}; // getWorldCenterAndRadiusSqr (raytraceCommonResources.hlsl:99-104)
    float worldRadiusSqr = 0;
    uint32_t permW = 0, permH = 0;    // size of the BDPT pixel permutation in dPerm
    int cieLmin = -1, cieLmax = -1;
    uint32_t cieN = 0;
    float cieYSumInv = 0, d65SumInv = 0;
    uint32_t filmW = 0, filmH = 0;
    bool featuresOn = false;
    // a-trous gather over the film renders since yg_film_clear: 0 none yet, 1 all gathered,
    // 2 none gathered, 3 mixed
    int atrousState = 0;
    // stats
    float lastMs = 0;
    uint64_t lastRays = 0;
    uint32_t lastLaunches = 0;

    ~yg_context()
    {
        DevBuf* all[] = {&dTris, &dNodes, &dInst, &dMat, &dLights, &dPos, &dNrm, &dTan, &dUV, &dIdx, &dSpec, &dCie, &dRgb,
                         &dSobol, &dSobolMat, &dSamples, &dDump, &dFeatA, &dFeatN, &dRelmse, &dRef, &dRayCount, &dFilmSum,
                         &dFilmComp, &dAccA, &dAccN, &dArena, &dPerm, &dPrimStart, &dTriOfPrim, &dBoundsErr, &dAtrousMom, &dAtrousOdd,
                         &dAtrousFeat, &dAtrousCol, &dAtrousVar};
        for (DevBuf* b : all) b->release();
        for (DevBuf& b : texBufs) b.release();
        dTexTable.release();
        dDisplay.release();
        dDisplayOut.release();
        for (auto& b : dLut) b.release();
        for (cudaEvent_t e : kernelEvents) cudaEventDestroy(e);
        if (evStart) cudaEventDestroy(evStart);
        if (evStop) cudaEventDestroy(evStop);
        if (stream) cudaStreamDestroy(stream);
    }
};


namespace ygi
{
template <typename T>
int upload(yg_context* c, DevBuf& b, const T* src, size_t count)
{
    size_t bytes = std::max<size_t>(sizeof(T) * count, 16);
    YG_CUDA(b.ensure(bytes));
    if (count) YG_CUDA(cudaMemcpyAsync(b.p, src, sizeof(T) * count, cudaMemcpyHostToDevice, c->stream));
    return YG_OK;
}
int ensureCie(yg_context* c, int lmin, int lmax);
bool sceneNeedsRgbLut(const yg_context* c, float envScale);
int ensureRgbLut(yg_context* c, int lmin, int lmax);
// The scene arrays and tables of a context as one SceneView (Sobol points left unset); the
// CIE table of [lmin, lmax] (and the RGB table when needRgb) must be current.
void fillSceneView(const yg_context* c, float lmin, float lmax, bool needRgb, yg::SceneView& S);
int checkWideBvhStructure(yg_context* c);
// Fails (naming `what`) when a material refers to a texture id that is not resident, e.g.
// after yg_clear_textures: the device texture table then holds freed pointers.
int checkMaterialTextures(const yg_context* c, const char* what);
// the pixel order of the BDPT camera groups for a cw x ch crop
void pixelPermutation(uint32_t cw, uint32_t ch, std::vector<uint32_t>& perm);
} // namespace ygi
