// Serving loop: many render requests on the scenes of several resident contexts, with
// admission by device-memory footprint, continuous batching of uni/NEE requests into one
// merged wavefront per round (replayed as a captured CUDA graph) and BDPT requests advancing
// on a second stream. The interface is declared in include/yapt_gpu.h; the reference has no
// counterpart (it renders one interactive view, PathTraceStage.cpp:90-140).
//
// Every request is rendered in whole sample planes (one sample index over all its pixels),
// in sample-index order, into its own Kahan film: a sample depends only on the request
// (scene, camera, seed, sample index, pixel), so a result is the same film whether the
// request ran alone (yg_render) or merged with any others.
#include "yg_internal.h"
#include "yg_nvtx.h"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <thread>

using namespace ygi;

namespace
{
constexpr uint32_t kAgePriority = 8;      // rounds a request may be passed over before it goes first
constexpr uint32_t kMaxRoundPlanes = 4096; // sample planes (Sobol points) per merged round or BDPT slice

struct PlanIn
{
    uint64_t pixels;
    uint32_t planesLeft;
    bool admitted;
    uint64_t footprint;
    uint32_t integrator;
    uint32_t age;
};

// Admission in arrival order (no overtaking, so a large request is never starved), then one
// merged round for the admitted uni/NEE requests: fewest remaining samples first, except that
// requests passed over for kAgePriority rounds go first. A request gets whole planes; the
// round stops at roundSamples unless its first request alone needs more (one plane always fits
// waveCapacity, which the server checks at submission).
uint64_t planRound(const std::vector<PlanIn>& it, uint64_t budget, uint64_t inUse, uint32_t maxActive, uint32_t waveCapacity,
                   uint32_t roundSamples, std::vector<uint32_t>& admit, std::vector<uint32_t>& planes)
{
    const size_t n = it.size();
    admit.assign(n, 0);
    planes.assign(n, 0);
    uint32_t active = 0;
    for (const PlanIn& p : it) active += p.admitted ? 1u : 0u;
    for (size_t i = 0; i < n; ++i)
    {
        if (it[i].admitted) continue;
        if (active >= maxActive || inUse + it[i].footprint > budget) break;
        admit[i] = 1;
        inUse += it[i].footprint;
        ++active;
    }
    std::vector<size_t> cand;
    for (size_t i = 0; i < n; ++i)
        if ((it[i].admitted || admit[i]) && it[i].integrator != YG_INTEGRATOR_BDPT && it[i].planesLeft > 0) cand.push_back(i);
    std::stable_sort(cand.begin(), cand.end(), [&](size_t a, size_t b) {
        bool oa = it[a].age >= kAgePriority, ob = it[b].age >= kAgePriority;
        if (oa != ob) return oa;
        if (oa) return it[a].age > it[b].age;
        return it[a].pixels * it[a].planesLeft < it[b].pixels * it[b].planesLeft;
    });
    uint64_t total = 0, planesUsed = 0;
    for (size_t c : cand)
    {
        const uint64_t px = it[c].pixels;
        if (planesUsed >= kMaxRoundPlanes) break;
        uint64_t share = total < roundSamples ? (roundSamples - total) / px : 0;
        if (share == 0)
        {
            if (total != 0) continue;
            share = 1;
        }
        uint64_t room = (waveCapacity - total) / px;
        uint64_t k = std::min<uint64_t>({(uint64_t)it[c].planesLeft, share, room, kMaxRoundPlanes - planesUsed});
        if (k == 0) continue;
        planes[c] = (uint32_t)k;
        total += k * px;
        planesUsed += k;
    }
    return total;
}

double nowSince(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

struct Req
{
    uint64_t id = 0;
    uint32_t scene = 0;
    yg_render_params p{};
    uint32_t cx = 0, cy = 0, cw = 0, ch = 0;
    uint64_t npix = 0;
    uint32_t planesTotal = 0, planesDone = 0;
    bool bdpt = false, needRgb = false;
    uint32_t lightPaths = 0, lightVerts = 0, bdptPlanes = 0;
    uint64_t footprint = 0;
    int state = YG_REQ_QUEUED;
    int error = 0;
    std::string message;
    double tSubmit = -1, tAdmit = -1, tDone = -1;
    float4* film = nullptr; // W*H sums, then W*H compensations
    std::vector<float4> result;
    uint32_t age = 0;
    bool inFlight = false, cancelRequested = false;
};

struct Segment
{
    Req* r;
    uint32_t planes;
};
} // namespace

struct yg_server
{
    std::vector<yg_context*> scenes;
    yg_server_options opt{};
    int device = 0, smCount = 152;
    float lmin = 380.f, lmax = 700.f;
    cudaStream_t sA = nullptr, sB = nullptr;
    cudaEvent_t evA = nullptr, evB = nullptr;
    std::chrono::steady_clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv;
    std::map<uint64_t, std::unique_ptr<Req>> reqs;
    std::deque<uint64_t> queue;    // arrival order, not yet admitted
    std::vector<uint64_t> active;  // admitted, arrival order
    std::thread worker;
    bool stop = false;
    uint64_t nextId = 1;
    yg_server_stats st{};
    uint64_t bytesInUse = 0;
    // merged round
    void* waveArena = nullptr;
    float4* roundSamples = nullptr;
    char* tablesDev = nullptr;
    char* tablesHost = nullptr; // pinned
    size_t tablesBytes = 0;
    uint32_t* sobolDev = nullptr;
    uint32_t* sobolHost = nullptr; // pinned
    uint32_t sobolPlanes = 0;
    yg::MultiTables M{};
    cudaGraphExec_t graph = nullptr;
    yg::GridBarrier* barrier = nullptr; // persistent round: 4 words of device memory
    bool persistentUncaptured = false;   // the cooperative round could not be captured
    uint32_t* barrierErrHost = nullptr; // pinned copy of the barrier's error word after a round
    std::vector<Segment> inFlightA;
    // BDPT slice
    Req* inFlightB = nullptr;
    uint32_t planesB = 0;
    void* bdptArena = nullptr;
    float4* bdptSamples = nullptr;
    uint32_t* sobolDevB = nullptr;
    uint32_t* sobolHostB = nullptr;
    std::map<std::pair<uint32_t, uint32_t>, uint32_t*> perms;
    std::string fatal;
};

namespace
{
size_t alignUp(size_t b) { return (b + 255) & ~size_t(255); }

// device table layout (fixed offsets; the captured round reads them every replay)
struct TableLayout
{
    size_t views, params, segReq, segStart, segPixStart, nSeg, filmSum, filmComp, total;
};
TableLayout tableLayout(uint32_t slots)
{
    TableLayout L;
    size_t o = 0;
    L.views = o; o += alignUp(sizeof(yg::SceneView) * slots);
    L.params = o; o += alignUp(sizeof(yg::LaunchParams) * slots);
    L.segReq = o; o += alignUp(4 * (size_t)slots);
    L.segStart = o; o += alignUp(4 * ((size_t)slots + 1));
    L.segPixStart = o; o += alignUp(4 * ((size_t)slots + 1));
    L.nSeg = o; o += alignUp(4);
    L.filmSum = o; o += alignUp(sizeof(void*) * slots);
    L.filmComp = o; o += alignUp(sizeof(void*) * slots);
    L.total = o;
    return L;
}

int validate(yg_server* s, const yg_request* q, Req& r)
{
    const yg_render_params& p = q->params;
    if (q->scene >= s->scenes.size()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: no such scene");
    if (p.integrator > YG_INTEGRATOR_BDPT) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown integrator");
    if (p.width == 0 || p.height == 0 || p.spp_count == 0) return fail(YG_ERR_INVALID_ARGUMENT, "serve: empty request");
    if (p.flags & ~YG_FLAG_DISABLE_TEXEL_JITTER) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unsupported flags");
    float lminf = p.lambda_min, lmaxf = p.lambda_max;
    if (lminf == 0.0f && lmaxf == 0.0f)
    {
        lminf = 380.f;
        lmaxf = 700.f;
    }
    if (lminf != s->lmin || lmaxf != s->lmax) return fail(YG_ERR_INVALID_ARGUMENT, "serve: spectral range differs from the server's");
    r.cx = p.crop_x;
    r.cy = p.crop_y;
    r.cw = p.crop_w;
    r.ch = p.crop_h;
    if (r.cw == 0 || r.ch == 0)
    {
        r.cx = r.cy = 0;
        r.cw = p.width;
        r.ch = p.height;
    }
    if ((uint64_t)r.cx + r.cw > p.width || (uint64_t)r.cy + r.ch > p.height)
        return fail(YG_ERR_INVALID_ARGUMENT, "serve: crop outside image");
    r.npix = (uint64_t)r.cw * r.ch;
    if (r.npix > s->opt.wave_capacity) return fail(YG_ERR_INVALID_ARGUMENT, "serve: one sample plane exceeds the wave capacity");
    r.bdpt = p.integrator == YG_INTEGRATOR_BDPT;
    if (!r.bdpt && p.max_depth > s->opt.max_depth) return fail(YG_ERR_INVALID_ARGUMENT, "serve: max_depth above the server's");
    yg_context* ctx = s->scenes[q->scene];
    r.needRgb = sceneNeedsRgbLut(ctx, p.env_intensity_scale);
    r.scene = q->scene;
    r.p = p;
    r.planesTotal = p.spp_count;
    r.footprint = alignUp((size_t)p.width * p.height * 32);
    if (r.bdpt)
    {
        r.lightVerts = p.bdpt_light_vertices ? p.bdpt_light_vertices : yg::kBdptMaxLightVertices;
        if (r.lightVerts < 2 || r.lightVerts > yg::kBdptMaxLightVertices)
            return fail(YG_ERR_INVALID_ARGUMENT, "serve: bdpt_light_vertices must be 2..16");
        r.lightPaths = p.bdpt_light_paths ? p.bdpt_light_paths : ((r.cw + 7) / 8) * ((r.ch + 7) / 8);
        r.bdptPlanes = (uint32_t)std::max<uint64_t>(
            1, std::min<uint64_t>({(uint64_t)r.planesTotal, (1ull << 19) / r.npix, (uint64_t)kMaxRoundPlanes}));
        r.footprint += alignUp(yg::bdptArenaBytes(r.bdptPlanes, r.lightPaths, r.lightVerts, r.npix)) +
                       alignUp(r.npix * r.bdptPlanes * 16);
    }
    if (r.footprint > s->opt.memory_budget_bytes) return fail(YG_ERR_ADMISSION, "serve: request exceeds the memory budget");
    return YG_OK;
}

void markDone(yg_server* s, Req* r, int state, int err, const std::string& msg)
{
    r->state = state;
    r->error = err;
    r->message = msg;
    r->tDone = nowSince(s->t0);
    if (state == YG_REQ_DONE) ++s->st.completed;
    else if (state == YG_REQ_FAILED) ++s->st.failed;
    else if (state == YG_REQ_CANCELLED) ++s->st.cancelled;
    s->cv.notify_all();
}

// returns the film and footprint of an admitted request (stream-ordered free)
void releaseActive(yg_server* s, Req* r, cudaStream_t stream)
{
    if (r->film) cudaFreeAsync(r->film, stream);
    r->film = nullptr;
    s->bytesInUse -= r->footprint;
    s->active.erase(std::find(s->active.begin(), s->active.end(), r->id));
}

int admit(yg_server* s, Req* r)
{
    cudaStream_t st = r->bdpt ? s->sB : s->sA;
    size_t bytes = (size_t)r->p.width * r->p.height * 32;
    cudaError_t e = cudaMallocAsync((void**)&r->film, bytes, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(r->film, 0, bytes, st);
    if (e != cudaSuccess) return fail(YG_ERR_OUT_OF_MEMORY, std::string("serve: film: ") + cudaGetErrorString(e));
    r->state = YG_REQ_ACTIVE;
    r->tAdmit = nowSince(s->t0);
    s->bytesInUse += r->footprint;
    s->st.peak_bytes_in_use = std::max(s->st.peak_bytes_in_use, (uint64_t)s->bytesInUse);
    s->active.push_back(r->id);
    return YG_OK;
}

void fillLaunch(yg_server* s, const Req& r, uint32_t planes, yg::LaunchParams& L)
{
    L = yg::LaunchParams{};
    const yg_render_params& p = r.p;
    L.integrator = p.integrator;
    L.width = p.width;
    L.height = p.height;
    L.cropX = r.cx;
    L.cropY = r.cy;
    L.cropW = r.cw;
    L.cropH = r.ch;
    L.sppStart = p.spp_start + r.planesDone;
    L.sppCount = planes;
    L.maxDepth = p.max_depth;
    L.regularizeAfter = p.regularize_after_vertices;
    L.regularizeEnable = p.regularize_enable;
    L.envScale = p.env_intensity_scale;
    L.seed = p.seed;
    L.flags = p.flags;
    L.nSamples = r.npix * planes;
    (void)s;
}

void sobolPlanes(yg_context* ctx, uint32_t first, uint32_t count, uint32_t* out)
{
    for (uint32_t k = 0; k < count; ++k)
        for (uint32_t d = 0; d < (uint32_t)yg::kSobolDims; ++d)
            out[(size_t)k * yg::kSobolDims + d] = yg::sobolUint(ctx->sobolMatrices.data(), first + k, d);
}

// launches one merged round for the planned segments on stream A
int launchMerged(yg_server* s, std::vector<Segment>& segs)
{
    yg::NvtxRange range("serve merged round");
    const uint32_t slots = s->opt.max_active;
    TableLayout T = tableLayout(slots);
    char* h = s->tablesHost;
    yg::SceneView* views = reinterpret_cast<yg::SceneView*>(h + T.views);
    yg::LaunchParams* params = reinterpret_cast<yg::LaunchParams*>(h + T.params);
    uint32_t* segReq = reinterpret_cast<uint32_t*>(h + T.segReq);
    uint32_t* segStart = reinterpret_cast<uint32_t*>(h + T.segStart);
    uint32_t* segPix = reinterpret_cast<uint32_t*>(h + T.segPixStart);
    uint32_t* nSeg = reinterpret_cast<uint32_t*>(h + T.nSeg);
    float4** fs = reinterpret_cast<float4**>(h + T.filmSum);
    float4** fc = reinterpret_cast<float4**>(h + T.filmComp);
    uint32_t wave = 0, pix = 0, plane = 0;
    for (uint32_t k = 0; k < segs.size(); ++k)
    {
        Req& r = *segs[k].r;
        const uint32_t planes = segs[k].planes;
        yg_context* ctx = s->scenes[r.scene];
        fillSceneView(ctx, s->lmin, s->lmax, r.needRgb, views[k]);
        views[k].sobol = s->sobolDev + (size_t)plane * yg::kSobolDims;
        sobolPlanes(ctx, r.p.spp_start + r.planesDone, planes, s->sobolHost + (size_t)plane * yg::kSobolDims);
        fillLaunch(s, r, planes, params[k]);
        params[k].sampleXYZ = s->roundSamples + wave;
        segReq[k] = k;
        segStart[k] = wave;
        segPix[k] = pix;
        fs[k] = r.film;
        fc[k] = r.film + (size_t)r.p.width * r.p.height;
        wave += (uint32_t)(r.npix * planes);
        pix += (uint32_t)r.npix;
        plane += planes;
    }
    segStart[segs.size()] = wave;
    segPix[segs.size()] = pix;
    *nSeg = (uint32_t)segs.size();
    YG_CUDA(cudaMemcpyAsync(s->tablesDev, s->tablesHost, T.total, cudaMemcpyHostToDevice, s->sA));
    YG_CUDA(cudaMemcpyAsync(s->sobolDev, s->sobolHost, (size_t)plane * yg::kSobolDims * 4, cudaMemcpyHostToDevice, s->sA));
    if (s->opt.persistent)
    {
        // the barrier set-up and the cooperative round, captured once when graphs are on
        // (replayed like the multi-kernel round), else launched directly
        if (s->opt.use_graphs && !s->graph && !s->persistentUncaptured)
        {
            cudaGraph_t g = nullptr;
            YG_CUDA(cudaStreamBeginCapture(s->sA, cudaStreamCaptureModeThreadLocal));
            int n = yg::launchWavefrontMultiPersistent(s->M, s->waveArena, s->opt.wave_capacity, s->opt.max_depth, nullptr,
                                                      s->smCount, s->sA, s->barrier, s->opt.barrier_polls);
            cudaError_t e = cudaStreamEndCapture(s->sA, &g);
            if (n >= 0 && e == cudaSuccess) e = cudaGraphInstantiate(&s->graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (n < 0 || e != cudaSuccess)
            {
                // this driver does not capture cooperative launches: launch them directly
                if (s->graph) cudaGraphExecDestroy(s->graph);
                s->graph = nullptr;
                s->persistentUncaptured = true;
                cudaGetLastError();
            }
        }
        if (s->graph)
        {
            YG_CUDA(cudaGraphLaunch(s->graph, s->sA));
            ++s->st.graph_replays;
        }
        else
        {
            int n = yg::launchWavefrontMultiPersistent(s->M, s->waveArena, s->opt.wave_capacity, s->opt.max_depth, nullptr,
                                                      s->smCount, s->sA, s->barrier, s->opt.barrier_polls);
            if (n < 0)
                return fail(YG_ERR_CUDA, std::string("serve: persistent round: ") + cudaGetErrorString((cudaError_t)(-n)));
        }
        YG_CUDA(cudaMemcpyAsync(s->barrierErrHost, reinterpret_cast<char*>(s->barrier) + 8, 4, cudaMemcpyDeviceToHost,
                                s->sA));
        ++s->st.persistent_rounds;
    }
    else if (s->opt.use_graphs)
    {
        if (!s->graph)
        {
            cudaGraph_t g = nullptr;
            YG_CUDA(cudaStreamBeginCapture(s->sA, cudaStreamCaptureModeThreadLocal));
            yg::launchWavefrontMulti(s->M, s->waveArena, s->opt.wave_capacity, s->opt.max_depth, nullptr, s->smCount, s->sA);
            YG_CUDA(cudaStreamEndCapture(s->sA, &g));
            cudaError_t e = cudaGraphInstantiate(&s->graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) return fail(YG_ERR_CUDA, std::string("serve: graph: ") + cudaGetErrorString(e));
        }
        YG_CUDA(cudaGraphLaunch(s->graph, s->sA));
        ++s->st.graph_replays;
    }
    else
    {
        yg::launchWavefrontMulti(s->M, s->waveArena, s->opt.wave_capacity, s->opt.max_depth, nullptr, s->smCount, s->sA);
    }
    YG_CUDA(cudaGetLastError());
    YG_CUDA(cudaEventRecord(s->evA, s->sA));
    s->st.samples += wave;
    ++s->st.rounds;
    return YG_OK;
}

int launchBdptSlice(yg_server* s, Req& r, uint32_t planes)
{
    yg::NvtxRange range("serve BDPT slice");
    yg_context* ctx = s->scenes[r.scene];
    auto key = std::make_pair(r.cw, r.ch);
    if (!s->perms.count(key))
    {
        std::vector<uint32_t> perm;
        pixelPermutation(r.cw, r.ch, perm);
        uint32_t* d = nullptr;
        YG_CUDA(cudaMalloc((void**)&d, perm.size() * 4));
        YG_CUDA(cudaMemcpy(d, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice));
        s->perms[key] = d;
    }
    yg::SceneView S;
    fillSceneView(ctx, s->lmin, s->lmax, r.needRgb, S);
    sobolPlanes(ctx, r.p.spp_start + r.planesDone, planes, s->sobolHostB);
    YG_CUDA(cudaMemcpyAsync(s->sobolDevB, s->sobolHostB, (size_t)planes * yg::kSobolDims * 4, cudaMemcpyHostToDevice, s->sB));
    S.sobol = s->sobolDevB;
    size_t arenaBytes = yg::bdptArenaBytes(planes, r.lightPaths, r.lightVerts, r.npix);
    YG_CUDA(cudaMallocAsync(&s->bdptArena, arenaBytes, s->sB));
    YG_CUDA(cudaMallocAsync((void**)&s->bdptSamples, r.npix * planes * 16, s->sB));
    yg::LaunchParams L;
    fillLaunch(s, r, planes, L);
    L.sampleXYZ = s->bdptSamples;
    yg::launchBdpt(S, L, s->bdptArena, s->perms[key], r.lightPaths, r.lightVerts,
                   make_float3(ctx->worldCenter[0], ctx->worldCenter[1], ctx->worldCenter[2]), ctx->worldRadiusSqr, s->smCount,
                   s->sB);
    yg::launchFilm(r.film, r.film + (size_t)r.p.width * r.p.height, s->bdptSamples, r.p.width, r.cx, r.cy, r.cw, r.ch,
                   planes, s->smCount, s->sB);
    YG_CUDA(cudaFreeAsync(s->bdptArena, s->sB));
    YG_CUDA(cudaFreeAsync(s->bdptSamples, s->sB));
    s->bdptArena = nullptr;
    s->bdptSamples = nullptr;
    YG_CUDA(cudaGetLastError());
    YG_CUDA(cudaEventRecord(s->evB, s->sB));
    s->st.samples += r.npix * planes;
    ++s->st.bdpt_slices;
    return YG_OK;
}

// copies the film of a finished request to the host and frees its device memory
int finishRequest(yg_server* s, Req* r, cudaStream_t stream)
{
    size_t n = (size_t)r->p.width * r->p.height;
    r->result.resize(n);
    YG_CUDA(cudaMemcpyAsync(r->result.data(), r->film, n * sizeof(float4), cudaMemcpyDeviceToHost, stream));
    YG_CUDA(cudaStreamSynchronize(stream));
    releaseActive(s, r, stream);
    markDone(s, r, YG_REQ_DONE, 0, "");
    return YG_OK;
}

void failAll(yg_server* s, const std::string& why)
{
    s->fatal = why;
    for (auto& kv : s->reqs)
    {
        Req* r = kv.second.get();
        if (r->state == YG_REQ_QUEUED || r->state == YG_REQ_ACTIVE) markDone(s, r, YG_REQ_FAILED, YG_ERR_CUDA, why);
    }
    s->queue.clear();
    s->active.clear();
}

void workerLoop(yg_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lk(s->mu);
    while (true)
    {
        // completions
        if (!s->inFlightA.empty() && cudaEventQuery(s->evA) != cudaErrorNotReady)
        {
            cudaError_t e = cudaEventSynchronize(s->evA);
            if (e != cudaSuccess)
            {
                failAll(s, std::string("serve: merged round: ") + cudaGetErrorString(e));
                s->inFlightA.clear();
            }
            else if (s->opt.persistent && *s->barrierErrHost != 0)
            {
                // a grid barrier ran out of polls: the round's films are incomplete, the
                // context is intact; the requests of the round fail, the server goes on
                for (Segment& g : s->inFlightA)
                {
                    g.r->inFlight = false;
                    releaseActive(s, g.r, s->sA);
                    markDone(s, g.r, YG_REQ_FAILED, YG_ERR_DEVICE_TIMEOUT,
                             "serve: persistent round: a grid barrier wait ran out");
                }
                s->inFlightA.clear();
                *s->barrierErrHost = 0;
            }
            for (Segment& g : s->inFlightA)
            {
                Req* r = g.r;
                r->inFlight = false;
                r->planesDone += g.planes;
                if (r->planesDone == r->planesTotal && finishRequest(s, r, s->sA) != YG_OK)
                    markDone(s, r, YG_REQ_FAILED, YG_ERR_CUDA, yg_last_error());
            }
            s->inFlightA.clear();
            s->cv.notify_all();
        }
        if (s->inFlightB && cudaEventQuery(s->evB) != cudaErrorNotReady)
        {
            Req* r = s->inFlightB;
            cudaError_t e = cudaEventSynchronize(s->evB);
            r->inFlight = false;
            s->inFlightB = nullptr;
            if (e != cudaSuccess) failAll(s, std::string("serve: BDPT slice: ") + cudaGetErrorString(e));
            else
            {
                r->planesDone += s->planesB;
                if (r->planesDone == r->planesTotal && finishRequest(s, r, s->sB) != YG_OK)
                    markDone(s, r, YG_REQ_FAILED, YG_ERR_CUDA, yg_last_error());
            }
            s->cv.notify_all();
        }
        // cancelled requests that are not on the device any more
        for (size_t i = 0; i < s->active.size();)
        {
            Req* r = s->reqs[s->active[i]].get();
            if (r->cancelRequested && !r->inFlight)
            {
                releaseActive(s, r, r->bdpt ? s->sB : s->sA);
                markDone(s, r, YG_REQ_CANCELLED, 0, "cancelled");
                s->cv.notify_all();
                continue;
            }
            ++i;
        }
        if (s->stop && s->inFlightA.empty() && !s->inFlightB) break;
        if (s->stop)
        {
            s->cv.wait_for(lk, std::chrono::microseconds(50));
            continue;
        }
        // admission + merged round plan (only when stream A is free, so admission sees fresh state)
        if (s->inFlightA.empty())
        {
            std::vector<PlanIn> in;
            std::vector<Req*> rs;
            for (uint64_t id : s->active)
            {
                Req* r = s->reqs[id].get();
                in.push_back({r->npix, r->planesTotal - r->planesDone, true, r->footprint, r->p.integrator, r->age});
                rs.push_back(r);
            }
            for (uint64_t id : s->queue)
            {
                Req* r = s->reqs[id].get();
                in.push_back({r->npix, r->planesTotal, false, r->footprint, r->p.integrator, 0});
                rs.push_back(r);
            }
            // requests being cancelled or already on stream B take no planes here
            for (size_t i = 0; i < rs.size(); ++i)
                if (rs[i]->cancelRequested || rs[i]->inFlight) in[i].planesLeft = 0;
            std::vector<uint32_t> adm, planes;
            planRound(in, s->opt.memory_budget_bytes, s->bytesInUse, s->opt.max_active, s->opt.wave_capacity,
                      s->opt.round_samples, adm, planes);
            for (size_t i = 0; i < rs.size(); ++i)
            {
                if (!adm[i]) continue;
                Req* r = rs[i];
                s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r->id));
                if (admit(s, r) != YG_OK)
                {
                    markDone(s, r, YG_REQ_FAILED, YG_ERR_OUT_OF_MEMORY, yg_last_error());
                    planes[i] = 0;
                }
            }
            std::vector<Segment> segs;
            for (size_t i = 0; i < rs.size(); ++i)
            {
                Req* r = rs[i];
                if (r->state != YG_REQ_ACTIVE || r->bdpt) continue;
                if (planes[i]) segs.push_back({r, planes[i]});
                else if (r->planesDone < r->planesTotal && !r->cancelRequested) ++r->age;
            }
            if (!segs.empty())
            {
                for (Segment& g : segs)
                {
                    g.r->inFlight = true;
                    g.r->age = 0;
                }
                if (launchMerged(s, segs) != YG_OK)
                {
                    failAll(s, yg_last_error());
                    for (Segment& g : segs) g.r->inFlight = false;
                }
                else s->inFlightA = segs;
            }
        }
        // one BDPT slice on stream B: the active BDPT request with the least work left
        if (!s->inFlightB)
        {
            Req* best = nullptr;
            for (uint64_t id : s->active)
            {
                Req* r = s->reqs[id].get();
                if (!r->bdpt || r->cancelRequested || r->planesDone == r->planesTotal) continue;
                uint64_t left = r->npix * (r->planesTotal - r->planesDone);
                if (!best || left < best->npix * (best->planesTotal - best->planesDone)) best = r;
            }
            if (best)
            {
                uint32_t planes = std::min(best->bdptPlanes, best->planesTotal - best->planesDone);
                best->inFlight = true;
                if (launchBdptSlice(s, *best, planes) != YG_OK)
                {
                    best->inFlight = false;
                    failAll(s, yg_last_error());
                }
                else
                {
                    s->inFlightB = best;
                    s->planesB = planes;
                }
            }
        }
        if (s->inFlightA.empty() && !s->inFlightB && s->queue.empty() && s->active.empty())
            s->cv.wait(lk, [&] { return s->stop || !s->queue.empty(); });
        else
            s->cv.wait_for(lk, std::chrono::microseconds(50));
    }
}

void fillInfo(const Req& r, yg_request_info* info)
{
    if (!info) return;
    info->state = r.state;
    info->error = r.error;
    info->t_submit = r.tSubmit;
    info->t_admit = r.tAdmit;
    info->t_done = r.tDone;
    info->footprint_bytes = r.footprint;
    info->samples = r.npix * r.planesTotal;
}
} // namespace

extern "C" {

YG_API int yg_server_create(yg_context* const* scenes, uint32_t n, const yg_server_options* options, yg_server** out)
{
    if (!scenes || n == 0 || !out) return fail(YG_ERR_INVALID_ARGUMENT, "serve: no scenes");
    *out = nullptr;
    std::unique_ptr<yg_server> s(new yg_server());
    if (options) s->opt = *options;
    yg_server_options& o = s->opt;
    if (o.memory_budget_bytes == 0) o.memory_budget_bytes = 8ull << 30;
    if (o.max_active == 0) o.max_active = 64;
    if (o.max_active > 256) return fail(YG_ERR_INVALID_ARGUMENT, "serve: max_active above 256");
    if (o.wave_capacity == 0) o.wave_capacity = 1u << 21;
    if (o.round_samples == 0) o.round_samples = 1u << 19;
    if (o.max_depth == 0) o.max_depth = 16;
    if (o.barrier_polls == 0) o.barrier_polls = 1u << 24;
    if (o.lambda_min != 0.0f || o.lambda_max != 0.0f)
    {
        s->lmin = o.lambda_min;
        s->lmax = o.lambda_max;
    }
    if ((float)(int)s->lmin != s->lmin || (float)(int)s->lmax != s->lmax)
        return fail(YG_ERR_INVALID_ARGUMENT, "serve: spectral range must be whole nm");
    s->device = scenes[0]->device;
    for (uint32_t i = 0; i < n; ++i)
    {
        yg_context* c = scenes[i];
        if (!c || c->device != s->device) return fail(YG_ERR_INVALID_ARGUMENT, "serve: scenes must share one device");
        std::lock_guard<std::mutex> g(c->lock);
        if (!c->sceneBuilt || !c->cameraSet) return fail(YG_ERR_NOT_READY, "serve: scene not built or camera not set");
        int r = checkMaterialTextures(c, "serve");
        if (r) return r;
        r = ensureCie(c, (int)s->lmin, (int)s->lmax);
        if (r) return r;
        if (i > 0 && !scenes[0]->rgbToSpd.empty() && c->rgbToSpd.empty())
        {
            c->rgbToSpd = scenes[0]->rgbToSpd; // the table depends only on the spectral range
            c->rgbLmin = scenes[0]->rgbLmin;
            c->rgbLmax = scenes[0]->rgbLmax;
            if ((r = upload(c, c->dRgb, c->rgbToSpd.data(), c->rgbToSpd.size()))) return r;
        }
        if ((r = ensureRgbLut(c, (int)s->lmin, (int)s->lmax))) return r;
        YG_CUDA(cudaStreamSynchronize(c->stream));
        s->scenes.push_back(c);
    }
    YG_CUDA(cudaSetDevice(s->device));
    cudaDeviceGetAttribute(&s->smCount, cudaDevAttrMultiProcessorCount, s->device);
    if (o.persistent)
    {
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device);
        if (!coop) return fail(YG_ERR_INVALID_ARGUMENT, "serve: persistent rounds need cooperative launch");
    }
    // merged rounds are short and carry most requests: their stream gets the higher priority,
    // so their blocks are scheduled ahead of the long BDPT kernels on the other stream
    int prLeast = 0, prGreatest = 0;
    YG_CUDA(cudaDeviceGetStreamPriorityRange(&prLeast, &prGreatest));
    YG_CUDA(cudaStreamCreateWithPriority(&s->sA, cudaStreamNonBlocking, prGreatest));
    YG_CUDA(cudaStreamCreateWithPriority(&s->sB, cudaStreamNonBlocking, prLeast));
    YG_CUDA(cudaEventCreateWithFlags(&s->evA, cudaEventDisableTiming));
    YG_CUDA(cudaEventCreateWithFlags(&s->evB, cudaEventDisableTiming));
    TableLayout T = tableLayout(o.max_active);
    s->tablesBytes = T.total;
    YG_CUDA(cudaMalloc((void**)&s->tablesDev, T.total));
    YG_CUDA(cudaMallocHost((void**)&s->tablesHost, T.total));
    std::memset(s->tablesHost, 0, T.total);
    s->sobolPlanes = kMaxRoundPlanes;
    const size_t sobolBytes = (size_t)kMaxRoundPlanes * yg::kSobolDims * 4;
    YG_CUDA(cudaMalloc((void**)&s->sobolDev, sobolBytes));
    YG_CUDA(cudaMallocHost((void**)&s->sobolHost, sobolBytes));
    YG_CUDA(cudaMalloc((void**)&s->sobolDevB, sobolBytes));
    YG_CUDA(cudaMallocHost((void**)&s->sobolHostB, sobolBytes));
    YG_CUDA(cudaMalloc(&s->waveArena, yg::multiWaveBytes(o.wave_capacity)));
    YG_CUDA(cudaMalloc((void**)&s->barrier, 16));
    YG_CUDA(cudaMallocHost((void**)&s->barrierErrHost, 4));
    *s->barrierErrHost = 0;
    YG_CUDA(cudaMalloc((void**)&s->roundSamples, (size_t)o.wave_capacity * 16));
    s->M.views = reinterpret_cast<const yg::SceneView*>(s->tablesDev + T.views);
    s->M.params = reinterpret_cast<const yg::LaunchParams*>(s->tablesDev + T.params);
    s->M.segReq = reinterpret_cast<const uint32_t*>(s->tablesDev + T.segReq);
    s->M.segStart = reinterpret_cast<const uint32_t*>(s->tablesDev + T.segStart);
    s->M.segPixStart = reinterpret_cast<const uint32_t*>(s->tablesDev + T.segPixStart);
    s->M.nSeg = reinterpret_cast<const uint32_t*>(s->tablesDev + T.nSeg);
    s->M.filmSum = reinterpret_cast<float4* const*>(s->tablesDev + T.filmSum);
    s->M.filmComp = reinterpret_cast<float4* const*>(s->tablesDev + T.filmComp);
    s->t0 = std::chrono::steady_clock::now();
    yg_server* raw = s.release();
    raw->worker = std::thread(workerLoop, raw);
    *out = raw;
    return YG_OK;
}

YG_API int yg_server_submit(yg_server* s, const yg_request* q, uint64_t* id)
{
    if (!s || !q || !id) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null argument");
    std::unique_ptr<Req> r(new Req());
    int rc = validate(s, q, *r);
    if (rc) return rc;
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return fail(YG_ERR_NOT_READY, "serve: server is shutting down");
    if (!s->fatal.empty()) return fail(YG_ERR_CUDA, s->fatal);
    r->id = s->nextId++;
    r->tSubmit = nowSince(s->t0);
    *id = r->id;
    s->queue.push_back(r->id);
    s->reqs[r->id] = std::move(r);
    ++s->st.submitted;
    s->cv.notify_all();
    return YG_OK;
}

YG_API int yg_server_wait(yg_server* s, uint64_t id, double timeout_s, yg_request_info* info)
{
    if (!s) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null server");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown request");
    Req* r = it->second.get();
    auto finished = [&] { return r->state >= YG_REQ_DONE; };
    if (timeout_s < 0) s->cv.wait(lk, finished);
    else if (!s->cv.wait_for(lk, std::chrono::duration<double>(timeout_s), finished))
    {
        fillInfo(*r, info);
        return fail(YG_ERR_NOT_READY, "serve: timeout");
    }
    fillInfo(*r, info);
    return YG_OK;
}

YG_API int yg_server_info(yg_server* s, uint64_t id, yg_request_info* info)
{
    if (!s || !info) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown request");
    fillInfo(*it->second, info);
    return YG_OK;
}

YG_API int yg_server_result(yg_server* s, uint64_t id, float* xyz, float* counts)
{
    if (!s || !xyz) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null argument");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown request");
    const Req& r = *it->second;
    if (r.state != YG_REQ_DONE) return fail(YG_ERR_NOT_READY, r.state == YG_REQ_FAILED ? r.message : "serve: request not done");
    for (size_t i = 0; i < r.result.size(); ++i)
    {
        float c = r.result[i].w;
        float inv = c > 0.0f ? 1.0f / c : 0.0f;
        xyz[3 * i] = r.result[i].x * inv;
        xyz[3 * i + 1] = r.result[i].y * inv;
        xyz[3 * i + 2] = r.result[i].z * inv;
        if (counts) counts[i] = c;
    }
    return YG_OK;
}

YG_API int yg_server_cancel(yg_server* s, uint64_t id)
{
    if (!s) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null server");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown request");
    Req* r = it->second.get();
    if (r->state == YG_REQ_QUEUED)
    {
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), id));
        markDone(s, r, YG_REQ_CANCELLED, 0, "cancelled");
    }
    else if (r->state == YG_REQ_ACTIVE)
        r->cancelRequested = true;
    s->cv.notify_all();
    return YG_OK;
}

YG_API int yg_server_release(yg_server* s, uint64_t id)
{
    if (!s) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null server");
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end()) return fail(YG_ERR_INVALID_ARGUMENT, "serve: unknown request");
    if (it->second->state < YG_REQ_DONE) return fail(YG_ERR_NOT_READY, "serve: request still queued or active");
    s->reqs.erase(it);
    return YG_OK;
}

YG_API int yg_grid_barrier_selftest(yg_context* ctx, uint32_t missing, uint32_t pollLimit, uint32_t* blocks,
                                    uint32_t* passes, uint32_t* timedOut)
{
    if (!ctx || !blocks || !passes || !timedOut) return fail(YG_ERR_INVALID_ARGUMENT, "barrier selftest: null argument");
    if (missing > 1024 || pollLimit == 0)
        return fail(YG_ERR_INVALID_ARGUMENT, "barrier selftest: missing <= 1024 and poll_limit > 0");
    std::lock_guard<std::mutex> g(ctx->lock);
    YG_CUDA(cudaSetDevice(ctx->device));
    char* d = nullptr;
    YG_CUDA(cudaMalloc((void**)&d, 32));
    uint32_t h[8] = {};
    cudaError_t e = cudaMemsetAsync(d, 0, 32, ctx->stream);
    if (e == cudaSuccess)
    {
        int r = yg::gridBarrierCheck(reinterpret_cast<yg::GridBarrier*>(d), reinterpret_cast<uint32_t*>(d + 16), missing,
                                     pollLimit, ctx->smCount, ctx->stream, blocks);
        e = (cudaError_t)r;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, d, 32, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(d);
    if (e != cudaSuccess) return fail(YG_ERR_CUDA, std::string("barrier selftest: ") + cudaGetErrorString(e));
    *passes = h[4];
    *timedOut = h[2] != 0 ? 1u : 0u;
    return YG_OK;
}

YG_API int yg_server_stats_get(yg_server* s, yg_server_stats* out)
{
    if (!s || !out) return fail(YG_ERR_INVALID_ARGUMENT, "serve: null argument");
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
    out->bytes_in_use = s->bytesInUse;
    out->active = (uint32_t)s->active.size();
    out->queued = (uint32_t)s->queue.size();
    out->seconds = nowSince(s->t0);
    return YG_OK;
}

YG_API int yg_server_destroy(yg_server* s)
{
    if (!s) return YG_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        for (uint64_t id : s->queue) markDone(s, s->reqs[id].get(), YG_REQ_CANCELLED, 0, "server destroyed");
        s->queue.clear();
        for (uint64_t id : s->active) s->reqs[id]->cancelRequested = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto& kv : s->reqs)
        if (kv.second->film) cudaFreeAsync(kv.second->film, s->sA);
    if (s->sA) cudaStreamSynchronize(s->sA);
    if (s->sB) cudaStreamSynchronize(s->sB);
    if (s->graph) cudaGraphExecDestroy(s->graph);
    for (auto& kv : s->perms) cudaFree(kv.second);
    if (s->tablesDev) cudaFree(s->tablesDev);
    if (s->tablesHost) cudaFreeHost(s->tablesHost);
    if (s->sobolDev) cudaFree(s->sobolDev);
    if (s->sobolHost) cudaFreeHost(s->sobolHost);
    if (s->sobolDevB) cudaFree(s->sobolDevB);
    if (s->sobolHostB) cudaFreeHost(s->sobolHostB);
    if (s->waveArena) cudaFree(s->waveArena);
    if (s->barrier) cudaFree(s->barrier);
    if (s->barrierErrHost) cudaFreeHost(s->barrierErrHost);
    if (s->roundSamples) cudaFree(s->roundSamples);
    if (s->evA) cudaEventDestroy(s->evA);
    if (s->evB) cudaEventDestroy(s->evB);
    if (s->sA) cudaStreamDestroy(s->sA);
    if (s->sB) cudaStreamDestroy(s->sB);
    delete s;
    return YG_OK;
}

YG_API int64_t yg_server_plan(const yg_sched_item* items, uint32_t n, uint64_t budget, uint64_t inUse, uint32_t maxActive,
                              uint32_t waveCapacity, uint32_t roundSamples, uint32_t* admitOut, uint32_t* planesOut)
{
    if ((!items && n) || !admitOut || !planesOut) return fail(YG_ERR_INVALID_ARGUMENT, "plan: null argument");
    std::vector<PlanIn> in(n);
    for (uint32_t i = 0; i < n; ++i)
    {
        if (items[i].pixels == 0 || items[i].pixels > waveCapacity) return fail(YG_ERR_INVALID_ARGUMENT, "plan: bad pixel count");
        in[i] = {items[i].pixels, items[i].planes_left, items[i].admitted != 0, items[i].footprint_bytes, items[i].integrator,
                 items[i].rounds_waited};
    }
    std::vector<uint32_t> adm, planes;
    uint64_t total = planRound(in, budget, inUse, maxActive, waveCapacity, roundSamples, adm, planes);
    for (uint32_t i = 0; i < n; ++i)
    {
        admitOut[i] = adm[i];
        planesOut[i] = planes[i];
    }
    return (int64_t)total;
}

} // extern "C"
