// Host side of libdrmlt.so: scene upload, prepass orchestration, the chain
// iteration schedule and the C ABI declared in include/drmlt_capi.h.
#include "drmlt_capi.h"
#include "wave.cuh"
#include "persist.h"
#include "bvh.h"
#include "errors.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

using namespace drmlt;

namespace {
thread_local std::string g_error;
}  // namespace

int drmlt::set_error(int code, const char *msg) {
    g_error = msg;
    return code;
}

namespace {

int fail(int code, const std::string &msg) { return set_error(code, msg.c_str()); }

#define CK(call)                                                                                \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess)                                                                  \
            return fail(DRMLT_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));      \
    } while (0)

template <class T>
int dalloc(T **p, size_t n) {
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) return fail(DRMLT_E_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return DRMLT_OK;
}

// Lets the Gaussian kernels take their dynamic shared scratch (up to
// gauss_smem_bytes(kMaxDim), above the 48 KB default) on the current device.
int gauss_kernels_setup();

template <class T>
int upload(T **p, const T *src, size_t n) {
    int rc = dalloc(p, n);
    if (rc) return rc;
    if (n) CK(cudaMemcpy(*p, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return DRMLT_OK;
}

// PiecewiseConstant1D construction (src/distribution.h:9-25) in single precision.
void piecewise_constant(const std::vector<float> &f, std::vector<float> &cdf, float &funcInt) {
    const int n = int(f.size());
    cdf.assign(n + 1, 0.0f);
    for (int i = 1; i < n + 1; i++) cdf[i] = cdf[i - 1] + f[i - 1] / float(n);
    funcInt = cdf[n];
    if (funcInt == 0.0f) {
        for (int i = 1; i < n + 1; i++) cdf[i] = float(i) / float(n);
    } else {
        for (int i = 1; i < n + 1; i++) cdf[i] /= funcInt;
    }
}

// CreateEnvmapSampleInfo (src/envlight.cpp:24-71) in single precision, with
// the reference's accumulation order: per-row luminance CDFs over the columns,
// a row CDF weighted by sin(theta) of the row centre, and the normalisation of
// the sampled pdf. Returns false when the image has no finite positive weight.
bool envmap_sample_info(const float *rgb, int width, int height, std::vector<float> &cdfRows,
                        std::vector<float> &cdfCols, std::vector<float> &rowWeights, float &normalization,
                        float pixelSize[2]) {
    const float pi = 3.14159265358979323846f;
    cdfCols.assign(size_t(width + 1) * height, 0.0f);
    cdfRows.assign(height + 1, 0.0f);
    rowWeights.assign(height, 0.0f);
    size_t colPos = 0, rowPos = 0;
    float rowSum = 0.0f;
    cdfRows[rowPos++] = 0.0f;
    for (int y = 0; y < height; y++) {
        float colSum = 0.0f;
        cdfCols[colPos++] = 0.0f;
        for (int x = 0; x < width; x++) {
            const float *v = rgb + 3 * (size_t(y) * width + x);
            colSum += v[0] * 0.212671f + v[1] * 0.715160f + v[2] * 0.072169f;
            cdfCols[colPos++] = colSum;
        }
        const float norm = 1.0f / colSum;
        for (int x = 1; x < width; x++) cdfCols[colPos - x - 1] *= norm;
        cdfCols[colPos - 1] = 1.0f;
        const float weight = std::sin((float(y) + 0.5f) * pi / float(height));
        rowWeights[y] = weight;
        rowSum += colSum * weight;
        cdfRows[rowPos++] = rowSum;
    }
    const float norm = 1.0f / rowSum;
    for (int y = 1; y < height; y++) cdfRows[rowPos - y - 1] *= norm;
    cdfRows[rowPos - 1] = 1.0f;
    if (rowSum == 0.0f || !std::isfinite(rowSum)) return false;
    const float twoPi = 2.0f * pi;
    normalization = 1.0f / (rowSum * (twoPi / float(width)) * (pi / float(height)));
    pixelSize[0] = twoPi / float(width);
    pixelSize[1] = float(3.14159265358979323846 / double(height));
    return true;
}

struct Renderer {
    drmlt_options opt{};
    SceneView sv{};
    int N = 0;
    int W = 0, H = 0;
    std::vector<void *> owned;
    ChainView cv{};
    float b = 0.0f;
    bool prepassDone = false;
    bool directDone = false;
    long long samplesPerChain = 0, extraChains = 0;
    long long iterDone = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float lastRunMs = 0.0f;
    long long launches = 0;  // kernels launched by run() so far
    cudaGraphExec_t graph = nullptr;
    int *dIters = nullptr;  // per chain group: its current iteration
    // chain groups, each stepped on its own stream
    int G = 1, chunk = 0;
    int gaussGrid = 1, derivsGrid = 1, derivsAdjGrid = 1;  // blocks of the list-driven kernels (grid-stride over their lists)
    std::vector<cudaStream_t> gstreams;
    std::vector<cudaEvent_t> gevents;
    unsigned long long bootSeed = 0;
    // wavefront queues (wave.cuh): per chain its machine and y* record; per
    // queue slot (sliced per chain group) the chain, its ray and the answer
    WaveChain *waveChains = nullptr;
    PathRec *waveYstar = nullptr;
    int *waveQ[2] = {nullptr, nullptr};
    float4 *waveRayO[2] = {nullptr, nullptr}, *waveRayD[2] = {nullptr, nullptr};
    int *waveHit = nullptr;
    int *waveCount = nullptr;  // per group: 3 stage passes x kWaveCountStride
    // persistent schedule (persist.cu): queues, per-chain counters and the team
    // workers' derivative rows, allocated on its first run
    PersistBuffers pb{};
    bool pbReady = false;
    int persistGrid = 0, persistRegs = 0, numSms = 0;
    int lastTeamSms = 0;

    template <class T>
    int alloc(T **p, size_t n) {
        int rc = dalloc(p, n);
        if (!rc) owned.push_back(*p);
        return rc;
    }
    template <class T>
    int up(T **p, const T *src, size_t n) {
        int rc = upload(p, src, n);
        if (!rc) owned.push_back(*p);
        return rc;
    }
    ~Renderer() {
        if (hStats) cudaFreeHost(hStats);
        for (cudaEvent_t e : statsEv)
            if (e) cudaEventDestroy(e);
        if (graph) cudaGraphExecDestroy(graph);
        if (forkEv) cudaEventDestroy(forkEv);
        if (midEv) cudaEventDestroy(midEv);
        for (cudaStream_t s : gstreams) cudaStreamDestroy(s);
        for (cudaEvent_t e : gevents) cudaEventDestroy(e);
        for (void *p : owned) cudaFree(p);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }

    // all chains at once (prepass seeding)
    RunParams params() const {
        RunParams p;
        p.s = sv;
        p.d = cv;
        p.N = N;
        p.c0 = 0;
        p.samplesPerChain = samplesPerChain;
        p.extraChains = extraChains;
        p.b = b;
        p.sigma1 = opt.perturb_stddev;
        p.sigma2 = opt.aniso_perturb_stddev;
        p.largeProb = opt.large_step_prob;
        p.anisoProb = opt.aniso_perturb_prob;
        p.drType = opt.dr_type;
        p.integrator = opt.integrator;
        p.uniformMix = opt.uniform_mixing_prob;
        p.lensProb = opt.integrator == DRMLT_INTEGRATOR_H2MC ? opt.lens_perturb_prob : 0.0f;
        p.lensSigma = opt.lens_perturb_stddev;
        p.accMap = opt.acceptance_map;
        p.maxDerv = opt.max_derivative_depth;
        p.gaussDim = std::min(2 * opt.max_depth, kMaxDim);
        p.lanes = opt.stage_lanes > 0 ? std::min(opt.stage_lanes, 32) : 16;
        // the second-stage lists are compacted and short: fewer chains per warp,
        // more warps (config 2: 0.843 ms per iteration at 4 against 0.871 at 16)
        p.lanes2 = opt.stage2_lanes > 0 ? std::min(opt.stage2_lanes, 32) : std::min(p.lanes, 4);
        p.headChains = opt.head_chains > 0 ? opt.head_chains : 0;
        p.headLanes = opt.head_lanes > 0 ? std::min(opt.head_lanes, 32) : 2;
        p.iterp = dIters;
        p.derivWarps = opt.deriv_warps > 0 ? std::min(opt.deriv_warps, 4) : 2;
        p.adjMinDim = opt.adjoint_min_dim > 0 ? opt.adjoint_min_dim
                                              : (opt.adjoint_min_dim < 0 ? kNoAdjoint : kDefaultAdjMinDim);
        p.lists = 1;
        p.wave = opt.wavefront > 0 ? 1 : 0;
        p.waveRounds = std::min(std::min(opt.max_depth, kMaxLen) + 1, kWaveMaxRounds);
        p.seed = opt.seed;
        return p;
    }

    // Chain group g's queues for stage pass `stage` (1: stage 1, 2: stage 2, 3: y*).
    WaveView wave_view(int g, int stage) const {
        const RunParams p = params(g);
        WaveView w;
        w.chains = waveChains;
        w.ystar = waveYstar;
        for (int b = 0; b < 2; b++) {
            w.q[b] = waveQ[b] + p.c0;
            w.rayO[b] = waveRayO[b] + p.c0;
            w.rayD[b] = waveRayD[b] + p.c0;
        }
        w.hit = waveHit + p.c0;
        w.count = waveCount + size_t(kWaveCountStride) * (3 * g + stage - 1);
        w.cap = p.N;
        w.rounds = p.waveRounds;
        return w;
    }

    // chain group g: its chain range and its slices of the lists, counters and derivative rows
    RunParams params(int g) const {
        RunParams p = params();
        p.c0 = g * chunk;
        p.N = std::min(chunk, N - p.c0);
        p.d.listX += p.c0;
        p.d.listZ += p.c0;
        p.d.listS += p.c0;
        p.d.listA += p.c0;
        p.d.listL += p.c0;
        p.d.counters += kNumCounters * g;
        p.d.hist += size_t(kPlanBins) * g;
        p.d.order += p.c0;
        p.iterp = dIters + g;
        p.d.grad += size_t(p.c0) * kMaxDim;
        p.d.hess += size_t(p.c0) * kMaxDim * kMaxDim;
        return p;
    }

    int create(const drmlt_scene_desc *sd, const drmlt_options *o) {
        opt = *o;
        if (sd->num_tris <= 0 || sd->num_lights <= 0 || sd->width <= 0 || sd->height <= 0)
            return fail(DRMLT_E_ARG, "scene needs triangles, a light and a film size");
        if (opt.max_depth > kMaxLen || opt.max_depth < 3)
            return fail(DRMLT_E_ARG, "max_depth must be in [3, 12]");
        if (opt.num_chains <= 0) return fail(DRMLT_E_ARG, "num_chains must be positive");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
            return fail(DRMLT_E_CUDA, "no CUDA device available");
        CK(cudaSetDevice(opt.device));
        if (int rc = gauss_kernels_setup()) return rc;
        {
            // grids of the list-driven kernels: four times as many blocks as the GPU
            // holds at once (lists that long are rare; shorter lists keep one entry
            // per block, scheduled dynamically, without thousands of idle blocks)
            int sms = 0, perSm = 0;
            CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, opt.device));
            CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_gauss, 32 * kGaussTeamWarps,
                                                             gauss_smem_bytes(std::min(2 * opt.max_depth, kMaxDim))));
            gaussGrid = std::max(1, 4 * sms * std::max(perSm, 1));
            derivsGrid = std::max(1, 4 * sms * derivs_blocks_per_sm());
            derivsAdjGrid = std::max(1, 4 * sms * derivs_adj_blocks_per_sm());
        }
        if (opt.smem_carveout >= 0) {
            // one shared-memory carveout for every chain-loop kernel, so that
            // kernels of different stages can share an SM
            const int c = std::min(opt.smem_carveout, 100);
            CK(cudaFuncSetAttribute(k_reset_counters, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_plan, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_scatter, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_stage1, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(set_derivs_carveout(c));
            CK(cudaFuncSetAttribute(k_gauss, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_stage2, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_ystar, cudaFuncAttributePreferredSharedMemoryCarveout, c));
            CK(cudaFuncSetAttribute(k_finish, cudaFuncAttributePreferredSharedMemoryCarveout, c));
        }
        CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&ev0));
        CK(cudaEventCreate(&ev1));
        W = sd->width;
        H = sd->height;
        const int T = sd->num_tris;
        // triangles: p0, e1 = p1 - p0, e2 = p2 - p0 (single precision, as TriangleMesh)
        std::vector<float> triP(9 * size_t(T)), triN(9 * size_t(T));
        std::vector<int> triShape(T, -1);
        for (int t = 0; t < T; t++) {
            const float *v = sd->positions + 9 * size_t(t);
            for (int k = 0; k < 3; k++) {
                triP[9 * t + k] = v[k];
                triP[9 * t + 3 + k] = v[3 + k] - v[k];
                triP[9 * t + 6 + k] = v[6 + k] - v[k];
            }
            std::memcpy(&triN[9 * t], sd->normals + 9 * size_t(t), 9 * sizeof(float));
        }
        std::vector<Shape> shapes(sd->num_shapes);
        for (int s = 0; s < sd->num_shapes; s++) {
            shapes[s].bsdf = sd->shape_bsdf[s];
            shapes[s].areaLight = sd->shape_light[s];
            shapes[s].triOffset = sd->shape_first_tri[s];
            shapes[s].numTris = sd->shape_num_tris[s];
            if (shapes[s].bsdf < 0 || shapes[s].bsdf >= sd->num_bsdfs) return fail(DRMLT_E_ARG, "bad shape bsdf");
            for (int t = 0; t < shapes[s].numTris; t++) {
                const int g = shapes[s].triOffset + t;
                if (g < 0 || g >= T) return fail(DRMLT_E_ARG, "shape triangle range out of bounds");
                triShape[g] = s;
            }
        }
        for (int t = 0; t < T; t++)
            if (triShape[t] < 0) return fail(DRMLT_E_ARG, "triangle without shape");
        std::vector<Bsdf> bsdfs(sd->num_bsdfs);
        for (int i = 0; i < sd->num_bsdfs; i++) {
            const drmlt_bsdf &in = sd->bsdfs[i];
            Bsdf &b0 = bsdfs[i];
            std::memset(&b0, 0, sizeof(Bsdf));
            b0.type = in.type;
            b0.twoSided = in.two_sided;
            for (int k = 0; k < 3; k++) {
                b0.kd[k] = in.kd[k];
                b0.ks[k] = in.ks[k];
                b0.kt[k] = in.kt[k];
            }
            b0.exponent = in.exponent;
            // Phong::GetKsWeight (src/phong.cpp:158-167) on the constant textures
            const float ksAvg = in.ks[0] * 0.212671f + in.ks[1] * 0.715160f + in.ks[2] * 0.072169f;
            const float kdAvg = in.kd[0] * 0.212671f + in.kd[1] * 0.715160f + in.kd[2] * 0.072169f;
            const float sum = ksAvg + kdAvg;
            b0.ksWeight = in.type == DRMLT_BSDF_PHONG ? (sum <= 0.0f ? 0.0f : ksAvg / sum) : 0.0f;
            b0.intIOR = in.int_ior;
            b0.extIOR = in.ext_ior;
            b0.alpha = in.alpha;
            if (in.type == DRMLT_BSDF_ROUGHDIELECTRIC) {
                if (!(in.int_ior > 0.0f && in.ext_ior > 0.0f && in.alpha > 0.0f))
                    return fail(DRMLT_E_ARG, "roughdielectric needs positive IORs and alpha");
                b0.eta = in.int_ior / in.ext_ior;
                b0.invEta = 1.0f / b0.eta;
            }
        }
        // lights, light pick distribution and per-area-light triangle CDFs
        std::vector<Light> lights(sd->num_lights);
        std::vector<float> lightFunc(sd->num_lights), lightTriCdf;
        std::vector<float> envImg, envCdfRows, envCdfCols, envRowW;
        sv.envLight = -1;
        float weightSum = 0.0f;
        for (int i = 0; i < sd->num_lights; i++) {
            const drmlt_light &in = sd->lights[i];
            Light &L = lights[i];
            std::memset(&L, 0, sizeof(Light));
            L.type = in.type;
            L.shape = in.shape;
            for (int k = 0; k < 3; k++) {
                L.emission[k] = in.emission[k];
                L.pos[k] = in.pos[k];
            }
            L.samplingWeight = in.sampling_weight;
            lightFunc[i] = in.sampling_weight;
            weightSum += in.sampling_weight;
            if (in.type == DRMLT_LIGHT_AREA) {
                if (in.shape < 0 || in.shape >= sd->num_shapes) return fail(DRMLT_E_ARG, "area light shape");
                const Shape &sh = shapes[in.shape];
                // TriangleMesh::SetAreaLight (src/trianglemesh.cpp:298-311)
                std::vector<float> area(sh.numTris);
                float total = 0.0f;
                for (int t = 0; t < sh.numTris; t++) {
                    const float *P = &triP[9 * size_t(sh.triOffset + t)];
                    const float cx = P[4] * P[8] - P[5] * P[7];
                    const float cy = P[5] * P[6] - P[3] * P[8];
                    const float cz = P[3] * P[7] - P[4] * P[6];
                    area[t] = 0.5f * std::sqrt(cx * cx + cy * cy + cz * cz);
                    total += area[t];
                }
                std::vector<float> cdf;
                float fi;
                piecewise_constant(area, cdf, fi);
                L.triCdfOffset = int(lightTriCdf.size());
                L.numTris = sh.numTris;
                L.invTotalArea = 1.0f / total;
                lightTriCdf.insert(lightTriCdf.end(), cdf.begin(), cdf.end());
            } else if (in.type == DRMLT_LIGHT_ENV) {
                if (sv.envLight >= 0) return fail(DRMLT_E_ARG, "at most one environment light");
                if (!in.env_rgb || in.env_width < 1 || in.env_height < 1)
                    return fail(DRMLT_E_ARG, "environment light needs an image");
                const size_t npix = size_t(in.env_width) * in.env_height;
                envImg.assign(in.env_rgb, in.env_rgb + 3 * npix);
                if (!envmap_sample_info(envImg.data(), in.env_width, in.env_height, envCdfRows, envCdfCols,
                                        envRowW, sv.envNorm, sv.envPix))
                    return fail(DRMLT_E_ARG, "invalid environment map");
                // toWorld's upper-left 3x3 and, for toLight = Invert(toWorld), its inverse
                const float *m = in.to_world;
                const double a00 = m[0], a01 = m[1], a02 = m[2], a10 = m[4], a11 = m[5], a12 = m[6], a20 = m[8],
                             a21 = m[9], a22 = m[10];
                const double det = a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) +
                                   a02 * (a10 * a21 - a11 * a20);
                if (!(std::fabs(det) > 0.0)) return fail(DRMLT_E_ARG, "environment toWorld is singular");
                const double inv[9] = {(a11 * a22 - a12 * a21) / det, (a02 * a21 - a01 * a22) / det,
                                       (a01 * a12 - a02 * a11) / det, (a12 * a20 - a10 * a22) / det,
                                       (a00 * a22 - a02 * a20) / det, (a02 * a10 - a00 * a12) / det,
                                       (a10 * a21 - a11 * a20) / det, (a01 * a20 - a00 * a21) / det,
                                       (a00 * a11 - a01 * a10) / det};
                for (int r = 0; r < 3; r++)
                    for (int c = 0; c < 3; c++) {
                        sv.envToWorld[3 * r + c] = m[4 * r + c];
                        sv.envToLight[3 * r + c] = float(inv[3 * r + c]);
                    }
                sv.envLight = i;
                sv.envW = in.env_width;
                sv.envH = in.env_height;
            } else if (in.type != DRMLT_LIGHT_POINT) {
                return fail(DRMLT_E_ARG, "unknown light type");
            }
        }
        std::vector<float> lightCdf;
        float lightFuncInt;
        piecewise_constant(lightFunc, lightCdf, lightFuncInt);
        // BVH
        std::vector<BvhNode> nodes;
        std::vector<Tri> tris;
        BuildBvh(triP.data(), triShape.data(), T, nodes, tris);
        Tri *dTris;
        float *dTriN, *dTriP, *dLightCdf, *dLightFunc, *dLightTriCdf;
        int *dTriShape;
        BvhNode *dNodes;
        Shape *dShapes;
        Bsdf *dBsdfs;
        Light *dLights;
        int rc;
        if ((rc = up(&dTris, tris.data(), tris.size()))) return rc;
        if ((rc = up(&dTriN, triN.data(), triN.size()))) return rc;
        if ((rc = up(&dTriP, triP.data(), triP.size()))) return rc;
        if ((rc = up(&dTriShape, triShape.data(), triShape.size()))) return rc;
        if ((rc = up(&dNodes, nodes.data(), nodes.size()))) return rc;
        if ((rc = up(&dShapes, shapes.data(), shapes.size()))) return rc;
        if ((rc = up(&dBsdfs, bsdfs.data(), bsdfs.size()))) return rc;
        if ((rc = up(&dLights, lights.data(), lights.size()))) return rc;
        if ((rc = up(&dLightCdf, lightCdf.data(), lightCdf.size()))) return rc;
        if ((rc = up(&dLightFunc, lightFunc.data(), lightFunc.size()))) return rc;
        if ((rc = up(&dLightTriCdf, lightTriCdf.data(), lightTriCdf.size()))) return rc;
        if (sv.envLight >= 0) {
            float *dEnv[4];
            if ((rc = up(&dEnv[0], envImg.data(), envImg.size()))) return rc;
            if ((rc = up(&dEnv[1], envCdfRows.data(), envCdfRows.size()))) return rc;
            if ((rc = up(&dEnv[2], envCdfCols.data(), envCdfCols.size()))) return rc;
            if ((rc = up(&dEnv[3], envRowW.data(), envRowW.size()))) return rc;
            sv.envImg = dEnv[0];
            sv.envCdfRows = dEnv[1];
            sv.envCdfCols = dEnv[2];
            sv.envRowW = dEnv[3];
        }
        sv.tris = dTris;
        sv.triN = dTriN;
        sv.triP = dTriP;
        sv.triShape = dTriShape;
        sv.nodes = dNodes;
        sv.shapes = dShapes;
        sv.bsdfs = dBsdfs;
        sv.lights = dLights;
        sv.lightCdf = dLightCdf;
        sv.lightFunc = dLightFunc;
        sv.lightTriCdf = dLightTriCdf;
        sv.numLights = sd->num_lights;
        sv.numTris = T;
        sv.lightFuncInt = lightFuncInt;
        sv.lightWeightSum = weightSum;
        for (int k = 0; k < 3; k++) sv.bsCenter[k] = sd->bsphere_center[k];
        sv.bsRadius = sd->bsphere_radius;
        std::memcpy(sv.cam.sampleToCam, sd->sample_to_cam, 64);
        std::memcpy(sv.cam.camToSample, sd->cam_to_sample, 64);
        std::memcpy(sv.cam.camToWorld, sd->cam_to_world, 64);
        std::memcpy(sv.cam.worldToCam, sd->world_to_cam, 64);
        sv.cam.dist = sd->cam_dist;
        sv.cam.nearClip = sd->near_clip;
        sv.cam.farClip = sd->far_clip;
        sv.cam.width = W;
        sv.cam.height = H;
        sv.opt.roughnessThreshold = opt.roughness_threshold;
        sv.opt.useLightCoordinateSampling = opt.use_light_coordinate_sampling;
        sv.opt.discreteStdDev = opt.discrete_stddev;
        sv.opt.minDepth = opt.min_depth;
        sv.opt.maxDepth = opt.max_depth;
        // chain state
        N = opt.num_chains;
        if ((rc = alloc(&cv.slots, size_t(N) * 3))) return rc;
        if ((rc = alloc(&cv.gauss, size_t(N) * 3 * kGaussStride))) return rc;
        if ((rc = alloc(&cv.perm, size_t(N) * 3))) return rc;
        if ((rc = alloc(&cv.scr, size_t(N)))) return rc;
        if ((rc = alloc(&cv.listX, size_t(N)))) return rc;
        if ((rc = alloc(&cv.listZ, size_t(N)))) return rc;
        if ((rc = alloc(&cv.listS, size_t(N)))) return rc;
        if ((rc = alloc(&cv.listA, size_t(N)))) return rc;
        if ((rc = alloc(&cv.listL, size_t(N)))) return rc;
        graphIters = opt.graph_iters > 0 ? std::min(opt.graph_iters, 8) : 1;
        G = opt.chain_groups > 0 ? std::min(opt.chain_groups, 16) : 2;
        G = std::min(G, N);
        chunk = (N + G - 1) / G;
        G = (N + chunk - 1) / chunk;
        for (int g = 0; g < G; g++) {
            cudaStream_t s;
            cudaEvent_t e;
            CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
            gstreams.push_back(s);
            CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            gevents.push_back(e);
        }
        if ((rc = alloc(&waveChains, size_t(N)))) return rc;
        if ((rc = alloc(&waveYstar, size_t(N)))) return rc;
        for (int b = 0; b < 2; b++) {
            if ((rc = alloc(&waveQ[b], size_t(N)))) return rc;
            if ((rc = alloc(&waveRayO[b], size_t(N)))) return rc;
            if ((rc = alloc(&waveRayD[b], size_t(N)))) return rc;
        }
        if ((rc = alloc(&waveHit, size_t(N)))) return rc;

        if ((rc = alloc(&waveCount, size_t(3) * kWaveCountStride * G))) return rc;
        CK(cudaMemset(waveCount, 0, size_t(3) * kWaveCountStride * G * sizeof(int)));
        if ((rc = alloc(&cv.counters, kNumCounters * size_t(G)))) return rc;
        if ((rc = alloc(&cv.hist, size_t(kPlanBins) * G))) return rc;
        if ((rc = alloc(&dIters, size_t(G)))) return rc;
        if ((rc = alloc(&cv.order, size_t(N)))) return rc;
        if ((rc = alloc(&cv.grad, size_t(N) * kMaxDim))) return rc;
        if ((rc = alloc(&cv.hess, size_t(N) * kMaxDim * kMaxDim))) return rc;
        if ((rc = alloc(&cv.stats, kNumStatsAll))) return rc;
        if ((rc = alloc(&cv.film, size_t(W) * H))) return rc;
        if ((rc = alloc(&cv.direct, size_t(W) * H))) return rc;
        CK(cudaMemset(cv.stats, 0, kNumStatsAll * sizeof(unsigned long long)));
        CK(cudaMemset(cv.film, 0, size_t(W) * H * sizeof(float4)));
        CK(cudaMemset(cv.direct, 0, size_t(W) * H * sizeof(float4)));
        CK(cudaMemset(cv.counters, 0, kNumCounters * size_t(G) * sizeof(int)));
        // sample split of delayed.cpp:205-210, including its extra-sample rule
        const long long totalSamples = (long long)opt.spp * W * H;
        samplesPerChain = totalSamples / N;
        extraChains = samplesPerChain % N;
        bootSeed = opt.seed ^ 0x5EEDull;
        return DRMLT_OK;
    }

    int prepass(float *bOut) {
        if (graph) {  // its launch parameters carry the old normalisation
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        const int minDepth = std::max(opt.min_depth, 3);
        const int ns = opt.num_init_samples;
        if (ns <= 0) return fail(DRMLT_E_ARG, "num_init_samples must be positive");
        // Contribution records: 8 per bootstrap path first; the kernel counts every
        // contribution, so an overflowing pass is rerun once (same streams, same
        // records) with the exact count.
        long long cap = (long long)ns * 8;
        BootRecord *dRec = nullptr;
        int *dCount;
        int rc;
        int hc[2] = {0, 0};
        if ((rc = dalloc(&dCount, 2))) return rc;
        for (int attempt = 0; attempt < 2; attempt++) {
            if (cap > (1ll << 31) - 1) {
                cudaFree(dCount);
                return fail(DRMLT_E_OVERFLOW, "bootstrap contribution count exceeds 2^31");
            }
            if ((rc = dalloc(&dRec, size_t(cap)))) {
                cudaFree(dCount);
                return rc;
            }
            CK(cudaMemsetAsync(dCount, 0, 2 * sizeof(int), stream));
            k_bootstrap<<<(ns + 127) / 128, 128, 0, stream>>>(sv, bootSeed, ns, minDepth, opt.max_depth, dRec, dCount,
                                                              int(cap), dCount + 1);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(hc, dCount, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
            CK(cudaStreamSynchronize(stream));
            if (!hc[1]) break;
            cudaFree(dRec);
            dRec = nullptr;
            cap = (long long)(unsigned)hc[0] + 1;
        }
        if (hc[1]) {
            cudaFree(dCount);
            return fail(DRMLT_E_OVERFLOW, "bootstrap contribution buffer overflow");
        }
        std::vector<BootRecord> recs(hc[0]);
        if (hc[0]) CK(cudaMemcpy(recs.data(), dRec, size_t(hc[0]) * sizeof(BootRecord), cudaMemcpyDeviceToHost));
        cudaFree(dRec);
        cudaFree(dCount);
        if (recs.empty()) return fail(DRMLT_E_STATE, "bootstrap found no contributing path");
        // deterministic order: by sample, then technique
        std::sort(recs.begin(), recs.end(), [](const BootRecord &a, const BootRecord &c) {
            if (a.sample != c.sample) return a.sample < c.sample;
            if (a.c != c.c) return a.c < c.c;
            return a.l < c.l;
        });
        // totalScore, lengthContrib (delayed.cpp:97-117)
        double totalScore = 0.0;
        std::vector<float> lengthContrib;
        for (const BootRecord &r : recs) {
            totalScore += r.ls;
            const int len = r.c + r.l - 1;
            if (len >= int(lengthContrib.size())) lengthContrib.resize(len + 1, 0.0f);
            lengthContrib[len] += r.ls;
        }
        std::vector<float> lcdf;
        float lfi;
        piecewise_constant(lengthContrib, lcdf, lfi);
        float *dLcdf, *dLfunc;
        if ((rc = up(&dLcdf, lcdf.data(), lcdf.size()))) return rc;
        if ((rc = up(&dLfunc, lengthContrib.data(), lengthContrib.size()))) return rc;
        cv.lengthCdf = dLcdf;
        cv.lengthFunc = dLfunc;
        cv.lengthCount = int(lengthContrib.size());
        cv.lengthFuncInt = lfi;
        // equal-spaced seeding (delayed.cpp:125-167)
        std::vector<double> cdf(recs.size() + 1, 0.0);
        for (size_t i = 0; i < recs.size(); i++) cdf[i + 1] = cdf[i] + recs[i].ls;
        const double interval = cdf.back() / double(N);
        // offset in [0, interval) from a fixed hash of the record count
        unsigned long long h = 0x9E3779B97F4A7C15ull * (recs.size() + 1) ^ opt.seed;
        h ^= h >> 33;
        h *= 0xff51afd7ed558ccdull;
        h ^= h >> 33;
        double pos = double(h >> 11) * (1.0 / 9007199254740992.0) * interval;
        std::vector<int> sampleOf(N), techC(N), techL(N);
        size_t cdfPos = 0;
        for (int i = 0; i < N; i++) {
            while (pos > cdf[cdfPos]) cdfPos = std::min(cdfPos + 1, recs.size() - 1 + 1);
            const size_t ri = cdfPos == 0 ? 0 : cdfPos - 1;
            sampleOf[i] = recs[ri].sample;
            techC[i] = recs[ri].c;
            techL[i] = recs[ri].l;
            pos += interval;
        }
        int *dS, *dC, *dL;
        if ((rc = dalloc(&dS, N)) || (rc = dalloc(&dC, N)) || (rc = dalloc(&dL, N))) return rc;
        CK(cudaMemcpy(dS, sampleOf.data(), N * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dC, techC.data(), N * sizeof(int), cudaMemcpyHostToDevice));
        CK(cudaMemcpy(dL, techL.data(), N * sizeof(int), cudaMemcpyHostToDevice));
        b = float(totalScore) * (1.0f / float(ns));
        k_seed<<<(N + 127) / 128, 128, 0, stream>>>(params(), bootSeed, dS, dC, dL, minDepth, opt.max_depth);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream));
        cudaFree(dS);
        cudaFree(dC);
        cudaFree(dL);
        prepassDone = true;
        iterDone = 0;
        if (bOut) *bOut = b;
        return DRMLT_OK;
    }

    int direct() {
        if (opt.min_depth > 2 || opt.max_depth < 1 || opt.direct_spp <= 0) {
            directDone = true;
            return DRMLT_OK;
        }
        const long long n = (long long)W * H * opt.direct_spp;
        k_direct<<<unsigned((n + 127) / 128), 128, 0, stream>>>(sv, opt.seed, opt.direct_spp,
                                                                std::min(opt.min_depth, 2), std::min(opt.max_depth, 2),
                                                                cv.direct);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream));
        directDone = true;
        return DRMLT_OK;
    }

    // Stage k of iteration `iter` for chain group g on stream s:
    //   0 stage1 (counter reset, plan, order, stage-1 kernel), 1 derivatives at x,
    //   2 Gaussians at x and the H2MC offsets, 3 stage2, 4 derivatives at z, 5 Gaussians at z,
    //   6 finish (Green's y* trace, acceptance, splats, swap).
    // The list-driven kernels are sized for the whole group and exit past the
    // list's device-side length.
    static constexpr int kNumStagesRun = 7;
    int launch_stage(int k, int g, cudaStream_t s) const {
        const RunParams p = params(g);
        const int nb = (p.N + kStageBlock - 1) / kStageBlock;
        const int nbS = sparse_blocks(p.N, p.lanes);
        const int nbS1 = stage1_blocks(p.N, p.headChains, p.headLanes, p.lanes);
        const int nbS2 = sparse_blocks(p.N, p.lanes2);
        const int nbWarp = std::min((p.N * 32 * p.derivWarps + 127) / 128, derivsGrid);
        const int nbAdj = std::min((p.N * 32 + kAdjBlock - 1) / kAdjBlock, derivsAdjGrid);
        const int nDerivs = p.adjMinDim <= kMaxDim ? 2 : 1;
        const int nbG = std::min(p.N, gaussGrid);
        const size_t gsm = gauss_smem_bytes(p.gaussDim);
        const bool ystar = p.drType == 0 && p.integrator == 0;
        switch (k) {
            case 0: {
                k_reset_counters<<<1, 128, 0, s>>>(p.d.counters, p.d.hist,
                                                  waveCount + size_t(3) * kWaveCountStride * g,
                                                  p.wave ? 3 * kWaveCountStride : 0);
                k_plan<<<nb, kStageBlock, 0, s>>>(p);
                k_scatter<<<std::min((p.N + kScatterBlock - 1) / kScatterBlock, 64), kScatterBlock, 0, s>>>(p);
                const int nLens = p.lensProb > 0.0f ? 1 : 0;
                if (p.wave) {
                    const int n = 3 + launch_wave<1>(p, g, s);
                    if (nLens) k_lens<<<(p.N + kLensBlock - 1) / kLensBlock, kLensBlock, 0, s>>>(p);
                    return n + nLens;
                }
                k_stage1<<<nbS1, kStageBlock, 0, s>>>(p);
                if (nLens) k_lens<<<(p.N + kLensBlock - 1) / kLensBlock, kLensBlock, 0, s>>>(p);
                return 4 + nLens;
            }
            case 1: launch_derivs(p, 0, nbWarp, nbAdj, s); return nDerivs;
            case 2:
                k_gauss<<<nbG, 32 * kGaussTeamWarps, gsm, s>>>(p, 0);
                k_h2mc_offset<<<(p.N * 32 + 127) / 128, 128, 0, s>>>(p);
                return 2;
            case 3:
                if (p.wave) return launch_wave<2>(p, g, s);
                k_stage2<<<nbS2, kStageBlock, 0, s>>>(p);
                return 1;
            case 4: launch_derivs(p, 2, nbWarp, nbAdj, s); return nDerivs;
            case 5: k_gauss<<<nbG, 32 * kGaussTeamWarps, gsm, s>>>(p, 2); return 1;
            default: {
                int n = 2;
                if (ystar && p.wave) n += launch_wave<3>(p, g, s);
                if (ystar && !p.wave) {
                    k_ystar<<<nbS2, kStageBlock, 0, s>>>(p);
                    n += 1;
                }
                k_finish<<<nbS, kStageBlock, 0, s>>>(p);
                k_advance_iter<<<1, 1, 0, s>>>(dIters + g);
                return n;
            }
        }
    }
    // One wavefront stage pass of chain group g: the prologue kernel, then
    // waveRounds rounds of (traversal, machine steps). Returns the launches.
    template <int kStage>
    int launch_wave(const RunParams &p, int g, cudaStream_t s) const {
        const WaveView w = wave_view(g, kStage);
        const int nb = (p.N + kWaveBlock - 1) / kWaveBlock;
        k_wave_begin<kStage><<<nb, kWaveBlock, 0, s>>>(p, w);
        for (int r = 0; r < w.rounds; r++) {
            k_wave_trace<<<nb, kWaveBlock, 0, s>>>(p.s, w, r);
            k_wave_advance<kStage><<<nb, kWaveBlock, 0, s>>>(p, w, r);
        }
        return 1 + 2 * w.rounds;
    }
    // returns the number of kernels launched
    int launch_iteration(int g, cudaStream_t s) const {
        int n = 0;
        for (int k = 0; k < kNumStagesRun; k++) n += launch_stage(k, g, s);
        return n;
    }

    // The same iterations with CUDA events around each stage (on the launching
    // stream); accumulates per-stage milliseconds into ms[kNumStages].
    static constexpr int kNumStages = kNumStagesRun;
    int profile(long long iterations, float *ms, long long *done) {
        if (!prepassDone) return fail(DRMLT_E_STATE, "profile before prepass");
        const long long end = std::min(iterDone + iterations, total_iterations());
        cudaEvent_t ev[kNumStages + 1];
        for (int k = 0; k <= kNumStages; k++) CK(cudaEventCreate(&ev[k]));
        for (int k = 0; k < kNumStages; k++) ms[k] = 0.0f;
        long long mutations = 0;
        k_set_iters<<<1, 32, 0, stream>>>(dIters, G, int(iterDone));
        for (long long it = iterDone; it < end; it++) {
            // stage by stage over all groups on one stream, so each stage's
            // events bracket that stage for every chain
            cudaEventRecord(ev[0], stream);
            for (int k = 0; k < kNumStagesRun; k++) {
                for (int g = 0; g < G; g++) launch_stage(k, g, stream);
                cudaEventRecord(ev[k + 1], stream);
            }
            CK(cudaEventSynchronize(ev[kNumStages]));
            for (int k = 0; k < kNumStages; k++) {
                float t;
                cudaEventElapsedTime(&t, ev[k], ev[k + 1]);
                ms[k] += t;
            }
            mutations += (it < samplesPerChain) ? N : extraChains;
        }
        CK(cudaGetLastError());
        for (int k = 0; k <= kNumStages; k++) cudaEventDestroy(ev[k]);
        iterDone = end;
        if (done) *done = mutations;
        return DRMLT_OK;
    }

    // One iteration of every chain group as a CUDA graph: forked from the main
    // stream onto the group streams and joined back, replayed once per
    // iteration by run() (the kernels read the iteration from dIters, which the
    // graph advances). Built after the prepass, since the launch parameters
    // carry its normalisation b.
    long long graphLaunches = 0;
    cudaEvent_t forkEv = nullptr;
    cudaEvent_t midEv = nullptr;
    // Iterations per graph launch (drmlt_options.graph_iters, or 1 or 4 picked
    // by the autotuner). The chain
    // groups run free within a graph and join at its end: on config 4 joining
    // them every iteration costs 3% (5.67 against 5.48 ms per iteration), on
    // config 2 the join helps by 1% (0.815 against 0.823 ms).
    int graphIters = 1;
    int build_graph() {
        if (!forkEv) CK(cudaEventCreateWithFlags(&forkEv, cudaEventDisableTiming));
        CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        long long n = 0;
        cudaError_t e = cudaEventRecord(forkEv, stream);
        for (int g = 0; g < G && e == cudaSuccess; g++) {
            e = cudaStreamWaitEvent(gstreams[g], forkEv, 0);
            for (int k = 0; k < graphIters && e == cudaSuccess; k++) n += launch_iteration(g, gstreams[g]);
            if (e == cudaSuccess) e = cudaEventRecord(gevents[g], gstreams[g]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, gevents[g], 0);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        cudaGraph_t gr = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(stream, &gr);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return fail(DRMLT_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        const cudaError_t e3 = cudaGraphInstantiate(&graph, gr, 0);
        cudaGraphDestroy(gr);
        if (e3 != cudaSuccess) {
            graph = nullptr;
            return fail(DRMLT_E_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e3));
        }
        graphLaunches = n;
        return DRMLT_OK;
    }

    long long total_iterations() const { return samplesPerChain + (extraChains > 0 ? 1 : 0); }

    bool persistent_schedule() const { return opt.persistent > 0 && opt.integrator == DRMLT_INTEGRATOR_DRMLT; }
    size_t persist_smem() const { return gauss_smem_bytes(params().gaussDim); }

    int persist_setup() {
        if (pbReady) return DRMLT_OK;
        int dev = 0;
        CK(cudaGetDevice(&dev));
        CK(cudaDeviceGetAttribute(&numSms, cudaDevAttrMultiProcessorCount, dev));
        int coop = 0;
        CK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        if (!coop) return fail(DRMLT_E_CUDA, "the persistent schedule needs cooperative launches");
        const int occ = persist_blocks_per_sm(persist_smem(), &persistRegs);
        if (occ < 1) return fail(DRMLT_E_CUDA, "the persistent kernel does not fit on an SM");
        persistGrid = occ * numSms;
        int rc;
        if ((rc = alloc(reinterpret_cast<float4 **>(&pb.laneCells), size_t(N)))) return rc;
        if ((rc = alloc(reinterpret_cast<float4 **>(&pb.teamCells), size_t(N)))) return rc;
        if ((rc = alloc(&pb.ctl, size_t(8)))) return rc;
        if ((rc = alloc(&pb.status, size_t(1)))) return rc;
        if ((rc = alloc(&pb.chainIter, size_t(N)))) return rc;
        if ((rc = alloc(&pb.chainPhase, size_t(N)))) return rc;
        if ((rc = alloc(&pb.rows, size_t(persistGrid) * (kMaxDim + kMaxDim * kMaxDim)))) return rc;
        pb.ystar = waveYstar;
        pb.rowBlocks = persistGrid;
        pbReady = true;
        return DRMLT_OK;
    }

    // Iterations iterDone .. end of every chain in one persistent launch.
    int run_persistent(long long end, long long *done) {
        if (int rc = persist_setup()) return rc;
        const int teamSms = opt.team_sms > 0 ? std::min(opt.team_sms, numSms - 1) : std::max(1, numSms / 4);
        const long long waitLimit = opt.wait_limit > 0 ? opt.wait_limit : (1ll << 22);
        RunParams p = params();
        p.lists = 0;
        CK(cudaEventRecord(ev0, stream));
        const cudaError_t e = persist_run(p, pb, iterDone, end, persistGrid, teamSms, waitLimit, persist_smem(), stream);
        if (e != cudaSuccess) return fail(DRMLT_E_CUDA, std::string("persistent launch: ") + cudaGetErrorString(e));
        CK(cudaEventRecord(ev1, stream));
        CK(cudaEventSynchronize(ev1));
        CK(cudaEventElapsedTime(&lastRunMs, ev0, ev1));
        launches += 2;
        lastTeamSms = teamSms;
        int status = 0;
        CK(cudaMemcpy(&status, pb.status, sizeof(int), cudaMemcpyDeviceToHost));
        if (status)
            return fail(DRMLT_E_TIMEOUT, "persistent schedule: a device wait gave up (status " + std::to_string(status) +
                                             "); the chain state is undefined");
        long long mutations = 0;
        for (long long it = iterDone; it < end; it++) mutations += (it < samplesPerChain) ? N : extraChains;
        iterDone = end;
        if (done) *done = mutations;
        return DRMLT_OK;
    }

    int run(long long iterations, long long *done) {
        if (!prepassDone) return fail(DRMLT_E_STATE, "run before prepass");
        const long long end = std::min(iterDone + iterations, total_iterations());
        if (persistent_schedule()) return run_persistent(end, done);
        long long mutations = 0;
        if (opt.use_graph && !graph) {
            if (int rc = build_graph()) return rc;
        }
        k_set_iters<<<1, 32, 0, stream>>>(dIters, G, int(iterDone));
        CK(cudaEventRecord(ev0, stream));
        if (int rc = enqueue(end, mutations)) return rc;
        CK(cudaEventRecord(ev1, stream));
        CK(cudaGetLastError());
        CK(cudaEventSynchronize(ev1));
        CK(cudaEventElapsedTime(&lastRunMs, ev0, ev1));
        iterDone = end;
        if (done) *done = mutations;
        return DRMLT_OK;
    }

    // Pipelined stepping (drmlt_run_async / drmlt_wait_stats): the iterations
    // and a copy of the statistics counters into pinned slot `slot`, enqueued
    // on the handle's stream without a host wait. The persistent schedule
    // (one cooperative launch that the host waits on) is not offered here.
    unsigned long long *hStats = nullptr;  // 2 pinned slots of kNumStatsAll counters
    cudaEvent_t statsEv[2] = {nullptr, nullptr};
    int run_async(long long iterations, int slot, long long *done) {
        if (!prepassDone) return fail(DRMLT_E_STATE, "run before prepass");
        if (slot < 0 || slot > 1) return fail(DRMLT_E_ARG, "slot must be 0 or 1");
        if (persistent_schedule()) return fail(DRMLT_E_STATE, "the persistent schedule has no pipelined run");
        if (!hStats) {
            CK(cudaMallocHost(&hStats, 2 * kNumStatsAll * sizeof(unsigned long long)));
            for (int k = 0; k < 2; k++) CK(cudaEventCreateWithFlags(&statsEv[k], cudaEventDisableTiming));
        }
        const long long end = std::min(iterDone + iterations, total_iterations());
        long long mutations = 0;
        if (opt.use_graph && !graph) {
            if (int rc = build_graph()) return rc;
        }
        k_set_iters<<<1, 32, 0, stream>>>(dIters, G, int(iterDone));
        if (int rc = enqueue(end, mutations)) return rc;
        CK(cudaMemcpyAsync(hStats + slot * kNumStatsAll, cv.stats, kNumStatsAll * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost, stream));
        CK(cudaEventRecord(statsEv[slot], stream));
        CK(cudaGetLastError());
        iterDone = end;
        if (done) *done = mutations;
        return DRMLT_OK;
    }
    int wait_stats(int slot, unsigned long long *h) {
        if (slot < 0 || slot > 1 || !hStats) return fail(DRMLT_E_STATE, "no pipelined run in this slot");
        CK(cudaEventSynchronize(statsEv[slot]));
        std::memcpy(h, hStats + slot * kNumStatsAll, kNumStatsAll * sizeof(unsigned long long));
        return DRMLT_OK;
    }

    // The chain-loop launches from iteration iterDone up to `end` on the
    // handle's stream (graph replays, then per-stage launches on the group
    // streams for iterations short of a whole graph), joined back into it.
    int enqueue(long long end, long long &mutations) {
        long long it = iterDone;
        if (graph) {
            for (; it + graphIters <= end; it += graphIters) {
                CK(cudaGraphLaunch(graph, stream));
                launches += graphLaunches;
                for (int k = 0; k < graphIters; k++) mutations += (it + k < samplesPerChain) ? N : extraChains;
            }
        }
        if (it < end) {  // without graphs, or the last iterations short of a graph's
            if (!midEv) CK(cudaEventCreateWithFlags(&midEv, cudaEventDisableTiming));
            CK(cudaEventRecord(midEv, stream));
            for (int g = 0; g < G; g++) CK(cudaStreamWaitEvent(gstreams[g], midEv, 0));
            for (; it < end; it++) {
                for (int g = 0; g < G; g++) launches += launch_iteration(g, gstreams[g]);
                mutations += (it < samplesPerChain) ? N : extraChains;
            }
            for (int g = 0; g < G; g++) {
                CK(cudaEventRecord(gevents[g], gstreams[g]));
                CK(cudaStreamWaitEvent(stream, gevents[g], 0));
            }
        }
        return DRMLT_OK;
    }

    // Launch-shape autotuner: after `per` untimed iterations (past the first
    // iterations' transient), times `per` real iterations under each candidate
    // in two passes of opposite order (so that a drift of the iteration cost
    // over the render cancels) and keeps the fastest: the number of chains per warp in the
    // per-chain stage kernels, then the number of warps sharing one chain's
    // derivatives, then the stage-1 head tier (none, or the longest half of the
    // chains at half as many per warp, the rest at the tuned count or twice it),
    // then (graphs on, `per` a multiple of 4) the number of
    // iterations per graph launch. The iterations are part of the render:
    // the launch shape never changes which steps the chains take. Stops early
    // when the render runs out of iterations.
    int autotune(int per, int *lanesOut, int *warpsOut) {
        if (!prepassDone) return fail(DRMLT_E_STATE, "autotune before prepass");
        if (per < 1) return fail(DRMLT_E_ARG, "autotune needs at least one iteration per candidate");
        static const int kLanes[] = {2, 4, 8, 16, 32};
        static const int kWarps[] = {1, 2, 4};
        int bestL = params().lanes, bestW = params().derivWarps;
        bool out = false;  // ran out of iterations
        auto trial = [&](int lanes, int warps, float &ms) -> int {
            if (total_iterations() - iterDone < per) {
                out = true;
                return DRMLT_OK;
            }
            opt.stage_lanes = lanes;
            opt.deriv_warps = warps;
            if (graph) {
                cudaGraphExecDestroy(graph);
                graph = nullptr;
            }
            if (int rc = run(per, nullptr)) return rc;
            ms += lastRunMs;
            return DRMLT_OK;
        };
        float warm = 0.0f;
        if (int rc = trial(bestL, bestW, warm)) return rc;
        // chains per warp
        float tl[5] = {0, 0, 0, 0, 0};
        for (int pass = 0; pass < 2 && !out; pass++)
            for (int k = 0; k < 5 && !out; k++) {
                const int i = pass == 0 ? k : 4 - k;
                if (int rc = trial(kLanes[i], bestW, tl[i])) return rc;
            }
        if (!out) {
            int bi = 0;
            for (int i = 1; i < 5; i++)
                if (tl[i] < tl[bi]) bi = i;
            bestL = kLanes[bi];
        }
        // derivative warps
        float tw[3] = {0, 0, 0};
        for (int pass = 0; pass < 2 && !out; pass++)
            for (int k = 0; k < 3 && !out; k++) {
                const int i = pass == 0 ? k : 2 - k;
                if (int rc = trial(bestL, kWarps[i], tw[i])) return rc;
            }
        if (!out) {
            int bi = 0;
            for (int i = 1; i < 3; i++)
                if (tw[i] < tw[bi]) bi = i;
            bestW = kWarps[bi];
        }
        // two-tier stage 1: no head tier; the longest half of each group's
        // chains at half the chains per warp; the same with twice the chains
        // per warp for the shorter half (config 4: 4.21, 4.21, 4.02 ms per
        // iteration at 16 chains per warp)
        {
            const int hl = std::max(1, bestL / 2);
            const int heads[3] = {0, chunk / 2, chunk / 2};
            const int tails[3] = {bestL, bestL, std::min(32, 2 * bestL)};
            float th[3] = {0, 0, 0};
            for (int pass = 0; pass < 2 && !out; pass++)
                for (int k = 0; k < 3 && !out; k++) {
                    const int i = pass == 0 ? k : 2 - k;
                    opt.head_chains = heads[i];
                    opt.head_lanes = hl;
                    if (int rc = trial(tails[i], bestW, th[i])) return rc;
                }
            int bi = 0;
            if (!out)
                for (int i = 1; i < 3; i++)
                    if (th[i] < th[bi]) bi = i;
            opt.head_chains = heads[bi];
            opt.head_lanes = hl;
            bestL = tails[bi];
        }
        // iterations per graph launch
        if (opt.use_graph && per % 4 == 0) {
            static const int kIters[] = {1, 4};
            float tg[2] = {0, 0};
            for (int pass = 0; pass < 2 && !out; pass++)
                for (int k = 0; k < 2 && !out; k++) {
                    const int i = pass == 0 ? k : 1 - k;
                    graphIters = kIters[i];
                    if (int rc = trial(bestL, bestW, tg[i])) return rc;
                }
            // graphs of 4 only when clearly faster: on config 4 at the two-tier
            // shape they measured 3% slower, and two passes of `per` iterations
            // differ by a few percent from run to run
            graphIters = (!out && tg[1] < 0.97f * tg[0]) ? 4 : 1;
        }
        opt.stage_lanes = bestL;
        opt.deriv_warps = bestW;
        if (graph) {
            cudaGraphExecDestroy(graph);
            graph = nullptr;
        }
        if (lanesOut) *lanesOut = bestL;
        if (warpsOut) *warpsOut = bestW;
        return DRMLT_OK;
    }

    // The device films hold float4 pixels (RGB + an unused lane); the host film is RGB.
    // The final image: MergeBuffer (src/image.h:76-93, delayed.cpp:681-685) of
    // the direct and indirect films on the device, then one copy of the RGB
    // floats to the caller (12 bytes a pixel instead of two float4 films).
    float *dRgb = nullptr;
    int film(float *rgb) {
        const size_t n = size_t(W) * H;
        if (!dRgb) {
            if (int rc = alloc(&dRgb, 3 * n)) return rc;
        }
        const float dw = opt.direct_spp > 0 ? 1.0f / float(opt.direct_spp) : 0.0f;
        const float iw = opt.spp > 0 ? 1.0f / float(opt.spp) : 0.0f;
        k_merge_film<<<unsigned((n + 255) / 256), 256, 0, stream>>>(cv.film, cv.direct, dw, iw, n, dRgb);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(rgb, dRgb, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, stream));
        CK(cudaStreamSynchronize(stream));
        return DRMLT_OK;
    }

    int partial_film(float *rgb) {
        const size_t n = size_t(W) * H;
        std::vector<float4> ind(n);
        unsigned long long h[kNumStats];
        CK(cudaMemcpy(ind.data(), cv.film, n * sizeof(float4), cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(h, cv.stats, sizeof(h), cudaMemcpyDeviceToHost));
        const unsigned long long work = h[kStatMutations];
        const float factor = work > 0 ? float(double(W) * double(H) / double(work)) : 0.0f;
        for (size_t i = 0; i < n; i++) {
            rgb[3 * i + 0] = factor * ind[i].x;
            rgb[3 * i + 1] = factor * ind[i].y;
            rgb[3 * i + 2] = factor * ind[i].z;
        }
        return DRMLT_OK;
    }
};

}  // namespace

// ============================================================================ C ABI
extern "C" {

void drmlt_default_options(drmlt_options *o) {
    std::memset(o, 0, sizeof(*o));
    o->integrator = DRMLT_INTEGRATOR_DRMLT;
    o->dr_type = DRMLT_DR_GREEN;
    o->aniso_perturb_prob = 0.5f;
    o->aniso_perturb_stddev = 0.0025f;
    o->acceptance_map = 0;
    o->perturb_stddev = 0.01f;
    o->large_step_prob = 0.3f;
    o->roughness_threshold = 0.03f;
    o->discrete_stddev = 0.01f;
    o->uniform_mixing_prob = 0.2f;
    o->num_chains = 1024;
    o->num_init_samples = 100000;
    o->spp = 16;
    o->direct_spp = 16;
    o->min_depth = -1;
    o->max_depth = -1;
    o->seed_offset = 0;
    o->use_light_coordinate_sampling = 1;
    o->max_derivative_depth = 9;
    o->seed = 0x1234ABCDull;
    o->device = 0;
    o->use_graph = 1;
    o->chain_groups = 0;
    o->stage_lanes = 0;
    o->deriv_warps = 0;
    o->autotune = 1;
    o->smem_carveout = -1;
    o->stage2_lanes = 0;
    o->graph_iters = 0;
    o->wavefront = -1;
    o->adjoint_min_dim = 0;
    o->lens_perturb_prob = 0.3f;
    o->lens_perturb_stddev = 0.01f;
}

const char *drmlt_last_error(void) { return g_error.c_str(); }

int drmlt_create(const drmlt_scene_desc *scene, const drmlt_options *opt, void **handle) {
    if (!scene || !opt || !handle) return fail(DRMLT_E_ARG, "null argument");
    Renderer *r = new Renderer();
    const int rc = r->create(scene, opt);
    if (rc) {
        delete r;
        return rc;
    }
    *handle = r;
    return DRMLT_OK;
}

int drmlt_destroy(void *handle) {
    delete static_cast<Renderer *>(handle);
    return DRMLT_OK;
}

int drmlt_prepass(void *handle, float *b_out) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    return static_cast<Renderer *>(handle)->prepass(b_out);
}

int drmlt_direct(void *handle) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    return static_cast<Renderer *>(handle)->direct();
}

int drmlt_run(void *handle, int64_t iterations, int64_t *done) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    long long d = 0;
    const int rc = static_cast<Renderer *>(handle)->run(iterations, &d);
    if (done) *done = d;
    return rc;
}

int drmlt_run_async(void *handle, int64_t iterations, int slot, int64_t *done) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    long long d = 0;
    const int rc = static_cast<Renderer *>(handle)->run_async(iterations, slot, &d);
    if (done) *done = d;
    return rc;
}

int drmlt_render(void *handle) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    Renderer *r = static_cast<Renderer *>(handle);
    int rc = r->direct();
    if (rc) return rc;
    rc = r->prepass(nullptr);
    if (rc) return rc;
    // autotune on renders long enough that its 17 runs of 8 iterations are a small part
    if (r->opt.autotune && r->total_iterations() >= 1024) {
        rc = r->autotune(8, nullptr, nullptr);
        if (rc) return rc;
    }
    return r->run(r->total_iterations() - r->iterDone, nullptr);
}

int drmlt_autotune(void *handle, int iterations_per_candidate, int *stage_lanes, int *deriv_warps) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    return static_cast<Renderer *>(handle)->autotune(iterations_per_candidate, stage_lanes, deriv_warps);
}

int drmlt_get_launch_shape(void *handle, int *stage_lanes, int *stage2_lanes, int *deriv_warps, int *graph_iters) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    const Renderer *r = static_cast<const Renderer *>(handle);
    const RunParams p = r->params();
    if (stage_lanes) *stage_lanes = p.lanes;
    if (stage2_lanes) *stage2_lanes = p.lanes2;
    if (deriv_warps) *deriv_warps = p.derivWarps;
    if (graph_iters) *graph_iters = r->opt.use_graph ? r->graphIters : 0;
    return DRMLT_OK;
}

int drmlt_get_head_tier(void *handle, int *head_chains, int *head_lanes) {
    if (!handle) return fail(DRMLT_E_ARG, "null handle");
    const RunParams p = static_cast<const Renderer *>(handle)->params();
    if (head_chains) *head_chains = p.headChains;
    if (head_lanes) *head_lanes = p.headLanes;
    return DRMLT_OK;
}

int drmlt_get_adjoint_min_dim(void *handle, int *adjoint_min_dim) {
    if (!handle || !adjoint_min_dim) return fail(DRMLT_E_ARG, "null argument");
    const int a = static_cast<const Renderer *>(handle)->params().adjMinDim;
    *adjoint_min_dim = a > kMaxDim ? -1 : a;
    return DRMLT_OK;
}

int drmlt_get_wavefront(void *handle, int *wavefront) {
    if (!handle || !wavefront) return fail(DRMLT_E_ARG, "null argument");
    *wavefront = static_cast<const Renderer *>(handle)->params().wave;
    return DRMLT_OK;
}

int drmlt_get_film(void *handle, float *rgb) {
    if (!handle || !rgb) return fail(DRMLT_E_ARG, "null argument");
    return static_cast<Renderer *>(handle)->film(rgb);
}

int drmlt_get_partial_film(void *handle, float *rgb) {
    if (!handle || !rgb) return fail(DRMLT_E_ARG, "null argument");
    return static_cast<Renderer *>(handle)->partial_film(rgb);
}

static void stats_from_counters(const unsigned long long *h, drmlt_stats *st) {
    st->large_step = h[kStatLarge];
    st->large_step_accepted = h[kStatLargeAcc];
    st->stage1 = h[kStatStage1];
    st->stage1_accepted = h[kStatStage1Acc];
    st->stage2_iso = h[kStatIso];
    st->stage2_iso_accepted = h[kStatIsoAcc];
    st->stage2_h2mc = h[kStatH2mc];
    st->stage2_h2mc_accepted = h[kStatH2mcAcc];
    st->mutations = h[kStatMutations];
    st->gaussians = h[kStatGauss];
    st->gaussians_fp64_fallback = h[kStatGaussFallback];
    st->lens = h[kStatLens];
    st->lens_accepted = h[kStatLensAcc];
}

int drmlt_get_stats(void *handle, drmlt_stats *st) {
    if (!handle || !st) return fail(DRMLT_E_ARG, "null argument");
    Renderer *r = static_cast<Renderer *>(handle);
    unsigned long long h[kNumStatsAll];
    CK(cudaMemcpy(h, r->cv.stats, sizeof(h), cudaMemcpyDeviceToHost));
    stats_from_counters(h, st);
    return DRMLT_OK;
}

int drmlt_wait_stats(void *handle, int slot, drmlt_stats *st) {
    if (!handle || !st) return fail(DRMLT_E_ARG, "null argument");
    unsigned long long h[kNumStatsAll];
    if (int rc = static_cast<Renderer *>(handle)->wait_stats(slot, h)) return rc;
    stats_from_counters(h, st);
    return DRMLT_OK;
}

int drmlt_profile(void *handle, int64_t iterations, float *stage_ms, int64_t *done) {
    if (!handle || !stage_ms) return fail(DRMLT_E_ARG, "null argument");
    long long d = 0;
    const int rc = static_cast<Renderer *>(handle)->profile(iterations, stage_ms, &d);
    if (done) *done = d;
    return rc;
}

int drmlt_total_iterations(void *handle, int64_t *iterations) {
    if (!handle || !iterations) return fail(DRMLT_E_ARG, "null argument");
    *iterations = static_cast<Renderer *>(handle)->total_iterations();
    return DRMLT_OK;
}

int drmlt_kernel_launches(void *handle, int64_t *n) {
    if (!handle || !n) return fail(DRMLT_E_ARG, "null argument");
    *n = static_cast<Renderer *>(handle)->launches;
    return DRMLT_OK;
}

int drmlt_last_run_ms(void *handle, float *ms) {
    if (!handle || !ms) return fail(DRMLT_E_ARG, "null argument");
    *ms = static_cast<Renderer *>(handle)->lastRunMs;
    return DRMLT_OK;
}

}  // extern "C"

#include "parity.cuh"

namespace {
int gauss_kernels_setup() {
    const int bytes = int(gauss_smem_bytes(kMaxDim));
    CK(cudaFuncSetAttribute(k_gauss, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    CK(cudaFuncSetAttribute(k_gauss_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    return DRMLT_OK;
}
}  // namespace

// ============================================================================ no-allocation entry point
// Scratch for drmlt_compute_gaussian_noalloc: the FP64 eigen-basis store of up
// to kNoAllocMaxGaussians Gaussians (kGaussStride doubles each, 1.29 MB). It is
// a file-scope device array, so every GPU that loads libdrmlt.so holds it until
// the process exits, and it needs no cudaMalloc.
namespace {
constexpr int kNoAllocMaxGaussians = 256;
__device__ __align__(256) double g_noallocGaussStore[size_t(kNoAllocMaxGaussians) * kGaussStride];

// Device address of g_noallocGaussStore, looked up once per device. In host
// code the symbol name is only a host-side stand-in, never a device address.
// The lookup is guarded by a mutex, so host threads whose first calls on a
// device overlap do not race on it.
constexpr int kNoAllocMaxDevices = 64;
double *g_noallocStorePtr[kNoAllocMaxDevices] = {nullptr};
std::mutex g_noallocSetupMutex;
}  // namespace

extern "C" int drmlt_compute_gaussian_noalloc(int n, const int32_t *dims, const float *ss, const float *grad,
                                              const float *hess, float sigma, double *mean, double *inv_cov,
                                              double *cov, double *log_det, void *stream) {
    if (n < 0) return fail(DRMLT_E_ARG, "n must be non-negative");
    if (n > kNoAllocMaxGaussians)
        return fail(DRMLT_E_ARG, "drmlt_compute_gaussian_noalloc: n = " + std::to_string(n) +
                                     " exceeds the fixed scratch capacity of " +
                                     std::to_string(kNoAllocMaxGaussians) + " Gaussians per call");
    if (n == 0) return DRMLT_OK;
    if (!dims || !ss || !grad || !hess || !mean || !inv_cov || !cov || !log_det)
        return fail(DRMLT_E_ARG, "null device pointer");
    if (!(sigma > 0.0f)) return fail(DRMLT_E_ARG, "sigma must be positive");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(DRMLT_E_ARG, "device ordinal out of range");
    double *store = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noallocSetupMutex);
        if (g_noallocStorePtr[dev] == nullptr) {
            // set-up on this device's first call (the device is current here)
            int rc = gauss_kernels_setup();
            if (rc) return rc;
            double *p = nullptr;
            CK(cudaGetSymbolAddress((void **)&p, g_noallocGaussStore));
            g_noallocStorePtr[dev] = p;
        }
        store = g_noallocStorePtr[dev];
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // entries past each Gaussian's dimension are zero, as in drmlt_compute_gaussian
    CK(cudaMemsetAsync(mean, 0, size_t(n) * kMaxDim * sizeof(double), st));
    CK(cudaMemsetAsync(inv_cov, 0, size_t(n) * kMaxDim * kMaxDim * sizeof(double), st));
    CK(cudaMemsetAsync(cov, 0, size_t(n) * kMaxDim * kMaxDim * sizeof(double), st));
    // dims are device data here: scratch is sized for kMaxDim, and an odd or
    // out-of-range dimension yields zero outputs and a NaN log-determinant
    k_gauss_batch<<<n, 32 * kGaussTeamWarps, gauss_smem_bytes(kMaxDim), st>>>(
        dims, ss, grad, hess, n, sigma, kMaxDim, store, mean, inv_cov, cov, log_det);
    CK(cudaGetLastError());
    return DRMLT_OK;
}
