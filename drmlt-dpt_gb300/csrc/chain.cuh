// Chain state of the DRMLT loop in device memory and the launch parameters
// shared by every chain-loop kernel (kernels.cuh, derivs.cu).
//
// Chain states live in HBM as three slots per chain (current, first proposal,
// second proposal) addressed through a per-chain permutation, so accepting a
// proposal swaps two indices instead of copying a state.
#pragma once
#include "pathad.cuh"
#include "gauss.cuh"

namespace drmlt {

// MarkovState (src/mutation.h:38-59): path, its contribution and one
// toSplat entry (screen, rgb value = contrib * b / ls).
struct Slot {
    PathRec rec;
    float screen[2];
    float rgb[3];
    float ls, ss;
    float splat[5];
    int hasSplat;
    int valid;
    int gaussInit;
};

enum : int {
    kActive = 1, kAccept1 = 2, kLarge = 4, kSecond = 8, kAniso = 16, kZValid = 32, kAccept2 = 64,
    kSingle = 128,  // integrator=h2mc: the anisotropic proposal is the only stage
    kLens = 256     // integrator=h2mc: a lens-mutation candidate (k_lens)
};

struct Scratch {
    float a1, a2;
    int flags;
    int key, rank;      // stage-1 work class and rank within it (k_plan)
    float aStar;        // Green's reverse first-stage acceptance (k_ystar)
    double logRatio;    // H2MC: log N_z(-o) - log N_x(o) (k_gauss at z)
    float offset[kMaxDim];
};

// byte sizes that the throughput accounting (bench.py) assumes
static_assert(sizeof(Slot) == 328, "Slot layout");
static_assert(sizeof(Scratch) == 128, "Scratch layout");

// Stage-1 work classes: 0 idle chain; 1 + 16 (c + l) + c small step of
// technique (c, l); 256 + 16 L + lgtLength large step of sampled length L.
// Higher classes are longer work; k_scatter orders the chains by descending
// class, so the longest traces start first and the short ones fill the tail.
constexpr int kPlanBins = 512;

enum : int {
    kStatLarge = 0, kStatLargeAcc, kStatStage1, kStatStage1Acc, kStatIso, kStatIsoAcc, kStatH2mc,
    kStatH2mcAcc, kStatMutations, kStatGauss, kStatGaussFallback, kNumStats
};
// Counters outside the per-thread StatAcc (added with single atomics where the
// rare event happens): integrator=h2mc's lens mutations and their acceptances.
enum : int { kStatLens = kNumStats, kStatLensAcc, kNumStatsAll };

// Work-list lengths per chain group: [0] listX, [1] listZ, [2] listS, [3] listA, [4] listL.
constexpr int kNumCounters = 8;

struct ChainView {
    Slot *slots;        // N x 3
    double *gauss;      // N x 3 x kGaussStride
    int *perm;          // N x 3: slot of (current, first, second)
    Scratch *scr;       // N
    int *listX;         // chains needing a Gaussian at the current state
    int *listZ;         // chains needing a Gaussian at the second proposal
    int *listS;         // chains taking a second stage this iteration
    int *listA;         // chains taking the anisotropic (H2MC) second stage
    int *listL;         // integrator=h2mc: chains drawn for the lens mutation
    int *order;         // stage-1 processing order (chains grouped by work class)
    int *hist;          // kPlanBins counters of the work classes
    int *counters;      // [0] = |listX|, [1] = |listZ|, [2] = |listS|, [3] = |listA|, [4] = |listL|
    float *grad;        // N x kMaxDim (indexed by list position)
    float *hess;        // N x kMaxDim^2
    unsigned long long *stats;
    float4 *film;       // W x H (indirect), RGB + unused
    float4 *direct;     // W x H
    const float *lengthCdf;
    const float *lengthFunc;
    int lengthCount;
    float lengthFuncInt;
};

// One launch covers one chain group: chains c0 .. c0 + N - 1. The lists,
// counters and gradient/Hessian rows in `d` are the group's own slices.
struct RunParams {
    SceneView s;
    ChainView d;
    int N;
    int c0;
    long long samplesPerChain;
    long long extraChains;
    float b;
    float sigma1, sigma2;
    float largeProb, anisoProb;
    int drType;          // 0 green, 1 mira
    int integrator;      // 0 drmlt, 1 h2mc, 2 mcmc
    float uniformMix;
    float lensProb;      // integrator=h2mc: lensPerturbProb
    float lensSigma;     // integrator=h2mc: lensPerturbStdDev
    int accMap;
    int maxDerv;
    int gaussDim;        // largest path dimension (2 max_depth): sizes the Gaussian scratch
    int lanes;           // chains per warp in the per-chain stage kernels (1..32)
    int lanes2;          // chains per warp in the second-stage list kernels (1..32)
    int headChains;      // k_stage1: the first headChains chains of the stage-1 order (the
    int headLanes;       // longest work classes) run headLanes to a warp, the rest `lanes`
    const int *iterp;    // the group's current iteration (device memory)
    int derivWarps;      // warps sharing one chain's Hessian in k_derivs (1..4)
    int adjMinDim;       // paths of this dimension and up take the reverse-mode adjoint, the others
                         // hyper-dual forward mode
    int lists;           // 1: the stage epilogues append the chain to the group's work lists (the
                         // staged schedule); 0: they only set the chain's flags (persistent schedule)
    int wave;            // 1: path tracing in wavefront rounds (wave.cuh), 0: one chain per lane
    int waveRounds;      // rounds of a wavefront stage pass (max_depth + 1)
    unsigned long long seed;
};

constexpr int kStageBlock = 64;  // threads per block of the per-chain stage kernels

// The per-chain stage kernels put `lanes` chains on each warp and leave the
// other lanes idle. Lanes of a warp that trace different paths serialise, and
// at these chain counts the GPU has room for far more warps than there are
// chains per 32, so fewer chains per warp shortens every warp's run.
DEV int sparse_index(int lanes, bool &active) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    active = lane < lanes;
    return warp * lanes + lane;
}
inline int sparse_blocks(int n, int lanes) {
    const int warps = (n + lanes - 1) / lanes;
    return (warps + kStageBlock / 32 - 1) / (kStageBlock / 32);
}

// Stage 1 in two tiers: the chains are in descending work-class order, so the
// first headChains are the longest traces; they get headLanes chains per warp
// (fewer lanes whose divergent work a warp serialises on the iteration's
// critical path), the rest `lanes` per warp.
HD int head_warps(int headChains, int headLanes) { return headChains > 0 ? (headChains + headLanes - 1) / headLanes : 0; }
DEV int stage1_index(int headChains, int headLanes, int lanes, bool &active) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int hw = head_warps(headChains, headLanes);
    if (warp < hw) {
        const int t = warp * headLanes + lane;
        active = lane < headLanes && t < headChains;
        return t;
    }
    active = lane < lanes;
    return headChains + (warp - hw) * lanes + lane;
}
inline int stage1_blocks(int n, int headChains, int headLanes, int lanes) {
    const int head = headChains < n ? headChains : n;
    const int warps = head_warps(head, headLanes) + (n - head + lanes - 1) / lanes;
    return (warps + kStageBlock / 32 - 1) / (kStageBlock / 32);
}

// ------------------------------------------------------------- reference lambdas
DEV bool flip_coin(float x, float d) { return (x == 1.0f) || (d < x); }      // delayed.cpp:250
DEV float metropolis_clamp(float x) { return x < 1.0f ? x : 1.0f; }         // std::min(1.0f, x)
DEV bool is_invalid(float x) { return isnan(x) || isinf(x) || x < 0.0f; }   // delayed.cpp:252
DEV float clamp01(float x) {                                                 // Clamp(x, 0, 1)
    const float t = (x < 0.0f) ? 0.0f : x;
    return (1.0f < t) ? 1.0f : t;
}

DEV Slot &slot_of(const ChainView &d, int chain, int which) { return d.slots[3 * chain + d.perm[3 * chain + which]]; }
DEV double *gauss_of(const ChainView &d, int chain, int which) {
    return d.gauss + size_t(3 * chain + d.perm[3 * chain + which]) * kGaussStride;
}

DEV void set_contrib(Slot &st, const Emit &e, float b) {
    st.screen[0] = e.screen[0];
    st.screen[1] = e.screen[1];
    st.rgb[0] = e.rgb.x;
    st.rgb[1] = e.rgb.y;
    st.rgb[2] = e.rgb.z;
    st.ls = e.ls;
    st.ss = e.ss;
    const float w = b / e.ls;
    st.splat[0] = e.screen[0];
    st.splat[1] = e.screen[1];
    st.splat[2] = e.rgb.x * w;
    st.splat[3] = e.rgb.y * w;
    st.splat[4] = e.rgb.z * w;
    st.hasSplat = 1;
}

// Films are W x H float4 pixels (RGB + an unused lane), so that one splat is one
// 16-byte vector reduction (red.global.add.v4.f32) instead of three scalar ones.
//
// Splat (src/image.h:65-74): nearest pixel, finite values only. Returns the
// pixel index, or -1 when the value is zero or not finite (nothing to add).
DEV int splat_pixel(int W, int H, float sx, float sy, float r, float g, float b) {
    if (r == 0.0f && g == 0.0f && b == 0.0f) return -1;
    if (!(isfinite(r) && isfinite(g) && isfinite(b))) return -1;
    int ix = int(sx * float(W));
    int iy = int(sy * float(H));
    ix = ix < 0 ? 0 : (ix > W - 1 ? W - 1 : ix);
    iy = iy < 0 ? 0 : (iy > H - 1 ? H - 1 : iy);
    return iy * W + ix;
}
DEV void splat(float4 *film, int W, int H, float sx, float sy, float r, float g, float b) {
    const int px = splat_pixel(W, H, sx, sy, r, g, b);
    if (px >= 0) atomicAdd(film + px, make_float4(r, g, b, 0.0f));
}

// WeightedSplat (src/integrators/delayed/delayed.cpp:255-265): weight times the
// stored splat, skipped when Eigen's isZero() holds for the product. Fills one
// pending splat (pixel -1: none) for warp_splat.
struct PendingSplat {
    int px;
    float r, g, b;
};
DEV PendingSplat weighted_splat_of(int W, int H, const float *sp, float w) {
    const V3 v(w * sp[2], w * sp[3], w * sp[4]);
    if (is_zero(v)) return PendingSplat{-1, 0.0f, 0.0f, 0.0f};
    return PendingSplat{splat_pixel(W, H, sp[0], sp[1], v.x, v.y, v.z), v.x, v.y, v.z};
}

// Warp-aggregated splat: called by all 32 lanes of a warp together, each with
// one pending splat (px = -1 for none). Lanes that hit the same pixel are
// grouped with __match_any_sync; the lowest lane of each group adds the
// group's sum with one vector reduction. The combining loop runs once per
// lane that shares its pixel with a lower lane (rare at these chain counts:
// most warps issue one reduction per distinct pixel and skip the loop).
DEV void warp_splat(float4 *film, PendingSplat s) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned peers = __match_any_sync(kFull, s.px);
    const int leader = __ffs(peers) - 1;
    unsigned pending = __ballot_sync(kFull, s.px >= 0 && lane != leader);
    while (pending) {
        const int j = __ffs(pending) - 1;
        const float r = __shfl_sync(kFull, s.r, j);
        const float g = __shfl_sync(kFull, s.g, j);
        const float b = __shfl_sync(kFull, s.b, j);
        const unsigned pj = __shfl_sync(kFull, peers, j);
        if (lane == __ffs(pj) - 1) {
            s.r += r;
            s.g += g;
            s.b += b;
        }
        pending &= pending - 1u;
    }
    if (s.px >= 0 && lane == leader) atomicAdd(film + s.px, make_float4(s.r, s.g, s.b, 0.0f));
}

// Block-aggregated statistics: one global atomic per counter per block.
struct StatAcc {
    unsigned c[kNumStats];
    DEV StatAcc() {
        for (int k = 0; k < kNumStats; k++) c[k] = 0u;
    }
};
DEV void flush_stats(const StatAcc &acc, unsigned long long *global) {
    __shared__ unsigned sh[kNumStats];
    if (threadIdx.x < kNumStats) sh[threadIdx.x] = 0u;
    __syncthreads();
    for (int k = 0; k < kNumStats; k++)
        if (acc.c[k]) atomicAdd_block(&sh[k], acc.c[k]);
    __syncthreads();
    if (threadIdx.x < kNumStats && sh[threadIdx.x]) atomicAdd(global + threadIdx.x, (unsigned long long)sh[threadIdx.x]);
}

DEV long long samples_of(const RunParams &p, int i) { return p.samplesPerChain + (i < p.extraChains ? 1 : 0); }


}  // namespace drmlt
