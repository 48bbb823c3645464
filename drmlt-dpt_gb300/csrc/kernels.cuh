// Device kernels of the DRMLT chain loop (delayed.cpp:334-673), its prepass
// (delayed.cpp:14-173) and the direct-lighting pass (integrator.h:33-75).
//
// One thread owns one Markov chain in the stage kernels. Each iteration runs
//   stage1   coin flips, large step or isotropic small step, first acceptance
//   derivs   gradient + Hessian of log f for chains that need a Gaussian at x
//            (one warp per chain, one Hessian entry per lane and pass)
//   gauss    FP64 eigen-decomposition + H2MC Gaussian (one thread per chain)
//   stage2   second-stage proposal z (H2MC sample or isotropic sigma2)
//   derivs + gauss at z for H2MC proposals
//   finish   Green (y* trace) or Mira acceptance, weighted splats, state swap
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
    kActive = 1, kAccept1 = 2, kLarge = 4, kSecond = 8, kAniso = 16, kZValid = 32, kAccept2 = 64
};

struct Scratch {
    float a1, a2;
    int flags;
    int key, rank;      // stage-1 work class and rank within it (k_plan)
    float aStar;        // Green's reverse first-stage acceptance (k_ystar)
    double logRatio;    // H2MC: log N_z(-o) - log N_x(o) (k_gauss at z)
    float offset[kMaxDim];
};

// Stage-1 work classes: 0 idle chain; 1 + 14 c + l small step of technique
// (c, l); 200 + 14 L + lgtLength large step of sampled length L.
constexpr int kPlanBins = 512;

enum : int {
    kStatLarge = 0, kStatLargeAcc, kStatStage1, kStatStage1Acc, kStatIso, kStatIsoAcc, kStatH2mc,
    kStatH2mcAcc, kStatMutations, kStatGauss, kStatGaussFallback, kNumStats
};

struct ChainView {
    Slot *slots;        // N x 3
    double *gauss;      // N x 3 x kGaussStride
    int *perm;          // N x 3: slot of (current, first, second)
    Scratch *scr;       // N
    int *listX;         // chains needing a Gaussian at the current state
    int *listZ;         // chains needing a Gaussian at the second proposal
    int *listS;         // chains taking a second stage this iteration
    int *order;         // stage-1 processing order (chains grouped by work class)
    int *hist;          // kPlanBins counters of the work classes
    int *counters;      // [0] = |listX|, [1] = |listZ|, [2] = |listS|
    float *grad;        // N x kMaxDim (indexed by list position)
    float *hess;        // N x kMaxDim^2
    unsigned long long *stats;
    float *film;        // W x H x 3 (indirect)
    float *direct;      // W x H x 3
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
    int accMap;
    int maxDerv;
    int gaussDim;        // largest path dimension (2 max_depth): sizes the Gaussian scratch
    int lanes;           // chains per warp in the per-chain stage kernels (1..32)
    int derivWarps;      // warps sharing one chain's Hessian in k_derivs (1..4)
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

// Splat (src/image.h:65-74): nearest pixel, finite values only.
DEV void splat(float *film, int W, int H, float sx, float sy, float r, float g, float b) {
    if (r == 0.0f && g == 0.0f && b == 0.0f) return;
    if (!(isfinite(r) && isfinite(g) && isfinite(b))) return;
    int ix = int(sx * float(W));
    int iy = int(sy * float(H));
    ix = ix < 0 ? 0 : (ix > W - 1 ? W - 1 : ix);
    iy = iy < 0 ? 0 : (iy > H - 1 ? H - 1 : iy);
    float *px = film + 3 * (size_t(iy) * W + ix);
    atomicAdd(px, r);
    atomicAdd(px + 1, g);
    atomicAdd(px + 2, b);
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

DEV float length_pmf(const ChainView &d, int len) {
    return d.lengthFunc[len] / (d.lengthFuncInt * float(d.lengthCount));
}

// ------------------------------------------------------------- stage-1 plan
// Draws each chain's stage-1 coin and, for a large step, its length and light
// subpath length exactly as k_stage1 will (same stream, same order), and bins
// the chain by the resulting work class. k_scatter then orders the chains by
// class so that the lanes of a warp trace the same technique.
DEV int plan_key(const RunParams &p, int i, int iter) {
    if (iter >= samples_of(p, i)) return 0;
    Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 0ull);
    const Slot &cur = slot_of(p.d, i, 0);
    const bool isLarge = flip_coin(p.largeProb, rng.uniform());
    if (!cur.valid || isLarge) {
        const int length = sample_discrete(p.d.lengthCdf, p.d.lengthCount, rng.uniform());
        int lgtLength = int(rng.uniform() * float(length + 1));
        lgtLength = lgtLength < 0 ? 0 : (lgtLength > length ? length : lgtLength);
        return 200 + 14 * length + lgtLength;
    }
    return 1 + 14 * cur.rec.c + cur.rec.l;
}

__global__ void __launch_bounds__(kStageBlock) k_plan(RunParams p, int iter) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.N) return;
    const int i = p.c0 + t;
    int key = plan_key(p, i, iter);
    key = key < 0 ? 0 : (key >= kPlanBins ? kPlanBins - 1 : key);
    Scratch &sc = p.d.scr[i];
    sc.key = key;
    sc.rank = atomicAdd(&p.d.hist[key], 1);
}

constexpr int kScatterBlock = 256;
__global__ void __launch_bounds__(kScatterBlock) k_scatter(RunParams p) {
    __shared__ int start[kPlanBins];
    __shared__ int warpSum[kScatterBlock / 32];
    // exclusive scan of the class counts (two bins per thread)
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int h0 = p.d.hist[2 * tid], h1 = p.d.hist[2 * tid + 1];
    int v = h0 + h1, incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += n;
    }
    if (lane == 31) warpSum[wid] = incl;
    __syncthreads();
    int base = 0;
    for (int w = 0; w < wid; w++) base += warpSum[w];
    const int excl = base + incl - v;
    start[2 * tid] = excl;
    start[2 * tid + 1] = excl + h0;
    __syncthreads();
    for (int t = blockIdx.x * blockDim.x + tid; t < p.N; t += gridDim.x * blockDim.x) {
        const int i = p.c0 + t;
        const Scratch &sc = p.d.scr[i];
        p.d.order[start[sc.key] + sc.rank] = i;
    }
}
static_assert(2 * kScatterBlock == kPlanBins, "k_scatter scans two bins per thread");

// ------------------------------------------------------------- stage 1
__global__ void __launch_bounds__(kStageBlock) k_stage1(RunParams p, int iter) {
    bool on;
    const int t = sparse_index(p.lanes, on);
    StatAcc acc;
    if (on && t < p.N) {
        const int i = p.d.order[t];
        Scratch &sc = p.d.scr[i];
        int flags = 0;
        float a1 = 0.0f;
        if (iter < samples_of(p, i)) {
            flags |= kActive;
            acc.c[kStatMutations]++;
            Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 0ull);
            Slot &cur = slot_of(p.d, i, 0);
            Slot &F = slot_of(p.d, i, 1);
            const bool isLarge = flip_coin(p.largeProb, rng.uniform());
            if (isLarge) flags |= kLarge;
            bool accept1 = false;
            if (!cur.valid || isLarge) {
                // LargeStep::Mutate, multiplexed + bidirectional (src/mutation.cpp:7-120)
                acc.c[kStatLarge]++;
                const int length = sample_discrete(p.d.lengthCdf, p.d.lengthCount, rng.uniform());
                int lgtLength = int(rng.uniform() * float(length + 1));
                lgtLength = lgtLength < 0 ? 0 : (lgtLength > length ? length : lgtLength);
                const int camLength = length - lgtLength + 1;
                Emit e;
                const bool ok = length >= 1 && generate_subpath(p.s, camLength, lgtLength, rng, F.rec, e);
                F.gaussInit = 0;
                if (ok) {
                    rng.uniform();  // contribution pick over a single candidate
                    set_contrib(F, e, p.b);
                    if (cur.valid) {
                        const int lc = cur.rec.c + cur.rec.l - 1;
                        const int ly = e.c + e.l - 1;
                        a1 = clamp01((float(ly + 1) * e.ls / length_pmf(p.d, ly)) /
                                     (float(lc + 1) * cur.ls / length_pmf(p.d, lc)));
                    }
                }
                if (is_invalid(a1)) {
                    a1 = 0.0f;
                } else {
                    accept1 = flip_coin(a1, rng.uniform());
                    if (accept1) acc.c[kStatLargeAcc]++;
                }
            } else {
                // SmallStep::Mutate with perturbStdDev (src/mutation.cpp:126-166)
                acc.c[kStatStage1]++;
                const int dim = path_dim(cur.rec.c, cur.rec.l);
                float off[kMaxDim];
                for (int k = 0; k < dim; k++) off[k] = p.sigma1 * rng.normal();
                Emit e;
                const bool ok = perturb_path(p.s, cur.rec, off, rng, F.rec, e);
                F.gaussInit = 0;
                if (ok) {
                    set_contrib(F, e, p.b);
                    a1 = clamp01(e.ss / cur.ss);
                }
                if (is_invalid(a1)) {
                    a1 = 0.0f;
                } else {
                    accept1 = flip_coin(a1, rng.uniform());
                    if (accept1) acc.c[kStatStage1Acc]++;
                }
            }
            if (accept1) flags |= kAccept1;
            const bool doSecond = !accept1 && !isLarge && cur.valid && p.integrator == 0;
            if (doSecond) {
                flags |= kSecond;
                p.d.listS[atomicAdd(&p.d.counters[2], 1)] = i;
                if (flip_coin(p.anisoProb, rng.uniform())) {
                    flags |= kAniso;
                    acc.c[kStatH2mc]++;
                    if (!cur.gaussInit) p.d.listX[atomicAdd(&p.d.counters[0], 1)] = i;
                } else {
                    acc.c[kStatIso]++;
                }
            }
        }
        sc.flags = flags;
        sc.a1 = a1;
        sc.a2 = 0.0f;
    }
    flush_stats(acc, p.d.stats);
}

// ------------------------------------------------------------- derivatives
// One warp per listed chain: lanes stride over the D(D+1)/2 Hessian entries.
// which: 0 = current state, 2 = second proposal.
__device__ void derivs_for_path(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H,
                                int member = threadIdx.x & 31, int team = 32) {
    const int lane = member;
    const int L = r.c + r.l - 1;
    const int dim = 2 * L;
    if (!(L <= maxDerv && ss > 1e-15f)) {
        for (int k = lane; k < dim; k += team) g[k] = 0.0f;
        for (int k = lane; k < dim * dim; k += team) H[k] = 0.0f;
        return;
    }
    const int npairs = dim * (dim + 1) / 2;
    for (int pidx = lane; pidx < npairs; pidx += team) {
        // decode pidx -> (i0, j0), i0 <= j0, row-major over the upper triangle
        int i0 = 0, rem = pidx;
        while (rem >= dim - i0) {
            rem -= dim - i0;
            i0++;
        }
        const int j0 = i0 + rem;
        HyperDual u[kMaxDim];
        for (int k = 0; k < dim; k++)
            u[k] = HyperDual(r.u[k], k == i0 ? 1.0f : 0.0f, k == j0 ? 1.0f : 0.0f, 0.0f);
        const HyperDual f = ad_eval_path<HyperDual>(s, r, u);
        H[i0 * dim + j0] = f.ab;
        H[j0 * dim + i0] = f.ab;
        if (i0 == j0) g[i0] = f.a;
    }
}

// A team of p.derivWarps warps per listed chain shares its Hessian entries.
__global__ void __launch_bounds__(128) k_derivs(RunParams p, int which) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int w = gw / p.derivWarps;
    const int n = p.d.counters[which == 0 ? 0 : 1];
    if (w >= n) return;
    const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
    const Slot &st = slot_of(p.d, chain, which);
    derivs_for_path(p.s, st.rec, st.ss, p.maxDerv, p.d.grad + size_t(w) * kMaxDim,
                    p.d.hess + size_t(w) * kMaxDim * kMaxDim, (gw % p.derivWarps) * 32 + (threadIdx.x & 31),
                    32 * p.derivWarps);
}

// One warp per listed chain; 4 warps per block, each with its own slice of
// dynamic shared memory (gauss_smem_doubles(maxDim) doubles).
constexpr int kGaussWarps = 4;
inline size_t gauss_smem_bytes(int maxDim) { return size_t(kGaussWarps) * gauss_smem_doubles(maxDim) * sizeof(double); }

__global__ void __launch_bounds__(32 * kGaussWarps) k_gauss(RunParams p, int which) {
    extern __shared__ double gsm[];
    const int wib = threadIdx.x >> 5;
    const int w = blockIdx.x * kGaussWarps + wib;
    const int n = p.d.counters[which == 0 ? 0 : 1];
    if (w >= n) return;
    const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
    Slot &st = slot_of(p.d, chain, which);
    const int dim = path_dim(st.rec.c, st.rec.l);
    GaussSmem sm(gsm + size_t(wib) * gauss_smem_doubles(p.gaussDim), p.gaussDim);
    // dim <= gaussDim holds by construction (max_depth bounds every path); the
    // isotropic branch needs no scratch, so an impossible larger dim stays in bounds
    const int kind = compute_gaussian_warp(dim, H2mcParam(p.sigma1), dim <= sm.m ? st.ss : 0.0f,
                                           p.d.grad + size_t(w) * kMaxDim, p.d.hess + size_t(w) * kMaxDim * kMaxDim, sm,
                                           GaussView(gauss_of(p.d, chain, which)));
    if (which == 2) {
        // the H2MC kernel ratio of PH2MCSmallStep::Mutate (drsmallstep.cpp:191-196), FP64
        Scratch &sc = p.d.scr[chain];
        const int d = dim <= sm.m ? dim : 0;
        const double px = gauss_logpdf_warp(d, sc.offset, -1.0, GaussView(gauss_of(p.d, chain, 2)));
        const double py = gauss_logpdf_warp(d, sc.offset, 1.0, GaussView(gauss_of(p.d, chain, 0)));
        if ((threadIdx.x & 31) == 0) sc.logRatio = px - py;
    }
    if ((threadIdx.x & 31) == 0) {
        st.gaussInit = 1;
        if (kind != kGaussIsotropic) atomicAdd(&p.d.stats[kStatGauss], 1ull);
        if (kind == kGaussFp64Jacobi) atomicAdd(&p.d.stats[kStatGaussFallback], 1ull);
    }
}

// ------------------------------------------------------------- stage 2 proposal
// Over the group's second-stage list only (compacted by k_stage1).
__global__ void __launch_bounds__(kStageBlock) k_stage2(RunParams p, int iter) {
    bool on;
    const int t = sparse_index(p.lanes, on);
    if (!on || t >= p.d.counters[2]) return;
    const int i = p.d.listS[t];
    Scratch &sc = p.d.scr[i];
    Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
    Slot &cur = slot_of(p.d, i, 0);
    Slot &S = slot_of(p.d, i, 2);
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    float off[kMaxDim];
    const bool aniso = sc.flags & kAniso;
    if (aniso) {
        // PH2MCSmallStep::Mutate (drsmallstep.cpp:113-212)
        double od[kMaxDim];
        gauss_sample(dim, GaussView(gauss_of(p.d, i, 0)), rng, od);
        for (int k = 0; k < dim; k++) {
            off[k] = float(od[k]);
            sc.offset[k] = off[k];
        }
    } else {
        // SmallStep::Mutate with the second-stage sigma (mutation.cpp:167-208)
        for (int k = 0; k < dim; k++) off[k] = p.sigma2 * rng.normal();
    }
    Emit e;
    const bool ok = perturb_path(p.s, cur.rec, off, rng, S.rec, e);
    S.gaussInit = 0;
    float a2 = 0.0f;
    if (ok) {
        sc.flags |= kZValid;
        S.screen[0] = e.screen[0];
        S.screen[1] = e.screen[1];
        S.rgb[0] = e.rgb.x;
        S.rgb[1] = e.rgb.y;
        S.rgb[2] = e.rgb.z;
        S.ls = e.ls;
        S.ss = e.ss;
        if (!aniso || (e.ls > 0.0f && isfinite(e.ls))) set_contrib(S, e, p.b); else S.hasSplat = 0;
        if (aniso) {
            p.d.listZ[atomicAdd(&p.d.counters[1], 1)] = i;
        } else {
            a2 = clamp01(e.ss / cur.ss);
        }
    }
    sc.a2 = a2;
}

// Green's reverse path y* = z + (x - y) and its first-stage acceptance from z
// (SmallStep::Trace, mutation.cpp:210-238), over the second-stage list only.
__global__ void __launch_bounds__(kStageBlock) k_ystar(RunParams p, int iter) {
    bool on;
    const int t = sparse_index(p.lanes, on);
    if (!on || t >= p.d.counters[2]) return;
    const int i = p.d.listS[t];
    Scratch &sc = p.d.scr[i];
    const Slot &cur = slot_of(p.d, i, 0);
    const Slot &F = slot_of(p.d, i, 1);
    const Slot &S = slot_of(p.d, i, 2);
    float aStar = 0.0f;
    if (S.valid) {
        const int dim = path_dim(cur.rec.c, cur.rec.l);
        float off[kMaxDim];
        for (int k = 0; k < dim; k++) off[k] = cur.rec.u[k] - F.rec.u[k];
        Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 3ull);
        PathRec ystar;
        Emit e;
        if (perturb_path(p.s, S.rec, off, rng, ystar, e)) aStar = clamp01(e.ss / S.ss);
    }
    sc.aStar = aStar;
}

// log N(d | 0, sigma^2 I) differences for Mira's Q1 ratio (delayed.cpp:512-523), FP64.
DEV double iso_quad(int dim, const float *a, const float *b) {
    double q = 0.0;
    for (int k = 0; k < dim; k++) {
        const double d = double(a[k]) - double(b[k]);
        q += d * d;
    }
    return q;
}

// ------------------------------------------------------------- finish
__global__ void __launch_bounds__(kStageBlock) k_finish(RunParams p, int iter) {
    bool on;
    const int t = sparse_index(p.lanes, on);
    const int i = p.c0 + t;
    StatAcc acc;
    if (on && t < p.N && (p.d.scr[i].flags & kActive)) {
        Scratch &sc = p.d.scr[i];
        const int flags = sc.flags;
        const float a1 = sc.a1;
        float a2 = sc.a2;
        bool accept2 = false;
        Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 2ull);
        Slot &cur = slot_of(p.d, i, 0);
        Slot &F = slot_of(p.d, i, 1);
        Slot &S = slot_of(p.d, i, 2);
        const bool aniso = flags & kAniso;
        if (flags & kSecond) {
            const int dim = path_dim(cur.rec.c, cur.rec.l);
            if (aniso) {
                if (flags & kZValid) {
                    a2 = float(::exp(sc.logRatio)) * S.ss / cur.ss;
                } else {
                    a2 = 0.0f;
                }
            }
            if (is_invalid(a2)) {
                a2 = 0.0f;
            } else if (p.drType == 0) {
                // Green & Mira (2001) (delayed.cpp:473-500); y* traced by k_ystar
                float aStar = sc.aStar;
                if (is_invalid(aStar)) aStar = 0.0f;
                if (aStar == 1.0f) {
                    a2 = 0.0f;
                } else {
                    a2 = metropolis_clamp(a2 * (1.0f - aStar) / (1.0f - a1));
                    accept2 = flip_coin(a2, rng.uniform());
                }
            } else {
                // Tierney & Mira (1999) (delayed.cpp:502-541)
                float aStar = metropolis_clamp(F.ss / S.ss);
                if (is_invalid(aStar)) aStar = 1.0f;
                if (aStar == 1.0f) {
                    a2 = 0.0f;
                } else {
                    const double inv2s2 = 0.5 / (double(p.sigma1) * double(p.sigma1));
                    const double lr = -inv2s2 * (iso_quad(dim, S.rec.u, F.rec.u) - iso_quad(dim, cur.rec.u, F.rec.u));
                    const float transRatio = float(::exp(lr));
                    if (is_invalid(transRatio)) {
                        a2 = 0.0f;
                    } else {
                        a2 = metropolis_clamp(a2 * transRatio * (1.0f - aStar) / (1.0f - a1));
                        accept2 = flip_coin(a2, rng.uniform());
                    }
                }
            }
            if (accept2) acc.c[aniso ? kStatH2mcAcc : kStatIsoAcc]++;
        }
        // weighted splats (delayed.cpp:547-561)
        const float w1 = a1;
        const float w2 = (1.0f - w1) * a2;
        const float wc = 1.0f - w1 - w2;
        const int W = p.s.cam.width, H = p.s.cam.height;
        if (!p.accMap) {
            if (cur.valid && wc > 0.0f && cur.hasSplat)
                splat(p.d.film, W, H, cur.splat[0], cur.splat[1], wc * cur.splat[2], wc * cur.splat[3], wc * cur.splat[4]);
            if (w1 > 0.0f && F.hasSplat)
                splat(p.d.film, W, H, F.splat[0], F.splat[1], w1 * F.splat[2], w1 * F.splat[3], w1 * F.splat[4]);
            if (w2 > 0.0f && S.hasSplat)
                splat(p.d.film, W, H, S.splat[0], S.splat[1], w2 * S.splat[2], w2 * S.splat[3], w2 * S.splat[4]);
        }
        // accept / swap (delayed.cpp:563-606)
        int *perm = p.d.perm + 3 * i;
        if (flags & kAccept1) {
            const int t = perm[0];
            perm[0] = perm[1];
            perm[1] = t;
            Slot &nc = slot_of(p.d, i, 0);
            nc.gaussInit = 0;
            nc.valid = 1;
            const Slot &old = slot_of(p.d, i, 1);
            if (p.accMap && !(flags & kLarge) && old.hasSplat) splat(p.d.film, W, H, old.splat[0], old.splat[1], 1.0f, 0.0f, 0.0f);
        } else if (accept2) {
            const int t = perm[0];
            perm[0] = perm[2];
            perm[2] = t;
            Slot &nc = slot_of(p.d, i, 0);
            if (!aniso) nc.gaussInit = 0;
            nc.valid = 1;
            const Slot &old = slot_of(p.d, i, 2);
            if (p.accMap && old.hasSplat) splat(p.d.film, W, H, old.splat[0], old.splat[1], 0.0f, 1.0f, 0.0f);
        }
        sc.flags = flags | (accept2 ? kAccept2 : 0);
        sc.a2 = a2;
    }
    flush_stats(acc, p.d.stats);
}

__global__ void k_reset_counters(int *counters, int *hist) {
    if (threadIdx.x < 4) counters[threadIdx.x] = 0;
    for (int k = threadIdx.x; k < kPlanBins; k += blockDim.x) hist[k] = 0;
}

// ------------------------------------------------------------- prepass
struct BootRecord {
    int sample;
    int c, l;
    float ls;
};

struct SinkAppend {
    BootRecord *out;
    int *count;
    int cap;
    int sample;
    int *overflow;
    DEV void operator()(const Emit &e) {
        const int k = atomicAdd(count, 1);
        if (k < cap) {
            out[k].sample = sample;
            out[k].c = e.c;
            out[k].l = e.l;
            out[k].ls = e.ls;
        } else {
            atomicExch(overflow, 1);
        }
    }
};

struct SinkTarget {
    int c, l;
    bool found;
    Emit e;
    DEV void operator()(const Emit &x) {
        if (x.c == c && x.l == l) {
            e = x;
            found = true;
        }
    }
};

__global__ void __launch_bounds__(128) k_bootstrap(SceneView s, unsigned long long seed, int numSamples, int minDepth,
                                                   int maxDepth, BootRecord *out, int *count, int cap, int *overflow) {
    const int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= numSamples) return;
    Rng rng(seed, (unsigned long long)sidx, 0xB007ull);
    FullPath f;
    SinkAppend sink{out, count, cap, sidx, overflow};
    generate_path_bidir(s, minDepth, maxDepth, rng, f, sink);
}

__global__ void __launch_bounds__(128) k_seed(RunParams p, unsigned long long bootSeed, const int *sampleOf,
                                              const int *techC, const int *techL, int minDepth, int maxDepth) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.N) return;
    Rng rng(bootSeed, (unsigned long long)sampleOf[i], 0xB007ull);
    FullPath f;
    SinkTarget sink{techC[i], techL[i], false, Emit()};
    generate_path_bidir(p.s, minDepth, maxDepth, rng, f, sink);
    for (int k = 0; k < 3; k++) {
        p.d.perm[3 * i + k] = k;
        Slot &st = p.d.slots[3 * i + k];
        st.valid = 0;
        st.hasSplat = 0;
        st.gaussInit = 0;
        st.ls = st.ss = 0.0f;
    }
    Slot &cur = p.d.slots[3 * i];
    if (sink.found) {
        make_rec(f, sink.c, sink.l, cur.rec);
        cur.screen[0] = sink.e.screen[0];
        cur.screen[1] = sink.e.screen[1];
        cur.rgb[0] = sink.e.rgb.x;
        cur.rgb[1] = sink.e.rgb.y;
        cur.rgb[2] = sink.e.rgb.z;
        cur.ls = sink.e.ls;
        cur.ss = sink.e.ss;
        cur.valid = 1;
    }
    // Seeded states carry no toSplat entry (delayed.cpp:138-167 never fills it).
}

// ------------------------------------------------------------- direct lighting pass
struct SinkSplat {
    float *film;
    int W, H;
    DEV void operator()(const Emit &e) { splat(film, W, H, e.screen[0], e.screen[1], e.rgb.x, e.rgb.y, e.rgb.z); }
};

__global__ void __launch_bounds__(128) k_direct(SceneView s, unsigned long long seed, int spp, int minDepth,
                                                int maxDepth, float *film) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long npix = (long long)s.cam.width * s.cam.height;
    if (t >= npix * spp) return;
    const int pix = int(t / spp);
    const int smp = int(t % spp);
    Rng rng(seed ^ 0xD1ECull, (unsigned long long)pix, (unsigned long long)smp);
    SinkSplat sink{film, s.cam.width, s.cam.height};
    generate_path_direct(s, pix % s.cam.width, pix / s.cam.width, minDepth, maxDepth, rng, sink);
}

}  // namespace drmlt
