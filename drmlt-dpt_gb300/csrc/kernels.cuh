// Device kernels of the DRMLT chain loop (delayed.cpp:334-673), its prepass
// (delayed.cpp:14-173) and the direct-lighting pass (integrator.h:33-75).
//
// Each iteration runs, per chain (16 chains per warp by default in the stage kernels):
//   plan/scatter  order the chains by stage-1 work class (technique)
//   stage1   coin flips, large step or isotropic small step, first acceptance
//   derivs   gradient + Hessian of log f for chains that need a Gaussian at x
//            (a team of warps per chain, one Hessian entry per lane and pass; derivs.cu)
//   gauss    H2MC Gaussian, FP32 Jacobi refined to FP64 (one warp per chain)
//   stage2   second-stage proposal z (H2MC sample or isotropic sigma2)
//   derivs + gauss at z for H2MC proposals, with the FP64 log-density ratio
//   ystar    Green's reverse path y* (second-stage chains only)
//   finish   Green or Mira acceptance, weighted splats, state swap
#pragma once
#include "chain.cuh"
#include "derivs.h"
#include "lens.cuh"

namespace drmlt {

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
        return 256 + 16 * length + lgtLength;
    }
    if (p.integrator == 1 && !(rng.uniform() < p.uniformMix)) return 0;  // H2MC step: no stage-1 trace
    return 1 + 16 * (cur.rec.c + cur.rec.l) + cur.rec.c;
}

static __global__ void __launch_bounds__(kStageBlock) k_plan(RunParams p) {
    const int iter = *p.iterp;
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
static __global__ void __launch_bounds__(kScatterBlock) k_scatter(RunParams p) {
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
        p.d.order[p.N - 1 - (start[sc.key] + sc.rank)] = i;  // descending class
    }
}
static_assert(2 * kScatterBlock == kPlanBins, "k_scatter scans two bins per thread");

// ------------------------------------------------------------- stage 1
// The path-tracing stages (stage 1, stage 2, Green's y*) are written as a
// prologue, the path machine (path.cuh) and an epilogue, shared by the
// per-lane kernels below (one chain per lane traces its whole path) and the
// wavefront kernels (wave.cuh), so that both schedules take identical steps.
enum : int {
    kTraceNone = 0,     // no path to trace: the prologue finished the stage
    kTraceFail = 1,     // a large step whose sampled length is empty: finish as a failed proposal
    kTracePerturb = 2,  // PerturbPathBidir machine
    kTraceSubpath = 3   // GenerateSubpath machine
};

// The multiplexed large step's acceptance (src/mutation.cpp:86-98): technique
// pmfs 1 / (length + 1) and the path-length distribution's pmf
// (PiecewiseConstant1D::Pmf of func over count lengths), for the current
// technique of length lc and score lsc and the proposal's (ly, lsy).
DEV float large_step_ratio(const float *lengthFunc, float lengthFuncInt, int lengthCount, int lc, float lsc, int ly,
                           float lsy) {
    const float pmfY = lengthFunc[ly] / (lengthFuncInt * float(lengthCount));
    const float pmfC = lengthFunc[lc] / (lengthFuncInt * float(lengthCount));
    return clamp01((float(ly + 1) * lsy / pmfY) / (float(lc + 1) * lsc / pmfC));
}

// Stage-1 prologue of chain i (delayed.cpp:396-441 up to the proposal's path
// sampling): the large-step coin and, for a large step, its length and light
// subpath length (LargeStep::Mutate, src/mutation.cpp:7-120, multiplexed and
// bidirectional); for a small step the sigma1 offsets (SmallStep::Mutate,
// src/mutation.cpp:126-166). Chains that trace nothing (inactive, or
// integrator=h2mc's H2MC step) are finished here.
DEV int stage1_begin(const RunParams &p, int i, int iter, Rng &rng, float *off, PathM &m, int &flags, StatAcc &acc) {
    Scratch &sc = p.d.scr[i];
    flags = 0;
    if (iter >= samples_of(p, i)) {
        sc.flags = 0;
        sc.a1 = 0.0f;
        sc.a2 = 0.0f;
        return kTraceNone;
    }
    flags = kActive;
    acc.c[kStatMutations]++;
    rng = Rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 0ull);
    const Slot &cur = slot_of(p.d, i, 0);
    Slot &F = slot_of(p.d, i, 1);
    const bool isLarge = flip_coin(p.largeProb, rng.uniform());
    if (isLarge) flags |= kLarge;
    if (!cur.valid || isLarge) {
        acc.c[kStatLarge]++;
        const int length = sample_discrete(p.d.lengthCdf, p.d.lengthCount, rng.uniform());
        int lgtLength = int(rng.uniform() * float(length + 1));
        lgtLength = lgtLength < 0 ? 0 : (lgtLength > length ? length : lgtLength);
        F.gaussInit = 0;
        if (length < 1) return kTraceFail;
        m.pc = kGStart;
        m.camLength = length - lgtLength + 1;
        m.lgtLength = lgtLength;
        return kTraceSubpath;
    }
    if (p.integrator == 1 && !(rng.uniform() < p.uniformMix)) {
        // H2MCIntegrator (src/integrators/h2mc.cpp:200-240): H2MCSmallStep::Mutate
        // (h2mc.cpp:448-606) as the single stage. Its lens branch (taken for a
        // lens score > 0 with probability lensPerturbProb) draws the coin here
        // and leaves the score test to k_lens, which sends a chain with a zero
        // score on to the H2MC step; the H2MC step runs in the second-stage kernels.
        if (p.lensProb > 0.0f && rng.uniform() < p.lensProb) {
            flags |= kSecond | kSingle | kLens;
            if (p.lists) p.d.listL[atomicAdd(&p.d.counters[4], 1)] = i;
            sc.flags = flags;
            sc.a1 = 0.0f;
            sc.a2 = 0.0f;
            return kTraceNone;
        }
        flags |= kSecond | kAniso | kSingle;
        acc.c[kStatH2mc]++;
        if (p.lists) {
            p.d.listS[atomicAdd(&p.d.counters[2], 1)] = i;
            if (!cur.gaussInit) p.d.listX[atomicAdd(&p.d.counters[0], 1)] = i;
            p.d.listA[atomicAdd(&p.d.counters[3], 1)] = i;
        }
        sc.flags = flags;
        sc.a1 = 0.0f;
        sc.a2 = 0.0f;
        return kTraceNone;
    }
    // SmallStep::Mutate with perturbStdDev; for integrator=h2mc the
    // uniform-mixing step (h2mc.cpp:454-459)
    acc.c[kStatStage1]++;
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    for (int k = 0; k < dim; k++) off[k] = p.sigma1 * rng.normal();
    F.gaussInit = 0;
    m.pc = kPStart;
    return kTracePerturb;
}

// Stage-1 epilogue: the first acceptance (mutation.cpp:86-98 for a large step,
// :155 for a small one), the second-stage decision (delayed.cpp:443-451) and
// the chain's entries in the second-stage lists. `st` is the sampler's result
// (kStepDone with the proposal's contribution in e, or kStepFail).
DEV void stage1_end(const RunParams &p, int i, int mode, int flags, Rng &rng, int st, const Emit &e, StatAcc &acc) {
    Scratch &sc = p.d.scr[i];
    const Slot &cur = slot_of(p.d, i, 0);
    Slot &F = slot_of(p.d, i, 1);
    const bool ok = st == kStepDone;
    float a1 = 0.0f;
    bool accept1 = false;
    if (mode != kTracePerturb) {
        if (ok) {
            rng.uniform();  // contribution pick over a single candidate
            set_contrib(F, e, p.b);
            if (cur.valid)
                a1 = large_step_ratio(p.d.lengthFunc, p.d.lengthFuncInt, p.d.lengthCount, cur.rec.c + cur.rec.l - 1,
                                      cur.ls, e.c + e.l - 1, e.ls);
        }
        if (is_invalid(a1)) {
            a1 = 0.0f;
        } else {
            accept1 = flip_coin(a1, rng.uniform());
            if (accept1) acc.c[kStatLargeAcc]++;
        }
    } else {
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
    const bool doSecond = !accept1 && !(flags & kLarge) && cur.valid && p.integrator == 0;
    if (doSecond) {
        flags |= kSecond;
        if (p.lists) p.d.listS[atomicAdd(&p.d.counters[2], 1)] = i;
        if (flip_coin(p.anisoProb, rng.uniform())) {
            flags |= kAniso;
            acc.c[kStatH2mc]++;
            if (p.lists) {
                if (!cur.gaussInit) p.d.listX[atomicAdd(&p.d.counters[0], 1)] = i;
                p.d.listA[atomicAdd(&p.d.counters[3], 1)] = i;
            }
        } else {
            acc.c[kStatIso]++;
        }
    }
    sc.flags = flags;
    sc.a1 = a1;
    sc.a2 = 0.0f;
}

// The machines with every ray answered on the spot (per-lane kernels).
template <class R>
DEV int run_subpath(const SceneView &s, R &rng, PathRec &rec, PathM &m) {
    int hit = -1, st;
    while ((st = subpath_step(s, rng, rec, m, hit)) == kStepRay) hit = answer_ray(s, m);
    return st;
}
template <class J>
DEV int run_perturb(const SceneView &s, const PathRec &in, const float *off, J &jit, PathRec &out, PathM &m) {
    int hit = -1, st;
    while ((st = perturb_step(s, in, off, jit, out, m, hit)) == kStepRay) hit = answer_ray(s, m);
    return st;
}

static __global__ void __launch_bounds__(kStageBlock) k_stage1(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = stage1_index(p.headChains < p.N ? p.headChains : p.N, p.headLanes, p.lanes, on);
    StatAcc acc;
    if (on && t < p.N) {
        const int i = p.d.order[t];
        Rng rng;
        float off[kMaxDim];
        PathM m;
        int flags;
        const int mode = stage1_begin(p, i, iter, rng, off, m, flags, acc);
        if (mode != kTraceNone) {
            int st = kStepFail;
            if (mode == kTraceSubpath) st = run_subpath(p.s, rng, slot_of(p.d, i, 1).rec, m);
            if (mode == kTracePerturb) st = run_perturb(p.s, slot_of(p.d, i, 0).rec, off, rng, slot_of(p.d, i, 1).rec, m);
            stage1_end(p, i, mode, flags, rng, st, m.e, acc);
        }
    }
    flush_stats(acc, p.d.stats);
}

// ------------------------------------------------------------- derivatives
// k_derivs lives in derivs.cu (its own translation unit); see derivs.h.

// One block (a team of kGaussTeamWarps warps) per listed chain, with
// gauss_smem_doubles(maxDim) doubles of dynamic shared memory.
constexpr int kGaussTeamWarps = 4;
inline size_t gauss_smem_bytes(int maxDim) { return size_t(gauss_smem_doubles(maxDim)) * sizeof(double); }

// The Gaussian of chain `chain` at its slot `which` (0 current state, 2 second
// proposal) from the gradient / Hessian rows grad / hess, by the whole block
// (a team of kGaussTeamWarps warps) with gauss_smem_doubles(gaussDim) doubles of
// shared scratch at gsm; at the second proposal also the H2MC kernel ratio.
DEV void gauss_for_chain(const RunParams &p, int chain, int which, const float *grad, const float *hess, double *gsm) {
    Slot &st = slot_of(p.d, chain, which);
    const int dim = path_dim(st.rec.c, st.rec.l);
    GaussSmem sm(gsm, p.gaussDim);
    const Team tm(gauss_reduction(gsm, p.gaussDim));
    // dim <= gaussDim holds by construction (max_depth bounds every path); the
    // isotropic branch needs no scratch, so an impossible larger dim stays in bounds
    const int kind = compute_gaussian_team(dim, H2mcParam(p.sigma1), dim <= sm.m ? st.ss : 0.0f, grad, hess, sm,
                                           GaussView(gauss_of(p.d, chain, which)), tm);
    if (which == 2) {
        // the H2MC kernel ratio of PH2MCSmallStep::Mutate (drsmallstep.cpp:191-196), FP64
        Scratch &sc = p.d.scr[chain];
        const int d = dim <= sm.m ? dim : 0;
        const double px = gauss_logpdf_team(d, sc.offset, -1.0, GaussView(gauss_of(p.d, chain, 2)), tm);
        const double py = gauss_logpdf_team(d, sc.offset, 1.0, GaussView(gauss_of(p.d, chain, 0)), tm);
        if (threadIdx.x == 0) sc.logRatio = px - py;
    }
    if (threadIdx.x == 0) {
        st.gaussInit = 1;
        if (kind != kGaussIsotropic) atomicAdd(&p.d.stats[kStatGauss], 1ull);
        if (kind == kGaussFp64Jacobi) atomicAdd(&p.d.stats[kStatGaussFallback], 1ull);
    }
}

DEV void gauss_for_entry(const RunParams &p, int which, int w, double *gsm) {
    const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
    gauss_for_chain(p, chain, which, p.d.grad + size_t(w) * kMaxDim, p.d.hess + size_t(w) * kMaxDim * kMaxDim, gsm);
}

// The grid is sized for the GPU, not the list: each block takes list entries
// blockIdx.x, blockIdx.x + gridDim.x, ... (the list's length is known only on
// the device).
static __global__ void __launch_bounds__(32 * kGaussTeamWarps) k_gauss(RunParams p, int which) {
    extern __shared__ double gsm[];
    const int n = p.d.counters[which == 0 ? 0 : 1];
    for (int k = blockIdx.x; k < n; k += gridDim.x) {
        gauss_for_entry(p, which, n - 1 - k, gsm);  // longest paths first (the lists fill shortest first)
        __syncthreads();  // the block's shared scratch is reused by its next entry
    }
}

// ------------------------------------------------------------- H2MC offsets
// GenerateSample (src/gaussian.cpp:36-47) for the chains taking the
// anisotropic second stage, one warp per chain: offset = mean + V diag(p^-1/2) n
// in FP64, with n the first dim normals of the chain's stage-2 stream (which
// k_stage2 then skips).
// One warp: the H2MC offset of chain i at iteration iter (zs: kMaxDim doubles of
// the warp's shared scratch).
DEV void h2mc_offset_warp(const RunParams &p, int i, int iter, double *zs) {
    const int lane = threadIdx.x & 31;
    const Slot &cur = slot_of(p.d, i, 0);
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    const GaussView g(gauss_of(p.d, i, 0));
    if (lane == 0) {
        Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
        for (int k = 0; k < dim; k++) zs[k] = double(rng.normal());
    }
    __syncwarp();
    if (lane < dim) zs[lane] /= ::sqrt(g.p[lane]);
    __syncwarp();
    if (lane < dim) {
        double o = g.mean[lane];
        for (int k = 0; k < dim; k++) o = ::fma(g.V[lane * dim + k], zs[k], o);
        p.d.scr[i].offset[lane] = float(o);
    }
    __syncwarp();
}

static __global__ void __launch_bounds__(128) k_h2mc_offset(RunParams p) {
    const int iter = *p.iterp;
    __shared__ double zs[4][kMaxDim];
    const int wib = threadIdx.x >> 5;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= p.d.counters[3]) return;
    h2mc_offset_warp(p, p.d.listA[w], iter, zs[wib]);
}

// ------------------------------------------------------------- stage 2 proposal
// Stage-2 prologue (chains of the second-stage list built by stage 1): the
// second proposal's offsets -- for PH2MCSmallStep::Mutate (drsmallstep.cpp:113-212)
// the ones k_h2mc_offset sampled from this stream's first dim normals (skipped
// here), for SmallStep::Mutate with the second-stage sigma (mutation.cpp:167-208)
// sigma2 normals -- and the perturbation machine.
DEV void stage2_begin(const RunParams &p, int i, int iter, Rng &rng, float *off, PathM &m) {
    const Scratch &sc = p.d.scr[i];
    rng = Rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
    const Slot &cur = slot_of(p.d, i, 0);
    Slot &S = slot_of(p.d, i, 2);
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    if (sc.flags & kAniso) {
        for (int k = 0; k < dim; k++) {
            rng.normal();
            off[k] = sc.offset[k];
        }
    } else {
        for (int k = 0; k < dim; k++) off[k] = p.sigma2 * rng.normal();
    }
    S.gaussInit = 0;
    m.pc = kPStart;
}

// Stage-2 epilogue: the proposal's state, its isotropic acceptance, or its
// entry in the list of Gaussians at z (H2MC).
DEV void stage2_end(const RunParams &p, int i, int st, const Emit &e) {
    Scratch &sc = p.d.scr[i];
    const Slot &cur = slot_of(p.d, i, 0);
    Slot &S = slot_of(p.d, i, 2);
    const bool aniso = sc.flags & kAniso;
    float a2 = 0.0f;
    if (st == kStepDone) {
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
            if (p.lists) p.d.listZ[atomicAdd(&p.d.counters[1], 1)] = i;
        } else {
            a2 = clamp01(e.ss / cur.ss);
        }
    }
    sc.a2 = a2;
}

// Over the group's second-stage list only (compacted by stage 1).
// The second-stage list fills in the order stage 1 finishes its chains, so the
// longest traces come last; the list kernels take it from the back, longest
// first, so that the slowest chains start first and the short ones fill in.
DEV int longest_first(const int *list, int n, int t) { return list[n - 1 - t]; }

static __global__ void __launch_bounds__(kStageBlock) k_stage2(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = sparse_index(p.lanes2, on);
    const int n = p.d.counters[2];
    if (!on || t >= n) return;
    const int i = longest_first(p.d.listS, n, t);
    Rng rng;
    float off[kMaxDim];
    PathM m;
    stage2_begin(p, i, iter, rng, off, m);
    const int st = run_perturb(p.s, slot_of(p.d, i, 0).rec, off, rng, slot_of(p.d, i, 2).rec, m);
    stage2_end(p, i, st, m.e);
}

// ------------------------------------------------------------- lens mutation
// integrator=h2mc's lens branch (H2MCSmallStep::Mutate, h2mc.cpp:466-532) for
// the chains stage 1 drew for it (listL), one chain per thread, between stage
// 1 and the derivatives at x: the current state's lens score -- zero sends the
// chain to the H2MC step instead (its list entries are made here) -- its lens
// Gaussian, the offset (GenerateSample: two normals of the chain's stage-2
// stream, which the chain does not otherwise use this iteration), the screen
// position (x.screen + offset) mod 1, PerturbLensBidir into the second slot,
// the proposal's lens Gaussian, and the unclamped acceptance
// exp(log N_z(-o) - log N_x(o)) lens(z) / lens(x) that k_finish clamps and draws.
// One chain per thread, one warp per block, so that the list's warps spread
// over every SM: the kernel is large (two path walks, six hyper-dual path
// evaluations, two Gaussians) and bound by instruction fetch once several of
// its warps share an SM. Config 4, h2mc, per launch (ncu, serialised): 32
// chains on each warp of 64-thread blocks 1.13-1.35 ms (the list's blocks on
// ~86 SMs), 4 chains per warp 1.66-1.79 ms (8 warps per SM, 30 cycles of
// instruction-fetch stall per issued instruction).
constexpr int kLensBlock = 32;
static __global__ void __launch_bounds__(kLensBlock) k_lens(RunParams p) {
    const int iter = *p.iterp;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= p.d.counters[4]) return;
    const int i = p.d.listL[t];
    Scratch &sc = p.d.scr[i];
    const Slot &cur = slot_of(p.d, i, 0);
    Slot &S = slot_of(p.d, i, 2);
    Emit e;
    float lsx;
    LensAnchor ax;
    V3 lensPos;
    // the walk's copy of the path goes to the second slot, which the proposal overwrites
    const bool okx = lens_walk<false>(p.s, cur.rec, cur.screen[0], cur.screen[1], V3(0.0f, 0.0f, 0.0f), S.rec, e,
                                      lsx, ax, lensPos);
    if (!(okx && lsx > 0.0f)) {
        sc.flags = (sc.flags & ~kLens) | kAniso;
        atomicAdd(p.d.stats + kStatH2mc, 1ull);
        p.d.listS[atomicAdd(&p.d.counters[2], 1)] = i;
        if (!cur.gaussInit) p.d.listX[atomicAdd(&p.d.counters[0], 1)] = i;
        p.d.listA[atomicAdd(&p.d.counters[3], 1)] = i;
        return;
    }
    atomicAdd(p.d.stats + kStatLens, 1ull);
    const H2mcParam prm(p.lensSigma);
    LensGauss gx;
    lens_gaussian_of(p.s, cur.rec, ax, cur.screen[0], cur.screen[1], lsx, cur.ss, p.maxDerv, prm, gx);
    Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
    const double z0 = double(rng.normal()), z1 = double(rng.normal());
    const double w0 = z0 / ::sqrt(gx.p[0]), w1 = z1 / ::sqrt(gx.p[1]);
    float off[2];
    for (int r = 0; r < 2; r++) off[r] = float(gx.mean[r] + gx.V[r * 2] * w0 + gx.V[r * 2 + 1] * w1);
    const float sx = mod1(cur.screen[0] + off[0]), sy = mod1(cur.screen[1] + off[1]);
    float lsz;
    LensAnchor az;
    V3 lensPosZ;
    const bool okz = lens_walk<true>(p.s, cur.rec, sx, sy, lensPos, S.rec, e, lsz, az, lensPosZ);
    float a2 = 0.0f;
    S.gaussInit = 0;
    if (okz) {
        sc.flags |= kZValid;
        set_contrib(S, e, p.b);
        LensGauss gz;
        lens_gaussian_of(p.s, S.rec, az, e.screen[0], e.screen[1], lsz, e.ss, p.maxDerv, prm, gz);
        const double px = lens_logpdf(gz, off, -1.0), py = lens_logpdf(gx, off, 1.0);
        a2 = float(::exp(px - py)) * lsz / lsx;
    } else {
        S.hasSplat = 0;
    }
    sc.a2 = a2;
}

// Green's reverse path y* = z + (x - y) and its first-stage acceptance from z
// (SmallStep::Trace, mutation.cpp:210-238), over the second-stage list only.
// Prologue: false (aStar = 0 written) when z holds no valid state.
DEV bool ystar_begin(const RunParams &p, int i, int iter, Rng &rng, float *off, PathM &m) {
    Scratch &sc = p.d.scr[i];
    const Slot &cur = slot_of(p.d, i, 0);
    const Slot &F = slot_of(p.d, i, 1);
    const Slot &S = slot_of(p.d, i, 2);
    if (!S.valid) {
        sc.aStar = 0.0f;
        return false;
    }
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    for (int k = 0; k < dim; k++) off[k] = cur.rec.u[k] - F.rec.u[k];
    rng = Rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 3ull);
    m.pc = kPStart;
    return true;
}
DEV void ystar_end(const RunParams &p, int i, int st, const Emit &e) {
    const Slot &S = slot_of(p.d, i, 2);
    p.d.scr[i].aStar = st == kStepDone ? clamp01(e.ss / S.ss) : 0.0f;
}

static __global__ void __launch_bounds__(kStageBlock) k_ystar(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = sparse_index(p.lanes2, on);
    const int n = p.d.counters[2];
    if (!on || t >= n) return;
    const int i = longest_first(p.d.listS, n, t);
    Rng rng;
    float off[kMaxDim];
    PathM m;
    if (!ystar_begin(p, i, iter, rng, off, m)) return;
    PathRec ystar;
    const int st = run_perturb(p.s, slot_of(p.d, i, 2).rec, off, rng, ystar, m);
    ystar_end(p, i, st, m.e);
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

// log of Mira's transition-kernel ratio Q1(z, y) / Q1(x, y) with the isotropic
// first-stage kernel of sigma1 (delayed.cpp:512-523: GaussianLogPdf(z - y) -
// GaussianLogPdf(x - y), whose normalisation terms cancel), in FP64.
DEV double mira_log_q(int dim, const float *x, const float *y, const float *z, float sigma1) {
    const double inv2s2 = 0.5 / (double(sigma1) * double(sigma1));
    return -inv2s2 * (iso_quad(dim, z, y) - iso_quad(dim, x, y));
}

// The second-stage acceptance probability of delayed rejection for a valid
// (non-negative, finite) second-stage ratio a2 and the first stage's a1:
//   Green & Mira (2001) (delayed.cpp:473-500): min(1, a2 (1 - a*) / (1 - a1))
//     with a* the acceptance of Green's reverse path y* (aStarGreen; an invalid
//     value counts as 0), 0 when a* = 1;
//   Tierney & Mira (1999) (delayed.cpp:502-541): a* = min(1, ss(y) / ss(z)) (an
//     invalid value counts as 1), 0 when a* = 1, else min(1, a2 Q (1 - a*) /
//     (1 - a1)) with Q = Q1(z, y) / Q1(x, y), 0 when Q is invalid.
// `draw` is set when a uniform decides the acceptance (not when the proposal is
// rejected outright); x, y, z are the primary vectors of the current state and
// the two proposals.
DEV float dr_second_acceptance(int drType, float a1, float a2, float aStarGreen, float ssY, float ssZ, int dim,
                               const float *x, const float *y, const float *z, float sigma1, bool &draw) {
    draw = false;
    if (drType == 0) {
        float aStar = aStarGreen;
        if (is_invalid(aStar)) aStar = 0.0f;
        if (aStar == 1.0f) return 0.0f;
        draw = true;
        return metropolis_clamp(a2 * (1.0f - aStar) / (1.0f - a1));
    }
    float aStar = metropolis_clamp(ssY / ssZ);
    if (is_invalid(aStar)) aStar = 1.0f;
    if (aStar == 1.0f) return 0.0f;
    const float transRatio = float(::exp(mira_log_q(dim, x, y, z, sigma1)));
    if (is_invalid(transRatio)) return 0.0f;
    draw = true;
    return metropolis_clamp(a2 * transRatio * (1.0f - aStar) / (1.0f - a1));
}

// ------------------------------------------------------------- finish
// The end of chain i's iteration `iter` (delayed.cpp:466-606): Green or Mira
// second-stage acceptance, the weighted splats (returned in sp[0..2] as
// pending splats; pixel -1 = none), accept / swap and the statistics.
DEV void finish_chain(const RunParams &p, int i, int iter, StatAcc &acc, PendingSplat *sp) {
    const int W = p.s.cam.width, H = p.s.cam.height;
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
        } else if (flags & kSingle) {
            // the usual MH acceptance, Clamp(a, 0, 1) (h2mc.cpp:580-584, 220)
            a2 = clamp01(a2);
            accept2 = flip_coin(a2, rng.uniform());
        } else {
            bool draw;
            a2 = dr_second_acceptance(p.drType, a1, a2, sc.aStar, F.ss, S.ss, dim, cur.rec.u, F.rec.u, S.rec.u,
                                      p.sigma1, draw);
            if (draw) accept2 = flip_coin(a2, rng.uniform());
        }
        if (accept2) {
            if (flags & kLens) atomicAdd(p.d.stats + kStatLensAcc, 1ull);
            else acc.c[aniso ? kStatH2mcAcc : kStatIsoAcc]++;
        }
    }
    // weighted splats (delayed.cpp:547-561)
    const float w1 = a1;
    const float w2 = (1.0f - w1) * a2;
    const float wc = 1.0f - w1 - w2;
    if (!p.accMap) {
        if (cur.valid && wc > 0.0f && cur.hasSplat) sp[0] = weighted_splat_of(W, H, cur.splat, wc);
        if (w1 > 0.0f && F.hasSplat) sp[1] = weighted_splat_of(W, H, F.splat, w1);
        if (w2 > 0.0f && S.hasSplat) sp[2] = weighted_splat_of(W, H, S.splat, w2);
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
        if (p.accMap && !(flags & kLarge) && old.hasSplat)
            sp[0] = PendingSplat{splat_pixel(W, H, old.splat[0], old.splat[1], 1.0f, 0.0f, 0.0f), 1.0f, 0.0f, 0.0f};
    } else if (accept2) {
        const int t = perm[0];
        perm[0] = perm[2];
        perm[2] = t;
        Slot &nc = slot_of(p.d, i, 0);
        if (!aniso) nc.gaussInit = 0;
        nc.valid = 1;
        const Slot &old = slot_of(p.d, i, 2);
        if (p.accMap && old.hasSplat)
            sp[0] = PendingSplat{splat_pixel(W, H, old.splat[0], old.splat[1], 0.0f, 1.0f, 0.0f), 0.0f, 1.0f, 0.0f};
    }
    sc.flags = flags | (accept2 ? kAccept2 : 0);
    sc.a2 = a2;
}

static __global__ void __launch_bounds__(kStageBlock) k_finish(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = sparse_index(p.lanes, on);
    const int i = p.c0 + t;
    StatAcc acc;
    // up to three splats per chain, added warp-aggregated after the chain's work
    PendingSplat sp[3] = {{-1, 0.0f, 0.0f, 0.0f}, {-1, 0.0f, 0.0f, 0.0f}, {-1, 0.0f, 0.0f, 0.0f}};
    if (on && t < p.N && (p.d.scr[i].flags & kActive)) finish_chain(p, i, iter, acc, sp);
    for (int k = 0; k < 3; k++) warp_splat(p.d.film, sp[k]);
    flush_stats(acc, p.d.stats);
}

// MergeBuffer (src/image.h:76-93, delayed.cpp:681-685): direct * 1/directSpp +
// indirect * 1/spp per channel, rounded after every operation as the host
// loop it replaces did.
static __global__ void k_merge_film(const float4 *ind, const float4 *dir, float dw, float iw, size_t n, float *rgb) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 d = dir[i], v = ind[i];
    rgb[3 * i + 0] = __fadd_rn(__fmul_rn(dw, d.x), __fmul_rn(iw, v.x));
    rgb[3 * i + 1] = __fadd_rn(__fmul_rn(dw, d.y), __fmul_rn(iw, v.y));
    rgb[3 * i + 2] = __fadd_rn(__fmul_rn(dw, d.z), __fmul_rn(iw, v.z));
}

// One chain group's iteration counter, advanced after each of its iterations
// on the group's stream (so a captured iteration replays as the next one).
static __global__ void k_advance_iter(int *iterp) { *iterp += 1; }
static __global__ void k_set_iters(int *iters, int n, int value) {
    for (int g = threadIdx.x; g < n; g += blockDim.x) iters[g] = value;
}

// A chain group's list counters, work-class histogram and (nWave > 0) the
// queue counters of its wavefront stage passes, at the start of an iteration.
static __global__ void k_reset_counters(int *counters, int *hist, int *waveCount, int nWave) {
    if (threadIdx.x < kNumCounters) counters[threadIdx.x] = 0;
    for (int k = threadIdx.x; k < kPlanBins; k += blockDim.x) hist[k] = 0;
    for (int k = threadIdx.x; k < nWave; k += blockDim.x) waveCount[k] = 0;
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

static __global__ void __launch_bounds__(128) k_bootstrap(SceneView s, unsigned long long seed, int numSamples, int minDepth,
                                                   int maxDepth, BootRecord *out, int *count, int cap, int *overflow) {
    const int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= numSamples) return;
    Rng rng(seed, (unsigned long long)sidx, 0xB007ull);
    FullPath f;
    SinkAppend sink{out, count, cap, sidx, overflow};
    generate_path_bidir(s, minDepth, maxDepth, rng, f, sink);
}

static __global__ void __launch_bounds__(128) k_seed(RunParams p, unsigned long long bootSeed, const int *sampleOf,
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
    float4 *film;
    int W, H;
    DEV void operator()(const Emit &e) { splat(film, W, H, e.screen[0], e.screen[1], e.rgb.x, e.rgb.y, e.rgb.z); }
};

static __global__ void __launch_bounds__(128) k_direct(SceneView s, unsigned long long seed, int spp, int minDepth,
                                                int maxDepth, float4 *film) {
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
