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

__global__ void __launch_bounds__(kStageBlock) k_plan(RunParams p) {
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
        p.d.order[p.N - 1 - (start[sc.key] + sc.rank)] = i;  // descending class
    }
}
static_assert(2 * kScatterBlock == kPlanBins, "k_scatter scans two bins per thread");

// ------------------------------------------------------------- stage 1
__global__ void __launch_bounds__(kStageBlock) k_stage1(RunParams p) {
    const int iter = *p.iterp;
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
            } else if (p.integrator == 1 && !(rng.uniform() < p.uniformMix)) {
                // H2MCIntegrator (src/integrators/h2mc.cpp:200-240): H2MCSmallStep::Mutate
                // (h2mc.cpp:448-606) without its lens branch, as the single stage,
                // run by the second-stage kernels
                flags |= kSecond | kAniso | kSingle;
                acc.c[kStatH2mc]++;
                p.d.listS[atomicAdd(&p.d.counters[2], 1)] = i;
                if (!cur.gaussInit) p.d.listX[atomicAdd(&p.d.counters[0], 1)] = i;
                p.d.listA[atomicAdd(&p.d.counters[3], 1)] = i;
            } else {
                // SmallStep::Mutate with perturbStdDev (src/mutation.cpp:126-166); for
                // integrator=h2mc the uniform-mixing step (h2mc.cpp:454-459)
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
                    p.d.listA[atomicAdd(&p.d.counters[3], 1)] = i;
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
// k_derivs lives in derivs.cu (its own translation unit); see derivs.h.

// One block (a team of kGaussTeamWarps warps) per listed chain, with
// gauss_smem_doubles(maxDim) doubles of dynamic shared memory.
constexpr int kGaussTeamWarps = 4;
inline size_t gauss_smem_bytes(int maxDim) { return size_t(gauss_smem_doubles(maxDim)) * sizeof(double); }

DEV void gauss_for_entry(const RunParams &p, int which, int w, double *gsm) {
    const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
    Slot &st = slot_of(p.d, chain, which);
    const int dim = path_dim(st.rec.c, st.rec.l);
    GaussSmem sm(gsm, p.gaussDim);
    const Team tm(gauss_reduction(gsm, p.gaussDim));
    // dim <= gaussDim holds by construction (max_depth bounds every path); the
    // isotropic branch needs no scratch, so an impossible larger dim stays in bounds
    const int kind = compute_gaussian_team(dim, H2mcParam(p.sigma1), dim <= sm.m ? st.ss : 0.0f,
                                           p.d.grad + size_t(w) * kMaxDim, p.d.hess + size_t(w) * kMaxDim * kMaxDim, sm,
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

// The grid is sized for the GPU, not the list: each block takes list entries
// blockIdx.x, blockIdx.x + gridDim.x, ... (the list's length is known only on
// the device).
__global__ void __launch_bounds__(32 * kGaussTeamWarps) k_gauss(RunParams p, int which) {
    extern __shared__ double gsm[];
    const int n = p.d.counters[which == 0 ? 0 : 1];
    for (int w = blockIdx.x; w < n; w += gridDim.x) {
        gauss_for_entry(p, which, w, gsm);
        __syncthreads();  // the block's shared scratch is reused by its next entry
    }
}

// ------------------------------------------------------------- H2MC offsets
// GenerateSample (src/gaussian.cpp:36-47) for the chains taking the
// anisotropic second stage, one warp per chain: offset = mean + V diag(p^-1/2) n
// in FP64, with n the first dim normals of the chain's stage-2 stream (which
// k_stage2 then skips).
__global__ void __launch_bounds__(128) k_h2mc_offset(RunParams p) {
    const int iter = *p.iterp;
    __shared__ double zs[4][kMaxDim];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= p.d.counters[3]) return;
    const int i = p.d.listA[w];
    const Slot &cur = slot_of(p.d, i, 0);
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    const GaussView g(gauss_of(p.d, i, 0));
    if (lane == 0) {
        Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
        for (int k = 0; k < dim; k++) zs[wib][k] = double(rng.normal());
    }
    __syncwarp();
    if (lane < dim) zs[wib][lane] /= ::sqrt(g.p[lane]);
    __syncwarp();
    if (lane < dim) {
        double o = g.mean[lane];
        for (int k = 0; k < dim; k++) o = ::fma(g.V[lane * dim + k], zs[wib][k], o);
        p.d.scr[i].offset[lane] = float(o);
    }
}

// ------------------------------------------------------------- stage 2 proposal
// Over the group's second-stage list only (compacted by k_stage1).
__global__ void __launch_bounds__(kStageBlock) k_stage2(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = sparse_index(p.lanes2, on);
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
        // PH2MCSmallStep::Mutate (drsmallstep.cpp:113-212): the offset was
        // sampled by k_h2mc_offset from this stream's first dim normals
        for (int k = 0; k < dim; k++) {
            rng.normal();
            off[k] = sc.offset[k];
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
__global__ void __launch_bounds__(kStageBlock) k_ystar(RunParams p) {
    const int iter = *p.iterp;
    bool on;
    const int t = sparse_index(p.lanes2, on);
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
__global__ void __launch_bounds__(kStageBlock) k_finish(RunParams p) {
    const int iter = *p.iterp;
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
            } else if (flags & kSingle) {
                // the usual MH acceptance, Clamp(a, 0, 1) (h2mc.cpp:580-584, 220)
                a2 = clamp01(a2);
                accept2 = flip_coin(a2, rng.uniform());
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
                weighted_splat(p.d.film, W, H, cur.splat, wc);
            if (w1 > 0.0f && F.hasSplat)
                weighted_splat(p.d.film, W, H, F.splat, w1);
            if (w2 > 0.0f && S.hasSplat)
                weighted_splat(p.d.film, W, H, S.splat, w2);
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

// One chain group's iteration counter, advanced after each of its iterations
// on the group's stream (so a captured iteration replays as the next one).
__global__ void k_advance_iter(int *iterp) { *iterp += 1; }
__global__ void k_set_iters(int *iters, int n, int value) {
    for (int g = threadIdx.x; g < n; g += blockDim.x) iters[g] = value;
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
