// Wavefront form of the three path-tracing stages of an iteration: stage 1
// (GenerateSubpath / PerturbPathBidir, src/path.cpp:1123-1269, 1480-1628),
// stage 2 (PerturbPathBidir) and Green's y* (SmallStep::Trace,
// src/mutation.cpp:210-238), with the BVH casts of src/scene.cpp:80-111 split
// out of the per-chain code.
//
// Per-lane path tracing leaves most lanes of a warp idle: lanes follow their
// own paths through the BVH, so a traversal runs as long as the warp's longest
// one, and the stage kernels carry the whole path sampler's registers. Here a
// stage pass runs as rounds instead:
//   k_wave_begin    per chain: the stage prologue and the path machine's first
//                   step, which parks the chain at its first ray cast;
//   k_wave_trace    one ray per lane over the round's queue (closest-hit rays
//                   from the front of the queue, shadow rays from the back, so
//                   a warp runs one kind), answers written per queue slot;
//   k_wave_advance  per queued chain: the machine consumes its answer and runs
//                   to its next ray (queued for the next round) or to its end
//                   (the stage epilogue).
// A path of L segments needs at most L + 1 casts, so max_depth + 1 rounds
// finish every valid technique; a chain still waiting after the last round is
// finished as a failed proposal (only the degenerate large step with
// camLength = lgtLength = 1, which can never connect, gets there). The
// machines, prologues and epilogues are the ones the per-lane kernels run, so
// the two schedules take identical steps.
#pragma once
#include "kernels.cuh"

namespace drmlt {

// One chain's machine between rounds (global memory; each chain has at most
// one ray in flight).
struct WaveChain {
    PathM m;
    Rng rng;              // the stage's random stream
    float off[kMaxDim];   // the proposal's offsets
    int mode;             // sampler (kTrace*)
    int flags;            // stage-1 flags of the prologue
};

constexpr int kWaveBlock = 128;
constexpr int kWaveMaxRounds = kMaxLen + 1;
constexpr int kWaveCountStride = 2 * (kWaveMaxRounds + 1);  // counters of one stage pass

// One chain group's queues for one stage pass.
struct WaveView {
    WaveChain *chains;  // indexed by chain
    PathRec *ystar;     // indexed by chain: Green's reverse path (the y* perturbation's output)
    int *q[2];          // per slot: the chain (double-buffered by round parity)
    float4 *rayO[2];    // per slot: origin, tmin
    float4 *rayD[2];    // per slot: direction, tmax
    int *hit;           // per slot: the answer of the current round
    int *count;         // round r: count[2r] closest-hit rays in slots 0, 1, ...,
                        // count[2r + 1] shadow rays in slots cap - 1, cap - 2, ...
    int cap;            // slots per queue (the group's chains)
    int rounds;
};

DEV int wave_slot(int t, int nClosest, int nAny, int cap) {
    if (t < nClosest) return t;
    if (t < nClosest + nAny) return cap - 1 - (t - nClosest);
    return -1;
}

// Queues the pending ray of every lane with `want` set for round r: one atomic
// per warp and ray kind. Every lane of the warp calls it.
DEV void wave_push(const WaveView &w, int r, bool want, int chain, const PathM *m) {
    const bool closest = want && m->kind == kRayClosest;
    const bool any = want && !closest;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned below = (1u << lane) - 1u;
    const unsigned mc = __ballot_sync(0xffffffffu, closest);
    const unsigned ma = __ballot_sync(0xffffffffu, any);
    if (!(mc | ma)) return;
    int bc = 0, ba = 0;
    if (lane == 0) {
        if (mc) bc = atomicAdd(w.count + 2 * r, __popc(mc));
        if (ma) ba = atomicAdd(w.count + 2 * r + 1, __popc(ma));
    }
    bc = __shfl_sync(0xffffffffu, bc, 0);
    ba = __shfl_sync(0xffffffffu, ba, 0);
    if (!want) return;
    const int slot = closest ? bc + __popc(mc & below) : w.cap - 1 - (ba + __popc(ma & below));
    const int b = r & 1;
    w.q[b][slot] = chain;
    w.rayO[b][slot] = make_float4(m->org.x, m->org.y, m->org.z, m->tmin);
    w.rayD[b][slot] = make_float4(m->dir.x, m->dir.y, m->dir.z, m->tmax);
}

// One machine step of stage kStage (1: stage 1, 2: stage 2, 3: Green's y*).
template <int kStage>
DEV int wave_step(const RunParams &p, const WaveView &w, int i, WaveChain &wc, int hit) {
    if (kStage == 1) {
        if (wc.mode == kTraceSubpath) return subpath_step(p.s, wc.rng, slot_of(p.d, i, 1).rec, wc.m, hit);
        return perturb_step(p.s, slot_of(p.d, i, 0).rec, wc.off, wc.rng, slot_of(p.d, i, 1).rec, wc.m, hit);
    }
    if (kStage == 2) return perturb_step(p.s, slot_of(p.d, i, 0).rec, wc.off, wc.rng, slot_of(p.d, i, 2).rec, wc.m, hit);
    return perturb_step(p.s, slot_of(p.d, i, 2).rec, wc.off, wc.rng, w.ystar[i], wc.m, hit);
}

template <int kStage>
DEV void wave_end(const RunParams &p, int i, WaveChain &wc, int st, StatAcc &acc) {
    if (kStage == 1) stage1_end(p, i, wc.mode, wc.flags, wc.rng, st, wc.m.e, acc);
    if (kStage == 2) stage2_end(p, i, st, wc.m.e);
    if (kStage == 3) ystar_end(p, i, st, wc.m.e);
}

// Round 0: the stage prologue of every chain of the pass (stage 1: the group's
// chains in k_scatter's order; stages 2 and 3: the second-stage list) and the
// first machine step.
template <int kStage>
__global__ void __launch_bounds__(kWaveBlock) k_wave_begin(RunParams p, WaveView w) {
    const int iter = *p.iterp;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = kStage == 1 ? p.N : p.d.counters[2];
    StatAcc acc;
    bool want = false;
    int chain = -1;
    WaveChain *wc = nullptr;
    if (t < n) {
        chain = kStage == 1 ? p.d.order[t] : p.d.listS[t];
        wc = &w.chains[chain];
        int mode = kTracePerturb;
        if (kStage == 1) mode = stage1_begin(p, chain, iter, wc->rng, wc->off, wc->m, wc->flags, acc);
        if (kStage == 2) stage2_begin(p, chain, iter, wc->rng, wc->off, wc->m);
        if (kStage == 3) mode = ystar_begin(p, chain, iter, wc->rng, wc->off, wc->m) ? kTracePerturb : kTraceNone;
        wc->mode = mode;
        if (mode == kTraceFail) {
            wave_end<kStage>(p, chain, *wc, kStepFail, acc);
        } else if (mode != kTraceNone) {
            const int st = wave_step<kStage>(p, w, chain, *wc, -1);
            if (st == kStepRay) want = true;
            else wave_end<kStage>(p, chain, *wc, st, acc);
        }
    }
    wave_push(w, 0, want, chain, wc ? &wc->m : nullptr);
    if (kStage == 1) flush_stats(acc, p.d.stats);
}

// Round r's casts: closest hits (the BVH's triangle or -1) and shadow rays
// (1 when occluded).
__global__ void __launch_bounds__(kWaveBlock) k_wave_trace(SceneView s, WaveView w, int r) {
    const int nc = w.count[2 * r], na = w.count[2 * r + 1];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nc + na) return;
    const int slot = wave_slot(t, nc, na, w.cap);
    const int b = r & 1;
    const float4 a = w.rayO[b][slot], d4 = w.rayD[b][slot];
    const V3 o(a.x, a.y, a.z), d(d4.x, d4.y, d4.z);
    w.hit[slot] = t < nc ? traverse<false>(s, o, d, a.w, d4.w) : (traverse<true>(s, o, d, a.w, d4.w) >= 0 ? 1 : 0);
}

// Round r's machine steps; rays for round r + 1 (after the last round a chain
// still waiting finishes as a failed proposal).
template <int kStage>
__global__ void __launch_bounds__(kWaveBlock) k_wave_advance(RunParams p, WaveView w, int r) {
    const int nc = w.count[2 * r], na = w.count[2 * r + 1];
    if (int(blockIdx.x * blockDim.x) >= nc + na) return;  // the whole block is past the queue
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int slot = wave_slot(t, nc, na, w.cap);
    StatAcc acc;
    bool want = false;
    int chain = -1;
    WaveChain *wc = nullptr;
    if (slot >= 0) {
        chain = w.q[r & 1][slot];
        wc = &w.chains[chain];
        const int st = wave_step<kStage>(p, w, chain, *wc, w.hit[slot]);
        if (st == kStepRay && r + 1 < w.rounds) want = true;
        else wave_end<kStage>(p, chain, *wc, st == kStepRay ? kStepFail : st, acc);
    }
    wave_push(w, r + 1, want, chain, wc ? &wc->m : nullptr);
    if (kStage == 1) flush_stats(acc, p.d.stats);
}

}  // namespace drmlt
