// Persistent schedule of the DRMLT chain loop (delayed.cpp:334-673): one
// cooperative launch runs every chain through all of its iterations, with no
// barrier between stages or iterations.
//
// In the staged schedule each stage is a kernel over all chains, so an
// iteration costs the sum over stages of the slowest chain in each stage
// (paths of 2 to 13 vertices: the longest trace sets every stage kernel's
// length while most SMs idle). Here chains move independently through two
// work queues:
//   lane queue  chains ready for path tracing. Lane workers (one chain per
//               active lane) run a chain's stage 1 (large step or sigma1
//               perturbation), its isotropic second stage, Green's y* and the
//               finish -- iteration after iteration -- until the chain needs an
//               H2MC Gaussian or has done its iterations;
//   team queue  chains that need the Gaussian at the current state x (before
//               the H2MC proposal) or at the proposal z (for the ratio). Team
//               workers (a block of four warps per chain) compute the
//               gradient and Hessian of log f (derivs.cu), the FP64-refined
//               Gaussian, and the H2MC offset or kernel ratio, and hand the
//               chain back to the lane queue.
// A chain is in at most one queue or one worker at a time, and its random
// streams are keyed by (seed, chain, iteration, stage), so every chain takes
// exactly the steps it takes under the staged schedule; only the order of the
// film's float additions changes.
//
// Roles are assigned per SM (%smid < teamSms: team workers), so each SM keeps
// one role's code in its instruction cache. The launch is cooperative: every
// block is resident, so a queued chain is always taken by a running worker.
// Every wait is bounded: a worker that sees no progress (no queue push and no
// chain finishing) for `waitLimit` polls, or a queue cell that is not handed
// over within the limit, sets a status bit and returns; the host turns it into
// DRMLT_E_TIMEOUT.
#include <cuda/atomic>

#include "kernels.cuh"
#include "persist.h"

namespace drmlt {

namespace {

using AtomicU64 = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
using AtomicI32 = cuda::atomic_ref<int, cuda::thread_scope_device>;

enum : int { kPhS1 = 0, kPhS2 = 1, kPhYS = 2 };
enum : int { kCtlLaneHead = 0, kCtlLaneTail, kCtlTeamHead, kCtlTeamTail, kCtlProgress, kCtlDone, kCtlCount };

// A bounded multi-producer multi-consumer queue (D. Vyukov's cell-sequence
// scheme): cell s % cap is free for the push of slot s when its sequence is
// s, holds that push's value when it is s + 1, and is released for slot
// s + cap by the pop.
struct QCell {
    unsigned long long seq;
    int val;
    int pad;
};
static_assert(sizeof(QCell) == 16, "queue cell");

struct PQueue {
    QCell *cells;
    unsigned long long *head, *tail;
    unsigned long long cap;
};

struct PersistView {
    PQueue lane, team;
    unsigned long long *progress, *done;
    int *status;
    int *chainIter, *chainPhase;
    PathRec *ystar;
    float *rows;
    long long end;        // iteration every chain runs up to (capped by its samples)
    int teamSms;
    long long waitLimit;  // idle polls without progress before giving up
};

DEV unsigned long long load_acq(unsigned long long *p) { return AtomicU64(*p).load(cuda::memory_order_acquire); }
DEV unsigned long long load_rlx(unsigned long long *p) { return AtomicU64(*p).load(cuda::memory_order_relaxed); }
DEV int status_of(const PersistView &v) { return AtomicI32(*v.status).load(cuda::memory_order_relaxed); }
DEV void fail_with(const PersistView &v, int bit) { atomicOr(v.status, bit); }

DEV long long target_of(const RunParams &p, const PersistView &v, int i) {
    const long long s = samples_of(p, i);
    return v.end < s ? v.end : s;
}

// Push by one thread. Returns false when the cell was not released in time.
DEV bool q_push(const PQueue &q, const PersistView &v, int val) {
    const unsigned long long s = atomicAdd(q.tail, 1ull);
    QCell &c = q.cells[s % q.cap];
    for (long long k = 0; load_acq(&c.seq) != s; k++) {
        if (k > v.waitLimit) {
            fail_with(v, kPersistCellWait);
            return false;
        }
        __nanosleep(32);
    }
    c.val = val;
    AtomicU64(c.seq).store(s + 1, cuda::memory_order_release);
    atomicAdd(v.progress, 1ull);
    return true;
}

// Claims up to `want` slots (one thread); returns the first, *got the count.
DEV unsigned long long q_claim(const PQueue &q, int want, int *got) {
    unsigned long long h = load_rlx(q.head);
    for (int tries = 0; tries < 32; tries++) {
        const unsigned long long t = load_rlx(q.tail);
        if (t <= h) break;
        const unsigned long long k = t - h < (unsigned long long)want ? t - h : (unsigned long long)want;
        if (AtomicU64(*q.head).compare_exchange_weak(h, h + k, cuda::memory_order_relaxed)) {
            *got = int(k);
            return h;
        }
    }
    *got = 0;
    return 0;
}

// Takes the value of claimed slot s (its push may still be completing).
// Returns -1 when it was not handed over in time.
DEV int q_take(const PQueue &q, const PersistView &v, unsigned long long s) {
    QCell &c = q.cells[s % q.cap];
    for (long long k = 0; load_acq(&c.seq) != s + 1; k++) {
        if (k > v.waitLimit) {
            fail_with(v, kPersistCellWait);
            return -1;
        }
        __nanosleep(32);
    }
    const int val = c.val;
    AtomicU64(c.seq).store(s + q.cap, cuda::memory_order_release);
    return val;
}

// ------------------------------------------------------------------ lane workers
struct LaneCtx {
    int chain;   // -1: the lane holds no chain
    int iter;
    int phase;
    int mode;    // stage-1 machine (kTrace*)
    int flags;   // stage-1 flags of the prologue
    int traced;  // the current phase traced a path (else it ended in its prologue)
    int rays;    // rays the current phase has cast
    bool want;   // a ray is pending
    bool fresh;  // the phase starts at its prologue
    Rng rng;
    float off[kMaxDim];
    PathM m;
};

// GenerateSample (src/gaussian.cpp:36-47) for chain i by one lane: the same
// FP64 operations, element by element and in the same order, as the warp form
// (h2mc_offset_warp), used when the Gaussian at x is still valid.
DEV void h2mc_offset_lane(const RunParams &p, int i, int iter) {
    const Slot &cur = slot_of(p.d, i, 0);
    const int dim = path_dim(cur.rec.c, cur.rec.l);
    const GaussView g(gauss_of(p.d, i, 0));
    Rng rng(p.seed, (unsigned long long)i, (unsigned long long)iter * 4ull + 1ull);
    double zs[kMaxDim];
    for (int k = 0; k < dim; k++) zs[k] = double(rng.normal());
    for (int k = 0; k < dim; k++) zs[k] /= ::sqrt(g.p[k]);
    for (int l = 0; l < dim; l++) {
        double o = g.mean[l];
        for (int k = 0; k < dim; k++) o = ::fma(g.V[l * dim + k], zs[k], o);
        p.d.scr[i].offset[l] = float(o);
    }
}

// One step of the chain's current path machine with the answer `hit` to its
// last ray (-1 at the first step).
DEV int lane_step(const RunParams &p, const PersistView &v, LaneCtx &c, int hit) {
    const int i = c.chain;
    if (c.phase == kPhS1 && c.mode == kTraceSubpath) return subpath_step(p.s, c.rng, slot_of(p.d, i, 1).rec, c.m, hit);
    const PathRec *in = &slot_of(p.d, i, c.phase == kPhYS ? 2 : 0).rec;
    PathRec *out = c.phase == kPhS1 ? &slot_of(p.d, i, 1).rec : (c.phase == kPhS2 ? &slot_of(p.d, i, 2).rec : &v.ystar[i]);
    return perturb_step(p.s, *in, c.off, c.rng, *out, c.m, hit);
}

// Hands the chain to the team queue (job 2 i + (which == 2)) and releases the lane.
DEV bool lane_to_team(const PersistView &v, LaneCtx &c, int which, int phaseAfter) {
    v.chainIter[c.chain] = c.iter;
    v.chainPhase[c.chain] = phaseAfter;
    __threadfence();
    q_push(v.team, v, 2 * c.chain + (which == 2 ? 1 : 0));
    return false;
}

// Advances the lane's chain until it has a ray pending (returns true) or
// leaves the lane (false): `st` is the machine's result after the last answer
// (ignored when c.fresh: the phase starts at its prologue).
DEV bool lane_advance(const RunParams &p, const PersistView &v, LaneCtx &c, int st, StatAcc &acc) {
    const int i = c.chain;
    for (int guard = 0; guard < 4 * kMaxLen + 16; guard++) {
        if (c.fresh) {
            c.fresh = false;
            c.traced = 0;
            c.rays = 0;
            if (c.phase == kPhS1) {
                if (c.iter >= target_of(p, v, i)) {
                    v.chainIter[i] = c.iter;
                    __threadfence();
                    atomicAdd(v.done, 1ull);
                    atomicAdd(v.progress, 1ull);
                    return false;
                }
                c.mode = stage1_begin(p, i, c.iter, c.rng, c.off, c.m, c.flags, acc);
                if (c.mode == kTraceSubpath || c.mode == kTracePerturb) {
                    c.traced = 1;
                    st = lane_step(p, v, c, -1);
                } else if (c.mode == kTraceFail) {
                    st = kStepFail;  // an empty large step
                } else {
                    // kTraceNone: an exhausted chain or the h2mc integrator's single
                    // stage, neither of which this schedule runs
                    fail_with(v, kPersistBadPhase);
                    return false;
                }
            } else if (c.phase == kPhS2) {
                stage2_begin(p, i, c.iter, c.rng, c.off, c.m);
                c.traced = 1;
                st = lane_step(p, v, c, -1);
            } else if (c.phase == kPhYS) {
                if (p.drType == 0 && ystar_begin(p, i, c.iter, c.rng, c.off, c.m)) {
                    c.traced = 1;
                    st = lane_step(p, v, c, -1);
                }
            } else {
                fail_with(v, kPersistBadPhase);
                return false;
            }
        }
        if (c.traced && st == kStepRay) {
            // a path of L segments casts at most L + 1 rays (a bound the
            // machines keep by construction; this only guards the loop)
            if (++c.rays > 4 * (kMaxLen + 2)) {
                fail_with(v, kPersistBadPhase);
                return false;
            }
            return true;
        }
        // the phase's path is finished (or there was none)
        bool finish = false;
        if (c.phase == kPhS1) {
            stage1_end(p, i, c.mode, c.flags, c.rng, st, c.m.e, acc);
            const int flags = p.d.scr[i].flags;
            if (!(flags & kSecond)) {
                finish = true;
            } else if (flags & kAniso) {
                if (!slot_of(p.d, i, 0).gaussInit) return lane_to_team(v, c, 0, kPhS2);
                h2mc_offset_lane(p, i, c.iter);
                c.phase = kPhS2;
                c.fresh = true;
            } else {
                c.phase = kPhS2;
                c.fresh = true;
            }
        } else if (c.phase == kPhS2) {
            stage2_end(p, i, st, c.m.e);
            const int flags = p.d.scr[i].flags;
            if ((flags & kAniso) && (flags & kZValid)) return lane_to_team(v, c, 2, kPhYS);
            c.phase = kPhYS;
            c.fresh = true;
        } else {
            if (c.traced) ystar_end(p, i, st, c.m.e);
            finish = true;
        }
        if (finish) {
            PendingSplat sp[3] = {{-1, 0.0f, 0.0f, 0.0f}, {-1, 0.0f, 0.0f, 0.0f}, {-1, 0.0f, 0.0f, 0.0f}};
            finish_chain(p, i, c.iter, acc, sp);
            for (int k = 0; k < 3; k++)
                if (sp[k].px >= 0) atomicAdd(p.d.film + sp[k].px, make_float4(sp[k].r, sp[k].g, sp[k].b, 0.0f));
            c.iter++;
            c.phase = kPhS1;
            c.fresh = true;
        }
    }
    fail_with(v, kPersistBadPhase);
    return false;
}

DEV void lane_worker(const RunParams &p, const PersistView &v, StatAcc &acc) {
    constexpr unsigned kFull = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool on = lane < p.lanes;
    LaneCtx c;
    c.chain = -1;
    c.want = false;
    c.fresh = false;
    unsigned long long lastProgress = 0;
    long long idle = 0;
    for (unsigned loop = 0;; loop++) {
        // idle lanes take chains from the lane queue (one claim per warp)
        const unsigned need = __ballot_sync(kFull, on && c.chain < 0);
        if (need) {
            const int leader = __ffs(need) - 1;
            int got = 0;
            unsigned long long base = 0;
            if (lane == leader) base = q_claim(v.lane, __popc(need), &got);
            got = __shfl_sync(kFull, got, leader);
            base = __shfl_sync(kFull, base, leader);
            const int rank = __popc(need & ((1u << lane) - 1u));
            if (on && c.chain < 0 && rank < got) {
                const int i = q_take(v.lane, v, base + (unsigned long long)rank);
                if (i >= 0) {
                    __threadfence();
                    c.chain = i;
                    c.iter = v.chainIter[i];
                    c.phase = v.chainPhase[i];
                    c.fresh = true;
                    c.want = false;
                }
            }
        }
        // rays of the lanes that have one (one traversal call for the warp)
        int hit = -1;
        if (c.chain >= 0 && c.want) hit = answer_ray(p.s, c.m);
        if (c.chain >= 0) {
            const int st = c.fresh ? kStepFail : lane_step(p, v, c, hit);
            c.want = lane_advance(p, v, c, st, acc);
            if (!c.want) c.chain = -1;
        }
        const bool busy = __any_sync(kFull, c.chain >= 0);
        if ((loop & 15u) == 0u || !busy) {
            int stop = 0;
            if (lane == 0) {
                if (status_of(v) != 0) {
                    stop = 1;
                } else if (!busy) {
                    if (load_rlx(v.done) >= (unsigned long long)p.N) {
                        stop = 1;
                    } else {
                        const unsigned long long pr = load_rlx(v.progress);
                        if (pr != lastProgress) {
                            lastProgress = pr;
                            idle = 0;
                        } else if (++idle > v.waitLimit) {
                            fail_with(v, kPersistIdleLane);
                            stop = 1;
                        } else {
                            __nanosleep(128);
                        }
                    }
                }
            }
            if (__shfl_sync(kFull, stop, 0)) break;
        }
    }
}

// ------------------------------------------------------------------ team workers
// Thread 0 takes the next job (2 chain + which), or -1 to stop.
DEV int team_next(const RunParams &p, const PersistView &v) {
    unsigned long long lastProgress = load_rlx(v.progress);
    long long idle = 0;
    for (;;) {
        int got = 0;
        const unsigned long long s = q_claim(v.team, 1, &got);
        if (got) return q_take(v.team, v, s);
        if (status_of(v) != 0 || load_rlx(v.done) >= (unsigned long long)p.N) return -1;
        const unsigned long long pr = load_rlx(v.progress);
        if (pr != lastProgress) {
            lastProgress = pr;
            idle = 0;
        } else if (++idle > v.waitLimit) {
            fail_with(v, kPersistIdleTeam);
            return -1;
        }
        __nanosleep(128);
    }
}

DEV void team_worker(const RunParams &p, const PersistView &v, double *gsm) {
    __shared__ int job;
    __shared__ double zs[kMaxDim];
    float *grad = v.rows + size_t(blockIdx.x) * (kMaxDim + kMaxDim * kMaxDim);
    float *hess = grad + kMaxDim;
    for (;;) {
        if (threadIdx.x == 0) {
            job = team_next(p, v);
            __threadfence();
        }
        __syncthreads();
        const int j = job;
        if (j < 0) break;
        const int i = j >> 1;
        const int which = (j & 1) ? 2 : 0;
        const Slot &st = slot_of(p.d, i, which);
        persist_derivs(p.s, st.rec, st.ss, p.maxDerv, grad, hess, threadIdx.x, blockDim.x);
        __syncthreads();
        gauss_for_chain(p, i, which, grad, hess, gsm);
        __syncthreads();
        if (which == 0 && threadIdx.x < 32) h2mc_offset_warp(p, i, v.chainIter[i], zs);
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            q_push(v.lane, v, i);
        }
        __syncthreads();  // `job` is rewritten by thread 0 next
    }
}

__global__ void __launch_bounds__(128, 4) k_persist(RunParams p, PersistView v) {
    extern __shared__ double gsm[];
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    StatAcc acc;
    if (int(smid) < v.teamSms) team_worker(p, v, gsm);
    else lane_worker(p, v, acc);
    flush_stats(acc, p.d.stats);
}

// Queues and per-chain counters at the start of a run: chains [0, m) -- the
// chains with iterations left -- fill the lane queue in order.
__global__ void k_persist_init(PersistView v, int n, int m, long long begin) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) {
        v.lane.cells[t].seq = (unsigned long long)t + (t < m ? 1ull : 0ull);
        v.lane.cells[t].val = t < m ? t : -1;
        v.team.cells[t].seq = (unsigned long long)t;
        v.team.cells[t].val = -1;
        v.chainIter[t] = int(begin);
        v.chainPhase[t] = kPhS1;
    }
    if (t == 0) {
        *v.lane.head = 0;
        *v.lane.tail = (unsigned long long)m;
        *v.team.head = 0;
        *v.team.tail = 0;
        *v.progress = 0;
        *v.done = (unsigned long long)(n - m);
        *v.status = 0;
    }
}

}  // namespace

int persist_blocks_per_sm(size_t smem, int *regs) {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persist, 128, smem) != cudaSuccess) n = 0;
    if (regs) {
        cudaFuncAttributes a{};
        *regs = cudaFuncGetAttributes(&a, k_persist) == cudaSuccess ? a.numRegs : 0;
    }
    return n;
}

cudaError_t persist_run(const RunParams &p, const PersistBuffers &b, long long begin, long long end, int grid,
                        int teamSms, long long waitLimit, size_t smem, cudaStream_t stream) {
    unsigned long long *ctl = b.ctl;
    PersistView v;
    v.lane = PQueue{static_cast<QCell *>(b.laneCells), ctl + kCtlLaneHead, ctl + kCtlLaneTail,
                    (unsigned long long)p.N};
    v.team = PQueue{static_cast<QCell *>(b.teamCells), ctl + kCtlTeamHead, ctl + kCtlTeamTail,
                    (unsigned long long)p.N};
    v.progress = ctl + kCtlProgress;
    v.done = ctl + kCtlDone;
    v.status = b.status;
    v.chainIter = b.chainIter;
    v.chainPhase = b.chainPhase;
    v.ystar = b.ystar;
    v.rows = b.rows;
    v.end = end;
    v.teamSms = teamSms;
    v.waitLimit = waitLimit;
    // chains with iterations left: all of them before the last iteration, the
    // first extraChains at it (delayed.cpp:205-210)
    int m = 0;
    if (begin < p.samplesPerChain) m = p.N;
    else if (begin == p.samplesPerChain) m = int(p.extraChains < p.N ? p.extraChains : p.N);
    if (end <= begin) m = 0;
    k_persist_init<<<(p.N + 255) / 256, 256, 0, stream>>>(v, p.N, m, begin);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (grid > b.rowBlocks) return cudaErrorInvalidValue;
    RunParams pp = p;
    void *args[] = {&pp, &v};
    return cudaLaunchCooperativeKernel(reinterpret_cast<const void *>(k_persist), dim3(grid), dim3(128), args, smem,
                                       stream);
}

}  // namespace drmlt
