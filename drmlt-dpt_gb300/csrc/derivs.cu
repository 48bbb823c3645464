// Path derivatives for H2MC: gradient and Hessian of log f with respect to the
// primary sample coordinates (the chad-generated evaluate_path_bidir_*_derv of
// the reference, registered in src/path.cpp:2987-3175), by hyper-dual forward
// mode on the AD path function of pathad.cuh or, for paths of dimension
// adjMinDim and up, by its reverse-mode adjoint with forward-over-reverse
// Hessian rows (pathadj.cuh).
#include "chain.cuh"
#include "derivs.h"
#include "derivs_path.cuh"

namespace drmlt {

// A team of p.derivWarps warps per listed chain shares its Hessian entries. The
// grid is sized for the GPU: team t takes list entries t, t + teams, ...
// Four resident blocks per SM (128 registers a thread, 16 warps) hide more of
// the instruction-fetch and memory latency than the 254 registers the
// compiler takes unbounded (8 warps), for 28 bytes of spills: config 2 0.843 ->
// 0.815 ms per iteration (three blocks 0.822, five 0.825), config 4 6.09 ->
// 5.73 ms. Entries of dimension p.adjMinDim and up are left to k_derivs_adj
// (their derivatives wanted: path length <= maxDerv, ss > 1e-15).
__global__ void __launch_bounds__(128, 4) k_derivs(RunParams p, int which) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int teams = (gridDim.x * blockDim.x >> 5) / p.derivWarps;
    const int n = p.d.counters[which == 0 ? 0 : 1];
    for (int k = gw / p.derivWarps; k < n; k += teams) {
        const int w = n - 1 - k;  // longest paths first: the lists fill in the order their stage finishes
        const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
        const Slot &st = slot_of(p.d, chain, which);
        const int L = st.rec.c + st.rec.l - 1;
        if (derivs_wanted(L, st.ss, p.maxDerv) && 2 * L >= p.adjMinDim) continue;
        derivs_for_path<false>(p.s, st.rec, st.ss, p.maxDerv, p.d.grad + size_t(w) * kMaxDim,
                               p.d.hess + size_t(w) * kMaxDim * kMaxDim, (gw % p.derivWarps) * 32 + (threadIdx.x & 31),
                               32 * p.derivWarps, kNoAdjoint);
    }
}

// The list entries of dimension p.adjMinDim and up by the reverse-mode
// adjoint: one warp per chain, one Hessian row (a forward and a backward sweep
// in Dual numbers) per lane. A separate kernel, so that the hyper-dual kernel
// keeps its register bound. At 4 blocks per SM (128 registers, the adjoint's
// Dual state, adjoints and checkpoints partly spilled) it runs faster than at
// 2 (255 registers) or 5-8 (more spills): config 4, every derivative by the
// adjoint, 0.72 / 0.63 / 0.55 / 0.57 / 0.62 / 0.68 ms at x for 2 / 3 / 4 / 5 /
// 6 / 8 blocks. Two chains per warp (a half-warp each when both have at most
// 16 rows) measured slower still (0.78 ms): the two paths diverge. So did
// out-of-line copies of the BSDF adjoints and of the forward BSDF calls (0.68
// ms: the Dual arguments go through the stack; ncu had shown instruction-fetch
// stalls, 14 a issued instruction, as the kernel's first limiter).
__global__ void __launch_bounds__(kAdjBlock, kAdjBlocksPerSm) k_derivs_adj(RunParams p, int which) {
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps = gridDim.x * blockDim.x >> 5;
    const int n = p.d.counters[which == 0 ? 0 : 1];
    const int lane = threadIdx.x & 31;
    for (int k = gw; k < n; k += warps) {
        const int w = n - 1 - k;  // longest paths first: the lists fill in the order their stage finishes
        const int chain = (which == 0 ? p.d.listX : p.d.listZ)[w];
        const Slot &st = slot_of(p.d, chain, which);
        const int L = st.rec.c + st.rec.l - 1;
        const int dim = 2 * L;
        if (!(derivs_wanted(L, st.ss, p.maxDerv) && dim >= p.adjMinDim)) continue;
        derivs_adj_for_path(p.s, st.rec, dim, p.d.grad + size_t(w) * kMaxDim, p.d.hess + size_t(w) * kMaxDim * kMaxDim,
                            lane, 32);
    }
}

int derivs_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_derivs, 128, 0) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}

__global__ void __launch_bounds__(128) k_gradhess_paths(SceneView s, const PathRec *paths, const float *u, int n,
                                                        float *grad, float *hess, int adjMinDim) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= n) return;
    PathRec r = paths[w];
    const int dim = path_dim(r.c, r.l);
    for (int k = 0; k < dim; k++) r.u[k] = u[size_t(w) * kMaxDim + k];
    // derivatives are always taken here (no ss / depth gate)
    derivs_for_path(s, r, 1.0f, kMaxLen, grad + size_t(w) * kMaxDim, hess + size_t(w) * kMaxDim * kMaxDim,
                    threadIdx.x & 31, 32, adjMinDim);
}

// Gradient + Hessian at each path's own primary vector, gated as in the chain
// loop: zero (the isotropic fallback of drsmallstep.cpp:133-163) for a path
// longer than maxDerv segments or with ss <= 1e-15.
__global__ void __launch_bounds__(128) k_gradhess_gated(SceneView s, const PathRec *paths, const float *ss, int n,
                                                        int maxDerv, float *grad, float *hess) {
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= n) return;
    derivs_for_path<false>(s, paths[w], ss[w], maxDerv, grad + size_t(w) * kMaxDim,
                           hess + size_t(w) * kMaxDim * kMaxDim, threadIdx.x & 31, 32, kNoAdjoint);
}

void launch_gradhess_gated(const SceneView &s, const PathRec *paths, const float *ss, int n, int maxDerv, float *grad,
                           float *hess, cudaStream_t st) {
    k_gradhess_gated<<<(n * 32 + 127) / 128, 128, 0, st>>>(s, paths, ss, n, maxDerv, grad, hess);
}

void launch_derivs(const RunParams &p, int which, int blocks, int adjBlocks, cudaStream_t s) {
    k_derivs<<<blocks, 128, 0, s>>>(p, which);
    if (p.adjMinDim <= kMaxDim) k_derivs_adj<<<adjBlocks, kAdjBlock, 0, s>>>(p, which);
}

int derivs_adj_blocks_per_sm() {
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_derivs_adj, kAdjBlock, 0) != cudaSuccess) n = 1;
    return n > 0 ? n : 1;
}

void launch_gradhess_paths(const SceneView &s, const PathRec *paths, const float *u, int n, float *grad,
                           float *hess, int adjMinDim, cudaStream_t st) {
    k_gradhess_paths<<<(n * 32 + 127) / 128, 128, 0, st>>>(s, paths, u, n, grad, hess, adjMinDim);
}

cudaError_t set_derivs_carveout(int percent) {
    cudaError_t e = cudaFuncSetAttribute(k_derivs, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_derivs_adj, cudaFuncAttributePreferredSharedMemoryCarveout, percent);
}

}  // namespace drmlt
