// Host launchers of the path-derivative kernels, which are compiled in their
// own translation unit (derivs.cu).
#pragma once
#include <cuda_runtime.h>

namespace drmlt {

struct RunParams;
struct SceneView;
struct PathRec;

// adjMinDim that selects hyper-dual forward mode for every path, which is
// also the chain loop's default (drmlt_options.adjoint_min_dim = 0): with the
// adjoint from dimension 10 on, config 4's derivative stages take 0.46 / 0.56
// instead of 0.50 / 0.64 ms per iteration, but the iteration as a whole ties
// (4.02 against 4.00 ms in a time-to-relMSE loop).
constexpr int kNoAdjoint = 1 << 20;
constexpr int kDefaultAdjMinDim = kNoAdjoint;

// Gradient + Hessian of log f of path r (ss its score) for a team of `team`
// threads, `member` the caller's index in it, by hyper-dual forward mode: zero
// (the isotropic fallback) for a path longer than maxDerv segments or with
// ss <= 1e-15. g: kMaxDim floats, H: kMaxDim^2. Defined in derivs_dev.cu
// (relocatable device code,
// the derivative kernels' flags) for the persistent schedule, which takes
// hyper-dual derivatives for every path.
__device__ void persist_derivs(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H,
                               int member, int team);

// Threads per block and resident blocks per SM of the adjoint derivative kernel.
constexpr int kAdjBlock = 128;
constexpr int kAdjBlocksPerSm = 4;

// Gradient + Hessian of log f for the chains of list `which` (0: listX at the
// current states, 2: listZ at the second proposals) of one chain group: the
// hyper-dual kernel (`blocks` blocks) for paths shorter than p.adjMinDim, then
// the adjoint kernel (`adjBlocks` blocks) for the others.
void launch_derivs(const RunParams &p, int which, int blocks, int adjBlocks, cudaStream_t s);
// Resident blocks of the adjoint derivative kernel per SM.
int derivs_adj_blocks_per_sm();
// The same for caller-supplied paths and primary samples (u: n x kMaxDim),
// by the adjoint for paths of dimension adjMinDim and up (0: every path,
// kNoAdjoint: none).
void launch_gradhess_paths(const SceneView &s, const PathRec *paths, const float *u, int n, float *grad,
                           float *hess, int adjMinDim, cudaStream_t st);
// The same at each path's own primary vector, gated by path length and ss as the chain loop gates it.
void launch_gradhess_gated(const SceneView &s, const PathRec *paths, const float *ss, int n, int maxDerv, float *grad,
                           float *hess, cudaStream_t st);
cudaError_t set_derivs_carveout(int percent);
// Resident blocks of the derivative kernel per SM (its grid-stride grid).
int derivs_blocks_per_sm();

}  // namespace drmlt
