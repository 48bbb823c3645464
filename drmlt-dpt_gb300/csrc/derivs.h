// Host launchers of the path-derivative kernels, which are compiled in their
// own translation unit (derivs.cu).
#pragma once
#include <cuda_runtime.h>

namespace drmlt {

struct RunParams;
struct SceneView;
struct PathRec;

// Gradient + Hessian of log f of path r (ss its score) for a team of `team`
// threads, `member` the caller's index in it: zero (the isotropic fallback)
// for a path longer than maxDerv segments or with ss <= 1e-15. g: kMaxDim
// floats, H: kMaxDim^2. Defined in derivs_dev.cu (relocatable device code,
// the derivative kernels' flags) for the persistent schedule.
__device__ void persist_derivs(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H,
                               int member, int team);

// Gradient + Hessian of log f for the chains of list `which` (0: listX at the
// current states, 2: listZ at the second proposals) of one chain group.
void launch_derivs(const RunParams &p, int which, int blocks, cudaStream_t s);
// The same for caller-supplied paths and primary samples (u: n x kMaxDim).
void launch_gradhess_paths(const SceneView &s, const PathRec *paths, const float *u, int n, float *grad,
                           float *hess, cudaStream_t st);
// The same at each path's own primary vector, gated by path length and ss as the chain loop gates it.
void launch_gradhess_gated(const SceneView &s, const PathRec *paths, const float *ss, int n, int maxDerv, float *grad,
                           float *hess, cudaStream_t st);
cudaError_t set_derivs_carveout(int percent);
// Resident blocks of the derivative kernel per SM (its grid-stride grid).
int derivs_blocks_per_sm();

}  // namespace drmlt
