// derivs_for_path as an external device function for the persistent
// schedule (persist.cu), which is compiled without fast math: relocatable
// device code with the derivative kernels' flags, held to the 128 registers of
// the kernel that calls it.
#include "derivs.h"
#include "derivs_path.cuh"

namespace drmlt {

__device__ void persist_derivs(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H,
                               int member, int team) {
    // hyper-dual forward mode for every path, the body k_derivs runs (the
    // reverse-mode adjoint is a staged-schedule option: compiled into this
    // relocatable unit, its rounding would differ from k_derivs_adj's)
    derivs_for_path<false>(s, r, ss, maxDerv, g, H, member, team, kNoAdjoint);
}

}  // namespace drmlt
