// The gradient and Hessian of log f of one path by a team of threads, shared
// by the derivative kernels (derivs.cu) and, compiled separately as
// relocatable device code, by the persistent schedule (derivs_dev.cu). Both
// translation units take the derivative kernels' flags (fast-math
// intrinsics), so both give the same values.
#pragma once
#include "chain.cuh"

namespace drmlt {

// A team of `team` threads strides over the D(D+1)/2 Hessian entries.
DEV void derivs_for_path(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H, int member,
                         int team) {
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

}  // namespace drmlt
