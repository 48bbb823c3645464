// The gradient and Hessian of log f of one path by a team of threads, shared
// by the derivative kernels (derivs.cu) and, compiled separately as
// relocatable device code, by the persistent schedule (derivs_dev.cu). Both
// translation units take the derivative kernels' flags (fast-math
// intrinsics), so both give the same values.
#pragma once
#include "chain.cuh"
#include "pathadj.cuh"

namespace drmlt {

// Hessian entry `pidx` (row-major over the upper triangle) of log f of path r
// (dimension dim) by one hyper-dual evaluation seeded in u_i and u_j; the
// diagonal entries also give the gradient.
DEV void derivs_entry(const SceneView &s, const PathRec &r, int dim, int pidx, float *g, float *H) {
    int i0 = 0, rem = pidx;
    while (rem >= dim - i0) {
        rem -= dim - i0;
        i0++;
    }
    const int j0 = i0 + rem;
    HyperDual u[kMaxDim];
    for (int k = 0; k < dim; k++) u[k] = HyperDual(r.u[k], k == i0 ? 1.0f : 0.0f, k == j0 ? 1.0f : 0.0f, 0.0f);
    const HyperDual f = ad_eval_path<HyperDual>(s, r, u);
    H[i0 * dim + j0] = f.ab;
    H[j0 * dim + i0] = f.ab;
    if (i0 == j0) g[i0] = f.a;
}

// Whether the chain loop takes derivatives of a path of L segments and score ss
// (else the isotropic fallback of drsmallstep.cpp:133-163 with zero rows).
DEV bool derivs_wanted(int L, float ss, int maxDerv) { return L <= maxDerv && ss > 1e-15f; }

// The rows of the adjoint (pathadj.cuh) of a path of dimension dim, strided
// over a team of `team` threads.
DEV void derivs_adj_for_path(const SceneView &s, const PathRec &r, int dim, float *g, float *H, int member,
                             int team) {
    for (int row = member; row < dim; row += team) adj_row(s, r, dim, row, row == 0 ? g : nullptr, H);
}

// A team of `team` threads strides over the D(D+1)/2 Hessian entries
// (hyper-dual forward mode), or, for a path of dimension D >= adjMinDim, over
// the D rows of the reverse-mode adjoint (pathadj.cuh: one forward and one
// backward sweep per row, D sweeps for the whole Hessian against D(D+1)/2
// hyper-dual evaluations).
// kAdjoint = false compiles the hyper-dual form alone (adjMinDim ignored).
template <bool kAdjoint = true>
DEV void derivs_for_path(const SceneView &s, const PathRec &r, float ss, int maxDerv, float *g, float *H, int member,
                         int team, int adjMinDim) {
    const int lane = member;
    const int L = r.c + r.l - 1;
    const int dim = 2 * L;
    if (!derivs_wanted(L, ss, maxDerv)) {
        for (int k = lane; k < dim; k += team) g[k] = 0.0f;
        for (int k = lane; k < dim * dim; k += team) H[k] = 0.0f;
        return;
    }
    if (kAdjoint && dim >= adjMinDim) {
        derivs_adj_for_path(s, r, dim, g, H, member, team);
        return;
    }
    const int npairs = dim * (dim + 1) / 2;
    for (int pidx = lane; pidx < npairs; pidx += team) derivs_entry(s, r, dim, pidx, g, H);
}

}  // namespace drmlt
