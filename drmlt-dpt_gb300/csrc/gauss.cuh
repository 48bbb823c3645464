// H2MC anisotropic Gaussian in double precision.
//
// ComputeGaussian (src/integrators/delayed/drsmallstep.cpp:19-93, 219-266):
// isotropic fallback test, eigen-decomposition of the Hessian of log f,
// eigenvalue bounding with the L = pi/2 H2MC factors (drsmallstep.h:26-42),
// prior 1/sigma^2, drifted mean. IsotropicGaussian / GaussianLogPdf /
// GenerateSample (src/gaussian.cpp:4-47).
//
// A Gaussian is stored as its precision eigen-basis: invCov = V diag(p) V^T,
// covL = V diag(p^-1/2), mean, logDet = sum log p. The eigen-decomposition is a
// cyclic Jacobi sweep in FP64 (any symmetric eigensolver gives the same
// invCov, mean and covariance; only the column order/sign of covL differ,
// which leaves the sampled distribution unchanged).
#pragma once
#include "common.cuh"

namespace drmlt {

constexpr int kGaussStride = kMaxDim * kMaxDim + 2 * kMaxDim + 2;  // doubles per stored Gaussian

struct GaussView {  // layout inside one stored Gaussian
    double *V;      // D x D row-major (V[i*D + k]: component i of eigenvector k)
    double *p;      // D precision eigenvalues
    double *mean;   // D
    double *logDet; // 1
    double *dimv;   // 1 (dimension as double, for checking)
    DEV explicit GaussView(double *base) {
        V = base;
        p = base + kMaxDim * kMaxDim;
        mean = p + kMaxDim;
        logDet = mean + kMaxDim;
        dimv = logDet + 1;
    }
};

// H2MC step-size factors computed in single precision as the reference does.
struct H2mcParam {
    float sigma;
    float posScale, posOffset, negScale, negOffset, L;
    DEV explicit H2mcParam(float s) : sigma(s) {
        L = float(3.14159265358979323846 / 2.0);
        posScale = 0.5f * (expf(L) - expf(-L)) * 0.5f * (expf(L) - expf(-L));
        posOffset = 0.5f * (expf(L) + expf(-L) - 1.0f);
        negScale = sinf(L) * sinf(L);
        negOffset = -(cosf(L) - 1.0f);
    }
};

DEV void gauss_isotropic(int dim, double sigma, GaussView g) {
    const double invSigmaSq = 1.0 / (sigma * sigma);
    double logDet = 0.0;
    for (int i = 0; i < dim; i++) {
        for (int k = 0; k < dim; k++) g.V[i * dim + k] = i == k ? 1.0 : 0.0;
        g.p[i] = invSigmaSq;
        g.mean[i] = 0.0;
        logDet += ::log(invSigmaSq);
    }
    *g.logDet = logDet;
    *g.dimv = double(dim);
}

// Warp-cooperative two-sided Jacobi with round-robin (Brent-Luk) ordering:
// each round rotates n/2 disjoint index pairs at once, so the 32 lanes of a
// warp share the row and column updates of one matrix held in shared memory.
// A (n x n, row-major, symmetric, n even) is destroyed: on return its diagonal
// holds the eigenvalues and V (row-major) the eigenvectors as columns.
// cs: 2 * kMaxDim doubles of shared scratch for the rotations of a round.
DEV int rr_partner(int k, int round, int n, bool second) {
    // circle method: position 0 is fixed, positions 1..n-1 rotate by `round`
    const int m = n - 1;
    auto player = [&](int pos) { return pos == 0 ? 0 : 1 + (pos - 1 + round) % m; };
    return second ? player(n - 1 - k) : player(k);
}

DEV void jacobi_eigen_warp(double *A, double *V, double *cs, int n) {
    const int lane = threadIdx.x & 31;
    for (int e = lane; e < n * n; e += 32) V[e] = (e / n == e % n) ? 1.0 : 0.0;
    __syncwarp();
    const int half = n / 2;
    for (int sweep = 0; sweep < 30; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int e = lane; e < n * n; e += 32) {
            const int i = e / n, k = e % n;
            if (i == k) diag += A[e] * A[e];
            else if (k > i) off += A[e] * A[e];
        }
        for (int o = 16; o > 0; o >>= 1) {
            off += __shfl_xor_sync(0xffffffffu, off, o);
            diag += __shfl_xor_sync(0xffffffffu, diag, o);
        }
        // stop once the off-diagonal mass is at FP64 round-off of the diagonal
        if (off <= 1e-26 * diag || off == 0.0) break;
        for (int round = 0; round < n - 1; round++) {
            if (lane < half) {
                int p = rr_partner(lane, round, n, false), q = rr_partner(lane, round, n, true);
                if (p > q) { const int t = p; p = q; q = t; }
                const double apq = A[p * n + q];
                double c = 1.0, s = 0.0;
                if (apq != 0.0) {
                    const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                    const double t = (theta >= 0.0 ? 1.0 : -1.0) / (::fabs(theta) + ::sqrt(theta * theta + 1.0));
                    c = 1.0 / ::sqrt(t * t + 1.0);
                    s = t * c;
                }
                cs[2 * lane] = c;
                cs[2 * lane + 1] = s;
            }
            __syncwarp();
            // rows p, q of every pair
            for (int task = lane; task < half * n; task += 32) {
                const int k = task / n, j = task % n;
                int p = rr_partner(k, round, n, false), q = rr_partner(k, round, n, true);
                if (p > q) { const int t = p; p = q; q = t; }
                const double c = cs[2 * k], s = cs[2 * k + 1];
                const double apj = A[p * n + j], aqj = A[q * n + j];
                A[p * n + j] = c * apj - s * aqj;
                A[q * n + j] = s * apj + c * aqj;
            }
            __syncwarp();
            // columns p, q of every pair, and the eigenvector columns
            for (int task = lane; task < half * n; task += 32) {
                const int k = task / n, i = task % n;
                int p = rr_partner(k, round, n, false), q = rr_partner(k, round, n, true);
                if (p > q) { const int t = p; p = q; q = t; }
                const double c = cs[2 * k], s = cs[2 * k + 1];
                const double aip = A[i * n + p], aiq = A[i * n + q];
                A[i * n + p] = c * aip - s * aiq;
                A[i * n + q] = s * aip + c * aiq;
                const double vip = V[i * n + p], viq = V[i * n + q];
                V[i * n + p] = c * vip - s * viq;
                V[i * n + q] = s * vip + c * viq;
            }
            __syncwarp();
        }
    }
}

// ComputeGaussian with one warp: grad (D floats), hess (D x D floats,
// row-major) in global memory; A, V (kMaxDim^2 doubles each) and cs (2 kMaxDim)
// in this warp's shared memory. Non-finite derivatives are scrubbed to zero
// first (drsmallstep.cpp:149-154). All 32 lanes must call it.
DEV void compute_gaussian_warp(int dim, const H2mcParam &prm, float ss, const float *grad, const float *hess,
                               double *A, double *V, double *cs, GaussView g) {
    const int lane = threadIdx.x & 31;
    bool finite = true;
    for (int i = lane; i < dim; i += 32) finite = finite && isfinite(grad[i]);
    for (int i = lane; i < dim * dim; i += 32) finite = finite && isfinite(hess[i]);
    finite = __all_sync(0xffffffffu, finite);
    double fro = 0.0;
    for (int e = lane; e < dim * dim; e += 32) {
        const double h = finite ? double(hess[e]) : 0.0;
        fro += h * h;
    }
    for (int o = 16; o > 0; o >>= 1) fro += __shfl_xor_sync(0xffffffffu, fro, o);
    const double sigma = double(prm.sigma);
    const double invSigmaSq = 1.0 / (sigma * sigma);
    if (ss <= 1e-15f || ::sqrt(fro) < 0.5 / (sigma * sigma)) {
        for (int e = lane; e < dim * dim; e += 32) g.V[e] = (e / dim == e % dim) ? 1.0 : 0.0;
        for (int i = lane; i < dim; i += 32) {
            g.p[i] = invSigmaSq;
            g.mean[i] = 0.0;
        }
        if (lane == 0) {
            *g.logDet = double(dim) * ::log(invSigmaSq);
            *g.dimv = double(dim);
        }
        __syncwarp();
        return;
    }
    // symmetrise: the reference maps the row-major Hessian as a column-major
    // matrix and SelfAdjointEigenSolver reads its lower triangle, i.e. the
    // row-major upper triangle
    for (int e = lane; e < dim * dim; e += 32) {
        const int i = e / dim, k = e % dim;
        A[e] = finite ? double(hess[i <= k ? e : k * dim + i]) : 0.0;
    }
    __syncwarp();
    jacobi_eigen_warp(A, V, cs, dim);
    // per eigenvalue (lane k): H2MC bounding and the drifted mean's eigen-coordinates
    double mt = 0.0, logp = 0.0;
    if (lane < dim) {
        const int k = lane;
        const double lam = A[k * dim + k];
        double vg = 0.0;
        for (int i = 0; i < dim; i++) vg += V[i * dim + k] * (finite ? double(grad[i]) : 0.0);
        double eb = ::fabs(lam) > 1e-10 ? 1.0 / ::fabs(lam) : 0.0;
        const double ob = eb * vg;
        double s2, o;
        if (::fabs(lam) > 1e-10) {
            o = ob;
            if (lam > 0.0) {
                s2 = prm.posScale;
                o *= prm.posOffset;
            } else {
                s2 = prm.negScale;
                o *= prm.negOffset;
            }
        } else {
            s2 = double(prm.L) * double(prm.L);
            o = 0.5 * ob * double(prm.L) * double(prm.L);
        }
        eb *= s2;
        eb = eb > 1e-10 ? 1.0 / eb : 0.0;
        const double post = eb + invSigmaSq;
        g.p[k] = post;
        mt = eb / post * o;
        logp = ::log(post);
        cs[k] = mt;
    }
    for (int o = 16; o > 0; o >>= 1) logp += __shfl_xor_sync(0xffffffffu, logp, o);
    __syncwarp();
    for (int e = lane; e < dim * dim; e += 32) g.V[e] = V[e];
    for (int i = lane; i < dim; i += 32) {
        double m = 0.0;
        for (int k = 0; k < dim; k++) m += V[i * dim + k] * cs[k];
        g.mean[i] = m;
    }
    if (lane == 0) {
        *g.logDet = logp;
        *g.dimv = double(dim);
    }
    __syncwarp();
}

// GaussianLogPdf (src/gaussian.cpp:18-26) in FP64.
DEV double gauss_logpdf(int dim, const double *offset, GaussView g) {
    double d[kMaxDim];
    for (int i = 0; i < dim; i++) d[i] = offset[i] - g.mean[i];
    double quad = 0.0;
    for (int k = 0; k < dim; k++) {
        double proj = 0.0;
        for (int i = 0; i < dim; i++) proj += g.V[i * dim + k] * d[i];
        quad += g.p[k] * proj * proj;
    }
    return double(dim) * (-0.5 * ::log(2.0 * 3.14159265358979323846)) + 0.5 * (*g.logDet) - 0.5 * quad;
}

// GenerateSample (src/gaussian.cpp:36-47): offset = covL n + mean.
template <class R>
DEV void gauss_sample(int dim, GaussView g, R &rng, double *offset) {
    double z[kMaxDim];
    for (int k = 0; k < dim; k++) z[k] = double(rng.normal()) / ::sqrt(g.p[k]);
    for (int i = 0; i < dim; i++) {
        double o = g.mean[i];
        for (int k = 0; k < dim; k++) o += g.V[i * dim + k] * z[k];
        offset[i] = o;
    }
}

}  // namespace drmlt
