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

// Cyclic Jacobi: A (n x n, row-major, symmetric) is destroyed; on return its
// diagonal holds the eigenvalues and V the eigenvectors (columns).
DEV void jacobi_eigen(double *A, double *V, int n) {
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++) V[i * n + k] = i == k ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; i++) {
            diag += A[i * n + i] * A[i * n + i];
            for (int k = i + 1; k < n; k++) off += A[i * n + k] * A[i * n + k];
        }
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < n - 1; p++) {
            for (int q = p + 1; q < n; q++) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double app = A[p * n + p], aqq = A[q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (::fabs(theta) + ::sqrt(theta * theta + 1.0));
                const double c = 1.0 / ::sqrt(t * t + 1.0);
                const double s = t * c;
                for (int k = 0; k < n; k++) {  // rotate columns p, q
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {  // rotate rows p, q
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; k++) {
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
}

// grad: D, hess: D x D (row-major). Non-finite derivatives are scrubbed to zero
// first (drsmallstep.cpp:149-154). `work` holds D*D doubles.
DEV void compute_gaussian(int dim, const H2mcParam &prm, float ss, const float *grad, const float *hess,
                          double *work, GaussView g) {
    bool finite = true;
    for (int i = 0; i < dim; i++) finite = finite && isfinite(grad[i]);
    for (int i = 0; i < dim * dim; i++) finite = finite && isfinite(hess[i]);
    double fro = 0.0;
    for (int i = 0; i < dim * dim; i++) {
        const double h = finite ? double(hess[i]) : 0.0;
        work[i] = h;
        fro += h * h;
    }
    const double sigma = double(prm.sigma);
    if (ss <= 1e-15f || ::sqrt(fro) < 0.5 / (sigma * sigma)) {
        gauss_isotropic(dim, sigma, g);
        return;
    }
    // symmetrise: the reference maps the row-major Hessian as a column-major
    // matrix and SelfAdjointEigenSolver reads its lower triangle, i.e. the
    // row-major upper triangle
    for (int i = 0; i < dim; i++)
        for (int k = i + 1; k < dim; k++) work[k * dim + i] = work[i * dim + k];
    jacobi_eigen(work, g.V, dim);
    const double invSigmaSq = 1.0 / (sigma * sigma);
    double logDet = 0.0;
    double mt[kMaxDim];
    for (int k = 0; k < dim; k++) {
        const double lam = work[k * dim + k];
        double vg = 0.0;
        for (int i = 0; i < dim; i++) vg += g.V[i * dim + k] * (finite ? double(grad[i]) : 0.0);
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
        mt[k] = eb / post * o;
        logDet += ::log(post);
    }
    for (int i = 0; i < dim; i++) {
        double m = 0.0;
        for (int k = 0; k < dim; k++) m += g.V[i * dim + k] * mt[k];
        g.mean[i] = m;
    }
    *g.logDet = logDet;
    *g.dimv = double(dim);
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
