// H2MC anisotropic Gaussian in double precision.
//
// ComputeGaussian (src/integrators/delayed/drsmallstep.cpp:19-93, 219-266):
// isotropic fallback test, eigen-decomposition of the Hessian of log f,
// eigenvalue bounding with the L = pi/2 H2MC factors (drsmallstep.h:26-42),
// prior 1/sigma^2, drifted mean. IsotropicGaussian / GaussianLogPdf /
// GenerateSample (src/gaussian.cpp:4-47).
//
// A Gaussian is stored as its precision eigen-basis: invCov = V diag(p) V^T,
// covL = V diag(p^-1/2), mean, logDet = sum log p. The eigen-decomposition is
// FP32 cyclic Jacobi refined to FP64 accuracy (any symmetric eigensolver gives
// the same invCov, mean and covariance; only the column order/sign of covL
// differ, which leaves the sampled distribution unchanged).
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

// Shared-memory scratch for one Gaussian of dimension <= m. Matrices are
// row-major with a padded row stride ld = m + 1, so threads walking down a
// column hit distinct banks.
struct GaussSmem {
    int m, ld;
    double *A64;   // m x ld: the symmetrised Hessian (destroyed by the FP64 fallback)
    double *X;     // m x ld: eigenvectors (columns) in FP64
    double *lam;   // m: eigenvalues in FP64
    double *cs64;  // 2m: rotations of the FP64 fallback
    float *A32;    // m x ld: FP32 Jacobi working matrix, then the residual Z, then X E
    float *V32;    // m x ld: FP32 eigenvectors
    float *R32;    // m x ld: I - X^T X
    float *T32;    // m x ld: X^T Z, then the correction E
    float *l32;    // m: FP32 eigenvalues
    float *cs32;   // 2m
    int *pq;       // 2m
    DEV GaussSmem(double *base, int maxDim) {
        m = maxDim;
        ld = maxDim + 1;
        A64 = base;
        X = A64 + m * ld;
        lam = X + m * ld;
        cs64 = lam + m;
        A32 = reinterpret_cast<float *>(cs64 + 2 * m);
        V32 = A32 + m * ld;
        R32 = V32 + m * ld;
        T32 = R32 + m * ld;
        l32 = T32 + m * ld;
        cs32 = l32 + m;
        pq = reinterpret_cast<int *>(cs32 + 2 * m);
    }
};

// doubles of GaussSmem for dimension m, and of shared memory per Gaussian:
// GaussSmem, then 32 doubles for the team reductions (rounded up to a
// multiple of 2 for 16-byte alignment)
HD constexpr int gauss_scratch_doubles(int m) { return 2 * m * (m + 1) + 3 * m + (4 * m * (m + 1) + 5 * m + 1) / 2 + 1; }
HD constexpr int gauss_smem_doubles(int m) { return (gauss_scratch_doubles(m) + 32 + 1) & ~1; }
DEV double *gauss_reduction(double *base, int m) { return base + gauss_scratch_doubles(m); }

// The threads of one block (whole warps) cooperate on one Gaussian. red: 32
// doubles of shared scratch for the reductions.
struct Team {
    int tid, size;
    double *red;
    DEV explicit Team(double *r) : tid(threadIdx.x), size(blockDim.x), red(r) {}
    DEV void sync() const { __syncthreads(); }
    DEV bool all(bool pred) const { return __syncthreads_and(pred) != 0; }
    DEV double sum(double v) const {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();  // earlier readers of red are done
        if ((tid & 31) == 0) red[tid >> 5] = v;
        __syncthreads();
        double t = 0.0;
        for (int w = 0; w < (size >> 5); w++) t += red[w];
        return t;
    }
    DEV float sum(float v) const {
        float *r = reinterpret_cast<float *>(red);
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        __syncthreads();
        if ((tid & 31) == 0) r[tid >> 5] = v;
        __syncthreads();
        float t = 0.0f;
        for (int w = 0; w < (size >> 5); w++) t += r[w];
        return t;
    }
};

// Thread layout of an n x n elementwise pass: tid = h * np2 + j, column j,
// rows h, h + G, ... (np2 = next power of two >= n, G = team size / np2).
struct LaneGrid {
    int j, h, G;
    DEV LaneGrid(int n, const Team &t) {
        const int lg = n <= 8 ? 3 : (n <= 16 ? 4 : 5);
        j = t.tid & ((1 << lg) - 1);
        h = t.tid >> lg;
        G = t.size >> lg;
    }
};

// Jacobi rotation (c, s) that annihilates a_pq. FP32: the classic formula.
// FP64 (used only to polish an almost diagonal matrix): the tangent comes from
// the FP32 formula, which leaves ~1e-7 a_pq behind and keeps the sweeps
// converging, and c = (1 + t^2)^-1/2 is brought to FP64 accuracy by two steps
// of Newton's iteration for the reciprocal square root from the FP32
// estimate, so the rotation is orthogonal in FP64 without FP64 division or
// square-root sequences.
DEV void rot_params(float app, float aqq, float apq, float &c, float &s) {
    c = 1.0f;
    s = 0.0f;
    if (apq == 0.0f) return;
    const float theta = (aqq - app) / (2.0f * apq);
    const float at = fabsf(theta);
    const float t = at > 1e18f ? 0.5f / theta : (theta >= 0.0f ? 1.0f : -1.0f) / (at + sqrtf(theta * theta + 1.0f));
    c = 1.0f / sqrtf(t * t + 1.0f);
    s = t * c;
}
DEV void rot_params(double app, double aqq, double apq, double &c, double &s) {
    c = 1.0;
    s = 0.0;
    // below FP64 resolution of the diagonal pair: leave it (threshold Jacobi)
    if (apq * apq <= 1e-34 * ::fabs(app * aqq)) return;
    const float fpq = float(apq);
    if (fpq == 0.0f || !isfinite(fpq)) return;
    const float theta = float(aqq - app) / (2.0f * fpq);
    const float at = fabsf(theta);
    const float tf = at > 1e18f ? 0.5f / theta : (theta >= 0.0f ? 1.0f : -1.0f) / (at + sqrtf(theta * theta + 1.0f));
    const double t = double(tf);
    const double q = ::fma(t, t, 1.0);
    double r = double(rsqrtf(float(q)));
    r = r * ::fma(-0.5 * q, r * r, 1.5);
    r = r * ::fma(-0.5 * q, r * r, 1.5);
    c = r;
    s = t * r;
}

// Round-robin (Brent-Luk circle method) partner of slot k in `round`: slot 0 is
// fixed, slots 1..n-1 rotate.
DEV int rr_player(int pos, int round, int m) {
    if (pos == 0) return 0;
    int t = pos - 1 + round;
    if (t >= m) t -= m;
    return 1 + t;
}

// Two-sided cyclic Jacobi by one team, round-robin ordering: each round
// rotates n/2 disjoint index pairs at once. A (n x ld, symmetric, n even) is
// destroyed: its diagonal ends up holding the eigenvalues and V the
// eigenvectors as columns. T = float for the fast first pass, double for the
// polish.
template <class T>
DEV void jacobi_team(T *A, T *V, T *cs, int *pq, int n, int ld, T offTol, int maxSweeps, const Team &tm) {
    const LaneGrid g(n, tm);
    for (int i = g.h; i < n; i += g.G)
        if (g.j < n) V[i * ld + g.j] = i == g.j ? T(1) : T(0);
    tm.sync();
    const int half = n / 2, m = n - 1;
    T prevOff = T(0);
    for (int sweep = 0; sweep < maxSweeps; sweep++) {
        T off = T(0), diag = T(0);
        for (int i = g.h; i < n; i += g.G) {
            if (g.j >= n) continue;
            const T a = A[i * ld + g.j];
            if (i == g.j) diag += a * a;
            else if (g.j > i) off += a * a;
        }
        off = tm.sum(off);
        diag = tm.sum(diag);
        // converged, or (single precision) stalled at round-off
        if (off <= offTol * diag || off == T(0) || (sweep >= 6 && off > T(0.5) * prevOff)) break;
        prevOff = off;
        for (int round = 0; round < m; round++) {
            if (tm.tid < half) {
                int p = rr_player(tm.tid, round, m), q = rr_player(n - 1 - tm.tid, round, m);
                if (p > q) { const int t = p; p = q; q = t; }
                T c, s;
                rot_params(A[p * ld + p], A[q * ld + q], A[p * ld + q], c, s);
                pq[2 * tm.tid] = p;
                pq[2 * tm.tid + 1] = q;
                cs[2 * tm.tid] = c;
                cs[2 * tm.tid + 1] = s;
            }
            // (a barrier) a round whose rotations are all the identity changes nothing
            if (tm.all(tm.tid >= half || cs[2 * tm.tid + 1] == T(0))) continue;
            if (g.j < n) {
                for (int k = g.h; k < half; k += g.G) {  // rows p, q
                    const int p = pq[2 * k], q = pq[2 * k + 1];
                    const T c = cs[2 * k], s = cs[2 * k + 1];
                    const T a = A[p * ld + g.j], b = A[q * ld + g.j];
                    A[p * ld + g.j] = c * a - s * b;
                    A[q * ld + g.j] = s * a + c * b;
                }
            }
            tm.sync();
            if (g.j < n) {
                for (int k = g.h; k < half; k += g.G) {  // columns p, q and the eigenvector columns
                    const int p = pq[2 * k], q = pq[2 * k + 1];
                    const T c = cs[2 * k], s = cs[2 * k + 1];
                    const int r = g.j * ld;
                    const T a = A[r + p], b = A[r + q];
                    A[r + p] = c * a - s * b;
                    A[r + q] = s * a + c * b;
                    const T va = V[r + p], vb = V[r + q];
                    V[r + p] = c * va - s * vb;
                    V[r + q] = s * va + c * vb;
                }
            }
            tm.sync();
        }
    }
}

// FP64-accumulated residuals of an approximate eigen-decomposition (X, lam):
// Z = A X - X diag(lam) into sm.A32 and, unless skipR, R = I - X^T X into
// sm.R32. Both are ~1e-7 or smaller, so FP32 storage keeps their accuracy; the
// sums cancel and run in FP64. X is sm.X. Returns |Z|_F^2.
DEV double eigen_residuals(GaussSmem &sm, int n, bool skipR, const Team &tm) {
    const LaneGrid g(n, tm);
    const int ld = sm.ld;
    const double *A = sm.A64;
    double res = 0.0;
    if (g.j < n) {
        const double lj = sm.lam[g.j];
        for (int i = g.h; i < n; i += g.G) {
            const double xij = sm.X[i * ld + g.j];
            double z = -xij * lj;
            double r = i == g.j ? 1.0 : 0.0;
            for (int k = 0; k < n; k++) {
                const double xkj = sm.X[k * ld + g.j];
                z = ::fma(A[i * ld + k], xkj, z);
                if (!skipR) r = ::fma(-sm.X[k * ld + i], xkj, r);
            }
            sm.A32[i * ld + g.j] = float(z);
            if (!skipR) sm.R32[i * ld + g.j] = float(r);
            res += z * z;
        }
    }
    return tm.sum(res);  // includes a barrier
}

// Iterative refinement of the symmetric eigen-decomposition (Ogita & Aishima,
// "Iterative refinement for symmetric eigenvalue decomposition", 2018), from
// the FP32 Jacobi result (sm.V32, sm.l32) towards FP64 accuracy. Per step, with
// Z = A X - X diag(lam) and R = I - X^T X from eigen_residuals:
//   T = X^T Z,  lam~_i = lam_i + T_ii / (1 - R_ii),
//   E_ij = (T_ij + R_ij (lam~_j - lam_j)) / (lam~_j - lam~_i)  if |lam~_j - lam~_i| > delta,
//   E_ij = R_ij / 2  otherwise (clusters, and i = j),
//   X' = X + X E,  delta = 2 (|offdiag(X^T A X)|_F + |A|_F |R|_F).
// T, E and X E are ~1e-7 and are formed in FP32 from a float copy of X; only
// the residual sums and X + X E are FP64. A step is accepted when the FP64
// residual of (X', lam~) is below 1e-11 |A|_F; at most three steps (a third
// step certifies three quarters of the Gaussians the second leaves, at a fifth
// of the polish's cost), then the caller falls back to the FP64 polish.
// Leaves X and lam in sm.
DEV bool refine_eigen_team(GaussSmem &sm, int n, double froA, const Team &tm) {
    const LaneGrid g(n, tm);
    const int ld = sm.ld;
    const double tol2 = 1e-22 * froA * froA;
    if (tm.tid < n) sm.lam[tm.tid] = double(sm.l32[tm.tid]);
    if (g.j < n)
        for (int i = g.h; i < n; i += g.G) sm.X[i * ld + g.j] = double(sm.V32[i * ld + g.j]);
    tm.sync();
    eigen_residuals(sm, n, false, tm);
    double *lamNew = sm.cs64;
    for (int step = 0; step < 3; step++) {
        const float *X32 = sm.V32;
        const float *Z = sm.A32;
        // T = X^T Z
        if (g.j < n) {
            for (int i = g.h; i < n; i += g.G) {
                float t = 0.0f;
                for (int k = 0; k < n; k++) t = fmaf(X32[k * ld + i], Z[k * ld + g.j], t);
                sm.T32[i * ld + g.j] = t;
            }
        }
        tm.sync();
        if (tm.tid < n)
            lamNew[tm.tid] =
                sm.lam[tm.tid] + double(sm.T32[tm.tid * ld + tm.tid]) / (1.0 - double(sm.R32[tm.tid * ld + tm.tid]));
        float offS = 0.0f, nR = 0.0f;
        if (g.j < n) {
            const float lj = float(sm.lam[g.j]);
            for (int i = g.h; i < n; i += g.G) {
                const float r = sm.R32[i * ld + g.j];
                nR += r * r;
                if (i != g.j) {
                    const float sij = sm.T32[i * ld + g.j] - r * lj;
                    offS += sij * sij;
                }
            }
        }
        offS = tm.sum(offS);
        nR = tm.sum(nR);  // the barriers also publish lamNew
        const float delta = 2.0f * (sqrtf(offS) + float(froA) * sqrtf(nR));
        // E in place of T
        if (g.j < n) {
            const double ltj = lamNew[g.j];
            const float dj = float(ltj - sm.lam[g.j]);
            for (int i = g.h; i < n; i += g.G) {
                const float r = sm.R32[i * ld + g.j];
                const float gap = float(ltj - lamNew[i]);
                float e;
                if (i == g.j || !(fabsf(gap) > delta)) e = 0.5f * r;
                else e = (sm.T32[i * ld + g.j] + r * dj) / gap;
                sm.T32[i * ld + g.j] = e;
            }
        }
        tm.sync();
        // X' = X + X E: the product in FP32 (it is ~1e-7), the sum in FP64
        if (g.j < n) {
            for (int i = g.h; i < n; i += g.G) {
                float c = 0.0f;
                for (int k = 0; k < n; k++) c = fmaf(X32[i * ld + k], sm.T32[k * ld + g.j], c);
                sm.X[i * ld + g.j] += double(c);
            }
        }
        if (tm.tid < n) sm.lam[tm.tid] = lamNew[tm.tid];
        tm.sync();
        // certificate: FP64 residual of the refined pairs (also the next step's Z)
        const double res = eigen_residuals(sm, n, true, tm);
        if (res <= tol2) return true;  // false for NaN
        if (step == 2) break;
        if (g.j < n)
            for (int i = g.h; i < n; i += g.G) sm.V32[i * ld + g.j] = float(sm.X[i * ld + g.j]);
        // R for the refined X (FP64; Z is already in place)
        if (g.j < n) {
            for (int i = g.h; i < n; i += g.G) {
                double r = i == g.j ? 1.0 : 0.0;
                for (int k = 0; k < n; k++) r = ::fma(-sm.X[k * ld + i], sm.X[k * ld + g.j], r);
                sm.R32[i * ld + g.j] = float(r);
            }
        }
        tm.sync();
    }
    return false;
}

// Fallback when the refinement cannot certify (eigenvalue clusters it could not
// separate; its first-order updates can then also leave X non-orthogonal):
// Newton-Schulz orthonormalisation of X in FP64 (X <- X (3I - X^T X) / 2,
// quadratically convergent), FP64 Jacobi on S = X^T A X, which is diagonal up
// to ~1e-6 |A| in that basis, then X <- X W. Scratch: Y and M/W use the FP32
// matrices' storage as FP64 matrices (A32+V32 and R32+T32 are each m x ld
// doubles of contiguous space).
DEV void polish_eigen_team(GaussSmem &sm, int n, const Team &tm) {
    const LaneGrid g(n, tm);
    const int ld = sm.ld;
    double *Y = reinterpret_cast<double *>(sm.A32);
    double *M = reinterpret_cast<double *>(sm.R32);
    for (int it = 0; it < 3; it++) {
        double dev = 0.0;
        if (g.j < n) {  // M = X^T X
            for (int i = g.h; i < n; i += g.G) {
                double v = 0.0;
                for (int k = 0; k < n; k++) v = ::fma(sm.X[k * ld + i], sm.X[k * ld + g.j], v);
                M[i * ld + g.j] = v;
                const double e = v - (i == g.j ? 1.0 : 0.0);
                dev += e * e;
            }
        }
        dev = tm.sum(dev);
        if (dev <= 1e-28) break;
        if (g.j < n) {  // Y = X (3I - M) / 2
            for (int i = g.h; i < n; i += g.G) {
                double v = 1.5 * sm.X[i * ld + g.j];
                for (int k = 0; k < n; k++) v = ::fma(-0.5 * sm.X[i * ld + k], M[k * ld + g.j], v);
                Y[i * ld + g.j] = v;
            }
        }
        tm.sync();
        if (g.j < n)
            for (int i = g.h; i < n; i += g.G) sm.X[i * ld + g.j] = Y[i * ld + g.j];
        tm.sync();
    }
    if (g.j < n) {  // Y = A X
        for (int i = g.h; i < n; i += g.G) {
            double y = 0.0;
            for (int k = 0; k < n; k++) y = ::fma(sm.A64[i * ld + k], sm.X[k * ld + g.j], y);
            Y[i * ld + g.j] = y;
        }
    }
    tm.sync();
    if (g.j < n) {  // S = X^T Y over A64 (A is no longer needed)
        for (int i = g.h; i < n; i += g.G) {
            double v = 0.0;
            for (int k = 0; k < n; k++) v = ::fma(sm.X[k * ld + i], Y[k * ld + g.j], v);
            sm.A64[i * ld + g.j] = v;
        }
    }
    tm.sync();
    if (g.j < n) {  // symmetrise S against round-off
        for (int i = g.h; i < n; i += g.G) {
            if (i < g.j) {
                const double v = 0.5 * (sm.A64[i * ld + g.j] + sm.A64[g.j * ld + i]);
                sm.A64[i * ld + g.j] = v;
                sm.A64[g.j * ld + i] = v;
            }
        }
    }
    tm.sync();
    jacobi_team<double>(sm.A64, M, sm.cs64, sm.pq, n, ld, 1e-28, 8, tm);
    if (g.j < n) {  // X <- X W (through Y)
        for (int i = g.h; i < n; i += g.G) {
            double v = 0.0;
            for (int k = 0; k < n; k++) v = ::fma(sm.X[i * ld + k], M[k * ld + g.j], v);
            Y[i * ld + g.j] = v;
        }
    }
    tm.sync();
    if (g.j < n)
        for (int i = g.h; i < n; i += g.G) sm.X[i * ld + g.j] = Y[i * ld + g.j];
    if (tm.tid < n) sm.lam[tm.tid] = sm.A64[tm.tid * ld + tm.tid];
    tm.sync();
}

enum : int { kGaussIsotropic = 0, kGaussRefined = 1, kGaussFp64Jacobi = 2 };

// ComputeGaussian by one team (the whole block): grad (D floats), hess (D x D
// floats, row-major) in global memory; scratch in the block's shared memory
// (GaussSmem sized for the launch's largest dimension, then the team's
// reduction scratch). Non-finite derivatives are scrubbed to zero first
// (drsmallstep.cpp:149-154). Every thread of the block must call it. The
// eigen-decomposition is FP32 Jacobi refined to FP64 (refine_eigen_team), or
// the FP64 polish when the refinement's certificate fails. Returns which of
// the three (isotropic fallback, refined, FP64 polish) produced the Gaussian.
DEV int compute_gaussian_team(int dim, const H2mcParam &prm, float ss, const float *grad, const float *hess,
                              GaussSmem &sm, GaussView g, const Team &tm) {
    const int ld = sm.ld;
    bool finite = true;
    for (int i = tm.tid; i < dim; i += tm.size) finite = finite && isfinite(grad[i]);
    for (int i = tm.tid; i < dim * dim; i += tm.size) finite = finite && isfinite(hess[i]);
    finite = tm.all(finite);
    double fro = 0.0;
    for (int e = tm.tid; e < dim * dim; e += tm.size) {
        const double h = finite ? double(hess[e]) : 0.0;
        fro += h * h;
    }
    fro = tm.sum(fro);
    const double sigma = double(prm.sigma);
    const double invSigmaSq = 1.0 / (sigma * sigma);
    if (ss <= 1e-15f || ::sqrt(fro) < 0.5 / (sigma * sigma)) {
        for (int e = tm.tid; e < dim * dim; e += tm.size) g.V[e] = (e / dim == e % dim) ? 1.0 : 0.0;
        for (int i = tm.tid; i < dim; i += tm.size) {
            g.p[i] = invSigmaSq;
            g.mean[i] = 0.0;
        }
        if (tm.tid == 0) {
            *g.logDet = double(dim) * ::log(invSigmaSq);
            *g.dimv = double(dim);
        }
        tm.sync();
        return kGaussIsotropic;
    }
    // symmetrise: the reference maps the row-major Hessian as a column-major
    // matrix and SelfAdjointEigenSolver reads its lower triangle, i.e. the
    // row-major upper triangle
    {
        const LaneGrid lg(dim, tm);
        if (lg.j < dim) {
            for (int i = lg.h; i < dim; i += lg.G) {
                const int k = lg.j;
                const float h = finite ? hess[i <= k ? i * dim + k : k * dim + i] : 0.0f;
                sm.A64[i * ld + k] = double(h);
                sm.A32[i * ld + k] = h;
            }
        }
    }
    tm.sync();
    jacobi_team<float>(sm.A32, sm.V32, sm.cs32, sm.pq, dim, ld, 1e-14f, 12, tm);
    if (tm.tid < dim) sm.l32[tm.tid] = sm.A32[tm.tid * ld + tm.tid];
    tm.sync();
    int kind = kGaussRefined;
    if (!refine_eigen_team(sm, dim, ::sqrt(fro), tm)) {
        kind = kGaussFp64Jacobi;
        polish_eigen_team(sm, dim, tm);
    }
    // per eigenvalue (thread k): H2MC bounding and the drifted mean's eigen-coordinates
    double logp = 0.0;
    if (tm.tid < dim) {
        const int k = tm.tid;
        const double lam = sm.lam[k];
        double vg = 0.0;
        for (int i = 0; i < dim; i++) vg += sm.X[i * ld + k] * (finite ? double(grad[i]) : 0.0);
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
        logp = ::log(post);
        sm.cs64[k] = eb / post * o;
    }
    logp = tm.sum(logp);  // includes a barrier
    for (int e = tm.tid; e < dim * dim; e += tm.size) g.V[e] = sm.X[(e / dim) * ld + e % dim];
    for (int i = tm.tid; i < dim; i += tm.size) {
        double mu = 0.0;
        for (int k = 0; k < dim; k++) mu += sm.X[i * ld + k] * sm.cs64[k];
        g.mean[i] = mu;
    }
    if (tm.tid == 0) {
        *g.logDet = logp;
        *g.dimv = double(dim);
    }
    tm.sync();
    return kind;
}

// GaussianLogPdf (src/gaussian.cpp:18-26) in FP64 of sign * off (off: dim
// floats) by one team: thread k projects the offset on eigenvector k.
DEV double gauss_logpdf_team(int dim, const float *off, double sign, GaussView g, const Team &tm) {
    double quad = 0.0;
    if (tm.tid < dim) {
        double proj = 0.0;
        for (int i = 0; i < dim; i++) proj = ::fma(g.V[i * dim + tm.tid], sign * double(off[i]) - g.mean[i], proj);
        quad = g.p[tm.tid] * proj * proj;
    }
    quad = tm.sum(quad);
    return double(dim) * (-0.5 * ::log(2.0 * 3.14159265358979323846)) + 0.5 * (*g.logDet) - 0.5 * quad;
}


}  // namespace drmlt
