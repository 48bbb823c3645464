// Per-path entry points of the C ABI: forward/backward path derivatives,
// perturbation, recorded-stream replay of the samplers, and the FP64 Gaussian.
// They run the same device functions as the chain kernels on caller-supplied
// inputs so that each piece can be compared with the reference's own output.
// Included at the end of drmlt.cu (same translation unit as Renderer).
#pragma once

namespace {

__global__ void k_eval_paths(SceneView s, const PathRec *paths, const float *u, int n, float *logf) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    logf[i] = ad_eval_path<float>(s, paths[i], u + size_t(i) * kMaxDim);
}

struct NoJitter {
    DEV float normal() { return 0.0f; }
};

__global__ void k_perturb_paths(SceneView s, const PathRec *in, const float *offset, int n, PathRec *out,
                                drmlt_contrib *ct) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    NoJitter nj;
    Emit e;
    SceneView sv = s;
    sv.opt.discreteStdDev = 0.0f;
    const bool ok = perturb_path(sv, in[i], offset + size_t(i) * kMaxDim, nj, out[i], e);
    drmlt_contrib c;
    std::memset(&c, 0, sizeof(c));
    if (ok) {
        c.screen[0] = e.screen[0];
        c.screen[1] = e.screen[1];
        c.rgb[0] = e.rgb.x;
        c.rgb[1] = e.rgb.y;
        c.rgb[2] = e.rgb.z;
        c.ls = e.ls;
        c.ss = e.ss;
        c.valid = 1;
    }
    ct[i] = c;
}

__global__ void k_lens_eval(SceneView s, const PathRec *paths, const float *screen, const float *ss, int n,
                            float sigma, int maxDerv, float *score, float *pos, float *logf, float *grad, float *hess,
                            double *gauss) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    PathRec tmp;
    Emit e;
    LensAnchor a;
    V3 lp;
    float ls = 0.0f;
    const PathRec &r = paths[i];
    const float sx = screen[2 * i], sy = screen[2 * i + 1];
    if (!lens_walk<false>(s, r, sx, sy, V3(0.0f, 0.0f, 0.0f), tmp, e, ls, a, lp)) ls = 0.0f;
    score[i] = ls;
    pos[3 * i] = lp.x;
    pos[3 * i + 1] = lp.y;
    pos[3 * i + 2] = lp.z;
    float g[2] = {0.0f, 0.0f}, h[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    float f = 0.0f;
    const bool have = lens_func_exists(r.c, r.l, maxDerv);
    if (have && ls > 1e-15f) {
        lens_derivs(s, a, sx, sy, ls, g, h);
        f = lens_logf<float>(s, a, sx, sy);
    }
    logf[i] = f;
    for (int k = 0; k < 2; k++) grad[2 * i + k] = g[k];
    for (int k = 0; k < 4; k++) hess[4 * i + k] = h[k];
    LensGauss G;
    const H2mcParam prm(sigma);
    if (have) lens_gaussian(prm, ss[i], g, h, G); else lens_gauss_isotropic(double(prm.sigma), G);
    double *o = gauss + 7 * size_t(i);
    o[0] = G.mean[0];
    o[1] = G.mean[1];
    for (int r2 = 0; r2 < 2; r2++)
        for (int c2 = 0; c2 < 2; c2++)
            o[2 + r2 * 2 + c2] = G.V[r2 * 2] * G.p[0] * G.V[c2 * 2] + G.V[r2 * 2 + 1] * G.p[1] * G.V[c2 * 2 + 1];
    o[6] = G.logDet;
}

__global__ void k_lens_perturb(SceneView s, const PathRec *in, const float *screen, const float *lensPos, int n,
                               PathRec *out, drmlt_contrib *ct, float *score) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Emit e;
    LensAnchor a;
    V3 lp;
    float ls = 0.0f;
    const V3 pos(lensPos[3 * i], lensPos[3 * i + 1], lensPos[3 * i + 2]);
    const bool ok = lens_walk<true>(s, in[i], screen[2 * i], screen[2 * i + 1], pos, out[i], e, ls, a, lp);
    drmlt_contrib c;
    std::memset(&c, 0, sizeof(c));
    if (ok) {
        c.screen[0] = e.screen[0];
        c.screen[1] = e.screen[1];
        c.rgb[0] = e.rgb.x;
        c.rgb[1] = e.rgb.y;
        c.rgb[2] = e.rgb.z;
        c.ls = e.ls;
        c.ss = e.ss;
        c.valid = 1;
    }
    ct[i] = c;
    score[i] = ok ? ls : 0.0f;
}

struct SinkList {
    int *tech;
    drmlt_contrib *ct;
    int cap;
    int n;
    DEV void operator()(const Emit &e) {
        if (n < cap) {
            tech[2 * n] = e.c;
            tech[2 * n + 1] = e.l;
            drmlt_contrib c;
            c.screen[0] = e.screen[0];
            c.screen[1] = e.screen[1];
            c.rgb[0] = e.rgb.x;
            c.rgb[1] = e.rgb.y;
            c.rgb[2] = e.rgb.z;
            c.ls = e.ls;
            c.ss = e.ss;
            c.valid = 1;
            ct[n] = c;
        }
        n++;
    }
};

__global__ void k_replay(SceneView s, int mode, const float *tapes, const int *tapeLen, int stride, int n,
                         const int *camLen, const int *lgtLen, int maxContribs, int *outCount, int *outTech,
                         drmlt_contrib *outCt, PathRec *outPath, int *outConsumed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TapeRng rng{tapes + size_t(i) * stride, tapeLen[i], 0};
    if (mode == 2) {  // direct-lighting pass for pixel (camLen[i], lgtLen[i])
        SinkList sink{outTech + size_t(i) * 2 * maxContribs, outCt + size_t(i) * maxContribs, maxContribs, 0};
        generate_path_direct(s, camLen[i], lgtLen[i], min(s.opt.minDepth, 2), min(s.opt.maxDepth, 2), rng, sink);
        outCount[i] = sink.n;
    } else if (mode == 0) {
        FullPath f;
        SinkList sink{outTech + size_t(i) * 2 * maxContribs, outCt + size_t(i) * maxContribs, maxContribs, 0};
        generate_path_bidir(s, max(s.opt.minDepth, 3), s.opt.maxDepth, rng, f, sink);
        outCount[i] = sink.n;
        // vertex dump: c = camera vertices, l = light vertices, tri = light then
        // camera triangles, u = camera vertex direction parameters
        PathRec rec;
        std::memset(&rec, 0, sizeof(rec));
        rec.c = f.nCam;
        rec.l = f.nLgt;
        int k = 0;
        for (int v = 0; v < f.nLgt && k < kMaxVerts; v++) rec.tri[k++] = f.lgt[v].tri;
        for (int v = 0; v < f.nCam && k < kMaxVerts; v++) rec.tri[k++] = f.cam[v].tri;
        for (int v = 0; v < f.nCam && 2 * v + 1 < kMaxDim; v++) {
            rec.u[2 * v] = f.cam[v].rnd[0];
            rec.u[2 * v + 1] = f.cam[v].rnd[1];
        }
        outPath[i] = rec;
    } else {
        Emit e;
        PathRec rec;
        std::memset(&rec, 0, sizeof(rec));
        const bool ok = generate_subpath(s, camLen[i], lgtLen[i], rng, rec, e);
        outCount[i] = ok ? 1 : 0;
        drmlt_contrib c;
        std::memset(&c, 0, sizeof(c));
        if (ok) {
            c.screen[0] = e.screen[0];
            c.screen[1] = e.screen[1];
            c.rgb[0] = e.rgb.x;
            c.rgb[1] = e.rgb.y;
            c.rgb[2] = e.rgb.z;
            c.ls = e.ls;
            c.ss = e.ss;
            c.valid = 1;
            outTech[2 * size_t(i)] = e.c;
            outTech[2 * size_t(i) + 1] = e.l;
        }
        outCt[i] = c;
        outPath[i] = rec;
    }
    outConsumed[i] = rng.pos;
}

// One block (team) per Gaussian. dims[i] must be even and <= maxDim (checked by
// the callers); dynamic shared memory gauss_smem_bytes(maxDim).
__global__ void __launch_bounds__(32 * kGaussTeamWarps) k_gauss_batch(const int *dims, const float *ss,
                                                                     const float *grad, const float *hess, int n,
                                                                     float sigma, int maxDim, double *store,
                                                                     double *mean, double *invCov, double *cov,
                                                                     double *logDet) {
    extern __shared__ double gsm[];
    const int i = blockIdx.x;
    if (i >= n) return;
    const int dim = dims[i];
    if (dim <= 0 || dim > maxDim || (dim & 1)) {
        if (threadIdx.x == 0) logDet[i] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    GaussView g(store + size_t(i) * kGaussStride);
    GaussSmem sm(gsm, maxDim);
    const Team tm(gauss_reduction(gsm, maxDim));
    compute_gaussian_team(dim, H2mcParam(sigma), ss[i], grad + size_t(i) * kMaxDim, hess + size_t(i) * kMaxDim * kMaxDim,
                          sm, g, tm);
    for (int r = threadIdx.x; r < dim; r += blockDim.x) mean[size_t(i) * kMaxDim + r] = g.mean[r];
    for (int e = threadIdx.x; e < dim * dim; e += blockDim.x) {
        const int r = e / dim, c = e % dim;
        double ic = 0.0, cv = 0.0;
        for (int k = 0; k < dim; k++) {
            const double vr = g.V[r * dim + k], vc = g.V[c * dim + k];
            ic += vr * g.p[k] * vc;
            cv += vr * vc / g.p[k];
        }
        invCov[size_t(i) * kMaxDim * kMaxDim + r * dim + c] = ic;
        cov[size_t(i) * kMaxDim * kMaxDim + r * dim + c] = cv;
    }
    if (threadIdx.x == 0) logDet[i] = *g.logDet;
}

__global__ void k_trace_rays(SceneView s, const float *org, const float *dir, float tmin, float tmax, int n,
                             int anyHit, int *tri, float *thit) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3 o(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
    const V3 d(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
    const int t = anyHit ? traverse<true>(s, o, d, tmin, tmax) : traverse<false>(s, o, d, tmin, tmax);
    tri[i] = t;
    float th = -1.0f;
    if (t >= 0) {
        const float *P = s.triP + 9 * t;
        th = hit_triangle(o, d, make_float4(P[0], P[1], P[2], 0.f), make_float4(P[3], P[4], P[5], 0.f),
                          make_float4(P[6], P[7], P[8], 0.f));
    }
    thit[i] = th;
}

template <class T>
struct DevBuf {
    T *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    int alloc(size_t n) { return dalloc(&p, n); }
    int put(const T *src, size_t n) {
        int rc = dalloc(&p, n);
        if (rc) return rc;
        if (cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(DRMLT_E_CUDA, "cudaMemcpy H2D");
        return DRMLT_OK;
    }
    int get(T *dst, size_t n) const {
        if (cudaMemcpy(dst, p, n * sizeof(T), cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(DRMLT_E_CUDA, "cudaMemcpy D2H");
        return DRMLT_OK;
    }
};

static_assert(sizeof(PathRec) == sizeof(drmlt_path), "drmlt_path must mirror the device path record");

int check_paths(const drmlt_path *p, int n) {
    for (int i = 0; i < n; i++) {
        const int L = p[i].c + p[i].l - 1;
        if (p[i].c < 1 || p[i].l < 0 || L < 1 || L > kMaxLen)
            return fail(DRMLT_E_ARG, "path technique out of range");
    }
    return DRMLT_OK;
}

}  // namespace

extern "C" {

int drmlt_path_eval(void *handle, const drmlt_path *paths, const float *u, int n, float *logf) {
    if (!handle || n < 0 || (n && (!paths || !u || !logf))) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(paths, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> dp;
    DevBuf<float> du, dl;
    if ((rc = dp.put(reinterpret_cast<const PathRec *>(paths), n)) || (rc = du.put(u, size_t(n) * kMaxDim)) ||
        (rc = dl.alloc(n)))
        return rc;
    k_eval_paths<<<(n + 127) / 128, 128>>>(r->sv, dp.p, du.p, n, dl.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    return dl.get(logf, n);
}

int drmlt_path_grad_hess(void *handle, const drmlt_path *paths, const float *u, int n, float *grad, float *hess) {
    if (!handle || n < 0 || (n && (!paths || !u || !grad || !hess))) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(paths, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> dp;
    DevBuf<float> du, dg, dh;
    if ((rc = dp.put(reinterpret_cast<const PathRec *>(paths), n)) || (rc = du.put(u, size_t(n) * kMaxDim)) ||
        (rc = dg.alloc(size_t(n) * kMaxDim)) || (rc = dh.alloc(size_t(n) * kMaxDim * kMaxDim)))
        return rc;
    launch_gradhess_paths(r->sv, dp.p, du.p, n, dg.p, dh.p, kNoAdjoint, 0);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dg.get(grad, size_t(n) * kMaxDim))) return rc;
    return dh.get(hess, size_t(n) * kMaxDim * kMaxDim);
}

int drmlt_path_adjoint(void *handle, const drmlt_path *paths, const float *u, int n, float *grad, float *hess) {
    if (!handle || n < 0 || (n && (!paths || !u || !grad || !hess))) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(paths, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> dp;
    DevBuf<float> du, dg, dh;
    if ((rc = dp.put(reinterpret_cast<const PathRec *>(paths), n)) || (rc = du.put(u, size_t(n) * kMaxDim)) ||
        (rc = dg.alloc(size_t(n) * kMaxDim)) || (rc = dh.alloc(size_t(n) * kMaxDim * kMaxDim)))
        return rc;
    launch_gradhess_paths(r->sv, dp.p, du.p, n, dg.p, dh.p, 0, 0);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dg.get(grad, size_t(n) * kMaxDim))) return rc;
    return dh.get(hess, size_t(n) * kMaxDim * kMaxDim);
}

int drmlt_perturb(void *handle, const drmlt_path *in, const float *offset, int n, drmlt_path *out,
                  drmlt_contrib *contrib) {
    if (!handle || n < 0 || (n && (!in || !offset || !out || !contrib))) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(in, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> di, dout;
    DevBuf<float> doff;
    DevBuf<drmlt_contrib> dc;
    if ((rc = di.put(reinterpret_cast<const PathRec *>(in), n)) || (rc = doff.put(offset, size_t(n) * kMaxDim)) ||
        (rc = dout.alloc(n)) || (rc = dc.alloc(n)))
        return rc;
    k_perturb_paths<<<(n + 127) / 128, 128>>>(r->sv, di.p, doff.p, n, dout.p, dc.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dout.get(reinterpret_cast<PathRec *>(out), n))) return rc;
    return dc.get(contrib, n);
}

int drmlt_lens_eval(void *handle, const drmlt_path *paths, const float *screen, const float *ss, int n,
                    float lens_sigma, int max_derivative_depth, float *lens_score, float *lens_pos, float *logf,
                    float *grad, float *hess, double *gauss) {
    if (!handle || n < 0 ||
        (n && (!paths || !screen || !ss || !lens_score || !lens_pos || !logf || !grad || !hess || !gauss)))
        return fail(DRMLT_E_ARG, "bad argument");
    if (!(lens_sigma > 0.0f)) return fail(DRMLT_E_ARG, "lens_sigma must be positive");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(paths, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> dp;
    DevBuf<float> dsc, dss, dls, dpos, dlf, dg, dh;
    DevBuf<double> dga;
    if ((rc = dp.put(reinterpret_cast<const PathRec *>(paths), n)) || (rc = dsc.put(screen, size_t(n) * 2)) ||
        (rc = dss.put(ss, n)) || (rc = dls.alloc(n)) || (rc = dpos.alloc(size_t(n) * 3)) || (rc = dlf.alloc(n)) ||
        (rc = dg.alloc(size_t(n) * 2)) || (rc = dh.alloc(size_t(n) * 4)) || (rc = dga.alloc(size_t(n) * 7)))
        return rc;
    k_lens_eval<<<(n + 63) / 64, 64>>>(r->sv, dp.p, dsc.p, dss.p, n, lens_sigma, max_derivative_depth, dls.p, dpos.p,
                                       dlf.p, dg.p, dh.p, dga.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dls.get(lens_score, n)) || (rc = dpos.get(lens_pos, size_t(n) * 3)) || (rc = dlf.get(logf, n)) ||
        (rc = dg.get(grad, size_t(n) * 2)) || (rc = dh.get(hess, size_t(n) * 4)))
        return rc;
    return dga.get(gauss, size_t(n) * 7);
}

int drmlt_lens_perturb(void *handle, const drmlt_path *in, const float *screen_new, const float *lens_pos, int n,
                       drmlt_path *out, drmlt_contrib *contrib, float *lens_score) {
    if (!handle || n < 0 || (n && (!in || !screen_new || !lens_pos || !out || !contrib || !lens_score)))
        return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(in, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    DevBuf<PathRec> di, dout;
    DevBuf<float> dsc, dlp, dls;
    DevBuf<drmlt_contrib> dc;
    if ((rc = di.put(reinterpret_cast<const PathRec *>(in), n)) || (rc = dsc.put(screen_new, size_t(n) * 2)) ||
        (rc = dlp.put(lens_pos, size_t(n) * 3)) || (rc = dout.alloc(n)) || (rc = dc.alloc(n)) || (rc = dls.alloc(n)))
        return rc;
    k_lens_perturb<<<(n + 63) / 64, 64>>>(r->sv, di.p, dsc.p, dlp.p, n, dout.p, dc.p, dls.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dout.get(reinterpret_cast<PathRec *>(out), n)) || (rc = dc.get(contrib, n))) return rc;
    return dls.get(lens_score, n);
}

int drmlt_replay(void *handle, int mode, const float *tapes, const int32_t *tape_len, int stride, int n,
                 const int32_t *cam_len, const int32_t *lgt_len, int max_contribs, int32_t *out_count,
                 int32_t *out_tech, drmlt_contrib *out_contrib, drmlt_path *out_path, int32_t *out_consumed) {
    if (!handle || n < 0 || stride <= 0 || mode < 0 || mode > 2) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    if (mode >= 1 && (!cam_len || !lgt_len || !out_path)) return fail(DRMLT_E_ARG, "replay mode needs cam_len/lgt_len");
    const int mc = mode != 1 ? max_contribs : 1;
    if (mc <= 0) return fail(DRMLT_E_ARG, "max_contribs must be positive");
    Renderer *r = static_cast<Renderer *>(handle);
    int rc;
    DevBuf<float> dt;
    DevBuf<int> dlen, dcam, dlgt, dcount, dtech, dcons;
    DevBuf<drmlt_contrib> dct;
    DevBuf<PathRec> dpath;
    std::vector<int> zeros(n, 0);
    if ((rc = dt.put(tapes, size_t(n) * stride)) || (rc = dlen.put(tape_len, n)) ||
        (rc = dcam.put(mode >= 1 ? cam_len : zeros.data(), n)) || (rc = dlgt.put(mode >= 1 ? lgt_len : zeros.data(), n)) ||
        (rc = dcount.alloc(n)) || (rc = dtech.alloc(size_t(n) * 2 * mc)) || (rc = dcons.alloc(n)) ||
        (rc = dct.alloc(size_t(n) * mc)) || (rc = dpath.alloc(n)))
        return rc;
    CK(cudaMemset(dtech.p, 0, size_t(n) * 2 * mc * sizeof(int)));
    CK(cudaMemset(dct.p, 0, size_t(n) * mc * sizeof(drmlt_contrib)));
    k_replay<<<(n + 63) / 64, 64>>>(r->sv, mode, dt.p, dlen.p, stride, n, dcam.p, dlgt.p, mc, dcount.p, dtech.p, dct.p,
                                    dpath.p, dcons.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dcount.get(out_count, n)) || (rc = dtech.get(out_tech, size_t(n) * 2 * mc)) ||
        (rc = dct.get(out_contrib, size_t(n) * mc)) || (rc = dcons.get(out_consumed, n)))
        return rc;
    if (out_path && mode != 2) return dpath.get(reinterpret_cast<PathRec *>(out_path), n);
    return DRMLT_OK;
}

int drmlt_trace_rays(void *handle, const float *org, const float *dir, float tmin, float tmax, int n, int any_hit,
                     int32_t *tri, float *t) {
    if (!handle || n < 0 || (n && (!org || !dir || !tri || !t))) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    Renderer *r = static_cast<Renderer *>(handle);
    int rc;
    DevBuf<float> dorg, ddir, dt;
    DevBuf<int> dtri;
    if ((rc = dorg.put(org, size_t(n) * 3)) || (rc = ddir.put(dir, size_t(n) * 3)) || (rc = dt.alloc(n)) ||
        (rc = dtri.alloc(n)))
        return rc;
    k_trace_rays<<<(n + 127) / 128, 128>>>(r->sv, dorg.p, ddir.p, tmin, tmax, n, any_hit, dtri.p, dt.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dtri.get(tri, n))) return rc;
    return dt.get(t, n);
}

int drmlt_compute_gaussian(void *handle, const int32_t *dims, const float *ss, const float *grad, const float *hess,
                           int n, double *mean, double *inv_cov, double *cov, double *log_det) {
    if (!handle || n < 0) return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int maxDim = 2;
    for (int i = 0; i < n; i++) {
        if (dims[i] < 2 || dims[i] > kMaxDim || (dims[i] & 1))
            return fail(DRMLT_E_ARG, "dimension must be even and in [2, 24]");
        maxDim = std::max(maxDim, int(dims[i]));
    }
    Renderer *r = static_cast<Renderer *>(handle);
    int rc;
    DevBuf<int> dd;
    DevBuf<float> dss, dg, dh;
    DevBuf<double> dstore, dm, dic, dc, dl;
    if ((rc = dd.put(dims, n)) || (rc = dss.put(ss, n)) || (rc = dg.put(grad, size_t(n) * kMaxDim)) ||
        (rc = dh.put(hess, size_t(n) * kMaxDim * kMaxDim)) || (rc = dstore.alloc(size_t(n) * kGaussStride)) ||
        (rc = dm.alloc(size_t(n) * kMaxDim)) || (rc = dic.alloc(size_t(n) * kMaxDim * kMaxDim)) ||
        (rc = dc.alloc(size_t(n) * kMaxDim * kMaxDim)) || (rc = dl.alloc(n)))
        return rc;
    CK(cudaMemset(dm.p, 0, size_t(n) * kMaxDim * sizeof(double)));
    CK(cudaMemset(dic.p, 0, size_t(n) * kMaxDim * kMaxDim * sizeof(double)));
    CK(cudaMemset(dc.p, 0, size_t(n) * kMaxDim * kMaxDim * sizeof(double)));
    k_gauss_batch<<<n, 32 * kGaussTeamWarps, gauss_smem_bytes(maxDim)>>>(
        dd.p, dss.p, dg.p, dh.p, n, r->opt.perturb_stddev, maxDim, dstore.p, dm.p, dic.p, dc.p, dl.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dm.get(mean, size_t(n) * kMaxDim)) || (rc = dic.get(inv_cov, size_t(n) * kMaxDim * kMaxDim)) ||
        (rc = dc.get(cov, size_t(n) * kMaxDim * kMaxDim)))
        return rc;
    return dl.get(log_det, n);
}

}  // extern "C"

// ============================================================================ ray-casting benchmark
#include "raybench.cuh"

extern "C" {

int drmlt_ray_benchmark(void *handle, int kind, int n_rays, int repeats, float *ms_per_pass, double *counts) {
    if (!handle || !ms_per_pass || !counts) return fail(DRMLT_E_ARG, "null argument");
    if (kind < 0 || kind > 2 || n_rays <= 0 || repeats <= 0) return fail(DRMLT_E_ARG, "bad ray benchmark shape");
    Renderer *r = static_cast<Renderer *>(handle);
    const int n = n_rays;
    int rc;
    DevBuf<float4> org, dir;
    DevBuf<int> hit;
    DevBuf<unsigned long long> cnt;
    if ((rc = org.alloc(n)) || (rc = dir.alloc(n)) || (rc = hit.alloc(n)) || (rc = cnt.alloc(3))) return rc;
    const int nb = (n + 127) / 128;
    k_rays_setup<<<nb, 128>>>(r->sv, kind, n, r->opt.seed ^ 0xBE7Cull, org.p, dir.p);
    CK(cudaMemset(cnt.p, 0, 3 * sizeof(unsigned long long)));
    const int anyHit = kind == 2;
    k_rays_trace<true><<<nb, 128>>>(r->sv, anyHit, n, org.p, dir.p, hit.p, cnt.p);
    k_rays_trace<false><<<nb, 128>>>(r->sv, anyHit, n, org.p, dir.p, hit.p, cnt.p);
    CK(cudaGetLastError());
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0));
    for (int k = 0; k < repeats; k++) k_rays_trace<false><<<nb, 128>>>(r->sv, anyHit, n, org.p, dir.p, hit.p, cnt.p);
    CK(cudaEventRecord(e1));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    unsigned long long h[3];
    if ((rc = cnt.get(h, 3))) return rc;
    *ms_per_pass = ms / float(repeats);
    for (int k = 0; k < 3; k++) counts[k] = double(h[k]);
    return DRMLT_OK;
}

int drmlt_fma_benchmark(void *handle, int fp64, int iterations, float *ms, double *flops) {
    if (!handle || !ms || !flops) return fail(DRMLT_E_ARG, "null argument");
    if (iterations <= 0) return fail(DRMLT_E_ARG, "iterations must be positive");
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = 4 * sms, threads = 256;
    DevBuf<double> sink;
    int rc;
    if ((rc = sink.alloc(blocks))) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    for (int pass = 0; pass < 2; pass++) {  // pass 0: warm-up at a tenth of the length
        const int it = pass == 0 ? iterations / 10 + 1 : iterations;
        if (pass == 1) CK(cudaEventRecord(e0));
        if (fp64)
            k_fma_peak<double><<<blocks, threads>>>(it, 0.999999, 1e-6, sink.p);
        else
            k_fma_peak<float><<<blocks, threads>>>(it, 0.9999f, 1e-6f, reinterpret_cast<float *>(sink.p));
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(e1));
    CK(cudaEventSynchronize(e1));
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t;
    *flops = 2.0 * 8.0 * double(blocks) * threads * double(iterations);
    return DRMLT_OK;
}

}  // extern "C"

// ============================================================================ per-stage acceptances
namespace {

// y = x + o1, z = x + o2 and Green's y* = z + (x - y), with the first-stage and
// isotropic second-stage acceptances (the chain loop's prologue / epilogue
// arithmetic on given offsets; discrete jitter off).
__global__ void k_dr_eval_trace(SceneView s, const PathRec *x, const drmlt_contrib *xc, const float *o1,
                                const float *o2, int n, PathRec *y, PathRec *z, float *ssz, drmlt_dr_result *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    NoJitter nj;
    SceneView sv = s;
    sv.opt.discreteStdDev = 0.0f;
    drmlt_dr_result ev;
    memset(&ev, 0, sizeof(ev));
    PathM m;
    m.pc = kPStart;
    int st = run_perturb(sv, x[i], o1 + size_t(i) * kMaxDim, nj, y[i], m);
    float a1 = 0.0f;
    if (st == kStepDone) {
        ev.valid_y = 1;
        ev.ss_y = m.e.ss;
        a1 = clamp01(m.e.ss / xc[i].ss);
    }
    ev.a1 = is_invalid(a1) ? 0.0f : a1;
    m.pc = kPStart;
    st = run_perturb(sv, x[i], o2 + size_t(i) * kMaxDim, nj, z[i], m);
    if (st == kStepDone) {
        ev.valid_z = 1;
        ev.ss_z = m.e.ss;
        const int dim = path_dim(x[i].c, x[i].l);
        float off[kMaxDim];
        for (int k = 0; k < dim; k++) off[k] = x[i].u[k] - y[i].u[k];
        PathRec ys;
        m.pc = kPStart;
        if (run_perturb(sv, z[i], off, nj, ys, m) == kStepDone) ev.a_star_green = clamp01(m.e.ss / ev.ss_z);
    }
    ssz[i] = ev.ss_z;
    out[i] = ev;
}

// The H2MC kernel ratio of PH2MCSmallStep::Mutate (drsmallstep.cpp:169-196) as
// the chain loop's Gaussian kernel computes it: the Gaussians at x and z from
// their derivatives (grad/hess rows i and n + i), then log N_z(-o) - log N_x(o)
// in FP64. One team per H2MC case with a contributing z.
__global__ void __launch_bounds__(32 * kGaussTeamWarps) k_dr_eval_ratio(const PathRec *x, const drmlt_contrib *xc,
                                                                       const float *ssz, const float *o2,
                                                                       const int *aniso, int n, float sigma,
                                                                       int maxDim, const float *grad,
                                                                       const float *hess, double *store,
                                                                       drmlt_dr_result *out) {
    extern __shared__ double gsm[];
    const int i = blockIdx.x;
    if (i >= n || !aniso[i] || !out[i].valid_z) return;
    const int dim = path_dim(x[i].c, x[i].l);
    if (dim > maxDim) return;
    GaussSmem sm(gsm, maxDim);
    const Team tm(gauss_reduction(gsm, maxDim));
    double *gx = store + size_t(2 * i) * kGaussStride, *gz = store + size_t(2 * i + 1) * kGaussStride;
    compute_gaussian_team(dim, H2mcParam(sigma), xc[i].ss, grad + size_t(i) * kMaxDim,
                          hess + size_t(i) * kMaxDim * kMaxDim, sm, GaussView(gx), tm);
    __syncthreads();
    compute_gaussian_team(dim, H2mcParam(sigma), ssz[i], grad + size_t(n + i) * kMaxDim,
                          hess + size_t(n + i) * kMaxDim * kMaxDim, sm, GaussView(gz), tm);
    __syncthreads();
    const float *o = o2 + size_t(i) * kMaxDim;
    const double px = gauss_logpdf_team(dim, o, -1.0, GaussView(gz), tm);
    const double py = gauss_logpdf_team(dim, o, 1.0, GaussView(gx), tm);
    if (threadIdx.x == 0) out[i].log_ratio = px - py;
}

// The second-stage ratio and the Green / Mira acceptances (k_finish's arithmetic).
__global__ void k_dr_eval_finish(const PathRec *x, const drmlt_contrib *xc, const PathRec *y, const PathRec *z,
                                 const int *aniso, int n, float sigma1, drmlt_dr_result *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    drmlt_dr_result ev = out[i];
    const int dim = path_dim(x[i].c, x[i].l);
    float a2 = 0.0f;
    if (ev.valid_z) a2 = aniso[i] ? float(::exp(ev.log_ratio)) * ev.ss_z / xc[i].ss : clamp01(ev.ss_z / xc[i].ss);
    ev.log_q_mira = mira_log_q(dim, x[i].u, y[i].u, z[i].u, sigma1);
    if (is_invalid(a2)) {
        ev.a2 = 0.0f;
    } else {
        ev.a2 = a2;
        bool draw;
        ev.alpha2_green = dr_second_acceptance(0, ev.a1, a2, ev.a_star_green, ev.ss_y, ev.ss_z, dim, x[i].u, y[i].u,
                                               z[i].u, sigma1, draw);
        ev.alpha2_mira = dr_second_acceptance(1, ev.a1, a2, ev.a_star_green, ev.ss_y, ev.ss_z, dim, x[i].u, y[i].u,
                                              z[i].u, sigma1, draw);
    }
    out[i] = ev;
}

__global__ void k_large_step_eval(SceneView s, const float *tapes, const int *tapeLen, int stride, int n,
                                  const PathRec *x, const drmlt_contrib *xc, const float *lengthCdf,
                                  const float *lengthFunc, float lengthFuncInt, int lengthCount, float *a1,
                                  int *tech, drmlt_contrib *ct, int *consumed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    TapeRng rng{tapes + size_t(i) * stride, tapeLen[i], 0};
    const int length = sample_discrete(lengthCdf, lengthCount, rng.uniform());
    int lgtLength = int(rng.uniform() * float(length + 1));
    lgtLength = lgtLength < 0 ? 0 : (lgtLength > length ? length : lgtLength);
    float a = 0.0f;
    drmlt_contrib c;
    memset(&c, 0, sizeof(c));
    tech[2 * i] = tech[2 * i + 1] = 0;
    if (length >= 1) {
        PathRec rec;
        Emit e;
        if (generate_subpath(s, length - lgtLength + 1, lgtLength, rng, rec, e)) {
            rng.uniform();  // contribution pick over a single candidate
            a = large_step_ratio(lengthFunc, lengthFuncInt, lengthCount, x[i].c + x[i].l - 1, xc[i].ls, e.c + e.l - 1,
                                 e.ls);
            tech[2 * i] = e.c;
            tech[2 * i + 1] = e.l;
            c.screen[0] = e.screen[0];
            c.screen[1] = e.screen[1];
            c.rgb[0] = e.rgb.x;
            c.rgb[1] = e.rgb.y;
            c.rgb[2] = e.rgb.z;
            c.ls = e.ls;
            c.ss = e.ss;
            c.valid = 1;
        }
    }
    a1[i] = a;
    ct[i] = c;
    consumed[i] = rng.pos;
}

}  // namespace

extern "C" {

int drmlt_dr_eval(void *handle, int n, const drmlt_path *x, const drmlt_contrib *x_contrib, const float *offset1,
                  const float *offset2, const int32_t *aniso, drmlt_dr_result *out, drmlt_path *y_out,
                  drmlt_path *z_out) {
    if (!handle || n < 0 || (n && (!x || !x_contrib || !offset1 || !offset2 || !aniso || !out)))
        return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(x, n);
    if (rc) return rc;
    Renderer *r = static_cast<Renderer *>(handle);
    const int maxDim = kMaxDim;
    DevBuf<PathRec> dx, dyz;
    DevBuf<drmlt_contrib> dxc;
    DevBuf<float> do1, do2, dss, dg, dh;
    DevBuf<int> dan;
    DevBuf<drmlt_dr_result> dout;
    DevBuf<double> dstore;
    if ((rc = dx.put(reinterpret_cast<const PathRec *>(x), n)) || (rc = dxc.put(x_contrib, n)) ||
        (rc = do1.put(offset1, size_t(n) * kMaxDim)) || (rc = do2.put(offset2, size_t(n) * kMaxDim)) ||
        (rc = dan.put(aniso, n)) || (rc = dyz.alloc(2 * size_t(n))) || (rc = dss.alloc(2 * size_t(n))) ||
        (rc = dout.alloc(n)) || (rc = dg.alloc(2 * size_t(n) * kMaxDim)) ||
        (rc = dh.alloc(2 * size_t(n) * kMaxDim * kMaxDim)) || (rc = dstore.alloc(2 * size_t(n) * kGaussStride)))
        return rc;
    PathRec *dy = dyz.p, *dz = dyz.p + n;
    k_dr_eval_trace<<<(n + 127) / 128, 128>>>(r->sv, dx.p, dxc.p, do1.p, do2.p, n, dy, dz, dss.p + n, dout.p);
    CK(cudaGetLastError());
    // derivatives at x (rows 0..n-1, score ss(x)) and z (rows n..2n-1, score ss(z))
    std::vector<float> ssx(n);
    for (int i = 0; i < n; i++) ssx[i] = x_contrib[i].ss;
    CK(cudaMemcpy(dss.p, ssx.data(), n * sizeof(float), cudaMemcpyHostToDevice));
    DevBuf<PathRec> dxz;
    if ((rc = dxz.alloc(2 * size_t(n)))) return rc;
    CK(cudaMemcpy(dxz.p, dx.p, n * sizeof(PathRec), cudaMemcpyDeviceToDevice));
    CK(cudaMemcpy(dxz.p + n, dz, n * sizeof(PathRec), cudaMemcpyDeviceToDevice));
    launch_gradhess_gated(r->sv, dxz.p, dss.p, 2 * n, r->opt.max_derivative_depth, dg.p, dh.p, 0);
    CK(cudaGetLastError());
    k_dr_eval_ratio<<<n, 32 * kGaussTeamWarps, gauss_smem_bytes(maxDim)>>>(
        dx.p, dxc.p, dss.p + n, do2.p, dan.p, n, r->opt.perturb_stddev, maxDim, dg.p, dh.p, dstore.p, dout.p);
    CK(cudaGetLastError());
    k_dr_eval_finish<<<(n + 127) / 128, 128>>>(dx.p, dxc.p, dy, dz, dan.p, n, r->opt.perturb_stddev, dout.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = dout.get(out, n))) return rc;
    if (y_out) CK(cudaMemcpy(y_out, dy, n * sizeof(PathRec), cudaMemcpyDeviceToHost));
    if (z_out) CK(cudaMemcpy(z_out, dz, n * sizeof(PathRec), cudaMemcpyDeviceToHost));
    return DRMLT_OK;
}

int drmlt_large_step_eval(void *handle, int n, const float *tapes, const int32_t *tape_len, int stride,
                          const drmlt_path *x, const drmlt_contrib *x_contrib, const float *length_func,
                          int num_lengths, float *a1, int32_t *out_tech, drmlt_contrib *out_contrib,
                          int32_t *out_consumed) {
    if (!handle || n < 0 || stride < 1 || num_lengths < 1 ||
        (n && (!tapes || !tape_len || !x || !x_contrib || !length_func || !a1 || !out_tech || !out_contrib ||
               !out_consumed)))
        return fail(DRMLT_E_ARG, "bad argument");
    if (n == 0) return DRMLT_OK;
    int rc = check_paths(x, n);
    if (rc) return rc;
    for (int i = 0; i < n; i++) {
        if (tape_len[i] < 0 || tape_len[i] > stride) return fail(DRMLT_E_ARG, "tape length out of range");
        if (x[i].c + x[i].l - 1 >= num_lengths) return fail(DRMLT_E_ARG, "current path longer than the length table");
    }
    Renderer *r = static_cast<Renderer *>(handle);
    std::vector<float> func(length_func, length_func + num_lengths), cdf;
    float funcInt;
    piecewise_constant(func, cdf, funcInt);
    DevBuf<float> dt, dcdf, dfunc, da;
    DevBuf<int> dlen, dtech, dcons;
    DevBuf<PathRec> dx;
    DevBuf<drmlt_contrib> dxc, dct;
    if ((rc = dt.put(tapes, size_t(n) * stride)) || (rc = dlen.put(tape_len, n)) ||
        (rc = dx.put(reinterpret_cast<const PathRec *>(x), n)) || (rc = dxc.put(x_contrib, n)) ||
        (rc = dcdf.put(cdf.data(), cdf.size())) || (rc = dfunc.put(func.data(), func.size())) ||
        (rc = da.alloc(n)) || (rc = dtech.alloc(2 * size_t(n))) || (rc = dct.alloc(n)) || (rc = dcons.alloc(n)))
        return rc;
    k_large_step_eval<<<(n + 127) / 128, 128>>>(r->sv, dt.p, dlen.p, stride, n, dx.p, dxc.p, dcdf.p, dfunc.p, funcInt,
                                                num_lengths, da.p, dtech.p, dct.p, dcons.p);
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    if ((rc = da.get(a1, n)) || (rc = dtech.get(out_tech, 2 * size_t(n))) || (rc = dct.get(out_contrib, n)))
        return rc;
    return dcons.get(out_consumed, n);
}

}  // extern "C"
