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
    launch_gradhess_paths(r->sv, dp.p, du.p, n, dg.p, dh.p, 0);
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
