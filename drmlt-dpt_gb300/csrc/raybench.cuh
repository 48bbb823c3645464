// Ray-casting benchmark on the scene BVH: device-generated ray batches of three
// kinds and a traversal kernel timed on its own, with node / triangle visit
// counters for the bytes-visited roofline.
//   kind 0  primary camera rays, one per pixel sample (closest hit)
//   kind 1  diffuse bounce rays from the camera rays' first hits, cosine-
//           distributed about the shading normal (closest hit)
//   kind 2  shadow rays of length 2 from the same hits (any hit)
// Also the arithmetic-peak benchmark (k_fma_peak) that the compute rooflines
// of the derivative (FP32) and Gaussian (FP64) kernels are quoted against.
#pragma once
#include "bsdf_light.cuh"

namespace drmlt {

__global__ void k_rays_setup(SceneView s, int kind, int n, unsigned long long seed, float4 *org, float4 *dir) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Rng rng(seed, (unsigned long long)i, 0x7A7ull);
    const int W = s.cam.width, H = s.cam.height;
    const int pix = i % (W * H);
    const float sx = (float(pix % W) + rng.uniform()) / float(W);
    const float sy = (float(pix / W) + rng.uniform()) / float(H);
    V3 o, d;
    float minT, maxT;
    sample_primary(s.cam, sx, sy, o, d, minT, maxT);
    if (kind == 0) {
        org[i] = make_float4(o.x, o.y, o.z, minT);
        dir[i] = make_float4(d.x, d.y, d.z, maxT);
        return;
    }
    Isect is;
    int tri = -1;
    if (!intersect(s, o, d, minT, maxT, tri, is)) {
        org[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
        dir[i] = make_float4(0.0f, 0.0f, 1.0f, -1.0f);  // tmax < tmin: no ray
        return;
    }
    V3 nrm = is.shadingNormal;
    if (dot(nrm, d) > 0.0f) nrm = -nrm;
    const V3 l = sample_cos_hemisphere(rng.uniform(), rng.uniform());
    V3 b0, b1;
    coordinate_system(nrm, b0, b1);
    const V3 w = l.x * b0 + l.y * b1 + l.z * nrm;
    org[i] = make_float4(is.position.x, is.position.y, is.position.z, kIsectEps);
    dir[i] = make_float4(w.x, w.y, w.z, kind == 1 ? INFINITY : 2.0f);
}

// One traversal per ray; kCount adds per-warp sums of the visit counters to
// counters[0..2] (rays traced, nodes fetched, triangles tested).
template <bool kCount>
__global__ void __launch_bounds__(128) k_rays_trace(SceneView s, int anyHit, int n, const float4 *org,
                                                    const float4 *dir, int *hit, unsigned long long *counters) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned nodes = 0, tests = 0, rays = 0;
    if (i < n) {
        const float4 a = org[i], b = dir[i];
        int t = -1;
        if (b.w >= a.w) {
            rays = 1;
            const V3 o(a.x, a.y, a.z), d(b.x, b.y, b.z);
            t = anyHit ? traverse<true, kCount>(s, o, d, a.w, b.w, &nodes, &tests)
                       : traverse<false, kCount>(s, o, d, a.w, b.w, &nodes, &tests);
        }
        hit[i] = t;
    }
    if (kCount) {
        for (int off = 16; off > 0; off >>= 1) {
            rays += __shfl_down_sync(0xffffffffu, rays, off);
            nodes += __shfl_down_sync(0xffffffffu, nodes, off);
            tests += __shfl_down_sync(0xffffffffu, tests, off);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(counters, (unsigned long long)rays);
            atomicAdd(counters + 1, (unsigned long long)nodes);
            atomicAdd(counters + 2, (unsigned long long)tests);
        }
    }
}

// FMA throughput: 8 independent fused multiply-add chains per thread (enough
// in flight to cover the FMA latency on every SM sub-partition), iterated
// `iters` times; 2 flops per FMA. The chains converge to b / (1 - a) > 0, so
// the sink store never happens; it keeps the chains live.
__device__ __forceinline__ float fma_t(float x, float a, float b) { return fmaf(x, a, b); }
__device__ __forceinline__ double fma_t(double x, double a, double b) { return fma(x, a, b); }

template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T a, T b, T *sink) {
    T x[8];
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = T(threadIdx.x + k) * T(1e-3);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int k = 0; k < 8; k++) x[k] = fma_t(x[k], a, b);
    }
    T sum = T(0);
#pragma unroll
    for (int k = 0; k < 8; k++) sum += x[k];
    if (sum == T(-1)) sink[blockIdx.x] = sum;
}

}  // namespace drmlt
