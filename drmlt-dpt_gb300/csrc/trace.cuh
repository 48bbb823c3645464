// Ray casting on the device: closest hit and occlusion over the binary SAH BVH
// built by bvh.cpp, then the exact re-intersection of the hit triangle that the
// reference performs after Embree returns a primitive ID
// (src/scene.cpp:80-111 Intersect/Occluded, src/trianglemesh.cpp:30-79,187-236).
#pragma once
#include "common.cuh"

namespace drmlt {

struct Isect {
    V3 position;
    V3 shadingNormal;
    V3 geomNormal;
};

DEV V3 ld3(const float *p) { return V3(__ldg(p), __ldg(p + 1), __ldg(p + 2)); }

// Moller-Trumbore; returns t, or -1 for a miss (edges inclusive). The miss value
// must fail `t > tmin` for every tmin >= 0, including rays with tmax = +inf.
DEV float hit_triangle(const V3 &o, const V3 &d, const float4 &p0, const float4 &e1, const float4 &e2) {
    const V3 E1(e1.x, e1.y, e1.z), E2(e2.x, e2.y, e2.z);
    const V3 pv = cross(d, E2);
    const float det = dot(E1, pv);
    if (det == 0.0f) return -1.0f;
    const float inv = 1.0f / det;
    const V3 s = o - V3(p0.x, p0.y, p0.z);
    const float u = dot(s, pv) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return -1.0f;
    const V3 q = cross(s, E1);
    const float v = dot(d, q) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return -1.0f;
    return dot(E2, q) * inv;
}

DEV bool slab(const V3 &o, const V3 &inv, float lx, float ly, float lz, float hx, float hy, float hz,
              float tmin, float tmax, float &tenter) {
    float t0x = (lx - o.x) * inv.x, t1x = (hx - o.x) * inv.x;
    float t0y = (ly - o.y) * inv.y, t1y = (hy - o.y) * inv.y;
    float t0z = (lz - o.z) * inv.z, t1z = (hz - o.z) * inv.z;
    const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    tenter = tn;
    return tn <= tf;
}

// Traverses the BVH. anyHit: stop at the first hit in (tmin, tmax).
// Returns the global triangle index of the closest hit or -1. kCount: adds the
// nodes fetched and triangles tested to *nodes / *tests (the ray benchmark).
template <bool anyHit, bool kCount = false>
DEV_SHARED int traverse(const SceneView &s, const V3 &o, const V3 &d, float tmin, float tmax, unsigned *nodes = nullptr,
                 unsigned *tests = nullptr) {
    const float tiny = 1e-20f;
    const V3 inv(1.0f / (fabsf(d.x) > tiny ? d.x : copysignf(tiny, d.x)),
                 1.0f / (fabsf(d.y) > tiny ? d.y : copysignf(tiny, d.y)),
                 1.0f / (fabsf(d.z) > tiny ? d.z : copysignf(tiny, d.z)));
    int stack[64];
    int sp = 0;
    int node = 0;
    int best = -1;
    float tbest = tmax;
    for (int iter = 0; iter < (1 << 20); iter++) {
        const BvhNode n = s.nodes[node];
        if (kCount) ++*nodes;
        int next[2];
        int nn = 0;
        float te0, te1;
        const bool h0 = slab(o, inv, n.lo0.x, n.lo0.y, n.lo0.z, n.lo0.w, n.hi0.x, n.hi0.y, tmin, tbest, te0);
        const bool h1 = slab(o, inv, n.hi0.z, n.hi0.w, n.b1.x, n.b1.y, n.b1.z, n.b1.w, tmin, tbest, te1);
        const int child[2] = {n.link.x, n.link.y};
        const int count[2] = {n.link.z, n.link.w};
        const bool hit[2] = {h0, h1};
        for (int c = 0; c < 2; c++) {
            if (!hit[c]) continue;
            if (count[c] > 0) {
                for (int k = 0; k < count[c]; k++) {
                    const Tri tri = s.tris[child[c] + k];
                    if (kCount) ++*tests;
                    const float t = hit_triangle(o, d, tri.p0, tri.e1, tri.e2);
                    if (t > tmin && t <= tbest && t < INFINITY) {
                        best = __float_as_int(tri.p0.w);
                        if (anyHit) return best;
                        tbest = t;
                    }
                }
            } else if (count[c] == 0 && child[c] >= 0) {
                next[nn++] = child[c];
            }
        }
        if (nn == 2) {
            // visit the nearer child first
            if (te1 < te0) { const int t = next[0]; next[0] = next[1]; next[1] = t; }
            if (sp < 64) stack[sp++] = next[1];
            node = next[0];
        } else if (nn == 1) {
            node = next[0];
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return best;
}

// TriangleIntersect of src/trianglemesh.cpp:30-79 on the hit triangle: only the
// v >= 0 and u + v <= 1 tests are repeated, exactly as the reference does.
DEV bool reintersect(const SceneView &s, int tri, const V3 &org, const V3 &dir, Isect &isect) {
    const float *P = s.triP + 9 * tri;
    const V3 p0 = ld3(P), e1 = ld3(P + 3), e2 = ld3(P + 6);
    isect.geomNormal = normalize(cross(e1, e2));
    const V3 s1 = cross(dir, e2);
    const float divisor = dot(s1, e1);
    if (divisor == 0.0f) return false;
    const float invDivisor = 1.0f / divisor;
    const V3 sv = org - p0;
    const float u = dot(sv, s1) * invDivisor;
    const V3 s2 = cross(sv, e1);
    const float v = dot(dir, s2) * invDivisor;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    const float t = dot(e2, s2) * invDivisor;
    const float w = 1.0f - u - v;
    const float *N = s.triN + 9 * tri;
    const V3 n0 = ld3(N), n1 = ld3(N + 3), n2 = ld3(N + 6);
    isect.position = org + t * dir;
    isect.shadingNormal = normalize(V3(w * n0 + u * n1 + v * n2));
    if (dot(isect.geomNormal, isect.shadingNormal) < 0.0f) isect.geomNormal = -isect.geomNormal;
    return true;
}

// Intersect(scene, time, raySeg, shapeInst, isect) of src/path.cpp:94-103:
// `tri` is updated whenever the BVH reports a hit, even if the re-intersection fails.
DEV bool intersect(const SceneView &s, const V3 &org, const V3 &dir, float tmin, float tmax, int &tri,
                   Isect &isect) {
    const int hit = traverse<false>(s, org, dir, tmin, tmax);
    if (hit < 0) return false;
    tri = hit;
    return reintersect(s, hit, org, dir, isect);
}

// Occluded(scene, time, ray, dist) of src/scene.cpp:95-105.
DEV bool occluded(const SceneView &s, const V3 &org, const V3 &dir, float dist) {
    const float maxT = isinf(dist) ? INFINITY : (1.0f - kShadowEps) * dist;
    return traverse<true>(s, org, dir, kIsectEps, maxT) >= 0;
}

}  // namespace drmlt
