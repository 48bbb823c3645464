// ORACLE -- test infrastructure only (parity checker and CPU baseline; never
// part of the shipped GPU path).
//
// A CPU restatement of the reference's DRMLT hot path, written in C-style C++
// (templates are used only for the scalar type of the derivative restatement),
// following:
//   brute-force ray casting standing in for Embree  src/scene.cpp:80-111
//   re-intersection                                  src/trianglemesh.cpp:30-79,187-236
//   Lambertian / Phong BSDFs                         src/lambertian.cpp, src/phong.cpp:21-167
//   area / point lights                              src/arealight.cpp:29-102, src/pointlight.cpp
//   environment light                                src/envlight.cpp:24-247
//   camera                                           src/camera.cpp:38-75
//   GeneratePathBidir / GenerateSubpath              src/path.cpp:978-1269
//   PerturbPathBidir                                 src/path.cpp:1480-1628
//   GeneratePath (direct pass)                       src/path.cpp:343-445
//   chad path function (AD semantics)                src/path.cpp:2987-3175
//   derivatives: forward-over-reverse (chad's scheme, src/chad.cpp:342-418)
//                and FP64 central differences
//   ComputeGaussian / GaussianLogPdf / GenerateSample drsmallstep.cpp:19-266, gaussian.cpp
//   DR chain loop                                    src/integrators/delayed/delayed.cpp:14-673
// Pairs drawn as Vector2(u(), u()) take the second component first (the
// reference's compiler evaluates those arguments right to left).
#include "../include/drmlt_capi.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace ora {

const float PI = 3.14159265358979323846f;
const float INV_PI = 1.0f / PI;
const float TWO_PI = 2.0f * PI;
const float INV_TWO_PI = 1.0f / TWO_PI;
const float ISECT_EPS = 1e-3f, SHADOW_EPS = 1e-3f, COS_EPS = 1e-4f;
const int MAXL = 12, MAXD = 24, MAXF = 14;

struct V3 {
    float x, y, z;
};
static inline V3 mk(float x, float y, float z) { V3 v = {x, y, z}; return v; }
static inline V3 add(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 neg(V3 a) { return mk(-a.x, -a.y, -a.z); }
static inline V3 mul(V3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline V3 cmul(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) { return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float sq(float x) { return x * x; }
static inline float lensq(V3 a) { return sq(a.x) + sq(a.y) + sq(a.z); }
static inline V3 norm(V3 a) { float il = 1.0f / std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return mul(a, il); }
static inline float lum(V3 a) { return a.x * 0.212671f + a.y * 0.715160f + a.z * 0.072169f; }
// Eigen's isZero() at its default float precision 1e-5, the test the reference
// applies to BSDF values and splats (src/path.cpp:556, 651, 751, 889, 908, 1454;
// delayed.cpp:260).
static inline bool iszero(V3 a) { return std::fabs(a.x) <= 1e-5f && std::fabs(a.y) <= 1e-5f && std::fabs(a.z) <= 1e-5f; }
static inline float maxc(V3 a) { return std::max(a.x, std::max(a.y, a.z)); }
static inline float mis(float x) { return x * x; }
static inline float modulo1(float a) { float r = std::fmod(a, 1.0f); return r < 0 ? r + 1.0f : r; }

// ---------------------------------------------------------------- scene
struct Bsdf {
    int type, twoSided;
    V3 kd, ks, kt;
    float expo, ksW;
    float alpha, eta, invEta;  // rough dielectric (src/roughdielectric.h:10-18)
};
struct Light {
    int type, shape, triOff, ntri;
    V3 E, pos;
    float w, invArea;
    std::vector<float> triCdf;
};
// Bounding-volume hierarchy of the oracle's casts (built in ora_create, see cast_bvh).
struct BvhNodeO {
    float lo[3], hi[3];
    int first, count;  // count > 0: leaf over idx[first, first + count); else children first, first + 1
};
struct BvhO {
    std::vector<BvhNodeO> nodes;
    std::vector<int> idx;
};
struct Scene {
    int ntri;
    BvhO bvh;  // empty below kBvhMinTris triangles
    std::vector<V3> p0, e1, e2, n0, n1, n2;
    std::vector<int> triShape;
    std::vector<int> shapeBsdf, shapeLight, shapeFirst;
    std::vector<Bsdf> bsdfs;
    std::vector<Light> lights;
    std::vector<float> lightCdf, lightFunc;
    float lightFuncInt, lightWeightSum;
    float s2c[16], c2s[16], c2w[16], w2c[16], dist, nearc, farc;
    int W, H;
    drmlt_options opt;
    V3 bsC;
    float bsR;
    // environment light: image (top row first), EnvmapSampleInfo, toWorld / toLight 3x3
    int envL, envW, envH;
    std::vector<float> envImg, envRows, envCols, envRowW;
    float envNorm, envPix[2], envW2L[9], envL2W[9];
};

static void piecewise(const std::vector<float> &f, std::vector<float> &cdf, float &fi) {
    const int n = (int)f.size();
    cdf.assign(n + 1, 0.0f);
    for (int i = 1; i <= n; i++) cdf[i] = cdf[i - 1] + f[i - 1] / float(n);
    fi = cdf[n];
    for (int i = 1; i <= n; i++) cdf[i] = fi == 0.0f ? float(i) / float(n) : cdf[i] / fi;
}
static int sample_discrete(const std::vector<float> &cdf, float u) {
    const int count = (int)cdf.size() - 1;
    const int off = int(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin()) - 1;
    return std::min(std::max(off, 0), count - 1);
}

// ---------------------------------------------------------------- ray casting
// Float Moller-Trumbore (edges inclusive) of ray (o, d) against triangle t:
// the hit distance, or NaN for a miss.
static inline float tri_hit(const Scene &s, int t, V3 o, V3 d) {
    const V3 pv = cross(d, s.e2[t]);
    const float det = dot(s.e1[t], pv);
    if (det == 0.0f) return NAN;
    const float inv = 1.0f / det;
    const V3 sv = sub(o, s.p0[t]);
    const float u = dot(sv, pv) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return NAN;
    const V3 q = cross(sv, s.e1[t]);
    const float v = dot(d, q) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return NAN;
    return dot(s.e2[t], q) * inv;
}

// Closest hit over all triangles in index order: the nearest t in (tmin, tmax]
// and, among equal distances, the highest index (a later triangle at the same t
// replaces the earlier one). anyHit: the lowest-index triangle in range.
static int cast_brute(const Scene &s, V3 o, V3 d, float tmin, float tmax, bool anyHit) {
    int best = -1;
    float tb = tmax;
    for (int t = 0; t < s.ntri; t++) {
        const float th = tri_hit(s, t, o, d);
        if (th > tmin && th <= tb && std::isfinite(th)) {
            best = t;
            tb = th;
            if (anyHit) return t;
        }
    }
    return best;
}

// Bounding-volume hierarchy for the multi-million-triangle scenes, so that the
// oracle's casts stay O(log n). It is built independently of the GPU library's
// binned-SAH tree: object-median splits along the longest centroid axis, leaves
// of up to 4 triangles. Culling is conservative (boxes padded outward, the
// distance window widened), and the hit rule is cast_brute's (nearest t, the
// highest index on a tie), so a closest-hit cast returns the same triangle as
// the brute-force loop over every triangle; an any-hit cast returns some hit in
// range (the same occlusion answer, not necessarily the same triangle).
static const int kBvhMinTris = 1024;  // below this the brute-force loop is used

static void bvh_build(const Scene &s, BvhO &b) {
    const int n = s.ntri;
    b.idx.resize(n);
    std::vector<float> cen(3 * size_t(n)), lo(3 * size_t(n)), hi(3 * size_t(n));
    for (int t = 0; t < n; t++) {
        b.idx[t] = t;
        const V3 p[3] = {s.p0[t], add(s.p0[t], s.e1[t]), add(s.p0[t], s.e2[t])};
        for (int a = 0; a < 3; a++) {
            const float v0 = a == 0 ? p[0].x : a == 1 ? p[0].y : p[0].z;
            const float v1 = a == 0 ? p[1].x : a == 1 ? p[1].y : p[1].z;
            const float v2 = a == 0 ? p[2].x : a == 1 ? p[2].y : p[2].z;
            const float l = std::min(v0, std::min(v1, v2)), h = std::max(v0, std::max(v1, v2));
            // outward padding: relative to the coordinates' magnitude, so that a
            // hit point computed in float from (p0, e1, e2) stays inside
            const float pad = 1e-4f * std::max(std::fabs(l), std::fabs(h)) + 1e-6f;
            lo[3 * size_t(t) + a] = l - pad;
            hi[3 * size_t(t) + a] = h + pad;
            cen[3 * size_t(t) + a] = 0.5f * (l + h);
        }
    }
    b.nodes.clear();
    b.nodes.reserve(2 * size_t(n / 2 + 1));
    struct Job { int node, begin, end; };
    std::vector<Job> stack;
    b.nodes.push_back(BvhNodeO());
    stack.push_back({0, 0, n});
    while (!stack.empty()) {
        const Job j = stack.back();
        stack.pop_back();
        float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int i = j.begin; i < j.end; i++) {
            const size_t t = size_t(b.idx[i]);
            for (int a = 0; a < 3; a++) {
                blo[a] = std::min(blo[a], lo[3 * t + a]);
                bhi[a] = std::max(bhi[a], hi[3 * t + a]);
                clo[a] = std::min(clo[a], cen[3 * t + a]);
                chi[a] = std::max(chi[a], cen[3 * t + a]);
            }
        }
        BvhNodeO &nd = b.nodes[j.node];
        for (int a = 0; a < 3; a++) {
            nd.lo[a] = blo[a];
            nd.hi[a] = bhi[a];
        }
        const int cnt = j.end - j.begin;
        int axis = 0;
        for (int a = 1; a < 3; a++)
            if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
        if (cnt <= 4 || !(chi[axis] > clo[axis])) {
            nd.first = j.begin;
            nd.count = cnt;
            continue;
        }
        const int mid = j.begin + cnt / 2;
        std::nth_element(b.idx.begin() + j.begin, b.idx.begin() + mid, b.idx.begin() + j.end, [&](int x, int y) {
            const float cx = cen[3 * size_t(x) + axis], cy = cen[3 * size_t(y) + axis];
            return cx < cy || (cx == cy && x < y);
        });
        const int left = int(b.nodes.size());
        b.nodes[j.node].first = left;
        b.nodes[j.node].count = 0;
        b.nodes.push_back(BvhNodeO());
        b.nodes.push_back(BvhNodeO());
        stack.push_back({left, j.begin, mid});
        stack.push_back({left + 1, mid, j.end});
    }
}

// Ray-box overlap on [t0, t1]; NaN slab values (a zero direction component on
// a box face) leave the window unchanged, which only keeps more boxes.
static inline bool box_overlap(const BvhNodeO &n, const float o[3], const float inv[3], float t0, float t1,
                               float &tenter) {
    for (int a = 0; a < 3; a++) {
        float tn = (n.lo[a] - o[a]) * inv[a], tf = (n.hi[a] - o[a]) * inv[a];
        if (tn > tf) std::swap(tn, tf);
        t0 = std::max(t0, tn);
        t1 = std::min(t1, tf);
    }
    tenter = t0;
    return t0 <= t1;
}

static int cast_bvh(const Scene &s, V3 o, V3 d, float tmin, float tmax, bool anyHit) {
    const BvhO &b = s.bvh;
    const float of[3] = {o.x, o.y, o.z};
    const float inv[3] = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    int best = -1;
    float tb = tmax;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    const float lowT = tmin - 1e-3f - 1e-4f * std::fabs(tmin);
    while (sp > 0) {
        const BvhNodeO &n = b.nodes[stack[--sp]];
        // a triangle at exactly tb can still replace the best hit (tie rule)
        const float highT = std::isfinite(tb) ? tb + 1e-4f * std::fabs(tb) + 1e-5f : tb;
        float te;
        if (!box_overlap(n, of, inv, lowT, highT, te)) continue;
        if (n.count > 0) {
            for (int i = n.first; i < n.first + n.count; i++) {
                const int t = b.idx[i];
                const float th = tri_hit(s, t, o, d);
                if (th > tmin && std::isfinite(th) && (th < tb || (th == tb && t > best))) {
                    best = t;
                    tb = th;
                    if (anyHit) return t;
                }
            }
            continue;
        }
        float e0, e1;
        const bool h0 = box_overlap(b.nodes[n.first], of, inv, lowT, highT, e0);
        const bool h1 = box_overlap(b.nodes[n.first + 1], of, inv, lowT, highT, e1);
        if (h0 && h1) {
            // nearer child on top of the stack
            if (e0 <= e1) {
                stack[sp++] = n.first + 1;
                stack[sp++] = n.first;
            } else {
                stack[sp++] = n.first;
                stack[sp++] = n.first + 1;
            }
        } else if (h0) {
            stack[sp++] = n.first;
        } else if (h1) {
            stack[sp++] = n.first + 1;
        }
    }
    return best;
}

static int cast(const Scene &s, V3 o, V3 d, float tmin, float tmax, bool anyHit) {
    return s.ntri >= kBvhMinTris ? cast_bvh(s, o, d, tmin, tmax, anyHit) : cast_brute(s, o, d, tmin, tmax, anyHit);
}
struct Isect {
    V3 p, ns, ng;
};
static bool intersect(const Scene &s, V3 o, V3 d, float tmin, float tmax, int &tri, Isect &is) {
    const int t = cast(s, o, d, tmin, tmax, false);
    if (t < 0) return false;
    tri = t;
    is.ng = norm(cross(s.e1[t], s.e2[t]));
    const V3 s1 = cross(d, s.e2[t]);
    const float div = dot(s1, s.e1[t]);
    if (div == 0.0f) return false;
    const float inv = 1.0f / div;
    const V3 sv = sub(o, s.p0[t]);
    const float u = dot(sv, s1) * inv;
    const V3 s2 = cross(sv, s.e1[t]);
    const float v = dot(d, s2) * inv;
    if (!(v >= 0.0f && u + v <= 1.0f)) return false;
    const float th = dot(s.e2[t], s2) * inv;
    const float w = 1.0f - u - v;
    is.p = add(o, mul(d, th));
    is.ns = norm(add(add(mul(s.n0[t], w), mul(s.n1[t], u)), mul(s.n2[t], v)));
    if (dot(is.ng, is.ns) < 0.0f) is.ng = neg(is.ng);
    return true;
}
static bool occluded(const Scene &s, V3 o, V3 d, float dist) {
    const float maxT = std::isinf(dist) ? INFINITY : (1.0f - SHADOW_EPS) * dist;
    return cast(s, o, d, ISECT_EPS, maxT, true) >= 0;
}

// ---------------------------------------------------------------- BSDF
struct BOut {
    V3 f;
    float cosWo, pdf, rev;
};
static void frame(V3 n, V3 &b1, V3 &b2) {
    if (n.z < float(-1.0 + 1e-6)) {
        b1 = mk(0, -1, 0);
        b2 = mk(-1, 0, 0);
        return;
    }
    const float a = 1.0f / (1.0f + n.z), b = -n.x * n.y * a;
    b1 = mk(1.0f - sq(n.x) * a, b, -n.x);
    b2 = mk(b, 1.0f - sq(n.y) * a, -n.y);
}
static V3 reflect(V3 wi, V3 n) { return sub(mul(n, 2.0f * dot(wi, n)), wi); }
// ---- rough dielectric, Beckmann microfacets (src/roughdielectric.cpp, src/microfacet.h)
static float beck_d(V3 h, float a) {
    const float c2 = sq(h.z);
    return std::exp(-((sq(h.x) / sq(a) + sq(h.y) / sq(a)) / c2)) / (PI * a * a * sq(c2));
}
static float beck_g1(float a, float c) {
    const float t = std::sqrt(std::fabs(1.0f - sq(c))) / c;
    if (t <= 0.0f) return 1.0f;
    const float x = 1.0f / (a * t);
    if (x >= 1.6f) return 1.0f;
    return (3.535f * x + 2.181f * x * x) / (1.0f + 2.276f * x + 2.577f * x * x);
}
static float fresnel(float ci_, float &ct_, float eta, float inv) {
    const float sc = ci_ > 0.0f ? inv : eta;
    const float ct2 = 1.0f - (1.0f - sq(ci_)) * sq(sc);
    if (ct2 <= 0.0f) { ct_ = 0.0f; return 1.0f; }
    const float ci = std::fabs(ci_), ct = std::sqrt(ct2);
    const float rs = (ci - eta * ct) / (ci + eta * ct), rp = (eta * ci - ct) / (eta * ci + ct);
    ct_ = ci_ > 0.0f ? -ct : ct;
    return 0.5f * (sq(rs) + sq(rp));
}
static void rd_eval(const Bsdf &b, V3 wi, V3 n, V3 wo, BOut &o, bool adj) {
    o.f = mk(0, 0, 0);
    o.cosWo = 0;
    o.pdf = o.rev = 0;
    const float cwi = dot(wi, n);
    if (std::fabs(cwi) < COS_EPS) return;
    const float cwo = dot(wo, n);
    o.cosWo = cwo;
    if (std::fabs(cwo) < COS_EPS) return;
    const bool refl = cwi * cwo > 0.0f;
    const float e = cwi > 0.0f ? b.eta : b.invEta, re = cwo > 0.0f ? b.eta : b.invEta;
    V3 H = refl ? norm(add(wi, wo)) : norm(add(wi, mul(wo, e)));
    if (dot(H, n) < 0.0f) H = neg(H);
    const float chi = dot(wi, H), cho = dot(wo, H);
    if (std::fabs(chi) < COS_EPS || std::fabs(cho) < COS_EPS) return;
    if (chi * cwi <= 0.0f || cho * cwo <= 0.0f) return;
    V3 b0, b1;
    frame(n, b0, b1);
    const V3 lh = mk(dot(b0, H), dot(b1, H), dot(n, H));
    const float D = beck_d(lh, b.alpha);
    if (D <= 0.0f) return;
    float ct;
    const float F = fresnel(chi, ct, b.eta, b.invEta);
    const float aci = std::fabs(cwi), aco = std::fabs(cwo);
    const float G = beck_g1(b.alpha, aci) * beck_g1(b.alpha, aco);
    const float prob = lh.z * beck_d(lh, b.alpha * (1.2f - 0.2f * std::sqrt(aci)));
    if (prob < 1e-20f) return;
    const float rprob = lh.z * beck_d(lh, b.alpha * (1.2f - 0.2f * std::sqrt(aco)));
    if (refl) {
        o.f = mul(b.ks, std::fabs(F * D * G / (4.0f * cwi)));
        o.pdf = std::fabs(prob * F / (4.0f * cho));
        o.rev = std::fabs(rprob * F / (4.0f * chi));
    } else {
        const float den = chi + e * cho, rden = cho + re * chi;
        const float fac = adj ? 1.0f : sq(1.0f / e);
        o.f = mul(b.kt, std::fabs(fac * ((1.0f - F) * D * G * sq(e) * chi * cho) / (cwi * sq(den))));
        o.pdf = std::fabs(prob * (1.0f - F) * (sq(e) * cho) / sq(den));
        o.rev = std::fabs(rprob * (1.0f - F) * (sq(re) * chi) / sq(rden));
    }
}
static bool rd_sample(const Bsdf &b, V3 wi, V3 n, float r0, float r1, float ud, V3 &wo, BOut &o, bool adj) {
    const float cwi = dot(wi, n);
    if (std::fabs(cwi) < COS_EPS) return false;
    // SampleMicronormal (src/microfacet.h:166-185)
    const float sa = b.alpha * (1.2f - 0.2f * std::sqrt(std::fabs(cwi)));
    const float phi = TWO_PI * r1, a2 = sq(sa);
    const float t2 = a2 * (-std::log(std::max(1.0f - r0, 1e-6f)));
    const float cm = 1.0f / std::sqrt(1.0f + t2), cm2 = sq(cm);
    const float mpdf = (1.0f - r0) / (PI * a2 * cm * cm2);
    const float sm = std::sqrt(std::max(1.0f - cm2, 0.0f));
    const V3 lh = mk(sm * std::cos(phi), sm * std::sin(phi), cm);
    V3 b0, b1;
    frame(n, b0, b1);
    const V3 H = add(add(mul(b0, lh.x), mul(b1, lh.y)), mul(n, lh.z));
    const float chi = dot(wi, H);
    if (std::fabs(chi) < COS_EPS) return false;
    float ct = 0.0f;
    const float F = fresnel(chi, ct, b.eta, b.invEta);
    V3 kr;
    float cho;
    o.pdf = mpdf;
    if (ud <= F) {
        wo = reflect(wi, H);
        if (F <= 0.0f || dot(n, wo) * dot(n, wi) <= 0.0f) return false;
        kr = b.ks;
        cho = dot(wo, H);
        o.pdf = std::fabs(o.pdf * F / (4.0f * cho));
        o.cosWo = dot(wo, n);
        if (std::fabs(o.cosWo) < COS_EPS) return false;
        o.rev = std::fabs(F * beck_d(lh, b.alpha * (1.2f - 0.2f * std::sqrt(std::fabs(o.cosWo)))) * lh.z *
                          (1.0f / (4.0f * chi)));
    } else {
        const float er = ct < 0.0f ? b.invEta : b.eta;  // Refract (src/utils.h:202-210)
        wo = sub(mul(H, dot(wi, H) * er + ct), mul(wi, er));
        if (F >= 1.0f || ct == 0.0f || dot(n, wo) * dot(n, wi) >= 0.0f) return false;
        const float e = cwi > 0.0f ? b.eta : b.invEta;
        kr = mul(b.kt, adj ? 1.0f : sq(1.0f / e));
        cho = dot(wo, H);
        const float den = chi + e * cho;
        o.pdf = std::fabs(o.pdf * (1.0f - F) * std::fabs((sq(e) * cho) / sq(den)));
        o.cosWo = dot(wo, n);
        if (std::fabs(o.cosWo) < COS_EPS) return false;
        const float re = o.cosWo > 0.0f ? b.eta : b.invEta, rden = cho + re * chi;
        o.rev = std::fabs((1.0f - F) * beck_d(lh, b.alpha * (1.2f - 0.2f * std::sqrt(std::fabs(o.cosWo)))) * lh.z *
                          ((sq(re) * chi) / sq(rden)));
    }
    if (std::fabs(cho) < COS_EPS || o.pdf < 1e-20f) return false;
    if (chi * cwi <= 0.0f || cho * o.cosWo <= 0.0f) return false;
    const float D = beck_d(lh, b.alpha);
    const float G = beck_g1(b.alpha, std::fabs(cwi)) * beck_g1(b.alpha, std::fabs(o.cosWo));
    o.f = mul(kr, std::fabs((D * G * chi) / (mpdf * std::fabs(cwi))));
    return true;
}

static void bsdf_eval(const Bsdf &b, V3 wi, V3 n, V3 wo, BOut &o, bool adj = false) {
    if (b.type == DRMLT_BSDF_ROUGHDIELECTRIC) { rd_eval(b, wi, n, wo, o, adj); return; }
    o.f = mk(0, 0, 0);
    o.pdf = o.rev = 0;
    float cwi = dot(n, wi);
    if (b.twoSided && cwi < 0) { cwi = -cwi; n = neg(n); }
    o.cosWo = dot(n, wo);
    if (b.type == DRMLT_BSDF_LAMBERTIAN) {
        if (cwi < COS_EPS || o.cosWo < COS_EPS) return;
        o.f = mul(b.kd, o.cosWo * INV_PI);
        o.pdf = o.cosWo * INV_PI;
        o.rev = cwi * INV_PI;
        return;
    }
    if (cwi <= COS_EPS || o.cosWo <= COS_EPS) return;
    if (b.ksW > 0) {
        const float w = std::pow(std::max(dot(reflect(wi, n), wo), 0.0f), b.expo) * INV_TWO_PI;
        if (w > 1e-10f) {
            o.f = mul(b.ks, (b.expo + 2.0f) * w);
            o.pdf = o.rev = b.ksW * (b.expo + 1.0f) * w;
        }
    }
    if (b.ksW < 1) {
        o.pdf += (1.0f - b.ksW) * o.cosWo * INV_PI;
        o.rev += (1.0f - b.ksW) * cwi * INV_PI;
        o.f = add(o.f, mul(b.kd, INV_PI));
    }
    o.f = mul(o.f, o.cosWo);
    if (maxc(o.f) < 1e-10f) o.f = mk(0, 0, 0);
}
static bool bsdf_sample(const Bsdf &b, V3 wi, V3 n, float r0, float r1, float ud, V3 &wo, BOut &o, bool adj = false) {
    if (b.type == DRMLT_BSDF_ROUGHDIELECTRIC) return rd_sample(b, wi, n, r0, r1, ud, wo, o, adj);
    float cwi = dot(wi, n);
    if (std::fabs(cwi) < COS_EPS) return false;
    if (cwi < 0) {
        if (!b.twoSided) return false;
        cwi = -cwi;
        n = neg(n);
    }
    if (b.type == DRMLT_BSDF_LAMBERTIAN) {
        V3 b1, b2;
        frame(n, b1, b2);
        const float phi = TWO_PI * r0, tmp = std::sqrt(std::max(1.0f - r1, 0.0f)), z = std::sqrt(std::max(r1, 0.0f));
        wo = add(add(mul(b1, std::cos(phi) * tmp), mul(b2, std::sin(phi) * tmp)), mul(n, z));
        o.cosWo = z;
        o.pdf = z * INV_PI;
        if (o.cosWo < COS_EPS) return false;
        o.rev = cwi * INV_PI;
        o.f = b.kd;
        return true;
    }
    const V3 R = reflect(wi, n);
    const float g = ud > b.ksW ? 1.0f : b.expo;
    const V3 ax = ud > b.ksW ? n : R;
    const float ca = std::pow(r1, 1.0f / (g + 1.0f)), sa = std::sqrt(1.0f - sq(ca)), phi = TWO_PI * r0;
    V3 b1, b2;
    frame(ax, b1, b2);
    wo = add(add(mul(b1, sa * std::cos(phi)), mul(b2, sa * std::sin(phi))), mul(ax, ca));
    o.cosWo = dot(n, wo);
    if (o.cosWo < COS_EPS) return false;
    o.f = mk(0, 0, 0);
    o.pdf = o.rev = 0;
    if (b.ksW > 0) {
        const float w = std::pow(std::max(dot(R, wo), 0.0f), b.expo) * INV_TWO_PI;
        if (w > 1e-10f) {
            o.f = mul(b.ks, (b.expo + 2.0f) * w);
            o.pdf = b.ksW * (b.expo + 1.0f) * w;
        }
        o.rev = o.pdf;
    }
    if (b.ksW < 1) {
        o.f = add(o.f, mul(b.kd, INV_PI));
        o.pdf += (1.0f - b.ksW) * o.cosWo * INV_PI;
        o.rev += (1.0f - b.ksW) * cwi * INV_PI;
    }
    o.f = mul(o.f, o.cosWo);
    if (o.pdf < 1e-10f) return false;
    o.f = mul(o.f, 1.0f / o.pdf);
    return true;
}
static float roughness(const Bsdf &b, float ud) {
    if (b.type == DRMLT_BSDF_ROUGHDIELECTRIC) return b.alpha;
    return (b.type == DRMLT_BSDF_PHONG && ud < b.ksW) ? std::sqrt(2.0f / (2.0f + 4.0f * b.expo)) : 1.0f;
}
template <bool adj>
static float snc(V3 wi, const Isect &is, V3 wo) {
    const float cwi = dot(is.ns, wi), cwo = dot(is.ns, wo), wig = dot(is.ng, wi), wog = dot(is.ng, wo);
    if (wig * cwi <= 0 || wog * cwo <= 0) return 0;
    return adj ? std::fabs((wog * cwi) / (wig * cwo)) : 1.0f;
}
static const Bsdf &bsdf_of(const Scene &s, int tri) { return s.bsdfs[s.shapeBsdf[s.triShape[tri]]]; }
static int light_of(const Scene &s, int tri) { return s.shapeLight[s.triShape[tri]]; }

// ---------------------------------------------------------------- lights / camera
static void tri_sample(const Scene &s, int t, float r0, float r1, V3 &p, V3 &n) {
    const float a = std::sqrt(1.0f - r0), b1 = 1.0f - a, b2 = a * r1;
    p = add(add(s.p0[t], mul(s.e1[t], b1)), mul(s.e2[t], b2));
    n = norm(add(add(mul(s.n0[t], 1.0f - b1 - b2), mul(s.n1[t], b1)), mul(s.n2[t], b2)));
}
static void tri_param(const Scene &s, int t, V3 p, float &u0, float &u1) {
    const V3 e0 = sub(p, s.p0[t]);
    const float d11 = dot(s.e1[t], s.e1[t]), d12 = dot(s.e1[t], s.e2[t]), d22 = dot(s.e2[t], s.e2[t]);
    const float d01 = dot(e0, s.e1[t]), d02 = dot(e0, s.e2[t]), inv = 1.0f / (d11 * d22 - d12 * d12);
    const float b1 = (d22 * d01 - d12 * d02) * inv, b2 = (d11 * d02 - d12 * d01) * inv, a = 1.0f - b1;
    u0 = 1.0f - sq(a);
    u1 = b2 / a;
}
static int ltri(const Scene &s, int li, int prim) { return s.shapeFirst[s.lights[li].shape] + prim; }
static int pick_light(const Scene &s, float u, float &prob) {
    const int id = sample_discrete(s.lightCdf, u);
    prob = s.lightFunc[id] / (s.lightFuncInt * float(s.lights.size()));
    return id;
}
static float pick_prob(const Scene &s, int li) { return s.lights[li].w / s.lightWeightSum; }
// ---------------------------------------------------------------- environment light
static float tent(float u) { return u < 0.5f ? 1.0f - std::sqrt(2.0f * u) : std::sqrt(2.0f * (u - 0.5f)) - 1.0f; }
static V3 env_px(const Scene &s, int i) { return mk(s.envImg[3 * i], s.envImg[3 * i + 1], s.envImg[3 * i + 2]); }
// Image3::At: unwrapped y * width + x (the last pixel stands in past the end).
static V3 env_at(const Scene &s, int x, int y) { return env_px(s, std::min(y * s.envW + x, s.envW * s.envH - 1)); }
static V3 env_rep(const Scene &s, int x, int y) {
    const int yy = ((y % s.envH) + s.envH) % s.envH, xx = ((x % s.envW) + s.envW) % s.envW;
    return env_px(s, yy * s.envW + xx);
}
static float env_rw(const Scene &s, int row) { return s.envRowW[std::min(std::max(row, 0), s.envH - 1)]; }
static V3 rot3(const float *m, V3 v) {
    return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z, m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
// uToIndex (src/envlight.cpp:128-133): std::lower_bound over cdf[0..n].
static int env_index(const float *cdf, int n, float &u) {
    const int e = int(std::lower_bound(cdf, cdf + n + 1, u) - cdf);
    const int i = std::min(std::max(e - 1, 0), n - 1);
    u = (u - cdf[i]) / (cdf[i + 1] - cdf[i]);
    return i;
}
static void env_sample_dir(const Scene &s, float u0, float u1, V3 &dir, V3 &val, float &pdf) {
    const int row = env_index(s.envRows.data(), s.envH, u1);
    const int col = env_index(s.envCols.data() + row * (s.envW + 1), s.envW, u0);
    const float t0 = tent(u0), t1 = tent(u1);
    const float phi = (float(col) + t0 + 0.5f) * s.envPix[0], th = (float(row) + t1 + 0.5f) * s.envPix[1];
    const float sp = std::sin(phi), cp = std::cos(phi), st = std::sin(th), ct = std::cos(th);
    dir = rot3(s.envL2W, mk(sp * st, ct, -cp * st));
    const V3 v1 = add(mul(mul(env_at(s, col, row), 1.0f - t0), 1.0f - t1), mul(mul(env_at(s, col + 1, row), t0), 1.0f - t1));
    const V3 v2 = add(mul(mul(env_at(s, col, row + 1), 1.0f - t0), t1), mul(mul(env_at(s, col + 1, row + 1), t0), t1));
    val = add(v1, v2);
    pdf = (lum(v1) * env_rw(s, row) + lum(v2) * env_rw(s, row + 1)) * s.envNorm / std::max(std::fabs(st), 1e-7f);
}
static float env_pos_pdf(const Scene &s) { return INV_PI / sq(s.bsR); }
static void env_emission(const Scene &s, const Light &L, V3 dirToLight, V3 &E, float &dp, float &ep) {
    const V3 d = rot3(s.envW2L, dirToLight);
    const float ux = std::atan2(d.x, -d.z) * INV_TWO_PI * float(s.envW) - 0.5f;
    const float uy = std::acos(d.y) * INV_PI * float(s.envH) - 0.5f;
    const int col = int(std::floor(ux)), row = int(std::floor(uy));
    const float dx1 = ux - float(col), dy1 = uy - float(row);
    const V3 v1 = add(mul(mul(env_rep(s, col, row), 1.0f - dx1), 1.0f - dy1), mul(mul(env_rep(s, col + 1, row), dx1), 1.0f - dy1));
    const V3 v2 = add(mul(mul(env_rep(s, col, row + 1), 1.0f - dx1), dy1), mul(mul(env_rep(s, col + 1, row + 1), dx1), dy1));
    E = mul(add(v1, v2), L.w);
    const float st = std::sqrt(1.0f - sq(d.y));
    dp = (lum(v1) * env_rw(s, row) + lum(v2) * env_rw(s, row + 1)) * s.envNorm / std::max(std::fabs(st), 1e-7f);
    ep = dp * env_pos_pdf(s);
}

static bool sample_direct(const Scene &s, int li, int prim, V3 pos, float r0, float r1, V3 &dir, float &dist, V3 &c,
                          float &cosL, float &dpdf, float &epdf) {
    const Light &L = s.lights[li];
    if (L.type == DRMLT_LIGHT_ENV) {
        V3 val;
        env_sample_dir(s, r0, r1, dir, val, dpdf);
        dist = INFINITY;
        c = mul(mul(val, 1.0f / dpdf), L.w);
        cosL = 1.0f;
        epdf = dpdf * env_pos_pdf(s);
        return true;
    }
    if (L.type == DRMLT_LIGHT_AREA) {
        V3 p, n;
        tri_sample(s, ltri(s, li, prim), r0, r1, p, n);
        dir = sub(p, pos);
        const float d2 = lensq(dir);
        dist = std::sqrt(d2);
        dir = mk(dir.x / dist, dir.y / dist, dir.z / dist);
        cosL = -dot(dir, n);
        if (!(cosL > COS_EPS)) return false;
        c = mul(L.E, cosL / (d2 * L.invArea));
        dpdf = L.invArea * d2 / cosL;
        epdf = L.invArea * cosL * INV_PI;
        return true;
    }
    dir = sub(L.pos, pos);
    const float d2 = lensq(dir);
    dist = std::sqrt(d2);
    dir = mk(dir.x / dist, dir.y / dist, dir.z / dist);
    c = mul(L.E, 1.0f / d2);
    dpdf = d2;
    epdf = 1.0f / (4.0f * PI);
    cosL = 1.0f;
    return true;
}
static void xpoint(const float *m, V3 p, V3 &o) {
    const float x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3], y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    const float z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11], w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    const float iw = 1.0f / w;
    o = mk(x * iw, y * iw, z * iw);
}
static V3 xvec(const float *m, V3 v) {
    return mk(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z, m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
static void primary(const Scene &s, float sx, float sy, V3 &org, V3 &dir, float &t0, float &t1) {
    V3 o;
    xpoint(s.s2c, mk(sx, sy, 0), o);
    const V3 d = norm(o);
    const float iz = 1.0f / d.z;
    xpoint(s.c2w, mk(0, 0, 0), org);
    dir = xvec(s.c2w, d);
    t0 = s.nearc * iz;
    t1 = s.farc * iz;
}
static bool project(const Scene &s, V3 p, float &sx, float &sy) {
    V3 c, r;
    xpoint(s.w2c, p, c);
    if (c.z < s.nearc || c.z > s.farc) return false;
    xpoint(s.c2s, c, r);
    if (r.x < 0 || r.x > 1 || r.y < 0 || r.y > 1) return false;
    sx = r.x;
    sy = r.y;
    return true;
}

// ---------------------------------------------------------------- bidirectional path (primal)
struct St {
    Isect is;
    V3 wi, T;
    float prev, cur, ssJ, lcJ, lastPdf;
};
static void zst(St &a) { std::memset(&a, 0, sizeof(St)); }
struct Vx {
    int tri, useAbs, dlL, dlP;
    float rnd[2], disc, rr, dl[2];
};
static void zvx(Vx &v) {
    std::memset(&v, 0, sizeof(Vx));
    v.tri = v.dlL = v.dlP = -1;
}
struct Em {
    int c, l;
    float sx, sy, ls, ss;
    V3 rgb;
};
static bool fin(Em &e, int c, int l, float sx, float sy, V3 rgb, float ssJ) {
    const float score = lum(rgb);
    if (!(score > 0)) return false;
    e.c = c; e.l = l; e.sx = sx; e.sy = sy; e.rgb = rgb; e.ls = score; e.ss = score * ssJ;
    return true;
}
static void emit_cam(const Scene &s, float sx, float sy, V3 &o, V3 &d, float &t0, float &t1, St &ps) {
    V3 co, cd;
    float a, b;
    primary(s, 0.5f, 0.5f, co, cd, a, b);
    primary(s, sx, sy, o, d, t0, t1);
    const float cc = dot(cd, d), ip = s.dist / cc, pdfW = sq(ip) / cc;
    ps.T = mk(1, 1, 1);
    ps.prev = mis(float(s.W * s.H) / pdfW);
    ps.cur = 0;
    ps.ssJ = 1;
}
static void emit_light(const Scene &s, float pick, int li, int prim, const float pp[2], const float dp[2], V3 &o, V3 &d,
                       St &ps) {
    const Light &L = s.lights[li];
    float cosL, ep, dpd;
    if (L.type == DRMLT_LIGHT_AREA) {
        V3 n;
        tri_sample(s, ltri(s, li, prim), pp[0], pp[1], o, n);
        const float phi = TWO_PI * dp[0], tmp = std::sqrt(std::max(1.0f - dp[1], 0.0f)), z = std::sqrt(std::max(dp[1], 0.0f));
        V3 b1, b2;
        frame(n, b1, b2);
        d = add(add(mul(b1, std::cos(phi) * tmp), mul(b2, std::sin(phi) * tmp)), mul(n, z));
        ps.T = mul(L.E, PI / L.invArea);
        cosL = z;
        ep = z * INV_PI * L.invArea;
        dpd = L.invArea;
    } else if (L.type == DRMLT_LIGHT_ENV) {
        V3 val;
        env_sample_dir(s, dp[0], dp[1], d, val, dpd);
        ps.T = mul(val, L.w);
        d = neg(d);
        // SampleConcentricDisc (src/sampling.h:48-67)
        const float r1 = 2.0f * pp[0] - 1.0f, r2 = 2.0f * pp[1] - 1.0f;
        float r = 0.0f, phi = 0.0f;
        if (r1 != 0.0f && r2 != 0.0f) {
            if (sq(r1) > sq(r2)) { r = r1; phi = (0.25f * PI) * (r2 / r1); }
            else { r = r2; phi = 0.5f * PI - (r1 / r2) * (0.25f * PI); }
        }
        V3 b1, b2;
        frame(d, b1, b2);
        const V3 perp = add(mul(b1, r * std::cos(phi)), mul(b2, r * std::sin(phi)));
        o = add(s.bsC, mul(sub(perp, d), s.bsR));
        cosL = 1.0f;
        ep = dpd * env_pos_pdf(s);
    } else {
        o = L.pos;
        const float th = TWO_PI * dp[0], ph = PI * dp[1];
        d = mk(std::sin(ph) * std::cos(th), std::sin(ph) * std::sin(th), std::cos(ph));
        ps.T = L.E;
        ep = 1.0f / (4.0f * PI);
        cosL = dpd = 1.0f;
    }
    ep *= pick;
    dpd *= pick;
    ps.T = mul(ps.T, 1.0f / pick);
    ps.prev = mis(dpd / ep);
    ps.cur = L.type != DRMLT_LIGHT_POINT ? mis(cosL / ep) : 0.0f;
    ps.ssJ = 1;
}
static void conv_mis(const Scene &s, int depth, int li, V3 o, V3 d, St &ps) {
    if (depth > 0 || li < 0 || s.lights[li].type == DRMLT_LIGHT_AREA) ps.prev *= mis(lensq(sub(o, ps.is.p)));
    const float ic = 1.0f / mis(std::fabs(dot(d, ps.is.ns)));
    ps.prev *= ic;
    ps.cur *= ic;
}
static bool to_camera(const Scene &s, int ld, const St &ps, const Vx &v, Em &e) {
    V3 co, cd;
    float a, b;
    primary(s, 0.5f, 0.5f, co, cd, a, b);
    V3 dc = sub(co, ps.is.p);
    if (-dot(cd, dc) <= 0) return false;
    float sx, sy;
    if (!project(s, ps.is.p, sx, sy)) return false;
    const float d2 = lensq(dc), dist = std::sqrt(d2);
    dc = mul(dc, 1.0f / dist);
    if (occluded(s, ps.is.p, dc, dist)) return false;
    BOut bo;
    bsdf_eval(bsdf_of(s, v.tri), ps.wi, ps.is.ns, dc, bo, true);
    if (iszero(bo.f)) return false;
    const float f = snc<true>(ps.wi, ps.is, dc);
    if (f <= 0) return false;
    const V3 bc = mul(bo.f, f);
    const float cc = -dot(cd, dc), ip = s.dist / cc, i2s = sq(ip) / cc, i2surf = i2s * std::fabs(bo.cosWo) / d2;
    const float pix = float(s.W * s.H);
    const float wL = mis(i2surf / pix) * (ps.prev + ps.cur * mis(bo.rev)), mw = 1.0f / (wL + 1.0f);
    const float den = pix * (bo.cosWo / i2surf);
    const V3 c = cmul(mk((mw * bc.x) / den, (mw * bc.y) / den, (mw * bc.z) / den), ps.T);
    return fin(e, 1, 2 + ld, sx, sy, c, ps.ssJ);
}
template <bool adj, bool perturb>
static bool bsdf_sampling(const Scene &s, const St &ps, Vx &v, St &nx, bool fresh, V3 &dir, V3 &bc) {
    const Bsdf &b = bsdf_of(s, v.tri);
    v.useAbs = roughness(b, v.disc) > s.opt.roughness_threshold;
    BOut bo;
    float ssJ, lcJ;
    if (!perturb || !v.useAbs) {
        if (!bsdf_sample(b, ps.wi, ps.is.ns, v.rnd[0], v.rnd[1], v.disc, dir, bo, adj)) return false;
        if (v.useAbs) {
            float th = 0.0f;
            if (!(dir.y == 0 && dir.x == 0)) {
                th = std::atan2(dir.y, dir.x);
                if (th < 0) th += float(2.0 * M_PI);
            }
            th *= INV_TWO_PI;
            float ph = std::acos(dir.z);
            float jac = std::fabs(std::sin(ph));
            ph *= INV_PI;
            v.rnd[0] = th;
            v.rnd[1] = ph;
            lcJ = 1.0f / jac;
            jac *= bo.pdf;
            ssJ = ps.ssJ * jac;
        } else {
            lcJ = bo.pdf;
            ssJ = fresh ? 0.0f : ps.ssJ;
        }
    } else {
        const float th = TWO_PI * v.rnd[0], ph = PI * v.rnd[1], sp = std::sin(ph);
        float jac = std::fabs(sp);
        dir = mk(sp * std::cos(th), sp * std::sin(th), std::cos(ph));
        bsdf_eval(b, ps.wi, ps.is.ns, dir, bo, adj);
        if (iszero(bo.f) || bo.pdf <= 0) return false;
        bo.f = mul(bo.f, 1.0f / bo.pdf);
        lcJ = 1.0f / jac;
        jac *= bo.pdf;
        ssJ = ps.ssJ * jac;
    }
    const float f = snc<adj>(ps.wi, ps.is, dir);
    if (f <= 0) return false;
    bc = mul(bo.f, f);
    const float cur = mis(bo.cosWo / bo.pdf) * (ps.cur * mis(bo.rev) + ps.prev);
    const V3 T = cmul(ps.T, bc);
    nx.lcJ = lcJ; nx.ssJ = ssJ; nx.lastPdf = bo.pdf; nx.cur = cur; nx.prev = mis(1.0f / bo.pdf); nx.T = T;
    return true;
}
static bool direct(const Scene &s, int cd, const St &ps, float sx, float sy, float pick, const Vx &v, Em &e) {
    V3 dir, lc;
    float dist, cosL, dp, ep;
    if (!sample_direct(s, v.dlL, v.dlP, ps.is.p, v.dl[0], v.dl[1], dir, dist, lc, cosL, dp, ep)) return false;
    if (occluded(s, ps.is.p, dir, dist)) return false;
    BOut bo;
    bsdf_eval(bsdf_of(s, v.tri), ps.wi, ps.is.ns, dir, bo);
    if (iszero(bo.f)) return false;
    const float f = snc<false>(ps.wi, ps.is, dir);
    if (f <= 0) return false;
    V3 c = cmul(ps.T, mul(bo.f, f));
    c = mul(cmul(c, lc), 1.0f / pick);
    const float wL = s.lights[v.dlL].type == DRMLT_LIGHT_POINT ? 0.0f : mis(bo.pdf / (pick * dp));
    const float wC = mis(ep * bo.cosWo / (dp * cosL)) * (ps.prev + ps.cur * mis(bo.rev));
    c = mul(c, 1.0f / (wL + 1.0f + wC));
    return fin(e, 2 + cd, 1, sx, sy, c, ps.ssJ);
}
static bool hit_light(const Scene &s, int cd, int li, V3 d, float sx, float sy, const St &ps, Em &e) {
    const Light &L = s.lights[li];
    float dp, ep;
    V3 E;
    if (L.type == DRMLT_LIGHT_ENV) {
        env_emission(s, L, d, E, dp, ep);
        if (!(E.x + E.y + E.z > 0)) return false;
    } else {
        const float cosL = -dot(ps.is.ns, d);
        if (!(L.type == DRMLT_LIGHT_AREA && cosL > 0)) return false;
        dp = L.invArea;
        ep = cosL * dp * INV_PI;
        E = L.E;
    }
    V3 c = cmul(ps.T, E);
    if (cd > 0) {
        const float pk = pick_prob(s, li);
        dp *= pk;
        ep *= pk;
        c = mul(c, 1.0f / (1.0f + mis(dp) * ps.prev + mis(ep) * ps.cur));
    }
    return fin(e, 2 + cd, 0, sx, sy, c, ps.ssJ);
}
static bool connect(const Scene &s, int cd, int ld, const St &lp, const Vx &lv, const St &cp, const Vx &cv, float sx,
                    float sy, Em &e) {
    V3 d = sub(lp.is.p, cp.is.p);
    const float d2 = lensq(d), dist = std::sqrt(d2);
    d = mul(d, 1.0f / dist);
    if (occluded(s, cp.is.p, d, dist)) return false;
    BOut cb, lb;
    bsdf_eval(bsdf_of(s, cv.tri), cp.wi, cp.is.ns, d, cb);
    if (iszero(cb.f)) return false;
    const float cf = snc<false>(cp.wi, cp.is, d);
    if (cf <= 0) return false;
    bsdf_eval(bsdf_of(s, lv.tri), lp.wi, lp.is.ns, neg(d), lb, true);
    if (iszero(lb.f)) return false;
    const float lf = snc<true>(lp.wi, lp.is, neg(d));
    if (lf <= 0) return false;
    const float G = 1.0f / d2;
    const float wL = mis(cb.pdf * lb.cosWo * G) * (lp.prev + lp.cur * mis(lb.rev));
    const float wC = mis(lb.pdf * cb.cosWo * G) * (cp.prev + cp.cur * mis(cb.rev));
    V3 c = cmul(cmul(lp.T, cp.T), mul(cb.f, cf));
    c = mul(cmul(c, mul(lb.f, lf)), G);
    c = mul(c, 1.0f / (wL + 1.0f + wC));
    return fin(e, 2 + cd, 2 + ld, sx, sy, c, lp.ssJ * cp.ssJ);
}
static bool lcs(const Scene &s, const Vx &cur, int ntri, St &ps, V3 &dir) {
    V3 np, nn;
    tri_sample(s, ntri, cur.rnd[0], cur.rnd[1], np, nn);
    dir = sub(np, ps.is.p);
    const float d2 = lensq(dir), dist = std::sqrt(d2);
    dir = mul(dir, 1.0f / dist);
    if (occluded(s, ps.is.p, dir, dist)) return false;
    BOut bo;
    bsdf_eval(bsdf_of(s, cur.tri), ps.wi, ps.is.ns, dir, bo);
    if (iszero(bo.f)) return false;
    ps.T = cmul(ps.T, mul(bo.f, 1.0f / bo.pdf));
    ps.ssJ *= std::fabs(dot(dir, nn) * (1.0f / d2)) * bo.pdf;
    ps.cur = mis(bo.cosWo / bo.pdf) * (ps.cur * mis(bo.rev) + ps.prev);
    ps.prev = mis(1.0f / bo.pdf);
    return true;
}
template <class R>
static bool rr(int depth, V3 bc, float &w, V3 &T, R &rng) {
    float p = 1.0f;
    if (depth >= 3) p = std::min(maxc(bc), 0.95f);
    if (rng.uni() > p) return false;
    w = 1.0f / p;
    T = mul(T, w);
    return true;
}
static void lc_convert(const Scene &s, Vx &prev, int ltriI, V3 o, St &ps) {
    tri_param(s, ltriI, ps.is.p, prev.rnd[0], prev.rnd[1]);
    V3 d = sub(ps.is.p, o);
    const float d2 = lensq(d), id2 = 1.0f / d2, idist = std::sqrt(id2);
    d = mul(d, idist);
    ps.ssJ *= std::fabs(dot(d, ps.is.ns) * id2) * (ps.lcJ * s.lights[light_of(s, ltriI)].invArea);
}

struct Full {
    float pos[2], dir[2], screen[2];
    int lL, lP, nl, nc;
    Vx lg[MAXF], cm[MAXF];
};
static void make_rec(const Full &f, int c, int l, drmlt_path &r) {
    std::memset(&r, 0, sizeof(r));
    r.c = c; r.l = l; r.lgt_light = f.lL; r.lgt_prim = f.lP;
    const int nl = l > 1 ? l - 1 : 0, nc = c - 1;
    r.dl_light = nc > 0 ? f.cm[nc - 1].dlL : -1;
    r.dl_prim = nc > 0 ? f.cm[nc - 1].dlP : -1;
    int k = 0;
    if (l > 1) {
        r.u[k++] = f.pos[0]; r.u[k++] = f.pos[1]; r.u[k++] = f.dir[0]; r.u[k++] = f.dir[1];
        for (int i = 0; i < nl - 1; i++) { r.u[k++] = f.lg[i].rnd[0]; r.u[k++] = f.lg[i].rnd[1]; }
    }
    if (c > 1) {
        r.u[k++] = f.screen[0]; r.u[k++] = f.screen[1];
        for (int i = 0; i < nc - 1; i++) { r.u[k++] = f.cm[i].rnd[0]; r.u[k++] = f.cm[i].rnd[1]; }
        if (l == 1) { r.u[k++] = f.cm[nc - 1].dl[0]; r.u[k++] = f.cm[nc - 1].dl[1]; }
    }
    for (int i = 0; i < nl; i++) {
        r.tri[i] = f.lg[i].tri; r.disc[i] = f.lg[i].disc; r.rr[i] = f.lg[i].rr;
        if (f.lg[i].useAbs) r.use_abs |= 1u << i;
    }
    for (int i = 0; i < nc; i++) {
        r.tri[nl + i] = f.cm[i].tri; r.disc[nl + i] = f.cm[i].disc; r.rr[nl + i] = f.cm[i].rr;
        if (f.cm[i].useAbs) r.use_abs |= 1u << (nl + i);
    }
}
static int light_prim(const Scene &s, int li, float u) {
    return s.lights[li].type == DRMLT_LIGHT_AREA ? sample_discrete(s.lights[li].triCdf, u) : 0;
}

// GeneratePathBidir (src/path.cpp:978-1121).
template <class R, class Sink>
static void gen_bidir(const Scene &s, int minD, int maxD, R &rng, Full &f, Sink &sink) {
    St lp[MAXF];
    rng.uni();  // time
    f.pos[1] = rng.uni(); f.pos[0] = rng.uni(); f.dir[1] = rng.uni(); f.dir[0] = rng.uni();
    float pick;
    f.lL = pick_light(s, rng.uni(), pick);
    f.lP = s.lights[f.lL].type == DRMLT_LIGHT_AREA ? light_prim(s, f.lL, rng.uni()) : (rng.uni(), -1);
    V3 o, d;
    zst(lp[0]);
    emit_light(s, pick, f.lL, f.lP, f.pos, f.dir, o, d, lp[0]);
    f.nl = 0;
    int ns = 1;
    for (int k = 0; k < MAXF - 1; k++) {
        Vx &v = f.lg[k];
        zvx(v);
        f.nl = k + 1;
        int tri = -1;
        const bool hit = intersect(s, o, d, ISECT_EPS, INFINITY, tri, lp[k].is);
        v.tri = tri;
        if (!hit) { ns--; f.nl--; break; }
        v.disc = rng.uni();
        lp[k].wi = neg(d);
        conv_mis(s, k, f.lL, o, d, lp[k]);
        if (k + 2 >= minD) { Em e; if (to_camera(s, k, lp[k], v, e)) sink(e); }
        if (maxD != -1 && k + 2 >= maxD) break;
        zst(lp[k + 1]);
        ns++;
        v.rnd[1] = rng.uni(); v.rnd[0] = rng.uni();
        V3 bc;
        if (!bsdf_sampling<true, false>(s, lp[k], v, lp[k + 1], true, d, bc)) { ns--; break; }
        if (!rr(k, bc, v.rr, lp[k + 1].T, rng)) { ns--; break; }
        o = lp[k].is.p;
    }
    f.screen[1] = rng.uni(); f.screen[0] = rng.uni();
    St cp;
    zst(cp);
    float t0, t1;
    emit_cam(s, f.screen[0], f.screen[1], o, d, t0, t1, cp);
    f.nc = 0;
    for (int k = 0; k < MAXF; k++) {
        Vx &v = f.cm[k];
        zvx(v);
        f.nc = k + 1;
        int tri = -1;
        const bool hit = intersect(s, o, d, t0, t1, tri, cp.is);
        v.tri = tri;
        cp.wi = neg(d);
        if (hit) conv_mis(s, k, -1, o, d, cp);
        if (k + 1 >= minD) {
            const int li = hit ? light_of(s, tri) : s.envL;
            if (li >= 0) {
                if (!hit) v.tri = -1;
                if (s.opt.use_light_coordinate_sampling && k > 1 && s.lights[li].type == DRMLT_LIGHT_AREA)
                    lc_convert(s, f.cm[k - 1], tri, o, cp);
                Em e;
                if (hit_light(s, k, li, d, f.screen[0], f.screen[1], cp, e)) sink(e);
                return;
            }
        }
        if (!hit || (maxD != -1 && k + 1 >= maxD)) break;
        v.disc = rng.uni();
        if (k + 2 >= minD) {
            float dpk;
            v.dlL = pick_light(s, rng.uni(), dpk);
            v.dl[1] = rng.uni(); v.dl[0] = rng.uni();
            v.dlP = light_prim(s, v.dlL, rng.uni());
            Em e;
            if (direct(s, k, cp, f.screen[0], f.screen[1], dpk, v, e)) sink(e);
        }
        const int mld = maxD == -1 ? ns - 1 : std::min(maxD - k - 3, ns - 1);
        for (int ld = 0; ld <= mld; ld++)
            if (k + ld + 3 >= minD) { Em e; if (connect(s, k, ld, lp[ld], f.lg[ld], cp, v, f.screen[0], f.screen[1], e)) sink(e); }
        v.rnd[1] = rng.uni(); v.rnd[0] = rng.uni();
        V3 bc;
        if (!bsdf_sampling<false, false>(s, cp, v, cp, false, d, bc)) break;
        if (!rr(k, bc, v.rr, cp.T, rng)) break;
        o = cp.is.p;
        t0 = ISECT_EPS;
        t1 = INFINITY;
    }
}

// GenerateSubpath (src/path.cpp:1123-1269), bidirMIS = true.
template <class R>
static bool gen_subpath(const Scene &s, int camL, int lgtL, R &rng, drmlt_path &rec, Em &e) {
    Full f;
    std::memset(&f, 0, sizeof(f));
    rng.uni();
    St lp;
    zst(lp);
    f.lL = f.lP = -1;
    V3 o, d;
    if (lgtL > 1) {
        f.pos[1] = rng.uni(); f.pos[0] = rng.uni(); f.dir[1] = rng.uni(); f.dir[0] = rng.uni();
        float pick;
        f.lL = pick_light(s, rng.uni(), pick);
        f.lP = s.lights[f.lL].type == DRMLT_LIGHT_AREA ? light_prim(s, f.lL, rng.uni()) : (rng.uni(), -1);
        emit_light(s, pick, f.lL, f.lP, f.pos, f.dir, o, d, lp);
        for (int k = 0; k < MAXF; k++) {
            Vx &v = f.lg[k];
            zvx(v);
            f.nl = k + 1;
            int tri = -1;
            const bool hit = intersect(s, o, d, ISECT_EPS, INFINITY, tri, lp.is);
            v.tri = tri;
            if (!hit) return false;
            v.disc = rng.uni();
            lp.wi = neg(d);
            conv_mis(s, k, f.lL, o, d, lp);
            if (k + 2 == lgtL) {
                if (camL == 1) {
                    if (!to_camera(s, k, lp, v, e)) return false;
                    make_rec(f, 1, lgtL, rec);
                    return true;
                }
                break;
            }
            v.rnd[1] = rng.uni(); v.rnd[0] = rng.uni();
            V3 bc;
            if (!bsdf_sampling<true, false>(s, lp, v, lp, false, d, bc)) return false;
            v.rr = 1.0f;
            o = lp.is.p;
        }
    }
    f.screen[1] = rng.uni(); f.screen[0] = rng.uni();
    St cp;
    zst(cp);
    float t0, t1;
    emit_cam(s, f.screen[0], f.screen[1], o, d, t0, t1, cp);
    for (int k = 0; k < MAXF; k++) {
        Vx &v = f.cm[k];
        zvx(v);
        f.nc = k + 1;
        int tri = -1;
        const bool hit = intersect(s, o, d, t0, t1, tri, cp.is);
        v.tri = tri;
        cp.wi = neg(d);
        if (hit) conv_mis(s, k, -1, o, d, cp);
        if (k + 2 >= camL && lgtL == 0) {
            const int li = hit ? light_of(s, tri) : s.envL;
            if (li < 0) return false;
            if (!hit) v.tri = -1;
            if (k > 1 && s.lights[li].type == DRMLT_LIGHT_AREA) lc_convert(s, f.cm[k - 1], tri, o, cp);
            if (!hit_light(s, k, li, d, f.screen[0], f.screen[1], cp, e)) return false;
            make_rec(f, camL, 0, rec);
            return true;
        }
        if (!hit) return false;
        v.disc = rng.uni();
        if (k + 2 == camL) {
            bool ok;
            if (lgtL == 1) {
                float dpk;
                v.dlL = pick_light(s, rng.uni(), dpk);
                v.dl[1] = rng.uni(); v.dl[0] = rng.uni();
                v.dlP = light_prim(s, v.dlL, rng.uni());
                ok = direct(s, k, cp, f.screen[0], f.screen[1], dpk, v, e);
            } else {
                ok = connect(s, k, lgtL - 2, lp, f.lg[f.nl - 1], cp, v, f.screen[0], f.screen[1], e);
            }
            if (!ok) return false;
            make_rec(f, camL, lgtL, rec);
            return true;
        }
        v.rnd[1] = rng.uni(); v.rnd[0] = rng.uni();
        V3 bc;
        if (!bsdf_sampling<false, false>(s, cp, v, cp, false, d, bc)) return false;
        v.rr = 1.0f;
        o = cp.is.p;
        t0 = ISECT_EPS;
        t1 = INFINITY;
    }
    return false;
}

// PerturbPathBidir (src/path.cpp:1480-1628); jitter(): N(0, discreteStdDev) draw or 0.
template <class J>
static bool perturb(const Scene &s, const drmlt_path &in, const float *off, J &jit, drmlt_path &out, Em &e) {
    out = in;
    const int c = in.c, l = in.l, nl = l > 1 ? l - 1 : 0, nc = c - 1;
    int k = 0;
    St lp;
    zst(lp);
    Vx last;
    zvx(last);
    if (l > 1) {
        for (int i = 0; i < 4; i++, k++) out.u[k] = modulo1(in.u[k] + off[k]);
        const float pp[2] = {out.u[0], out.u[1]}, dp[2] = {out.u[2], out.u[3]};
        V3 o, d;
        emit_light(s, pick_prob(s, in.lgt_light), in.lgt_light, in.lgt_prim, pp, dp, o, d, lp);
        for (int q = 0; q < nl; q++) {
            Vx v;
            zvx(v);
            int tri = out.tri[q];
            const bool hit = intersect(s, o, d, ISECT_EPS, INFINITY, tri, lp.is);
            out.tri[q] = v.tri = tri;
            if (!hit) return false;
            lp.wi = neg(d);
            out.disc[q] = modulo1(out.disc[q] + jit.jitter());
            v.disc = out.disc[q];
            conv_mis(s, q, in.lgt_light, o, d, lp);
            if (q == nl - 1 && c == 1) return to_camera(s, q, lp, v, e);
            if (q == nl - 1) { last = v; break; }
            out.u[k] = modulo1(in.u[k] + off[k]);
            out.u[k + 1] = modulo1(in.u[k + 1] + off[k + 1]);
            v.rnd[0] = out.u[k]; v.rnd[1] = out.u[k + 1];
            k += 2;
            V3 bc;
            const bool ok = bsdf_sampling<true, true>(s, lp, v, lp, false, d, bc);
            if (v.useAbs) out.use_abs |= 1u << q; else out.use_abs &= ~(1u << q);
            if (!ok) return false;
            lp.T = mul(lp.T, out.rr[q]);
            o = lp.is.p;
        }
    }
    out.u[k] = modulo1(in.u[k] + off[k]);
    out.u[k + 1] = modulo1(in.u[k + 1] + off[k + 1]);
    const float sx = out.u[k], sy = out.u[k + 1];
    k += 2;
    V3 o, d;
    float t0, t1;
    St cp;
    zst(cp);
    emit_cam(s, sx, sy, o, d, t0, t1, cp);
    bool lcoord = false;
    for (int q = 0; q < nc; q++) {
        const int vi = nl + q;
        Vx v;
        zvx(v);
        int tri = out.tri[vi];
        const bool hit = intersect(s, o, d, t0, t1, tri, cp.is);
        out.tri[vi] = v.tri = tri;
        cp.wi = neg(d);
        if (hit) conv_mis(s, q, -1, o, d, cp);
        if (q == nc - 1 && l == 0) {
            const int li = hit ? light_of(s, tri) : s.envL;
            if (!hit) out.tri[vi] = -1;  // the path ends on the environment light
            return li >= 0 && hit_light(s, q, li, d, sx, sy, cp, e);
        }
        if (!hit) return false;
        out.disc[vi] = modulo1(out.disc[vi] + jit.jitter());
        v.disc = out.disc[vi];
        if (q == nc - 1) {
            if (l == 1) {
                out.u[k] = modulo1(in.u[k] + off[k]);
                out.u[k + 1] = modulo1(in.u[k + 1] + off[k + 1]);
                v.dlL = in.dl_light; v.dlP = in.dl_prim; v.dl[0] = out.u[k]; v.dl[1] = out.u[k + 1];
                return direct(s, q, cp, sx, sy, pick_prob(s, in.dl_light), v, e);
            }
            return connect(s, q, nl - 1, lp, last, cp, v, sx, sy, e);
        }
        out.u[k] = modulo1(in.u[k] + off[k]);
        out.u[k + 1] = modulo1(in.u[k + 1] + off[k + 1]);
        v.rnd[0] = out.u[k]; v.rnd[1] = out.u[k + 1];
        k += 2;
        if (s.opt.use_light_coordinate_sampling && q == nc - 2 && l == 0) {
            const int lt = in.tri[nl + nc - 1];
            if (lt >= 0 && light_of(s, lt) >= 0) lcoord = true;
        }
        V3 bc;
        if (lcoord) {
            if (!lcs(s, v, in.tri[nl + nc - 1], cp, d)) return false;
        } else {
            const bool ok = bsdf_sampling<false, true>(s, cp, v, cp, false, d, bc);
            if (v.useAbs) out.use_abs |= 1u << vi; else out.use_abs &= ~(1u << vi);
            if (!ok) return false;
        }
        cp.T = mul(cp.T, out.rr[vi]);
        o = cp.is.p;
        t0 = ISECT_EPS;
        t1 = INFINITY;
    }
    return false;
}

// GeneratePath, direct-lighting pass (src/path.cpp:343-445 via src/integrator.h:33-75).
template <class R, class Sink>
static void gen_direct(const Scene &s, int px, int py, int minD, int maxD, R &rng, Sink &sink) {
    rng.uni();
    const float sy = (float(py) + rng.uni()) / float(s.H);
    const float sx = (float(px) + rng.uni()) / float(s.W);
    V3 o, d;
    float t0, t1;
    primary(s, sx, sy, o, d, t0, t1);
    V3 T = mk(1, 1, 1);
    float lastPdf = 1.0f;
    for (int k = 0; k < 8; k++) {
        Isect is;
        int tri = -1;
        const bool hit = intersect(s, o, d, t0, t1, tri, is);
        const int li = hit ? light_of(s, tri) : s.envL;
        if (li >= 0 && k + 1 >= minD) {
            const Light &L = s.lights[li];
            const float cosL = hit ? -dot(is.ns, d) : 0.0f;
            if (L.type == DRMLT_LIGHT_ENV) {
                V3 E;
                float dp, ep;
                env_emission(s, L, d, E, dp, ep);
                if (E.x + E.y + E.z > 0) {
                    V3 c = cmul(T, E);
                    if (k > 0) c = mul(c, 1.0f / (1.0f + sq((dp * pick_prob(s, li)) / lastPdf)));
                    Em e;
                    if (fin(e, 2 + k, 0, sx, sy, c, 1.0f)) sink(e);
                }
            } else if (L.type == DRMLT_LIGHT_AREA && cosL > 0) {
                float dp = L.invArea * (lensq(sub(o, is.p)) / (-dot(d, is.ns)));
                V3 c = cmul(T, L.E);
                if (k > 0) c = mul(c, 1.0f / (1.0f + sq((dp * pick_prob(s, li)) / lastPdf)));
                Em e;
                if (fin(e, 2 + k, 0, sx, sy, c, 1.0f)) sink(e);
            }
            return;
        }
        if (!hit || (maxD != -1 && k + 1 >= maxD)) break;
        const float disc = rng.uni();
        const V3 wi = neg(d);
        const Bsdf &b = bsdf_of(s, tri);
        if (k + 2 >= minD) {
            float pk;
            const int dl = pick_light(s, rng.uni(), pk);
            const float r1 = rng.uni(), r0 = rng.uni();
            const int dlP = light_prim(s, dl, rng.uni());
            V3 dir, lc;
            float dist, cosL, dp, ep;
            if (sample_direct(s, dl, dlP, is.p, r0, r1, dir, dist, lc, cosL, dp, ep) && !occluded(s, is.p, dir, dist)) {
                BOut bo;
                bsdf_eval(b, wi, is.ns, dir, bo);
                if (!iszero(bo.f)) {
                    V3 c = mul(cmul(cmul(T, bo.f), lc), 1.0f / pk);
                    if (s.lights[dl].type != DRMLT_LIGHT_POINT) c = mul(c, 1.0f / (1.0f + sq(bo.pdf / (dp * pk))));
                    Em e;
                    if (fin(e, 2 + k, 1, sx, sy, c, 1.0f)) sink(e);
                }
            }
        }
        const float r1 = rng.uni(), r0 = rng.uni();
        BOut bo;
        V3 wo;
        if (!bsdf_sample(b, wi, is.ns, r0, r1, disc, wo, bo)) break;
        lastPdf = bo.pdf;
        T = cmul(T, bo.f);
        float w;
        if (!rr(k, bo.f, w, T, rng)) break;
        o = is.p;
        d = wo;
        t0 = ISECT_EPS;
        t1 = INFINITY;
    }
}

}  // namespace ora

#include "oracle_ad.inc"
#include "oracle_dr.inc"
