// Shared device math, scene layout and random-number sources for the DRMLT
// chain kernels. Float constants and vector helpers follow the reference's
// definitions (src/commondef.h:54-86, src/utils.h:126-232) so that values
// computed here round the same way as the reference's single-precision build.
#pragma once
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>

#define DEV __device__ __forceinline__
// Called from many sites of the large per-chain kernels: kept out of line so
// that one copy of the code serves every call site (instruction-cache footprint).
#define DEV_SHARED static __device__ __noinline__
#define HD __host__ __device__ __forceinline__

namespace drmlt {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 1.0f / kPi;
constexpr float kTwoPi = 2.0f * kPi;
constexpr float kInvTwoPi = 1.0f / kTwoPi;
constexpr float kPiOverTwo = 0.5f * kPi;
constexpr float kPiOverFour = 0.25f * kPi;
constexpr float kIsectEps = 1e-3f;   // c_IsectEpsilon (single precision)
constexpr float kShadowEps = 1e-3f;  // c_ShadowEpsilon
constexpr float kCosEps = 1e-4f;     // c_CosEpsilon

constexpr int kMaxLen = 12;          // longest path (segments) a chain may hold
constexpr int kMaxVerts = kMaxLen;   // surface vertices stored per path
constexpr int kMaxDim = 2 * kMaxLen; // primary-sample dimension 2L
constexpr int kMaxFull = kMaxLen + 2;// vertices kept per subpath by the bootstrap sampler

// ---------------------------------------------------------------- vectors
template <class T>
struct Vec3 {
    T x, y, z;
    HD Vec3() {}
    HD Vec3(T a, T b, T c) : x(a), y(b), z(c) {}
    HD T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
using V3 = Vec3<float>;

template <class T> HD Vec3<T> operator+(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class T> HD Vec3<T> operator-(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class T> HD Vec3<T> operator-(const Vec3<T> &a) { return Vec3<T>(-a.x, -a.y, -a.z); }
template <class T, class S> HD Vec3<T> operator*(const Vec3<T> &a, S s) { return Vec3<T>(a.x * s, a.y * s, a.z * s); }
template <class T, class S> HD Vec3<T> operator*(S s, const Vec3<T> &a) { return Vec3<T>(s * a.x, s * a.y, s * a.z); }
template <class T> HD Vec3<T> cmul(const Vec3<T> &a, const Vec3<T> &b) { return Vec3<T>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class T> HD T dot(const Vec3<T> &a, const Vec3<T> &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> HD Vec3<T> cross(const Vec3<T> &a, const Vec3<T> &b) {
    return Vec3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T> HD T sq(const T &x) { return x * x; }
template <class T> HD T length_sq(const Vec3<T> &v) { return sq(v.x) + sq(v.y) + sq(v.z); }
HD float luminance(const V3 &v) { return v.x * 0.212671f + v.y * 0.715160f + v.z * 0.072169f; }
// Eigen's DenseBase::isZero() with its default precision for float
// (NumTraits<float>::dummy_precision() = 1e-5): every |component| <= 1e-5. The
// reference rejects BSDF values and splats with this test (src/path.cpp:215,
// 556, 651, 751, 889, 908, 1454; src/integrators/delayed/delayed.cpp:260).
HD bool is_zero(const V3 &v) { return fabsf(v.x) <= 1e-5f && fabsf(v.y) <= 1e-5f && fabsf(v.z) <= 1e-5f; }
HD float max_coeff(const V3 &v) { return fmaxf(v.x, fmaxf(v.y, v.z)); }
HD bool all_finite(const V3 &v) { return isfinite(v.x) && isfinite(v.y) && isfinite(v.z); }
HD float length(const V3 &v) { return sqrtf(v.x * v.x + v.y * v.y + v.z * v.z); }
HD V3 normalize(const V3 &v) { float inv = 1.0f / length(v); return v * inv; }
HD float dist_sq(const V3 &a, const V3 &b) { return sq(a.x - b.x) + sq(a.y - b.y) + sq(a.z - b.z); }
HD V3 reflect(const V3 &wi, const V3 &n) { return (2.0f * dot(wi, n)) * n - wi; }
// Modulo(value, 1) of src/utils.h:383-386.
HD float mod1(float a) { float r = fmodf(a, 1.0f); return r < 0.0f ? r + 1.0f : r; }
// MIS power heuristic pieces of src/path.cpp:27-37.
HD float mis(float pdf) { return pdf * pdf; }
HD float mis_weight(float pdfA, float pdfB) { float r = sq(pdfB / pdfA); return 1.0f / (1.0f + r); }

// Orthonormal frame of src/utils.h:222-232.
HD void coordinate_system(const V3 &n, V3 &b1, V3 &b2) {
    if (n.z < float(-1.0 + 1e-6)) {
        b1 = V3(0.0f, -1.0f, 0.0f);
        b2 = V3(-1.0f, 0.0f, 0.0f);
        return;
    }
    const float a = 1.0f / (1.0f + n.z);
    const float b = -n.x * n.y * a;
    b1 = V3(1.0f - sq(n.x) * a, b, -n.x);
    b2 = V3(b, 1.0f - sq(n.y) * a, -n.y);
}

// Tent of src/utils.h:261-267 (as written there: 1 - sqrt(2u) below one half).
HD float tent(float u) { return u < 0.5f ? 1.0f - sqrtf(2.0f * u) : sqrtf(2.0f * (u - 0.5f)) - 1.0f; }

// SampleConcentricDisc of src/sampling.h:48-67.
HD void concentric_disc(float u0, float u1, float &x, float &y) {
    const float r1 = 2.0f * u0 - 1.0f;
    const float r2 = 2.0f * u1 - 1.0f;
    float phi, r;
    if (r1 == 0.0f || r2 == 0.0f) {
        r = phi = 0.0f;
    } else if (sq(r1) > sq(r2)) {
        r = r1;
        phi = kPiOverFour * (r2 / r1);
    } else {
        r = r2;
        phi = kPiOverTwo - (r1 / r2) * kPiOverFour;
    }
    x = r * cosf(phi);
    y = r * sinf(phi);
}

// Spherical direction parameterisation of src/sampling.h:7-40.
HD V3 sample_sphere(float u0, float u1, float &jacobian) {
    const float scaledTheta = kTwoPi * u0;
    const float scaledPhi = kPi * u1;
    const float sinPhi = sinf(scaledPhi);
    const float cosPhi = cosf(scaledPhi);
    jacobian = fabsf(sinPhi);
    return V3(sinPhi * cosf(scaledTheta), sinPhi * sinf(scaledTheta), cosPhi);
}
HD void to_spherical(const V3 &dir, float &u0, float &u1, float &jacobian) {
    float theta;
    if (dir.y == 0.0f && dir.x == 0.0f) {
        theta = 0.0f;
    } else {
        theta = atan2f(dir.y, dir.x);
        if (theta < 0.0f) theta += float(2.0 * 3.14159265358979323846);
    }
    theta *= kInvTwoPi;
    float phi = acosf(dir.z);
    jacobian = fabsf(sinf(phi));
    phi *= kInvPi;
    u0 = theta;
    u1 = phi;
}
HD V3 sample_cos_hemisphere(float u0, float u1) {
    const float phi = kTwoPi * u0;
    const float tmp = sqrtf(fmaxf(1.0f - u1, 0.0f));
    return V3(cosf(phi) * tmp, sinf(phi) * tmp, sqrtf(fmaxf(u1, 0.0f)));
}

// ---------------------------------------------------------------- scene layout
enum : int { kBsdfLambertian = 0, kBsdfPhong = 1, kBsdfRoughDielectric = 2 };
enum : int { kLightPoint = 0, kLightArea = 1, kLightEnv = 2 };  // src/light.h:7

struct Bsdf {
    int type;
    int twoSided;
    float kd[3];
    float ks[3];
    float exponent;
    float ksWeight;   // Phong::GetKsWeight (src/phong.cpp:158-167), precomputed on the host
    float intIOR, extIOR, alpha;
    float kt[3];
    float eta, invEta;  // RoughDielectric: intIOR / extIOR and its inverse (src/roughdielectric.h:17)
};

struct Light {
    int type;
    int shape;            // area light: emitting shape
    int triCdfOffset;     // area light: offset into Scene::lightTriCdf (numTris + 1 entries)
    int numTris;
    float emission[3];    // area: radiance; point: intensity
    float invTotalArea;   // area: SamplePdf (src/trianglemesh.cpp:364)
    float samplingWeight;
    float pos[3];         // point light position
};

struct Shape {
    int bsdf;
    int areaLight;   // light index or -1
    int triOffset;   // first global triangle of this shape
    int numTris;
};

// Triangle in BVH leaf order: p0 and the two edges (p1-p0, p2-p0) computed in
// single precision the way TriangleMesh does (src/trianglemesh.cpp:159-200).
struct Tri {
    float4 p0;   // w: global triangle index (int bits)
    float4 e1;   // w: shape index (int bits)
    float4 e2;
};

struct BvhNode {           // binary node holding both children's boxes (64 B)
    float4 lo0;            // child 0 min xyz, w = child 0 max x
    float4 hi0;            // child 0 max y z, child 1 min x y
    float4 b1;             // child 1 min z, max xyz
    int4 link;             // child0, child1, count0, count1 (count > 0: leaf [child, child+count))
};

struct Camera {
    float sampleToCam[16];
    float camToSample[16];
    float camToWorld[16];
    float worldToCam[16];
    float dist;
    float nearClip, farClip;
    int width, height;
};

struct Options {
    float roughnessThreshold;
    int useLightCoordinateSampling;
    float discreteStdDev;
    int minDepth, maxDepth;
};

struct SceneView {
    const Tri *tris;        // BVH-ordered triangles
    const float *triN;      // per global triangle: n0 n1 n2 (9 floats)
    const float *triP;      // per global triangle: p0 e1 e2 (9 floats) for re-intersection
    const int *triShape;    // per global triangle: shape index
    const BvhNode *nodes;
    const Shape *shapes;
    const Bsdf *bsdfs;
    const Light *lights;
    const float *lightCdf;     // numLights + 1 (PiecewiseConstant1D, src/distribution.h)
    const float *lightFunc;    // numLights
    const float *lightTriCdf;  // per area light: numTris + 1
    int numLights;
    int numTris;
    float lightFuncInt;
    float lightWeightSum;
    float bsCenter[3];
    float bsRadius;
    // environment light (EnvLight + EnvmapSampleInfo, src/envlight.cpp:24-81); envLight < 0: none
    const float *envImg;      // envW x envH RGB, row-major from the top row (Image3 layout)
    const float *envCdfRows;  // envH + 1
    const float *envCdfCols;  // envH x (envW + 1)
    const float *envRowW;     // envH: sin((y + 0.5) pi / envH)
    int envLight, envW, envH;
    float envNorm;            // 1 / (rowSum * pixelSize.x * pixelSize.y)
    float envPix[2];          // pixelSize: 2 pi / envW, pi / envH
    float envToWorld[9], envToLight[9];  // upper-left 3x3 of toWorld and its inverse
    Camera cam;
    Options opt;
};

// ---------------------------------------------------------------- samplers
// Counter-based stream: splitmix64 seeding of a 64-bit LCG with a permuted
// 32-bit output (PCG XSH-RR). Each (chain, iteration, stage) gets its own stream.
struct Rng {
    uint64_t state;
    Rng() = default;
    DEV static uint64_t mix(uint64_t z) {
        z += 0x9E3779B97F4A7C15ull;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    DEV Rng(uint64_t seed, uint64_t a, uint64_t b) {
        state = mix(seed ^ mix(a * 0x632BE59BD9B4E019ull + b));
        has_spare = false;
    }
    DEV uint32_t next_u32() {
        const uint64_t old = state;
        state = old * 6364136223846793005ull + 1442695040888963407ull;
        const uint32_t xorshifted = uint32_t(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = uint32_t(old >> 59u);
        return (xorshifted >> rot) | (xorshifted << ((32u - rot) & 31u));
    }
    DEV float uniform() { return float(next_u32() >> 8) * (1.0f / 16777216.0f); }
    bool has_spare;
    float spare;
    DEV float normal() {
        if (has_spare) { has_spare = false; return spare; }
        float u1 = uniform();
        const float u2 = uniform();
        if (u1 < 1e-30f) u1 = 1e-30f;
        const float r = sqrtf(-2.0f * logf(u1));
        float s, c;
        sincosf(kTwoPi * u2, &s, &c);
        spare = r * s;
        has_spare = true;
        return r * c;
    }
};

// Replays a recorded uniform stream (parity tests feed the reference's own draws).
struct TapeRng {
    const float *u;
    int n;
    int pos;
    DEV float uniform() { return pos < n ? u[pos++] : (pos++, 0.5f); }
    DEV float normal() { return 0.0f; }
};

}  // namespace drmlt
