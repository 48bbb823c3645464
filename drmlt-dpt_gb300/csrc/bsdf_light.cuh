// Single-precision BSDF, light and camera evaluation used by the path tracer.
// Each function states the reference routine whose arithmetic it reproduces.
#pragma once
#include "trace.cuh"

namespace drmlt {

struct BsdfOut {
    V3 contrib;
    float cosWo, pdf, revPdf;
};

DEV V3 kd_of(const Bsdf &b) { return V3(b.kd[0], b.kd[1], b.kd[2]); }
DEV V3 ks_of(const Bsdf &b) { return V3(b.ks[0], b.ks[1], b.ks[2]); }
DEV V3 kt_of(const Bsdf &b) { return V3(b.kt[0], b.kt[1], b.kt[2]); }

// ---------------------------------------------------------------- rough dielectric
// BeckmennDistributionTerm (src/microfacet.h:6-18), isotropic roughness.
DEV float beckmann_d(const V3 &h, float alpha) {
    const float cosTheta2 = sq(h.z);
    const float e = (sq(h.x) / sq(alpha) + sq(h.y) / sq(alpha)) / cosTheta2;
    return expf(-e) / (kPi * alpha * alpha * sq(cosTheta2));
}

// BeckmennGeometryTerm (src/microfacet.h:20-38, 62-67): the rational
// approximation of the shadowing-masking term, per direction.
DEV float beckmann_g1(float alpha, float cosTheta) {
    const float tanTheta = sqrtf(fabsf(1.0f - sq(cosTheta))) / cosTheta;
    if (tanTheta <= 0.0f) return 1.0f;
    const float a = 1.0f / (alpha * tanTheta);
    if (a >= 1.6f) return 1.0f;
    const float a2 = a * a;
    return (3.535f * a + 2.181f * a2) / (1.0f + 2.276f * a + 2.577f * a2);
}

// FresnelDielectricExt (src/microfacet.h:69-115); cosThetaT is signed as there.
DEV float fresnel_dielectric(float cosThetaI_, float &cosThetaT_, float eta, float invEta) {
    const float scale = cosThetaI_ > 0.0f ? invEta : eta;
    const float cosThetaTSqr = 1.0f - (1.0f - sq(cosThetaI_)) * sq(scale);
    if (cosThetaTSqr <= 0.0f) {
        cosThetaT_ = 0.0f;
        return 1.0f;
    }
    const float cosThetaI = fabsf(cosThetaI_);
    const float cosThetaT = sqrtf(cosThetaTSqr);
    const float Rs = (cosThetaI - eta * cosThetaT) / (cosThetaI + eta * cosThetaT);
    const float Rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
    cosThetaT_ = cosThetaI_ > 0.0f ? -cosThetaT : cosThetaT;
    return 0.5f * (sq(Rs) + sq(Rp));
}

// SampleMicronormal (src/microfacet.h:166-185), primal form.
DEV V3 sample_micronormal(float r0, float r1, float alpha, float &pdfW) {
    const float phiM = kTwoPi * r1;
    const float sinPhiM = sinf(phiM), cosPhiM = cosf(phiM);
    const float alphaSqr = sq(alpha);
    const float tanThetaMSqr = alphaSqr * (-logf(fmaxf(1.0f - r0, 1e-6f)));
    const float cosThetaM = 1.0f / sqrtf(1.0f + tanThetaMSqr);
    const float cosThetaMSqr = sq(cosThetaM);
    pdfW = (1.0f - r0) / (kPi * alphaSqr * cosThetaM * cosThetaMSqr);
    const float sinThetaM = sqrtf(fmaxf(1.0f - cosThetaMSqr, 0.0f));
    return V3(sinThetaM * cosPhiM, sinThetaM * sinPhiM, cosThetaM);
}

// Refract (src/utils.h:202-210).
DEV V3 refract_dir(const V3 &wi, const V3 &n, float cosThetaT, float eta, float invEta) {
    const float e = cosThetaT < 0.0f ? invEta : eta;
    return n * (dot(wi, n) * e + cosThetaT) - wi * e;
}

// Evaluate<adjoint> of src/roughdielectric.cpp:22-124.
template <bool adjoint>
DEV void rough_dielectric_evaluate(const Bsdf &b, const V3 &wi, const V3 &normal, const V3 &wo, BsdfOut &o) {
    const float cosWi = dot(wi, normal);
    o.contrib = V3(0.0f, 0.0f, 0.0f);
    o.cosWo = 0.0f;
    o.pdf = o.revPdf = 0.0f;
    if (fabsf(cosWi) < kCosEps) return;
    o.cosWo = dot(wo, normal);
    const float cosWo = o.cosWo;
    if (fabsf(cosWo) < kCosEps) return;
    const bool reflect = cosWi * cosWo > 0.0f;
    const float eta_ = cosWi > 0.0f ? b.eta : b.invEta;
    const float revEta_ = cosWo > 0.0f ? b.eta : b.invEta;
    V3 H = reflect ? normalize(V3(wi + wo)) : normalize(V3(wi + wo * eta_));
    if (dot(H, normal) < 0.0f) H = -H;
    const float cosHWi = dot(wi, H), cosHWo = dot(wo, H);
    if (fabsf(cosHWi) < kCosEps || fabsf(cosHWo) < kCosEps) return;
    if (cosHWi * cosWi <= 0.0f || cosHWo * cosWo <= 0.0f) return;
    V3 b0, b1;
    coordinate_system(normal, b0, b1);
    const V3 localH(dot(b0, H), dot(b1, H), dot(normal, H));
    const float alp = b.alpha;
    const float D = beckmann_d(localH, alp);
    if (D <= 0.0f) return;
    const float revCosHWi = cosHWo, revCosHWo = cosHWi;
    float ct;
    const float F = fresnel_dielectric(cosHWi, ct, b.eta, b.invEta);
    const float aCosWi = fabsf(cosWi), aCosWo = fabsf(cosWo);
    const float G = beckmann_g1(alp, aCosWi) * beckmann_g1(alp, aCosWo);
    const float scaledAlpha = alp * (1.2f - 0.2f * sqrtf(aCosWi));
    const float prob = localH.z * beckmann_d(localH, scaledAlpha);
    if (prob < 1e-20f) return;
    const float revScaledAlpha = alp * (1.2f - 0.2f * sqrtf(aCosWo));
    const float revProb = localH.z * beckmann_d(localH, revScaledAlpha);
    if (reflect) {
        const float scalar = fabsf(F * D * G / (4.0f * cosWi));
        o.contrib = ks_of(b) * scalar;
        o.pdf = fabsf(prob * F / (4.0f * cosHWo));
        o.revPdf = fabsf(revProb * F / (4.0f * revCosHWo));
    } else {
        const float sqrtDenom = cosHWi + eta_ * cosHWo;
        const float revSqrtDenom = revCosHWi + revEta_ * revCosHWo;
        const float factor = adjoint ? 1.0f : sq(1.0f / eta_);
        const float scalar = fabsf(factor * ((1.0f - F) * D * G * sq(eta_) * cosHWi * cosHWo) / (cosWi * sq(sqrtDenom)));
        o.contrib = kt_of(b) * scalar;
        o.pdf = fabsf(prob * (1.0f - F) * (sq(eta_) * cosHWo) / sq(sqrtDenom));
        o.revPdf = fabsf(revProb * (1.0f - F) * (sq(revEta_) * revCosHWo) / sq(revSqrtDenom));
    }
}

// Sample<adjoint> of src/roughdielectric.cpp:147-254.
template <bool adjoint>
DEV bool rough_dielectric_sample(const Bsdf &b, const V3 &wi, const V3 &normal, float r0, float r1, float uDiscrete,
                                 V3 &wo, BsdfOut &o) {
    const float cosWi = dot(wi, normal);
    if (fabsf(cosWi) < kCosEps) return false;
    const float alp = b.alpha;
    const float scaledAlp = alp * (1.2f - 0.2f * sqrtf(fabsf(cosWi)));
    float mPdf;
    const V3 localH = sample_micronormal(r0, r1, scaledAlp, mPdf);
    o.pdf = mPdf;
    V3 b0, b1;
    coordinate_system(normal, b0, b1);
    const V3 H = localH.x * b0 + localH.y * b1 + localH.z * normal;
    const float cosHWi = dot(wi, H);
    if (fabsf(cosHWi) < kCosEps) return false;
    float cosThetaT = 0.0f;
    const float F = fresnel_dielectric(cosHWi, cosThetaT, b.eta, b.invEta);
    V3 refl;
    float cosHWo;
    if (uDiscrete <= F) {
        wo = reflect(wi, H);
        if (F <= 0.0f || dot(normal, wo) * dot(normal, wi) <= 0.0f) return false;
        refl = ks_of(b);
        cosHWo = dot(wo, H);
        o.pdf = fabsf(o.pdf * F / (4.0f * cosHWo));
        const float rev_dwh_dwo = 1.0f / (4.0f * cosHWi);
        o.cosWo = dot(wo, normal);
        if (fabsf(o.cosWo) < kCosEps) return false;
        const float revScaledAlp = alp * (1.2f - 0.2f * sqrtf(fabsf(o.cosWo)));
        o.revPdf = fabsf(F * beckmann_d(localH, revScaledAlp) * localH.z * rev_dwh_dwo);
    } else {
        wo = refract_dir(wi, H, cosThetaT, b.eta, b.invEta);
        if (F >= 1.0f || cosThetaT == 0.0f || dot(normal, wo) * dot(normal, wi) >= 0.0f) return false;
        const float eta_ = cosWi > 0.0f ? b.eta : b.invEta;
        const float factor = adjoint ? 1.0f : sq(1.0f / eta_);
        refl = kt_of(b) * factor;
        cosHWo = dot(wo, H);
        const float sqrtDenom = cosHWi + eta_ * cosHWo;
        const float dwh_dwo = (sq(eta_) * cosHWo) / sq(sqrtDenom);
        o.pdf = fabsf(o.pdf * (1.0f - F) * fabsf(dwh_dwo));
        o.cosWo = dot(wo, normal);
        if (fabsf(o.cosWo) < kCosEps) return false;
        const float revEta_ = o.cosWo > 0.0f ? b.eta : b.invEta;
        const float revSqrtDenom = cosHWo + revEta_ * cosHWi;
        const float rev_dwh_dwo = (sq(revEta_) * cosHWi) / sq(revSqrtDenom);
        const float revScaledAlp = alp * (1.2f - 0.2f * sqrtf(fabsf(o.cosWo)));
        o.revPdf = fabsf((1.0f - F) * beckmann_d(localH, revScaledAlp) * localH.z * rev_dwh_dwo);
    }
    if (fabsf(cosHWo) < kCosEps) return false;
    if (o.pdf < 1e-20f) return false;
    if (cosHWi * cosWi <= 0.0f || cosHWo * o.cosWo <= 0.0f) return false;
    const float aCosWi = fabsf(cosWi), aCosWo = fabsf(o.cosWo);
    const float D = beckmann_d(localH, alp);
    const float G = beckmann_g1(alp, aCosWi) * beckmann_g1(alp, aCosWo);
    o.contrib = refl * fabsf((D * G * cosHWi) / (mPdf * aCosWi));
    return true;
}

// Lambertian::Evaluate (src/lambertian.cpp:15-38), Phong::Evaluate (src/phong.cpp:21-62),
// RoughDielectric::Evaluate / EvaluateAdjoint (src/roughdielectric.cpp:126-144).
template <bool adjoint = false>
DEV_SHARED void bsdf_evaluate(const Bsdf &b, const V3 &wi, const V3 &normal, const V3 &wo, BsdfOut &o) {
    if (b.type == kBsdfRoughDielectric) {
        rough_dielectric_evaluate<adjoint>(b, wi, normal, wo, o);
        return;
    }
    o.contrib = V3(0.0f, 0.0f, 0.0f);
    o.pdf = 0.0f;
    o.revPdf = 0.0f;
    float cosWi = dot(normal, wi);
    V3 n = normal;
    if (b.twoSided && cosWi < 0.0f) {
        cosWi = -cosWi;
        n = -n;
    }
    o.cosWo = dot(n, wo);
    if (b.type == kBsdfLambertian) {
        if (cosWi < kCosEps || o.cosWo < kCosEps) return;
        const float fwd = o.cosWo * kInvPi;
        o.contrib = fwd * kd_of(b);
        o.pdf = fwd;
        o.revPdf = cosWi * kInvPi;
        return;
    }
    // Phong
    if (cosWi <= kCosEps || o.cosWo <= kCosEps) return;
    if (b.ksWeight > 0.0f) {
        const float alpha = fmaxf(dot(reflect(wi, n), wo), 0.0f);
        const float weight = powf(alpha, b.exponent) * kInvTwoPi;
        if (weight > 1e-10f) {
            o.contrib = ks_of(b) * ((b.exponent + 2.0f) * weight);
            o.pdf = b.ksWeight * (b.exponent + 1.0f) * weight;
            o.revPdf = o.pdf;
        }
    }
    if (b.ksWeight < 1.0f) {
        o.pdf += (1.0f - b.ksWeight) * o.cosWo * kInvPi;
        o.revPdf += (1.0f - b.ksWeight) * cosWi * kInvPi;
        o.contrib = o.contrib + kd_of(b) * kInvPi;
    }
    o.contrib = o.contrib * o.cosWo;
    if (max_coeff(o.contrib) < 1e-10f) o.contrib = V3(0.0f, 0.0f, 0.0f);
}

// Lambertian::Sample (src/lambertian.cpp:56-90), Phong::Sample (src/phong.cpp:64-147),
// RoughDielectric::Sample / SampleAdjoint (src/roughdielectric.cpp:256-282).
template <bool adjoint = false>
DEV_SHARED bool bsdf_sample(const Bsdf &b, const V3 &wi, const V3 &normal, float r0, float r1, float uDiscrete,
                     V3 &wo, BsdfOut &o) {
    if (b.type == kBsdfRoughDielectric) return rough_dielectric_sample<adjoint>(b, wi, normal, r0, r1, uDiscrete, wo, o);
    float cosWi = dot(wi, normal);
    if (fabsf(cosWi) < kCosEps) return false;
    V3 n = normal;
    if (cosWi < 0.0f) {
        if (b.twoSided) {
            cosWi = -cosWi;
            n = -n;
        } else {
            return false;
        }
    }
    if (b.type == kBsdfLambertian) {
        V3 b0, b1;
        coordinate_system(n, b0, b1);
        const V3 l = sample_cos_hemisphere(r0, r1);
        wo = l.x * b0 + l.y * b1 + l.z * n;
        o.cosWo = l.z;
        o.pdf = l.z * kInvPi;
        if (o.cosWo < kCosEps) return false;
        o.revPdf = cosWi * kInvPi;
        o.contrib = kd_of(b);
        return true;
    }
    const V3 R = reflect(wi, n);
    float g;
    V3 axis;
    if (uDiscrete > b.ksWeight) {
        g = 1.0f;
        axis = n;
    } else {
        g = b.exponent;
        axis = R;
    }
    const float power = 1.0f / (g + 1.0f);
    const float cosAlpha = powf(r1, power);
    const float sinAlpha = sqrtf(1.0f - sq(cosAlpha));
    const float phi = kTwoPi * r0;
    const V3 local(sinAlpha * cosf(phi), sinAlpha * sinf(phi), cosAlpha);
    V3 b0, b1;
    coordinate_system(axis, b0, b1);
    wo = local.x * b0 + local.y * b1 + local.z * axis;
    o.cosWo = dot(n, wo);
    if (o.cosWo < kCosEps) return false;
    o.contrib = V3(0.0f, 0.0f, 0.0f);
    o.pdf = 0.0f;
    o.revPdf = 0.0f;
    if (b.ksWeight > 0.0f) {
        const float alpha = fmaxf(dot(R, wo), 0.0f);
        const float weight = powf(alpha, b.exponent) * kInvTwoPi;
        if (weight > 1e-10f) {
            o.contrib = ks_of(b) * ((b.exponent + 2.0f) * weight);
            o.pdf = b.ksWeight * (b.exponent + 1.0f) * weight;
        }
        o.revPdf = o.pdf;
    }
    if (b.ksWeight < 1.0f) {
        o.contrib = o.contrib + kd_of(b) * kInvPi;
        o.pdf += (1.0f - b.ksWeight) * o.cosWo * kInvPi;
        o.revPdf += (1.0f - b.ksWeight) * cosWi * kInvPi;
    }
    o.contrib = o.contrib * o.cosWo;
    if (o.pdf < 1e-10f) return false;
    o.contrib = o.contrib * (1.0f / o.pdf);
    return true;
}

// BSDF::Roughness: Lambertian 1 (src/lambertian.h:38-40), Phong (src/phong.cpp:149-156),
// RoughDielectric alpha (src/roughdielectric.h:60-62).
DEV float bsdf_roughness(const Bsdf &b, float uDiscrete) {
    if (b.type == kBsdfRoughDielectric) return b.alpha;
    if (b.type == kBsdfPhong && uDiscrete < b.ksWeight) return sqrtf(2.0f / (2.0f + 4.0f * b.exponent));
    return 1.0f;
}

// ShadingNormalCorrection<adjoint> of src/path.cpp:39-59.
template <bool adjoint>
DEV float shading_normal_correction(const V3 &wi, const Isect &isect, const V3 &wo) {
    const float cosWi = dot(isect.shadingNormal, wi);
    const float cosWo = dot(isect.shadingNormal, wo);
    const float wiDotGeoN = dot(isect.geomNormal, wi);
    const float woDotGeoN = dot(isect.geomNormal, wo);
    if (wiDotGeoN * cosWi <= 0.0f || woDotGeoN * cosWo <= 0.0f) return 0.0f;
    if (adjoint) return fabsf((woDotGeoN * cosWi) / (wiDotGeoN * cosWo));
    return 1.0f;
}

// ---------------------------------------------------------------- lights
// PiecewiseConstant1D::SampleDiscrete (src/distribution.h:45-51): upper_bound on the CDF.
DEV int sample_discrete(const float *cdf, int count, float u) {
    int lo = 0, hi = count + 1;   // first index with cdf[i] > u
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) > u) hi = mid; else lo = mid + 1;
    }
    int off = lo - 1;
    return off < 0 ? 0 : (off > count - 1 ? count - 1 : off);
}

// PickLight / PickLightProb (src/scene.cpp:113-121).
DEV int pick_light(const SceneView &s, float u, float &prob) {
    const int id = sample_discrete(s.lightCdf, s.numLights, u);
    prob = s.lightFunc[id] / (s.lightFuncInt * float(s.numLights));
    return id;
}
DEV float pick_light_prob(const SceneView &s, int light) {
    return s.lights[light].samplingWeight / s.lightWeightSum;
}

// TriangleMesh::Sample(rndParam, ...) + SampleDirect (src/trianglemesh.cpp:315-364).
DEV void sample_triangle(const SceneView &s, int tri, float r0, float r1, V3 &pos, V3 &normal) {
    const float *P = s.triP + 9 * tri;
    const V3 p0 = ld3(P), e1 = ld3(P + 3), e2 = ld3(P + 6);
    const float *N = s.triN + 9 * tri;
    const float a = sqrtf(1.0f - r0);
    const float b1 = 1.0f - a;
    const float b2 = a * r1;
    pos = p0 + (e1 * b1) + (e2 * b2);
    normal = normalize(V3(ld3(N) * (1.0f - b1 - b2) + ld3(N + 3) * b1 + ld3(N + 6) * b2));
}

// TriangleMesh::GetSampleParam (src/trianglemesh.cpp:238-296).
DEV void triangle_sample_param(const SceneView &s, int tri, const V3 &position, float &u0, float &u1) {
    const float *P = s.triP + 9 * tri;
    const V3 p0 = ld3(P), e1 = ld3(P + 3), e2 = ld3(P + 6);
    const V3 e0 = position - p0;
    const float d11 = dot(e1, e1), d12 = dot(e1, e2), d22 = dot(e2, e2);
    const float d01 = dot(e0, e1), d02 = dot(e0, e2);
    const float invDenom = 1.0f / (d11 * d22 - d12 * d12);
    const float b1 = (d22 * d01 - d12 * d02) * invDenom;
    const float b2 = (d11 * d02 - d12 * d01) * invDenom;
    const float a = 1.0f - b1;
    u0 = 1.0f - sq(a);
    u1 = b2 / a;
}

DEV int light_tri(const SceneView &s, const Light &L, int lPrim) {
    return s.shapes[L.shape].triOffset + lPrim;
}

// ---------------------------------------------------------------- environment light
// EnvLight (src/envlight.cpp:24-240) on an image with its EnvmapSampleInfo.
DEV V3 env_at(const SceneView &s, int x, int y) {
    // Image3::At (src/image.h:27-32) indexes y * width + x without wrapping: col + 1
    // past the last column reads the next row's first pixel. Indexes past the
    // image's end (undefined in the reference) are clamped to the last pixel.
    const int i = min(y * s.envW + x, s.envW * s.envH - 1);
    return ld3(s.envImg + 3 * i);
}
DEV V3 env_rep_at(const SceneView &s, int x, int y) {  // Image3::RepAt (src/image.h:33-38)
    int yy = y % s.envH, xx = x % s.envW;
    if (yy < 0) yy += s.envH;
    if (xx < 0) xx += s.envW;
    return ld3(s.envImg + 3 * (yy * s.envW + xx));
}
DEV float env_row_weight(const SceneView &s, int row) {
    return __ldg(s.envRowW + (row < 0 ? 0 : (row > s.envH - 1 ? s.envH - 1 : row)));
}
DEV V3 xform3(const float *m, const V3 &v) {
    return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
              m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
// uToIndex of SampleDirection: lower_bound over cdf[0..size], index clamped to
// [0, size-1], u rescaled to the cell.
DEV int env_u_to_index(const float *cdf, int size, float &u) {
    int lo = 0, hi = size + 1;  // first index with cdf[i] >= u
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid) < u) lo = mid + 1; else hi = mid;
    }
    const int index = min(max(lo - 1, 0), size - 1);
    const float c0 = __ldg(cdf + index);
    u = (u - c0) / (__ldg(cdf + index + 1) - c0);
    return index;
}
// SampleDirection (src/envlight.cpp:120-169). lPrim: the sampled pixel.
DEV_SHARED void env_sample_direction(const SceneView &s, float u0, float u1, V3 &dirToLight, V3 &value, float &pdf,
                              int &lPrim) {
    const int row = env_u_to_index(s.envCdfRows, s.envH, u1);
    const int col = env_u_to_index(s.envCdfCols + row * (s.envW + 1), s.envW, u0);
    lPrim = row * s.envW + col;
    const float t0 = tent(u0), t1 = tent(u1);
    const float phi = (float(col) + t0 + 0.5f) * s.envPix[0];
    const float theta = (float(row) + t1 + 0.5f) * s.envPix[1];
    float sinPhi, cosPhi, sinTheta, cosTheta;
    sinPhi = sinf(phi);
    cosPhi = cosf(phi);
    sinTheta = sinf(theta);
    cosTheta = cosf(theta);
    dirToLight = xform3(s.envToWorld, V3(sinPhi * sinTheta, cosTheta, -cosPhi * sinTheta));
    const float dx1 = t0, dx2 = 1.0f - t0, dy1 = t1, dy2 = 1.0f - t1;
    const V3 value1 = env_at(s, col, row) * dx2 * dy2 + env_at(s, col + 1, row) * dx1 * dy2;
    const V3 value2 = env_at(s, col, row + 1) * dx2 * dy1 + env_at(s, col + 1, row + 1) * dx1 * dy1;
    value = value1 + value2;
    pdf = (luminance(value1) * env_row_weight(s, row) + luminance(value2) * env_row_weight(s, row + 1)) *
          s.envNorm / fmaxf(fabsf(sinTheta), 1e-7f);
}
DEV float env_position_pdf(const SceneView &s) { return kInvPi / sq(s.bsRadius); }

// EnvLight::Emission (src/envlight.cpp:193-222).
DEV_SHARED void env_emission(const SceneView &s, const Light &L, const V3 &dirToLight, V3 &emission, float &directPdf,
                      float &emissionPdf) {
    const V3 d = xform3(s.envToLight, dirToLight);
    const float uvx = atan2f(d.x, -d.z) * kInvTwoPi * float(s.envW) - 0.5f;
    const float uvy = acosf(d.y) * kInvPi * float(s.envH) - 0.5f;
    const int col = int(floorf(uvx));
    const int row = int(floorf(uvy));
    const float dx1 = uvx - float(col), dx2 = 1.0f - dx1, dy1 = uvy - float(row), dy2 = 1.0f - dy1;
    const V3 value1 = env_rep_at(s, col, row) * dx2 * dy2 + env_rep_at(s, col + 1, row) * dx1 * dy2;
    const V3 value2 = env_rep_at(s, col, row + 1) * dx2 * dy1 + env_rep_at(s, col + 1, row + 1) * dx1 * dy1;
    emission = (value1 + value2) * L.samplingWeight;
    const float sinTheta = sqrtf(1.0f - sq(d.y));
    directPdf = (luminance(value1) * env_row_weight(s, row) + luminance(value2) * env_row_weight(s, row + 1)) *
                s.envNorm / fmaxf(fabsf(sinTheta), 1e-7f);
    emissionPdf = directPdf * env_position_pdf(s);
}

// AreaLight::SampleDirect (src/arealight.cpp:29-57).
DEV_SHARED bool light_sample_direct(const SceneView &s, int li, int lPrim, const V3 &pos, float r0, float r1,
                             V3 &dirToLight, float &dist, V3 &contrib, float &cosAtLight,
                             float &directPdf, float &emissionPdf) {
    const Light &L = s.lights[li];
    if (L.type == kLightArea) {
        V3 p, n;
        sample_triangle(s, light_tri(s, L, lPrim), r0, r1, p, n);
        const float shapePdf = L.invTotalArea;
        dirToLight = p - pos;
        const float distSq = length_sq(dirToLight);
        dist = sqrtf(distSq);
        dirToLight = V3(dirToLight.x / dist, dirToLight.y / dist, dirToLight.z / dist);
        cosAtLight = -dot(dirToLight, n);
        if (cosAtLight > kCosEps) {
            contrib = (cosAtLight / (distSq * shapePdf)) * V3(L.emission[0], L.emission[1], L.emission[2]);
            directPdf = shapePdf * distSq / cosAtLight;
            emissionPdf = shapePdf * cosAtLight * kInvPi;
            return true;
        }
        return false;
    }
    if (L.type == kLightEnv) {  // EnvLight::SampleDirect (src/envlight.cpp:171-191)
        V3 value;
        int lp;
        env_sample_direction(s, r0, r1, dirToLight, value, directPdf, lp);
        dist = INFINITY;
        contrib = value * (1.0f / directPdf) * L.samplingWeight;
        cosAtLight = 1.0f;
        emissionPdf = directPdf * env_position_pdf(s);
        return true;
    }
    // PointLight::SampleDirect (src/pointlight.cpp): delta light at a position.
    const V3 lp(L.pos[0], L.pos[1], L.pos[2]);
    dirToLight = lp - pos;
    const float distSq = length_sq(dirToLight);
    dist = sqrtf(distSq);
    dirToLight = V3(dirToLight.x / dist, dirToLight.y / dist, dirToLight.z / dist);
    contrib = V3(L.emission[0], L.emission[1], L.emission[2]) * (1.0f / distSq);
    cosAtLight = 1.0f;
    directPdf = distSq;
    emissionPdf = 1.0f / (4.0f * kPi);
    return true;
}

// AreaLight::Emission (src/arealight.cpp:59-76).
DEV_SHARED void light_emission(const SceneView &s, int li, const V3 &dirToLight, const V3 &normalOnLight, V3 &emission,
                        float &directPdf, float &emissionPdf) {
    const Light &L = s.lights[li];
    if (L.type == kLightEnv) {
        env_emission(s, L, dirToLight, emission, directPdf, emissionPdf);
        return;
    }
    const float cosAtLight = -dot(normalOnLight, dirToLight);
    if (L.type == kLightArea && cosAtLight > 0.0f) {
        emission = V3(L.emission[0], L.emission[1], L.emission[2]);
        directPdf = L.invTotalArea;
        emissionPdf = cosAtLight * directPdf * kInvPi;
    } else {
        emission = V3(0.0f, 0.0f, 0.0f);
        directPdf = 0.0f;
        emissionPdf = 0.0f;
    }
}

// AreaLight::Emit (src/arealight.cpp:78-102).
DEV_SHARED void light_emit(const SceneView &s, int li, int lPrim, float p0, float p1, float d0, float d1, V3 &org,
                    V3 &dir, V3 &emission, float &cosAtLight, float &emissionPdf, float &directPdf) {
    const Light &L = s.lights[li];
    if (L.type == kLightPoint) {  // PointLight::Emit (src/pointlight.cpp:58-72)
        float jac;
        org = V3(L.pos[0], L.pos[1], L.pos[2]);
        dir = sample_sphere(d0, d1, jac);
        emission = V3(L.emission[0], L.emission[1], L.emission[2]);
        emissionPdf = 1.0f / (4.0f * kPi);
        cosAtLight = directPdf = 1.0f;
        return;
    }
    if (L.type == kLightEnv) {  // EnvLight::Emit (src/envlight.cpp:224-247)
        int lp;
        env_sample_direction(s, d0, d1, dir, emission, directPdf, lp);
        emission = emission * L.samplingWeight;
        dir = -dir;
        float ox, oy;
        concentric_disc(p0, p1, ox, oy);
        V3 b0, b1;
        coordinate_system(dir, b0, b1);
        const V3 perp = ox * b0 + oy * b1;
        org = V3(s.bsCenter[0], s.bsCenter[1], s.bsCenter[2]) + (perp - dir) * s.bsRadius;
        cosAtLight = 1.0f;
        emissionPdf = directPdf * env_position_pdf(s);
        return;
    }
    V3 normal;
    sample_triangle(s, light_tri(s, L, lPrim), p0, p1, org, normal);
    const float shapePdf = L.invTotalArea;
    const V3 d = sample_cos_hemisphere(d0, d1);
    V3 b0, b1;
    coordinate_system(normal, b0, b1);
    dir = d.x * b0 + d.y * b1 + d.z * normal;
    emission = V3(L.emission[0], L.emission[1], L.emission[2]) * (kPi / shapePdf);
    cosAtLight = d.z;
    emissionPdf = d.z * kInvPi * shapePdf;
    directPdf = shapePdf;
}

DEV bool light_is_delta(const SceneView &s, int li) { return s.lights[li].type == kLightPoint; }
DEV bool light_is_finite(const SceneView &s, int li) { return s.lights[li].type == kLightArea; }

// ---------------------------------------------------------------- camera
DEV V3 xform_point(const float *m, const V3 &p) {
    const float x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    const float y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    const float z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    const float w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    const float invW = 1.0f / w;
    return V3(x * invW, y * invW, z * invW);
}
DEV V3 xform_vector(const float *m, const V3 &v) {
    return V3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
              m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

// SamplePrimary (src/camera.cpp:38-49).
DEV void sample_primary(const Camera &c, float sx, float sy, V3 &org, V3 &dir, float &minT, float &maxT) {
    const V3 o = xform_point(c.sampleToCam, V3(sx, sy, 0.0f));
    const V3 d = normalize(o);
    const float invZ = 1.0f / d.z;
    org = xform_point(c.camToWorld, V3(0.0f, 0.0f, 0.0f));
    dir = xform_vector(c.camToWorld, d);
    minT = c.nearClip * invZ;
    maxT = c.farClip * invZ;
}

// ProjectPoint (src/camera.cpp:58-75).
DEV bool project_point(const Camera &c, const V3 &p, float &sx, float &sy) {
    const V3 camP = xform_point(c.worldToCam, p);
    if (camP.z < c.nearClip || camP.z > c.farClip) return false;
    const V3 r = xform_point(c.camToSample, camP);
    if (r.x < 0.0f || r.x > 1.0f || r.y < 0.0f || r.y > 1.0f) return false;
    sx = r.x;
    sy = r.y;
    return true;
}

}  // namespace drmlt
