// Derivatives of f(u) = log Luminance(contribution) with respect to the
// primary sample vector u of a fixed technique path, on fixed triangles.
//
// f is the function the reference's chad code generator differentiates
// (RegisterPathFuncBidir, src/path.cpp:2987-3175, static mode: time excluded),
// including that builder's own rules: no occlusion tests, re-intersection with
// the stored triangle's plane, BSDF forms without the primal epsilon checks
// (src/lambertian.cpp:92-150, src/phong.cpp:168-392), the emitter's
// accMISWThis taken only for point lights (src/path.cpp:2600-2608), ADEpsilon
// 1e-6 clamps (src/utils.h:442-449), and branches selected by value with
// derivatives flowing through the taken branch (src/chad.cpp:70-110).
//
// The scalar type is templated: float for values, HyperDual for exact second
// derivatives. A HyperDual carries (f, df/du_i, df/du_j, d2f/du_i du_j): one
// evaluation yields one Hessian entry and two gradient entries, so a chain's
// D(D+1)/2 Hessian entries are independent threads that follow the same
// control flow (branches depend on values only).
#pragma once
#include "path.cuh"

namespace drmlt {

struct HyperDual {
    float v, a, b, ab;
    HD HyperDual() {}
    HD explicit HyperDual(float x) : v(x), a(0.0f), b(0.0f), ab(0.0f) {}
    HD HyperDual(float x, float da, float db, float dab) : v(x), a(da), b(db), ab(dab) {}
};
HD HyperDual operator+(const HyperDual &x, const HyperDual &y) { return HyperDual(x.v + y.v, x.a + y.a, x.b + y.b, x.ab + y.ab); }
HD HyperDual operator-(const HyperDual &x, const HyperDual &y) { return HyperDual(x.v - y.v, x.a - y.a, x.b - y.b, x.ab - y.ab); }
HD HyperDual operator-(const HyperDual &x) { return HyperDual(-x.v, -x.a, -x.b, -x.ab); }
HD HyperDual operator*(const HyperDual &x, const HyperDual &y) {
    return HyperDual(x.v * y.v, x.a * y.v + x.v * y.a, x.b * y.v + x.v * y.b,
                     x.ab * y.v + x.a * y.b + x.b * y.a + x.v * y.ab);
}
HD HyperDual operator*(const HyperDual &x, float s) { return HyperDual(x.v * s, x.a * s, x.b * s, x.ab * s); }
HD HyperDual operator*(float s, const HyperDual &x) { return x * s; }
HD HyperDual operator+(const HyperDual &x, float s) { return HyperDual(x.v + s, x.a, x.b, x.ab); }
HD HyperDual operator+(float s, const HyperDual &x) { return x + s; }
HD HyperDual operator-(const HyperDual &x, float s) { return HyperDual(x.v - s, x.a, x.b, x.ab); }
HD HyperDual operator-(float s, const HyperDual &x) { return HyperDual(s - x.v, -x.a, -x.b, -x.ab); }
// Generic unary rule: f(x) with first and second derivative d1, d2 at x.v.
HD HyperDual chain(const HyperDual &x, float f, float d1, float d2) {
    return HyperDual(f, d1 * x.a, d1 * x.b, d1 * x.ab + d2 * x.a * x.b);
}
HD HyperDual inv(const HyperDual &x) {
    const float r = 1.0f / x.v;
    return chain(x, r, -r * r, 2.0f * r * r * r);
}
HD HyperDual operator/(const HyperDual &x, const HyperDual &y) { return x * inv(y); }
HD HyperDual operator/(const HyperDual &x, float s) { return x * (1.0f / s); }
HD HyperDual operator/(float s, const HyperDual &y) { return s * inv(y); }
HD HyperDual sqrt(const HyperDual &x) {
    const float r = sqrtf(x.v);
    return chain(x, r, 0.5f / r, -0.25f / (r * x.v));
}
HD HyperDual sin(const HyperDual &x) {
    float s, c;
    sincosf(x.v, &s, &c);
    return chain(x, s, c, -s);
}
HD HyperDual cos(const HyperDual &x) {
    float s, c;
    sincosf(x.v, &s, &c);
    return chain(x, c, -s, -c);
}
HD HyperDual log(const HyperDual &x) {
    const float r = 1.0f / x.v;
    return chain(x, logf(x.v), r, -r * r);
}
HD HyperDual pow(const HyperDual &x, float e) {
    const float p = powf(x.v, e);
    const float d1 = e * powf(x.v, e - 1.0f);
    const float d2 = e * (e - 1.0f) * powf(x.v, e - 2.0f);
    return chain(x, p, d1, d2);
}
HD HyperDual exp(const HyperDual &x) {
    const float e = expf(x.v);
    return chain(x, e, e, e);
}
// atan2(y, x) with its first and second partial derivatives.
HD HyperDual atan2(const HyperDual &y, const HyperDual &x) {
    const float r2 = x.v * x.v + y.v * y.v;
    const float ir2 = 1.0f / r2;
    const float fy = x.v * ir2, fx = -y.v * ir2;
    const float ir4 = ir2 * ir2;
    const float fyy = -2.0f * x.v * y.v * ir4, fxx = -fyy, fxy = (y.v * y.v - x.v * x.v) * ir4;
    return HyperDual(atan2f(y.v, x.v), fy * y.a + fx * x.a, fy * y.b + fx * x.b,
                     fy * y.ab + fx * x.ab + fyy * y.a * y.b + fxx * x.a * x.b + fxy * (y.a * x.b + x.a * y.b));
}
HD HyperDual acos(const HyperDual &x) {
    const float q = (1.0f - x.v) * (1.0f + x.v);  // 1 - x^2 without cancellation near |x| = 1
    const float iq = 1.0f / sqrtf(q);
    return chain(x, acosf(x.v), -iq, -x.v * iq / q);
}
HD HyperDual fabs(const HyperDual &x) { return x.v >= 0.0f ? x : -x; }
HD HyperDual fmax(const HyperDual &x, float c) { return x.v >= c ? x : HyperDual(c); }
HD float sqrt(float x) { return sqrtf(x); }
HD float sin(float x) { return sinf(x); }
HD float cos(float x) { return cosf(x); }
HD float log(float x) { return logf(x); }
HD float exp(float x) { return expf(x); }
HD float fabs(float x) { return fabsf(x); }
HD float atan2(float y, float x) { return atan2f(y, x); }
HD float acos(float x) { return acosf(x); }
HD float fmax(float x, float c) { return fmaxf(x, c); }
HD float val(const HyperDual &x) { return x.v; }
HD float val(float x) { return x; }
HD float pow(float x, float e) { return powf(x, e); }

template <class T> using TV3 = Vec3<T>;

template <class T> HD T tlen(const TV3<T> &v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
template <class T> HD TV3<T> tnorm(const TV3<T> &v) { T il = 1.0f / tlen(v); return v * il; }
template <class T> HD TV3<T> tv(const V3 &v) { return TV3<T>(T(v.x), T(v.y), T(v.z)); }
template <class T> HD TV3<T> treflect(const TV3<T> &wi, const TV3<T> &n) { return (2.0f * dot(wi, n)) * n - wi; }
template <class T> HD T tmis(const T &x) { return x * x; }
template <class T> HD T tlum(const TV3<T> &v) { return v.x * 0.212671f + v.y * 0.715160f + v.z * 0.072169f; }

template <class T>
HD void tframe(const TV3<T> &n, TV3<T> &b1, TV3<T> &b2) {
    if (val(n.z) < float(-1.0 + 1e-6)) {
        b1 = TV3<T>(T(0.0f), T(-1.0f), T(0.0f));
        b2 = TV3<T>(T(-1.0f), T(0.0f), T(0.0f));
        return;
    }
    const T a = 1.0f / (1.0f + n.z);
    const T b = -n.x * n.y * a;
    b1 = TV3<T>(1.0f - n.x * n.x * a, b, -n.x);
    b2 = TV3<T>(b, 1.0f - n.y * n.y * a, -n.y);
}

template <class T>
HD TV3<T> tcos_hemisphere(const T &u0, const T &u1) {
    const T phi = kTwoPi * u0;
    const T tmp = sqrt(fmax(1.0f - u1, 1e-6f));
    return TV3<T>(cos(phi) * tmp, sin(phi) * tmp, sqrt(fmax(u1, 1e-6f)));
}

template <class T>
struct TIsect {
    TV3<T> position, shadingNormal, geomNormal;
};

template <class T>
struct TState {
    TIsect<T> isect;
    TV3<T> wi;
    T prev, cur;  // accMISWPrev, accMISWThis
    TV3<T> throughput;
};

template <class T>
struct TBsdf {
    TV3<T> contrib;
    T cosWo, pdf, revPdf;
};

// ---------------------------------------------------------------- rough dielectric (AD forms)
// BeckmennDistributionTerm (src/microfacet.h:6-18) with a constant or a path-dependent roughness.
template <class T, class A>
DEV T ad_beckmann_d(const TV3<T> &h, const A &alpha) {
    const T cosTheta2 = h.z * h.z;
    const T e = (h.x * h.x / (alpha * alpha) + h.y * h.y / (alpha * alpha)) / cosTheta2;
    return exp(-e) / (kPi * alpha * alpha * (cosTheta2 * cosTheta2));
}

// The AD BeckmennGeometryTerm (src/microfacet.h:40-60): 1 + 1e-6 under the root.
template <class T>
DEV T ad_beckmann_g1(float alpha, const T &cosTheta) {
    const T tanTheta = sqrt(fabs((1.0f + 1e-6f) - cosTheta * cosTheta)) / cosTheta;
    if (val(tanTheta) <= 0.0f) return T(1.0f);
    const T a = 1.0f / (alpha * tanTheta);
    if (val(a) >= 1.6f) return T(1.0f);
    const T a2 = a * a;
    return (3.535f * a + 2.181f * a2) / (1.0f + 2.276f * a + 2.577f * a2);
}

// The AD FresnelDielectricExt (src/microfacet.h:117-145).
template <class T>
DEV T ad_fresnel(const T &cosThetaI_, T &cosThetaT_, float eta, float invEta) {
    const float scale = val(cosThetaI_) > 0.0f ? invEta : eta;
    const T cosThetaTSqr = 1.0f - (1.0f - cosThetaI_ * cosThetaI_) * (scale * scale);
    if (val(cosThetaTSqr) <= 0.0f) {
        cosThetaT_ = T(0.0f);
        return T(1.0f);
    }
    const T cosThetaI = fabs(cosThetaI_);
    const T cosThetaT = sqrt(cosThetaTSqr);
    const T etaCosThetaT = eta * cosThetaT;
    const T etaCosThetaI = eta * cosThetaI;
    const T Rs = (cosThetaI - etaCosThetaT) / (cosThetaI + etaCosThetaT);
    const T Rp = (etaCosThetaI - cosThetaT) / (etaCosThetaI + cosThetaT);
    cosThetaT_ = val(cosThetaI_) > 0.0f ? -cosThetaT : cosThetaT;
    return 0.5f * (Rs * Rs + Rp * Rp);
}

// EvaluateRoughDielectric (src/roughdielectric.cpp:284-374).
template <class T>
DEV void ad_rough_dielectric_evaluate(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const TV3<T> &wo,
                                      TBsdf<T> &o, bool adjoint) {
    const T cosWi = dot(wi, normal);
    o.cosWo = dot(wo, normal);
    const T cosWo = o.cosWo;
    const bool reflect = val(cosWi) * val(cosWo) > 0.0f;
    const float eta_ = val(cosWi) > 0.0f ? b.eta : b.invEta;
    const float revEta_ = val(cosWo) > 0.0f ? b.eta : b.invEta;
    TV3<T> H = reflect ? tnorm(TV3<T>(wi + wo)) : tnorm(TV3<T>(wi + wo * eta_));
    if (val(dot(H, normal)) < 0.0f) H = -H;
    const T cosHWi = dot(wi, H), cosHWo = dot(wo, H);
    TV3<T> b0, b1;
    tframe(normal, b0, b1);
    const TV3<T> localH(dot(b0, H), dot(b1, H), dot(normal, H));
    const float alpha = b.alpha;
    const T D = ad_beckmann_d(localH, alpha);
    const T revCosHWi = cosHWo, revCosHWo = cosHWi;
    T ct;
    const T F = ad_fresnel(cosHWi, ct, b.eta, b.invEta);
    const T aCosWi = fabs(cosWi), aCosWo = fabs(cosWo);
    const T G = ad_beckmann_g1(alpha, aCosWi) * ad_beckmann_g1(alpha, aCosWo);
    const T scaledAlpha = alpha * (1.2f - 0.2f * sqrt(aCosWi));
    const T prob = localH.z * ad_beckmann_d(localH, scaledAlpha);
    const T revScaledAlpha = alpha * (1.2f - 0.2f * sqrt(aCosWo));
    const T revProb = localH.z * ad_beckmann_d(localH, revScaledAlpha);
    if (reflect) {
        const T scalar = fabs(F * D * G / (4.0f * cosWi));
        o.contrib = tv<T>(ks_of(b)) * scalar;
        o.pdf = fabs(prob * F / (4.0f * cosHWo));
        o.revPdf = fabs(revProb * F / (4.0f * revCosHWo));
    } else {
        const T sqrtDenom = cosHWi + eta_ * cosHWo;
        const T revSqrtDenom = revCosHWi + revEta_ * revCosHWo;
        const float factor = adjoint ? 1.0f : (1.0f / eta_) * (1.0f / eta_);
        const T scalar = fabs(factor * ((1.0f - F) * D * G * (eta_ * eta_) * cosHWi * cosHWo) /
                              (cosWi * (sqrtDenom * sqrtDenom)));
        o.contrib = tv<T>(kt_of(b)) * scalar;
        o.pdf = fabs(prob * (1.0f - F) * ((eta_ * eta_) * cosHWo) / (sqrtDenom * sqrtDenom));
        o.revPdf = fabs(revProb * (1.0f - F) * ((revEta_ * revEta_) * revCosHWo) / (revSqrtDenom * revSqrtDenom));
    }
}

// SampleRoughDielectric with fixDiscrete = false (src/roughdielectric.cpp:376-481).
template <class T>
DEV void ad_rough_dielectric_sample(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const T &r0, const T &r1,
                                    float uDiscrete, TV3<T> &wo, TBsdf<T> &o, bool adjoint) {
    const T cosWi = dot(wi, normal);
    const float alpha = b.alpha;
    const T scaledAlpha = alpha * (1.2f - 0.2f * sqrt(fabs(cosWi)));
    // SampleMicronormal (src/microfacet.h:166-185), AD form (1e-6 floor on sin^2)
    const T phiM = kTwoPi * r1;
    const T alphaSqr = scaledAlpha * scaledAlpha;
    const T tanThetaMSqr = alphaSqr * (-log(fmax(1.0f - r0, 1e-6f)));
    const T cosThetaM = 1.0f / sqrt(1.0f + tanThetaMSqr);
    const T cosThetaMSqr = cosThetaM * cosThetaM;
    const T mPdf = (1.0f - r0) / (kPi * alphaSqr * cosThetaM * cosThetaMSqr);
    const T sinThetaM = sqrt(fmax(1.0f - cosThetaMSqr, 1e-6f));
    const TV3<T> localH(sinThetaM * cos(phiM), sinThetaM * sin(phiM), cosThetaM);
    TV3<T> b0, b1;
    tframe(normal, b0, b1);
    const TV3<T> H = localH.x * b0 + localH.y * b1 + localH.z * normal;
    const T cosHWi = dot(wi, H);
    T cosThetaT;
    const T F = ad_fresnel(cosHWi, cosThetaT, b.eta, b.invEta);
    TV3<T> refl;
    if (uDiscrete <= val(F)) {
        wo = treflect(wi, H);
        refl = tv<T>(ks_of(b));
        const T cosHWo = dot(wo, H);
        o.pdf = fabs(mPdf * F / (4.0f * cosHWo));
        const T rev_dwh_dwo = 1.0f / (4.0f * cosHWi);
        o.cosWo = dot(wo, normal);
        const T revScaledAlp = alpha * (1.2f - 0.2f * sqrt(fabs(o.cosWo)));
        o.revPdf = fabs(F * ad_beckmann_d(localH, revScaledAlp) * localH.z * rev_dwh_dwo);
    } else {
        const float etaR = val(cosThetaT) < 0.0f ? b.invEta : b.eta;  // Refract (src/utils.h:202-210)
        wo = H * (dot(wi, H) * etaR + cosThetaT) - wi * etaR;
        const float eta_ = val(cosWi) > 0.0f ? b.eta : b.invEta;
        const float factor = adjoint ? 1.0f : (1.0f / eta_) * (1.0f / eta_);
        refl = tv<T>(kt_of(b) * factor);
        const T cosHWo = dot(wo, H);
        const T sqrtDenom = cosHWi + eta_ * cosHWo;
        const T dwh_dwo = ((eta_ * eta_) * cosHWo) / (sqrtDenom * sqrtDenom);
        o.pdf = fabs(mPdf * (1.0f - F) * fabs(dwh_dwo));
        o.cosWo = dot(wo, normal);
        const float revEta_ = val(o.cosWo) > 0.0f ? b.eta : b.invEta;
        const T revSqrtDenom = cosHWo + revEta_ * cosHWi;
        const T rev_dwh_dwo = ((revEta_ * revEta_) * cosHWi) / (revSqrtDenom * revSqrtDenom);
        const T revScaledAlp = alpha * (1.2f - 0.2f * sqrt(fabs(o.cosWo)));
        o.revPdf = fabs((1.0f - F) * ad_beckmann_d(localH, revScaledAlp) * localH.z * rev_dwh_dwo);
    }
    const T aCosWi = fabs(cosWi), aCosWo = fabs(o.cosWo);
    const T D = ad_beckmann_d(localH, alpha);
    const T G = ad_beckmann_g1(alpha, aCosWi) * ad_beckmann_g1(alpha, aCosWo);
    o.contrib = refl * fabs(D * G * cosHWi / (mPdf * aCosWi));
}

// EvaluateLambertian / EvaluatePhong / EvaluateRoughDielectric (AD forms);
// adjoint selects EvaluateBSDF(true, ...) where the BSDF distinguishes it.
template <class T>
DEV void ad_evaluate(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const TV3<T> &wo, TBsdf<T> &o,
                     bool adjoint = false) {
    if (b.type == kBsdfRoughDielectric) {
        ad_rough_dielectric_evaluate(b, wi, normal, wo, o, adjoint);
        return;
    }
    T cosWi = dot(normal, wi);
    TV3<T> n = normal;
    if (!(val(cosWi) > 0.0f)) {
        n = -normal;
        cosWi = -cosWi;
    }
    o.cosWo = dot(n, wo);
    const V3 kd = kd_of(b);
    if (b.type == kBsdfLambertian) {
        const T fwd = o.cosWo * kInvPi;
        o.contrib = fwd * tv<T>(kd);
        o.pdf = fwd;
        o.revPdf = cosWi * kInvPi;
        return;
    }
    TV3<T> spec(T(0.0f), T(0.0f), T(0.0f));
    T specPdf(0.0f);
    if (b.ksWeight > 0.0f) {
        const T alpha = dot(treflect(wi, n), wo);
        const float wv = powf(val(alpha), b.exponent) * kInvTwoPi;
        if (wv > 1e-10f) {
            const T weight = pow(alpha, b.exponent) * kInvTwoPi;
            spec = tv<T>(ks_of(b)) * ((b.exponent + 2.0f) * weight);
            specPdf = b.ksWeight * (b.exponent + 1.0f) * weight;
        }
    }
    o.contrib = spec;
    o.pdf = specPdf;
    o.revPdf = specPdf;
    if (b.ksWeight < 1.0f) {
        const float tmp = (1.0f - b.ksWeight) * kInvPi;
        o.contrib = o.contrib + tv<T>(kd * kInvPi);
        o.pdf = o.pdf + tmp * o.cosWo;
        o.revPdf = o.revPdf + tmp * cosWi;
    }
    o.contrib = o.contrib * o.cosWo;
}

// SampleLambertian / SamplePhong / SampleRoughDielectric (AD forms, fixDiscrete = false).
template <class T>
DEV void ad_sample(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const T &r0, const T &r1, float uDiscrete,
                   TV3<T> &wo, TBsdf<T> &o, bool adjoint = false) {
    if (b.type == kBsdfRoughDielectric) {
        ad_rough_dielectric_sample(b, wi, normal, r0, r1, uDiscrete, wo, o, adjoint);
        return;
    }
    T cosWi = dot(wi, normal);
    TV3<T> n = normal;
    if (!(val(cosWi) > 0.0f)) {
        n = -normal;
        cosWi = -cosWi;
    }
    if (b.type == kBsdfLambertian) {
        TV3<T> b0, b1;
        tframe(n, b0, b1);
        const TV3<T> l = tcos_hemisphere(r0, r1);
        wo = l.x * b0 + l.y * b1 + l.z * n;
        o.cosWo = l.z;
        o.pdf = l.z * kInvPi;
        o.contrib = tv<T>(kd_of(b));
        o.revPdf = cosWi * kInvPi;
        return;
    }
    const TV3<T> R = treflect(wi, n);
    if (uDiscrete > b.ksWeight) {
        const TV3<T> l = tcos_hemisphere(r0, r1);
        TV3<T> b0, b1;
        tframe(n, b0, b1);
        wo = l.x * b0 + l.y * b1 + l.z * n;
    } else {
        const float power = 1.0f / (b.exponent + 1.0f);
        const T cosAlpha = pow(r1, power);
        const T sinAlpha = sqrt(fmax(1.0f - cosAlpha * cosAlpha, 1e-6f));
        const T phi = kTwoPi * r0;
        const TV3<T> l(sinAlpha * cos(phi), sinAlpha * sin(phi), cosAlpha);
        TV3<T> b0, b1;
        tframe(R, b0, b1);
        wo = l.x * b0 + l.y * b1 + l.z * R;
    }
    o.cosWo = dot(n, wo);
    TV3<T> spec(T(0.0f), T(0.0f), T(0.0f));
    T specPdf(0.0f);
    if (b.ksWeight > 0.0f) {
        const T alpha = dot(R, wo);
        const float wv = powf(val(alpha), b.exponent) * kInvTwoPi;
        if (wv > 1e-10f) {
            const T weight = pow(alpha, b.exponent) * kInvTwoPi;
            spec = tv<T>(ks_of(b)) * ((b.exponent + 2.0f) * weight);
            specPdf = b.ksWeight * (b.exponent + 1.0f) * weight;
        }
    }
    o.contrib = spec;
    o.pdf = specPdf;
    o.revPdf = specPdf;
    if (b.ksWeight < 1.0f) {
        const float tmp = (1.0f - b.ksWeight) * kInvPi;
        o.contrib = o.contrib + tv<T>(kd_of(b) * kInvPi);
        o.pdf = o.pdf + tmp * o.cosWo;
        o.revPdf = o.revPdf + tmp * cosWi;
    }
    o.contrib = o.contrib * o.cosWo;
    o.contrib = o.contrib * (1.0f / o.pdf);
}

template <class T>
DEV T ad_snc(const TV3<T> &wi, const TIsect<T> &is, const TV3<T> &wo) {
    const T cosWi = dot(is.shadingNormal, wi);
    const T cosWo = dot(is.shadingNormal, wo);
    const T wiDotGeoN = dot(is.geomNormal, wi);
    const T woDotGeoN = dot(is.geomNormal, wo);
    return fabs((woDotGeoN * cosWi) / (wiDotGeoN * cosWo));
}

// IntersectTriangleMesh (AD, static) on a known triangle.
template <class T>
DEV void ad_intersect(const SceneView &s, int tri, const TV3<T> &org, const TV3<T> &dir, TIsect<T> &is) {
    const float *P = s.triP + 9 * tri;
    const V3 p0 = ld3(P), e1 = ld3(P + 3), e2 = ld3(P + 6);
    const float *N = s.triN + 9 * tri;
    const V3 gn = normalize(cross(e1, e2));
    is.geomNormal = tv<T>(gn);
    const TV3<T> E1 = tv<T>(e1), E2 = tv<T>(e2);
    const TV3<T> s1 = cross(dir, E2);
    const T divisor = dot(s1, E1);
    const T invDivisor = 1.0f / divisor;
    const TV3<T> sv = org - tv<T>(p0);
    const T u = dot(sv, s1) * invDivisor;
    const TV3<T> s2 = cross(sv, E1);
    const T v = dot(dir, s2) * invDivisor;
    const T t = dot(E2, s2) * invDivisor;
    const T w = 1.0f - u - v;
    is.position = org + t * dir;
    is.shadingNormal = tnorm(TV3<T>(w * tv<T>(ld3(N)) + u * tv<T>(ld3(N + 3)) + v * tv<T>(ld3(N + 6))));
}

// SampleShape (AD) on a triangle: a = sqrt((1 + 1e-6) - r0).
template <class T>
DEV void ad_sample_triangle(const SceneView &s, int tri, const T &r0, const T &r1, TV3<T> &pos, TV3<T> &normal) {
    const float *P = s.triP + 9 * tri;
    const float *N = s.triN + 9 * tri;
    const T a = sqrt((1.0f + 1e-6f) - r0);
    const T b1 = 1.0f - a;
    const T b2 = a * r1;
    pos = tv<T>(ld3(P)) + (tv<T>(ld3(P + 3)) * b1) + (tv<T>(ld3(P + 6)) * b2);
    normal = tnorm(TV3<T>(tv<T>(ld3(N)) * (1.0f - b1 - b2) + tv<T>(ld3(N + 3)) * b1 + tv<T>(ld3(N + 6)) * b2));
}

template <class T>
DEV TV3<T> ad_xform_point(const float *m, const TV3<T> &p) {
    const T x = m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3];
    const T y = m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7];
    const T z = m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11];
    const T w = m[12] * p.x + m[13] * p.y + m[14] * p.z + m[15];
    const T invW = 1.0f / w;
    return TV3<T>(x * invW, y * invW, z * invW);
}
template <class T>
DEV TV3<T> ad_xform_vector(const float *m, const TV3<T> &v) {
    return TV3<T>(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                  m[8] * v.x + m[9] * v.y + m[10] * v.z);
}
template <class T>
DEV void ad_sample_primary(const Camera &c, const T &sx, const T &sy, TV3<T> &org, TV3<T> &dir) {
    const TV3<T> o = ad_xform_point(c.sampleToCam, TV3<T>(sx, sy, T(0.0f)));
    const TV3<T> d = tnorm(o);
    org = ad_xform_point(c.camToWorld, TV3<T>(T(0.0f), T(0.0f), T(0.0f)));
    dir = ad_xform_vector(c.camToWorld, d);
}

// ---------------------------------------------------------------- environment light (AD)
// The forms of src/envlight.cpp:249-400 on the pixel the value part selects:
// the cell's CDF bounds, image values and row weights are constants and the
// derivatives flow through the cell-local coordinates. Image lookups use the
// primal's indexing (Image3::At for sampling, RepAt for emission) and the
// unwrapped column / row of the primal, so f is the primal's contribution;
// the light's sampling weight is kept as the primal keeps it.
template <class T>
HD T ad_tent(const T &u) { return val(u) < 0.5f ? 1.0f - sqrt(2.0f * u) : sqrt(2.0f * (u - 0.5f)) - 1.0f; }

template <class T>
DEV void ad_env_sample_direction(const SceneView &s, const T &u0, const T &u1, TV3<T> &dirToLight, TV3<T> &value,
                                 T &pdf) {
    float a = val(u0), b = val(u1);
    const int row = env_u_to_index(s.envCdfRows, s.envH, b);
    const float *cc = s.envCdfCols + row * (s.envW + 1);
    const int col = env_u_to_index(cc, s.envW, a);
    const float cr0 = __ldg(s.envCdfRows + row), cr1 = __ldg(s.envCdfRows + row + 1);
    const float cc0 = __ldg(cc + col), cc1 = __ldg(cc + col + 1);
    const T t0 = ad_tent<T>((u0 - cc0) / (cc1 - cc0));
    const T t1 = ad_tent<T>((u1 - cr0) / (cr1 - cr0));
    const T phi = (t0 + float(col) + 0.5f) * s.envPix[0];
    const T theta = (t1 + float(row) + 0.5f) * s.envPix[1];
    const T sinPhi = sin(phi), cosPhi = cos(phi), sinTheta = sin(theta), cosTheta = cos(theta);
    const TV3<T> d(sinPhi * sinTheta, cosTheta, -cosPhi * sinTheta);
    const float *m = s.envToWorld;
    dirToLight = TV3<T>(m[0] * d.x + m[1] * d.y + m[2] * d.z, m[3] * d.x + m[4] * d.y + m[5] * d.z,
                        m[6] * d.x + m[7] * d.y + m[8] * d.z);
    const T dx1 = t0, dx2 = 1.0f - t0, dy1 = t1, dy2 = 1.0f - t1;
    const TV3<T> value1 = tv<T>(env_at(s, col, row)) * (dx2 * dy2) + tv<T>(env_at(s, col + 1, row)) * (dx1 * dy2);
    const TV3<T> value2 =
        tv<T>(env_at(s, col, row + 1)) * (dx2 * dy1) + tv<T>(env_at(s, col + 1, row + 1)) * (dx1 * dy1);
    value = value1 + value2;
    pdf = (tlum(value1) * env_row_weight(s, row) + tlum(value2) * env_row_weight(s, row + 1)) * s.envNorm /
          fmax(fabs(sinTheta), 1e-7f);
}

template <class T>
DEV void ad_env_emission(const SceneView &s, const Light &L, const TV3<T> &dirToLight, TV3<T> &emission,
                         T &directPdf, T &emissionPdf) {
    const float *m = s.envToLight;
    const TV3<T> d(m[0] * dirToLight.x + m[1] * dirToLight.y + m[2] * dirToLight.z,
                   m[3] * dirToLight.x + m[4] * dirToLight.y + m[5] * dirToLight.z,
                   m[6] * dirToLight.x + m[7] * dirToLight.y + m[8] * dirToLight.z);
    const T uvx = atan2(d.x, -d.z) * kInvTwoPi * float(s.envW) - 0.5f;
    const T uvy = acos(d.y) * kInvPi * float(s.envH) - 0.5f;
    const int col = int(floorf(val(uvx)));
    const int row = int(floorf(val(uvy)));
    const T dx1 = uvx - float(col), dx2 = 1.0f - dx1, dy1 = uvy - float(row), dy2 = 1.0f - dy1;
    const TV3<T> value1 =
        tv<T>(env_rep_at(s, col, row)) * (dx2 * dy2) + tv<T>(env_rep_at(s, col + 1, row)) * (dx1 * dy2);
    const TV3<T> value2 =
        tv<T>(env_rep_at(s, col, row + 1)) * (dx2 * dy1) + tv<T>(env_rep_at(s, col + 1, row + 1)) * (dx1 * dy1);
    emission = (value1 + value2) * L.samplingWeight;
    // EmissionEnvLight's clamp against infinite derivatives at the poles
    // (src/envlight.cpp:353); 1 - y^2 as (1 - y)(1 + y), which keeps its digits
    // (and its second derivative) in single precision as |y| approaches 1
    const T sinTheta = sqrt(fmax((1.0f - d.y) * (1.0f + d.y), 1e-6f));
    directPdf = (tlum(value1) * env_row_weight(s, row) + tlum(value2) * env_row_weight(s, row + 1)) * s.envNorm /
                fmax(fabs(sinTheta), 1e-7f);
    emissionPdf = directPdf * env_position_pdf(s);
}

template <class T>
HD void ad_concentric_disc(const T &u0, const T &u1, T &x, T &y) {
    const T r1 = 2.0f * u0 - 1.0f;
    const T r2 = 2.0f * u1 - 1.0f;
    T r, phi;
    if (val(r1) == 0.0f || val(r2) == 0.0f) {
        r = T(0.0f);
        phi = T(0.0f);
    } else if (val(r1) * val(r1) > val(r2) * val(r2)) {
        r = r1;
        phi = kPiOverFour * (r2 / r1);
    } else {
        r = r2;
        phi = kPiOverTwo - (r1 / r2) * kPiOverFour;
    }
    x = r * cos(phi);
    y = r * sin(phi);
}

// BSDFSampling<adjoint, false> (AD, src/path.cpp:2671-2762).
template <class T, bool adjoint>
DEV void ad_bsdf_sampling(const SceneView &s, int tri, const T &r0, const T &r1, float disc, bool useAbs,
                          int lcsTri, TState<T> &ps, TV3<T> &dir) {
    const Bsdf &b = bsdf_of_tri(s, tri);
    TBsdf<T> o;
    T jacobian(1.0f);
    if (lcsTri >= 0) {
        TV3<T> nextPos, nextNormal;
        ad_sample_triangle(s, lcsTri, r0, r1, nextPos, nextNormal);
        const float shapePdf = s.lights[area_light_of_tri(s, lcsTri)].invTotalArea;
        dir = nextPos - ps.isect.position;
        const T distSq = dot(dir, dir);
        const T invDistSq = 1.0f / distSq;
        const T invDist = sqrt(invDistSq);
        dir = dir * invDist;
        ad_evaluate(b, ps.wi, ps.isect.shadingNormal, dir, o);
        jacobian = fabs(dot(nextNormal, dir) * invDistSq) / shapePdf;
    } else if (!useAbs) {
        ad_sample(b, ps.wi, ps.isect.shadingNormal, r0, r1, disc, dir, o, adjoint);
    } else {
        const T scaledTheta = kTwoPi * r0;
        const T scaledPhi = kPi * r1;
        const T sinPhi = sin(scaledPhi);
        const T cosPhi = cos(scaledPhi);
        jacobian = fabs(sinPhi);
        dir = TV3<T>(sinPhi * cos(scaledTheta), sinPhi * sin(scaledTheta), cosPhi);
        ad_evaluate(b, ps.wi, ps.isect.shadingNormal, dir, o, adjoint);
    }
    TV3<T> contrib = o.contrib;
    if (adjoint) contrib = contrib * ad_snc(ps.wi, ps.isect, dir);
    contrib = contrib * jacobian;
    ps.cur = tmis(o.cosWo / o.pdf) * (ps.cur * tmis(o.revPdf) + ps.prev);
    ps.prev = tmis(1.0f / o.pdf);
    ps.throughput = cmul(ps.throughput, contrib);
}

// Evaluates f = log Luminance(contribution) of technique path `r` at primary
// vector u (length 2(c+l-1), GetPathPos order) the way the generated
// evaluate_path_bidir_<c>_<l>_static does.
template <class T>
DEV T ad_eval_path(const SceneView &s, const PathRec &r, const T *u) {
    const int c = r.c, l = r.l;
    const int nl = n_lgt(l), nc = c - 1;
    const float pixelCount = float(s.cam.width * s.cam.height);
    int k = 0;
    TState<T> lp;
    TV3<T> contrib(T(0.0f), T(0.0f), T(0.0f));
    int lgtVertTri = -1;
    if (l > 1) {
        const int li = r.lgtLight;
        const Light &L = s.lights[li];
        const float pick = pick_light_prob(s, li);
        const T p0 = u[k++], p1 = u[k++], d0 = u[k++], d1 = u[k++];
        TV3<T> org, dir;
        T cosLight, emissionPdf, directPdf;
        if (L.type == kLightArea) {  // EmitAreaLight (AD)
            TV3<T> nrm;
            ad_sample_triangle(s, light_tri(s, L, r.lgtPrim), p0, p1, org, nrm);
            const TV3<T> d = tcos_hemisphere(d0, d1);
            TV3<T> b0, b1;
            tframe(nrm, b0, b1);
            dir = d.x * b0 + d.y * b1 + d.z * nrm;
            lp.throughput = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]) * (kPi / L.invTotalArea));
            cosLight = d.z;
            emissionPdf = d.z * kInvPi * L.invTotalArea;
            directPdf = T(L.invTotalArea);
        } else if (L.type == kLightEnv) {  // EmitEnvLight (AD)
            TV3<T> value;
            ad_env_sample_direction(s, d0, d1, dir, value, directPdf);
            lp.throughput = value * L.samplingWeight;
            dir = -dir;
            T ox, oy;
            ad_concentric_disc(p0, p1, ox, oy);
            TV3<T> b0, b1;
            tframe(dir, b0, b1);
            const TV3<T> perp = ox * b0 + oy * b1;
            org = tv<T>(V3(s.bsCenter[0], s.bsCenter[1], s.bsCenter[2])) + (perp - dir) * s.bsRadius;
            cosLight = T(1.0f);
            emissionPdf = directPdf * env_position_pdf(s);
        } else {  // EmitPointLight (AD)
            org = tv<T>(V3(L.pos[0], L.pos[1], L.pos[2]));
            const T scaledTheta = kTwoPi * d0;
            const T scaledPhi = kPi * d1;
            const T sinPhi = sin(scaledPhi);
            dir = TV3<T>(sinPhi * cos(scaledTheta), sinPhi * sin(scaledTheta), cos(scaledPhi));
            lp.throughput = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]));
            emissionPdf = T(1.0f / (4.0f * kPi));
            cosLight = T(1.0f);
            directPdf = T(1.0f);
        }
        emissionPdf = emissionPdf * pick;
        directPdf = directPdf * pick;
        lp.throughput = lp.throughput * (1.0f / pick);
        lp.prev = tmis(directPdf / emissionPdf);
        lp.cur = L.type == kLightPoint ? tmis(cosLight / emissionPdf) : T(0.0f);
        #pragma unroll 1
        for (int d = 0; d < nl; d++) {
            const int tri = r.tri[d];
            ad_intersect(s, tri, org, dir, lp.isect);
            lp.wi = -dir;
            if (d == 0) {  // ConvertMISLightEmit
                const T conv = L.type == kLightEnv ? T(1.0f) : tmis(dot(org - lp.isect.position, org - lp.isect.position));
                const T invCos = 1.0f / tmis(fabs(dot(dir, lp.isect.shadingNormal)));
                lp.prev = lp.prev * (invCos * conv);
                lp.cur = lp.cur * invCos;
            } else {
                lp.prev = lp.prev * tmis(dot(org - lp.isect.position, org - lp.isect.position));
                const T invCos = 1.0f / tmis(fabs(dot(dir, lp.isect.shadingNormal)));
                lp.prev = lp.prev * invCos;
                lp.cur = lp.cur * invCos;
            }
            if (d == nl - 1) {
                if (c == 1) {  // ConnectToCamera (AD)
                    TV3<T> camOrg, camDir;
                    ad_sample_primary(s.cam, T(0.5f), T(0.5f), camOrg, camDir);
                    TV3<T> dirToCamera = camOrg - lp.isect.position;
                    const T distSq = dot(dirToCamera, dirToCamera);
                    const T dist = sqrt(distSq);
                    dirToCamera = dirToCamera * (1.0f / dist);
                    TBsdf<T> o;
                    ad_evaluate(bsdf_of_tri(s, tri), lp.wi, lp.isect.shadingNormal, dirToCamera, o, true);
                    const TV3<T> bsdfContrib = o.contrib * ad_snc(lp.wi, lp.isect, dirToCamera);
                    const T invCosAtCamera = -(1.0f / dot(camDir, dirToCamera));
                    const T ip = s.cam.dist * invCosAtCamera;
                    const T imageToSolidAngleFactor = (ip * ip) * invCosAtCamera;
                    const T imageToSurfaceFactor = imageToSolidAngleFactor * fabs(o.cosWo) / distSq;
                    const T wLight = tmis(imageToSurfaceFactor / pixelCount) * (lp.prev + lp.cur * tmis(o.revPdf));
                    const T misWeight = 1.0f / (wLight + 1.0f);
                    const T surfaceToImageFactor = o.cosWo / imageToSurfaceFactor;
                    const T denom = pixelCount * surfaceToImageFactor;
                    const TV3<T> cc = (misWeight * bsdfContrib) * (1.0f / denom);
                    contrib = cmul(cc, lp.throughput);
                }
                lgtVertTri = tri;
                break;
            }
            const T r0 = u[k++], r1 = u[k++];
            ad_bsdf_sampling<T, true>(s, tri, r0, r1, r.disc[d], (r.useAbs >> d) & 1u, -1, lp, dir);
            lp.throughput = lp.throughput * r.rr[d];
            org = lp.isect.position;
        }
    }
    if (c > 1) {
        const T sx = u[k++], sy = u[k++];
        TV3<T> co, cd, org, dir;
        ad_sample_primary(s.cam, T(0.5f), T(0.5f), co, cd);
        ad_sample_primary(s.cam, sx, sy, org, dir);
        TState<T> cp;
        {
            const T cosAtCamera = dot(cd, dir);
            const T ip = s.cam.dist / cosAtCamera;
            const T cameraPdf = (ip * ip) / cosAtCamera;
            cp.throughput = TV3<T>(T(1.0f), T(1.0f), T(1.0f));
            cp.prev = tmis(pixelCount / cameraPdf);
            cp.cur = T(0.0f);
        }
        #pragma unroll 1
        for (int d = 0; d < nc; d++) {
            const int vi = nl + d;
            const int tri = r.tri[vi];
            if (d == nc - 1 && l == 0 && tri < 0) {
                // the camera ray leaves the scene: ConvertMISLightHit leaves the MIS
                // terms as they are, HandleHitLight with EmissionEnvLight (AD)
                const Light &L = s.lights[s.envLight];
                TV3<T> emission;
                T directPdf, emissionPdf;
                ad_env_emission(s, L, dir, emission, directPdf, emissionPdf);
                cp.throughput = cmul(cp.throughput, emission);
                const float pick = pick_light_prob(s, s.envLight);
                directPdf = directPdf * pick;
                emissionPdf = emissionPdf * pick;
                const T wCamera = tmis(directPdf) * cp.prev + tmis(emissionPdf) * cp.cur;
                cp.throughput = cp.throughput * (1.0f / (1.0f + wCamera));
                contrib = cp.throughput;
                break;
            }
            ad_intersect(s, tri, org, dir, cp.isect);
            cp.wi = -dir;
            if (d == nc - 1 && l == 0) {
                // ConvertMISLightHit + HandleHitLight (AD)
                const int li = area_light_of_tri(s, tri);
                const Light &L = s.lights[li];
                const T dsq = tmis(dot(org - cp.isect.position, org - cp.isect.position));
                const T invCos = 1.0f / tmis(fabs(dot(dir, cp.isect.shadingNormal)));
                cp.prev = cp.prev * (invCos * dsq);
                cp.cur = cp.cur * invCos;
                const T cosAtLight = -dot(cp.isect.shadingNormal, dir);
                T directPdf(L.invTotalArea);
                T emissionPdf = cosAtLight * directPdf * kInvPi;
                cp.throughput = cmul(cp.throughput, tv<T>(V3(L.emission[0], L.emission[1], L.emission[2])));
                const float pick = pick_light_prob(s, li);
                directPdf = directPdf * pick;
                emissionPdf = emissionPdf * pick;
                const T wCamera = tmis(directPdf) * cp.prev + tmis(emissionPdf) * cp.cur;
                cp.throughput = cp.throughput * (1.0f / (1.0f + wCamera));
                contrib = cp.throughput;
                break;
            }
            cp.prev = cp.prev * tmis(dot(org - cp.isect.position, org - cp.isect.position));
            {
                const T invCos = 1.0f / tmis(fabs(dot(dir, cp.isect.shadingNormal)));
                cp.prev = cp.prev * invCos;
                cp.cur = cp.cur * invCos;
            }
            if (d == nc - 1) {
                const Bsdf &b = bsdf_of_tri(s, tri);
                if (l == 1) {  // DirectLighting (AD)
                    const T r0 = u[k++], r1 = u[k++];
                    const Light &L = s.lights[r.dlLight];
                    TV3<T> dirToLight, lightContrib;
                    T cosAtLight, directPdf, emissionPdf;
                    if (L.type == kLightArea) {
                        TV3<T> pl, nl2;
                        ad_sample_triangle(s, light_tri(s, L, r.dlPrim), r0, r1, pl, nl2);
                        dirToLight = pl - cp.isect.position;
                        const T distSq = dot(dirToLight, dirToLight);
                        const T dist = sqrt(distSq);
                        dirToLight = TV3<T>(dirToLight.x / dist, dirToLight.y / dist, dirToLight.z / dist);
                        cosAtLight = -dot(dirToLight, nl2);
                        directPdf = L.invTotalArea * distSq / cosAtLight;
                        const TV3<T> E = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]));
                        lightContrib = TV3<T>(E.x / directPdf, E.y / directPdf, E.z / directPdf);
                        emissionPdf = L.invTotalArea * cosAtLight * kInvPi;
                    } else if (L.type == kLightEnv) {  // SampleDirectEnvLight
                        TV3<T> value;
                        ad_env_sample_direction(s, r0, r1, dirToLight, value, directPdf);
                        lightContrib = value * (1.0f / directPdf) * L.samplingWeight;
                        cosAtLight = T(1.0f);
                        emissionPdf = directPdf * env_position_pdf(s);
                    } else {
                        dirToLight = tv<T>(V3(L.pos[0], L.pos[1], L.pos[2])) - cp.isect.position;
                        const T distSq = dot(dirToLight, dirToLight);
                        directPdf = distSq;
                        const T dist = sqrt(distSq);
                        dirToLight = TV3<T>(dirToLight.x / dist, dirToLight.y / dist, dirToLight.z / dist);
                        lightContrib = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2])) * (1.0f / distSq);
                        emissionPdf = T(1.0f / (4.0f * kPi));
                        cosAtLight = T(1.0f);
                    }
                    TBsdf<T> o;
                    ad_evaluate(b, cp.wi, cp.isect.shadingNormal, dirToLight, o);
                    const float pick = pick_light_prob(s, r.dlLight);
                    cp.throughput = cmul(cp.throughput, o.contrib);
                    cp.throughput = cmul(cp.throughput, lightContrib) * (1.0f / pick);
                    const T wLight = L.type == kLightPoint ? T(0.0f) : tmis(o.pdf / (pick * directPdf));
                    const T wCamera = tmis(emissionPdf * o.cosWo / (directPdf * cosAtLight)) * (cp.prev + cp.cur * tmis(o.revPdf));
                    cp.throughput = cp.throughput * (1.0f / (wLight + 1.0f + wCamera));
                } else {  // ConnectVertex (AD)
                    TV3<T> dirToLight = lp.isect.position - cp.isect.position;
                    const T distSq = dot(dirToLight, dirToLight);
                    const T dist = sqrt(distSq);
                    dirToLight = dirToLight * (1.0f / dist);
                    TBsdf<T> cb, lb;
                    ad_evaluate(b, cp.wi, cp.isect.shadingNormal, dirToLight, cb);
                    ad_evaluate(bsdf_of_tri(s, lgtVertTri), lp.wi, lp.isect.shadingNormal, -dirToLight, lb, true);
                    const TV3<T> lgtF = lb.contrib * ad_snc(lp.wi, lp.isect, -dirToLight);
                    const T G = 1.0f / distSq;
                    const T camA = cb.pdf * lb.cosWo * G;
                    const T lgtA = lb.pdf * cb.cosWo * G;
                    const T wLight = tmis(camA) * (lp.prev + lp.cur * tmis(lb.revPdf));
                    const T wCamera = tmis(lgtA) * (cp.prev + cp.cur * tmis(cb.revPdf));
                    const T misWeight = 1.0f / (wLight + 1.0f + wCamera);
                    cp.throughput = cmul(lp.throughput, cp.throughput);
                    cp.throughput = cmul(cp.throughput, cb.contrib);
                    cp.throughput = cmul(cp.throughput, lgtF) * (G * misWeight);
                }
                contrib = cp.throughput;
                break;
            }
            const T r0 = u[k++], r1 = u[k++];
            int lcsTri = -1;
            if (l == 0 && d == nc - 2 && s.opt.useLightCoordinateSampling) {
                const int lastTri = r.tri[nl + nc - 1];
                const int li = lastTri >= 0 ? area_light_of_tri(s, lastTri) : -1;
                if (li >= 0 && s.lights[li].type == kLightArea) lcsTri = lastTri;
            }
            ad_bsdf_sampling<T, false>(s, tri, r0, r1, r.disc[vi], (r.useAbs >> vi) & 1u, lcsTri, cp, dir);
            cp.throughput = cp.throughput * r.rr[vi];
            org = cp.isect.position;
        }
    }
    return log(tlum(contrib));
}

}  // namespace drmlt
