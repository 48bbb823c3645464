// Reverse-mode derivatives of f(u) = log Luminance(contribution): a
// hand-written adjoint of the AD path function of pathad.cuh, with the
// Hessian by forward-over-reverse.
//
// The adjoint of every vertex operation is written out below (intersection,
// BSDF sampling and evaluation, emission, connections, the MIS recurrences);
// each recomputes its own intermediates from its inputs, and the path-level
// sweep keeps only the carried vertex state of each vertex (origin, direction,
// throughput and the two MIS accumulators) instead of a tape of operations:
// the backward sweep re-runs one vertex operation at a time from that
// checkpoint and pulls the adjoints through it.
//
// All of it is templated on the scalar. With T = Dual (a value and one
// tangent) seeded in u_i, the forward sweep carries d/du_i and the backward
// sweep, run in Dual arithmetic, yields the gradient (values) and row i of the
// Hessian (tangents) in one forward and one backward pass: D passes for the
// whole Hessian of a path of dimension D, against the D(D+1)/2 hyper-dual
// evaluations of pathad.cuh. Branches are taken on values, as the primal and
// chad's generated code take them (src/chad.cpp:70-110), so every direction
// follows the same control flow and a team of threads (one direction each)
// stays converged.
//
// Reference: the chad library builds the same pair, a reverse pass over the
// generated path function and forward-over-reverse for the Hessian
// (src/chad.cpp:342-418, 492-552), from a recorded expression graph; the
// function differentiated is RegisterPathFuncBidir's (src/path.cpp:2987-3175).
#pragma once
#include "pathad.cuh"

namespace drmlt {

// ---------------------------------------------------------------- Dual numbers
struct Dual {
    float v, d;
    HD Dual() {}
    HD explicit Dual(float x) : v(x), d(0.0f) {}
    HD Dual(float x, float dx) : v(x), d(dx) {}
};
HD Dual operator+(const Dual &x, const Dual &y) { return Dual(x.v + y.v, x.d + y.d); }
HD Dual operator-(const Dual &x, const Dual &y) { return Dual(x.v - y.v, x.d - y.d); }
HD Dual operator-(const Dual &x) { return Dual(-x.v, -x.d); }
HD Dual operator*(const Dual &x, const Dual &y) { return Dual(x.v * y.v, x.d * y.v + x.v * y.d); }
HD Dual operator*(const Dual &x, float s) { return Dual(x.v * s, x.d * s); }
HD Dual operator*(float s, const Dual &x) { return Dual(x.v * s, x.d * s); }
HD Dual operator+(const Dual &x, float s) { return Dual(x.v + s, x.d); }
HD Dual operator+(float s, const Dual &x) { return Dual(x.v + s, x.d); }
HD Dual operator-(const Dual &x, float s) { return Dual(x.v - s, x.d); }
HD Dual operator-(float s, const Dual &x) { return Dual(s - x.v, -x.d); }
HD Dual dchain(const Dual &x, float f, float d1) { return Dual(f, d1 * x.d); }
HD Dual inv(const Dual &x) {
    const float r = 1.0f / x.v;
    return Dual(r, -r * r * x.d);
}
HD Dual operator/(const Dual &x, const Dual &y) { return x * inv(y); }
HD Dual operator/(const Dual &x, float s) { return x * (1.0f / s); }
HD Dual operator/(float s, const Dual &y) { return s * inv(y); }
HD Dual sqrt(const Dual &x) {
    const float r = sqrtf(x.v);
    return dchain(x, r, 0.5f / r);
}
HD Dual sin(const Dual &x) {
    float s, c;
    sincosf(x.v, &s, &c);
    return dchain(x, s, c);
}
HD Dual cos(const Dual &x) {
    float s, c;
    sincosf(x.v, &s, &c);
    return dchain(x, c, -s);
}
HD Dual log(const Dual &x) { return dchain(x, logf(x.v), 1.0f / x.v); }
HD Dual pow(const Dual &x, float e) { return dchain(x, powf(x.v, e), e * powf(x.v, e - 1.0f)); }
HD Dual exp(const Dual &x) {
    const float e = expf(x.v);
    return dchain(x, e, e);
}
HD Dual atan2(const Dual &y, const Dual &x) {
    const float ir2 = 1.0f / (x.v * x.v + y.v * y.v);
    return Dual(atan2f(y.v, x.v), (x.v * y.d - y.v * x.d) * ir2);
}
HD Dual acos(const Dual &x) {
    const float q = (1.0f - x.v) * (1.0f + x.v);
    return dchain(x, acosf(x.v), -1.0f / sqrtf(q));
}
HD Dual fabs(const Dual &x) { return x.v >= 0.0f ? x : -x; }
HD Dual fmax(const Dual &x, float c) { return x.v >= c ? x : Dual(c); }
HD float val(const Dual &x) { return x.v; }

// Adjoint sign of fabs / activity of fmax at the value (the branch the primal took).
template <class T> HD float sgn_of(const T &x) { return val(x) >= 0.0f ? 1.0f : -1.0f; }
template <class T> HD bool fmax_active(const T &x, float c) { return val(x) >= c; }

template <class T> HD TV3<T> tzero() { return TV3<T>(T(0.0f), T(0.0f), T(0.0f)); }
template <class T> HD T tsq(const T &x) { return x * x; }

// ---------------------------------------------------------------- adjoints of vector helpers
// Accumulating form: every *_adj adds the input adjoints it produces.

// y = |v|
template <class T> DEV void tlen_adj(const TV3<T> &v, const T &yb, TV3<T> &vb) {
    const T il = 1.0f / tlen(v);
    vb = vb + v * (yb * il);
}
// y = v / |v| (tnorm)
template <class T> DEV void tnorm_adj(const TV3<T> &v, const TV3<T> &yb, TV3<T> &vb) {
    const T il = 1.0f / tlen(v);
    const TV3<T> y = v * il;
    vb = vb + (yb - y * dot(y, yb)) * il;
}
// y = tlum(v)
template <class T> DEV void tlum_adj(const T &yb, TV3<T> &vb) {
    vb = vb + TV3<T>(yb * 0.212671f, yb * 0.715160f, yb * 0.072169f);
}

// The adjoint of the path contribution that f = log Luminance(contrib) seeds.
template <class T> DEV TV3<T> logf_seed(const TV3<T> &contrib) {
    TV3<T> cb = tzero<T>();
    tlum_adj(1.0f / tlum(contrib), cb);
    return cb;
}

// tframe(n) -> (b1, b2), src/utils.h:222-232 as the AD builder writes it.
template <class T> DEV void tframe_adj(const TV3<T> &n, const TV3<T> &b1b, const TV3<T> &b2b, TV3<T> &nb) {
    if (val(n.z) < float(-1.0 + 1e-6)) return;  // constant frame
    const T a = 1.0f / (1.0f + n.z);
    const T bb = b1b.y + b2b.x;
    const T ab = -(n.x * n.x) * b1b.x - (n.y * n.y) * b2b.y - n.x * n.y * bb;
    nb.x = nb.x - 2.0f * n.x * a * b1b.x - b1b.z - n.y * a * bb;
    nb.y = nb.y - 2.0f * n.y * a * b2b.y - b2b.z - n.x * a * bb;
    nb.z = nb.z - a * a * ab;
}

// The frame product w = l.x b0 + l.y b1 + l.z F with (b0, b1) = tframe(F).
template <class T> DEV TV3<T> frame_apply(const TV3<T> &l, const TV3<T> &F) {
    TV3<T> b0, b1;
    tframe(F, b0, b1);
    return l.x * b0 + l.y * b1 + l.z * F;
}
template <class T> DEV void frame_apply_adj(const TV3<T> &l, const TV3<T> &F, const TV3<T> &wb, TV3<T> &lb, TV3<T> &Fb) {
    TV3<T> b0, b1;
    tframe(F, b0, b1);
    lb = lb + TV3<T>(dot(b0, wb), dot(b1, wb), dot(F, wb));
    Fb = Fb + wb * l.z;
    tframe_adj(F, wb * l.x, wb * l.y, Fb);
}

// tcos_hemisphere(u0, u1)
template <class T> DEV void tcos_hemisphere_adj(const T &u0, const T &u1, const TV3<T> &yb, T &u0b, T &u1b) {
    const T phi = kTwoPi * u0;
    const T c = cos(phi), s = sin(phi);
    const T q = 1.0f - u1;
    const T tmp = sqrt(fmax(q, 1e-6f));
    const T phib = tmp * (c * yb.y - s * yb.x);
    const T tmpb = c * yb.x + s * yb.y;
    u0b = u0b + kTwoPi * phib;
    if (fmax_active(q, 1e-6f)) u1b = u1b - tmpb * (0.5f / tmp);
    if (fmax_active(u1, 1e-6f)) u1b = u1b + yb.z * (0.5f / sqrt(u1));
}

// treflect(wi, n) = 2 (wi . n) n - wi
template <class T> DEV void treflect_adj(const TV3<T> &wi, const TV3<T> &n, const TV3<T> &Rb, TV3<T> &wib, TV3<T> &nb) {
    const T q = dot(wi, n);
    const T qb = 2.0f * dot(n, Rb);
    nb = nb + Rb * (2.0f * q) + wi * qb;
    wib = wib - Rb + n * qb;
}


// ---------------------------------------------------------------- BSDF adjoints
// Output adjoints of a BSDF evaluation or sample (TBsdf plus the sampled direction).
template <class T>
struct TBsdfAdj {
    TV3<T> contrib;
    T cosWo, pdf, revPdf;
    HD void zero() {
        contrib = tzero<T>();
        cosWo = pdf = revPdf = T(0.0f);
    }
};

// The BSDF adjoints below compute the forward outputs first and then ask the
// caller for their adjoints: obf(o, wo, wob) returns the adjoints of `o` and
// may add to wob, the adjoint of the direction wo. A caller that needs `o` to
// form them (the sampling step's MIS and throughput updates) gets it without
// a second forward evaluation; FixedOb serves callers that already know them.
template <class T>
struct FixedOb {
    TBsdfAdj<T> ob;
    DEV TBsdfAdj<T> operator()(const TBsdf<T> &, const TV3<T> &, TV3<T> &) const { return ob; }
};

// ad_beckmann_d(h, alpha), alpha a path-dependent roughness (a constant one
// passes T(alpha) and ignores alphab).
template <class T>
DEV void beckmann_d_adj(const TV3<T> &h, const T &alpha, const T &Db, TV3<T> &hb, T &alphab) {
    const T a2 = alpha * alpha;
    const T c2 = h.z * h.z;
    const T s = h.x * h.x / a2 + h.y * h.y / a2;
    const T e = s / c2;
    const T ex = exp(-e);
    const T den = kPi * a2 * (c2 * c2);
    const T D = ex / den;
    const T exb = Db / den;
    const T denb = -Db * D / den;
    const T eb = -ex * exb;
    const T sb = eb / c2;
    T c2b = -eb * e / c2 + denb * kPi * a2 * (2.0f * c2);
    alphab = alphab + denb * kPi * (2.0f * alpha) * (c2 * c2) - sb * (2.0f * s / alpha);
    hb.x = hb.x + sb * (2.0f * h.x / a2);
    hb.y = hb.y + sb * (2.0f * h.y / a2);
    hb.z = hb.z + c2b * (2.0f * h.z);
}

// ad_beckmann_g1(alpha, cosTheta)
template <class T>
DEV void beckmann_g1_adj(float alpha, const T &c, const T &Gb, T &cb) {
    const T q = (1.0f + 1e-6f) - c * c;
    const T r = sqrt(fabs(q));
    const T t = r / c;
    if (val(t) <= 0.0f) return;
    const T a = 1.0f / (alpha * t);
    if (val(a) >= 1.6f) return;
    const T a2 = a * a;
    const T num = 3.535f * a + 2.181f * a2;
    const T den = 1.0f + 2.276f * a + 2.577f * a2;
    const T ab = Gb * ((3.535f + 4.362f * a) * den - num * (2.276f + 5.154f * a)) / (den * den);
    const T tb = -ab * a / t;
    const T rb = tb / c;
    T cbl = -tb * t / c;
    const T qb = rb * (0.5f / r) * sgn_of(q);
    cbl = cbl - qb * (2.0f * c);
    cb = cb + cbl;
}

// ad_fresnel(cosThetaI) -> (F, cosThetaT)
template <class T>
DEV void fresnel_adj(const T &cosI_, float eta, float invEta, const T &Fb, const T &cosTb, T &cosIb) {
    const float scale = val(cosI_) > 0.0f ? invEta : eta;
    const T cTSqr = 1.0f - (1.0f - cosI_ * cosI_) * (scale * scale);
    if (val(cTSqr) <= 0.0f) return;
    const T cI = fabs(cosI_);
    const T cT = sqrt(cTSqr);
    const T d1 = cI + eta * cT, d2 = eta * cI + cT;
    const T Rs = (cI - eta * cT) / d1;
    const T Rp = (eta * cI - cT) / d2;
    const T Rsb = Fb * Rs, Rpb = Fb * Rp;
    const T n1b = Rsb / d1, d1b = -Rsb * Rs / d1;
    const T n2b = Rpb / d2, d2b = -Rpb * Rp / d2;
    const T cIb = n1b + d1b + eta * (n2b + d2b);
    T cTb = eta * (d1b - n1b) + (d2b - n2b);
    cTb = cTb + (val(cosI_) > 0.0f ? -cosTb : cosTb);
    const T cTSqrb = cTb * (0.5f / cT);
    cosIb = cosIb + sgn_of(cosI_) * cIb + cTSqrb * (2.0f * scale * scale) * cosI_;
}

// snc = |(wo.ng)(wi.ns) / ((wi.ng)(wo.ns))| (ng constant)
template <class T>
DEV void snc_adj(const TV3<T> &wi, const TIsect<T> &is, const TV3<T> &wo, const T &yb, TV3<T> &wib, TV3<T> &snb,
                 TV3<T> &wob) {
    const T cosWi = dot(is.shadingNormal, wi);
    const T cosWo = dot(is.shadingNormal, wo);
    const T wig = dot(is.geomNormal, wi);
    const T wog = dot(is.geomNormal, wo);
    const T num = wog * cosWi, den = wig * cosWo;
    const T x = num / den;
    const T xb = yb * sgn_of(x);
    const T numb = xb / den, denb = -xb * x / den;
    const T wogb = numb * cosWi, cosWib = numb * wog, wigb = denb * cosWo, cosWob = denb * wig;
    wib = wib + is.shadingNormal * cosWib + is.geomNormal * wigb;
    wob = wob + is.shadingNormal * cosWob + is.geomNormal * wogb;
    snb = snb + wi * cosWib + wo * cosWob;
}

// Rough dielectric evaluation (ad_rough_dielectric_evaluate).
template <class T, class ObF>
DEV void rough_dielectric_evaluate_adj(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const TV3<T> &wo,
                                       const ObF &obf, bool adjoint, TV3<T> &wib, TV3<T> &nb, TV3<T> &wob) {
    const T cosWi = dot(wi, normal);
    const T cosWo = dot(wo, normal);
    const bool reflect = val(cosWi) * val(cosWo) > 0.0f;
    const float eta_ = val(cosWi) > 0.0f ? b.eta : b.invEta;
    const float revEta_ = val(cosWo) > 0.0f ? b.eta : b.invEta;
    const TV3<T> hsum = reflect ? TV3<T>(wi + wo) : TV3<T>(wi + wo * eta_);
    TV3<T> H = tnorm(hsum);
    const bool flip = val(dot(H, normal)) < 0.0f;
    if (flip) H = -H;
    const T cHi = dot(wi, H), cHo = dot(wo, H);
    TV3<T> b0, b1;
    tframe(normal, b0, b1);
    const TV3<T> lH(dot(b0, H), dot(b1, H), dot(normal, H));
    const float alpha = b.alpha;
    const T D = ad_beckmann_d(lH, alpha);
    T ct;
    const T F = ad_fresnel(cHi, ct, b.eta, b.invEta);
    const T aWi = fabs(cosWi), aWo = fabs(cosWo);
    const T g1i = ad_beckmann_g1(alpha, aWi), g1o = ad_beckmann_g1(alpha, aWo);
    const T G = g1i * g1o;
    const T sA = alpha * (1.2f - 0.2f * sqrt(aWi));
    const T bdS = ad_beckmann_d(lH, sA);
    const T prob = lH.z * bdS;
    const T rsA = alpha * (1.2f - 0.2f * sqrt(aWo));
    const T bdR = ad_beckmann_d(lH, rsA);
    const T revProb = lH.z * bdR;
    TBsdf<T> o;
    o.cosWo = cosWo;
    if (reflect) {
        o.contrib = tv<T>(ks_of(b)) * fabs(F * D * G / (4.0f * cosWi));
        o.pdf = fabs(prob * F / (4.0f * cHo));
        o.revPdf = fabs(revProb * F / (4.0f * cHi));
    } else {
        const T sd = cHi + eta_ * cHo;
        const T rsd = cHo + revEta_ * cHi;
        const float factor = adjoint ? 1.0f : (1.0f / eta_) * (1.0f / eta_);
        const float e2 = eta_ * eta_, re2 = revEta_ * revEta_;
        const T omF = 1.0f - F;
        o.contrib = tv<T>(kt_of(b)) * fabs(factor * ((omF * D * G * e2 * cHi * cHo) / (cosWi * (sd * sd))));
        o.pdf = fabs(prob * omF * (e2 * cHo) / (sd * sd));
        o.revPdf = fabs(revProb * omF * (re2 * cHi) / (rsd * rsd));
    }
    const TBsdfAdj<T> ob = obf(o, wo, wob);
    T Fb(0.0f), Db(0.0f), Gb(0.0f), probb(0.0f), revProbb(0.0f), cHib(0.0f), cHob(0.0f), cosWib(0.0f);
    T cosWob = ob.cosWo;
    if (reflect) {
        const T fdg = F * D * G;
        const T Sx = fdg / (4.0f * cosWi);
        const T Sxb = dot(tv<T>(ks_of(b)), ob.contrib) * sgn_of(Sx);
        const T fdgb = Sxb / (4.0f * cosWi);
        cosWib = cosWib - Sxb * Sx / cosWi;
        Fb = Fb + fdgb * D * G;
        Db = Db + fdgb * F * G;
        Gb = Gb + fdgb * F * D;
        const T Px = prob * F / (4.0f * cHo);
        const T Pxb = ob.pdf * sgn_of(Px);
        probb = probb + Pxb * F / (4.0f * cHo);
        Fb = Fb + Pxb * prob / (4.0f * cHo);
        cHob = cHob - Pxb * Px / cHo;
        const T Rx = revProb * F / (4.0f * cHi);
        const T Rxb = ob.revPdf * sgn_of(Rx);
        revProbb = revProbb + Rxb * F / (4.0f * cHi);
        Fb = Fb + Rxb * revProb / (4.0f * cHi);
        cHib = cHib - Rxb * Rx / cHi;
    } else {
        const T sd = cHi + eta_ * cHo;
        const T rsd = cHo + revEta_ * cHi;
        const float factor = adjoint ? 1.0f : (1.0f / eta_) * (1.0f / eta_);
        const float e2 = eta_ * eta_, re2 = revEta_ * revEta_;
        const T omF = 1.0f - F;
        const T N = omF * D * G * e2 * cHi * cHo;
        const T M = cosWi * (sd * sd);
        const T Sx = factor * (N / M);
        const T Sxb = dot(tv<T>(kt_of(b)), ob.contrib) * sgn_of(Sx);
        const T Nb = Sxb * factor / M;
        const T Mb = -Sxb * Sx / M;
        cosWib = cosWib + Mb * (sd * sd);
        T sdb = Mb * cosWi * (2.0f * sd);
        T omFb = Nb * D * G * e2 * cHi * cHo;
        Db = Db + Nb * omF * G * e2 * cHi * cHo;
        Gb = Gb + Nb * omF * D * e2 * cHi * cHo;
        cHib = cHib + Nb * omF * D * G * e2 * cHo;
        cHob = cHob + Nb * omF * D * G * e2 * cHi;
        // pdf = |prob (1 - F) (e2 cHo) / sd^2|
        const T Px = prob * omF * (e2 * cHo) / (sd * sd);
        const T Pxb = ob.pdf * sgn_of(Px);
        probb = probb + Pxb * omF * (e2 * cHo) / (sd * sd);
        omFb = omFb + Pxb * prob * (e2 * cHo) / (sd * sd);
        cHob = cHob + Pxb * prob * omF * e2 / (sd * sd);
        sdb = sdb - Pxb * Px * 2.0f / sd;
        // revPdf = |revProb (1 - F) (re2 cHi) / rsd^2|
        const T Rx = revProb * omF * (re2 * cHi) / (rsd * rsd);
        const T Rxb = ob.revPdf * sgn_of(Rx);
        revProbb = revProbb + Rxb * omF * (re2 * cHi) / (rsd * rsd);
        omFb = omFb + Rxb * revProb * (re2 * cHi) / (rsd * rsd);
        cHib = cHib + Rxb * revProb * omF * re2 / (rsd * rsd);
        const T rsdb = -Rxb * Rx * 2.0f / rsd;
        Fb = Fb - omFb;
        cHib = cHib + sdb + revEta_ * rsdb;
        cHob = cHob + eta_ * sdb + rsdb;
    }
    // prob = lH.z bd(lH, sA), revProb = lH.z bd(lH, rsA)
    TV3<T> lHb = tzero<T>();
    lHb.z = lHb.z + probb * bdS + revProbb * bdR;
    T sAb(0.0f), rsAb(0.0f), dummy(0.0f);
    beckmann_d_adj(lH, sA, probb * lH.z, lHb, sAb);
    beckmann_d_adj(lH, rsA, revProbb * lH.z, lHb, rsAb);
    beckmann_d_adj(lH, T(alpha), Db, lHb, dummy);
    T aWib = sAb * alpha * (-0.1f) / sqrt(aWi);
    T aWob = rsAb * alpha * (-0.1f) / sqrt(aWo);
    beckmann_g1_adj(alpha, aWi, Gb * g1o, aWib);
    beckmann_g1_adj(alpha, aWo, Gb * g1i, aWob);
    cosWib = cosWib + sgn_of(cosWi) * aWib;
    cosWob = cosWob + sgn_of(cosWo) * aWob;
    fresnel_adj(cHi, b.eta, b.invEta, Fb, T(0.0f), cHib);
    // localH = (b0.H, b1.H, n.H)
    TV3<T> Hb = b0 * lHb.x + b1 * lHb.y + normal * lHb.z;
    nb = nb + H * lHb.z;
    tframe_adj(normal, H * lHb.x, H * lHb.y, nb);
    Hb = Hb + wi * cHib + wo * cHob;
    wib = wib + H * cHib;
    wob = wob + H * cHob;
    if (flip) Hb = -Hb;
    TV3<T> hsb = tzero<T>();
    tnorm_adj(hsum, Hb, hsb);
    wib = wib + hsb;
    wob = wob + (reflect ? hsb : hsb * eta_);
    wob = wob + normal * cosWob;
    wib = wib + normal * cosWib;
    nb = nb + wo * cosWob + wi * cosWib;
}

// Rough dielectric sampling (ad_rough_dielectric_sample, fixDiscrete = false).
// wob: on entry the adjoint of the sampled direction from its later uses.
template <class T, class ObF>
DEV void rough_dielectric_sample_adj(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const T &r0, const T &r1,
                                     float uDiscrete, TV3<T> &wob, const ObF &obf, bool adjoint, TV3<T> &wib,
                                     TV3<T> &nb, T &r0b, T &r1b) {
    const T cosWi = dot(wi, normal);
    const float alpha = b.alpha;
    const T aWi = fabs(cosWi);
    const T sA = alpha * (1.2f - 0.2f * sqrt(aWi));
    const T phiM = kTwoPi * r1;
    const T aS = sA * sA;
    const T lg = fmax(1.0f - r0, 1e-6f);
    const T tTS = aS * (-log(lg));
    const T cTM = 1.0f / sqrt(1.0f + tTS);
    const T cTM2 = cTM * cTM;
    const T mDen = kPi * aS * cTM * cTM2;
    const T mPdf = (1.0f - r0) / mDen;
    const T sq1 = fmax(1.0f - cTM2, 1e-6f);
    const T sTM = sqrt(sq1);
    const T cph = cos(phiM), sph = sin(phiM);
    const TV3<T> lH(sTM * cph, sTM * sph, cTM);
    const TV3<T> H = frame_apply(lH, normal);
    const T cHi = dot(wi, H);
    T cT;
    const T F = ad_fresnel(cHi, cT, b.eta, b.invEta);
    const bool refl = uDiscrete <= val(F);
    TV3<T> wo;
    float etaR = 1.0f, eta_ = 1.0f;
    if (refl) {
        wo = treflect(wi, H);
    } else {
        etaR = val(cT) < 0.0f ? b.invEta : b.eta;
        wo = H * (dot(wi, H) * etaR + cT) - wi * etaR;
        eta_ = val(cosWi) > 0.0f ? b.eta : b.invEta;
    }
    const T cHo = dot(wo, H);
    const T cosWo = dot(wo, normal);
    const T aWo = fabs(cosWo);
    const T rsA = alpha * (1.2f - 0.2f * sqrt(aWo));
    const T bdR = ad_beckmann_d(lH, rsA);
    const T D = ad_beckmann_d(lH, alpha);
    const T g1i = ad_beckmann_g1(alpha, aWi), g1o = ad_beckmann_g1(alpha, aWo);
    const T G = g1i * g1o;
    const V3 reflc = refl ? ks_of(b) : kt_of(b) * (adjoint ? 1.0f : (1.0f / eta_) * (1.0f / eta_));
    // contrib = reflc |D G cHi / (mPdf aWi)|
    const T num = D * G * cHi, den = mPdf * aWi;
    const T Cx = num / den;
    TBsdf<T> o;
    o.contrib = tv<T>(reflc) * fabs(Cx);
    o.cosWo = cosWo;
    if (refl) {
        o.pdf = fabs(mPdf * F / (4.0f * cHo));
        o.revPdf = fabs(F * bdR * lH.z * (1.0f / (4.0f * cHi)));
    } else {
        const T sd = cHi + eta_ * cHo;
        const T dwh = ((eta_ * eta_) * cHo) / (sd * sd);
        const T omF = 1.0f - F;
        o.pdf = fabs(mPdf * omF * fabs(dwh));
        const float revEta_ = val(cosWo) > 0.0f ? b.eta : b.invEta;
        const T rsd = cHo + revEta_ * cHi;
        o.revPdf = fabs(omF * bdR * lH.z * (((revEta_ * revEta_) * cHi) / (rsd * rsd)));
    }
    const TBsdfAdj<T> ob = obf(o, wo, wob);
    const T Cxb = dot(tv<T>(reflc), ob.contrib) * sgn_of(Cx);
    const T numb = Cxb / den, denb = -Cxb * Cx / den;
    T Db = numb * G * cHi, Gb = numb * D * cHi, cHib = numb * D * G;
    T mPdfb = denb * aWi, aWib = denb * mPdf;
    T Fb(0.0f), cTb(0.0f), cHob(0.0f), lHzb(0.0f), bdRb(0.0f), cosWob = ob.cosWo;
    if (refl) {
        const T Px = mPdf * F / (4.0f * cHo);
        const T Pxb = ob.pdf * sgn_of(Px);
        mPdfb = mPdfb + Pxb * F / (4.0f * cHo);
        Fb = Fb + Pxb * mPdf / (4.0f * cHo);
        cHob = cHob - Pxb * Px / cHo;
        const T rdw = 1.0f / (4.0f * cHi);
        const T Rx = F * bdR * lH.z * rdw;
        const T Rxb = ob.revPdf * sgn_of(Rx);
        Fb = Fb + Rxb * bdR * lH.z * rdw;
        bdRb = bdRb + Rxb * F * lH.z * rdw;
        lHzb = lHzb + Rxb * F * bdR * rdw;
        cHib = cHib - Rxb * Rx / cHi;
    } else {
        const T sd = cHi + eta_ * cHo;
        const T dwh = ((eta_ * eta_) * cHo) / (sd * sd);
        const T omF = 1.0f - F;
        const T Px = mPdf * omF * fabs(dwh);
        const T Pxb = ob.pdf * sgn_of(Px);
        mPdfb = mPdfb + Pxb * omF * fabs(dwh);
        T omFb = Pxb * mPdf * fabs(dwh);
        const T dwhb = Pxb * mPdf * omF * sgn_of(dwh);
        cHob = cHob + dwhb * (eta_ * eta_) / (sd * sd);
        const T sdb = -dwhb * dwh * 2.0f / sd;
        cHib = cHib + sdb;
        cHob = cHob + eta_ * sdb;
        const float revEta_ = val(cosWo) > 0.0f ? b.eta : b.invEta;
        const T rsd = cHo + revEta_ * cHi;
        const T rdwh = ((revEta_ * revEta_) * cHi) / (rsd * rsd);
        const T Rx = omF * bdR * lH.z * rdwh;
        const T Rxb = ob.revPdf * sgn_of(Rx);
        omFb = omFb + Rxb * bdR * lH.z * rdwh;
        bdRb = bdRb + Rxb * omF * lH.z * rdwh;
        lHzb = lHzb + Rxb * omF * bdR * rdwh;
        const T rdwhb = Rxb * omF * bdR * lH.z;
        cHib = cHib + rdwhb * (revEta_ * revEta_) / (rsd * rsd);
        const T rsdb = -rdwhb * rdwh * 2.0f / rsd;
        cHob = cHob + rsdb;
        cHib = cHib + revEta_ * rsdb;
        Fb = Fb - omFb;
    }
    // wo.H and the direction's other uses
    TV3<T> Hb = wo * cHob;
    wob = wob + H * cHob + normal * cosWob;
    TV3<T> nbl = wo * cosWob;
    // the roughness at wo, D and G
    T rsAb(0.0f), dummy(0.0f);
    TV3<T> lHb = tzero<T>();
    lHb.z = lHzb;
    beckmann_d_adj(lH, rsA, bdRb, lHb, rsAb);
    beckmann_d_adj(lH, T(alpha), Db, lHb, dummy);
    T aWob = rsAb * alpha * (-0.1f) / sqrt(aWo);
    beckmann_g1_adj(alpha, aWi, Gb * g1o, aWib);
    beckmann_g1_adj(alpha, aWo, Gb * g1i, aWob);
    const T cosWobl = sgn_of(cosWo) * aWob;
    wob = wob + normal * cosWobl;
    nbl = nbl + wo * cosWobl;
    // wo from (wi, H)
    if (refl) {
        treflect_adj(wi, H, wob, wib, Hb);
    } else {
        const T q = dot(wi, H);
        const T s = q * etaR + cT;
        Hb = Hb + wob * s;
        const T sb = dot(H, wob);
        wib = wib - wob * etaR;
        const T qb = sb * etaR;
        cTb = cTb + sb;
        wib = wib + H * qb;
        Hb = Hb + wi * qb;
    }
    fresnel_adj(cHi, b.eta, b.invEta, Fb, cTb, cHib);
    wib = wib + H * cHib;
    Hb = Hb + wi * cHib;
    // H = frame(normal) lH
    frame_apply_adj(lH, normal, Hb, lHb, nbl);
    // lH = (sTM cos phiM, sTM sin phiM, cTM)
    const T sTMb = lHb.x * cph + lHb.y * sph;
    const T phiMb = sTM * (lHb.y * cph - lHb.x * sph);
    T cTMb = lHb.z;
    if (fmax_active(1.0f - cTM2, 1e-6f)) cTMb = cTMb - sTMb * (0.5f / sTM) * 2.0f * cTM;
    // mPdf = (1 - r0) / (pi aS cTM^3)
    r0b = r0b - mPdfb / mDen;
    const T mDenb = -mPdfb * mPdf / mDen;
    T aSb = mDenb * kPi * cTM * cTM2;
    cTMb = cTMb + mDenb * kPi * aS * 3.0f * cTM2;
    // cTM = (1 + tTS)^(-1/2)
    const T tTSb = cTMb * (-0.5f) * cTM * cTM2;
    aSb = aSb + tTSb * (-log(lg));
    if (fmax_active(1.0f - r0, 1e-6f)) r0b = r0b + tTSb * aS / lg;
    r1b = r1b + kTwoPi * phiMb;
    const T sAb = aSb * 2.0f * sA;
    aWib = aWib + sAb * alpha * (-0.1f) / sqrt(aWi);
    const T cosWib = sgn_of(cosWi) * aWib;
    wib = wib + normal * cosWib;
    nbl = nbl + wi * cosWib;
    nb = nb + nbl;
}

// ad_evaluate: Lambertian, Phong and rough dielectric.
template <class T, class ObF>
DEV void evaluate_adj(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const TV3<T> &wo, const ObF &obf,
                      bool adjoint, TV3<T> &wib, TV3<T> &nb, TV3<T> &wob) {
    if (b.type == kBsdfRoughDielectric) {
        rough_dielectric_evaluate_adj(b, wi, normal, wo, obf, adjoint, wib, nb, wob);
        return;
    }
    const T cosWiRaw = dot(normal, wi);
    const float sg = val(cosWiRaw) > 0.0f ? 1.0f : -1.0f;
    const TV3<T> n = normal * sg;
    const T cosWi = cosWiRaw * sg;
    const T cosWo = dot(n, wo);
    const V3 kd = kd_of(b);
    T cosWib(0.0f);
    TV3<T> nbl = tzero<T>();
    TBsdf<T> o;
    o.cosWo = cosWo;
    T cosWob;
    if (b.type == kBsdfLambertian) {
        const T fwd = cosWo * kInvPi;
        o.contrib = fwd * tv<T>(kd);
        o.pdf = fwd;
        o.revPdf = cosWi * kInvPi;
        const TBsdfAdj<T> ob = obf(o, wo, wob);
        cosWob = ob.cosWo + (dot(tv<T>(kd), ob.contrib) + ob.pdf) * kInvPi;
        cosWib = cosWib + ob.revPdf * kInvPi;
    } else {
        // contrib = (spec + kd / pi) cosWo
        TV3<T> c0 = tzero<T>();
        TV3<T> R = tzero<T>();
        T alpha(0.0f), weight(0.0f), specPdf(0.0f);
        bool spec = false;
        if (b.ksWeight > 0.0f) {
            R = treflect(wi, n);
            alpha = dot(R, wo);
            const float wv = powf(val(alpha), b.exponent) * kInvTwoPi;
            if (wv > 1e-10f) {
                spec = true;
                weight = pow(alpha, b.exponent) * kInvTwoPi;
                c0 = tv<T>(ks_of(b)) * ((b.exponent + 2.0f) * weight);
                specPdf = b.ksWeight * (b.exponent + 1.0f) * weight;
            }
        }
        o.pdf = specPdf;
        o.revPdf = specPdf;
        const float tmp = (1.0f - b.ksWeight) * kInvPi;
        if (b.ksWeight < 1.0f) {
            c0 = c0 + tv<T>(kd * kInvPi);
            o.pdf = o.pdf + tmp * cosWo;
            o.revPdf = o.revPdf + tmp * cosWi;
        }
        o.contrib = c0 * cosWo;
        const TBsdfAdj<T> ob = obf(o, wo, wob);
        cosWob = ob.cosWo + dot(c0, ob.contrib);
        const TV3<T> c0b = ob.contrib * cosWo;
        if (b.ksWeight < 1.0f) {
            cosWob = cosWob + tmp * ob.pdf;
            cosWib = cosWib + tmp * ob.revPdf;
        }
        if (spec) {
            const T weightb = (b.exponent + 2.0f) * dot(tv<T>(ks_of(b)), c0b) +
                              b.ksWeight * (b.exponent + 1.0f) * (ob.pdf + ob.revPdf);
            const T alphab = weightb * kInvTwoPi * b.exponent * pow(alpha, b.exponent - 1.0f);
            const TV3<T> Rb = wo * alphab;
            wob = wob + R * alphab;
            treflect_adj(wi, n, Rb, wib, nbl);
        }
    }
    nbl = nbl + wo * cosWob;
    wob = wob + n * cosWob;
    // cosWi = sg (normal . wi)
    nb = nb + wi * (sg * cosWib) + nbl * sg;
    wib = wib + normal * (sg * cosWib);
}

// ad_sample: Lambertian, Phong and rough dielectric (fixDiscrete = false).
// wob: on entry the adjoint of the sampled direction from its later uses.
template <class T, class ObF>
DEV void sample_adj(const Bsdf &b, const TV3<T> &wi, const TV3<T> &normal, const T &r0, const T &r1, float uDiscrete,
                    TV3<T> &wob, const ObF &obf, bool adjoint, TV3<T> &wib, TV3<T> &nb, T &r0b, T &r1b) {
    if (b.type == kBsdfRoughDielectric) {
        rough_dielectric_sample_adj(b, wi, normal, r0, r1, uDiscrete, wob, obf, adjoint, wib, nb, r0b, r1b);
        return;
    }
    const T cosWiRaw = dot(wi, normal);
    const float sg = val(cosWiRaw) > 0.0f ? 1.0f : -1.0f;
    const TV3<T> n = normal * sg;
    const T cosWi = cosWiRaw * sg;
    T cosWib(0.0f);
    TV3<T> nbl = tzero<T>();
    TBsdf<T> o;
    if (b.type == kBsdfLambertian) {
        const TV3<T> l = tcos_hemisphere(r0, r1);
        const TV3<T> wo = frame_apply(l, n);
        o.cosWo = l.z;
        o.pdf = l.z * kInvPi;
        o.contrib = tv<T>(kd_of(b));
        o.revPdf = cosWi * kInvPi;
        const TBsdfAdj<T> ob = obf(o, wo, wob);
        TV3<T> lb = tzero<T>();
        lb.z = ob.cosWo + ob.pdf * kInvPi;
        cosWib = ob.revPdf * kInvPi;
        frame_apply_adj(l, n, wob, lb, nbl);
        tcos_hemisphere_adj(r0, r1, lb, r0b, r1b);
    } else {
        const TV3<T> R = treflect(wi, n);
        const bool diffuse = uDiscrete > b.ksWeight;
        TV3<T> l;
        T cosAlpha(0.0f), sinAlpha(0.0f), phi(0.0f);
        const float power = 1.0f / (b.exponent + 1.0f);
        if (diffuse) {
            l = tcos_hemisphere(r0, r1);
        } else {
            cosAlpha = pow(r1, power);
            sinAlpha = sqrt(fmax(1.0f - cosAlpha * cosAlpha, 1e-6f));
            phi = kTwoPi * r0;
            l = TV3<T>(sinAlpha * cos(phi), sinAlpha * sin(phi), cosAlpha);
        }
        const TV3<T> wo = frame_apply(l, diffuse ? n : R);
        const T cosWo = dot(n, wo);
        TV3<T> c0 = tzero<T>();
        T alpha(0.0f), weight(0.0f), specPdf(0.0f);
        bool spec = false;
        if (b.ksWeight > 0.0f) {
            alpha = dot(R, wo);
            const float wv = powf(val(alpha), b.exponent) * kInvTwoPi;
            if (wv > 1e-10f) {
                spec = true;
                weight = pow(alpha, b.exponent) * kInvTwoPi;
                c0 = tv<T>(ks_of(b)) * ((b.exponent + 2.0f) * weight);
                specPdf = b.ksWeight * (b.exponent + 1.0f) * weight;
            }
        }
        T pdf = specPdf;
        o.revPdf = specPdf;
        const float tmp = (1.0f - b.ksWeight) * kInvPi;
        if (b.ksWeight < 1.0f) {
            c0 = c0 + tv<T>(kd_of(b) * kInvPi);
            pdf = pdf + tmp * cosWo;
            o.revPdf = o.revPdf + tmp * cosWi;
        }
        // contrib = c0 cosWo / pdf
        const TV3<T> c1 = c0 * cosWo;
        const T ipdf = 1.0f / pdf;
        o.cosWo = cosWo;
        o.pdf = pdf;
        o.contrib = c1 * ipdf;
        const TBsdfAdj<T> ob = obf(o, wo, wob);
        const TV3<T> c1b = ob.contrib * ipdf;
        const T pdfb = ob.pdf - dot(c1, ob.contrib) * ipdf * ipdf;
        T cosWob = ob.cosWo + dot(c0, c1b);
        const TV3<T> c0b = c1b * cosWo;
        if (b.ksWeight < 1.0f) {
            cosWob = cosWob + tmp * pdfb;
            cosWib = cosWib + tmp * ob.revPdf;
        }
        TV3<T> Rb = tzero<T>();
        if (spec) {
            const T weightb = (b.exponent + 2.0f) * dot(tv<T>(ks_of(b)), c0b) +
                              b.ksWeight * (b.exponent + 1.0f) * (pdfb + ob.revPdf);
            const T alphab = weightb * kInvTwoPi * b.exponent * pow(alpha, b.exponent - 1.0f);
            Rb = Rb + wo * alphab;
            wob = wob + R * alphab;
        }
        nbl = nbl + wo * cosWob;
        wob = wob + n * cosWob;
        TV3<T> lb = tzero<T>();
        if (diffuse) {
            frame_apply_adj(l, n, wob, lb, nbl);
            tcos_hemisphere_adj(r0, r1, lb, r0b, r1b);
        } else {
            frame_apply_adj(l, R, wob, lb, Rb);
            const T sAb = lb.x * cos(phi) + lb.y * sin(phi);
            const T phib = sinAlpha * (lb.y * cos(phi) - lb.x * sin(phi));
            T cAb = lb.z;
            if (fmax_active(1.0f - cosAlpha * cosAlpha, 1e-6f)) cAb = cAb - sAb * cosAlpha / sinAlpha;
            r0b = r0b + kTwoPi * phib;
            r1b = r1b + cAb * power * pow(r1, power - 1.0f);
        }
        treflect_adj(wi, n, Rb, wib, nbl);
    }
    nb = nb + wi * (sg * cosWib) + nbl * sg;
    wib = wib + normal * (sg * cosWib);
}


// ---------------------------------------------------------------- geometry adjoints
// ad_intersect: (org, dir) -> (position, shading normal); the geometric normal
// is the triangle's and carries no derivative.
template <class T>
DEV void intersect_adj(const SceneView &s, int tri, const TV3<T> &org, const TV3<T> &dir, const TV3<T> &posb,
                       const TV3<T> &snb, TV3<T> &orgb, TV3<T> &dirb) {
    const float *P = s.triP + 9 * tri;
    const V3 p0 = ld3(P), e1 = ld3(P + 3), e2 = ld3(P + 6);
    const float *N = s.triN + 9 * tri;
    const TV3<T> E1 = tv<T>(e1), E2 = tv<T>(e2);
    const TV3<T> s1 = cross(dir, E2);
    const T divisor = dot(s1, E1);
    const T inv = 1.0f / divisor;
    const TV3<T> sv = org - tv<T>(p0);
    const T u = dot(sv, s1) * inv;
    const TV3<T> s2 = cross(sv, E1);
    const T v = dot(dir, s2) * inv;
    const T t = dot(E2, s2) * inv;
    const T w = 1.0f - u - v;
    const TV3<T> N0 = tv<T>(ld3(N)), N1 = tv<T>(ld3(N + 3)), N2 = tv<T>(ld3(N + 6));
    const TV3<T> nraw = w * N0 + u * N1 + v * N2;
    TV3<T> nrb = tzero<T>();
    tnorm_adj(nraw, snb, nrb);
    const T wb = dot(N0, nrb);
    const T ub = dot(N1, nrb) - wb;
    const T vb = dot(N2, nrb) - wb;
    orgb = orgb + posb;
    const T tb = dot(dir, posb);
    TV3<T> db = posb * t;
    TV3<T> s2b = E2 * (tb * inv) + dir * (vb * inv);
    T invb = tb * dot(E2, s2) + vb * dot(dir, s2) + ub * dot(sv, s1);
    db = db + s2 * (vb * inv);
    TV3<T> svb = cross(E1, s2b) + s1 * (ub * inv);
    TV3<T> s1b = sv * (ub * inv);
    orgb = orgb + svb;
    const T divb = -invb * inv * inv;
    s1b = s1b + E1 * divb;
    db = db + cross(E2, s1b);
    dirb = dirb + db;
}

// ad_sample_triangle: (r0, r1) -> (position, normal)
template <class T>
DEV void sample_triangle_adj(const SceneView &s, int tri, const T &r0, const T &r1, const TV3<T> &posb,
                             const TV3<T> &nb, T &r0b, T &r1b) {
    const float *P = s.triP + 9 * tri;
    const float *N = s.triN + 9 * tri;
    const T a = sqrt((1.0f + 1e-6f) - r0);
    const T b1 = 1.0f - a;
    const T b2 = a * r1;
    const TV3<T> N0 = tv<T>(ld3(N)), N1 = tv<T>(ld3(N + 3)), N2 = tv<T>(ld3(N + 6));
    const TV3<T> nraw = N0 * (1.0f - b1 - b2) + N1 * b1 + N2 * b2;
    TV3<T> nrb = tzero<T>();
    tnorm_adj(nraw, nb, nrb);
    const T b1b = dot(tv<T>(ld3(P + 3)), posb) + dot(N1 - N0, nrb);
    const T b2b = dot(tv<T>(ld3(P + 6)), posb) + dot(N2 - N0, nrb);
    const T ab = -b1b + r1 * b2b;
    r1b = r1b + a * b2b;
    r0b = r0b - ab * (0.5f / a);
}

// Spherical direction (sin phi cos theta, sin phi sin theta, cos phi) with
// theta = 2 pi r0, phi = pi r1: the absolute-parameter BSDF sampling and the
// point light's emission.
template <class T>
DEV void sphere_dir_adj(const T &r0, const T &r1, const TV3<T> &db, const T &sinPhib_, T &r0b, T &r1b) {
    const T sT = kTwoPi * r0, sP = kPi * r1;
    const T sinP = sin(sP), cosP = cos(sP), cT = cos(sT), snT = sin(sT);
    const T sinPb = sinPhib_ + db.x * cT + db.y * snT;
    const T sTb = sinP * (db.y * cT - db.x * snT);
    const T sPb = sinPb * cosP - db.z * sinP;
    r0b = r0b + kTwoPi * sTb;
    r1b = r1b + kPi * sPb;
}

// ---------------------------------------------------------------- BSDF sampling step
// ad_bsdf_sampling<T, adjoint> with the adjoint flag (light subpaths) as an
// argument: the vertex state (isect, wi, MIS accumulators, throughput) and
// (r0, r1) -> the next direction and the updated state.
template <class T>
DEV void bsdf_sampling_fwd(const SceneView &s, int tri, const T &r0, const T &r1, float disc, bool useAbs,
                           int lcsTri, bool adjoint, TState<T> &ps, TV3<T> &dir) {
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

// Its adjoint: the updated state's adjoints in `nb` (isect and wi unused), the
// direction's in dirb_; the input state's accumulate into `ib`. The BSDF's
// forward outputs reach the MIS and throughput adjoints through the BSDF
// adjoint's callback, so each vertex evaluates its BSDF once here.
template <class T>
DEV void bsdf_sampling_adj(const SceneView &s, int tri, const T &r0, const T &r1, float disc, bool useAbs,
                           int lcsTri, bool adjoint, const TState<T> &ps, const TV3<T> &dirb_, const TState<T> &nb,
                           TState<T> &ib, T &r0b, T &r1b) {
    const Bsdf &b = bsdf_of_tri(s, tri);
    T jacobian(1.0f);
    TV3<T> dir = tzero<T>();
    TV3<T> nextPos, nextNormal, d0;
    T distSq(0.0f), invDistSq(0.0f), invDist(0.0f), J0(0.0f), sinP(0.0f);
    float shapePdf = 1.0f;
    if (lcsTri >= 0) {
        ad_sample_triangle(s, lcsTri, r0, r1, nextPos, nextNormal);
        shapePdf = s.lights[area_light_of_tri(s, lcsTri)].invTotalArea;
        d0 = nextPos - ps.isect.position;
        distSq = dot(d0, d0);
        invDistSq = 1.0f / distSq;
        invDist = sqrt(invDistSq);
        dir = d0 * invDist;
        J0 = dot(nextNormal, dir) * invDistSq;
        jacobian = fabs(J0) / shapePdf;
    } else if (useAbs) {
        const T sP = kPi * r1;
        sinP = sin(sP);
        jacobian = fabs(sinP);
        dir = TV3<T>(sinP * cos(kTwoPi * r0), sinP * sin(kTwoPi * r0), cos(sP));
    }
    T jacb(0.0f);
    // the adjoints of the BSDF outputs o (and the snc factor's share of wo's adjoint)
    auto obf = [&](const TBsdf<T> &o, const TV3<T> &wo, TV3<T> &wob) -> TBsdfAdj<T> {
        T sncv(1.0f);
        if (adjoint) sncv = ad_snc(ps.wi, ps.isect, wo);
        const TV3<T> cs = o.contrib * sncv;
        const TV3<T> contrib = cs * jacobian;
        ib.throughput = ib.throughput + cmul(nb.throughput, contrib);
        const TV3<T> contribb = cmul(nb.throughput, ps.throughput);
        const T k = o.cosWo / o.pdf;
        const T rp2 = o.revPdf * o.revPdf;
        const T A = ps.cur * rp2 + ps.prev;
        const T m = k * k;
        TBsdfAdj<T> ob;
        const T mb = nb.cur * A;
        ib.cur = ib.cur + nb.cur * m * rp2;
        ib.prev = ib.prev + nb.cur * m;
        ob.revPdf = nb.cur * m * ps.cur * 2.0f * o.revPdf;
        const T kb = 2.0f * k * mb;
        ob.cosWo = kb / o.pdf;
        const T ip = 1.0f / o.pdf;
        ob.pdf = -kb * k / o.pdf - nb.prev * 2.0f * ip * ip * ip;
        jacb = dot(cs, contribb);
        const TV3<T> csb = contribb * jacobian;
        if (adjoint) {
            ob.contrib = csb * sncv;
            snc_adj(ps.wi, ps.isect, wo, dot(o.contrib, csb), ib.wi, ib.isect.shadingNormal, wob);
        } else {
            ob.contrib = csb;
        }
        return ob;
    };
    TV3<T> dirb = dirb_;
    if (lcsTri < 0 && !useAbs) {
        sample_adj(b, ps.wi, ps.isect.shadingNormal, r0, r1, disc, dirb, obf, adjoint, ib.wi, ib.isect.shadingNormal,
                   r0b, r1b);
        return;
    }
    evaluate_adj(b, ps.wi, ps.isect.shadingNormal, dir, obf, lcsTri >= 0 ? false : adjoint, ib.wi,
                 ib.isect.shadingNormal, dirb);
    if (lcsTri >= 0) {
        const T J0b = jacb * sgn_of(J0) / shapePdf;
        const TV3<T> nnb = dir * (J0b * invDistSq);
        dirb = dirb + nextNormal * (J0b * invDistSq);
        T invDistSqb = J0b * dot(nextNormal, dir);
        TV3<T> d0b = dirb * invDist;
        const T invDistb = dot(d0, dirb);
        invDistSqb = invDistSqb + invDistb * (0.5f / invDist);
        const T distSqb = -invDistSqb * invDistSq * invDistSq;
        d0b = d0b + d0 * (2.0f * distSqb);
        ib.isect.position = ib.isect.position - d0b;
        sample_triangle_adj(s, lcsTri, r0, r1, d0b, nnb, r0b, r1b);
    } else {
        sphere_dir_adj(r0, r1, dirb, jacb * sgn_of(sinP), r0b, r1b);
    }
}

// ---------------------------------------------------------------- environment light adjoints
template <class T> HD T ad_tent_d(const T &x) {
    return val(x) < 0.5f ? -1.0f / sqrt(2.0f * x) : 1.0f / sqrt(2.0f * (x - 0.5f));
}

// ad_env_sample_direction: (u0, u1) -> (direction to the light, value, pdf)
template <class T>
DEV void env_sample_direction_adj(const SceneView &s, const T &u0, const T &u1, const TV3<T> &dirb, const TV3<T> &valueb,
                                  const T &pdfb, T &u0b, T &u1b) {
    float a = val(u0), bb = val(u1);
    const int row = env_u_to_index(s.envCdfRows, s.envH, bb);
    const float *cc = s.envCdfCols + row * (s.envW + 1);
    const int col = env_u_to_index(cc, s.envW, a);
    const float cr0 = __ldg(s.envCdfRows + row), cr1 = __ldg(s.envCdfRows + row + 1);
    const float cc0 = __ldg(cc + col), cc1 = __ldg(cc + col + 1);
    const T x0 = (u0 - cc0) / (cc1 - cc0);
    const T x1 = (u1 - cr0) / (cr1 - cr0);
    const T t0 = ad_tent<T>(x0), t1 = ad_tent<T>(x1);
    const T phi = (t0 + float(col) + 0.5f) * s.envPix[0];
    const T theta = (t1 + float(row) + 0.5f) * s.envPix[1];
    const T sinPhi = sin(phi), cosPhi = cos(phi), sinTheta = sin(theta), cosTheta = cos(theta);
    const float *m = s.envToWorld;
    const TV3<T> db(m[0] * dirb.x + m[3] * dirb.y + m[6] * dirb.z, m[1] * dirb.x + m[4] * dirb.y + m[7] * dirb.z,
                    m[2] * dirb.x + m[5] * dirb.y + m[8] * dirb.z);
    const TV3<T> V00 = tv<T>(env_at(s, col, row)), V10 = tv<T>(env_at(s, col + 1, row));
    const TV3<T> V01 = tv<T>(env_at(s, col, row + 1)), V11 = tv<T>(env_at(s, col + 1, row + 1));
    const T dx1 = t0, dx2 = 1.0f - t0, dy1 = t1, dy2 = 1.0f - t1;
    const TV3<T> value1 = V00 * (dx2 * dy2) + V10 * (dx1 * dy2);
    const TV3<T> value2 = V01 * (dx2 * dy1) + V11 * (dx1 * dy1);
    const float rw0 = env_row_weight(s, row), rw1 = env_row_weight(s, row + 1);
    const T numer = (tlum(value1) * rw0 + tlum(value2) * rw1) * s.envNorm;
    const T aS = fabs(sinTheta);
    const T denom = fmax(aS, 1e-7f);
    const T pdf = numer / denom;
    const T numerb = pdfb / denom;
    const T denomb = -pdfb * pdf / denom;
    T sTb = fmax_active(aS, 1e-7f) ? denomb * sgn_of(sinTheta) : T(0.0f);
    TV3<T> v1b = valueb, v2b = valueb;
    tlum_adj(numerb * (rw0 * s.envNorm), v1b);
    tlum_adj(numerb * (rw1 * s.envNorm), v2b);
    T t0b = dot(v1b, (V10 - V00) * dy2) + dot(v2b, (V11 - V01) * dy1);
    T t1b = -dot(v1b, V00 * dx2 + V10 * dx1) + dot(v2b, V01 * dx2 + V11 * dx1);
    // d = (sinPhi sinTheta, cosTheta, -cosPhi sinTheta)
    const T sPb = db.x * sinTheta;
    sTb = sTb + db.x * sinPhi - db.z * cosPhi;
    const T cTb = db.y;
    const T cPb = -db.z * sinTheta;
    const T phib = sPb * cosPhi - cPb * sinPhi;
    const T thetab = sTb * cosTheta - cTb * sinTheta;
    t0b = t0b + phib * s.envPix[0];
    t1b = t1b + thetab * s.envPix[1];
    u0b = u0b + t0b * ad_tent_d(x0) / (cc1 - cc0);
    u1b = u1b + t1b * ad_tent_d(x1) / (cr1 - cr0);
}

// ad_env_emission: the direction to the light -> (emission, directPdf, emissionPdf)
template <class T>
DEV void env_emission_adj(const SceneView &s, const Light &L, const TV3<T> &dirToLight, const TV3<T> &emb,
                          const T &dpb_, const T &epb, TV3<T> &dirb) {
    const float *m = s.envToLight;
    const TV3<T> d(m[0] * dirToLight.x + m[1] * dirToLight.y + m[2] * dirToLight.z,
                   m[3] * dirToLight.x + m[4] * dirToLight.y + m[5] * dirToLight.z,
                   m[6] * dirToLight.x + m[7] * dirToLight.y + m[8] * dirToLight.z);
    const T uvx = atan2(d.x, -d.z) * kInvTwoPi * float(s.envW) - 0.5f;
    const T uvy = acos(d.y) * kInvPi * float(s.envH) - 0.5f;
    const int col = int(floorf(val(uvx)));
    const int row = int(floorf(val(uvy)));
    const T dx1 = uvx - float(col), dx2 = 1.0f - dx1, dy1 = uvy - float(row), dy2 = 1.0f - dy1;
    const TV3<T> R00 = tv<T>(env_rep_at(s, col, row)), R10 = tv<T>(env_rep_at(s, col + 1, row));
    const TV3<T> R01 = tv<T>(env_rep_at(s, col, row + 1)), R11 = tv<T>(env_rep_at(s, col + 1, row + 1));
    const TV3<T> value1 = R00 * (dx2 * dy2) + R10 * (dx1 * dy2);
    const TV3<T> value2 = R01 * (dx2 * dy1) + R11 * (dx1 * dy1);
    const float rw0 = env_row_weight(s, row), rw1 = env_row_weight(s, row + 1);
    const T q = (1.0f - d.y) * (1.0f + d.y);
    const T sinTheta = sqrt(fmax(q, 1e-6f));
    const T numer = (tlum(value1) * rw0 + tlum(value2) * rw1) * s.envNorm;
    const T aS = fabs(sinTheta);
    const T denom = fmax(aS, 1e-7f);
    const T dp = numer / denom;
    const T dpb = dpb_ + epb * env_position_pdf(s);
    const T numerb = dpb / denom;
    const T denomb = -dpb * dp / denom;
    const T sTb = fmax_active(aS, 1e-7f) ? denomb * sgn_of(sinTheta) : T(0.0f);
    TV3<T> db = tzero<T>();
    if (fmax_active(q, 1e-6f)) db.y = db.y + sTb * (0.5f / sinTheta) * (-2.0f * d.y);
    TV3<T> v1b = emb * L.samplingWeight, v2b = emb * L.samplingWeight;
    tlum_adj(numerb * (rw0 * s.envNorm), v1b);
    tlum_adj(numerb * (rw1 * s.envNorm), v2b);
    const T dx1b = dot(v1b, (R10 - R00) * dy2) + dot(v2b, (R11 - R01) * dy1);
    const T dy1b = -dot(v1b, R00 * dx2 + R10 * dx1) + dot(v2b, R01 * dx2 + R11 * dx1);
    const T g = dx1b * kInvTwoPi * float(s.envW);
    const T ir2 = 1.0f / (d.x * d.x + d.z * d.z);
    db.x = db.x + g * (-d.z) * ir2;
    db.z = db.z + g * d.x * ir2;
    db.y = db.y - dy1b * kInvPi * float(s.envH) / sqrt((1.0f - d.y) * (1.0f + d.y));
    dirb = dirb + TV3<T>(m[0] * db.x + m[3] * db.y + m[6] * db.z, m[1] * db.x + m[4] * db.y + m[7] * db.z,
                         m[2] * db.x + m[5] * db.y + m[8] * db.z);
}

template <class T>
DEV void concentric_disc_adj(const T &u0, const T &u1, const T &xb, const T &yb, T &u0b, T &u1b) {
    const T r1 = 2.0f * u0 - 1.0f;
    const T r2 = 2.0f * u1 - 1.0f;
    if (val(r1) == 0.0f || val(r2) == 0.0f) return;
    T r, phi;
    const bool first = val(r1) * val(r1) > val(r2) * val(r2);
    if (first) {
        r = r1;
        phi = kPiOverFour * (r2 / r1);
    } else {
        r = r2;
        phi = kPiOverTwo - (r1 / r2) * kPiOverFour;
    }
    const T c = cos(phi), sn = sin(phi);
    const T rb = xb * c + yb * sn;
    const T phib = r * (yb * c - xb * sn);
    T r1b(0.0f), r2b(0.0f);
    if (first) {
        r1b = rb - phib * kPiOverFour * r2 / (r1 * r1);
        r2b = phib * kPiOverFour / r1;
    } else {
        r2b = rb + phib * kPiOverFour * r1 / (r2 * r2);
        r1b = -phib * kPiOverFour / r2;
    }
    u0b = u0b + 2.0f * r1b;
    u1b = u1b + 2.0f * r2b;
}

// ad_sample_primary's direction from the film coordinates (its origin is constant).
template <class T>
DEV void sample_primary_dir_adj(const Camera &c, const T &sx, const T &sy, const TV3<T> &dirb, T &sxb, T &syb) {
    const float *S = c.sampleToCam;
    const T x = S[0] * sx + S[1] * sy + S[3];
    const T y = S[4] * sx + S[5] * sy + S[7];
    const T z = S[8] * sx + S[9] * sy + S[11];
    const T w = S[12] * sx + S[13] * sy + S[15];
    const T iw = 1.0f / w;
    const TV3<T> o(x * iw, y * iw, z * iw);
    const float *M = c.camToWorld;
    const TV3<T> db(M[0] * dirb.x + M[4] * dirb.y + M[8] * dirb.z, M[1] * dirb.x + M[5] * dirb.y + M[9] * dirb.z,
                    M[2] * dirb.x + M[6] * dirb.y + M[10] * dirb.z);
    TV3<T> ob = tzero<T>();
    tnorm_adj(o, db, ob);
    const T xb = ob.x * iw, yb = ob.y * iw, zb = ob.z * iw;
    const T wb = -(ob.x * o.x + ob.y * o.y + ob.z * o.z) * iw;
    sxb = sxb + S[0] * xb + S[4] * yb + S[8] * zb + S[12] * wb;
    syb = syb + S[1] * xb + S[5] * yb + S[9] * zb + S[13] * wb;
}


// ---------------------------------------------------------------- path-level sweep
// The state carried from one vertex to the next: the ray (origin, direction),
// the subpath throughput and the two MIS accumulators.
template <class T>
struct Carry {
    TV3<T> org, dir, tp;
    T prev, cur;
    HD void zero() {
        org = dir = tp = tzero<T>();
        prev = cur = T(0.0f);
    }
};
template <class T> HD void state_zero(TState<T> &v) {
    v.isect.position = v.isect.shadingNormal = v.isect.geomNormal = v.wi = v.throughput = tzero<T>();
    v.prev = v.cur = T(0.0f);
}

// How a vertex converts the MIS accumulators on arrival (ad_eval_path's three forms).
enum : int { kHitLightFirst = 0, kHitLightFirstEnv = 1, kHitGeneric = 2, kHitAreaLight = 3 };

template <class T>
DEV void hit_fwd(const SceneView &s, int tri, int kind, const Carry<T> &C, TState<T> &V) {
    ad_intersect(s, tri, C.org, C.dir, V.isect);
    V.wi = -C.dir;
    V.throughput = C.tp;
    V.prev = C.prev;
    V.cur = C.cur;
    const TV3<T> e = C.org - V.isect.position;
    if (kind == kHitLightFirst || kind == kHitLightFirstEnv || kind == kHitAreaLight) {
        const T conv = kind == kHitLightFirstEnv ? T(1.0f) : tmis(dot(e, e));
        const T invCos = 1.0f / tmis(fabs(dot(C.dir, V.isect.shadingNormal)));
        V.prev = V.prev * (invCos * conv);
        V.cur = V.cur * invCos;
    } else {
        V.prev = V.prev * tmis(dot(e, e));
        const T invCos = 1.0f / tmis(fabs(dot(C.dir, V.isect.shadingNormal)));
        V.prev = V.prev * invCos;
        V.cur = V.cur * invCos;
    }
}

// V: hit_fwd's output for C (its intersection is reused).
template <class T>
DEV void hit_adj(const SceneView &s, int tri, int kind, const Carry<T> &C, const TState<T> &V, const TState<T> &Vb,
                 Carry<T> &Cb) {
    const TIsect<T> &is = V.isect;
    const TV3<T> e = C.org - is.position;
    const T dd = dot(e, e);
    const T conv = kind == kHitLightFirstEnv ? T(1.0f) : dd * dd;
    const T q = dot(C.dir, is.shadingNormal);
    const T ic = 1.0f / (q * q);
    Cb.prev = Cb.prev + Vb.prev * ic * conv;
    Cb.cur = Cb.cur + Vb.cur * ic;
    Cb.tp = Cb.tp + Vb.throughput;
    const T icb = Vb.prev * C.prev * conv + Vb.cur * C.cur;
    const T convb = Vb.prev * C.prev * ic;
    const T qb = icb * (-2.0f) * ic / q;
    TV3<T> dirb = is.shadingNormal * qb - Vb.wi;
    TV3<T> snb = Vb.isect.shadingNormal + C.dir * qb;
    TV3<T> posb = Vb.isect.position;
    if (kind != kHitLightFirstEnv) {
        const TV3<T> eb = e * (4.0f * dd * convb);
        Cb.org = Cb.org + eb;
        posb = posb - eb;
    }
    intersect_adj(s, tri, C.org, C.dir, posb, snb, Cb.org, dirb);
    Cb.dir = Cb.dir + dirb;
}

// One BSDF sampling step at vertex vi: vertex state + (r0, r1) -> the next
// carry (adjoint: the light subpath's EvaluateBSDF(true, ...) forms).
template <class T>
DEV void step_fwd(const SceneView &s, const PathRec &r, int vi, int lcsTri, bool adjoint, const T &r0, const T &r1,
                  const TState<T> &V, Carry<T> &Cn) {
    TState<T> ps = V;
    TV3<T> dir;
    bsdf_sampling_fwd(s, r.tri[vi], r0, r1, r.disc[vi], (r.useAbs >> vi) & 1u, lcsTri, adjoint, ps, dir);
    Cn.tp = ps.throughput * r.rr[vi];
    Cn.org = V.isect.position;
    Cn.dir = dir;
    Cn.prev = ps.prev;
    Cn.cur = ps.cur;
}

template <class T>
DEV void step_adj(const SceneView &s, const PathRec &r, int vi, int lcsTri, bool adjoint, const T &r0, const T &r1,
                  const TState<T> &V, const Carry<T> &Cnb, TState<T> &Vb, T &r0b, T &r1b) {
    TState<T> nb;
    state_zero(nb);
    nb.throughput = Cnb.tp * r.rr[vi];
    nb.prev = Cnb.prev;
    nb.cur = Cnb.cur;
    Vb.isect.position = Vb.isect.position + Cnb.org;
    bsdf_sampling_adj(s, r.tri[vi], r0, r1, r.disc[vi], (r.useAbs >> vi) & 1u, lcsTri, adjoint, V, Cnb.dir, nb, Vb,
                      r0b, r1b);
}

// Light emission (EmitAreaLight / EmitEnvLight / EmitPointLight, AD forms):
// u[0..3] = (p0, p1, d0, d1) -> the first carry of the light subpath.
template <class T>
DEV void emit_fwd(const SceneView &s, const PathRec &r, const T *u, Carry<T> &C) {
    const Light &L = s.lights[r.lgtLight];
    const float pick = pick_light_prob(s, r.lgtLight);
    const T p0 = u[0], p1 = u[1], d0 = u[2], d1 = u[3];
    T cosLight, emissionPdf, directPdf;
    if (L.type == kLightArea) {
        TV3<T> nrm;
        ad_sample_triangle(s, light_tri(s, L, r.lgtPrim), p0, p1, C.org, nrm);
        const TV3<T> d = tcos_hemisphere(d0, d1);
        TV3<T> b0, b1;
        tframe(nrm, b0, b1);
        C.dir = d.x * b0 + d.y * b1 + d.z * nrm;
        C.tp = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]) * (kPi / L.invTotalArea));
        cosLight = d.z;
        emissionPdf = d.z * kInvPi * L.invTotalArea;
        directPdf = T(L.invTotalArea);
    } else if (L.type == kLightEnv) {
        TV3<T> value;
        ad_env_sample_direction(s, d0, d1, C.dir, value, directPdf);
        C.tp = value * L.samplingWeight;
        C.dir = -C.dir;
        T ox, oy;
        ad_concentric_disc(p0, p1, ox, oy);
        TV3<T> b0, b1;
        tframe(C.dir, b0, b1);
        const TV3<T> perp = ox * b0 + oy * b1;
        C.org = tv<T>(V3(s.bsCenter[0], s.bsCenter[1], s.bsCenter[2])) + (perp - C.dir) * s.bsRadius;
        cosLight = T(1.0f);
        emissionPdf = directPdf * env_position_pdf(s);
    } else {
        C.org = tv<T>(V3(L.pos[0], L.pos[1], L.pos[2]));
        const T scaledTheta = kTwoPi * d0;
        const T scaledPhi = kPi * d1;
        const T sinPhi = sin(scaledPhi);
        C.dir = TV3<T>(sinPhi * cos(scaledTheta), sinPhi * sin(scaledTheta), cos(scaledPhi));
        C.tp = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]));
        emissionPdf = T(1.0f / (4.0f * kPi));
        cosLight = T(1.0f);
        directPdf = T(1.0f);
    }
    emissionPdf = emissionPdf * pick;
    directPdf = directPdf * pick;
    C.tp = C.tp * (1.0f / pick);
    C.prev = tmis(directPdf / emissionPdf);
    C.cur = L.type == kLightPoint ? tmis(cosLight / emissionPdf) : T(0.0f);
}

template <class T>
DEV void emit_adj(const SceneView &s, const PathRec &r, const T *u, const Carry<T> &Cb, T *ub) {
    const Light &L = s.lights[r.lgtLight];
    const float pick = pick_light_prob(s, r.lgtLight);
    const T p0 = u[0], p1 = u[1], d0 = u[2], d1 = u[3];
    if (L.type == kLightArea) {
        TV3<T> org, nrm;
        const int tri = light_tri(s, L, r.lgtPrim);
        ad_sample_triangle(s, tri, p0, p1, org, nrm);
        const TV3<T> d = tcos_hemisphere(d0, d1);
        const T ep = d.z * kInvPi * L.invTotalArea * pick;
        const T k = T(L.invTotalArea * pick) / ep;
        const T epb = -2.0f * k * Cb.prev * k / ep;
        TV3<T> db = tzero<T>(), nrmb = tzero<T>();
        frame_apply_adj(d, nrm, Cb.dir, db, nrmb);
        db.z = db.z + epb * (kInvPi * L.invTotalArea * pick);
        tcos_hemisphere_adj(d0, d1, db, ub[2], ub[3]);
        sample_triangle_adj(s, tri, p0, p1, Cb.org, nrmb, ub[0], ub[1]);
    } else if (L.type == kLightEnv) {
        TV3<T> dir0, value;
        T dp;
        ad_env_sample_direction(s, d0, d1, dir0, value, dp);
        const TV3<T> dir = -dir0;
        T ox, oy;
        ad_concentric_disc(p0, p1, ox, oy);
        // prev = (dp pick / (dp pos pick))^2
        const float pos = env_position_pdf(s);
        const T dP = dp * pick, eP = dp * pos * pick;
        const T k = dP / eP;
        const T kb = 2.0f * k * Cb.prev;
        const T dpb = (kb / eP) * pick - (kb * k / eP) * (pos * pick);
        const TV3<T> valueb = Cb.tp * (L.samplingWeight * (1.0f / pick));
        // org = C + (perp - dir) R, perp = ox b0 + oy b1 (frame of dir)
        const TV3<T> perpb = Cb.org * s.bsRadius;
        TV3<T> dirb = Cb.dir - Cb.org * s.bsRadius;
        TV3<T> b0, b1;
        tframe(dir, b0, b1);
        const T oxb = dot(b0, perpb), oyb = dot(b1, perpb);
        tframe_adj(dir, perpb * ox, perpb * oy, dirb);
        concentric_disc_adj(p0, p1, oxb, oyb, ub[0], ub[1]);
        env_sample_direction_adj(s, d0, d1, -dirb, valueb, dpb, ub[2], ub[3]);
    } else {
        sphere_dir_adj(d0, d1, Cb.dir, T(0.0f), ub[2], ub[3]);
    }
}

// Camera start: (sx, sy) -> the first carry of the camera subpath.
template <class T>
DEV void camera_fwd(const SceneView &s, const T &sx, const T &sy, Carry<T> &C) {
    const float pixelCount = float(s.cam.width * s.cam.height);
    TV3<T> co, cd;
    ad_sample_primary(s.cam, T(0.5f), T(0.5f), co, cd);
    ad_sample_primary(s.cam, sx, sy, C.org, C.dir);
    const T cosAtCamera = dot(cd, C.dir);
    const T ip = s.cam.dist / cosAtCamera;
    const T cameraPdf = (ip * ip) / cosAtCamera;
    C.tp = TV3<T>(T(1.0f), T(1.0f), T(1.0f));
    C.prev = tmis(pixelCount / cameraPdf);
    C.cur = T(0.0f);
}

template <class T>
DEV void camera_adj(const SceneView &s, const T &sx, const T &sy, const Carry<T> &Cb, T &sxb, T &syb) {
    const float pixelCount = float(s.cam.width * s.cam.height);
    TV3<T> co, cd, org, dir;
    ad_sample_primary(s.cam, T(0.5f), T(0.5f), co, cd);
    ad_sample_primary(s.cam, sx, sy, org, dir);
    const T c = dot(cd, dir);
    const T ip = s.cam.dist / c;
    const T cameraPdf = (ip * ip) / c;
    const T k = pixelCount / cameraPdf;
    const T cpb = -2.0f * k * Cb.prev * k / cameraPdf;
    const T ipb = cpb * 2.0f * ip / c;
    const T cb = -cpb * cameraPdf / c - ipb * ip / c;
    sample_primary_dir_adj(s.cam, sx, sy, Cb.dir + cd * cb, sxb, syb);
}

// ConnectToCamera (AD) at the last light vertex V (technique c = 1).
template <class T>
DEV void connect_camera_adj(const SceneView &s, int tri, const TState<T> &V, TState<T> &Vb) {
    const float pixelCount = float(s.cam.width * s.cam.height);
    const Bsdf &b = bsdf_of_tri(s, tri);
    TV3<T> camOrg, camDir;
    ad_sample_primary(s.cam, T(0.5f), T(0.5f), camOrg, camDir);
    const TV3<T> dtc0 = camOrg - V.isect.position;
    const T distSq = dot(dtc0, dtc0);
    const T dist = sqrt(distSq);
    const T idist = 1.0f / dist;
    const TV3<T> dtc = dtc0 * idist;
    TBsdf<T> o;
    ad_evaluate(b, V.wi, V.isect.shadingNormal, dtc, o, true);
    const T sncv = ad_snc(V.wi, V.isect, dtc);
    const TV3<T> bsdfContrib = o.contrib * sncv;
    const T g = dot(camDir, dtc);
    const T ic = -(1.0f / g);
    const T ip = s.cam.dist * ic;
    const T i2sa = (ip * ip) * ic;
    const T i2s = i2sa * fabs(o.cosWo) / distSq;
    const T kk = i2s / pixelCount;
    const T rp2 = o.revPdf * o.revPdf;
    const T A = V.prev + V.cur * rp2;
    const T wLight = kk * kk * A;
    const T mis = 1.0f / (wLight + 1.0f);
    const T s2i = o.cosWo / i2s;
    const T denom = pixelCount * s2i;
    const T idn = 1.0f / denom;
    const TV3<T> mbc = mis * bsdfContrib;
    const TV3<T> cc = mbc * idn;
    const TV3<T> contribb = logf_seed(cmul(cc, V.throughput));
    // reverse
    const TV3<T> ccb = cmul(contribb, V.throughput);
    Vb.throughput = Vb.throughput + cmul(contribb, cc);
    const TV3<T> mbcb = ccb * idn;
    const T idnb = dot(mbc, ccb);
    const T denomb = -idnb * idn * idn;
    const T misb = dot(bsdfContrib, mbcb);
    const TV3<T> bcb = mbcb * mis;
    const T s2ib = denomb * pixelCount;
    TBsdfAdj<T> ob;
    ob.zero();
    ob.cosWo = s2ib / i2s;
    T i2sb = -s2ib * s2i / i2s;
    const T wLb = -misb * mis * mis;
    const T kkb = wLb * A * 2.0f * kk;
    Vb.prev = Vb.prev + wLb * kk * kk;
    Vb.cur = Vb.cur + wLb * kk * kk * rp2;
    ob.revPdf = wLb * kk * kk * V.cur * 2.0f * o.revPdf;
    i2sb = i2sb + kkb / pixelCount;
    const T aco = fabs(o.cosWo);
    const T i2sab = i2sb * aco / distSq;
    ob.cosWo = ob.cosWo + i2sb * i2sa * sgn_of(o.cosWo) / distSq;
    T distSqb = -i2sb * i2s / distSq;
    const T ipb = i2sab * 2.0f * ip * ic;
    const T icb = i2sab * ip * ip + ipb * s.cam.dist;
    const T gb = icb / (g * g);
    TV3<T> dtcb = camDir * gb;
    ob.contrib = bcb * sncv;
    const T sncb = dot(o.contrib, bcb);
    snc_adj(V.wi, V.isect, dtc, sncb, Vb.wi, Vb.isect.shadingNormal, dtcb);
    evaluate_adj(b, V.wi, V.isect.shadingNormal, dtc, FixedOb<T>{ob}, true, Vb.wi, Vb.isect.shadingNormal, dtcb);
    TV3<T> dtc0b = dtcb * idist;
    const T idistb = dot(dtc0, dtcb);
    const T distb = -idistb * idist * idist;
    distSqb = distSqb + distb * (0.5f / dist);
    dtc0b = dtc0b + dtc0 * (2.0f * distSqb);
    Vb.isect.position = Vb.isect.position - dtc0b;
}

// The camera ray leaves the scene: HandleHitLight with EmissionEnvLight (AD).
template <class T>
DEV void env_exit_adj(const SceneView &s, const Carry<T> &C, Carry<T> &Cb) {
    const Light &L = s.lights[s.envLight];
    TV3<T> emission;
    T dp, ep;
    ad_env_emission(s, L, C.dir, emission, dp, ep);
    const TV3<T> tpE = cmul(C.tp, emission);
    const float pick = pick_light_prob(s, s.envLight);
    const T dP = dp * pick, eP = ep * pick;
    const T wC = dP * dP * C.prev + eP * eP * C.cur;
    const T iS = 1.0f / (1.0f + wC);
    const TV3<T> contribb = logf_seed(tpE * iS);
    const TV3<T> tpEb = contribb * iS;
    const T wCb = -dot(tpE, contribb) * iS * iS;
    Cb.prev = Cb.prev + wCb * dP * dP;
    Cb.cur = Cb.cur + wCb * eP * eP;
    const T dpb = wCb * 2.0f * dP * C.prev * pick;
    const T epb = wCb * 2.0f * eP * C.cur * pick;
    Cb.tp = Cb.tp + cmul(tpEb, emission);
    env_emission_adj(s, L, C.dir, cmul(tpEb, C.tp), dpb, epb, Cb.dir);
}

// A camera ray that ends on an area light: HandleHitLight (AD), after the
// arrival's MIS conversion (hit kind kHitAreaLight).
template <class T>
DEV void area_hit_adj(const SceneView &s, int tri, const TState<T> &V, const TV3<T> &dir, TState<T> &Vb,
                      TV3<T> &dirb) {
    const int li = area_light_of_tri(s, tri);
    const Light &L = s.lights[li];
    const float pick = pick_light_prob(s, li);
    const TV3<T> E = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]));
    const T cal = -dot(V.isect.shadingNormal, dir);
    const T dP = T(L.invTotalArea * pick);
    const T eP = cal * L.invTotalArea * kInvPi * pick;
    const T wC = dP * dP * V.prev + eP * eP * V.cur;
    const T iS = 1.0f / (1.0f + wC);
    const TV3<T> tpE = cmul(V.throughput, E);
    const TV3<T> contribb = logf_seed(tpE * iS);
    const T wCb = -dot(tpE, contribb) * iS * iS;
    Vb.throughput = Vb.throughput + cmul(contribb * iS, E);
    Vb.prev = Vb.prev + wCb * dP * dP;
    Vb.cur = Vb.cur + wCb * eP * eP;
    const T calb = wCb * 2.0f * eP * V.cur * (L.invTotalArea * kInvPi * pick);
    Vb.isect.shadingNormal = Vb.isect.shadingNormal - dir * calb;
    dirb = dirb - V.isect.shadingNormal * calb;
}

// DirectLighting (AD) at the last camera vertex V, (r0, r1) the light sample.
template <class T>
DEV void direct_adj(const SceneView &s, const PathRec &r, int tri, const TState<T> &V, const T &r0, const T &r1,
                    TState<T> &Vb, T &r0b, T &r1b) {
    const Light &L = s.lights[r.dlLight];
    const Bsdf &b = bsdf_of_tri(s, tri);
    TV3<T> dtl, lc, dtl0, pl, nl2;
    T cal, dp, ep, distSq(0.0f), dist(0.0f);
    TV3<T> value;
    const TV3<T> E = tv<T>(V3(L.emission[0], L.emission[1], L.emission[2]));
    int ltri = -1;
    if (L.type == kLightArea) {
        ltri = light_tri(s, L, r.dlPrim);
        ad_sample_triangle(s, ltri, r0, r1, pl, nl2);
        dtl0 = pl - V.isect.position;
        distSq = dot(dtl0, dtl0);
        dist = sqrt(distSq);
        dtl = TV3<T>(dtl0.x / dist, dtl0.y / dist, dtl0.z / dist);
        cal = -dot(dtl, nl2);
        dp = L.invTotalArea * distSq / cal;
        lc = TV3<T>(E.x / dp, E.y / dp, E.z / dp);
        ep = L.invTotalArea * cal * kInvPi;
    } else if (L.type == kLightEnv) {
        ad_env_sample_direction(s, r0, r1, dtl, value, dp);
        lc = value * (1.0f / dp) * L.samplingWeight;
        cal = T(1.0f);
        ep = dp * env_position_pdf(s);
    } else {
        dtl0 = tv<T>(V3(L.pos[0], L.pos[1], L.pos[2])) - V.isect.position;
        distSq = dot(dtl0, dtl0);
        dp = distSq;
        dist = sqrt(distSq);
        dtl = TV3<T>(dtl0.x / dist, dtl0.y / dist, dtl0.z / dist);
        lc = E * (1.0f / distSq);
        ep = T(1.0f / (4.0f * kPi));
        cal = T(1.0f);
    }
    TBsdf<T> o;
    ad_evaluate(b, V.wi, V.isect.shadingNormal, dtl, o);
    const float pick = pick_light_prob(s, r.dlLight);
    const TV3<T> tp1 = cmul(V.throughput, o.contrib);
    const TV3<T> tp2 = cmul(tp1, lc) * (1.0f / pick);
    const bool point = L.type == kLightPoint;
    const T j = o.pdf / (pick * dp);
    const T wL = point ? T(0.0f) : j * j;
    const T num = ep * o.cosWo, den = dp * cal;
    const T kk = num / den;
    const T rp2 = o.revPdf * o.revPdf;
    const T A = V.prev + V.cur * rp2;
    const T wC = kk * kk * A;
    const T iS = 1.0f / (wL + 1.0f + wC);
    // reverse
    const TV3<T> contribb = logf_seed(tp2 * iS);
    const TV3<T> tp2b = contribb * iS;
    const T Sb = -dot(tp2, contribb) * iS * iS;
    const T kkb = Sb * A * 2.0f * kk;
    Vb.prev = Vb.prev + Sb * kk * kk;
    Vb.cur = Vb.cur + Sb * kk * kk * rp2;
    TBsdfAdj<T> ob;
    ob.revPdf = Sb * kk * kk * V.cur * 2.0f * o.revPdf;
    const T numb = kkb / den, denb = -kkb * kk / den;
    T epb = numb * o.cosWo;
    ob.cosWo = numb * ep;
    T dpb = denb * cal;
    T calb = denb * dp;
    ob.pdf = T(0.0f);
    if (!point) {
        const T jb = 2.0f * j * Sb;
        ob.pdf = jb / (pick * dp);
        dpb = dpb - jb * j / dp;
    }
    const TV3<T> tp1b = cmul(tp2b, lc) * (1.0f / pick);
    const TV3<T> lcb = cmul(tp2b, tp1) * (1.0f / pick);
    Vb.throughput = Vb.throughput + cmul(tp1b, o.contrib);
    ob.contrib = cmul(tp1b, V.throughput);
    TV3<T> dtlb = tzero<T>();
    evaluate_adj(b, V.wi, V.isect.shadingNormal, dtl, FixedOb<T>{ob}, false, Vb.wi, Vb.isect.shadingNormal, dtlb);
    if (L.type == kLightEnv) {
        dpb = dpb + epb * env_position_pdf(s) - dot(value, lcb) * L.samplingWeight / (dp * dp);
        env_sample_direction_adj(s, r0, r1, dtlb, lcb * (L.samplingWeight / dp), dpb, r0b, r1b);
        return;
    }
    T distSqb(0.0f);
    TV3<T> nl2b = tzero<T>();
    if (L.type == kLightArea) {
        calb = calb + epb * (L.invTotalArea * kInvPi);
        dpb = dpb - dot(E, lcb) / (dp * dp);
        distSqb = distSqb + dpb * L.invTotalArea / cal;
        calb = calb - dpb * dp / cal;
        dtlb = dtlb - nl2 * calb;
        nl2b = nl2b - dtl * calb;
    } else {
        distSqb = distSqb - dot(E, lcb) / (distSq * distSq) + dpb;
    }
    TV3<T> dtl0b = dtlb * (1.0f / dist);
    const T distb = -dot(dtl0, dtlb) / (dist * dist);
    distSqb = distSqb + distb * (0.5f / dist);
    dtl0b = dtl0b + dtl0 * (2.0f * distSqb);
    Vb.isect.position = Vb.isect.position - dtl0b;
    if (L.type == kLightArea) sample_triangle_adj(s, ltri, r0, r1, dtl0b, nl2b, r0b, r1b);
}

// ConnectVertex (AD): camera vertex V, light vertex W.
template <class T>
DEV void connect_adj(const SceneView &s, int ctri, int ltri, const TState<T> &V, const TState<T> &W,
                     TState<T> &Vb, TState<T> &Wb) {
    const Bsdf &bc = bsdf_of_tri(s, ctri), &bl = bsdf_of_tri(s, ltri);
    const TV3<T> dtl0 = W.isect.position - V.isect.position;
    const T distSq = dot(dtl0, dtl0);
    const T dist = sqrt(distSq);
    const T idist = 1.0f / dist;
    const TV3<T> dtl = dtl0 * idist;
    TBsdf<T> cb, lb;
    ad_evaluate(bc, V.wi, V.isect.shadingNormal, dtl, cb);
    ad_evaluate(bl, W.wi, W.isect.shadingNormal, -dtl, lb, true);
    const T snl = ad_snc(W.wi, W.isect, -dtl);
    const TV3<T> lgtF = lb.contrib * snl;
    const T G = 1.0f / distSq;
    const T camA = cb.pdf * lb.cosWo * G;
    const T lgtA = lb.pdf * cb.cosWo * G;
    const T lrp2 = lb.revPdf * lb.revPdf, crp2 = cb.revPdf * cb.revPdf;
    const T AL = W.prev + W.cur * lrp2, AC = V.prev + V.cur * crp2;
    const T wL = camA * camA * AL, wC = lgtA * lgtA * AC;
    const T mis = 1.0f / (wL + 1.0f + wC);
    const TV3<T> t1 = cmul(W.throughput, V.throughput);
    const TV3<T> t2 = cmul(t1, cb.contrib);
    const TV3<T> t3 = cmul(t2, lgtF);
    // reverse
    const TV3<T> contribb = logf_seed(t3 * (G * mis));
    const TV3<T> t3b = contribb * (G * mis);
    const T gmb = dot(t3, contribb);
    T Gb = gmb * mis;
    const T misb = gmb * G;
    const TV3<T> t2b = cmul(t3b, lgtF);
    const TV3<T> lgtFb = cmul(t3b, t2);
    const TV3<T> t1b = cmul(t2b, cb.contrib);
    TBsdfAdj<T> cbb, lbb;
    cbb.contrib = cmul(t2b, t1);
    Wb.throughput = Wb.throughput + cmul(t1b, V.throughput);
    Vb.throughput = Vb.throughput + cmul(t1b, W.throughput);
    const T Sb = -misb * mis * mis;
    const T camAb = Sb * 2.0f * camA * AL;
    const T lgtAb = Sb * 2.0f * lgtA * AC;
    Wb.prev = Wb.prev + Sb * camA * camA;
    Wb.cur = Wb.cur + Sb * camA * camA * lrp2;
    lbb.revPdf = Sb * camA * camA * W.cur * 2.0f * lb.revPdf;
    Vb.prev = Vb.prev + Sb * lgtA * lgtA;
    Vb.cur = Vb.cur + Sb * lgtA * lgtA * crp2;
    cbb.revPdf = Sb * lgtA * lgtA * V.cur * 2.0f * cb.revPdf;
    cbb.pdf = camAb * lb.cosWo * G;
    lbb.cosWo = camAb * cb.pdf * G;
    lbb.pdf = lgtAb * cb.cosWo * G;
    cbb.cosWo = lgtAb * lb.pdf * G;
    Gb = Gb + camAb * cb.pdf * lb.cosWo + lgtAb * lb.pdf * cb.cosWo;
    T distSqb = -Gb * G * G;
    lbb.contrib = lgtFb * snl;
    const T snlb = dot(lb.contrib, lgtFb);
    TV3<T> mdb = tzero<T>();
    snc_adj(W.wi, W.isect, -dtl, snlb, Wb.wi, Wb.isect.shadingNormal, mdb);
    evaluate_adj(bl, W.wi, W.isect.shadingNormal, -dtl, FixedOb<T>{lbb}, true, Wb.wi, Wb.isect.shadingNormal, mdb);
    TV3<T> dtlb = -mdb;
    evaluate_adj(bc, V.wi, V.isect.shadingNormal, dtl, FixedOb<T>{cbb}, false, Vb.wi, Vb.isect.shadingNormal, dtlb);
    TV3<T> dtl0b = dtlb * idist;
    const T idistb = dot(dtl0, dtlb);
    distSqb = distSqb - idistb * idist * idist * (0.5f / dist);
    dtl0b = dtl0b + dtl0 * (2.0f * distSqb);
    Wb.isect.position = Wb.isect.position + dtl0b;
    Vb.isect.position = Vb.isect.position - dtl0b;
}

// Gradient and Hessian row `row` of log f of path r at its own primary vector
// (dimension dim): one forward sweep in Dual numbers seeded in u_row, keeping
// the carry of every vertex, and one backward sweep. g (when non-null) gets
// the gradient, H[row * dim + k] and H[k * dim + row] the row from k = row on.
DEV void adj_row(const SceneView &s, const PathRec &r, int dim, int row, float *g, float *H) {
    using T = Dual;
    T u[kMaxDim], ub[kMaxDim];
    for (int k = 0; k < dim; k++) {
        u[k] = Dual(r.u[k], k == row ? 1.0f : 0.0f);
        ub[k] = Dual(0.0f);
    }
    const int c = r.c, l = r.l;
    const int nl = n_lgt(l), nc = c - 1;
    Carry<T> ck[kMaxLen];
    Carry<T> C;
    TState<T> lpFinal, V;
    const bool envLight = l > 1 && s.lights[r.lgtLight].type == kLightEnv;
    int k = 0;
    // ---- forward
    if (l > 1) {
        emit_fwd(s, r, u, C);
        k = 4;
        #pragma unroll 1
        for (int d = 0; d < nl; d++) {
            ck[d] = C;
            const int kind = d == 0 ? (envLight ? kHitLightFirstEnv : kHitLightFirst) : kHitGeneric;
            hit_fwd(s, r.tri[d], kind, C, V);
            if (d == nl - 1) {
                lpFinal = V;
                break;
            }
            step_fwd(s, r, d, -1, true, u[k], u[k + 1], V, C);
            k += 2;
        }
    }
    const int kc0 = k;
    int lcsTri = -1;
    if (c > 1) {
        camera_fwd(s, u[k], u[k + 1], C);
        k += 2;
        #pragma unroll 1
        for (int d = 0; d < nc; d++) {
            const int vi = nl + d;
            const int tri = r.tri[vi];
            ck[vi] = C;
            // the last vertex and its connection: in the backward sweep, which
            // evaluates the contribution (and with it log f's seed) there
            if (d == nc - 1) break;
            hit_fwd(s, tri, kHitGeneric, C, V);
            if (l == 0 && d == nc - 2 && s.opt.useLightCoordinateSampling) {
                const int lastTri = r.tri[nl + nc - 1];
                const int li = lastTri >= 0 ? area_light_of_tri(s, lastTri) : -1;
                if (li >= 0 && s.lights[li].type == kLightArea) lcsTri = lastTri;
            }
            step_fwd(s, r, vi, d == nc - 2 ? lcsTri : -1, false, u[k], u[k + 1], V, C);
            k += 2;
        }
    }
    // ---- backward: f = log(lum(contrib)), seeded in the final connection's adjoint
    TState<T> lpb;
    state_zero(lpb);
    if (c > 1) {
        Carry<T> Cb;
        Cb.zero();
        {
            const int d = nc - 1, vi = nl + d, tri = r.tri[vi];
            const Carry<T> &Cv = ck[vi];
            if (l == 0 && tri < 0) {
                env_exit_adj(s, Cv, Cb);
            } else {
                const int kind = l == 0 ? kHitAreaLight : kHitGeneric;
                hit_fwd(s, tri, kind, Cv, V);
                TState<T> Vb;
                state_zero(Vb);
                if (l == 0) {
                    TV3<T> dirb = tzero<T>();
                    area_hit_adj(s, tri, V, Cv.dir, Vb, dirb);
                    Cb.dir = Cb.dir + dirb;
                } else if (l == 1) {
                    const int kd = kc0 + 2 + 2 * d;
                    direct_adj(s, r, tri, V, u[kd], u[kd + 1], Vb, ub[kd], ub[kd + 1]);
                } else {
                    connect_adj(s, tri, r.tri[nl - 1], V, lpFinal, Vb, lpb);
                }
                hit_adj(s, tri, kind, Cv, V, Vb, Cb);
            }
        }
        #pragma unroll 1
        for (int d = nc - 2; d >= 0; d--) {
            const int vi = nl + d, tri = r.tri[vi];
            const int kd = kc0 + 2 + 2 * d;
            hit_fwd(s, tri, kHitGeneric, ck[vi], V);
            TState<T> Vb;
            state_zero(Vb);
            step_adj(s, r, vi, d == nc - 2 ? lcsTri : -1, false, u[kd], u[kd + 1], V, Cb, Vb, ub[kd], ub[kd + 1]);
            Cb.zero();
            hit_adj(s, tri, kHitGeneric, ck[vi], V, Vb, Cb);
        }
        camera_adj(s, u[kc0], u[kc0 + 1], Cb, ub[kc0], ub[kc0 + 1]);
    } else if (l > 1) {
        connect_camera_adj(s, r.tri[nl - 1], lpFinal, lpb);
    }
    if (l > 1) {
        Carry<T> Cb;
        Cb.zero();
        {
            const int d = nl - 1;
            const int kind = d == 0 ? (envLight ? kHitLightFirstEnv : kHitLightFirst) : kHitGeneric;
            hit_adj(s, r.tri[d], kind, ck[d], lpFinal, lpb, Cb);
        }
        #pragma unroll 1
        for (int d = nl - 2; d >= 0; d--) {
            const int kind = d == 0 ? (envLight ? kHitLightFirstEnv : kHitLightFirst) : kHitGeneric;
            const int kd = 4 + 2 * d;
            hit_fwd(s, r.tri[d], kind, ck[d], V);
            TState<T> Vb;
            state_zero(Vb);
            step_adj(s, r, d, -1, true, u[kd], u[kd + 1], V, Cb, Vb, ub[kd], ub[kd + 1]);
            Cb.zero();
            hit_adj(s, r.tri[d], kind, ck[d], V, Vb, Cb);
        }
        emit_adj(s, r, u, Cb, ub);
    }
    // row `row` of the Hessian from j = row on, mirrored: entry (i, j), i < j, is
    // written by row i's pass alone, so a team writes a symmetric matrix
    for (int j = row; j < dim; j++) {
        H[row * dim + j] = ub[j].d;
        H[j * dim + row] = ub[j].d;
    }
    if (g)
        for (int j = 0; j < dim; j++) g[j] = ub[j].v;
}

}  // namespace drmlt
