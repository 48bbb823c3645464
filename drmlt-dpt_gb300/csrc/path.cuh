// Bidirectional path sampling and perturbation for one Markov chain per thread.
//
// The control flow, MIS bookkeeping and random-number order follow
//   GeneratePathBidir   src/path.cpp:978-1121
//   GenerateSubpath     src/path.cpp:1123-1269
//   PerturbPathBidir    src/path.cpp:1480-1628
//   GeneratePath        src/path.cpp:343-445 (direct-lighting pass, depth <= 2)
// and the vertex operations they call (src/path.cpp:27-976, 1430-1478).
// Pairs of uniforms the reference draws as Vector2(u(), u()) are assigned
// second-component-first, because the reference's compiler evaluates those
// constructor arguments right to left; a replayed stream then reproduces the
// reference's paths. Lens-mutation quantities (lensContrib / lensScore) are not
// tracked here: the DR integrator never reads them; integrator=h2mc's lens
// mutation takes them by a walk of its own (lens.cuh).
#pragma once
#include "bsdf_light.cuh"

namespace drmlt {

// A technique path: what one Markov state stores between iterations.
// c = camDepth, l = lightDepth in the reference's SubpathContrib notation.
// Surface vertices: nLgt = max(l-1,0) light-subpath vertices first, then
// nCam = c-1 camera-subpath vertices. u[] holds the primary sample vector in
// GetPathPos order (src/path.cpp:2393-2439), dimension 2(c+l-1).
struct PathRec {
    int c, l;
    int lgtLight, lgtPrim;
    int dlLight, dlPrim;
    unsigned useAbs;  // bit v: vertex v's useAbsoluteParam; bit 31: kLensFormBit (lens.cuh)
    float u[kMaxDim];
    int tri[kMaxVerts];
    float disc[kMaxVerts];
    float rr[kMaxVerts];
};

// PathRec::useAbs bit 31, above the per-vertex bits: the path was made by
// integrator=h2mc's lens mutation (PerturbLensBidir), whose lens score of a
// light path connected to the camera carries a shading-normal factor of its
// own (lens.cuh). The other samplers clear it.
constexpr unsigned kLensFormBit = 1u << 31;

struct Contrib {
    float screen[2];
    float rgb[3];
    float ls, ss;
    int valid;
};

DEV int path_dim(int c, int l) { return 2 * (c + l - 1); }
DEV int n_lgt(int l) { return l > 1 ? l - 1 : 0; }

// BidirPathState of src/path.cpp:447-458 without lensContrib.
struct BState {
    Isect isect;
    V3 wi;
    float accMISWPrev, accMISWThis;
    V3 throughput;
    float ssJacobian, lcJacobian, lastBsdfPdf;
};

DEV void zero_state(BState &s) {
    s.throughput = V3(0.0f, 0.0f, 0.0f);
    s.accMISWPrev = s.accMISWThis = 0.0f;
    s.ssJacobian = s.lcJacobian = s.lastBsdfPdf = 0.0f;
}

// Per-vertex record kept while sampling (SurfaceVertex, src/path.h:34-42).
struct SVert {
    int tri;
    float rnd[2];
    float disc;
    float rr;
    int useAbs;
    int dlLight, dlPrim;
    float dl[2];
};

DEV void clear_vert(SVert &v) {
    v.tri = -1;
    v.rnd[0] = v.rnd[1] = 0.0f;
    v.disc = 0.0f;
    v.rr = 0.0f;
    v.useAbs = 0;
    v.dlLight = -1;
    v.dlPrim = -1;
    v.dl[0] = v.dl[1] = 0.0f;
}

DEV const Bsdf &bsdf_of_tri(const SceneView &s, int tri) { return s.bsdfs[s.shapes[s.triShape[tri]].bsdf]; }
DEV int area_light_of_tri(const SceneView &s, int tri) { return s.shapes[s.triShape[tri]].areaLight; }

struct Emit {  // a contribution produced by one technique
    int c, l;
    float screen[2];
    V3 rgb;
    float ls, ss;
};

// ---------------------------------------------------------------- vertex ops
DEV void emit_from_camera(const SceneView &s, float sx, float sy, V3 &org, V3 &dir, float &minT, float &maxT,
                          BState &ps) {
    V3 co, cd;
    float a, b;
    sample_primary(s.cam, 0.5f, 0.5f, co, cd, a, b);
    sample_primary(s.cam, sx, sy, org, dir, minT, maxT);
    const float cosAtCamera = dot(cd, dir);
    const float imagePointToCameraDist = s.cam.dist / cosAtCamera;
    const float imageToSolidAngleFactor = sq(imagePointToCameraDist) / cosAtCamera;
    const float screenPixelCount = float(s.cam.width * s.cam.height);
    ps.throughput = V3(1.0f, 1.0f, 1.0f);
    ps.accMISWPrev = mis(screenPixelCount / imageToSolidAngleFactor);
    ps.accMISWThis = 0.0f;
    ps.ssJacobian = 1.0f;
}

DEV void emit_from_light(const SceneView &s, float pickProb, int light, int lPrim, const float pos[2],
                         const float dirp[2], V3 &org, V3 &dir, BState &ps) {
    float cosLight, emissionPdf, directPdf;
    light_emit(s, light, lPrim, pos[0], pos[1], dirp[0], dirp[1], org, dir, ps.throughput, cosLight,
               emissionPdf, directPdf);
    emissionPdf *= pickProb;
    directPdf *= pickProb;
    ps.throughput = ps.throughput * (1.0f / pickProb);
    ps.accMISWPrev = mis(directPdf / emissionPdf);
    ps.accMISWThis = !light_is_delta(s, light) ? mis(cosLight / emissionPdf) : 0.0f;
    ps.ssJacobian = 1.0f;
}

// ConvertMIS (src/path.cpp:507-516). light < 0: camera subpath.
DEV void convert_mis(const SceneView &s, int depth, int light, const V3 &rayOrg, const V3 &rayDir, BState &ps) {
    if (depth > 0 || light < 0 || light_is_finite(s, light))
        ps.accMISWPrev *= mis(dist_sq(rayOrg, ps.isect.position));
    const float invCosTheta = 1.0f / mis(fabsf(dot(rayDir, ps.isect.shadingNormal)));
    ps.accMISWPrev *= invCosTheta;
    ps.accMISWThis *= invCosTheta;
}

// The shadow ray of a connection: the connection contributes iff nothing lies
// on (org, org + dist * dir) (Occluded, src/scene.cpp:95-105).
struct Shadow {
    V3 org, dir;
    float dist;
};

// The connections below are split in two: *_pre does every test and the whole
// evaluation except the visibility test and returns the shadow ray; the
// connection contributes iff *_pre succeeds and the ray is not occluded. The
// reference casts the shadow ray first, but the cast has no side effect and
// every failing test returns false, so the order does not change any result.
// This lets the wavefront sampler queue the shadow ray like any other ray.

// ConnectToCamera (src/path.cpp:518-606).
DEV bool connect_to_camera_pre(const SceneView &s, int lgtDepth, const BState &ps, const SVert &v, Emit &e,
                               Shadow &sh) {
    V3 camOrg, camDir;
    float a, b;
    sample_primary(s.cam, 0.5f, 0.5f, camOrg, camDir, a, b);
    V3 dirToCamera = camOrg - ps.isect.position;
    if (-dot(camDir, dirToCamera) <= 0.0f) return false;
    float sx, sy;
    if (!project_point(s.cam, ps.isect.position, sx, sy)) return false;
    const float distSq = length_sq(dirToCamera);
    const float dist = sqrtf(distSq);
    dirToCamera = dirToCamera * (1.0f / dist);
    sh.org = ps.isect.position;
    sh.dir = dirToCamera;
    sh.dist = dist;
    const Bsdf &bsdf = bsdf_of_tri(s, v.tri);
    BsdfOut bo;
    bsdf_evaluate<true>(bsdf, ps.wi, ps.isect.shadingNormal, dirToCamera, bo);
    if (is_zero(bo.contrib)) return false;
    const float factor = shading_normal_correction<true>(ps.wi, ps.isect, dirToCamera);
    if (factor <= 0.0f) return false;
    V3 bsdfContrib = bo.contrib * factor;
    const float cosAtCamera = -dot(camDir, dirToCamera);
    const float imagePointToCameraDist = s.cam.dist / cosAtCamera;
    const float imageToSolidAngleFactor = sq(imagePointToCameraDist) / cosAtCamera;
    const float imageToSurfaceFactor = imageToSolidAngleFactor * fabsf(bo.cosWo) / distSq;
    const float screenPixelCount = float(s.cam.width * s.cam.height);
    const float cameraPdf = imageToSurfaceFactor;
    const float wLight = mis(cameraPdf / screenPixelCount) * (ps.accMISWPrev + ps.accMISWThis * mis(bo.revPdf));
    const float misWeight = 1.0f / (wLight + 1.0f);
    const float surfaceToImageFactor = bo.cosWo / imageToSurfaceFactor;
    const float denom = screenPixelCount * surfaceToImageFactor;
    V3 contrib((misWeight * bsdfContrib.x) / denom, (misWeight * bsdfContrib.y) / denom,
               (misWeight * bsdfContrib.z) / denom);
    contrib = cmul(contrib, ps.throughput);
    const float score = luminance(contrib);
    if (!(score > 0.0f)) return false;
    e.c = 1;
    e.l = 2 + lgtDepth;
    e.screen[0] = sx;
    e.screen[1] = sy;
    e.rgb = contrib;
    e.ls = score;
    e.ss = score * ps.ssJacobian;
    return true;
}
DEV bool connect_to_camera(const SceneView &s, int lgtDepth, const BState &ps, const SVert &v, Emit &e) {
    Shadow sh;
    return connect_to_camera_pre(s, lgtDepth, ps, v, e, sh) && !occluded(s, sh.org, sh.dir, sh.dist);
}

// BSDFSampling<adjoint, perturb> (src/path.cpp:608-724). `next` may alias `ps`;
// freshNext marks a newly pushed state, whose ssJacobian the reference leaves
// zero-initialised when the relative parameterisation is used.
template <bool adjoint, bool perturb>
DEV bool bsdf_sampling(const SceneView &s, const BState &ps, SVert &v, BState &next, bool freshNext, V3 &dir,
                       V3 &bsdfContrib) {
    const Bsdf &bsdf = bsdf_of_tri(s, v.tri);
    v.useAbs = bsdf_roughness(bsdf, v.disc) > s.opt.roughnessThreshold;
    BsdfOut bo;
    float nextSsJ;
    float nextLcJ;
    if (!perturb || !v.useAbs) {
        if (!bsdf_sample<adjoint>(bsdf, ps.wi, ps.isect.shadingNormal, v.rnd[0], v.rnd[1], v.disc, dir, bo)) return false;
        if (v.useAbs) {
            float jac;
            to_spherical(dir, v.rnd[0], v.rnd[1], jac);
            nextLcJ = 1.0f / jac;
            jac *= bo.pdf;
            nextSsJ = ps.ssJacobian * jac;
        } else {
            nextLcJ = bo.pdf;
            nextSsJ = freshNext ? 0.0f : ps.ssJacobian;
        }
    } else {
        float jac;
        dir = sample_sphere(v.rnd[0], v.rnd[1], jac);
        bsdf_evaluate<adjoint>(bsdf, ps.wi, ps.isect.shadingNormal, dir, bo);
        if (is_zero(bo.contrib) || bo.pdf <= 0.0f) return false;
        bo.contrib = bo.contrib * (1.0f / bo.pdf);
        nextLcJ = 1.0f / jac;
        jac *= bo.pdf;
        nextSsJ = ps.ssJacobian * jac;
    }
    const float factor = shading_normal_correction<adjoint>(ps.wi, ps.isect, dir);
    if (factor <= 0.0f) return false;
    bsdfContrib = bo.contrib * factor;
    const float newThis = mis(bo.cosWo / bo.pdf) * (ps.accMISWThis * mis(bo.revPdf) + ps.accMISWPrev);
    const V3 newT = cmul(ps.throughput, bsdfContrib);
    next.lcJacobian = nextLcJ;
    next.ssJacobian = nextSsJ;
    next.lastBsdfPdf = bo.pdf;
    next.accMISWThis = newThis;
    next.accMISWPrev = mis(1.0f / bo.pdf);
    next.throughput = newT;
    return true;
}

// DirectLighting, bidirectional form (src/path.cpp:726-811).
DEV bool direct_lighting_pre(const SceneView &s, int camDepth, const BState &ps, float sx, float sy, float pickProb,
                             const SVert &v, Emit &e, Shadow &sh) {
    V3 dirToLight, lightContrib;
    float dist, cosAtLight, directPdf, emissionPdf;
    if (!light_sample_direct(s, v.dlLight, v.dlPrim, ps.isect.position, v.dl[0], v.dl[1], dirToLight, dist,
                             lightContrib, cosAtLight, directPdf, emissionPdf))
        return false;
    sh.org = ps.isect.position;
    sh.dir = dirToLight;
    sh.dist = dist;
    const Bsdf &bsdf = bsdf_of_tri(s, v.tri);
    BsdfOut bo;
    bsdf_evaluate(bsdf, ps.wi, ps.isect.shadingNormal, dirToLight, bo);
    if (is_zero(bo.contrib)) return false;
    const float factor = shading_normal_correction<false>(ps.wi, ps.isect, dirToLight);
    if (factor <= 0.0f) return false;
    const V3 bsdfContrib = bo.contrib * factor;
    V3 contrib = cmul(ps.throughput, bsdfContrib);
    contrib = cmul(contrib, lightContrib) * (1.0f / pickProb);
    const float wLight = light_is_delta(s, v.dlLight) ? 0.0f : mis(bo.pdf / (pickProb * directPdf));
    const float wCamera = mis(emissionPdf * bo.cosWo / (directPdf * cosAtLight)) *
                          (ps.accMISWPrev + ps.accMISWThis * mis(bo.revPdf));
    const float misWeight = 1.0f / (wLight + 1.0f + wCamera);
    contrib = contrib * misWeight;
    const float score = luminance(contrib);
    if (!(score > 0.0f)) return false;
    e.c = 2 + camDepth;
    e.l = 1;
    e.screen[0] = sx;
    e.screen[1] = sy;
    e.rgb = contrib;
    e.ls = score;
    e.ss = score * ps.ssJacobian;
    return true;
}
DEV bool direct_lighting(const SceneView &s, int camDepth, const BState &ps, float sx, float sy, float pickProb,
                         const SVert &v, Emit &e) {
    Shadow sh;
    return direct_lighting_pre(s, camDepth, ps, sx, sy, pickProb, v, e, sh) && !occluded(s, sh.org, sh.dir, sh.dist);
}

// HandleHitLight, bidirectional form (src/path.cpp:813-865).
DEV bool handle_hit_light(const SceneView &s, int camDepth, int light, const V3 &rayDir, float sx, float sy,
                          const BState &ps, Emit &e) {
    V3 emission;
    float directPdf, emissionPdf;
    light_emission(s, light, rayDir, ps.isect.shadingNormal, emission, directPdf, emissionPdf);
    if (!(emission.x + emission.y + emission.z > 0.0f)) return false;
    V3 contrib = cmul(ps.throughput, emission);
    if (camDepth > 0) {
        const float pick = pick_light_prob(s, light);
        directPdf *= pick;
        emissionPdf *= pick;
        const float wCamera = mis(directPdf) * ps.accMISWPrev + mis(emissionPdf) * ps.accMISWThis;
        contrib = contrib * (1.0f / (1.0f + wCamera));
    }
    const float score = luminance(contrib);
    if (!(score > 0.0f)) return false;
    e.c = 2 + camDepth;
    e.l = 0;
    e.screen[0] = sx;
    e.screen[1] = sy;
    e.rgb = contrib;
    e.ls = score;
    e.ss = score * ps.ssJacobian;
    return true;
}

// ConnectVertex (src/path.cpp:867-976).
DEV bool connect_vertex_pre(const SceneView &s, int camDepth, int lgtDepth, const BState &lp, const SVert &lv,
                            const BState &cp, const SVert &cv, float sx, float sy, Emit &e, Shadow &sh) {
    V3 dirToLight = lp.isect.position - cp.isect.position;
    const float distSq = length_sq(dirToLight);
    const float dist = sqrtf(distSq);
    dirToLight = dirToLight * (1.0f / dist);
    sh.org = cp.isect.position;
    sh.dir = dirToLight;
    sh.dist = dist;
    BsdfOut cb;
    bsdf_evaluate(bsdf_of_tri(s, cv.tri), cp.wi, cp.isect.shadingNormal, dirToLight, cb);
    if (is_zero(cb.contrib)) return false;
    const float camFactor = shading_normal_correction<false>(cp.wi, cp.isect, dirToLight);
    if (camFactor <= 0.0f) return false;
    const V3 camF = cb.contrib * camFactor;
    BsdfOut lb;
    bsdf_evaluate<true>(bsdf_of_tri(s, lv.tri), lp.wi, lp.isect.shadingNormal, -dirToLight, lb);
    if (is_zero(lb.contrib)) return false;
    const float lgtFactor = shading_normal_correction<true>(lp.wi, lp.isect, -dirToLight);
    if (lgtFactor <= 0.0f) return false;
    const V3 lgtF = lb.contrib * lgtFactor;
    const float G = 1.0f / distSq;
    const float camBsdfDirPdfA = cb.pdf * lb.cosWo * G;
    const float lgtBsdfDirPdfA = lb.pdf * cb.cosWo * G;
    const float wLight = mis(camBsdfDirPdfA) * (lp.accMISWPrev + lp.accMISWThis * mis(lb.revPdf));
    const float wCamera = mis(lgtBsdfDirPdfA) * (cp.accMISWPrev + cp.accMISWThis * mis(cb.revPdf));
    const float misWeight = 1.0f / (wLight + 1.0f + wCamera);
    const V3 T = cmul(lp.throughput, cp.throughput);
    V3 contrib = cmul(T, camF);
    contrib = cmul(contrib, lgtF) * G;
    contrib = contrib * misWeight;
    const float ssJ = lp.ssJacobian * cp.ssJacobian;
    const float score = luminance(contrib);
    if (!(score > 0.0f)) return false;
    e.c = 2 + camDepth;
    e.l = 2 + lgtDepth;
    e.screen[0] = sx;
    e.screen[1] = sy;
    e.rgb = contrib;
    e.ls = score;
    e.ss = score * ssJ;
    return true;
}
DEV bool connect_vertex(const SceneView &s, int camDepth, int lgtDepth, const BState &lp, const SVert &lv,
                        const BState &cp, const SVert &cv, float sx, float sy, Emit &e) {
    Shadow sh;
    return connect_vertex_pre(s, camDepth, lgtDepth, lp, lv, cp, cv, sx, sy, e, sh) &&
           !occluded(s, sh.org, sh.dir, sh.dist);
}

// LightCoordinateSampling, bidirectional form (src/path.cpp:1430-1478). The
// path continues from ps along `dir` only if the shadow ray is clear.
DEV bool light_coordinate_sampling_pre(const SceneView &s, const SVert &cur, int nextTri, BState &ps, V3 &dir,
                                       V3 &bsdfContrib, Shadow &sh) {
    V3 nextPos, nextNormal;
    sample_triangle(s, nextTri, cur.rnd[0], cur.rnd[1], nextPos, nextNormal);
    dir = nextPos - ps.isect.position;
    const float distToLightSq = length_sq(dir);
    const float distToLight = sqrtf(distToLightSq);
    dir = dir * (1.0f / distToLight);
    sh.org = ps.isect.position;
    sh.dir = dir;
    sh.dist = distToLight;
    BsdfOut bo;
    bsdf_evaluate(bsdf_of_tri(s, cur.tri), ps.wi, ps.isect.shadingNormal, dir, bo);
    if (is_zero(bo.contrib)) return false;
    bsdfContrib = bo.contrib * (1.0f / bo.pdf);
    ps.throughput = cmul(ps.throughput, bsdfContrib);
    ps.ssJacobian *= fabsf(dot(dir, nextNormal) * (1.0f / distToLightSq)) * bo.pdf;
    ps.accMISWThis = mis(bo.cosWo / bo.pdf) * (ps.accMISWThis * mis(bo.revPdf) + ps.accMISWPrev);
    ps.accMISWPrev = mis(1.0f / bo.pdf);
    return true;
}

// RussianRoulette (src/path.cpp:325-341): always consumes one uniform.
template <class R>
DEV bool russian_roulette(int depth, const V3 &bsdfContrib, float &rrWeight, V3 &throughput, R &rng) {
    float rrProb = 1.0f;
    if (depth >= 3) rrProb = fminf(max_coeff(bsdfContrib), 0.95f);
    if (rng.uniform() > rrProb) return false;
    rrWeight = 1.0f / rrProb;
    throughput = throughput * rrWeight;
    return true;
}

// Light-coordinate re-parameterisation when a camera subpath hits an area light
// (src/path.cpp:1056-1071 and 1208-1223).
// prevRnd0/1: the direction parameters of the previous camera vertex, rewritten
// as the light triangle's sample parameters.
DEV void light_coordinate_convert(const SceneView &s, float &prevRnd0, float &prevRnd1, int lightTri,
                                  const V3 &rayOrg, BState &ps) {
    triangle_sample_param(s, lightTri, ps.isect.position, prevRnd0, prevRnd1);
    V3 dirToPrev = ps.isect.position - rayOrg;
    const float distSq = length_sq(dirToPrev);
    const float invDistSq = 1.0f / distSq;
    const float invDist = sqrtf(invDistSq);
    dirToPrev = dirToPrev * invDist;
    const Light &L = s.lights[area_light_of_tri(s, lightTri)];
    ps.ssJacobian *= fabsf(dot(dirToPrev, ps.isect.shadingNormal) * invDistSq) * (ps.lcJacobian * L.invTotalArea);
}

// ---------------------------------------------------------------- full bootstrap sample
struct FullPath {
    float time;
    float lgtPos[2], lgtDir[2];
    int lgtLight, lgtPrim;
    float screen[2];
    int nLgt, nCam;
    SVert lgt[kMaxFull];
    SVert cam[kMaxFull];
};

// Builds the technique path (c, l) from a full bootstrap sample, the way
// Path::Initialize truncates it (src/path.h:109-120) and GetPathPos orders it.
DEV void make_rec(const FullPath &f, int c, int l, PathRec &r) {
    r.c = c;
    r.l = l;
    r.lgtLight = f.lgtLight;
    r.lgtPrim = f.lgtPrim;
    const int nl = n_lgt(l), nc = c - 1;
    const SVert *lastCam = nc > 0 ? &f.cam[nc - 1] : nullptr;
    r.dlLight = lastCam ? lastCam->dlLight : -1;
    r.dlPrim = lastCam ? lastCam->dlPrim : -1;
    r.useAbs = 0u;
    int k = 0;
    if (l > 1) {
        r.u[k++] = f.lgtPos[0];
        r.u[k++] = f.lgtPos[1];
        r.u[k++] = f.lgtDir[0];
        r.u[k++] = f.lgtDir[1];
        #pragma unroll 1
        for (int i = 0; i < nl - 1; i++) {
            r.u[k++] = f.lgt[i].rnd[0];
            r.u[k++] = f.lgt[i].rnd[1];
        }
    }
    if (c > 1) {
        r.u[k++] = f.screen[0];
        r.u[k++] = f.screen[1];
        #pragma unroll 1
        for (int i = 0; i < nc - 1; i++) {
            r.u[k++] = f.cam[i].rnd[0];
            r.u[k++] = f.cam[i].rnd[1];
        }
        if (l == 1) {
            r.u[k++] = lastCam->dl[0];
            r.u[k++] = lastCam->dl[1];
        }
    }
    #pragma unroll 1
    for (int i = 0; i < nl; i++) {
        r.tri[i] = f.lgt[i].tri;
        r.disc[i] = f.lgt[i].disc;
        r.rr[i] = f.lgt[i].rr;
        if (f.lgt[i].useAbs) r.useAbs |= 1u << i;
    }
    #pragma unroll 1
    for (int i = 0; i < nc; i++) {
        r.tri[nl + i] = f.cam[i].tri;
        r.disc[nl + i] = f.cam[i].disc;
        r.rr[nl + i] = f.cam[i].rr;
        if (f.cam[i].useAbs) r.useAbs |= 1u << (nl + i);
    }
}

// GeneratePathBidir (src/path.cpp:978-1121). Every contribution goes to sink(e).
template <class R, class Sink>
DEV void generate_path_bidir(const SceneView &s, int minDepth, int maxDepth, R &rng, FullPath &f, Sink &sink) {
    BState lps[kMaxFull];
    f.time = rng.uniform();
    // EmitFromLightInit (src/path.cpp:480-491)
    f.lgtPos[1] = rng.uniform();
    f.lgtPos[0] = rng.uniform();
    f.lgtDir[1] = rng.uniform();
    f.lgtDir[0] = rng.uniform();
    float pickProb;
    f.lgtLight = pick_light(s, rng.uniform(), pickProb);
    {
        const Light &L = s.lights[f.lgtLight];
        const float ud = rng.uniform();
        f.lgtPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : -1;
    }
    V3 org, dir;
    zero_state(lps[0]);
    emit_from_light(s, pickProb, f.lgtLight, f.lgtPrim, f.lgtPos, f.lgtDir, org, dir, lps[0]);
    f.nLgt = 0;
    int nStates = 1;
    #pragma unroll 1
    for (int d = 0; d < kMaxFull - 1; d++) {
        SVert &v = f.lgt[d];
        clear_vert(v);
        f.nLgt = d + 1;
        int tri = -1;
        const bool hit = intersect(s, org, dir, kIsectEps, INFINITY, tri, lps[d].isect);
        v.tri = tri;
        if (!hit) {
            nStates--;
            f.nLgt--;
            break;
        }
        v.disc = rng.uniform();
        lps[d].wi = -dir;
        convert_mis(s, d, f.lgtLight, org, dir, lps[d]);
        if (d + 2 >= minDepth) {
            Emit e;
            if (connect_to_camera(s, d, lps[d], v, e)) sink(e);
        }
        if (maxDepth != -1 && d + 2 >= maxDepth) break;
        zero_state(lps[d + 1]);
        nStates++;
        v.rnd[1] = rng.uniform();
        v.rnd[0] = rng.uniform();
        V3 bc;
        if (!bsdf_sampling<true, false>(s, lps[d], v, lps[d + 1], true, dir, bc)) {
            nStates--;
            break;
        }
        if (!russian_roulette(d, bc, v.rr, lps[d + 1].throughput, rng)) {
            nStates--;
            break;
        }
        org = lps[d].isect.position;
    }
    // camera subpath
    f.screen[1] = rng.uniform();
    f.screen[0] = rng.uniform();
    BState cp;
    zero_state(cp);
    float minT, maxT;
    emit_from_camera(s, f.screen[0], f.screen[1], org, dir, minT, maxT, cp);
    f.nCam = 0;
    #pragma unroll 1
    for (int d = 0; d < kMaxFull; d++) {
        SVert &v = f.cam[d];
        clear_vert(v);
        f.nCam = d + 1;
        int tri = -1;
        const bool hit = intersect(s, org, dir, minT, maxT, tri, cp.isect);
        v.tri = tri;
        cp.wi = -dir;
        if (hit) convert_mis(s, d, -1, org, dir, cp);
        if (d + 1 >= minDepth) {
            const int light = hit ? area_light_of_tri(s, tri) : s.envLight;  // GetHitLight
            if (light >= 0) {
                if (!hit) v.tri = -1;  // a path that ends on the environment light
                if (s.opt.useLightCoordinateSampling && d > 1 && s.lights[light].type == kLightArea)
                    light_coordinate_convert(s, f.cam[d - 1].rnd[0], f.cam[d - 1].rnd[1], tri, org, cp);
                Emit e;
                if (handle_hit_light(s, d, light, dir, f.screen[0], f.screen[1], cp, e)) sink(e);
                return;
            }
        }
        if (!hit || (maxDepth != -1 && d + 1 >= maxDepth)) break;
        v.disc = rng.uniform();
        if (d + 2 >= minDepth) {
            float dlPick;
            v.dlLight = pick_light(s, rng.uniform(), dlPick);
            v.dl[1] = rng.uniform();
            v.dl[0] = rng.uniform();
            const Light &L = s.lights[v.dlLight];
            const float ud = rng.uniform();
            v.dlPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : 0;
            Emit e;
            if (direct_lighting(s, d, cp, f.screen[0], f.screen[1], dlPick, v, e)) sink(e);
        }
        const int maxLgtDepth = maxDepth == -1 ? (nStates - 1) : min(maxDepth - d - 3, nStates - 1);
        #pragma unroll 1
        for (int ld = 0; ld <= maxLgtDepth; ld++) {
            if (d + ld + 3 >= minDepth) {
                Emit e;
                if (connect_vertex(s, d, ld, lps[ld], f.lgt[ld], cp, v, f.screen[0], f.screen[1], e)) sink(e);
            }
        }
        v.rnd[1] = rng.uniform();
        v.rnd[0] = rng.uniform();
        V3 bc;
        if (!bsdf_sampling<false, false>(s, cp, v, cp, false, dir, bc)) break;
        if (!russian_roulette(d, bc, v.rr, cp.throughput, rng)) break;
        org = cp.isect.position;
        minT = kIsectEps;
        maxT = INFINITY;
    }
}

// ---------------------------------------------------------------- path machines
// The two technique-path samplers of the chain loop -- the multiplexed large
// step (GenerateSubpath) and the small-step perturbation (PerturbPathBidir) --
// as resumable state machines. A step advances the path to its next ray cast,
// leaves that ray in the machine and returns kStepRay; the next step takes the
// cast's answer (closest hit: the BVH's triangle or -1; shadow ray: 1 if
// occluded). kStepDone leaves the contribution in m.e; kStepFail means the
// technique does not contribute. The sequential samplers below answer each ray
// on the spot; the wavefront sampler (wave.cuh) queues the rays of all chains
// and answers them with a separate traversal kernel. Both run these same
// (out-of-line) step functions, so both take identical steps.
enum : int { kStepRay = 0, kStepDone = 1, kStepFail = 2 };
enum : int { kRayClosest = 0, kRayAny = 1 };

struct PathM {
    int pc;                    // resume point
    int d;                     // vertex index within the subpath being traced
    int k;                     // next primary coordinate (perturbation)
    int lastLgtTri;            // triangle of the last light-subpath vertex (ConnectVertex)
    int lightCoords;           // perturbation: light-coordinate sampling of the last camera segment
    int camLength, lgtLength;  // large step: the technique
    int kind;                  // kind of the ray below: kRayClosest | kRayAny
    float sx, sy;              // screen position of the camera subpath
    V3 org, dir;               // the ray: closest hit in (tmin, tmax], or a shadow ray over [tmin, tmax]
    float tmin, tmax;
    BState lp, cp;             // light / camera subpath states
    Emit e;                    // the contribution (with kStepDone; before, one awaiting its shadow ray)
};

DEV int want_closest(PathM &m, int pc, float tmin, float tmax) {
    m.pc = pc;
    m.kind = kRayClosest;
    m.tmin = tmin;
    m.tmax = tmax;
    return kStepRay;
}
// The shadow ray of Occluded(scene, time, ray, dist) (src/scene.cpp:95-105).
DEV int want_shadow(PathM &m, int pc, const Shadow &sh) {
    m.pc = pc;
    m.kind = kRayAny;
    m.org = sh.org;
    m.dir = sh.dir;
    m.tmin = kIsectEps;
    m.tmax = isinf(sh.dist) ? INFINITY : (1.0f - kShadowEps) * sh.dist;
    return kStepRay;
}
// The answer to a closest-hit ray: Intersect of src/path.cpp:94-103 after the
// BVH returned `hit`; `tri` is updated whenever the BVH reports a hit, even if
// the re-intersection fails.
DEV bool take_hit(const SceneView &s, const PathM &m, int hit, int &tri, Isect &isect) {
    if (hit < 0) return false;
    tri = hit;
    return reintersect(s, hit, m.org, m.dir, isect);
}
// Answers the machine's pending ray on the spot (the sequential samplers).
DEV int answer_ray(const SceneView &s, const PathM &m) {
    if (m.kind == kRayAny) return traverse<true>(s, m.org, m.dir, m.tmin, m.tmax) >= 0 ? 1 : 0;
    return traverse<false>(s, m.org, m.dir, m.tmin, m.tmax);
}

// Guarded writes into a path record: a degenerate large step (camLength =
// lgtLength = 1, which never connects) keeps tracing camera vertices past the
// record's capacity, as the reference's loop does, and always fails.
DEV void rec_u(PathRec &r, int i, float v) {
    if (i >= 0 && i < kMaxDim) r.u[i] = v;
}
DEV void rec_clear_vert(PathRec &r, int vi, int tri) {
    if (vi >= kMaxVerts) return;
    r.tri[vi] = tri;
    r.disc[vi] = 0.0f;
    r.rr[vi] = 0.0f;
    r.useAbs &= ~(1u << vi);
}

// ---- multiplexed large step: GenerateSubpath (src/path.cpp:1123-1269) with
// bidirMIS = true for the technique (m.camLength, m.lgtLength). The path record
// is written as the path is built, in the layout Path::Initialize and
// GetPathPos give it (src/path.h:109-120, src/path.cpp:2393-2439): light
// vertices first, u = light position / direction, light-vertex directions,
// screen position, camera-vertex directions, direct-light sample.
enum : int { kGStart = 0, kGLgtHit, kGCamStart, kGCamHit, kGFinalShadow };

template <class R>
DEV_SHARED int subpath_step(const SceneView &s, R &rng, PathRec &rec, PathM &m, int hit) {
    const int camLength = m.camLength, lgtLength = m.lgtLength;
    const int nl = n_lgt(lgtLength);
    const int camBase = lgtLength > 1 ? 2 * nl + 2 : 0;  // u index of the screen position
    for (;;) {
        switch (m.pc) {
            case kGStart: {
                rng.uniform();  // time
                zero_state(m.lp);
                rec.c = camLength;
                rec.l = lgtLength;
                rec.lgtLight = -1;
                rec.lgtPrim = -1;
                rec.dlLight = -1;
                rec.dlPrim = -1;
                rec.useAbs = 0u;
                m.lastLgtTri = -1;
                if (lgtLength > 1) {
                    // EmitFromLightInit: position then direction, second components first
                    rec.u[1] = rng.uniform();
                    rec.u[0] = rng.uniform();
                    rec.u[3] = rng.uniform();
                    rec.u[2] = rng.uniform();
                    float pickProb;
                    rec.lgtLight = pick_light(s, rng.uniform(), pickProb);
                    const Light &L = s.lights[rec.lgtLight];
                    const float ud = rng.uniform();
                    rec.lgtPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : -1;
                    const float pos[2] = {rec.u[0], rec.u[1]};
                    const float dirp[2] = {rec.u[2], rec.u[3]};
                    emit_from_light(s, pickProb, rec.lgtLight, rec.lgtPrim, pos, dirp, m.org, m.dir, m.lp);
                    m.d = 0;
                    return want_closest(m, kGLgtHit, kIsectEps, INFINITY);
                }
                m.pc = kGCamStart;
                continue;
            }
            case kGLgtHit: {
                const int d = m.d;
                SVert v;
                clear_vert(v);
                int tri = -1;
                const bool okH = take_hit(s, m, hit, tri, m.lp.isect);
                v.tri = tri;
                rec_clear_vert(rec, d, tri);
                if (!okH) return kStepFail;
                v.disc = rng.uniform();
                rec.disc[d] = v.disc;
                m.lp.wi = -m.dir;
                convert_mis(s, d, rec.lgtLight, m.org, m.dir, m.lp);
                if (d + 2 == lgtLength) {
                    if (camLength == 1) {
                        Shadow sh;
                        if (!connect_to_camera_pre(s, d, m.lp, v, m.e, sh)) return kStepFail;
                        return want_shadow(m, kGFinalShadow, sh);
                    }
                    m.lastLgtTri = v.tri;
                    m.pc = kGCamStart;
                    continue;
                }
                v.rnd[1] = rng.uniform();
                v.rnd[0] = rng.uniform();
                V3 bc;
                const bool okS = bsdf_sampling<true, false>(s, m.lp, v, m.lp, false, m.dir, bc);
                rec_u(rec, 4 + 2 * d, v.rnd[0]);  // as sampled, or re-parameterised (absolute parameters)
                rec_u(rec, 5 + 2 * d, v.rnd[1]);
                if (v.useAbs) rec.useAbs |= 1u << d;
                if (!okS) return kStepFail;
                rec.rr[d] = 1.0f;
                m.org = m.lp.isect.position;
                m.d = d + 1;
                if (m.d >= kMaxFull) {  // the reference's vertex bound (unreachable for lgtLength <= 12)
                    m.pc = kGCamStart;
                    continue;
                }
                return want_closest(m, kGLgtHit, kIsectEps, INFINITY);
            }
            case kGCamStart: {
                m.sy = rng.uniform();
                m.sx = rng.uniform();
                rec_u(rec, camBase, m.sx);
                rec_u(rec, camBase + 1, m.sy);
                zero_state(m.cp);
                float minT, maxT;
                emit_from_camera(s, m.sx, m.sy, m.org, m.dir, minT, maxT, m.cp);
                m.d = 0;
                return want_closest(m, kGCamHit, minT, maxT);
            }
            case kGCamHit: {
                const int d = m.d, vi = nl + d;
                SVert v;
                clear_vert(v);
                int tri = -1;
                const bool okH = take_hit(s, m, hit, tri, m.cp.isect);
                v.tri = tri;
                rec_clear_vert(rec, vi, tri);
                m.cp.wi = -m.dir;
                if (okH) convert_mis(s, d, -1, m.org, m.dir, m.cp);
                if (d + 2 >= camLength && lgtLength == 0) {
                    const int light = okH ? area_light_of_tri(s, tri) : s.envLight;  // GetHitLight
                    if (light < 0) return kStepFail;
                    if (!okH) rec_clear_vert(rec, vi, -1);  // a path that ends on the environment light
                    if (d > 1 && s.lights[light].type == kLightArea)
                        light_coordinate_convert(s, rec.u[camBase + 2 * d], rec.u[camBase + 2 * d + 1], tri, m.org,
                                                 m.cp);
                    return handle_hit_light(s, d, light, m.dir, m.sx, m.sy, m.cp, m.e) ? kStepDone : kStepFail;
                }
                if (!okH) return kStepFail;
                v.disc = rng.uniform();
                if (vi < kMaxVerts) rec.disc[vi] = v.disc;
                if (d + 2 == camLength) {
                    Shadow sh;
                    bool okC;
                    if (lgtLength == 1) {
                        float dlPick;
                        v.dlLight = pick_light(s, rng.uniform(), dlPick);
                        v.dl[1] = rng.uniform();
                        v.dl[0] = rng.uniform();
                        const Light &L = s.lights[v.dlLight];
                        const float ud = rng.uniform();
                        v.dlPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : 0;
                        rec.dlLight = v.dlLight;
                        rec.dlPrim = v.dlPrim;
                        rec_u(rec, camBase + 2 * d + 2, v.dl[0]);
                        rec_u(rec, camBase + 2 * d + 3, v.dl[1]);
                        okC = direct_lighting_pre(s, d, m.cp, m.sx, m.sy, dlPick, v, m.e, sh);
                    } else {
                        SVert lv;
                        clear_vert(lv);
                        lv.tri = m.lastLgtTri;
                        okC = connect_vertex_pre(s, d, lgtLength - 2, m.lp, lv, m.cp, v, m.sx, m.sy, m.e, sh);
                    }
                    if (!okC) return kStepFail;
                    return want_shadow(m, kGFinalShadow, sh);
                }
                v.rnd[1] = rng.uniform();
                v.rnd[0] = rng.uniform();
                V3 bc;
                const bool okS = bsdf_sampling<false, false>(s, m.cp, v, m.cp, false, m.dir, bc);
                rec_u(rec, camBase + 2 + 2 * d, v.rnd[0]);
                rec_u(rec, camBase + 3 + 2 * d, v.rnd[1]);
                if (v.useAbs && vi < kMaxVerts) rec.useAbs |= 1u << vi;
                if (!okS) return kStepFail;
                if (vi < kMaxVerts) rec.rr[vi] = 1.0f;
                m.org = m.cp.isect.position;
                m.d = d + 1;
                if (m.d >= kMaxFull) return kStepFail;  // the reference's vertex bound
                return want_closest(m, kGCamHit, kIsectEps, INFINITY);
            }
            case kGFinalShadow:
                return hit ? kStepFail : kStepDone;
            default:
                return kStepFail;
        }
    }
}

// ---- small-step perturbation: PerturbPathBidir (src/path.cpp:1480-1628) of the
// technique path `in` by `offset`, into `out`. Coordinates are perturbed in
// order and `out` keeps whatever was updated before an early exit, as the
// reference's Path does. Discrete parameters get N(0, discreteStdDev) jitter
// drawn from `jit`.
enum : int { kPStart = 0, kPLgtHit, kPCamStart, kPCamHit, kPLcsShadow, kPCamNext, kPFinalShadow };

template <class J>
DEV_SHARED int perturb_step(const SceneView &s, const PathRec &in, const float *offset, J &jit, PathRec &out,
                            PathM &m, int hit) {
    const int c = in.c, l = in.l;
    const int nl = n_lgt(l), nc = c - 1;
    const float sd = s.opt.discreteStdDev;
    for (;;) {
        switch (m.pc) {
            case kPStart: {
                out = in;
                out.useAbs &= ~kLensFormBit;
                m.k = 0;
                zero_state(m.lp);
                m.lastLgtTri = -1;
                if (l > 1) {
                    const float pickProb = pick_light_prob(s, in.lgtLight);
                    for (int i = 0; i < 4; i++) out.u[i] = mod1(in.u[i] + offset[i]);
                    m.k = 4;
                    const float pos[2] = {out.u[0], out.u[1]};
                    const float dirp[2] = {out.u[2], out.u[3]};
                    emit_from_light(s, pickProb, in.lgtLight, in.lgtPrim, pos, dirp, m.org, m.dir, m.lp);
                    m.d = 0;
                    return want_closest(m, kPLgtHit, kIsectEps, INFINITY);
                }
                m.pc = kPCamStart;
                continue;
            }
            case kPLgtHit: {
                const int d = m.d;
                SVert v;
                clear_vert(v);
                int tri = out.tri[d];
                const bool okH = take_hit(s, m, hit, tri, m.lp.isect);
                out.tri[d] = tri;
                v.tri = tri;
                if (!okH) return kStepFail;
                m.lp.wi = -m.dir;
                out.disc[d] = mod1(out.disc[d] + (sd > 0.0f ? sd * jit.normal() : 0.0f));
                v.disc = out.disc[d];
                convert_mis(s, d, in.lgtLight, m.org, m.dir, m.lp);
                if (d == nl - 1 && c == 1) {
                    Shadow sh;
                    if (!connect_to_camera_pre(s, d, m.lp, v, m.e, sh)) return kStepFail;
                    return want_shadow(m, kPFinalShadow, sh);
                }
                if (d == nl - 1) {
                    m.lastLgtTri = v.tri;
                    m.pc = kPCamStart;
                    continue;
                }
                const int k = m.k;
                out.u[k] = mod1(in.u[k] + offset[k]);
                out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
                v.rnd[0] = out.u[k];
                v.rnd[1] = out.u[k + 1];
                m.k = k + 2;
                V3 bc;
                const bool okS = bsdf_sampling<true, true>(s, m.lp, v, m.lp, false, m.dir, bc);
                if (v.useAbs) out.useAbs |= 1u << d; else out.useAbs &= ~(1u << d);
                if (!okS) return kStepFail;
                m.lp.throughput = m.lp.throughput * out.rr[d];
                m.org = m.lp.isect.position;
                m.d = d + 1;
                return want_closest(m, kPLgtHit, kIsectEps, INFINITY);
            }
            case kPCamStart: {
                const int k = m.k;
                out.u[k] = mod1(in.u[k] + offset[k]);
                out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
                m.sx = out.u[k];
                m.sy = out.u[k + 1];
                m.k = k + 2;
                zero_state(m.cp);
                float minT, maxT;
                emit_from_camera(s, m.sx, m.sy, m.org, m.dir, minT, maxT, m.cp);
                m.lightCoords = 0;
                m.d = 0;
                if (nc <= 0) return kStepFail;
                return want_closest(m, kPCamHit, minT, maxT);
            }
            case kPCamHit: {
                const int d = m.d, vi = nl + d;
                SVert v;
                clear_vert(v);
                int tri = out.tri[vi];
                const bool okH = take_hit(s, m, hit, tri, m.cp.isect);
                out.tri[vi] = tri;
                v.tri = tri;
                m.cp.wi = -m.dir;
                if (okH) convert_mis(s, d, -1, m.org, m.dir, m.cp);
                if (d == nc - 1 && l == 0) {
                    const int light = okH ? area_light_of_tri(s, tri) : s.envLight;
                    if (light < 0) return kStepFail;
                    if (!okH) out.tri[vi] = -1;  // the path ends on the environment light
                    return handle_hit_light(s, d, light, m.dir, m.sx, m.sy, m.cp, m.e) ? kStepDone : kStepFail;
                }
                if (!okH) return kStepFail;
                out.disc[vi] = mod1(out.disc[vi] + (sd > 0.0f ? sd * jit.normal() : 0.0f));
                v.disc = out.disc[vi];
                if (d == nc - 1) {
                    Shadow sh;
                    bool okC;
                    if (l == 1) {
                        const int k = m.k;
                        out.u[k] = mod1(in.u[k] + offset[k]);
                        out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
                        v.dlLight = in.dlLight;
                        v.dlPrim = in.dlPrim;
                        v.dl[0] = out.u[k];
                        v.dl[1] = out.u[k + 1];
                        okC = direct_lighting_pre(s, d, m.cp, m.sx, m.sy, pick_light_prob(s, in.dlLight), v, m.e, sh);
                    } else {
                        SVert lv;
                        clear_vert(lv);
                        lv.tri = m.lastLgtTri;
                        okC = connect_vertex_pre(s, d, nl - 1, m.lp, lv, m.cp, v, m.sx, m.sy, m.e, sh);
                    }
                    if (!okC) return kStepFail;
                    return want_shadow(m, kPFinalShadow, sh);
                }
                const int k = m.k;
                out.u[k] = mod1(in.u[k] + offset[k]);
                out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
                v.rnd[0] = out.u[k];
                v.rnd[1] = out.u[k + 1];
                m.k = k + 2;
                if (s.opt.useLightCoordinateSampling && d == nc - 2 && l == 0) {
                    const int lastTri = in.tri[nl + nc - 1];
                    if (lastTri >= 0 && area_light_of_tri(s, lastTri) >= 0) m.lightCoords = 1;
                }
                V3 bc;
                if (m.lightCoords) {
                    // the next segment aims at the light triangle; its shadow ray
                    // leaves from the vertex along the new direction (m.org, m.dir)
                    Shadow sh;
                    if (!light_coordinate_sampling_pre(s, v, in.tri[nl + nc - 1], m.cp, m.dir, bc, sh))
                        return kStepFail;
                    return want_shadow(m, kPLcsShadow, sh);
                }
                const bool okS = bsdf_sampling<false, true>(s, m.cp, v, m.cp, false, m.dir, bc);
                if (v.useAbs) out.useAbs |= 1u << vi; else out.useAbs &= ~(1u << vi);
                if (!okS) return kStepFail;
                m.pc = kPCamNext;
                continue;
            }
            case kPLcsShadow:
                if (hit) return kStepFail;  // occluded
                m.pc = kPCamNext;
                continue;
            case kPCamNext: {
                // after sampling camera vertex d: the segment to vertex d + 1
                m.cp.throughput = m.cp.throughput * out.rr[nl + m.d];
                m.org = m.cp.isect.position;
                m.d += 1;
                if (m.d >= nc) return kStepFail;
                return want_closest(m, kPCamHit, kIsectEps, INFINITY);
            }
            case kPFinalShadow:
                return hit ? kStepFail : kStepDone;
            default:
                return kStepFail;
        }
    }
}

// Sequential samplers: the machines with every ray answered on the spot.
// GenerateSubpath: true and `rec` / `e` filled when technique (camLength,
// lgtLength) contributes (on failure `rec` holds a partial path).
template <class R>
DEV bool generate_subpath(const SceneView &s, int camLength, int lgtLength, R &rng, PathRec &rec, Emit &e) {
    PathM m;
    m.pc = kGStart;
    m.camLength = camLength;
    m.lgtLength = lgtLength;
    int hit = -1, st;
    while ((st = subpath_step(s, rng, rec, m, hit)) == kStepRay) hit = answer_ray(s, m);
    if (st != kStepDone) return false;
    e = m.e;
    return true;
}

// PerturbPathBidir: true with `e` filled if the perturbed path contributes.
template <class J>
DEV bool perturb_path(const SceneView &s, const PathRec &in, const float *offset, J &jit, PathRec &out, Emit &e) {
    PathM m;
    m.pc = kPStart;
    int hit = -1, st;
    while ((st = perturb_step(s, in, offset, jit, out, m, hit)) == kStepRay) hit = answer_ray(s, m);
    if (st != kStepDone) return false;
    e = m.e;
    return true;
}

// ---------------------------------------------------------------- direct-lighting pass
// GeneratePath (src/path.cpp:343-445) with minDepth = min(minDepth, 2) and
// maxDepth = min(maxDepth, 2) for pixel (px, py), as DirectLighting
// (src/integrator.h:33-75) calls it. Unidirectional MIS (src/path.cpp:115-323).
template <class R, class Sink>
DEV void generate_path_direct(const SceneView &s, int px, int py, int minDepth, int maxDepth, R &rng, Sink &sink) {
    rng.uniform();  // time
    const float sy = (float(py) + rng.uniform()) / float(s.cam.height);
    const float sx = (float(px) + rng.uniform()) / float(s.cam.width);
    V3 org, dir;
    float minT, maxT;
    sample_primary(s.cam, sx, sy, org, dir, minT, maxT);
    V3 throughput(1.0f, 1.0f, 1.0f);
    float lastBsdfPdf = 1.0f;
    #pragma unroll 1
    for (int d = 0; d < 8; d++) {
        Isect isect;
        int tri = -1;
        const bool hit = intersect(s, org, dir, minT, maxT, tri, isect);
        const int light = hit ? area_light_of_tri(s, tri) : s.envLight;
        if (light >= 0 && d + 1 >= minDepth) {
            V3 emission;
            float directPdf, emissionPdf;
            light_emission(s, light, dir, isect.shadingNormal, emission, directPdf, emissionPdf);
            if (emission.x + emission.y + emission.z > 0.0f) {
                if (hit) {
                    const float distSq = dist_sq(org, isect.position);
                    const float cosTheta = -dot(dir, isect.shadingNormal);
                    directPdf *= (distSq / cosTheta);
                }
                V3 contrib = cmul(throughput, emission);
                if (d > 0) contrib = contrib * mis_weight(lastBsdfPdf, directPdf * pick_light_prob(s, light));
                const float score = luminance(contrib);
                if (score > 0.0f) {
                    Emit e;
                    e.c = 2 + d;
                    e.l = 0;
                    e.screen[0] = sx;
                    e.screen[1] = sy;
                    e.rgb = contrib;
                    e.ls = e.ss = score;
                    sink(e);
                }
            }
            return;
        }
        if (!hit || (maxDepth != -1 && d + 1 >= maxDepth)) break;
        const float disc = rng.uniform();
        const V3 wi = -dir;
        const Bsdf &bsdf = bsdf_of_tri(s, tri);
        if (d + 2 >= minDepth) {
            float pick;
            const int dl = pick_light(s, rng.uniform(), pick);
            const float r1 = rng.uniform();
            const float r0 = rng.uniform();
            const Light &L = s.lights[dl];
            const float ud = rng.uniform();
            const int dlPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : 0;
            V3 dirToLight, lightContrib;
            float dist, cosAtLight, directPdf, emissionPdf;
            if (light_sample_direct(s, dl, dlPrim, isect.position, r0, r1, dirToLight, dist, lightContrib,
                                    cosAtLight, directPdf, emissionPdf) &&
                !occluded(s, isect.position, dirToLight, dist)) {
                BsdfOut bo;
                bsdf_evaluate(bsdf, wi, isect.shadingNormal, dirToLight, bo);
                if (!is_zero(bo.contrib)) {
                    V3 contrib = cmul(throughput, bo.contrib);
                    contrib = cmul(contrib, lightContrib) * (1.0f / pick);
                    if (!light_is_delta(s, dl)) contrib = contrib * mis_weight(directPdf * pick, bo.pdf);
                    const float score = luminance(contrib);
                    if (score > 0.0f) {
                        Emit e;
                        e.c = 2 + d;
                        e.l = 1;
                        e.screen[0] = sx;
                        e.screen[1] = sy;
                        e.rgb = contrib;
                        e.ls = e.ss = score;
                        sink(e);
                    }
                }
            }
        }
        const float r1 = rng.uniform();
        const float r0 = rng.uniform();
        BsdfOut bo;
        V3 wo;
        if (!bsdf_sample(bsdf, wi, isect.shadingNormal, r0, r1, disc, wo, bo)) break;
        lastBsdfPdf = bo.pdf;
        throughput = cmul(throughput, bo.contrib);
        float rrw;
        if (!russian_roulette(d, bo.contrib, rrw, throughput, rng)) break;
        org = isect.position;
        dir = wo;
        minT = kIsectEps;
        maxT = INFINITY;
    }
}

}  // namespace drmlt
