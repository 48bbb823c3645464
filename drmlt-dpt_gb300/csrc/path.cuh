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
// computed: the DR integrator never reads them.
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
    unsigned useAbs;
    float u[kMaxDim];
    int tri[kMaxVerts];
    float disc[kMaxVerts];
    float rr[kMaxVerts];
};

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

// ConnectToCamera (src/path.cpp:518-606).
DEV bool connect_to_camera(const SceneView &s, int lgtDepth, const BState &ps, const SVert &v, Emit &e) {
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
    if (occluded(s, ps.isect.position, dirToCamera, dist)) return false;
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
DEV bool direct_lighting(const SceneView &s, int camDepth, const BState &ps, float sx, float sy, float pickProb,
                         const SVert &v, Emit &e) {
    V3 dirToLight, lightContrib;
    float dist, cosAtLight, directPdf, emissionPdf;
    if (!light_sample_direct(s, v.dlLight, v.dlPrim, ps.isect.position, v.dl[0], v.dl[1], dirToLight, dist,
                             lightContrib, cosAtLight, directPdf, emissionPdf))
        return false;
    if (occluded(s, ps.isect.position, dirToLight, dist)) return false;
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
DEV bool connect_vertex(const SceneView &s, int camDepth, int lgtDepth, const BState &lp, const SVert &lv,
                        const BState &cp, const SVert &cv, float sx, float sy, Emit &e) {
    V3 dirToLight = lp.isect.position - cp.isect.position;
    const float distSq = length_sq(dirToLight);
    const float dist = sqrtf(distSq);
    dirToLight = dirToLight * (1.0f / dist);
    if (occluded(s, cp.isect.position, dirToLight, dist)) return false;
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

// LightCoordinateSampling, bidirectional form (src/path.cpp:1430-1478).
DEV bool light_coordinate_sampling(const SceneView &s, const SVert &cur, int nextTri, BState &ps, V3 &dir,
                                   V3 &bsdfContrib) {
    V3 nextPos, nextNormal;
    sample_triangle(s, nextTri, cur.rnd[0], cur.rnd[1], nextPos, nextNormal);
    dir = nextPos - ps.isect.position;
    const float distToLightSq = length_sq(dir);
    const float distToLight = sqrtf(distToLightSq);
    dir = dir * (1.0f / distToLight);
    if (occluded(s, ps.isect.position, dir, distToLight)) return false;
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
DEV void light_coordinate_convert(const SceneView &s, SVert &prev, int lightTri, const V3 &rayOrg, BState &ps) {
    triangle_sample_param(s, lightTri, ps.isect.position, prev.rnd[0], prev.rnd[1]);
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
                    light_coordinate_convert(s, f.cam[d - 1], tri, org, cp);
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

// ---------------------------------------------------------------- multiplexed large step
// GenerateSubpath (src/path.cpp:1123-1269) with bidirMIS = true. Returns true
// and fills `rec`/`e` when the technique (camLength, lgtLength) contributes.
template <class R>
DEV bool generate_subpath(const SceneView &s, int camLength, int lgtLength, R &rng, PathRec &rec, Emit &e) {
    FullPath f;
    f.time = rng.uniform();
    BState lp;
    zero_state(lp);
    f.nLgt = 0;
    f.lgtLight = -1;
    f.lgtPrim = -1;
    V3 org, dir;
    if (lgtLength > 1) {
        f.lgtPos[1] = rng.uniform();
        f.lgtPos[0] = rng.uniform();
        f.lgtDir[1] = rng.uniform();
        f.lgtDir[0] = rng.uniform();
        float pickProb;
        f.lgtLight = pick_light(s, rng.uniform(), pickProb);
        const Light &L = s.lights[f.lgtLight];
        const float ud = rng.uniform();
        f.lgtPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : -1;
        emit_from_light(s, pickProb, f.lgtLight, f.lgtPrim, f.lgtPos, f.lgtDir, org, dir, lp);
        #pragma unroll 1
        for (int d = 0; d < kMaxFull; d++) {
            SVert &v = f.lgt[d];
            clear_vert(v);
            f.nLgt = d + 1;
            int tri = -1;
            const bool hit = intersect(s, org, dir, kIsectEps, INFINITY, tri, lp.isect);
            v.tri = tri;
            if (!hit) return false;
            v.disc = rng.uniform();
            lp.wi = -dir;
            convert_mis(s, d, f.lgtLight, org, dir, lp);
            if (d + 2 == lgtLength) {
                if (camLength == 1) {
                    if (!connect_to_camera(s, d, lp, v, e)) return false;
                    make_rec(f, 1, lgtLength, rec);
                    return true;
                }
                break;
            }
            v.rnd[1] = rng.uniform();
            v.rnd[0] = rng.uniform();
            V3 bc;
            if (!bsdf_sampling<true, false>(s, lp, v, lp, false, dir, bc)) return false;
            v.rr = 1.0f;
            org = lp.isect.position;
        }
    }
    f.screen[1] = rng.uniform();
    f.screen[0] = rng.uniform();
    BState cp;
    zero_state(cp);
    float minT, maxT;
    emit_from_camera(s, f.screen[0], f.screen[1], org, dir, minT, maxT, cp);
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
        if (d + 2 >= camLength && lgtLength == 0) {
            const int light = hit ? area_light_of_tri(s, tri) : s.envLight;
            if (light < 0) return false;
            if (!hit) v.tri = -1;
            if (d > 1 && s.lights[light].type == kLightArea)
                light_coordinate_convert(s, f.cam[d - 1], tri, org, cp);
            if (!handle_hit_light(s, d, light, dir, f.screen[0], f.screen[1], cp, e)) return false;
            make_rec(f, camLength, 0, rec);
            return true;
        }
        if (!hit) return false;
        v.disc = rng.uniform();
        if (d + 2 == camLength) {
            bool ok;
            if (lgtLength == 1) {
                float dlPick;
                v.dlLight = pick_light(s, rng.uniform(), dlPick);
                v.dl[1] = rng.uniform();
                v.dl[0] = rng.uniform();
                const Light &L = s.lights[v.dlLight];
                const float ud = rng.uniform();
                v.dlPrim = L.type == kLightArea ? sample_discrete(s.lightTriCdf + L.triCdfOffset, L.numTris, ud) : 0;
                ok = direct_lighting(s, d, cp, f.screen[0], f.screen[1], dlPick, v, e);
            } else {
                ok = connect_vertex(s, d, lgtLength - 2, lp, f.lgt[f.nLgt - 1], cp, v, f.screen[0], f.screen[1], e);
            }
            if (!ok) return false;
            make_rec(f, camLength, lgtLength, rec);
            return true;
        }
        v.rnd[1] = rng.uniform();
        v.rnd[0] = rng.uniform();
        V3 bc;
        if (!bsdf_sampling<false, false>(s, cp, v, cp, false, dir, bc)) return false;
        v.rr = 1.0f;
        org = cp.isect.position;
        minT = kIsectEps;
        maxT = INFINITY;
    }
    return false;
}

// ---------------------------------------------------------------- small-step perturbation
// PerturbPathBidir (src/path.cpp:1480-1628) applied to a technique path.
// `out` receives the perturbed state (coordinates are perturbed in order and
// the state keeps whatever was updated before an early exit, as the
// reference's Path does). Discrete parameters get N(0, discreteStdDev) jitter
// drawn from `jit`. Returns true with `e` filled if the path contributes.
template <class J>
DEV bool perturb_path(const SceneView &s, const PathRec &in, const float *offset, J &jit, PathRec &out, Emit &e) {
    out = in;
    const int c = in.c, l = in.l;
    const int nl = n_lgt(l), nc = c - 1;
    const float sd = s.opt.discreteStdDev;
    int k = 0;
    BState lp;
    zero_state(lp);
    SVert lastLgt;
    clear_vert(lastLgt);
    if (l > 1) {
        const float pickProb = pick_light_prob(s, in.lgtLight);
        for (int i = 0; i < 4; i++, k++) out.u[k] = mod1(in.u[k] + offset[k]);
        const float pos[2] = {out.u[0], out.u[1]};
        const float dirp[2] = {out.u[2], out.u[3]};
        V3 org, dir;
        emit_from_light(s, pickProb, in.lgtLight, in.lgtPrim, pos, dirp, org, dir, lp);
        #pragma unroll 1
        for (int d = 0; d < nl; d++) {
            SVert v;
            clear_vert(v);
            v.tri = out.tri[d];
            int tri = v.tri;
            const bool hit = intersect(s, org, dir, kIsectEps, INFINITY, tri, lp.isect);
            out.tri[d] = tri;
            v.tri = tri;
            if (!hit) return false;
            lp.wi = -dir;
            out.disc[d] = mod1(out.disc[d] + (sd > 0.0f ? sd * jit.normal() : 0.0f));
            v.disc = out.disc[d];
            convert_mis(s, d, in.lgtLight, org, dir, lp);
            if (d == nl - 1 && c == 1) return connect_to_camera(s, d, lp, v, e);
            if (d == nl - 1) {
                lastLgt = v;
                break;
            }
            out.u[k] = mod1(in.u[k] + offset[k]);
            out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
            v.rnd[0] = out.u[k];
            v.rnd[1] = out.u[k + 1];
            k += 2;
            V3 bc;
            const bool ok = bsdf_sampling<true, true>(s, lp, v, lp, false, dir, bc);
            if (v.useAbs) out.useAbs |= 1u << d; else out.useAbs &= ~(1u << d);
            if (!ok) return false;
            lp.throughput = lp.throughput * out.rr[d];
            org = lp.isect.position;
        }
    }
    out.u[k] = mod1(in.u[k] + offset[k]);
    out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
    const float sx = out.u[k], sy = out.u[k + 1];
    k += 2;
    V3 org, dir;
    float minT, maxT;
    BState cp;
    zero_state(cp);
    emit_from_camera(s, sx, sy, org, dir, minT, maxT, cp);
    bool lightCoords = false;
    #pragma unroll 1
    for (int d = 0; d < nc; d++) {
        const int vi = nl + d;
        SVert v;
        clear_vert(v);
        int tri = out.tri[vi];
        const bool hit = intersect(s, org, dir, minT, maxT, tri, cp.isect);
        out.tri[vi] = tri;
        v.tri = tri;
        cp.wi = -dir;
        if (hit) convert_mis(s, d, -1, org, dir, cp);
        if (d == nc - 1 && l == 0) {
            const int light = hit ? area_light_of_tri(s, tri) : s.envLight;
            if (light < 0) return false;
            if (!hit) out.tri[vi] = -1;  // the path ends on the environment light
            return handle_hit_light(s, d, light, dir, sx, sy, cp, e);
        }
        if (!hit) return false;
        out.disc[vi] = mod1(out.disc[vi] + (sd > 0.0f ? sd * jit.normal() : 0.0f));
        v.disc = out.disc[vi];
        if (d == nc - 1) {
            if (l == 1) {
                out.u[k] = mod1(in.u[k] + offset[k]);
                out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
                v.dlLight = in.dlLight;
                v.dlPrim = in.dlPrim;
                v.dl[0] = out.u[k];
                v.dl[1] = out.u[k + 1];
                return direct_lighting(s, d, cp, sx, sy, pick_light_prob(s, in.dlLight), v, e);
            }
            return connect_vertex(s, d, nl - 1, lp, lastLgt, cp, v, sx, sy, e);
        }
        out.u[k] = mod1(in.u[k] + offset[k]);
        out.u[k + 1] = mod1(in.u[k + 1] + offset[k + 1]);
        v.rnd[0] = out.u[k];
        v.rnd[1] = out.u[k + 1];
        k += 2;
        if (s.opt.useLightCoordinateSampling && d == nc - 2 && l == 0) {
            const int lastTri = in.tri[nl + nc - 1];
            if (lastTri >= 0 && area_light_of_tri(s, lastTri) >= 0) lightCoords = true;
        }
        V3 bc;
        if (lightCoords) {
            if (!light_coordinate_sampling(s, v, in.tri[nl + nc - 1], cp, dir, bc)) return false;
        } else {
            const bool ok = bsdf_sampling<false, true>(s, cp, v, cp, false, dir, bc);
            if (v.useAbs) out.useAbs |= 1u << vi; else out.useAbs &= ~(1u << vi);
            if (!ok) return false;
        }
        cp.throughput = cp.throughput * out.rr[vi];
        org = cp.isect.position;
        minT = kIsectEps;
        maxT = INFINITY;
    }
    return false;
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
