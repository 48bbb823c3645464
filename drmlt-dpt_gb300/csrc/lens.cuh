// The lens mutation of integrator=h2mc: the lens branch of H2MCSmallStep::Mutate
// (src/integrators/h2mc.cpp:466-532), PerturbLensBidir with
// PerturbLensFirstVertex / PerturbLensLastVertex (src/path.cpp:1836-2078), the
// lens score of a path (SubpathContrib::lensScore: the lensContrib bookkeeping
// of src/path.cpp:560-976), the lens-mode path function log Lum(lensContrib)
// and its derivatives with respect to the screen position
// (RegisterPathFuncBidir with PathFuncMode::Lens, src/path.cpp:2941-3175), and
// the 2-D Gaussian the integrator's ComputeGaussian (h2mc.cpp:14-83, 607-640)
// builds from them.
//
// A lens mutation moves only the vertex next to the camera: x1 (c >= 2,
// aimed at the stored second vertex x2 for c >= 3) or, for a light path
// connected to the camera (c = 1), the last light vertex. Everything else is
// fixed, so the lens-mode function is written on the moving vertex and an
// anchor (the fixed neighbour and its fixed direction), which the path walk
// below records.
#pragma once
#include "chain.cuh"

namespace drmlt {

// kLensFormBit (PathRec::useAbs bit 31, path.cuh): the path was made by
// PerturbLensBidir. Its c = 1 lens score carries PerturbLensLastVertex's
// shading-normal factor (src/path.cpp:1862-1866, with wo and wi swapped
// against BSDFSampling's), so a later lens score of the same state is taken in
// that form.

struct LensAnchor {
    int c, l;       // technique camDepth, lightDepth
    int triMove;    // triangle of the moving vertex: x1 (c >= 2), the last light vertex (c = 1)
    int triFix;     // the fixed vertex: x2 (c >= 3), the last light vertex (c = 2), light vertex nl - 2 (c = 1)
    V3 pos, ns, ng; // the fixed vertex's position, shading and geometric normal
    V3 dir;         // c >= 3: x2's outgoing direction; c <= 2: the fixed vertex's wi
};

DEV bool lens_grazing(float cosWo, const V3 &d, const V3 &geomNormal) {
    return fabsf(cosWo) < 1e-2f || fabsf(dot(d, geomNormal)) < 1e-2f;
}

// The adjoint BSDF factor at camera depth 1 (src/path.cpp:685-699, 761-773,
// 929-941, 1464-1475): lens * EvaluateAdjoint(out, n, wi) * SNC<true>(out, x, wi).
// grazing: BSDFSampling's strict test (|cos| < 1e-2 zeroes the product).
DEV V3 lens_imp(const Bsdf &b, const Isect &is, const V3 &wi, const V3 &out, const V3 &lens, bool grazing) {
    BsdfOut ib;
    bsdf_evaluate<true>(b, out, is.shadingNormal, wi, ib);
    if (grazing && lens_grazing(ib.cosWo, wi, is.geomNormal)) return V3(0.0f, 0.0f, 0.0f);
    return cmul(lens, ib.contrib * shading_normal_correction<true>(out, is, wi));
}

// lensContrib after BSDFSampling<adjoint, true> at subpath depth `depth`
// (src/path.cpp:665-711), for the state ps the direction was sampled from.
template <bool adjoint>
DEV void lens_bsdf_sampling(const Bsdf &b, const BState &ps, bool useAbs, const V3 &dir, int depth, V3 &lens) {
    const V3 zero(0.0f, 0.0f, 0.0f);
    if (useAbs) {
        if (adjoint) {
            BsdfOut bo;
            bsdf_evaluate<true>(b, ps.wi, ps.isect.shadingNormal, dir, bo);
            lens = lens_grazing(bo.cosWo, dir, ps.isect.geomNormal)
                       ? zero
                       : bo.contrib * shading_normal_correction<true>(ps.wi, ps.isect, dir);
        } else if (depth == 0) {
            BsdfOut bo;
            bsdf_evaluate(b, ps.wi, ps.isect.shadingNormal, dir, bo);
            lens = lens_grazing(bo.cosWo, dir, ps.isect.geomNormal) ? zero : cmul(lens, bo.contrib);
        } else if (depth == 1) {
            lens = lens_imp(b, ps.isect, ps.wi, dir, lens, true);
        }
    } else if (adjoint || depth <= 1) {
        lens = zero;
    }
}

DEV void set_anchor_vertex(LensAnchor &a, int tri, const Isect &is) {
    a.triFix = tri;
    a.pos = is.position;
    a.ns = is.shadingNormal;
    a.ng = is.geomNormal;
}

// Walks technique path `in` with its lensContrib bookkeeping.
//   kMove = false: the path as it stands (PerturbPathBidir with zero offsets,
//     on its stored triangles, without visibility tests): its lens score, its
//     lens vertex position (x2) and anchor. (sx0, sy0): the contribution's
//     screen position.
//   kMove = true: PerturbLensBidir to screen position (sx0, sy0) with the
//     first camera vertex aimed at lensPos: true when the proposal `out`
//     contributes, with its contribution e, lens score and anchor.
// The proposal's lens score is taken as PerturbLensBidir takes it; a stored
// path's as the sampler that made it did (kLensFormBit).
template <bool kMove>
DEV bool lens_walk(const SceneView &s, const PathRec &in, float sx0, float sy0, const V3 &lensPos, PathRec &out,
                   Emit &e, float &lensScore, LensAnchor &a, V3 &lensPosOut) {
    const int c = in.c, l = in.l, nl = n_lgt(l), nc = c - 1;
    const float thr = s.opt.roughnessThreshold;
    const V3 zero(0.0f, 0.0f, 0.0f);
    const bool lensForm = kMove || (in.useAbs & kLensFormBit);
    out = in;
    out.useAbs = (in.useAbs & ~kLensFormBit) | (kMove ? kLensFormBit : 0u);
    lensScore = 0.0f;
    lensPosOut = zero;
    a.c = c;
    a.l = l;
    a.triMove = -1;
    a.triFix = -1;
    int k = 0;
    BState lp;
    zero_state(lp);
    V3 org, dir, lpLens = zero, prevLens = zero;
    int lastLgtTri = -1;
    if (l > 1) {
        const float pick = pick_light_prob(s, in.lgtLight);
        const float pos[2] = {in.u[0], in.u[1]};
        const float dirp[2] = {in.u[2], in.u[3]};
        k = 4;
        emit_from_light(s, pick, in.lgtLight, in.lgtPrim, pos, dirp, org, dir, lp);
        for (int d = 0; d < nl; d++) {
            SVert v;
            clear_vert(v);
            v.tri = out.tri[d];
            v.disc = out.disc[d];
            if (v.tri < 0 || !reintersect(s, v.tri, org, dir, lp.isect)) return false;
            lp.wi = -dir;
            convert_mis(s, d, in.lgtLight, org, dir, lp);
            const Bsdf &b = bsdf_of_tri(s, v.tri);
            if (d == nl - 1 && c == 1) {
                // ConnectToCamera (src/path.cpp:518-606) and its lensContrib (:565-580)
                if (kMove) {
                    Shadow sh;
                    if (!connect_to_camera_pre(s, d, lp, v, e, sh) || occluded(s, sh.org, sh.dir, sh.dist))
                        return false;
                }
                V3 lens = zero;
                if (bsdf_roughness(b, v.disc) > thr && d >= 1) {
                    V3 camOrg, camDir;
                    float t0, t1;
                    sample_primary(s.cam, 0.5f, 0.5f, camOrg, camDir, t0, t1);
                    V3 dtc = camOrg - lp.isect.position;
                    dtc = dtc * (1.0f / sqrtf(length_sq(dtc)));
                    BsdfOut bo;
                    bsdf_evaluate(b, dtc, lp.isect.shadingNormal, lp.wi, bo);
                    const float distSq = dist_sq(lp.isect.position, org);
                    if (!(distSq > 0.0f)) return false;
                    lens = cmul(bo.contrib, prevLens) * (1.0f / distSq);
                }
                lensScore = luminance(lens);
                a.triMove = v.tri;
                return true;
            }
            if (d == nl - 1) {
                lastLgtTri = v.tri;
                break;
            }
            v.rnd[0] = in.u[k];
            v.rnd[1] = in.u[k + 1];
            k += 2;
            if (c == 1 && d == nl - 2) {
                set_anchor_vertex(a, v.tri, lp.isect);
                a.dir = lp.wi;
            }
            if (kMove && c == 1 && d == nl - 2) {
                // PerturbLensLastVertex (src/path.cpp:1839-1875)
                v.useAbs = bsdf_roughness(b, v.disc) > thr;
                if (v.useAbs) out.useAbs |= 1u << d; else out.useAbs &= ~(1u << d);
                if (!v.useAbs) return false;
                V3 po, pd;
                float mn, mx;
                sample_primary(s.cam, sx0, sy0, po, pd, mn, mx);
                int nt = out.tri[d + 1];
                Isect ni;
                const bool hitN = intersect(s, po, pd, mn, mx, nt, ni);
                out.tri[d + 1] = nt;
                if (!hitN) return false;
                V3 nd = ni.position - lp.isect.position;
                const float dist = sqrtf(length_sq(nd));
                nd = nd * (1.0f / dist);
                if (occluded(s, lp.isect.position, nd, dist)) return false;
                float jac;
                to_spherical(nd, out.u[k - 2], out.u[k - 1], jac);
                BsdfOut bo;
                bsdf_evaluate<true>(b, lp.wi, lp.isect.shadingNormal, nd, bo);
                if (is_zero(bo.contrib) || bo.pdf <= 0.0f) return false;
                const float f = shading_normal_correction<true>(nd, lp.isect, lp.wi);
                if (f <= 0.0f) return false;
                const V3 bc = bo.contrib * f;
                lpLens = bc;
                lp.ssJacobian *= bo.pdf * fabsf(sinf(acosf(nd.z)));
                lp.accMISWThis = mis(bo.cosWo / bo.pdf) * (lp.accMISWThis * mis(bo.revPdf) + lp.accMISWPrev);
                lp.accMISWPrev = mis(1.0f / bo.pdf);
                lp.throughput = cmul(lp.throughput, bc * (1.0f / bo.pdf));
                dir = nd;
            } else {
                V3 bc;
                const BState before = lp;
                const bool okS = bsdf_sampling<true, true>(s, lp, v, lp, false, dir, bc);
                if (v.useAbs) out.useAbs |= 1u << d; else out.useAbs &= ~(1u << d);
                if (!okS) return false;
                if (lensForm && c == 1 && d == nl - 2) {
                    // the stored proposal of a lens mutation: PerturbLensLastVertex's factor
                    BsdfOut bo;
                    bsdf_evaluate<true>(b, before.wi, before.isect.shadingNormal, dir, bo);
                    lpLens = v.useAbs ? bo.contrib * shading_normal_correction<true>(dir, before.isect, before.wi)
                                      : zero;
                } else {
                    lens_bsdf_sampling<true>(b, before, v.useAbs, dir, d, lpLens);
                }
            }
            lp.throughput = lp.throughput * out.rr[d];
            prevLens = lpLens;
            org = lp.isect.position;
        }
    }
    if (nc <= 0) return false;
    float sx = in.u[k], sy = in.u[k + 1];
    if (kMove) {
        sx = sx0;
        sy = sy0;
        out.u[k] = sx;
        out.u[k + 1] = sy;
    }
    k += 2;
    BState cp;
    zero_state(cp);
    float minT, maxT;
    emit_from_camera(s, sx, sy, org, dir, minT, maxT, cp);
    V3 lens(1.0f, 1.0f, 1.0f);
    bool lightCoords = false;
    for (int d = 0; d < nc; d++) {
        const int vi = nl + d;
        SVert v;
        clear_vert(v);
        int tri = out.tri[vi];
        bool okH;
        if (kMove && d == 0) {
            okH = intersect(s, org, dir, minT, maxT, tri, cp.isect);  // the full scene (src/path.cpp:1984-1986)
        } else {
            okH = tri >= 0 && reintersect(s, tri, org, dir, cp.isect);
            if (tri >= 0 && !okH) return false;
        }
        out.tri[vi] = tri;
        v.tri = tri;
        v.disc = out.disc[vi];
        cp.wi = -dir;
        if (okH) convert_mis(s, d, -1, org, dir, cp);
        if (d == nc - 1 && l == 0) {
            // HandleHitLight: lensScore = Luminance(lensContrib) from camera depth 2 (src/path.cpp:845)
            const int light = okH ? area_light_of_tri(s, tri) : s.envLight;
            if (light < 0) return false;
            if (kMove && !handle_hit_light(s, d, light, dir, sx, sy, cp, e)) return false;
            lensScore = d >= 2 ? luminance(lens) : 0.0f;
            return true;
        }
        if (!okH) return false;
        if (d == 0) a.triMove = tri;
        if (d == 1) {
            lensPosOut = cp.isect.position;
            const float distSq = dist_sq(cp.isect.position, org);
            if (!(distSq > 0.0f)) return false;
            lens = lens * (1.0f / distSq);
            set_anchor_vertex(a, tri, cp.isect);
        }
        const Bsdf &b = bsdf_of_tri(s, tri);
        if (d == nc - 1) {
            const bool useAbs = bsdf_roughness(b, v.disc) > thr;
            if (l == 1) {
                // DirectLighting without a visibility test in the lens mutation
                // (src/path.cpp:2026-2029), its lensContrib (:760-775)
                v.dlLight = in.dlLight;
                v.dlPrim = in.dlPrim;
                v.dl[0] = in.u[k];
                v.dl[1] = in.u[k + 1];
                if (kMove) {
                    Shadow sh;
                    if (!direct_lighting_pre(s, d, cp, sx, sy, pick_light_prob(s, in.dlLight), v, e, sh)) return false;
                }
                V3 dtl, lc;
                float dist, cosAtLight, directPdf, emissionPdf;
                if (!light_sample_direct(s, v.dlLight, v.dlPrim, cp.isect.position, v.dl[0], v.dl[1], dtl, dist, lc,
                                         cosAtLight, directPdf, emissionPdf))
                    return false;
                if (d == 1) {
                    lens = useAbs ? lens_imp(b, cp.isect, cp.wi, dtl, lens, false) : zero;
                    a.dir = dtl;
                }
                lensScore = d >= 1 ? luminance(lens) : 0.0f;
            } else {
                // ConnectVertex, visibility tested at camera depth 0 only
                // (src/path.cpp:2031), its lensContrib (:920-941)
                SVert lv;
                clear_vert(lv);
                lv.tri = lastLgtTri;
                lv.disc = out.disc[nl - 1];
                if (kMove) {
                    Shadow sh;
                    if (!connect_vertex_pre(s, d, nl - 1, lp, lv, cp, v, sx, sy, e, sh)) return false;
                    if (d == 0 && occluded(s, sh.org, sh.dir, sh.dist)) return false;
                }
                V3 dtl = lp.isect.position - cp.isect.position;
                const float distSq = length_sq(dtl);
                dtl = dtl * (1.0f / sqrtf(distSq));
                if (d == 0) {
                    const Bsdf &lb = bsdf_of_tri(s, lastLgtTri);
                    if (useAbs && bsdf_roughness(lb, lv.disc) > thr) {
                        BsdfOut cb, lo;
                        bsdf_evaluate(b, cp.wi, cp.isect.shadingNormal, dtl, cb);
                        bsdf_evaluate<true>(lb, lp.wi, lp.isect.shadingNormal, -dtl, lo);
                        const V3 lgtF = lo.contrib * shading_normal_correction<true>(lp.wi, lp.isect, -dtl);
                        const V3 camF = cb.contrib * shading_normal_correction<false>(cp.wi, cp.isect, dtl);
                        lens = cmul(lgtF, camF) * (1.0f / distSq);
                    } else {
                        lens = zero;
                    }
                    set_anchor_vertex(a, lastLgtTri, lp.isect);
                    a.dir = lp.wi;
                } else if (d == 1) {
                    lens = useAbs ? lens_imp(b, cp.isect, cp.wi, dtl, lens, false) : zero;
                    a.dir = dtl;
                }
                lensScore = luminance(lens);
            }
            return true;
        }
        v.rnd[0] = in.u[k];
        v.rnd[1] = in.u[k + 1];
        k += 2;
        if (s.opt.useLightCoordinateSampling && d == nc - 2 && l == 0) {
            const int lastTri = in.tri[nl + nc - 1];
            if (lastTri >= 0 && area_light_of_tri(s, lastTri) >= 0) lightCoords = true;
        }
        if (kMove && d == 0) {
            // PerturbLensFirstVertex (src/path.cpp:1879-1910)
            v.useAbs = bsdf_roughness(b, v.disc) > thr;
            if (v.useAbs) out.useAbs |= 1u << vi; else out.useAbs &= ~(1u << vi);
            if (!v.useAbs) return false;
            V3 nd = lensPos - cp.isect.position;
            const float dist = sqrtf(length_sq(nd));
            nd = nd * (1.0f / dist);
            if (occluded(s, cp.isect.position, nd, dist)) return false;
            float jac;
            to_spherical(nd, out.u[k - 2], out.u[k - 1], jac);
            BsdfOut bo;
            bsdf_evaluate(b, cp.wi, cp.isect.shadingNormal, nd, bo);
            if (is_zero(bo.contrib) || bo.pdf <= 0.0f || lens_grazing(bo.cosWo, nd, cp.isect.geomNormal)) return false;
            lens = cmul(lens, bo.contrib);
            cp.ssJacobian *= bo.pdf * fabsf(sinf(acosf(nd.z)));
            cp.accMISWThis = mis(bo.cosWo / bo.pdf) * (cp.accMISWThis * mis(bo.revPdf) + cp.accMISWPrev);
            cp.accMISWPrev = mis(1.0f / bo.pdf);
            cp.throughput = cmul(cp.throughput, bo.contrib * (1.0f / bo.pdf));
            dir = nd;
        } else if (lightCoords) {
            // LightCoordinateSampling, without a visibility test in either walk
            // (the lens mutation passes doOcclusion = false), its lensContrib (:1462-1476)
            Shadow sh;
            V3 bc;
            if (!light_coordinate_sampling_pre(s, v, in.tri[nl + nc - 1], cp, dir, bc, sh)) return false;
            if (d == 1) lens = bsdf_roughness(b, v.disc) > thr ? lens_imp(b, cp.isect, cp.wi, dir, lens, false) : zero;
        } else {
            V3 bc;
            const BState before = cp;
            const bool okS = bsdf_sampling<false, true>(s, cp, v, cp, false, dir, bc);
            if (v.useAbs) out.useAbs |= 1u << vi; else out.useAbs &= ~(1u << vi);
            if (!okS) return false;
            lens_bsdf_sampling<false>(b, before, v.useAbs, dir, d, lens);
        }
        if (d == 1) a.dir = dir;
        cp.throughput = cp.throughput * out.rr[vi];
        org = cp.isect.position;
    }
    return false;
}

// The lens-mode path function (src/path.cpp:2941-2970, 3028-3160 with
// mode == Lens) on the anchor of lens_walk, at screen position (sx, sy):
//   c >= 3  PerturbLensFirstVertex (AD): x1 aimed at x2, EvaluateBSDF(false);
//           1 / |x2 - x1|^2; x2's adjoint factor toward its fixed direction,
//           except for direct lighting at x2 (c = 3, l = 1), where the
//           reference's AD DirectLighting keeps that factor in a local copy
//           and never stores it (src/path.cpp:2857-2868), so the function
//           stops at 1 / |x2 - x1|^2;
//   c = 2   ConnectVertex at camera depth 0 (AD);
//   c = 1   PerturbLensLastVertex (AD) at light vertex nl - 2, ConnectToCamera (AD).
template <class T>
DEV T lens_logf(const SceneView &s, const LensAnchor &a, const T &sx, const T &sy) {
    TV3<T> org, dir;
    ad_sample_primary(s.cam, sx, sy, org, dir);
    TIsect<T> fix;
    fix.position = tv<T>(a.pos);
    fix.shadingNormal = tv<T>(a.ns);
    fix.geomNormal = tv<T>(a.ng);
    const TV3<T> fdir = tv<T>(a.dir);
    TV3<T> lens;
    TIsect<T> xm;
    ad_intersect(s, a.triMove, org, dir, xm);
    if (a.c >= 2) {
        const TV3<T> wi1 = -dir;
        TV3<T> w = fix.position - xm.position;
        const T distSq = dot(w, w);
        w = tnorm(w);
        TBsdf<T> o1, o2;
        ad_evaluate(bsdf_of_tri(s, a.triMove), wi1, xm.shadingNormal, w, o1);
        if (a.c == 3 && a.l == 1) {
            lens = o1.contrib * (1.0f / distSq);
        } else if (a.c >= 3) {
            const TV3<T> wi2 = -w;
            ad_evaluate(bsdf_of_tri(s, a.triFix), fdir, fix.shadingNormal, wi2, o2, true);
            lens = cmul(o1.contrib, o2.contrib * ad_snc(fdir, fix, wi2)) * (1.0f / distSq);
        } else {
            ad_evaluate(bsdf_of_tri(s, a.triFix), fdir, fix.shadingNormal, -w, o2, true);
            lens = cmul(o2.contrib * ad_snc(fdir, fix, -w), o1.contrib) * (1.0f / distSq);
        }
    } else {
        const TV3<T> w = tnorm(xm.position - fix.position);
        TBsdf<T> ob;
        ad_evaluate(bsdf_of_tri(s, a.triFix), fdir, fix.shadingNormal, w, ob, true);
        const TV3<T> prev = ob.contrib * ad_snc(w, fix, fdir);
        TIsect<T> xl;
        ad_intersect(s, a.triMove, fix.position, w, xl);
        TV3<T> co, cd;
        ad_sample_primary(s.cam, T(0.5f), T(0.5f), co, cd);
        const TV3<T> dtc = tnorm(co - xl.position);
        TBsdf<T> oc;
        ad_evaluate(bsdf_of_tri(s, a.triMove), dtc, xl.shadingNormal, -w, oc);
        const TV3<T> d2 = xl.position - fix.position;
        lens = cmul(oc.contrib, prev) * (1.0f / dot(d2, d2));
    }
    return log(tlum(lens));
}

// Whether the reference has a lens-mode derivative for technique (c, l)
// (CompilePathFuncLibrary, src/path.cpp:3186-3199: c + l > 3, c + l - 1 <= the
// derivative depth).
DEV bool lens_func_exists(int c, int l, int maxDerv) { return c + l > 3 && c + l - 1 <= maxDerv; }

// Gradient (2) and Hessian (2 x 2, row-major) of the lens-mode function at
// (sx, sy) by three hyper-dual evaluations; zeros unless the lens score exceeds
// 1e-15 (initLensGaussian, h2mc.cpp:470-491), non-finite results scrubbed.
DEV void lens_derivs(const SceneView &s, const LensAnchor &a, float sx, float sy, float lensScore, float *g,
                     float *h) {
    g[0] = g[1] = 0.0f;
    h[0] = h[1] = h[2] = h[3] = 0.0f;
    if (!(lensScore > 1e-15f)) return;
    const HyperDual fxx = lens_logf<HyperDual>(s, a, HyperDual(sx, 1.0f, 1.0f, 0.0f), HyperDual(sy));
    const HyperDual fxy = lens_logf<HyperDual>(s, a, HyperDual(sx, 1.0f, 0.0f, 0.0f), HyperDual(sy, 0.0f, 1.0f, 0.0f));
    const HyperDual fyy = lens_logf<HyperDual>(s, a, HyperDual(sx), HyperDual(sy, 1.0f, 1.0f, 0.0f));
    g[0] = fxx.a;
    g[1] = fyy.a;
    h[0] = fxx.ab;
    h[1] = h[2] = fxy.ab;
    h[3] = fyy.ab;
    bool finite = true;
    for (int i = 0; i < 2; i++) finite = finite && isfinite(g[i]);
    for (int i = 0; i < 4; i++) finite = finite && isfinite(h[i]);
    if (!finite) {
        g[0] = g[1] = 0.0f;
        h[0] = h[1] = h[2] = h[3] = 0.0f;
    }
}

// The 2-D lens Gaussian in its precision eigen-basis (invCov = V diag(p) V^T,
// V[i * 2 + k]: component i of eigenvector k), FP64.
struct LensGauss {
    double V[4], p[2], mean[2], logDet;
};

DEV void lens_gauss_isotropic(double sigma, LensGauss &G) {
    const double inv = 1.0 / (sigma * sigma);
    G.V[0] = G.V[3] = 1.0;
    G.V[1] = G.V[2] = 0.0;
    G.p[0] = G.p[1] = inv;
    G.mean[0] = G.mean[1] = 0.0;
    G.logDet = 2.0 * ::log(inv);
}

// ComputeGaussian (h2mc.cpp:607-640 and 14-83) for dimension 2: isotropic
// below the Frobenius-norm threshold or for ss <= 1e-15, else the eigenvalues
// of the Hessian's symmetric part (its upper triangle, as the reference's
// self-adjoint solver reads it) bounded with the L = pi/2 factors.
DEV void lens_gaussian(const H2mcParam &prm, float ss, const float *g, const float *h, LensGauss &G) {
    const double sigma = double(prm.sigma);
    double fro = 0.0;
    for (int i = 0; i < 4; i++) fro += double(h[i]) * double(h[i]);
    if (ss <= 1e-15f || ::sqrt(fro) < 0.5 / (sigma * sigma)) {
        lens_gauss_isotropic(sigma, G);
        return;
    }
    const double invSigmaSq = 1.0 / (sigma * sigma);
    const double A = h[0], B = h[1], D = h[3];
    const double m = 0.5 * (A + D), q = 0.5 * (A - D), r = ::hypot(q, B);
    const double th = 0.5 * ::atan2(2.0 * B, A - D);
    const double ct = ::cos(th), st = ::sin(th);
    const double lam[2] = {m - r, m + r};
    // eigenvector of m + r: (cos th, sin th); of m - r: (-sin th, cos th)
    G.V[0] = -st;
    G.V[2] = ct;
    G.V[1] = ct;
    G.V[3] = st;
    double logDet = 0.0, mc[2];
    for (int k = 0; k < 2; k++) {
        const double vg = G.V[k] * double(g[0]) + G.V[2 + k] * double(g[1]);
        double eb = ::fabs(lam[k]) > 1e-10 ? 1.0 / ::fabs(lam[k]) : 0.0;
        const double ob = eb * vg;
        double s2, o;
        if (::fabs(lam[k]) > 1e-10) {
            o = ob;
            if (lam[k] > 0.0) {
                s2 = prm.posScale;
                o *= prm.posOffset;
            } else {
                s2 = prm.negScale;
                o *= prm.negOffset;
            }
        } else {
            s2 = double(prm.L) * double(prm.L);
            o = 0.5 * ob * double(prm.L) * double(prm.L);
        }
        eb *= s2;
        eb = eb > 1e-10 ? 1.0 / eb : 0.0;
        const double post = eb + invSigmaSq;
        G.p[k] = post;
        logDet += ::log(post);
        mc[k] = eb / post * o;
    }
    for (int i = 0; i < 2; i++) G.mean[i] = G.V[i * 2] * mc[0] + G.V[i * 2 + 1] * mc[1];
    G.logDet = logDet;
}

// GaussianLogPdf (src/gaussian.cpp:18-26) of sign * off.
DEV double lens_logpdf(const LensGauss &G, const float *off, double sign) {
    double quad = 0.0;
    for (int k = 0; k < 2; k++) {
        const double proj = G.V[k] * (sign * double(off[0]) - G.mean[0]) + G.V[2 + k] * (sign * double(off[1]) - G.mean[1]);
        quad += G.p[k] * proj * proj;
    }
    return 2.0 * (-0.5 * ::log(2.0 * 3.14159265358979323846)) + 0.5 * G.logDet - 0.5 * quad;
}

// The lens Gaussian of a state: its derivatives and ComputeGaussian when the
// reference has a lens function for the technique, else IsotropicGaussian.
DEV void lens_gaussian_of(const SceneView &s, const PathRec &r, const LensAnchor &a, float sx, float sy, float lensScore,
                          float ss, int maxDerv, const H2mcParam &prm, LensGauss &G) {
    if (!lens_func_exists(r.c, r.l, maxDerv)) {
        lens_gauss_isotropic(double(prm.sigma), G);
        return;
    }
    float g[2], h[4];
    lens_derivs(s, a, sx, sy, lensScore, g, h);
    lens_gaussian(prm, ss, g, h, G);
}

}  // namespace drmlt
