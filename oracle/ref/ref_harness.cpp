// Golden-vector harness around the reference's own functions (test
// infrastructure; links the reference objects built by oracle/ref/Makefile).
//
// It calls, unmodified:
//   GeneratePathBidir      src/path.cpp:978-1121  (prepass / bootstrap sampler)
//   GenerateSubpath        src/path.cpp:1123-1269 (multiplexed large step)
//   GeneratePath           src/path.cpp:343-445   (direct-lighting pass)
//   PerturbPathBidir       src/path.cpp:1480-1628 (small steps, Green y*)
//   GetPathPos / Serialize src/path.cpp:2303-2439
//   chad static path function + derivative (generated pathlibbidir.so)
//   PH2MCSmallStep::ComputeGaussian src/integrators/delayed/drsmallstep.cpp:219-266
//   PerturbLensBidir + chad lens-mode functions, ComputeGaussian (h2mc.cpp:607-640)
// and writes JSON lines. Every random number a sampler consumed is recorded
// (the reference draws them with std::uniform_real_distribution from a
// pcg32_k64_fast stream), so a replay of the same stream must reproduce the
// same path exactly. Perturbations run with discreteStdDev = 0 so that only
// the continuous offsets move the path.
//
// usage: ref_harness <scene.xml> <libdir> <maxDervDepth> <out.jsonl> <mode> <seed0> <count> [extra]
//   mode = camera | bidir | subpath | direct | tech | accept | lens | mesh
//   (mesh: every shape's triangles as loaded by ParseObj / LoadSerialized,
//    src/parseobj.cpp:148-264, src/loadserialized.cpp:236-317)
#include "parsescene.h"
#include "path.h"
#include "scene.h"
#include "shape.h"
#include "trianglemesh.h"
#include "light.h"
#include "camera.h"
#include "gaussian.h"
#include "integrators/delayed/drsmallstep.h"
#include "integrators/h2mc.h"
#include "mutation.h"
#include "distribution.h"
#include "texturesystem.h"
#include <cstdio>
#include <unistd.h>

namespace {

const Scene *g_scene = nullptr;
FILE *g_out = nullptr;

int ShapeIndex(const Shape *s) {
    if (s == nullptr) return -1;
    for (size_t i = 0; i < g_scene->objects.size(); i++)
        if (g_scene->objects[i].get() == s) return int(i);
    return -2;
}

int LightIndex(const Light *l) {
    if (l == nullptr) return -1;
    for (size_t i = 0; i < g_scene->lights.size(); i++)
        if (g_scene->lights[i].get() == l) return int(i);
    return -2;
}

void F(double v) {
    if (std::isfinite(v)) fprintf(g_out, "%.9g", v);
    else fprintf(g_out, "null");
}

template <typename V>
void Arr(const V &v, int n) {
    fputc('[', g_out);
    for (int i = 0; i < n; i++) {
        if (i) fputc(',', g_out);
        F(double(v[i]));
    }
    fputc(']', g_out);
}

void DumpVertex(const SurfaceVertex &v) {
    fprintf(g_out, "{\"shape\":%d,\"prim\":%d,\"bsdfRnd\":", ShapeIndex(v.shapeInst.obj),
            v.shapeInst.obj ? v.shapeInst.primID : -1);
    Arr(v.bsdfRndParam, 2);
    fprintf(g_out, ",\"disc\":");
    F(v.bsdfDiscrete);
    fprintf(g_out, ",\"useAbs\":");
    F(v.useAbsoluteParam);
    fprintf(g_out, ",\"rr\":");
    F(v.rrWeight);
    fprintf(g_out, ",\"dlLight\":%d,\"dlPrim\":%d,\"dlRnd\":", LightIndex(v.directLightInst.light),
            v.directLightInst.light ? v.directLightInst.lPrimID : -1);
    Arr(v.directLightRndParam, 2);
    fputc('}', g_out);
}

void DumpPath(const Path &p) {
    fprintf(g_out, "{\"time\":");
    F(p.time);
    fprintf(g_out, ",\"lgtLight\":%d,\"lgtPrim\":%d,\"lgtPos\":", LightIndex(p.lgtVertex.lightInst.light),
            p.lgtVertex.lightInst.light ? p.lgtVertex.lightInst.lPrimID : -1);
    Arr(p.lgtVertex.rndParamPos, 2);
    fprintf(g_out, ",\"lgtDir\":");
    Arr(p.lgtVertex.rndParamDir, 2);
    fprintf(g_out, ",\"screen\":");
    Arr(p.camVertex.screenPos, 2);
    fprintf(g_out, ",\"lgtSurf\":[");
    for (size_t i = 0; i < p.lgtSurfaceVertex.size(); i++) {
        if (i) fputc(',', g_out);
        DumpVertex(p.lgtSurfaceVertex[i]);
    }
    fprintf(g_out, "],\"camSurf\":[");
    for (size_t i = 0; i < p.camSurfaceVertex.size(); i++) {
        if (i) fputc(',', g_out);
        DumpVertex(p.camSurfaceVertex[i]);
    }
    fprintf(g_out, "],\"isSubpath\":%d,\"camDepth\":%d,\"lgtDepth\":%d}", int(p.isSubpath),
            p.isSubpath ? p.camDepth : -1, p.isSubpath ? p.lgtDepth : -1);
}

void DumpContribs(const std::vector<SubpathContrib> &cs) {
    fputc('[', g_out);
    for (size_t i = 0; i < cs.size(); i++) {
        const SubpathContrib &c = cs[i];
        if (i) fputc(',', g_out);
        fprintf(g_out, "{\"camDepth\":%d,\"lightDepth\":%d,\"screen\":", c.camDepth, c.lightDepth);
        Arr(c.screenPos, 2);
        fprintf(g_out, ",\"contrib\":");
        Arr(c.contrib, 3);
        fprintf(g_out, ",\"ls\":");
        F(c.lsScore);
        fprintf(g_out, ",\"ss\":");
        F(c.ssScore);
        fprintf(g_out, ",\"mis\":");
        F(c.misWeight);
        fprintf(g_out, ",\"lens\":");
        F(c.lensScore);
        fputc('}', g_out);
    }
    fputc(']', g_out);
}

// Records the uniforms a sampler seeded with `seed` will hand out, and after the
// sampler ran, how many it consumed.
struct UniformTape {
    std::vector<float> values;
    RNG start;
    explicit UniformTape(uint64_t seed, int n) : start(seed) {
        RNG copy = start;
        std::uniform_real_distribution<Float> uni(Float(0.0), Float(1.0));
        for (int i = 0; i < n; i++) values.push_back(uni(copy));
    }
    // Number of uniforms consumed: the position in the recorded stream where the
    // sampler's remaining draws continue.
    int Consumed(const RNG &after) const {
        RNG next = after;
        std::uniform_real_distribution<Float> uni(Float(0.0), Float(1.0));
        float probe[8];
        for (int k = 0; k < 8; k++) probe[k] = uni(next);
        for (int i = 0; i + 8 <= int(values.size()); i++) {
            bool same = true;
            for (int k = 0; k < 8 && same; k++) same = values[i + k] == probe[k];
            if (same) return i;
        }
        return -1;
    }
    void Dump(int consumed) {
        fprintf(g_out, "\"uniforms\":");
        Arr(values, consumed < 0 ? int(values.size()) : consumed);
        fprintf(g_out, ",\"consumed\":%d", consumed);
    }
};

void ModeBidir(uint64_t seed0, int count, int minDepth, int maxDepth) {
    for (int s = 0; s < count; s++) {
        UniformTape tape(seed0 + s, 512);
        RNG rng = tape.start;
        Path path;
        std::vector<SubpathContrib> contribs;
        GeneratePathBidir(g_scene, Vector2i(-1, -1), minDepth, maxDepth, path, contribs, rng);
        fprintf(g_out, "{\"mode\":\"bidir\",\"seed\":%llu,", (unsigned long long)(seed0 + s));
        tape.Dump(tape.Consumed(rng));
        fprintf(g_out, ",\"minDepth\":%d,\"maxDepth\":%d,\"path\":", minDepth, maxDepth);
        DumpPath(path);
        fprintf(g_out, ",\"contribs\":");
        DumpContribs(contribs);
        fprintf(g_out, "}\n");
    }
}

void ModeSubpath(uint64_t seed0, int count, int maxDepth) {
    for (int s = 0; s < count; s++) {
        // Technique from the seed, the same way LargeStep::Mutate draws it
        // (src/mutation.cpp:32-42) but from a separate stream.
        RNG pick(1000003u * (seed0 + s) + 7u);
        std::uniform_real_distribution<Float> uni(Float(0.0), Float(1.0));
        const int length = 3 + std::min(int(uni(pick) * (maxDepth - 2)), maxDepth - 3);
        const int lgtLength = Clamp(int(uni(pick) * (length + 1)), 0, length);
        const int camLength = length - lgtLength + 1;
        UniformTape tape(seed0 + s, 256);
        RNG rng = tape.start;
        Path path;
        std::vector<SubpathContrib> contribs;
        GenerateSubpath(g_scene, Vector2i(-1, -1), camLength, lgtLength, true, path, contribs, rng);
        fprintf(g_out, "{\"mode\":\"subpath\",\"seed\":%llu,\"camLength\":%d,\"lgtLength\":%d,",
                (unsigned long long)(seed0 + s), camLength, lgtLength);
        tape.Dump(tape.Consumed(rng));
        fprintf(g_out, ",\"path\":");
        DumpPath(path);
        fprintf(g_out, ",\"contribs\":");
        DumpContribs(contribs);
        fprintf(g_out, "}\n");
    }
}

void ModeDirect(uint64_t seed0, int count) {
    const Camera *camera = g_scene->camera.get();
    const int w = GetPixelWidth(camera), h = GetPixelHeight(camera);
    for (int s = 0; s < count; s++) {
        const int x = int((seed0 + s) * 7919u % unsigned(w));
        const int y = int((seed0 + s) * 104729u % unsigned(h));
        UniformTape tape(seed0 + s, 64);
        RNG rng = tape.start;
        Path path;
        std::vector<SubpathContrib> contribs;
        GeneratePath(g_scene, Vector2i(x, y), std::min(g_scene->options->minDepth, 2),
                     std::min(g_scene->options->maxDepth, 2), path, contribs, rng);
        fprintf(g_out, "{\"mode\":\"direct\",\"seed\":%llu,\"pixel\":[%d,%d],",
                (unsigned long long)(seed0 + s), x, y);
        tape.Dump(tape.Consumed(rng));
        fprintf(g_out, ",\"contribs\":");
        DumpContribs(contribs);
        fprintf(g_out, "}\n");
    }
}

void ModeTech(uint64_t seed0, int count, int nPerturb, const PathFuncLib &lib, int maxDervDepth) {
    const int maxDepth = g_scene->options->maxDepth;
    const int minDepth = std::max(g_scene->options->minDepth, 3);
    AlignedStdVector sceneParams(GetSceneSerializedSize());
    Serialize(g_scene, &sceneParams[0]);
    SerializedSubpath ssub;
    ssub.primary.resize(GetPrimaryParamSize(maxDervDepth, maxDervDepth));
    ssub.vertParams.resize(GetVertParamSize(maxDervDepth, maxDervDepth));
    PH2MCSmallStep h2mc(g_scene, maxDervDepth, g_scene->options->perturbStdDev);
    const Float sigmas[3] = {g_scene->options->perturbStdDev, Float(0.0025), Float(0.05)};
    int written = 0;
    for (int s = 0; written < count && s < 100 * count; s++) {
        RNG rng(seed0 + s);
        Path full;
        std::vector<SubpathContrib> contribs;
        GeneratePathBidir(g_scene, Vector2i(-1, -1), minDepth, maxDepth, full, contribs, rng);
        for (const SubpathContrib &c : contribs) {
            if (written >= count) break;
            Path path = full;
            path.Initialize(c.camDepth, c.lightDepth);
            const int dim = GetDimension(path);
            const Vector x = GetPathPos(path);
            fprintf(g_out, "{\"mode\":\"tech\",\"seed\":%llu,\"dim\":%d,\"path\":",
                    (unsigned long long)(seed0 + s), dim);
            DumpPath(path);
            fprintf(g_out, ",\"contrib\":");
            DumpContribs({c});
            fprintf(g_out, ",\"pos\":");
            Arr(x, dim);
            // Derivatives of log Lum(contrib) from the chad library (static mode,
            // time excluded), as PH2MCSmallStep::Mutate calls them
            // (src/integrators/delayed/drsmallstep.cpp:128-158).
            AlignedStdVector grad(dim, Float(0.0)), hess(dim * dim, Float(0.0));
            auto dit = lib.staticDervFuncMap.find({c.camDepth, c.lightDepth});
            auto fit = lib.staticFuncMap.find({c.camDepth, c.lightDepth});
            bool haveDerv = dit != lib.staticDervFuncMap.end();
            Float logf = Float(0.0);
            bool scrubbed = false;
            if (haveDerv && c.ssScore > Float(1e-15)) {
                Serialize(g_scene, path, ssub);
                dit->second(&c.screenPos[0], &ssub.primary[0], &sceneParams[0], &ssub.vertParams[0],
                            &grad[0], &hess[0]);
                if (fit != lib.staticFuncMap.end())
                    fit->second(&c.screenPos[0], &ssub.primary[0], &sceneParams[0], &ssub.vertParams[0],
                                &logf);
                if (!IsFinite(grad) || !IsFinite(hess)) {
                    scrubbed = true;
                    std::fill(grad.begin(), grad.end(), Float(0.0));
                    std::fill(hess.begin(), hess.end(), Float(0.0));
                }
            }
            // Central differences of the chad gradient (h = 1e-3, same library): a
            // consistency check of chad's own Hessian.
            std::vector<double> fdH(size_t(dim) * dim, 0.0);
            if (haveDerv && c.ssScore > Float(1e-15)) {
                AlignedStdVector g2(dim), h2(dim * dim);
                for (int j = 0; j < dim; j++) {
                    for (int sgn = -1; sgn <= 1; sgn += 2) {
                        Path q = path;
                        SerializedSubpath sq = ssub;
                        Serialize(g_scene, q, sq);
                        sq.primary[1 + j] += Float(sgn) * Float(1e-3);
                        dit->second(&c.screenPos[0], &sq.primary[0], &sceneParams[0], &sq.vertParams[0], &g2[0], &h2[0]);
                        for (int i = 0; i < dim; i++) fdH[size_t(i) * dim + j] += double(sgn) * double(g2[i]) / 2e-3;
                    }
                }
            }
            fprintf(g_out, ",\"fdHess\":");
            Arr(fdH, dim * dim);
            fprintf(g_out, ",\"haveDerv\":%d,\"scrubbed\":%d,\"logf\":", int(haveDerv), int(scrubbed));
            F(logf);
            fprintf(g_out, ",\"grad\":");
            Arr(grad, dim);
            fprintf(g_out, ",\"hess\":");
            Arr(hess, dim * dim);
            Gaussian g;
            if (haveDerv) {
                h2mc.ComputeGaussian(h2mc.param, c.ssScore, grad, hess, g);
            } else {
                IsotropicGaussian(dim, h2mc.param.sigma, g);
            }
            fprintf(g_out, ",\"gauss\":{\"mean\":");
            Arr(g.mean, dim);
            Matrix cov = g.covL * g.covL.transpose();
            fprintf(g_out, ",\"invCov\":");
            Arr(g.invCov.data(), dim * dim);
            fprintf(g_out, ",\"covL\":");
            Arr(g.covL.data(), dim * dim);
            fprintf(g_out, ",\"cov\":");
            Arr(cov.data(), dim * dim);
            fprintf(g_out, ",\"logDet\":");
            F(g.logDet);
            fprintf(g_out, "},\"perturb\":[");
            for (int p = 0; p < nPerturb; p++) {
                RNG prng(7777u * (seed0 + s) + 31u * written + p);
                std::normal_distribution<Float> nd(Float(0.0), sigmas[p % 3]);
                Vector offset(dim);
                for (int i = 0; i < dim; i++) offset[i] = nd(prng);
                Path y = path;
                std::vector<SubpathContrib> ycs;
                PerturbPathBidir(g_scene, offset, y, ycs, prng);
                if (p) fputc(',', g_out);
                fprintf(g_out, "{\"offset\":");
                Arr(offset, dim);
                fprintf(g_out, ",\"logpdf\":");
                F(GaussianLogPdf(offset, g));
                fprintf(g_out, ",\"ypos\":");
                Arr(GetPathPos(y), dim);
                fprintf(g_out, ",\"path\":");
                DumpPath(y);
                fprintf(g_out, ",\"contribs\":");
                DumpContribs(ycs);
                fputc('}', g_out);
            }
            fprintf(g_out, "]}\n");
            written++;
        }
    }
}

// The lens mutation of H2MCSmallStep::Mutate (src/integrators/h2mc.cpp:466-532)
// on technique paths x (bootstrap samples, as in ModeTech): x's lens score
// (SubpathContrib::lensScore from the sampler), its lens vertex position, the
// chad lens-mode log f and its gradient / Hessian with respect to the screen
// position (lensFuncMap / lensDervFuncMap, called as initLensGaussian calls
// them), the 2-D Gaussian the integrator's ComputeGaussian (h2mc.cpp:607-640)
// builds from them with lensPerturbStdDev, and PerturbLensBidir
// (src/path.cpp:1913-2078) at screen positions x.screen + offset (mod 1).
// Techniques with a zero lens score are kept one in four (no perturbation).
void ModeLens(uint64_t seed0, int count, int nPerturb, const PathFuncLib &lib, int maxDervDepth) {
    const int maxDepth = g_scene->options->maxDepth;
    const int minDepth = std::max(g_scene->options->minDepth, 3);
    AlignedStdVector sceneParams(GetSceneSerializedSize());
    Serialize(g_scene, &sceneParams[0]);
    SerializedSubpath ssub;
    ssub.primary.resize(GetPrimaryParamSize(maxDervDepth, maxDervDepth));
    ssub.vertParams.resize(GetVertParamSize(maxDervDepth, maxDervDepth));
    const H2MCIntegrator::H2MCParam lensParam(g_scene->options->lensPerturbStdDev);
    const Float sigmas[3] = {lensParam.sigma, Float(0.003), Float(0.03)};
    int written = 0, zeros = 0;
    for (int s = 0; written < count && s < 100 * count; s++) {
        RNG rng(seed0 + s);
        Path full;
        std::vector<SubpathContrib> contribs;
        GeneratePathBidir(g_scene, Vector2i(-1, -1), minDepth, maxDepth, full, contribs, rng);
        for (const SubpathContrib &c : contribs) {
            if (written >= count) break;
            if (!(c.lensScore > Float(0.0)) && (zeros++ % 4) != 0) continue;
            Path path = full;
            path.Initialize(c.camDepth, c.lightDepth);
            const int dim = GetDimension(path);
            fprintf(g_out, "{\"mode\":\"lens\",\"seed\":%llu,\"dim\":%d,\"path\":", (unsigned long long)(seed0 + s),
                    dim);
            DumpPath(path);
            fprintf(g_out, ",\"contrib\":");
            DumpContribs({c});
            fprintf(g_out, ",\"pos\":");
            Arr(GetPathPos(path), dim);
            fprintf(g_out, ",\"lensPos\":");
            Arr(path.lensVertexPos, 3);
            AlignedStdVector grad(2, Float(0.0)), hess(4, Float(0.0));
            auto dit = lib.lensDervFuncMap.find({c.camDepth, c.lightDepth});
            auto fit = lib.lensFuncMap.find({c.camDepth, c.lightDepth});
            const bool haveDerv = dit != lib.lensDervFuncMap.end();
            Float logf = Float(0.0);
            bool scrubbed = false;
            if (haveDerv && c.lensScore > Float(1e-15)) {
                Serialize(g_scene, path, ssub);
                dit->second(&c.screenPos[0], &ssub.primary[0], &sceneParams[0], &ssub.vertParams[0], &grad[0],
                            &hess[0]);
                if (fit != lib.lensFuncMap.end())
                    fit->second(&c.screenPos[0], &ssub.primary[0], &sceneParams[0], &ssub.vertParams[0], &logf);
                if (!IsFinite(grad) || !IsFinite(hess)) {
                    scrubbed = true;
                    std::fill(grad.begin(), grad.end(), Float(0.0));
                    std::fill(hess.begin(), hess.end(), Float(0.0));
                }
            }
            // Central differences of chad's lens gradient (h = 1e-4 in the screen
            // position): a consistency check of chad's own lens Hessian.
            std::vector<double> fdH(4, 0.0);
            if (haveDerv && c.lensScore > Float(1e-15)) {
                AlignedStdVector g2(2), h2(4);
                for (int j = 0; j < 2; j++) {
                    for (int sgn = -1; sgn <= 1; sgn += 2) {
                        Vector2 sp = c.screenPos;
                        sp[j] += Float(sgn) * Float(1e-4);
                        dit->second(&sp[0], &ssub.primary[0], &sceneParams[0], &ssub.vertParams[0], &g2[0], &h2[0]);
                        for (int i = 0; i < 2; i++) fdH[i * 2 + j] += double(sgn) * double(g2[i]) / 2e-4;
                    }
                }
            }
            fprintf(g_out, ",\"haveDerv\":%d,\"scrubbed\":%d,\"logf\":", int(haveDerv), int(scrubbed));
            F(logf);
            fprintf(g_out, ",\"grad\":");
            Arr(grad, 2);
            fprintf(g_out, ",\"hess\":");
            Arr(hess, 4);
            fprintf(g_out, ",\"fdHess\":");
            Arr(fdH, 4);
            Gaussian g;
            if (haveDerv) {
                ComputeGaussian(lensParam, c.ssScore, grad, hess, g);
            } else {
                IsotropicGaussian(2, lensParam.sigma, g);
            }
            fprintf(g_out, ",\"gauss\":{\"mean\":");
            Arr(g.mean, 2);
            fprintf(g_out, ",\"invCov\":");
            Arr(g.invCov.data(), 4);
            fprintf(g_out, ",\"logDet\":");
            F(g.logDet);
            fprintf(g_out, "},\"perturb\":[");
            for (int p = 0; c.lensScore > Float(0.0) && p < nPerturb; p++) {
                RNG prng(9191u * (seed0 + s) + 37u * written + p);
                std::normal_distribution<Float> nd(Float(0.0), sigmas[p % 3]);
                Vector offset(2);
                offset[0] = nd(prng);
                offset[1] = nd(prng);
                Vector2 screen(Modulo(c.screenPos[0] + offset[0], Float(1.0)),
                               Modulo(c.screenPos[1] + offset[1], Float(1.0)));
                Path y = path;
                std::vector<SubpathContrib> ycs;
                PerturbLensBidir(g_scene, screen, y, ycs);
                if (p) fputc(',', g_out);
                fprintf(g_out, "{\"offset\":");
                Arr(offset, 2);
                fprintf(g_out, ",\"screen\":");
                Arr(screen, 2);
                fprintf(g_out, ",\"logpdf\":");
                F(GaussianLogPdf(offset, g));
                fprintf(g_out, ",\"ypos\":");
                Arr(GetPathPos(y), dim);
                fprintf(g_out, ",\"path\":");
                DumpPath(y);
                fprintf(g_out, ",\"lensPos\":");
                Arr(y.lensVertexPos, 3);
                fprintf(g_out, ",\"contribs\":");
                DumpContribs(ycs);
                fputc('}', g_out);
            }
            fprintf(g_out, "]}\n");
            written++;
        }
    }
}

// Per-stage acceptances of one delayed-rejection iteration, from the
// reference's own mutation code on fixed current states with recorded draws.
// For each technique path x (bootstrap samples, as in ModeTech):
//   large   LargeStep::Mutate (src/mutation.cpp:7-120) on a recorded uniform
//           stream with a fixed path-length distribution: its proposal and a1;
//   small   SmallStep::Mutate (mutation.cpp:126-166): offsets o1 (recorded from
//           the same stream) -> y and a1;
//   iso     SmallStep::Mutate with the second-stage sigma (mutation.cpp:167-208):
//           o2 -> z and a2;
//   h2mc    PH2MCSmallStep::Mutate (drsmallstep.cpp:113-212): its offset
//           (GenerateSample from the Gaussian at x, recorded by replaying the
//           stream), z, the unclamped ratio a2 and log N_z(-o) - log N_x(o)
//           (GaussianLogPdf, gaussian.cpp:18-34);
//   y*      SmallStep::Trace (mutation.cpp:210-238) of z by x - y, per second stage;
// and the second-stage acceptances of Green & Mira and of Tierney & Mira, the
// blocks of delayed.cpp:466-541 restated below on those values (they are
// inline in DRIntegrator::Render, so there is no function to call).
void ModeAccept(uint64_t seed0, int count, const PathFuncLib &lib, int maxDervDepth) {
    const Scene *scene = g_scene;
    const int maxDepth = scene->options->maxDepth;
    const int minDepth = std::max(scene->options->minDepth, 3);
    const MLTState mltState{scene, GeneratePathBidir, PerturbPathBidir, PerturbLensBidir, lib.funcMap,
                            lib.dervFuncMap, lib.staticFuncMap, lib.staticDervFuncMap, lib.lensFuncMap,
                            lib.lensDervFuncMap};
    // a fixed, uneven path-length distribution over lengths 0..maxDepth
    std::vector<Float> lengthFunc(maxDepth + 1, Float(0.0));
    for (int L = 2; L <= maxDepth; L++) lengthFunc[L] = Float(1.0) + Float(0.25) * Float(L % 3) + Float(L);
    auto lengthDist = std::make_shared<PiecewiseConstant1D>(&lengthFunc[0], int(lengthFunc.size()));
    LargeStep largeStep(lengthDist);
    SmallStep smallStep;
    PH2MCSmallStep h2mc(scene, maxDervDepth, scene->options->perturbStdDev);
    const Float sigma1 = scene->options->perturbStdDev;
    const Float sigma2 = scene->options->anisoperturbstddev;
    const Float b = Float(1.0);
    auto isInvalid = [](Float x) { return std::isnan(x) || std::isinf(x) || x < Float(0.0); };
    auto metropolisClamp = [](Float x) { return std::min(Float(1.0), x); };
    int written = 0;
    for (int s = 0; written < count && s < 100 * count; s++) {
        RNG brng(seed0 + s);
        Path full;
        std::vector<SubpathContrib> contribs;
        GeneratePathBidir(scene, Vector2i(-1, -1), minDepth, maxDepth, full, contribs, brng);
        for (const SubpathContrib &c : contribs) {
            if (written >= count) break;
            const uint64_t cs = 1000u * (seed0 + s) + uint64_t(written);
            MarkovState cur;
            cur.valid = true;
            cur.spContrib = c;
            cur.path = full;
            cur.path.Initialize(c.camDepth, c.lightDepth);
            const int dim = GetDimension(cur.path);
            const Vector x = GetPathPos(cur.path);
            fprintf(g_out, "{\"mode\":\"accept\",\"seed\":%llu,\"dim\":%d,\"path\":", (unsigned long long)(seed0 + s),
                    dim);
            DumpPath(cur.path);
            fprintf(g_out, ",\"contrib\":");
            DumpContribs({c});
            fprintf(g_out, ",\"pos\":");
            Arr(x, dim);
            fprintf(g_out, ",\"sigma1\":");
            F(sigma1);
            fprintf(g_out, ",\"sigma2\":");
            F(sigma2);
            fprintf(g_out, ",\"lengthFunc\":");
            Arr(lengthFunc, int(lengthFunc.size()));
            // ---- large step
            {
                UniformTape tape(cs * 4u + 0u, 1024);
                RNG rng = tape.start;
                MarkovState prop;
                const Float a = largeStep.Mutate(mltState, b, cur, prop, rng);
                fprintf(g_out, ",\"large\":{");
                tape.Dump(tape.Consumed(rng));
                fprintf(g_out, ",\"a1\":");
                F(a);
                fprintf(g_out, ",\"contribs\":");
                DumpContribs(largeStep.spContribs);
                fputc('}', g_out);
            }
            // ---- first stage, isotropic small step
            MarkovState Y;
            Vector o1(dim);
            Float a1;
            {
                RNG rng(cs * 4u + 1u);
                RNG copy = rng;
                std::normal_distribution<Float> nd(Float(0.0), sigma1);
                for (int i = 0; i < dim; i++) o1[i] = nd(copy);
                a1 = smallStep.Mutate(mltState, b, cur, Y, rng);
                const bool valid = !smallStep.spContribs.empty();
                fprintf(g_out, ",\"small\":{\"offset\":");
                Arr(o1, dim);
                fprintf(g_out, ",\"a1\":");
                F(a1);
                fprintf(g_out, ",\"valid\":%d,\"ss\":", int(valid));
                F(valid ? Y.spContrib.ssScore : Float(0.0));
                fprintf(g_out, ",\"ypos\":");
                Arr(GetPathPos(Y.path), dim);
                fputc('}', g_out);
                if (isInvalid(a1)) a1 = Float(0.0);
            }
            const Vector y = GetPathPos(Y.path);
            // ---- second stages
            for (int kind = 0; kind < 2; kind++) {
                MarkovState Z;
                Vector o2(dim);
                Float a2;
                double logRatio = 0.0;
                RNG rng(cs * 4u + 2u + kind);
                if (kind == 0) {
                    RNG copy = rng;
                    std::normal_distribution<Float> nd(Float(0.0), sigma2);
                    for (int i = 0; i < dim; i++) o2[i] = nd(copy);
                    a2 = smallStep.Mutate(mltState, b, cur, Z, sigma2, rng);
                } else {
                    // the offset GenerateSample draws from the Gaussian at x: Mutate
                    // computes that Gaussian first without drawing, so the same
                    // Gaussian and a copy of the stream give the same offset
                    cur.gaussianInitialized = false;
                    a2 = h2mc.Mutate(mltState, b, cur, Z, rng);
                    RNG copy(cs * 4u + 2u + kind);
                    GenerateSample(cur.gaussian, o2, copy);
                    if (!h2mc.spContribs.empty()) {
                        const Float py = GaussianLogPdf(o2, cur.gaussian);
                        const Float px = GaussianLogPdf(Vector(-o2), Z.gaussian);
                        logRatio = double(px) - double(py);
                    }
                }
                const bool validZ = kind == 0 ? !smallStep.spContribs.empty() : !h2mc.spContribs.empty();
                const Float ssZ = validZ ? Z.spContrib.ssScore : Float(0.0);
                // Green's reverse path from z (the proposal object counts as a
                // valid state, as after the chain's first second-stage accept)
                Float aStar = Float(0.0);
                if (validZ) {
                    Z.valid = true;
                    MarkovState star;
                    RNG trng(cs * 4u + 3u);
                    Vector off = x - y;
                    aStar = smallStep.Trace(mltState, off, Z, star, trng);
                }
                // delayed.cpp:466-541
                Float alphaGreen = Float(0.0), alphaMira = Float(0.0), transRatio = Float(0.0);
                Float a2v = a2;
                if (!isInvalid(a2v)) {
                    Float as = isInvalid(aStar) ? Float(0.0) : aStar;
                    alphaGreen = as == Float(1.0) ? Float(0.0) : metropolisClamp(a2v * (Float(1.0) - as) / (Float(1.0) - a1));
                    // Y.spContrib keeps its zero default when the first stage did not contribute
                    Float am = metropolisClamp(Y.spContrib.ssScore / ssZ);
                    am = isInvalid(am) ? Float(1.0) : am;
                    if (am != Float(1.0)) {
                        const Vector z = GetPathPos(Z.path);
                        Gaussian gaussIso;
                        IsotropicGaussian(int(y.size()), sigma1, gaussIso);
                        transRatio = std::exp(GaussianLogPdf(Vector(z - y), gaussIso) - GaussianLogPdf(Vector(x - y), gaussIso));
                        if (!isInvalid(transRatio))
                            alphaMira = metropolisClamp(a2v * transRatio * (Float(1.0) - am) / (Float(1.0) - a1));
                    }
                }
                fprintf(g_out, ",\"%s\":{\"offset\":", kind == 0 ? "iso" : "h2mc");
                Arr(o2, dim);
                fprintf(g_out, ",\"a2\":");
                F(a2);
                fprintf(g_out, ",\"logRatio\":");
                F(logRatio);
                fprintf(g_out, ",\"valid\":%d,\"ss\":", int(validZ));
                F(ssZ);
                fprintf(g_out, ",\"zpos\":");
                Arr(GetPathPos(Z.path), dim);
                fprintf(g_out, ",\"aStar\":");
                F(aStar);
                fprintf(g_out, ",\"transRatio\":");
                F(transRatio);
                fprintf(g_out, ",\"alphaGreen\":");
                F(alphaGreen);
                fprintf(g_out, ",\"alphaMira\":");
                F(alphaMira);
                fputc('}', g_out);
            }
            fprintf(g_out, "}\n");
            written++;
        }
    }
}

// Per shape: the world-space corner positions and shading normals of every
// triangle, in TriMeshData index order.
void ModeMesh() {
    for (size_t i = 0; i < g_scene->objects.size(); i++) {
        const TriangleMesh *m = dynamic_cast<const TriangleMesh *>(g_scene->objects[i].get());
        if (m == nullptr) continue;
        const TriMeshData &d = *m->data;
        for (int pass = 0; pass < 2; pass++) {
            fprintf(g_out, pass == 0 ? "{\"shape\":%d,\"p\":[" : "],\"n\":[", int(i));
            const std::vector<Vector3> &v = pass == 0 ? d.position0 : d.normal0;
            bool first = true;
            for (const TriIndex &t : d.indices)
                for (int k = 0; k < 3; k++)
                    for (int c = 0; c < 3; c++) {
                        if (!first) fputc(',', g_out);
                        first = false;
                        F(v[t.index[k]][c]);
                    }
        }
        fprintf(g_out, "]}\n");
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc < 8) {
        fprintf(stderr, "usage: %s scene.xml libdir maxDervDepth out.jsonl mode seed0 count [extra]\n", argv[0]);
        return 2;
    }
    TextureSystem::Init();
    std::unique_ptr<Scene> scene = ParseScene(argv[1]);
    scene->options->bidirectional = true;
    scene->options->discreteStdDev = Float(0.0);
    g_scene = scene.get();
    const std::string libdir = argv[2];
    const int maxDervDepth = atoi(argv[3]);
    g_out = fopen(argv[4], "w");
    const std::string mode = argv[5];
    const uint64_t seed0 = strtoull(argv[6], nullptr, 10);
    const int count = atoi(argv[7]);
    const int extra = argc > 8 ? atoi(argv[8]) : 0;
    if (mode == "camera") {
        // The reference camera's matrices (src/camera.cpp:11-28, animatedtransform.cpp:33-44).
        const Camera *cam = scene->camera.get();
        const Matrix4x4 c2w = Interpolate(cam->camToWorld, Float(0.0));
        const Matrix4x4 w2c = Interpolate(cam->worldToCamera, Float(0.0));
        auto M = [&](const char *name, const Matrix4x4 &m) {
            fprintf(g_out, "\"%s\":[", name);
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) {
                    if (r || c) fputc(',', g_out);
                    F(m(r, c));
                }
            fprintf(g_out, "],");
        };
        fputc('{', g_out);
        M("sampleToCam", cam->sampleToCam);
        M("camToSample", cam->camToSample);
        M("camToWorld", c2w);
        M("worldToCam", w2c);
        fprintf(g_out, "\"dist\":");
        F(cam->dist);
        fprintf(g_out, ",\"near\":");
        F(cam->nearClip);
        fprintf(g_out, ",\"far\":");
        F(cam->farClip);
        fprintf(g_out, ",\"bsCenter\":");
        Arr(scene->bSphere.center, 3);
        fprintf(g_out, ",\"bsRadius\":");
        F(scene->bSphere.radius);
        fprintf(g_out, "}\n");
    } else if (mode == "bidir") {
        ModeBidir(seed0, count, std::max(scene->options->minDepth, 3), scene->options->maxDepth);
    } else if (mode == "subpath") {
        ModeSubpath(seed0, count, scene->options->maxDepth);
    } else if (mode == "direct") {
        ModeDirect(seed0, count);
    } else if (mode == "mesh") {
        ModeMesh();
    } else if (mode == "tech") {
        if (chdir(libdir.c_str()) != 0) return 3;
        std::shared_ptr<const PathFuncLib> lib = BuildPathFuncLibrary(true, maxDervDepth, true);
        ModeTech(seed0, count, extra, *lib, maxDervDepth);
    } else if (mode == "lens") {
        if (chdir(libdir.c_str()) != 0) return 3;
        std::shared_ptr<const PathFuncLib> lib = BuildPathFuncLibrary(true, maxDervDepth, true);
        ModeLens(seed0, count, extra, *lib, maxDervDepth);
    } else if (mode == "accept") {
        if (chdir(libdir.c_str()) != 0) return 3;
        std::shared_ptr<const PathFuncLib> lib = BuildPathFuncLibrary(true, maxDervDepth, true);
        ModeAccept(seed0, count, *lib, maxDervDepth);
    } else {
        return 2;
    }
    fclose(g_out);
    return 0;
}
