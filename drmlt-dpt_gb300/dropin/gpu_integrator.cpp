// GPU drop-in for the reference renderer's Markov-chain integrators (see
// gpu_integrator.h). Compiled against the reference's headers and linked with
// the reference's scene code and libdrmlt.so.
#include "gpu_integrator.h"

#include <cmath>
#include <cstring>
#include <iostream>
#include <map>
#include <stdexcept>

#include "animatedtransform.h"
#include "arealight.h"
#include "camera.h"
#include "envlight.h"
#include "image.h"
#include "lambertian.h"
#include "phong.h"
#include "pointlight.h"
#include "roughdielectric.h"
#include "scene.h"
#include "shape.h"
#include "texture.h"
#include "trianglemesh.h"

namespace drmlt_dropin {

void Check(int rc, const char *what) {
    if (rc != DRMLT_OK)
        throw std::runtime_error(std::string(what) + ": libdrmlt error " + std::to_string(rc) + ": " +
                                 drmlt_last_error());
}

namespace {

void put3(float *dst, const Vector3 &v) {
    dst[0] = float(v[0]);
    dst[1] = float(v[1]);
    dst[2] = float(v[2]);
}

// Row-major copy of a 4x4 matrix.
void put16(float *dst, const Matrix4x4 &m) {
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) dst[4 * r + c] = float(m(r, c));
}

drmlt_bsdf bsdf_record(const BSDF *b) {
    drmlt_bsdf r;
    std::memset(&r, 0, sizeof(r));
    if (auto *l = dynamic_cast<const Lambertian *>(b)) {
        r.type = DRMLT_BSDF_LAMBERTIAN;
        r.two_sided = l->twoSided ? 1 : 0;
        put3(r.kd, l->Kd->Avg());
    } else if (auto *p = dynamic_cast<const Phong *>(b)) {
        r.type = DRMLT_BSDF_PHONG;
        r.two_sided = p->twoSided ? 1 : 0;
        put3(r.kd, p->Kd->Avg());
        put3(r.ks, p->Ks->Avg());
        r.exponent = float(p->exponent->Avg()[0]);
    } else if (auto *d = dynamic_cast<const RoughDielectric *>(b)) {
        // the reference keeps only the ratio eta = intIOR / extIOR
        r.type = DRMLT_BSDF_ROUGHDIELECTRIC;
        r.int_ior = float(d->eta);
        r.ext_ior = 1.0f;
        r.alpha = float(d->alpha->Avg()[0]);
        put3(r.ks, d->Ks->Avg());
        put3(r.kt, d->Kt->Avg());
    } else {
        throw std::runtime_error("GPU integrator: unsupported BSDF");
    }
    return r;
}

}  // namespace

void BuildSceneDesc(const Scene *scene, SceneDesc &out) {
    out = SceneDesc();
    std::map<const Shape *, int> shapeIndex;
    int total = 0;
    for (size_t k = 0; k < scene->objects.size(); k++) {
        const Shape *shape = scene->objects[k].get();
        const auto *mesh = dynamic_cast<const TriangleMesh *>(shape);
        if (!mesh) throw std::runtime_error("GPU integrator: only triangle meshes are supported");
        if (mesh->IsMoving()) throw std::runtime_error("GPU integrator: animated shapes are not supported");
        shapeIndex[shape] = int(k);
        const TriMeshData &data = *mesh->data;
        out.firstTri.push_back(total);
        out.numTris.push_back(int32_t(data.indices.size()));
        for (const TriIndex &t : data.indices) {
            for (int v = 0; v < 3; v++) {
                float p[3], n[3];
                put3(p, data.position0[t.index[v]]);
                put3(n, data.normal0[t.index[v]]);
                out.positions.insert(out.positions.end(), p, p + 3);
                out.normals.insert(out.normals.end(), n, n + 3);
            }
        }
        total += int(data.indices.size());
        out.shapeBsdf.push_back(int32_t(out.bsdfs.size()));
        out.bsdfs.push_back(bsdf_record(shape->bsdf.get()));
        out.shapeLight.push_back(-1);
    }
    int envCount = 0;
    for (size_t k = 0; k < scene->lights.size(); k++) {
        const Light *light = scene->lights[k].get();
        drmlt_light L;
        std::memset(&L, 0, sizeof(L));
        L.shape = -1;
        L.sampling_weight = float(light->samplingWeight);
        if (auto *a = dynamic_cast<const AreaLight *>(light)) {
            L.type = DRMLT_LIGHT_AREA;
            const auto it = shapeIndex.find(a->shape);
            if (it == shapeIndex.end()) throw std::runtime_error("GPU integrator: area light on an unknown shape");
            L.shape = it->second;
            out.shapeLight[size_t(it->second)] = int32_t(k);
            put3(L.emission, a->emission);
        } else if (auto *p = dynamic_cast<const PointLight *>(light)) {
            L.type = DRMLT_LIGHT_POINT;
            put3(L.pos, p->lightPos);
            put3(L.emission, p->emission);
        } else if (auto *e = dynamic_cast<const EnvLight *>(light)) {
            if (++envCount > 1) throw std::runtime_error("GPU integrator: at most one environment light");
            if (e->toWorld.isMoving == FTRUE)
                throw std::runtime_error("GPU integrator: animated environment lights are not supported");
            L.type = DRMLT_LIGHT_ENV;
            const Image3 &img = *e->image;
            L.env_width = img.pixelWidth;
            L.env_height = img.pixelHeight;
            out.envRgb.resize(size_t(img.pixelWidth) * img.pixelHeight * 3);
            for (size_t i = 0; i < img.data.size(); i++) put3(&out.envRgb[3 * i], img.data[i]);
            put16(L.to_world, Interpolate(e->toWorld, Float(0.0)));
        } else {
            throw std::runtime_error("GPU integrator: unsupported light");
        }
        out.lights.push_back(L);
    }
    for (drmlt_light &L : out.lights)
        if (L.type == DRMLT_LIGHT_ENV) L.env_rgb = out.envRgb.data();

    drmlt_scene_desc &d = out.desc;
    d.num_tris = total;
    d.positions = out.positions.data();
    d.normals = out.normals.data();
    d.num_shapes = int32_t(out.firstTri.size());
    d.shape_first_tri = out.firstTri.data();
    d.shape_num_tris = out.numTris.data();
    d.shape_bsdf = out.shapeBsdf.data();
    d.shape_light = out.shapeLight.data();
    d.num_bsdfs = int32_t(out.bsdfs.size());
    d.bsdfs = out.bsdfs.data();
    d.num_lights = int32_t(out.lights.size());
    d.lights = out.lights.data();
    const Camera &cam = *scene->camera;
    put16(d.sample_to_cam, cam.sampleToCam);
    put16(d.cam_to_sample, cam.camToSample);
    put16(d.cam_to_world, Interpolate(cam.camToWorld, Float(0.0)));
    put16(d.world_to_cam, Interpolate(cam.worldToCamera, Float(0.0)));
    d.cam_dist = float(cam.dist);
    d.near_clip = float(cam.nearClip);
    d.far_clip = float(cam.farClip);
    d.width = cam.film->pixelWidth;
    d.height = cam.film->pixelHeight;
    put3(d.bsphere_center, scene->bSphere.center);
    d.bsphere_radius = float(scene->bSphere.radius);
}

drmlt_options BuildOptions(const DptOptions &o, int maxDervDepth, uint64_t seed) {
    drmlt_options r;
    drmlt_default_options(&r);
    if (o.integrator == "drmlt") r.integrator = DRMLT_INTEGRATOR_DRMLT;
    else if (o.integrator == "h2mc") r.integrator = DRMLT_INTEGRATOR_H2MC;
    else if (o.integrator == "mcmc") r.integrator = DRMLT_INTEGRATOR_MCMC;
    else throw std::runtime_error("GPU integrator: unknown integrator " + o.integrator);
    // an unknown DR type is green (delayed.cpp:352-362)
    r.dr_type = o.type == "mira" ? DRMLT_DR_MIRA : DRMLT_DR_GREEN;
    r.aniso_perturb_prob = float(o.anisoPerturbProb);
    r.aniso_perturb_stddev = float(o.anisoperturbstddev);
    r.acceptance_map = o.acceptanceMap ? 1 : 0;
    r.perturb_stddev = float(o.perturbStdDev);
    r.large_step_prob = float(o.largeStepProb);
    r.roughness_threshold = float(o.roughnessThreshold);
    r.discrete_stddev = float(o.discreteStdDev);
    r.uniform_mixing_prob = float(o.uniformMixingProbability);
    r.num_chains = o.numChains;
    r.num_init_samples = o.numInitSamples;
    r.spp = o.spp;
    r.direct_spp = o.directSpp;
    r.min_depth = o.minDepth;
    r.max_depth = o.maxDepth;
    r.seed_offset = o.seedOffset;
    r.use_light_coordinate_sampling = o.useLightCoordinateSampling ? 1 : 0;
    r.lens_perturb_prob = float(o.lensPerturbProb);
    r.lens_perturb_stddev = float(o.lensPerturbStdDev);
    r.max_derivative_depth = maxDervDepth;
    r.seed = seed + uint64_t(int64_t(o.seedOffset));
    return r;
}

GpuDRIntegrator::GpuDRIntegrator(const Scene *scene, int maxDervDepth, int device) : Integrator(scene, nullptr) {
    BuildSceneDesc(scene, desc_);
    opt_ = BuildOptions(*scene->options, maxDervDepth, 0x1234ABCDull);
    opt_.device = device;
}

GpuDRIntegrator::~GpuDRIntegrator() {
    if (handle_) drmlt_destroy(handle_);
}

void *GpuDRIntegrator::handle() {
    if (!handle_) Check(drmlt_create(&desc_.desc, &opt_, &handle_), "drmlt_create");
    return handle_;
}

Float GpuDRIntegrator::PrePass(const MLTState &, const int64_t numInitSamples, const int numChains, MarkovStates &,
                               std::shared_ptr<PiecewiseConstant1D> &) {
    if (numInitSamples != opt_.num_init_samples || numChains != opt_.num_chains)
        throw std::runtime_error("GPU integrator: PrePass sizes differ from the scene's options");
    float b = 0.0f;
    Check(drmlt_prepass(handle(), &b), "drmlt_prepass");
    return Float(b);
}

void GpuDRIntegrator::Render() {
    void *h = handle();
    Check(drmlt_render(h), "drmlt_render");
    const int W = desc_.desc.width, H = desc_.desc.height;
    std::vector<float> rgb(size_t(W) * H * 3);
    Check(drmlt_get_film(h, rgb.data()), "drmlt_get_film");
    std::shared_ptr<Image3> film = GetFilm(scene->camera.get());
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            const float *p = &rgb[3 * (size_t(y) * W + x)];
            film->At(x, y) = Vector3(Float(p[0]), Float(p[1]), Float(p[2]));
        }
    if (verbose) {
        drmlt_stats st;
        Check(drmlt_get_stats(h, &st), "drmlt_get_stats");
        std::cout << "GPU integrator: " << st.mutations << " mutations" << std::endl;
    }
}

}  // namespace drmlt_dropin
