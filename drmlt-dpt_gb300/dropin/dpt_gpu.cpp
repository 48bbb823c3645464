// A `dpt`-compatible front end for the GPU integrator: parses the scene with
// the reference's own parser (src/parsescene.cpp), renders it with
// GpuDRIntegrator for integrator=drmlt|h2mc|mcmc (src/main.cpp:104-128) and
// writes the image where the reference writes it (WriteImage,
// src/image.cpp:45-58).
//
// usage: dpt_gpu [-o name] [--max-derivatives-depth N] [--device D]
//                [--dump-desc out.json] scene.xml
// --dump-desc writes the scene descriptor and options the integrator would
// hand to libdrmlt.so as JSON and exits without touching a GPU.
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "camera.h"
#include "gpu_integrator.h"
#include "image.h"
#include "parsescene.h"
#include "scene.h"
#include "texturesystem.h"

namespace {

void arr(FILE *f, const char *name, const float *v, size_t n, bool comma = true) {
    std::fprintf(f, "\"%s\":[", name);
    for (size_t i = 0; i < n; i++) std::fprintf(f, "%s%.9g", i ? "," : "", double(v[i]));
    std::fprintf(f, "]%s", comma ? "," : "");
}
void iarr(FILE *f, const char *name, const int32_t *v, size_t n, bool comma = true) {
    std::fprintf(f, "\"%s\":[", name);
    for (size_t i = 0; i < n; i++) std::fprintf(f, "%s%d", i ? "," : "", int(v[i]));
    std::fprintf(f, "]%s", comma ? "," : "");
}

void dump(const drmlt_dropin::GpuDRIntegrator &gi, const std::string &path) {
    const drmlt_scene_desc &d = gi.scene_desc().desc;
    const drmlt_options &o = gi.options();
    FILE *f = std::fopen(path.c_str(), "w");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fprintf(f, "{\"num_tris\":%d,", d.num_tris);
    arr(f, "positions", d.positions, size_t(d.num_tris) * 9);
    arr(f, "normals", d.normals, size_t(d.num_tris) * 9);
    iarr(f, "shape_first_tri", d.shape_first_tri, size_t(d.num_shapes));
    iarr(f, "shape_num_tris", d.shape_num_tris, size_t(d.num_shapes));
    iarr(f, "shape_bsdf", d.shape_bsdf, size_t(d.num_shapes));
    iarr(f, "shape_light", d.shape_light, size_t(d.num_shapes));
    std::fprintf(f, "\"bsdfs\":[");
    for (int i = 0; i < d.num_bsdfs; i++) {
        const drmlt_bsdf &b = d.bsdfs[i];
        std::fprintf(f, "%s{\"type\":%d,\"two_sided\":%d,", i ? "," : "", b.type, b.two_sided);
        arr(f, "kd", b.kd, 3);
        arr(f, "ks", b.ks, 3);
        arr(f, "kt", b.kt, 3);
        std::fprintf(f, "\"exponent\":%.9g,\"eta\":%.9g,\"alpha\":%.9g}", double(b.exponent),
                     b.ext_ior != 0.0f ? double(b.int_ior / b.ext_ior) : 0.0, double(b.alpha));
    }
    std::fprintf(f, "],\"lights\":[");
    for (int i = 0; i < d.num_lights; i++) {
        const drmlt_light &L = d.lights[i];
        std::fprintf(f, "%s{\"type\":%d,\"shape\":%d,\"sampling_weight\":%.9g,", i ? "," : "", L.type, L.shape,
                     double(L.sampling_weight));
        arr(f, "emission", L.emission, 3);
        arr(f, "pos", L.pos, 3);
        std::fprintf(f, "\"env_width\":%d,\"env_height\":%d,", L.env_width, L.env_height);
        if (L.type == DRMLT_LIGHT_ENV) arr(f, "env_rgb", L.env_rgb, size_t(L.env_width) * L.env_height * 3);
        arr(f, "to_world", L.to_world, 16, false);
        std::fprintf(f, "}");
    }
    std::fprintf(f, "],");
    arr(f, "sample_to_cam", d.sample_to_cam, 16);
    arr(f, "cam_to_sample", d.cam_to_sample, 16);
    arr(f, "cam_to_world", d.cam_to_world, 16);
    arr(f, "world_to_cam", d.world_to_cam, 16);
    std::fprintf(f, "\"cam_dist\":%.9g,\"near_clip\":%.9g,\"far_clip\":%.9g,\"width\":%d,\"height\":%d,",
                 double(d.cam_dist), double(d.near_clip), double(d.far_clip), d.width, d.height);
    arr(f, "bsphere_center", d.bsphere_center, 3);
    std::fprintf(f, "\"bsphere_radius\":%.9g,", double(d.bsphere_radius));
    std::fprintf(f,
                 "\"options\":{\"integrator\":%d,\"dr_type\":%d,\"aniso_perturb_prob\":%.9g,"
                 "\"aniso_perturb_stddev\":%.9g,\"acceptance_map\":%d,\"perturb_stddev\":%.9g,"
                 "\"large_step_prob\":%.9g,\"roughness_threshold\":%.9g,\"discrete_stddev\":%.9g,"
                 "\"uniform_mixing_prob\":%.9g,\"num_chains\":%d,\"num_init_samples\":%d,\"spp\":%d,"
                 "\"direct_spp\":%d,\"min_depth\":%d,\"max_depth\":%d,\"seed_offset\":%d,"
                 "\"use_light_coordinate_sampling\":%d,\"max_derivative_depth\":%d,"
                 "\"lens_perturb_prob\":%.9g,\"lens_perturb_stddev\":%.9g}}\n",
                 o.integrator, o.dr_type, double(o.aniso_perturb_prob), double(o.aniso_perturb_stddev),
                 o.acceptance_map, double(o.perturb_stddev), double(o.large_step_prob),
                 double(o.roughness_threshold), double(o.discrete_stddev), double(o.uniform_mixing_prob),
                 o.num_chains, o.num_init_samples, o.spp, o.direct_spp, o.min_depth, o.max_depth, o.seed_offset,
                 o.use_light_coordinate_sampling, o.max_derivative_depth, double(o.lens_perturb_prob),
                 double(o.lens_perturb_stddev));
    std::fclose(f);
}

}  // namespace

int main(int argc, char *argv[]) {
    std::string scenePath, outputName, dumpPath;
    int maxDervDepth = 9, device = 0;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "-o" && i + 1 < argc) outputName = argv[++i];
        else if (a.rfind("--max-derivatives-depth=", 0) == 0) maxDervDepth = std::atoi(a.c_str() + 24);
        else if (a == "--max-derivatives-depth" && i + 1 < argc) maxDervDepth = std::atoi(argv[++i]);
        else if (a == "--device" && i + 1 < argc) device = std::atoi(argv[++i]);
        else if (a == "--dump-desc" && i + 1 < argc) dumpPath = argv[++i];
        else if (a == "-d" || a == "--z" || a.rfind("--p", 0) == 0) continue;  // reference flags with no GPU meaning
        else if (!a.empty() && a[0] != '-') scenePath = a;
        else {
            std::cerr << "unknown argument " << a << std::endl;
            return 2;
        }
    }
    if (scenePath.empty()) {
        std::cerr << "usage: dpt_gpu [-o name] [--max-derivatives-depth N] [--device D] [--dump-desc out.json] "
                     "scene.xml"
                  << std::endl;
        return 2;
    }
    try {
        TextureSystem::Init();
        std::unique_ptr<Scene> scene = ParseScene(scenePath);
        const std::string integrator = scene->options->integrator;
        if (integrator != "drmlt" && integrator != "h2mc" && integrator != "mcmc")
            throw std::runtime_error("dpt_gpu renders integrator=drmlt|h2mc|mcmc, not " + integrator);
        drmlt_dropin::GpuDRIntegrator gi(scene.get(), maxDervDepth, device);
        if (!dumpPath.empty()) {
            dump(gi, dumpPath);
            TextureSystem::Destroy();
            return 0;
        }
        gi.output_name = outputName;
        gi.Render();
        WriteImage(scene->outputName, GetFilm(scene->camera.get()).get());
        std::cout << "Final image written to: " << scene->outputName << std::endl;
        TextureSystem::Destroy();
    } catch (std::exception &ex) {
        std::cerr << ex.what() << std::endl;
        return 1;
    }
    return 0;
}
