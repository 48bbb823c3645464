// GPU drop-in for the reference renderer's Markov-chain integrators.
//
// GpuDRIntegrator is an Integrator (src/integrator.h:9-22) whose Render()
// runs the whole render -- direct-lighting pass, prepass, chain loop -- in
// libdrmlt.so through the C ABI of include/drmlt_capi.h, so a `dpt` build can
// construct it where src/main.cpp:104-128 constructs DRIntegrator,
// H2MCIntegrator or MCMCIntegrator. The scene is the reference's own parsed
// Scene; BuildSceneDesc maps it onto drmlt_scene_desc (triangles in world
// space with their shading normals, one BSDF record per shape, lights in the
// scene's order, the camera's matrices at time 0, the scene's bounding
// sphere). Errors of the library become std::runtime_error, which the
// reference's main() catches like every Error().
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "drmlt_capi.h"
#include "integrator.h"

namespace drmlt_dropin {

// A drmlt_scene_desc and the arrays it points to.
struct SceneDesc {
    drmlt_scene_desc desc{};
    std::vector<float> positions, normals;
    std::vector<int32_t> firstTri, numTris, shapeBsdf, shapeLight;
    std::vector<drmlt_bsdf> bsdfs;
    std::vector<drmlt_light> lights;
    std::vector<float> envRgb;  // the environment map's pixels (at most one env light)
};

// The reference's parsed scene as the GPU library's scene descriptor. Throws
// std::runtime_error for what the GPU path does not take: animated shapes or
// lights, non-triangle shapes, unknown BSDF or light kinds.
void BuildSceneDesc(const Scene *scene, SceneDesc &out);

// drmlt_options from the scene's DptOptions (src/dptoptions.h:7-38); the GPU
// controls keep the library's defaults.
drmlt_options BuildOptions(const DptOptions &o, int maxDervDepth, uint64_t seed);

class GpuDRIntegrator : public Integrator {
   public:
    GpuDRIntegrator(const Scene *scene, int maxDervDepth = 9, int device = 0);
    ~GpuDRIntegrator();
    GpuDRIntegrator(const GpuDRIntegrator &) = delete;
    GpuDRIntegrator &operator=(const GpuDRIntegrator &) = delete;

    // DRIntegrator::Render (delayed.cpp:181-686): direct pass, prepass, chain
    // loop on the GPU, then the merged image into the camera's film.
    void Render() override;
    // DRIntegrator::PrePass (delayed.cpp:14-173) on the GPU: returns b. The
    // seeded Markov states and the path-length distribution stay on the device
    // (initStates and lengthDist are left as they are).
    Float PrePass(const MLTState &mltState, const int64_t numInitSamples, const int numChains,
                  MarkovStates &initStates, std::shared_ptr<PiecewiseConstant1D> &lengthDist) override;

    // The library handle for this scene, created on first use.
    void *handle();
    const SceneDesc &scene_desc() const { return desc_; }
    const drmlt_options &options() const { return opt_; }

   private:
    SceneDesc desc_;
    drmlt_options opt_{};
    void *handle_ = nullptr;
};

// Throws std::runtime_error with the library's message when rc is an error.
void Check(int rc, const char *what);

}  // namespace drmlt_dropin
