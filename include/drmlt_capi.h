/*
 * drmlt_capi.h -- C ABI of the GB300 DRMLT hot path (libdrmlt.so).
 *
 * One handle owns a scene uploaded to one CUDA device, the Markov-chain state
 * of one render and its film. Handles are not thread-safe; use one per host
 * thread / stream. Every call returns 0 on success or a negative DRMLT_E*
 * code; drmlt_last_error() gives a message. All pointers are host pointers.
 *
 * Reference interfaces replaced (joeylitalien/drmlt-dpt):
 *   Integrator{Render, PrePass}            src/integrator.h:9-22
 *   DRIntegrator                           src/integrators/delayed/delayed.{h,cpp}
 *   H2MCIntegrator / MCMCIntegrator        src/integrators/h2mc.cpp, src/integrators/mcmc.cpp
 *   DptOptions (<dpt> XML block)           src/dptoptions.h:7-38, src/parsescene.cpp:505-564
 *   PathFuncDerv (chad-generated library)  src/path.h:145-160
 */
#ifndef DRMLT_CAPI_H
#define DRMLT_CAPI_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DRMLT_OK 0
#define DRMLT_E_ARG (-1)       /* invalid argument */
#define DRMLT_E_CUDA (-2)      /* CUDA error (device missing, launch failure, ...) */
#define DRMLT_E_STATE (-3)     /* call out of order (e.g. run before prepass) */
#define DRMLT_E_OVERFLOW (-4)  /* a fixed-capacity buffer overflowed */
#define DRMLT_E_IO (-5)        /* a file could not be written */
#define DRMLT_E_TIMEOUT (-6)   /* a bounded device-side wait ran out (persistent schedule); the
                                  handle's chain state is undefined afterwards: destroy it */

#define DRMLT_MAX_LEN 12           /* longest path (segments) a chain may hold */
#define DRMLT_MAX_DIM 24           /* 2 * DRMLT_MAX_LEN */

/* BSDF kinds (src/bsdf.h:7) */
#define DRMLT_BSDF_LAMBERTIAN 0
#define DRMLT_BSDF_PHONG 1
#define DRMLT_BSDF_ROUGHDIELECTRIC 2
/* light kinds (src/light.h:7) */
#define DRMLT_LIGHT_POINT 0
#define DRMLT_LIGHT_AREA 1
#define DRMLT_LIGHT_ENV 2
/* integrators (src/main.cpp:104-120) and DR frameworks (delayed.h:22-25) */
#define DRMLT_INTEGRATOR_DRMLT 0
#define DRMLT_INTEGRATOR_H2MC 1
#define DRMLT_INTEGRATOR_MCMC 2
#define DRMLT_DR_GREEN 0
#define DRMLT_DR_MIRA 1

typedef struct drmlt_bsdf {
    int32_t type;
    int32_t two_sided;
    float kd[3];         /* Lambertian reflectance / Phong diffuse */
    float ks[3];         /* Phong specular */
    float exponent;      /* Phong exponent */
    float int_ior, ext_ior, alpha;  /* rough dielectric (Beckmann): IORs and roughness */
    float kt[3];         /* rough dielectric: specular transmittance (ks: reflectance) */
} drmlt_bsdf;

typedef struct drmlt_light {
    int32_t type;
    int32_t shape;       /* area light: emitting shape index */
    float emission[3];   /* area: radiance, point: intensity */
    float pos[3];        /* point light position */
    float sampling_weight;
    /* environment light (EnvLight, src/envlight.h; at most one per scene): the
     * envmap image as env_width x env_height RGB floats, row-major from the top
     * row (the reference's Image3 layout), and toWorld as a row-major 4x4 whose
     * upper-left 3x3 rotates directions (src/envlight.cpp:73-81). */
    const float *env_rgb;
    int32_t env_width, env_height;
    float to_world[16];
} drmlt_light;

/* Triangles are listed shape by shape (shape k owns a contiguous range).
 * Matrices are row-major 4x4, exactly the reference camera's
 * sampleToCam / camToSample / camToWorld / worldToCamera (src/camera.cpp:11-28). */
typedef struct drmlt_scene_desc {
    int32_t num_tris;
    const float *positions;   /* num_tris x 3 vertices x xyz */
    const float *normals;     /* num_tris x 3 vertices x xyz (shading normals) */
    int32_t num_shapes;
    const int32_t *shape_first_tri;
    const int32_t *shape_num_tris;
    const int32_t *shape_bsdf;
    const int32_t *shape_light;  /* area light index or -1 */
    int32_t num_bsdfs;
    const drmlt_bsdf *bsdfs;
    int32_t num_lights;
    const drmlt_light *lights;
    float sample_to_cam[16], cam_to_sample[16], cam_to_world[16], world_to_cam[16];
    float cam_dist, near_clip, far_clip;
    int32_t width, height;
    float bsphere_center[3], bsphere_radius;
} drmlt_scene_desc;

/* DptOptions (src/dptoptions.h:7-38) plus GPU controls. */
typedef struct drmlt_options {
    int32_t integrator;          /* DRMLT_INTEGRATOR_* */
    int32_t dr_type;             /* DRMLT_DR_GREEN | DRMLT_DR_MIRA */
    float aniso_perturb_prob;    /* anisoperturbprob */
    float aniso_perturb_stddev;  /* second-stage isotropic sigma. The reference parses the XML
                                     anisoperturbstddev into lensPerturbStdDev instead
                                     (src/parsescene.cpp:553-554), so its sigma stays at the
                                     0.0025 default; this value is honoured as given. */
    int32_t acceptance_map;
    float perturb_stddev;
    float large_step_prob;
    float roughness_threshold;
    float discrete_stddev;
    float uniform_mixing_prob;   /* h2mc integrator */
    int32_t num_chains;
    int32_t num_init_samples;
    int32_t spp;
    int32_t direct_spp;
    int32_t min_depth;
    int32_t max_depth;
    int32_t seed_offset;
    int32_t use_light_coordinate_sampling;
    int32_t max_derivative_depth; /* --max-derivatives-depth (default 9) */
    uint64_t seed;                /* GPU random-stream key */
    int32_t device;               /* CUDA device ordinal */
    int32_t use_graph;            /* replay iterations as CUDA graphs of 1 (or, autotuned, 4)
                                     iterations (default 1) */
    int32_t chain_groups;         /* chains are split into this many groups, each stepped on its own
                                     CUDA stream so the groups' kernels overlap (0 = default, 2) */
    int32_t stage_lanes;          /* chains per warp in the per-chain stage kernels, 1..32 (0 = 16) */
    int32_t deriv_warps;          /* warps sharing one chain's Hessian entries, 1..4 (0 = 2) */
    int32_t smem_carveout;        /* shared-memory carveout (percent) for every chain-loop kernel,
                                     -1 = the driver's choice per kernel */
    int32_t autotune;             /* drmlt_render picks stage_lanes / deriv_warps with drmlt_autotune
                                     (default 1; renders of fewer than 1024 iterations are not tuned) */
    int32_t stage2_lanes;         /* chains per warp in the second-stage list kernels (stage 2 and
                                     Green's y*), 1..32 (0 = min(stage_lanes, 4)) */
    int32_t graph_iters;          /* iterations per CUDA graph launch, 1..8 (0 = 1; drmlt_autotune may
                                     switch between 1 and 4). Iterations short of a whole graph at
                                     the end of a run are launched without the graph. */
    int32_t wavefront;            /* path tracing of stage 1, stage 2 and Green's y*: 1 = wavefront
                                     rounds (rays of all chains queued per bounce and traced by a
                                     separate full-warp traversal kernel), 0 = one chain per lane
                                     traces its whole path; -1 = default (0). Both take identical
                                     steps. */
    int32_t head_chains;          /* stage 1 of the staged schedule: the first head_chains chains of
                                     each group's work-class order (the longest traces) run
                                     head_lanes to a warp, the others stage_lanes (0 = off) */
    int32_t head_lanes;           /* chains per warp of those head chains, 1..32 (0 = 2) */
    int32_t persistent;           /* chain-loop schedule of drmlt_run for integrator=drmlt: 1 = one
                                     persistent cooperative kernel per run, in which every chain moves
                                     through its iterations on its own (work queues between path
                                     tracing and the H2MC derivative / Gaussian workers, no barrier
                                     between stages or iterations); 0 = staged (one kernel per stage
                                     and chain group). Both take identical steps. Default 0. The h2mc
                                     and mcmc integrators are always staged. */
    int32_t team_sms;             /* persistent schedule: SMs that run the derivative / Gaussian
                                     workers; the others run path tracing (0 = a quarter of the SMs) */
    int32_t wait_limit;           /* persistent schedule: idle polls (about 0.2-0.5 us each) a device
                                     worker makes without seeing any progress before it gives up and
                                     the run fails with DRMLT_E_TIMEOUT (0 = 4194304, seconds) */
    int32_t adjoint_min_dim;      /* H2MC path derivatives: paths of this primary-sample dimension and
                                     up take the reverse-mode adjoint (one forward and one backward
                                     sweep per Hessian row, D sweeps), shorter ones hyper-dual forward
                                     mode (D(D+1)/2 evaluations); 0 = default (hyper-dual for every
                                     path, as -1), 1 = the adjoint for every path. The two agree to
                                     FP32 rounding; drmlt_autotune does not change this setting (a
                                     switch of method mid-render would change later accept
                                     decisions). The persistent schedule takes hyper-dual
                                     derivatives for every path. */
    float lens_perturb_prob;      /* lensperturbprob: integrator=h2mc's lens mutation (default 0.3) */
    float lens_perturb_stddev;    /* lensperturbstddev: its isotropic sigma (default 0.01). The
                                     reference's parser also writes the XML anisoperturbstddev
                                     here (src/parsescene.cpp:553-554); a front end that mirrors
                                     it passes that value. */
} drmlt_options;

/* DR statistics counters (delayed.cpp:287-329, raw, unswapped labels), plus
 * two counters of this implementation: anisotropic Gaussians computed, and how
 * many of them needed the FP64 Jacobi fallback (eigenvalue clusters the
 * FP32-then-refined eigensolver could not certify); for integrator=h2mc the
 * lens mutations and their acceptances (h2mc.cpp:139-149, lensStep). */
typedef struct drmlt_stats {
    uint64_t large_step, large_step_accepted;
    uint64_t stage1, stage1_accepted;
    uint64_t stage2_iso, stage2_iso_accepted;
    uint64_t stage2_h2mc, stage2_h2mc_accepted;
    uint64_t mutations;
    uint64_t gaussians, gaussians_fp64_fallback;
    uint64_t lens, lens_accepted;
} drmlt_stats;

/* A technique path (one Markov state): SubpathContrib camDepth c / lightDepth l,
 * the primary sample vector u (GetPathPos order, src/path.cpp:2393-2439, 2(c+l-1)
 * entries), and per surface vertex (light-subpath vertices first, then camera
 * ones) the hit triangle (global index), bsdfDiscrete, rrWeight and
 * useAbsoluteParam bit. */
typedef struct drmlt_path {
    int32_t c, l;
    int32_t lgt_light, lgt_prim;
    int32_t dl_light, dl_prim;
    uint32_t use_abs;
    float u[DRMLT_MAX_DIM];
    int32_t tri[DRMLT_MAX_LEN];
    float disc[DRMLT_MAX_LEN];
    float rr[DRMLT_MAX_LEN];
} drmlt_path;

/* A contribution (SubpathContrib, src/path.h:12-24): screen[2], rgb[3], ls, ss, valid. */
typedef struct drmlt_contrib {
    float screen[2];
    float rgb[3];
    float ls, ss;
    int32_t valid;
} drmlt_contrib;

/* Fills *opt with the reference's DptOptions defaults. */
void drmlt_default_options(drmlt_options *opt);

const char *drmlt_last_error(void);

/* Integrator construction: uploads the scene and builds the BVH
 * (replaces Scene::Scene + DRIntegrator ctor, src/scene.cpp:10-54, delayed.cpp:7-8). */
int drmlt_create(const drmlt_scene_desc *scene, const drmlt_options *opt, void **handle);
int drmlt_destroy(void *handle);

/* PrePass (delayed.cpp:14-173): bootstrap sampling, length distribution,
 * equal-spaced chain seeding. Writes the normalisation b. */
int drmlt_prepass(void *handle, float *b_out);

/* DirectLighting pass (src/integrator.h:33-75). */
int drmlt_direct(void *handle);

/* Runs `iterations` Markov-chain iterations on every chain (each chain runs at
 * most its share spp*W*H/numChains, the reference's sample split, delayed.cpp:205-210).
 * Returns the number of mutations done in *done (may be NULL). */
int drmlt_run(void *handle, int64_t iterations, int64_t *done);

/* Pipelined stepping for a host that reads every step's statistics without
 * idling the GPU between steps: drmlt_run_async enqueues `iterations`
 * iterations as drmlt_run does (not timed: drmlt_last_run_ms is not updated)
 * and then a copy of the statistics counters into pinned slot `slot` (0 or
 * 1), and returns without waiting; drmlt_wait_stats waits for the copy in
 * `slot` and returns those statistics. A host keeps one step in flight:
 * drmlt_run_async(step k, slot k % 2), then drmlt_wait_stats of step k - 1.
 * Not for the persistent schedule (DRMLT_E_STATE). */
int drmlt_run_async(void *handle, int64_t iterations, int slot, int64_t *done);
int drmlt_wait_stats(void *handle, int slot, drmlt_stats *st);

/* Integrator::Render (delayed.cpp:181-686): prepass + direct + all iterations. */
int drmlt_render(void *handle);

/* Final film (direct/directSpp + indirect/spp, delayed.cpp:681-685), W*H*3 floats. */
int drmlt_get_film(void *handle, float *rgb);
/* The film of the reference's intermediate images (delayed.cpp:612-637:
 * BufferToFilm of the indirect buffer alone, scaled by numPixels / mutations
 * done so far), W*H*3 floats; zeros before the first mutation. */
int drmlt_get_partial_film(void *handle, float *rgb);
/* WriteImage (src/image.cpp:45-58): a width x height RGB float image, rows top
 * to bottom, to an OpenEXR file (scanline, HALF channels, no compression;
 * floats rounded to nearest even half). Host only: needs no device.
 * DRMLT_E_IO when the file cannot be written. */
int drmlt_write_exr(const char *filename, int width, int height, const float *rgb);
int drmlt_get_stats(void *handle, drmlt_stats *stats);
/* Device time of the last drmlt_run in milliseconds (CUDA events). */
int drmlt_last_run_ms(void *handle, float *ms);
/* Kernels launched by drmlt_run on this handle so far (all chain groups). */
int drmlt_kernel_launches(void *handle, int64_t *n);

/* Launch-shape autotuner (after drmlt_prepass) of the staged schedule: after
 * one untimed run of `iterations_per_candidate` iterations, times that many
 * iterations of the render under each candidate chains-per-warp count of the
 * per-chain kernels (2, 4, 8, 16, 32), then each derivative team size (1, 2, 4
 * warps), then the stage-1 head tier (head_chains 0, or half of a chain
 * group at half the chains per warp with the other half at the tuned count or
 * twice it), every choice in two passes of
 * opposite order (CUDA events), and keeps the fastest (chains per warp and
 * team size written to the outputs, which may be NULL; the head tier is
 * reported by drmlt_get_head_tier): 23 runs. With CUDA graphs on and
 * iterations_per_candidate a multiple of 4 it then times graphs of 1 and of 4
 * iterations (4 more runs) and keeps the faster. The wavefront and persistent
 * schedules are not candidates (both measured slower on every benchmark scene;
 * they stay selectable through drmlt_options). The iterations count toward the
 * render; the launch shape does not change the chains' steps. */
int drmlt_autotune(void *handle, int iterations_per_candidate, int *stage_lanes, int *deriv_warps);

/* The launch shape the next drmlt_run uses (after drmlt_autotune: the tuned
 * one): chains per warp of the stage kernels and of the second-stage list
 * kernels, warps per derivative team, iterations per CUDA graph launch (0 when
 * graphs are off). Any output may be NULL. drmlt_get_wavefront gives the path
 * tracing schedule (1 wavefront rounds, 0 one chain per lane). */
int drmlt_get_launch_shape(void *handle, int *stage_lanes, int *stage2_lanes, int *deriv_warps, int *graph_iters);
int drmlt_get_wavefront(void *handle, int *wavefront);
/* The stage-1 head tier the next drmlt_run uses: head_chains (0 = none) and
 * head_lanes (drmlt_options.head_chains / head_lanes, or the autotuner's
 * choice). Either output may be NULL. */
int drmlt_get_head_tier(void *handle, int *head_chains, int *head_lanes);
/* The derivative method the next drmlt_run uses: paths of this primary-sample
 * dimension and up take the reverse-mode adjoint (-1: none, hyper-dual for
 * every path). */
int drmlt_get_adjoint_min_dim(void *handle, int *adjoint_min_dim);

/* drmlt_run with CUDA events around each stage kernel (same work, serialised
 * per stage): stage_ms[7] accumulates stage1, derivs(x), gauss(x), stage2,
 * derivs(z), gauss(z), finish milliseconds. */
int drmlt_profile(void *handle, int64_t iterations, float *stage_ms, int64_t *done);

/* Iterations a full render runs (spp*W*H/numChains, plus one for the chains
 * that get an extra sample). */
int drmlt_total_iterations(void *handle, int64_t *iterations);

/* ---- per-path entry points (parity harness; n paths per call) ---- */

/* Forward: log Luminance(contribution) of each technique path at primary vector
 * u (2(c+l-1) floats per path, DRMLT_MAX_DIM stride), as the chad-generated
 * evaluate_path_bidir_<c>_<l>_static computes it (src/path.cpp:2987-3175). */
int drmlt_path_eval(void *handle, const drmlt_path *paths, const float *u, int n, float *logf);

/* Backward pair of drmlt_path_eval: gradient (DRMLT_MAX_DIM stride) and Hessian
 * (DRMLT_MAX_DIM^2 stride per path; within it the dim x dim matrix row-major,
 * dim = 2(c+l-1)) of log f, the PathFuncDerv call of drsmallstep.cpp:128-158. */
int drmlt_path_grad_hess(void *handle, const drmlt_path *paths, const float *u, int n, float *grad,
                         float *hess);

/* The same backward pair by the reverse-mode adjoint: per path, D forward and
 * backward sweeps (forward-over-reverse, one Hessian row each) that keep each
 * vertex's carried state and recompute its operations instead of recording a
 * tape -- the reverse pass and forward-over-reverse Hessian that chad builds
 * over its recorded expression graph (src/chad.cpp:342-418, 492-552). Same
 * layout as drmlt_path_grad_hess; the Hessian is symmetric by construction
 * (entry (i, j), i < j, from row i). */
int drmlt_path_adjoint(void *handle, const drmlt_path *paths, const float *u, int n, float *grad, float *hess);

/* PerturbPathBidir (src/path.cpp:1480-1628) with discrete jitter off:
 * offsets (DRMLT_MAX_DIM stride) -> perturbed paths and contributions. */
int drmlt_perturb(void *handle, const drmlt_path *in, const float *offset, int n, drmlt_path *out,
                  drmlt_contrib *contrib);

/* integrator=h2mc's lens mutation, per path (H2MCSmallStep::Mutate's lens
 * branch, src/integrators/h2mc.cpp:466-532).
 * drmlt_lens_eval: for technique paths with their contributions' screen
 * positions (screen, 2 per path) and ss scores, the lens score
 * (SubpathContrib::lensScore, as the sampler that made the path computes it),
 * the lens vertex position (Path::lensVertexPos, 3 per path), and the lens-mode
 * path function (RegisterPathFuncBidir with PathFuncMode::Lens,
 * src/path.cpp:2987-3175): log f (logf), its gradient (grad, 2) and Hessian
 * (hess, 2 x 2 row-major) w.r.t. the screen position -- zeros where the lens
 * score is <= 1e-15 or the reference has no lens function for the technique
 * (c + l <= 3 or c + l - 1 > max_derivative_depth), logf 0 there -- and the
 * 2-D Gaussian ComputeGaussian (h2mc.cpp:607-640) builds from them with
 * sigma lens_sigma: gauss = mean[2], inv_cov[4], log_det (7 doubles per path).
 * It replaces the lens-function lookup of the chad library
 * (lensFuncMap / lensDervFuncMap, src/path.h:158-159). */
int drmlt_lens_eval(void *handle, const drmlt_path *paths, const float *screen, const float *ss, int n,
                    float lens_sigma, int max_derivative_depth, float *lens_score, float *lens_pos, float *logf,
                    float *grad, float *hess, double *gauss);

/* PerturbLensBidir (src/path.cpp:1913-2078): each path moved to screen
 * position screen_new (2 per path) with its first camera vertex aimed at
 * lens_pos (3 per path) -> the perturbed path, its contribution and its lens
 * score. The output paths carry bit 31 of use_abs (made by the lens
 * mutation: a later lens score of the path takes that sampler's form). */
int drmlt_lens_perturb(void *handle, const drmlt_path *in, const float *screen_new, const float *lens_pos, int n,
                       drmlt_path *out, drmlt_contrib *contrib, float *lens_score);

/* Replays recorded uniform streams through GeneratePathBidir (mode 0,
 * src/path.cpp:978-1121), GenerateSubpath (mode 1, camLength/lgtLength per
 * stream in cam_len/lgt_len, src/path.cpp:1123-1269) or the direct-lighting
 * GeneratePath (mode 2, pixel x/y in cam_len/lgt_len, src/path.cpp:343-445 as
 * called by src/integrator.h:33-75). tapes: n x stride floats, tape_len[i] used.
 * Modes 0 and 2 write up to max_contribs contributions per stream (c, l in
 * out_tech[2*k], count in out_count); mode 1 writes one path and contribution. */
int drmlt_replay(void *handle, int mode, const float *tapes, const int32_t *tape_len, int stride, int n,
                 const int32_t *cam_len, const int32_t *lgt_len, int max_contribs, int32_t *out_count,
                 int32_t *out_tech, drmlt_contrib *out_contrib, drmlt_path *out_path, int32_t *out_consumed);

/* The acceptance quantities of one delayed-rejection iteration from a current
 * state x with the proposals' offsets given (for the parity tests; the chain
 * loop computes the same quantities with the same device code):
 *   a1          first-stage acceptance of y = PerturbPathBidir(x, offset1):
 *               Clamp(ss(y) / ss(x), 0, 1), 0 when y does not contribute or the
 *               value is invalid (SmallStep::Mutate, src/mutation.cpp:126-166;
 *               delayed.cpp:430-437)
 *   a2          second-stage ratio for z = PerturbPathBidir(x, offset2): with
 *               aniso = 0 the isotropic Clamp(ss(z) / ss(x), 0, 1)
 *               (mutation.cpp:167-208), with aniso = 1 the unclamped H2MC ratio
 *               exp(log_ratio) ss(z) / ss(x) (PH2MCSmallStep::Mutate,
 *               drsmallstep.cpp:169-196); 0 when z does not contribute
 *   log_ratio   H2MC: log N_z(-offset2) - log N_x(offset2), the Gaussians at x
 *               and z from the path derivatives (gated like the chain loop by
 *               max_derivative_depth and ss), in FP64
 *   a_star_green acceptance of Green's reverse path y* = PerturbPathBidir(z,
 *               x - y) from z (SmallStep::Trace, mutation.cpp:210-238; 0 when z
 *               does not contribute)
 *   log_q_mira  log Q1(z, y) / Q1(x, y), Mira's isotropic kernel ratio with
 *               sigma = perturb_stddev (delayed.cpp:512-523), in FP64
 *   alpha2_green, alpha2_mira  the second-stage acceptance probabilities of
 *               Green & Mira and of Tierney & Mira (delayed.cpp:466-541)
 * y and z are evaluated with the discrete jitter off. */
typedef struct drmlt_dr_result {
    float a1;
    float ss_y, ss_z;
    int32_t valid_y, valid_z;
    float a2;
    double log_ratio;
    float a_star_green;
    float alpha2_green, alpha2_mira;
    int32_t pad;
    double log_q_mira;
} drmlt_dr_result;

/* Per-stage acceptances (above) for n current states x (paths and their
 * contributions: ss and ls are used), offsets (DRMLT_MAX_DIM stride) and the
 * second stage's kind per state (aniso[i]: 0 isotropic, 1 H2MC). The
 * first-stage proposals y and second-stage proposals z are written to y_out /
 * z_out (may be NULL). */
int drmlt_dr_eval(void *handle, int n, const drmlt_path *x, const drmlt_contrib *x_contrib, const float *offset1,
                  const float *offset2, const int32_t *aniso, drmlt_dr_result *out, drmlt_path *y_out,
                  drmlt_path *z_out);

/* LargeStep::Mutate (src/mutation.cpp:7-120, multiplexed, bidirectional) on n
 * recorded uniform streams (stride floats each, tape_len[i] used): the path
 * length from the distribution of per-length weights length_func[num_lengths]
 * (PiecewiseConstant1D), the light subpath length, GenerateSubpath and the
 * contribution pick, then the acceptance against the current state x[i] (its
 * technique and ls). Writes a1, the proposal's technique (c, l; 0, 0 when it
 * does not contribute), its contribution and the uniforms consumed. */
int drmlt_large_step_eval(void *handle, int n, const float *tapes, const int32_t *tape_len, int stride,
                          const drmlt_path *x, const drmlt_contrib *x_contrib, const float *length_func,
                          int num_lengths, float *a1, int32_t *out_tech, drmlt_contrib *out_contrib,
                          int32_t *out_consumed);

/* Closest-hit (any_hit = 0) or occlusion (any_hit = 1) ray casts against the
 * scene BVH, the rtcIntersect / rtcOccluded calls of src/scene.cpp:80-111.
 * org/dir: n x 3 floats. Writes the global triangle index (-1 = miss) and hit t. */
int drmlt_trace_rays(void *handle, const float *org, const float *dir, float tmin, float tmax, int n, int any_hit,
                     int32_t *tri, float *t);

/* Ray-casting benchmark on the scene BVH (no reference counterpart): n_rays
 * device-generated rays of one kind -- 0 primary camera rays (closest hit),
 * 1 diffuse bounce rays from their first hits (closest hit), 2 shadow rays of
 * length 2 from the same hits (any hit) -- traced `repeats` times by a kernel
 * timed on its own with CUDA events. Writes the mean milliseconds per pass and
 * counts[3] = rays traced, BVH nodes fetched (64 B each) and triangles tested
 * (48 B each) in one pass. */
int drmlt_ray_benchmark(void *handle, int kind, int n_rays, int repeats, float *ms_per_pass, double *counts);

/* Arithmetic peak of the current device: a full-occupancy kernel of
 * independent FMA chains (fp64 = 0: FP32 fmaf, 1: FP64 fma), `iterations`
 * steps per chain, event-timed after a short warm-up launch. Returns the
 * kernel time in *ms and its floating-point operations in *flops (2 per FMA).
 * The compute rooflines of the derivative (FP32) and Gaussian (FP64) kernels
 * are quoted against it. */
int drmlt_fma_benchmark(void *handle, int fp64, int iterations, float *ms, double *flops);

/* ComputeGaussian (drsmallstep.cpp:219-266) in FP64: returns mean (MAX_DIM),
 * invCov and cov (MAX_DIM^2 each, row-major) and logDet per input. */
int drmlt_compute_gaussian(void *handle, const int32_t *dims, const float *ss, const float *grad,
                           const float *hess, int n, double *mean, double *inv_cov, double *cov,
                           double *log_det);

/* No counterpart in the reference. drmlt_compute_gaussian without any device
 * allocation, for callers that cannot call cudaMalloc: a host renderer that
 * hands the library buffers carved from its own pre-allocated device pool, or
 * code that must not hit cudaMalloc's implicit device-wide synchronisation
 * while other streams are running. All array arguments are DEVICE pointers the
 * caller owns (same layouts as drmlt_compute_gaussian; dims/ss/log_det have n
 * entries, grad/mean DRMLT_MAX_DIM per Gaussian, hess/inv_cov/cov
 * DRMLT_MAX_DIM^2). sigma is the H2MC prior (perturbstddev). The work is queued
 * on `stream` (a cudaStream_t, NULL = legacy default stream) and the call
 * returns without synchronising.
 *
 * Scratch lives in a fixed library-owned device array sized for 256 Gaussians
 * (about 1.3 MB, held on every device that loads the library until the process
 * exits); n > 256 is rejected with DRMLT_E_ARG. The first call on each device
 * looks the array's device address up (cudaGetSymbolAddress, once per device
 * under a lock, so first calls from several host threads are safe), so make
 * that first call before any stream capture. An odd, non-positive or too
 * large dims[i] gives zero mean / inv_cov / cov rows and a NaN log_det[i].
 * Every call shares the one array:
 * calls that overlap on the GPU (on different streams, or from different host
 * threads) race on it and must be serialised by the caller. */
int drmlt_compute_gaussian_noalloc(int n, const int32_t *dims, const float *ss, const float *grad,
                                   const float *hess, float sigma, double *mean, double *inv_cov, double *cov,
                                   double *log_det, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* DRMLT_CAPI_H */
