/*
 * pg3gpu.h -- C ABI of the GB300 (sm_103a) path-tracing hot path.
 *
 * This library replaces the reference renderer's path-tracing core behind its
 * renderer interface:
 *
 *   reference                                          here
 *   ---------------------------------------------------------------------------
 *   AbstractRenderer(const Config&) ctor               pg3gpu_create
 *     (src/renderer.hxx:236-240)
 *   PathTracerBase::RunIteration(Algorithm, uint32_t)  pg3gpu_run_iteration
 *     (src/path_tracer_base.hxx:57-90,
 *      src/path_tracer.hxx:16-41)
 *   AbstractRenderer::GetFramebuffer(Framebuffer&)     pg3gpu_read_framebuffer
 *     (src/renderer.hxx:255-262)
 *   AbstractRenderer::WasUsed()                        pg3gpu_iterations(ctx) > 0
 *     (src/renderer.hxx:269)
 *   GetRendererIntrospectionData()                     pg3gpu_get_stats
 *     (src/renderer.hxx:263-266, path stats :11-228)
 *   PG3_FATAL_ERROR on bad input                       nonzero status + pg3gpu_last_error
 *     (src/debugging.hxx:44-66, src/pg3render.cxx:46-48)
 *
 * Conventions: every call returns an int status (PG3GPU_OK == 0); no call
 * keeps a pointer to caller memory after it returns (scene data are copied to
 * the device in pg3gpu_create); no torch or CUDA types appear in signatures
 * (streams are passed as void*). A context belongs to one thread at a time,
 * like the reference's renderers (src/pg3render.cxx:84-128).
 */
#ifndef PG3GPU_H
#define PG3GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
    PG3GPU_OK = 0,
    PG3GPU_ERR_INVALID_ARGUMENT = 1, /* bad scene / option / pointer */
    PG3GPU_ERR_UNSUPPORTED = 2,      /* valid for the reference, not implemented here */
    PG3GPU_ERR_CUDA = 3,             /* a CUDA runtime call failed */
    PG3GPU_ERR_OUT_OF_MEMORY = 4,
    PG3GPU_ERR_DEVICE_LIMIT = 5      /* a kernel hit a bounded loop / stack limit; see last_error */
};

/* ---- enumerations (values follow the reference where it has them) ----- */
/* Algorithm ids of src/config.hxx:23-34. 7 runs on the wavefront pipeline (by default), the
 * others on the megakernel; 0-5 shade the first hit only (src/eye_light.hxx,
 * src/normal_visualiser.hxx, src/direct_illumination.hxx). */
enum {
    PG3GPU_ALG_EYE_LIGHT = 0,
    PG3GPU_ALG_NORMAL_VISUALISER = 1,
    PG3GPU_ALG_DIRECT_BSDF_SAMPLING = 2,
    PG3GPU_ALG_DIRECT_LIGHT_SAMPLING_ALL = 3,
    PG3GPU_ALG_DIRECT_LIGHT_SAMPLING_SINGLE = 4,
    PG3GPU_ALG_DIRECT_MIS = 5,
    PG3GPU_ALG_PATH_TRACING_NAIVE = 6,
    PG3GPU_ALG_PATH_TRACING = 7
};

/* Material kinds: LambertMaterial, MicrofacetGGXConductorMaterial, MicrofacetGGXDielectricMaterial,
   PhongMaterial, SmoothConductorMaterial, SmoothDielectricMaterial, SraLayeredMaterial
   (src/materials.hxx:250-1566). The SRA layered material is rendered by the one-hit algorithms
   only: the reference's path tracers stop with a fatal error on it (its IsReflectanceZero and
   GetRRContinuationProb are not implemented, :1544-1557), and so they are refused here. */
enum {
    PG3GPU_MAT_LAMBERT = 0,
    PG3GPU_MAT_GGX_CONDUCTOR = 1,
    PG3GPU_MAT_GGX_DIELECTRIC = 2,
    PG3GPU_MAT_PHONG = 3,
    PG3GPU_MAT_SMOOTH_CONDUCTOR = 4,
    PG3GPU_MAT_SMOOTH_DIELECTRIC = 5,
    PG3GPU_MAT_SRA_LAYERED = 6
};
enum { PG3GPU_BG_NONE = 0, PG3GPU_BG_CONSTANT = 1, PG3GPU_BG_ENVMAP = 2 };
/* Environment-map light samplers (compile-time choice in src/hard_config.hxx:17-18, run-time here). */
enum { PG3GPU_EM_CDF = 0, PG3GPU_EM_COSINE = 1, PG3GPU_EM_STEERABLE = 2 };
/* Ray queries: AUTO takes the primitive list up to 32 primitives and the binary LBVH above; LIST
 * tests every primitive in order (the reference's GeometryList, src/scene_graph.hxx:33-82); BVH
 * the binary LBVH built on the device; BVH4 the 4-wide BVH collapsed from it (same hits; about 6%
 * slower than the binary tree on a 40968-triangle mesh; batches use the binary tree). */
enum { PG3GPU_TRAVERSAL_AUTO = 0, PG3GPU_TRAVERSAL_LIST = 1, PG3GPU_TRAVERSAL_BVH = 2, PG3GPU_TRAVERSAL_BVH4 = 3 };
/* Pipelines of the path tracers: AUTO (= WAVEFRONT) runs one kernel per stage and bounce over
 * queues of rays, the throughput choice for calls of many samples; MEGAKERNEL traces whole paths
 * per thread in one launch, faster for calls of one sample per pixel (the reference's
 * per-iteration pattern: about 9% at 512x512) and leaving the path-length histogram empty. The
 * splitting and clipping options always run as a megakernel. */
enum { PG3GPU_PIPELINE_AUTO = 0, PG3GPU_PIPELINE_MEGAKERNEL = 1, PG3GPU_PIPELINE_WAVEFRONT = 2 };

/* ---- scene description (copied at create time) ------------------------- */
typedef struct pg3gpu_camera {       /* Camera::Setup arguments, src/camera.hxx:13-59 */
    float position[3];
    float forward[3];
    float up[3];
    uint32_t width, height;
    float hfov_deg;
} pg3gpu_camera;

typedef struct pg3gpu_material {
    int32_t kind;                    /* PG3GPU_MAT_* */
    float albedo[3];                 /* Lambert reflectance (src/materials.hxx:262-266); Phong diffuse
                                        reflectance as the material holds it, i.e. already halved when
                                        the glossy lobe is on (src/materials.hxx:366-381) */
    float alpha;                     /* GGX roughness, clamped to [0.001, 1] (src/materials.hxx:805) */
    float ior;                       /* inner IOR n (GGX and smooth conductor / dielectric) */
    float ior_outer;                 /* outer IOR */
    float absorb;                    /* conductor absorbance k */
    float glossy[3];                 /* Phong glossy reflectance (mPhongReflectance) */
    float phong_exponent;            /* Phong lobe exponent (mPhongExponent), >= 0 */
    /* PG3GPU_MAT_SRA_LAYERED: the outer layer is a GGX dielectric (alpha, ior, ior_outer), the
       inner layer a Lambert (albedo) or a GGX conductor (inner_alpha, inner_ior, inner_ior_outer,
       absorb), with a medium of attenuation coefficients medium_attenuation and thickness
       medium_thickness between them (SraLayeredMaterial, src/materials.hxx:1304-1324) */
    int32_t inner_kind;              /* PG3GPU_MAT_LAMBERT or PG3GPU_MAT_GGX_CONDUCTOR */
    float inner_alpha, inner_ior, inner_ior_outer;
    float medium_attenuation[3];
    float medium_thickness;
} pg3gpu_material;

typedef struct pg3gpu_triangle {     /* Triangle(p0, p1, p2, matId), src/scene_graph.hxx:88-101 */
    float p[9];
    int32_t material;
} pg3gpu_triangle;

typedef struct pg3gpu_sphere {       /* Sphere(center, radius, matId), src/scene_graph.hxx:162-173 */
    float center[3];
    float radius;
    int32_t material;
} pg3gpu_sphere;

typedef struct pg3gpu_area_light {   /* AreaLight over one scene triangle, src/lights.hxx:55-112 */
    uint32_t triangle;               /* index into triangles; its material becomes the emitter */
    float radiance[3];
} pg3gpu_area_light;

typedef struct pg3gpu_point_light {  /* PointLight, src/lights.hxx:232-343 */
    float position[3];
    float power[3];                  /* PointLight::SetPower: intensity = power / (4 pi) */
} pg3gpu_point_light;

typedef struct pg3gpu_scene {
    pg3gpu_camera camera;
    const pg3gpu_material *materials;
    uint32_t num_materials;
    const pg3gpu_triangle *triangles;
    uint32_t num_triangles;
    const pg3gpu_sphere *spheres;
    uint32_t num_spheres;
    const pg3gpu_area_light *area_lights;
    uint32_t num_area_lights;
    int32_t background;              /* PG3GPU_BG_* ; the background is the last light id */
    float background_radiance[3];    /* PG3GPU_BG_CONSTANT */
    const float *env_map;            /* PG3GPU_BG_ENVMAP: host RGB float32, env_height rows of
                                        env_width pixels, row 0 at theta = 0 (src/em_image.hxx:51-93) */
    uint32_t env_width, env_height;
    const pg3gpu_point_light *point_lights;   /* light ids after the area lights, before the background */
    uint32_t num_point_lights;
} pg3gpu_scene;

/* ---- options (src/config.hxx:1100-1137, src/hard_config.hxx:7-27) ------- */
typedef struct pg3gpu_options {
    int32_t algorithm;               /* PG3GPU_ALG_* (mAlgorithm) */
    uint32_t min_path_length;        /* mMinPathLength (>= 1) */
    uint32_t max_path_length;        /* mMaxPathLength; 0 = Russian roulette ends paths */
    uint32_t rr_min_path_length;     /* extension: >0 applies Russian roulette from this path length
                                        on even when max_path_length is set; 0 = reference rule */
    float indirect_clipping;         /* mIndirectIllumClipping (0: off; the reference's default is 16) */
    uint32_t splitting_budget;       /* mSplittingBudget, 1..64 (the reference's default is 4) */
    int32_t em_sampler;              /* PG3GPU_EM_* */
    int32_t traversal;               /* PG3GPU_TRAVERSAL_* */
    int32_t pipeline;                /* PG3GPU_PIPELINE_* */
    uint32_t steer_subdiv_level;     /* steerable sampler: icosahedron subdivision level (3 -> 1280 triangles) */
    uint64_t seed;                   /* mBaseSeed: keys every random stream */
    uint32_t max_paths_in_flight;    /* 0 = automatic; upper bound on paths per launch chunk */
    int32_t ggx_sampler;             /* PG3GPU_GGX_*: visible-normal sampling of the GGX materials */
    float splitting_level;           /* mDbgSplittingLevel in [0, 1] (1: the whole budget at the first vertex) */
    float light_to_bsdf_ratio;       /* mDbgSplittingLightToBrdfSmplRatio, > 0 */
    int32_t steer_weights;           /* PG3GPU_STEER_WEIGHTS_*: vertex luminance of the steerable sampler */
    uint32_t steer_max_subdiv_level; /* steerable sampler: above steer_subdiv_level, an adaptive triangulation
                                        between the two levels (the reference's BuildParameters min / max
                                        subdivision level, src/em_steerable_sampler.hxx:26-98; its defaults are
                                        4 and 9); 0 or equal: one uniform level */
    float steer_max_approx_error;    /* adaptive triangulation: a triangle is subdivided where its linear
                                        approximation misses the map's luminance by more than the factor
                                        1 + this (the reference's default 5) */
    uint32_t reserved;
} pg3gpu_options;
/* With a splitting budget above 1, indirect clipping, or a light-to-BSDF ratio that gives more
 * than one light sample per vertex, algorithm 7 runs the reference's recursive estimator with
 * its tree of sub-paths (src/path_tracer.hxx:167-454) on the megakernel; batches and the
 * differentiable entry points reject these options. */

/* Adaptive steerable triangulations (steer_max_subdiv_level > steer_subdiv_level, at most 12 and
 * 2^22 leaves) are built on the host at pg3gpu_create from the map with the reference's refinement
 * rule (TriangulateEm, src/em_steerable_sampler.hxx:2963-3472): every triangle is subdivided down to
 * the minimum level and, between the levels, wherever the linear interpolation of its vertices'
 * luminance differs from the map's by more than the factor 1 + steer_max_approx_error at one of its
 * test samples. Leaves then sit at several levels; the sampler stays exact (its pdf is located
 * through a quadtree per icosahedron face). The triangulation is kept when pg3gpu_set_params changes
 * the map (only the weights follow the map). pg3gpu_load_steerable reads the reference's adaptive
 * files, replacing the context's triangulation by the file's. */

/* Vertex luminance of the steerable sampler's piecewise-linear approximation: the map's value in
 * the vertex direction, as the reference builds it (src/em_steerable_sampler.hxx:3084-3095), or
 * (the default of pg3gpu_default_options) the projection of the map onto the vertex's hat
 * function, which keeps the energy of features smaller than a triangle: a sun between vertices
 * is missed by point samples and then found only by BSDF sampling. Both give an exact, unbiased
 * sampler; on the 1280-triangle sky of the environment-map benchmark the projection has a 3-4x
 * lower relative MSE at equal samples. */
enum { PG3GPU_STEER_WEIGHTS_POINT = 0, PG3GPU_STEER_WEIGHTS_PROJECTED = 1 };

/* GGX visible-normal sampling: exact (Heitz 2018, default) or the reference's routine with its
 * rational fit of the slope CDF (src/microfacet.hxx:610-729), which is approximate in its tails. */
enum { PG3GPU_GGX_VNDF_EXACT = 0, PG3GPU_GGX_VNDF_REFERENCE_FIT = 1 };

/* Path statistics: counts of the reference's PathTerminationReason
 * (src/renderer.hxx:11-28) plus traced-ray totals. */
typedef struct pg3gpu_stats {
    uint64_t paths;
    uint64_t extension_rays;         /* closest-hit rays (camera + BSDF continuations) */
    uint64_t shadow_rays;
    uint64_t terminated_by_russian_roulette;
    uint64_t terminated_by_background;
    uint64_t terminated_by_blocker;
    uint64_t terminated_by_max_limit;
    uint64_t terminated_by_safety_limit;
    double last_iteration_ms;        /* device time of the last pg3gpu_run_iteration */
    double path_kernel_ms;           /* summed device time of path-kernel launches since reset
                                        (CUDA events on the context's stream) */
    uint64_t path_kernel_launches;   /* path-kernel launches since reset */
    uint64_t kernel_launches;        /* all kernel launches of this library since reset */
    /* Lengths of the paths that ended (all reasons but the safety limit), as the reference's
     * RendererIntrospectionData collects them (src/renderer.hxx:80-118): bin b counts lengths
     * 2^b - 1 .. 2^(b+1) - 2, i.e. floor(log2(length + 1)) = b; a path that leaves to the
     * background counts the length of its last vertex. Filled by the wavefront pipeline (algorithm
     * 7, the default); the megakernel pipelines and batches leave them 0. */
    uint64_t length_histogram[16];
    uint32_t min_path_length;        /* shortest and longest of those lengths (0 / 0: none) */
    uint32_t max_path_length;
} pg3gpu_stats;

typedef struct pg3gpu_ctx pg3gpu_ctx;

/* Fills opts with the reference's unbiased defaults for this path:
 * algorithm PT, min 1, max 0 (RR), clipping 0, splitting 1 (level 1, light-to-BSDF ratio 1),
 * CDF sampler. (The reference's command line defaults to -sb 4 -iic 16.) */
void pg3gpu_default_options(pg3gpu_options *opts);

/* Uploads the scene, builds the acceleration structure and the light-sampling
 * tables on `device`, and returns a context with a cleared framebuffer.
 * Replaces AbstractRenderer's constructor (src/renderer.hxx:236-240). */
int pg3gpu_create(const pg3gpu_scene *scene, const pg3gpu_options *opts, int device, pg3gpu_ctx **out);

/* Frees the context. Its wavefront queues and per-sample outputs come from a device memory
 * pool of the library (one per device) that keeps up to 8 GiB of freed memory for the next
 * context, so a loop of create, render, destroy reuses them instead of allocating each time;
 * that memory stays reserved on the device until the process ends (build option
 * PG3_QUEUE_POOL=0 allocates and frees per context). */
int pg3gpu_destroy(pg3gpu_ctx *ctx);

/* All work of the context is issued on this CUDA stream (cudaStream_t as void*;
 * NULL = the legacy default stream). */
int pg3gpu_set_stream(pg3gpu_ctx *ctx, void *cuda_stream);

/* Renders `spp` samples per pixel (iterations `iteration` .. iteration+spp-1 of
 * the reference's RunIteration loop) and adds them to the framebuffer.
 * Asynchronous with respect to the host; `algorithm` is PG3GPU_ALG_*.
 * Replaces PathTracerBase::RunIteration (src/path_tracer_base.hxx:57-90). */
int pg3gpu_run_iteration(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp);

/* Waits for the context's stream and reports any kernel-side limit flag. */
int pg3gpu_synchronize(pg3gpu_ctx *ctx);

/* Copies the accumulated image to host memory: mean_rgb = sum / iterations
 * (width*height*3 doubles, row 0 at the top), like GetFramebuffer
 * (src/renderer.hxx:255-262). var_rgb (may be NULL) receives the per-pixel
 * sample variance of the radiance estimates. iterations (may be NULL)
 * receives the number of accumulated samples per pixel. */
int pg3gpu_read_framebuffer(pg3gpu_ctx *ctx, double *mean_rgb, double *var_rgb, uint64_t *iterations);

/* Clears the framebuffer and the iteration counter. */
int pg3gpu_clear_framebuffer(pg3gpu_ctx *ctx);

/* Image files (Framebuffer::SaveBMP / SaveHDR, src/frame_buffer.hxx:114-200), the format by
 * the extension as src/pg3render.cxx:266-273 chooses it: ".hdr" Radiance RGBE, anything else
 * a 24-bit BMP of pow(value, 1/gamma) (the reference writes gamma 2.2). pg3gpu_write_image
 * writes a caller's mean image (width*height*3 doubles, row 0 at the top; needs no context
 * and no GPU); pg3gpu_save_image the context's current mean image. */
int pg3gpu_write_image(const double *mean_rgb, uint32_t width, uint32_t height, const char *path, float gamma);
int pg3gpu_save_image(pg3gpu_ctx *ctx, const char *path, float gamma);

/* Steerable-sampler data files in the reference's ".emssd" format 2.1
 * (EnvironmentMapSteerableSampler::SaveToDisk / LoadFromDisk, src/em_steerable_sampler.hxx:1648-2058),
 * for a context created with em_sampler PG3GPU_EM_STEERABLE.
 * pg3gpu_save_steerable writes the context's triangulation (its uniform subdivision level as
 * both the minimum and the maximum level, the reference's default debugging parameters, 6
 * children per tree node), its vertex weights and its 6-ary tree; max_approx_error is the value
 * written into the parameter block (the reference's default is 5.0; it checks the parameters of
 * a file against its own before loading it). pg3gpu_load_steerable reads a file of that format
 * whose leaf triangles are exactly those of the context's level (any vertex numbering, tree order
 * or duplicated vertices), replaces the context's vertex weights with the file's and rebuilds the
 * tree weights on the device; a file of an adaptive triangulation (leaves at several levels)
 * returns PG3GPU_ERR_UNSUPPORTED, a malformed one PG3GPU_ERR_INVALID_ARGUMENT. A later map change
 * through pg3gpu_set_params recomputes the weights from the map. */
int pg3gpu_save_steerable(pg3gpu_ctx *ctx, const char *path, float max_approx_error);
int pg3gpu_load_steerable(pg3gpu_ctx *ctx, const char *path);

/* Number of samples per pixel accumulated so far (WasUsed() == (n > 0)). */
uint64_t pg3gpu_iterations(const pg3gpu_ctx *ctx);

/* Renders samples `iteration` .. iteration+spp-1 and writes each sample's
 * radiance to host memory out_rgb[(s * height * width + pixel) * 3 + c]
 * without touching the framebuffer (path-by-path comparisons). */
int pg3gpu_render_samples(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp, float *out_rgb);

int pg3gpu_get_stats(pg3gpu_ctx *ctx, pg3gpu_stats *stats);
int pg3gpu_reset_stats(pg3gpu_ctx *ctx);

/* Device pointers to the framebuffer accumulators (width*height*3 doubles
 * each: sum and sum of squares), valid until destroy; for callers that keep
 * results on the GPU. */
int pg3gpu_device_framebuffer(pg3gpu_ctx *ctx, const double **sum_rgb, const double **sumsq_rgb);

/* Sampler probes (test entry points, no counterpart in the reference): run one
 * sampler of the path kernels n times, one sample per thread, on host arrays.
 * pg3gpu_probe_bsdf samples material `material` for outgoing local directions wol
 * (n x 3) and returns the incoming directions, the sampled pdf (pdfW * compProb),
 * the pdf the evaluation path gives for the same pair, and both attenuations
 * (src/materials.hxx SampleBsdf / EvalBsdf). pg3gpu_probe_light samples light
 * `light` (area light id, or the background's id = number of area lights) from
 * surface points/normals as next-event estimation does and returns direction,
 * sampled pdf, evaluated pdf (the emitter-hit MIS path) and radiance * cos.
 * The *_pdf variants evaluate the pdf of given directions only. */
int pg3gpu_probe_bsdf(pg3gpu_ctx *ctx, int32_t material, uint32_t n, const float *wol, uint32_t seed, float *wil,
                      float *pdf_sampled, float *pdf_eval, float *att_sampled, float *att_eval);
int pg3gpu_probe_bsdf_pdf(pg3gpu_ctx *ctx, int32_t material, uint32_t n, const float *wol, const float *wil,
                          float *pdf, float *att_max);   /* att_max (may be NULL): max channel of the BSDF value */
int pg3gpu_probe_light(pg3gpu_ctx *ctx, int32_t light, uint32_t n, const float *points, const float *normals,
                       uint32_t seed, float *dirs, float *pdf_sampled, float *pdf_eval, float *radiance_cos);
int pg3gpu_probe_light_pdf(pg3gpu_ctx *ctx, int32_t light, uint32_t n, const float *points, const float *normals,
                           const float *dirs, float *pdf);

/* LBVH export (test entry point, no counterpart in the reference, which has no
 * acceleration structure): *num_prims = triangles + spheres; for num_prims >= 2 and
 * non-NULL arrays, the sorted 30-bit Morton codes and primitive ids (num_prims each)
 * and the num_prims-1 nodes (16 floats each: left box min xyz + child id bits, left box
 * max xyz + 0, right box min xyz + child id bits, right box max xyz + 0; child ids >= 0
 * are nodes, < 0 are ~primitive). */
int pg3gpu_export_bvh(pg3gpu_ctx *ctx, uint32_t *num_prims, uint32_t *codes, uint32_t *ids, float *nodes);

/* Adaptive steerable triangulation of a map (test entry point; needs no GPU): the leaves the
 * reference's refinement rule (TriangulateEm, src/em_steerable_sampler.hxx:2963-3472) produces for
 * an RGB float map (width*height*3, row 0 at theta = 0) between min_level and max_level with the
 * maximum approximation error max_error -- the triangulation pg3gpu_create builds for
 * steer_max_subdiv_level > steer_subdiv_level. *num_leaves receives the leaf count; for non-NULL
 * arrays of that many entries, levels[i] the leaf's subdivision level and corners[9 i ..] its three
 * unit corner directions. */
int pg3gpu_steer_triangulate(const float *rgb, uint32_t width, uint32_t height, uint32_t min_level,
                             uint32_t max_level, float max_error, uint32_t *num_leaves, uint32_t *levels,
                             float *corners);

/* Allocation-free rendering. No counterpart in the reference.
 * For callers that may not allocate device memory once they are running: a plugin
 * inside a host application or engine whose device memory belongs to that host's own
 * allocator, or a real-time loop with a fixed memory budget that must not fail for lack
 * of memory half-way through a session. Renders samples
 * `iteration` .. iteration+spp-1 of the context's scene like pg3gpu_run_iteration
 * (same paths, same refusals), but adds them to the caller's device arrays sum_rgb and
 * sumsq_rgb (width*height*3 doubles each; sum and sum of squares; never cleared by
 * this call) instead of the context's framebuffer. It always runs the megakernel
 * pipeline (one kernel per path; the wavefront pipeline's queues would need device
 * memory): on the 512x512 environment-map benchmark under half the throughput of
 * pg3gpu_run_iteration (which runs algorithm 7 on the wavefront pipeline) for calls of many
 * samples per pixel, and above it for one sample per pixel per call. The
 * per-sample radiance lives in a scratch area compiled into the library:
 * PG3GPU_NOALLOC_MAX_PATHS paths (12 MiB); a GPU holds it from the first
 * pg3gpu_create on that device until the process exits, because pg3gpu_create looks up
 * the area's device address (and so loads it). The call itself then allocates nothing
 * and makes no lookup (no cudaMalloc, cudaFree, module load or allocating library
 * routine); images of more than PG3GPU_NOALLOC_MAX_PATHS pixels are rejected with
 * PG3GPU_ERR_INVALID_ARGUMENT, splitting or clipping options (frame stacks in device
 * memory) with PG3GPU_ERR_UNSUPPORTED. All calls share the one scratch area and it
 * keeps the last call's contents (nothing in it needs to start at zero): calls that
 * overlap on the GPU -- on other streams or from other host threads -- race, so the
 * caller must serialise them. Asynchronous, on the context's stream, like
 * pg3gpu_run_iteration. */
#define PG3GPU_NOALLOC_MAX_PATHS (1u << 20)
int pg3gpu_run_iteration_noalloc(pg3gpu_ctx *ctx, int32_t algorithm, uint32_t iteration, uint32_t spp,
                                 double *sum_rgb, double *sumsq_rgb);

/* ---- Differentiable rendering (no counterpart in the reference) ----------------------
 * Path-replay backpropagation (Vicini, Speierer and Jakob, SIGGRAPH 2021) on the wavefront
 * pipeline of algorithm 7. pg3gpu_diff_forward renders samples iteration..iteration+spp-1 of
 * the current parameters, writes their mean image and keeps each path's radiance (12 bytes
 * per path). pg3gpu_diff_adjoint then re-traces the same paths from their random-number keys
 * (no path vertices are stored) and ADDS dLoss/dparameters to the caller's gradient arrays,
 * given dLoss/dimage. Sampling (directions, pdfs, MIS weights, roulette) is treated as
 * constant ("detached"). Differentiable parameters, in the layouts below:
 *   materials: 4 floats per material -- Lambert: albedo rgb, w unused; GGX: xyz unused,
 *              w = roughness alpha (derivative with respect to the clamped alpha),
 *   environment map: env_height x env_width x 3 texels (rgb, the scene's layout).
 * Not for algorithm 6, the megakernel pipeline or scenes with more than 2048 materials.
 * All device pointers are stream-ordered on the context's stream: the calls allocate only on
 * their first use (or when spp grows), so after one warm-up call they can be captured into a
 * CUDA graph together with the caller's loss and optimiser. */
#define PG3GPU_PARAMS_DEVICE 1u          /* pointers are device memory (else host memory) */
#define PG3GPU_PARAMS_KEEP_SAMPLING 2u   /* keep the sampling data (roulette probabilities, GGX sampling
                                            roughness, environment-map sampler tables) of the current
                                            parameters */
/* Replaces the parameters; either pointer may be NULL. Clamps albedo to >= 0, alpha to
 * [0.001, 1] and texels to >= 0. Unless KEEP_SAMPLING, the sampling data follow the new
 * values: the environment-map CDF and the steerable sampler's weights are rebuilt on the
 * device. */
int pg3gpu_set_params(pg3gpu_ctx *ctx, const float *material_params, const float *env_texels, uint32_t flags);
/* Current parameters into host arrays (either may be NULL). */
int pg3gpu_get_params(pg3gpu_ctx *ctx, float *material_params, float *env_texels);
/* image: width x height x 3 floats (device memory), the mean of the spp samples. The
 * context's framebuffer is not touched. */
int pg3gpu_diff_forward(pg3gpu_ctx *ctx, uint32_t iteration, uint32_t spp, float *image);
/* dloss_dimage: width x height x 3 (device); grad_materials: num_materials x 4 (device, added
 * to); grad_env: env_height x env_width x 3 (device, added to; NULL skips the map). Replays the
 * paths of the last pg3gpu_diff_forward, whose parameters must still be current. */
int pg3gpu_diff_adjoint(pg3gpu_ctx *ctx, const float *dloss_dimage, float *grad_materials, float *grad_env);
/* offset: a device word (NULL: none) that pg3gpu_diff_forward and pg3gpu_diff_adjoint read when
 * they run and add to their sample indices, so a captured graph can advance it between replays
 * and render new samples each time; a forward and its adjoint must see the same value. */
int pg3gpu_set_sample_offset(pg3gpu_ctx *ctx, const uint32_t *offset);

/* ---- Batched rendering (no counterpart in the reference) ----------------------------
 * Many scene instances, each with its own scene, options (algorithm 7 on the wavefront
 * pipeline; the options' seed keys its random numbers) and samples per pixel, rendered by
 * one persistent wavefront. Paths of all instances share `capacity` slots: a finished path
 * adds its radiance to its instance's framebuffer and frees its slot, and when fewer than
 * regen_threshold * capacity paths are active the free slots are refilled with camera paths
 * of whichever instances have samples left. A run renders spp[i] samples of every instance i;
 * with use_graph the whole run is one CUDA graph launch whose device-side loop (a conditional
 * while node) ends when every path of every instance has finished. Instance i renders exactly
 * the paths (and radiance per path) that a context created from scenes[i] and opts[i] renders
 * for the same sample indices. All instances with an environment map must use the same
 * environment-map sampler. At most PG3GPU_BATCH_MAX_INSTANCES instances. */
#define PG3GPU_BATCH_MAX_INSTANCES 128u
typedef struct pg3gpu_batch pg3gpu_batch;

typedef struct pg3gpu_batch_tuning {
    uint32_t capacity;        /* path slots (0: automatic; at most 2^24) */
    uint32_t block_size;      /* threads per block of the stage kernels: 128 or 256 (0: 256) */
    uint32_t blocks_per_sm;   /* persistent blocks per SM of the stage kernels (0: automatic) */
    float regen_threshold;    /* refill when active paths < this fraction of capacity, in (0, 0.875] (0: 0.5) */
    int32_t use_graph;        /* 1: one CUDA graph launch per run, 0: host-driven steps */
    uint32_t reserved[3];
} pg3gpu_batch_tuning;

int pg3gpu_batch_create(const pg3gpu_scene *scenes, const pg3gpu_options *opts, const uint32_t *spp, uint32_t n,
                        int device, pg3gpu_batch **out);
int pg3gpu_batch_destroy(pg3gpu_batch *batch);
int pg3gpu_batch_set_stream(pg3gpu_batch *batch, void *cuda_stream);
int pg3gpu_batch_set_tuning(pg3gpu_batch *batch, const pg3gpu_batch_tuning *tuning);
int pg3gpu_batch_get_tuning(pg3gpu_batch *batch, pg3gpu_batch_tuning *tuning);
/* Renders one run (asynchronous): samples k*spp[i] .. (k+1)*spp[i]-1 of instance i on the k-th run. */
int pg3gpu_batch_run(pg3gpu_batch *batch);
/* Waits for the batch's stream; PG3GPU_ERR_DEVICE_LIMIT if a device-side limit was hit. */
int pg3gpu_batch_synchronize(pg3gpu_batch *batch);
/* Mean (and per-pixel variance of the mean's samples) of instance `instance`, as pg3gpu_read_framebuffer. */
int pg3gpu_batch_read_framebuffer(pg3gpu_batch *batch, uint32_t instance, double *mean_rgb, double *var_rgb,
                                  uint64_t *spp);
int pg3gpu_batch_clear(pg3gpu_batch *batch);
/* Instance `instance`'s mean image as a file, as pg3gpu_save_image. */
int pg3gpu_batch_save_image(pg3gpu_batch *batch, uint32_t instance, const char *path, float gamma);
/* Autotuner: times up to max_trials runs over capacities, refill thresholds and block shapes
 * (coordinate descent, graph launches), keeps the fastest tuning and writes it to *chosen
 * (may be NULL). The trial runs are cleared from the framebuffers afterwards. */
int pg3gpu_batch_autotune(pg3gpu_batch *batch, uint32_t max_trials, pg3gpu_batch_tuning *chosen);
/* Counters over all runs since creation: paths, rays, termination reasons, kernel launches;
 * last_iteration_ms is the device time of the last run (valid after a synchronize). */
int pg3gpu_batch_get_stats(pg3gpu_batch *batch, pg3gpu_stats *stats);
const char *pg3gpu_batch_last_error(const pg3gpu_batch *batch);

/* Text of the last error of this context (or of the last failed create when ctx is NULL). */
const char *pg3gpu_last_error(const pg3gpu_ctx *ctx);
const char *pg3gpu_status_string(int status);

/* Library version, e.g. "pg3gpu 0.1 sm_103a". */
const char *pg3gpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PG3GPU_H */
