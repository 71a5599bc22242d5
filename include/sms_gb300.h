/*
 * sms_gb300.h -- C ABI of the GB300 (sm_103a) Specular Manifold Sampling library.
 *
 * This is the drop-in boundary for the reference's SMS solvers.  Every entry point
 * takes plain pointers and sizes; no C++ or torch types cross it, no exception
 * escapes it, and every function returns an sms_status code (0 = ok).
 *
 * Reference interfaces replaced (paths relative to the reference project):
 *   SMSConfig                                 include/mitsuba/render/manifold.h:11-45
 *   integrator XML parameters                 src/integrators/path_sms_ss.cpp:47-61,
 *                                             src/integrators/path_sms_ms.cpp:149-161,
 *                                             src/integrators/path_sms_glints.cpp:42-54
 *   SpecularManifoldSingleScatter             include/mitsuba/render/manifold_ss.h:9-159
 *     ::specular_manifold_sampling(si,sampler) src/librender/manifold_ss.cpp:28-201
 *     ::sample_path(shape,si,ei,sampler,n_offset,p_start)
 *                                             src/librender/manifold_ss.cpp:203-279
 *   SpecularManifoldMultiScatter              include/mitsuba/render/manifold_ms.h:9-166
 *     ::specular_manifold_sampling            src/librender/manifold_ms.cpp:27-201
 *     ::sample_path                           src/librender/manifold_ms.cpp:203-227
 *   SpecularManifoldGlints(+Vectorized)       include/mitsuba/render/manifold_glints.h:9-208
 *     ::specular_manifold_sampling            src/librender/manifold_glints.cpp:28-223
 *     ::sample_glint(...,xi_start)            src/librender/manifold_glints.cpp:225-265
 *   print_statistics() counters               src/librender/manifold_ss.cpp:14-18,859-883
 *   PathIntegrator / SMS path integrators     src/integrators/path.cpp:94-226,
 *     ::sample (whole images: sms_render)     src/integrators/path_sms_ss.cpp:69-251,
 *                                             src/integrators/path_sms_ms.cpp:172-330
 *
 * Where the reference calls the solver once per shading point from many host
 * threads, this library takes a whole wavefront of shading points ("queries")
 * per call and solves them on the GPU.  Query and result buffers are
 * component-major SoA: field f of query i lives at buf[f * n + i].
 */
#ifndef SMS_GB300_H
#define SMS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */
typedef enum sms_status {
    SMS_OK = 0,
    SMS_ERR_INVALID_ARG = 1,   /* null pointer, bad size, unknown id            */
    SMS_ERR_CUDA = 2,          /* a CUDA runtime call failed                     */
    SMS_ERR_DEVICE_LIMIT = 3,  /* a bounded device loop hit its limit            */
    SMS_ERR_UNSUPPORTED = 4,   /* configuration the library does not implement   */
    SMS_ERR_PARSE = 5,         /* integrator XML block could not be parsed       */
    SMS_ERR_NO_DEVICE = 6      /* no CUDA device                                  */
} sms_status;

/* Human-readable text of the last error on this host thread. */
const char *sms_last_error(void);

/* ------------------------------------------------------------------ config */
/* Same fields, names and defaults as the reference's SMSConfig
 * (include/mitsuba/render/manifold.h:11-45) plus the integrator-level switches
 * the SMS integrators read (path_sms_glints.cpp:42-54). */
typedef struct sms_config {
    int32_t biased;                 /* false */
    int32_t twostage;               /* false; two-stage solver on normal-mapped
                                       single-scatter casters (every caster must
                                       carry the map, else SMS_ERR_UNSUPPORTED;
                                       multi-scatter and glints ignore it, as
                                       the reference does) */
    int32_t halfvector_constraints; /* false */
    int32_t mnee_init;              /* false; straight-line seeds (manifold_ss.cpp:229-241) */
    float   step_scale;             /* 1     */
    int32_t max_iterations;         /* 20    */
    float   solver_threshold;       /* 1e-5  */
    float   uniqueness_threshold;   /* 1e-4  */
    int32_t max_trials;             /* -1    */
    int32_t bounces;                /* 1 (path_sms_ms default is 2) */
    int32_t bsdf_strategy_only;     /* false */
    int32_t sms_strategy_only;      /* false */
    int32_t glints_vectorized;      /* false */
} sms_config;

/* Fill *cfg with the reference defaults. */
void sms_config_default(sms_config *cfg);

/* Parse one <integrator type="path_sms_ss|path_sms_ms|path_sms_glints"> block
 * (the XML subset the reference's integrators read with props.bool_/int_/float_).
 * Unknown parameters are ignored like the reference's Properties lookups ignore
 * them; type_out (may be NULL) receives the integrator type string. */
sms_status sms_config_parse_xml(const char *xml, sms_config *cfg,
                                char *type_out, size_t type_cap);

/* ------------------------------------------------------------------- scene */
/* Shape flags: src/librender/shape.cpp:78-82 */
#define SMS_SHAPE_CAUSTIC_RECEIVER      (1u << 0)
#define SMS_SHAPE_CAUSTIC_CASTER_SINGLE (1u << 1)
#define SMS_SHAPE_CAUSTIC_CASTER_MULTI  (1u << 2)
#define SMS_SHAPE_CAUSTIC_BOUNCER       (1u << 3)
#define SMS_SHAPE_GLINTY                (1u << 4)
/* Emitter flags: src/librender/emitter.cpp:9-10 */
#define SMS_EMITTER_CAUSTIC_SINGLE      (1u << 0)
#define SMS_EMITTER_CAUSTIC_MULTI       (1u << 1)

/* BSDF kinds the SMS path distinguishes (bsdf.cpp:53-60, dielectric.cpp:328-334,
 * conductor.cpp:288-295).  Only the fields the solver reads are kept. */
typedef enum sms_bsdf_type {
    SMS_BSDF_DIFFUSE = 0,     /* ior() = (0, 1): treated as eta = 1            */
    SMS_BSDF_DIELECTRIC = 1,  /* dielectric, eta = int_ior / ext_ior            */
    SMS_BSDF_CONDUCTOR = 2,   /* conductor, complex ior (eta, k)                */
    SMS_BSDF_ROUGHPLASTIC = 3 /* src/bsdfs/roughplastic.cpp: diffuse base
                                 (albedo) under a rough dielectric coating
                                 (eta = int_ior / ext_ior, Beckmann alpha > 0);
                                 for the path tracer only (no SMS caster)      */
} sms_bsdf_type;

/* alpha > 0 makes a dielectric / conductor the reference's roughdielectric /
 * roughconductor with an isotropic Beckmann distribution of that roughness
 * (src/bsdfs/roughdielectric.cpp, roughconductor.cpp; BSDF::roughness()).  A
 * rough single-scatter caster draws an offset normal per query
 * (manifold_ss.cpp:60-70). */
typedef struct sms_bsdf {
    int32_t type;       /* sms_bsdf_type                                        */
    float   eta;        /* dielectric relative IOR, or conductor real part      */
    float   k;          /* conductor imaginary part                             */
    float   albedo[3];  /* diffuse reflectance (receivers)                      */
    float   alpha;      /* Beckmann roughness, 0 = smooth                       */
    int32_t twosided;   /* the BSDF acts on both sides (src/bsdfs/twosided.cpp):
                           seen from the back, the local frame's normal is
                           reflected; not around a dielectric, as there      */
    int32_t nonlinear;  /* roughplastic: the base's internal scattering with the
                           nonlinear colour model (roughplastic.cpp:166, 290) */
} sms_bsdf;

typedef struct sms_scene sms_scene;  /* host-side scene builder (owned by caller) */

sms_status sms_scene_create(sms_scene **out);
void       sms_scene_destroy(sms_scene *scene);

/* Analytic sphere (src/shapes/sphere.cpp). shape_id_out may be NULL. */
sms_status sms_scene_add_sphere(sms_scene *scene, const float center[3], float radius,
                                int32_t flip_normals, const sms_bsdf *bsdf,
                                uint32_t flags, int32_t *shape_id_out);

/* Triangle mesh (src/librender/mesh.cpp).  positions: n_vertices*3 floats,
 * normals/texcoords: optional (NULL) n_vertices*3 / *2 floats, faces: n_faces*3
 * vertex indices.  Data is copied. */
sms_status sms_scene_add_mesh(sms_scene *scene, const float *positions,
                              const float *normals, const float *texcoords,
                              uint32_t n_vertices, const uint32_t *faces,
                              uint32_t n_faces, const sms_bsdf *bsdf,
                              uint32_t flags, int32_t *shape_id_out);

/* Wavefront OBJ reader (src/shapes/obj.cpp:90-330): one output vertex per
 * distinct (v, vt, vn) reference in order of first use, polygons
 * fan-triangulated, texture v flipped unless flip_tex_coords is 0, vertex
 * normals recomputed (angle-weighted, src/librender/mesh.cpp:420-470) when the
 * file has none, no vertex normals with face_normals.  Arrays are allocated
 * by the library (normals / texcoords NULL when absent); release them with
 * sms_mesh_data_free.  Feed them to sms_scene_add_mesh.  Errors:
 * SMS_ERR_PARSE with the line in sms_last_error(). */
typedef struct sms_mesh_data {
    uint32_t n_vertices, n_faces;
    float *positions;   /* 3 x n_vertices */
    float *normals;     /* 3 x n_vertices or NULL */
    float *texcoords;   /* 2 x n_vertices or NULL */
    uint32_t *faces;    /* 3 x n_faces */
} sms_mesh_data;
sms_status sms_obj_load(const char *path, int32_t face_normals, int32_t flip_tex_coords,
                        sms_mesh_data *out);
void sms_mesh_data_free(sms_mesh_data *mesh);

/* Point light (src/emitters/point.cpp). */
sms_status sms_scene_add_point_emitter(sms_scene *scene, const float position[3],
                                       const float intensity[3], uint32_t flags);

/* Area light attached to an existing sphere shape (src/emitters/area.cpp). */
sms_status sms_scene_add_area_emitter(sms_scene *scene, int32_t shape_id,
                                      const float radiance[3], uint32_t flags);

/* Slope-based normal map of a glinty shape (the level-0 (sx, sy) channels of
 * the reference's LEAN data, src/librender/normalmap.cpp:7-36, as used by
 * NormalmapBSDF::slope, src/bsdfs/normalmap.cpp:305-336).  slopes: res*res
 * interleaved FP16 pairs (IEEE binary16 bit patterns), row-major with v as the
 * row; tiles as the BSDF's "tiles" parameter.  A shape without caster or
 * bouncer flags becomes glinty.  On a caster / bouncer the map is the
 * reference's normalmap BSDF around the shape's dielectric / conductor: its
 * manifold vertices take the normal-mapped frame and its derivative
 * (src/bsdfs/normalmap.cpp:236-290), and cfg.twostage enables the two-stage
 * solver on it (manifold_ss.cpp:253-270): each walk first solves on the
 * smoothed surface (the top level of the map's LEAN pyramid) toward a slope
 * drawn from that level's Gaussian, then on the full map.  Walks on a
 * normal-mapped caster take a learned proposal's seeds: SMS_ERR_UNSUPPORTED.
 * One normal map per scene. */
sms_status sms_scene_set_normalmap(sms_scene *scene, int32_t shape_id,
                                   const uint16_t *slopes, uint32_t res, float tiles);

/* The normal map's LEAN fallback (NormalmapBSDF's lean_fallback,
 * src/bsdfs/normalmap.cpp:46-55, 80-112, 142-170, 187-203): at path vertices
 * without uv partials -- every vertex after the camera's first hit -- the
 * normal-mapped shape reflects like the glossy LEAN distribution of the map's
 * top mip level widened by the base roughness alpha (lean_fallback_alpha,
 * 1e-4 in the reference), with the Fresnel factor of the IOR eta + i k
 * (dielectric Fresnel when k = 0; the reference's defaults are eta 0, k 1).
 * The surface then also takes emitter samples (the BSDF is glossy).  Call
 * after sms_scene_set_normalmap. */
sms_status sms_scene_set_lean_fallback(sms_scene *scene, float alpha, float eta, float k);

/* --------------------------------------------------------------- context */
typedef struct sms_ctx sms_ctx;   /* device copy of a scene + config + scratch */

/* Upload the scene (BVH build on the host, copy to device 'device'). */
sms_status sms_ctx_create(const sms_scene *scene, const sms_config *cfg,
                          int32_t device, sms_ctx **out);
void       sms_ctx_destroy(sms_ctx *ctx);
sms_status sms_ctx_set_config(sms_ctx *ctx, const sms_config *cfg);
/* The CUDA stream all work of this context is issued on (a cudaStream_t). */
void      *sms_ctx_stream(sms_ctx *ctx);
/* Launch shape of the persistent kernels: blocks per SM and threads per block
 * (0 = library default).  Set by the autotuner. */
sms_status sms_ctx_set_launch(sms_ctx *ctx, int32_t blocks_per_sm, int32_t threads_per_block);
/* Lanes per query of the unbiased estimator's Bernoulli-trial kernel: 8, 16
 * or 32 trials of one query run side by side (the first success is found by
 * ballot, so results do not depend on it); 0 picks 32 for uniform seeding and
 * 8 with a learned proposal.  No counterpart in the reference (a tuning knob
 * of the batched solver). */
sms_status sms_ctx_set_trial_group(sms_ctx *ctx, int32_t group);
/* Top node records of the scene's tree (stored breadth first) that the
 * Bernoulli-trial kernel copies into each block's shared memory before it
 * traverses, 0..384 (0 = none, the default).  Replaces node fetches through
 * L1 for the top levels; results do not depend on it.  No counterpart in the
 * reference (a staging knob of the batched solver, set by the autotuner). */
sms_status sms_ctx_set_treelet(sms_ctx *ctx, int32_t nodes);
/* Queries a lane group of the Bernoulli-trial kernel claims from the work queue
 * per atomic, 1..64 (default 1).  Results do not depend on it.  No counterpart
 * in the reference (a tuning knob of the batched solver, set by the autotuner). */
sms_status sms_ctx_set_queue_chunk(sms_ctx *ctx, int32_t chunk);

/* ---------------------------------------------------------------- queries */
/* Shading-point query, SoA with SMS_QUERY_FIELDS rows of n floats each:
 *   row 0-2   p        position on the receiver
 *   row 3-5   n        shading normal (= geometric normal of the receiver)
 *   row 6-8   dp_du    position partial
 *   row 9-11  dp_dv    position partial
 *   row 12-14 albedo   diffuse reflectance of the receiver (RGB, >= 0), or,
 *                      for a receiver with any other BSDF: row 12 =
 *                      -(1 + shape id) of the receiver shape (its index among
 *                      the scene's shapes), rows 13-14 = x, y of the incident
 *                      (camera) direction in the frame built from n by the
 *                      branchless orthonormal basis of Duff et al. 2017; the
 *                      library then evaluates that shape's BSDF toward the
 *                      caster (manifold_ss.cpp:109, 191); an id outside the
 *                      scene contributes 0 and the call returns
 *                      SMS_ERR_DEVICE_LIMIT
 *   row 15    cos_i    cosine of the incident (camera) direction in the local
 *                      frame; the diffuse BSDF returns 0 when it is <= 0
 * The receiver is taken as locally flat (dn/du = dn/dv = 0), as for the
 * reference's rectangle receivers (src/shapes/rectangle.cpp:210-214). */
#define SMS_QUERY_FIELDS 16

/* Per-query estimator result, SoA:
 *   value   3 rows of n floats: RGB contribution of all caustic casters
 *   count   n int32: unbiased -> Bernoulli-trial count of the last caster
 *           (0 when its first walk failed or was occluded; -1 when the trial cap
 *           was hit); biased -> number of unique solutions summed over casters
 *   walks   n int32: number of sample_path() calls made for this query          */
typedef struct sms_result {
    float   *value;
    int32_t *count;
    int32_t *walks;
} sms_result;

/* Solver statistics, same counters as manifold_ss.cpp:14-18 (accumulated per
 * context since creation or the last reset). */
typedef struct sms_stats {
    uint64_t solver_succeeded;
    uint64_t solver_failed;
    uint64_t bernoulli_trial_calls;
    uint64_t bernoulli_trial_iterations;
    uint64_t bernoulli_trial_iterations_max;
    uint64_t walks;
    uint64_t newton_iterations;
    uint64_t connections;
    uint64_t rays;          /* rays cast by the connection kernel        */
    uint64_t bvh_nodes;     /* BVH nodes fetched (64 bytes each)         */
    uint64_t tri_tests;     /* triangles fetched (48 bytes each)         */
    uint64_t speculative_walks; /* Bernoulli trials run past the first
                                   success of their 32-trial chunk (work the
                                   sequential reference does not do)       */
} sms_stats;

sms_status sms_stats_read(sms_ctx *ctx, sms_stats *out);
sms_status sms_stats_reset(sms_ctx *ctx);   /* also clears the profile */

/* Per-phase device profile, the GPU counterpart of the reference's sampling
 * profiler phases SMSCaustics / SMSCausticsBernoulliTrials / SMSGlints
 * (include/mitsuba/core/profiler.h:25-28).  Kernel times come from CUDA events
 * recorded on the context stream around each launch while profiling is on;
 * ray / node / triangle counts are always accumulated. */
#define SMS_PHASES 8
#define SMS_PHASE_SS_FIRST   0   /* unbiased: first walk + visibility + contribution */
#define SMS_PHASE_SS_TRIALS  1   /* unbiased: Bernoulli trials                        */
#define SMS_PHASE_SS_BIASED  2   /* biased single scatter                             */
#define SMS_PHASE_SS_WALK    3   /* per-walk entry point                              */
#define SMS_PHASE_MS         4   /* multi-scatter connections                         */
#define SMS_PHASE_GLINTS     5   /* glint connections                                 */
#define SMS_PHASE_MS_WALK    6
#define SMS_PHASE_GLINT_WALK 7
typedef struct sms_profile {
    double   ms[SMS_PHASES];         /* summed kernel time (profiling on)  */
    uint64_t launches[SMS_PHASES];   /* timed launches                      */
    uint64_t rays[SMS_PHASES];
    uint64_t bvh_nodes[SMS_PHASES];  /* 64-byte node records fetched        */
    uint64_t tri_tests[SMS_PHASES];  /* 48-byte triangle records fetched    */
} sms_profile;

sms_status sms_ctx_set_profiling(sms_ctx *ctx, int32_t enable);
sms_status sms_profile_read(sms_ctx *ctx, sms_profile *out);

/* ------------------------------------------------------- single scatter */
/* SpecularManifoldSingleScatter::specular_manifold_sampling for n queries
 * (manifold_ss.cpp:28-201).  Query i draws its random numbers from a PCG32
 * stream (state seed 'seed', stream index i + stream_offset), in the same order
 * as the reference's per-query sampler calls.  Host pointers: copied in and out
 * on the context stream, synchronous. */
sms_status sms_ss_connect_batch(sms_ctx *ctx, const float *queries, uint32_t n,
                                uint64_t seed, uint64_t stream_offset,
                                sms_result *out);

/* Same, device pointers (queries, out->*), asynchronous on the context stream. */
sms_status sms_ss_connect_batch_device(sms_ctx *ctx, const float *queries_dev,
                                       uint32_t n, uint64_t seed,
                                       uint64_t stream_offset, sms_result *out_dev);

/* Allocation-free variant of sms_ss_connect_batch_device.  No counterpart in
 * the reference: it exists for callers that must not allocate device memory
 * while rendering (fixed-budget real-time loops, hosts that own every device
 * allocation and forbid libraries from calling cudaMalloc).  It runs the same kernels
 * and gives bit-identical results, but takes the unbiased estimator's
 * per-query scratch from a fixed device array inside the library instead of
 * growing the context's scratch with cudaMalloc, and calls no allocating CUDA
 * or library routine.
 *   - n may not exceed 262,144 queries (the array holds 32 bytes per query:
 *     8 MiB on every GPU that loads the library, kept until process exit);
 *     larger batches are rejected with SMS_ERR_INVALID_ARG -- split them and
 *     use stream_offset, which keeps results identical.
 *   - It accepts and refuses the same configurations as the device entry
 *     point (same checks), except that it never builds the two-stage solver's
 *     LEAN pyramid: with twostage, call sms_ss_connect_batch_device once first.
 *     A bound learned proposal is refused (its mixtures need more scratch).
 *   - The first call on a device (and the first after cudaDeviceReset) looks
 *     up the array's device address and lets the CUDA runtime load the module
 *     that holds it; make that first call before any stream capture.
 *   - Its kernels are not included in sms_profile_read's phase times.
 *   - It does not synchronize, so it cannot return SMS_ERR_DEVICE_LIMIT: a
 *     device limit its kernels hit (traversal stack, trial cap, solution
 *     capacity, a receiver shape outside the scene) is reported by the
 *     context's next synchronous call.
 *   - All calls, from every context on a device, share the one array: calls
 *     whose kernels overlap on the GPU (different streams, or different
 *     contexts) race on it.  Calls issued on one stream are safe.
 * Device pointers in and out; asynchronous on the context stream. */
sms_status sms_ss_connect_batch_noalloc(sms_ctx *ctx, const float *queries_dev,
                                        uint32_t n, uint64_t seed,
                                        uint64_t stream_offset, sms_result *out_dev);

/* Per-walk entry point: SpecularManifoldSingleScatter::sample_path with an
 * explicit start point (manifold_ss.cpp:203-279, p_start != 0), the harness
 * the reference's figure scripts use.
 *   queries   SoA as above (n columns)
 *   walk_in   SoA, SMS_WALK_IN_FIELDS rows: ei.p (3), p_start (3),
 *             sample (2; used by sample_position when p_start == 0); with
 *             cfg.twostage SMS_SS_WALK_IN_FIELDS_TWOSTAGE rows, the last two
 *             the sample of the smoothed solve's slope (manifold_ss.cpp:258)
 *   caster    shape id of the specular shape to walk on
 *   walk_out  SoA, SMS_WALK_OUT_FIELDS rows: ok, iterations, p_final (3),
 *             p_init (3), n_final (3)   (ok/iterations stored as floats;
 *             n_final is the vertex normal, the map's on a normal-mapped caster) */
#define SMS_WALK_IN_FIELDS 8
#define SMS_SS_WALK_IN_FIELDS_TWOSTAGE 10
#define SMS_WALK_OUT_FIELDS 11
sms_status sms_ss_walk_batch(sms_ctx *ctx, int32_t caster, const float *queries,
                             const float *walk_in, uint32_t n, float *walk_out);

/* ------------------------------------------------------- multi scatter */
/* SpecularManifoldMultiScatter::specular_manifold_sampling for n queries
 * (manifold_ms.cpp:27-201): k-bounce chains through shapes flagged
 * SMS_SHAPE_CAUSTIC_CASTER_MULTI / _BOUNCER, k = cfg.bounces (1..4), emitters
 * flagged SMS_EMITTER_CAUSTIC_MULTI.  Same buffers, random-number streams and
 * count/walks meaning as sms_ss_connect_batch. */
sms_status sms_ms_connect_batch(sms_ctx *ctx, const float *queries, uint32_t n,
                                uint64_t seed, uint64_t stream_offset,
                                sms_result *out);
sms_status sms_ms_connect_batch_device(sms_ctx *ctx, const float *queries_dev,
                                       uint32_t n, uint64_t seed,
                                       uint64_t stream_offset, sms_result *out_dev);

/* Per-walk multi-scatter sample_path with first_path = true
 * (manifold_ms.cpp:203-227, 280-408): walk_in as sms_ss_walk_batch; walk_out
 * SMS_MS_WALK_OUT_FIELDS rows: ok, iterations, first vertex (3), last vertex
 * (3), seed path ok. */
#define SMS_MS_WALK_OUT_FIELDS 9
sms_status sms_ms_walk_batch(sms_ctx *ctx, int32_t caster, const float *queries,
                             const float *walk_in, uint32_t n, float *walk_out);

/* --------------------------------------------------------------- glints */
/* Glint query (SoA, SMS_GLINT_QUERY_FIELDS rows): p (3), n (3), dp_du (3),
 * dp_dv (3), uv (2), duv_dx (2), duv_dy (2) of the pixel footprint (already
 * scaled like SamplingIntegrator::scale_differential), sensor position (3).   */
#define SMS_GLINT_QUERY_FIELDS 21

/* SpecularManifoldGlints::specular_manifold_sampling, SMS strategy
 * (manifold_glints.cpp:28-176, and the vectorized variant when
 * cfg.glints_vectorized): emitter sample over all emitters, shadow test, then
 * the biased or unbiased estimator over footprint seeds.  value =
 * sms_weight x ei.weight, i.e. everything except the MIS weight against BSDF
 * sampling (LEAN pdf) and the sensor importance We, which the integrator
 * multiplies in (:159-175).  count: unique glints (biased) or the Bernoulli
 * count (unbiased). */
sms_status sms_glint_connect_batch(sms_ctx *ctx, const float *queries, uint32_t n,
                                   uint64_t seed, uint64_t stream_offset,
                                   sms_result *out);
sms_status sms_glint_connect_batch_device(sms_ctx *ctx, const float *queries_dev,
                                          uint32_t n, uint64_t seed,
                                          uint64_t stream_offset, sms_result *out_dev);

/* sample_glint with an explicit footprint sample (xi_start,
 * manifold_glints.cpp:225-265).  walk_in SMS_GLINT_WALK_IN_FIELDS rows: light
 * point (3), footprint sample (2); walk_out SMS_GLINT_WALK_OUT_FIELDS rows: ok,
 * iterations, uv_final (2), uv_init (2). */
#define SMS_GLINT_WALK_IN_FIELDS 5
#define SMS_GLINT_WALK_OUT_FIELDS 6
sms_status sms_glint_walk_batch(sms_ctx *ctx, const float *queries,
                                const float *walk_in, uint32_t n, float *walk_out);

/* ---------------------------------------------------- learned proposal */
/* No counterpart in the reference, whose walks are always seeded uniformly on
 * the caster (manifold_ss.cpp:223, Shape::sample_position).  A proposal is a
 * small network (9 features: shading point, light sample, shading normal,
 * normalised and frequency-encoded -> 4 x 64 SiLU -> 8-component Gaussian
 * mixture over the caster's uv frame)
 * trained on the GPU from walks that the uniform-seed solver itself
 * converges.  Bound to a context, it seeds the unbiased single-scatter
 * estimator's first walk and every Bernoulli trial of that caster from
 *   q(uv) = defensive * uniform + (1 - defensive) * mixture(query),
 * three random numbers per walk instead of two.  The trials redraw from the
 * same q, so their count still estimates 1 / P(reaching the first solution)
 * and the estimator stays unbiased; the uniform component keeps every
 * solution reachable.
 * uv frame of a caster: mesh -> its bounding box spanned by the two widest
 * axes (uv in [0,1]^2 covers the box, the third axis at mid-height); sphere ->
 * (theta / pi, phi / 2 pi).  The network's mean outputs are offsets from an
 * anchor uv computed in FP32: where the segment from the shading point to the
 * light sample meets the frame's plane (mesh, clamped to [-1, 2]^2), or the
 * sphere point along the bisector of the directions from the centre to the
 * shading point and to the light sample (sphere). */
#define SMS_PROPOSAL_FEATURES 9      /* x (3), light sample (3), n (3)    */
#define SMS_PROPOSAL_OUTPUTS 40      /* 8 logits, 8 x 2 means, 8 x 2 raw  */
#define SMS_PROPOSAL_PARAMS 21808    /* FP32 master parameters            */
typedef struct sms_proposal sms_proposal;

/* A fresh network for caster shape `caster` of ctx (a SMS_SHAPE_CAUSTIC_CASTER_SINGLE
 * shape), initialised from `init_seed`, with room for `capacity` training
 * pairs on the device.  Destroy proposals before their context. */
sms_status sms_proposal_create(sms_ctx *ctx, int32_t caster, uint64_t init_seed,
                               uint32_t capacity, sms_proposal **out);
sms_status sms_proposal_destroy(sms_proposal *p);

/* Training pairs from the solver: for each query (device SoA, as
 * sms_ss_connect_batch) the emitter sample and `walks_per_query` uniformly
 * seeded walks on the stream (seed, stream_offset + i); each distinct solution
 * they converge to (uniqueness threshold of the config) that the light sample
 * sees appends one pair: features, uv of the solution, and a weight = the
 * solution's share of the query's summed contribution.  Pairs are appended to
 * those already held; *total = pairs held afterwards (at most capacity).
 * Synchronous. */
sms_status sms_proposal_collect(sms_proposal *p, const float *queries_dev, uint32_t n,
                                uint64_t seed, uint64_t stream_offset,
                                int32_t walks_per_query, uint32_t *total);
/* Replace the training set with host arrays (features SoA 9 x n, uv SoA 2 x n,
 * weights n or NULL for all ones). */
sms_status sms_proposal_set_data(sms_proposal *p, const float *features, const float *uv,
                                 const float *weights, uint32_t n);
/* Read the training set back (host arrays sized as above for the first
 * min(cap, count) pairs; weights may be NULL); *n = pairs held. */
sms_status sms_proposal_get_data(sms_proposal *p, float *features, float *uv, float *weights,
                                 uint32_t cap, uint32_t *n);
/* sigma_scale (> 0, default 1) multiplies every mixture sigma when seeds are
 * drawn (any fixed proposal keeps the estimator unbiased; a sharper one puts
 * more seeds inside the predicted basins).  weighted (default 1): the
 * training loss weights each pair by its contribution share. */
sms_status sms_proposal_set_options(sms_proposal *p, float sigma_scale, int32_t weighted);
/* Set the input normalisation (x - shift) * scale from the training set's
 * mean and standard deviation (features with zero spread get scale 0). */
sms_status sms_proposal_normalize(sms_proposal *p);

/* `steps` Adam steps (lr, beta 0.9 / 0.999, eps 1e-8) on batches of `batch`
 * pairs (multiple of 16, <= 65536) drawn with replacement from the training
 * set; the mean batch NLL of the last min(steps, 256) steps in *mean_loss.
 * Steps are replayed from a CUDA graph. Synchronous. */
sms_status sms_proposal_train(sms_proposal *p, int32_t steps, int32_t batch, float lr,
                              float *mean_loss);
/* Loss and gradient of the first `batch` pairs of the training set without
 * an update (gradient checks): *loss = mean NLL, grad = d loss / d params. */
sms_status sms_proposal_loss_grad(sms_proposal *p, int32_t batch, float *loss, float *grad);

/* Network state for checkpoint / resume.  params, adam_m, adam_v: 21808
 * floats each (any may be NULL on get); norm: shift (9) then scale (9);
 * step: Adam steps taken. */
sms_status sms_proposal_get_state(sms_proposal *p, float *params, float *adam_m, float *adam_v,
                                  float *norm, uint32_t *step);
sms_status sms_proposal_set_state(sms_proposal *p, const float *params, const float *adam_m,
                                  const float *adam_v, const float *norm, uint32_t step);

/* Network outputs for host feature arrays (9 x n): mixture = 0 gives the raw
 * 40 outputs (logits, mean offsets from the anchor, log-sigma logits),
 * mixture = 1 the processed mixture the seeding uses: cdf (8), means (8 x 2,
 * anchor added), sigmas (8 x 2).  out: 40 x n. */
sms_status sms_proposal_eval(sms_proposal *p, const float *features, uint32_t n, int32_t mixture,
                             float *out);

/* The caster's uv frame: kind (0 box, 1 sphere), org (3), ax_u (3), ax_v (3);
 * box: seed = org + u ax_u + v ax_v; sphere: org + ax_u[0] * (sin(pi u)
 * cos(2 pi v), sin(pi u) sin(2 pi v), cos(pi u)). */
sms_status sms_proposal_frame(sms_proposal *p, float frame[10]);

/* Bind a proposal to its context (NULL unbinds); defensive in (0, 1] is the
 * uniform seeding's share.  While bound, the unbiased single-scatter entry
 * points seed its caster from the proposal; the biased estimator and the
 * allocation-free entry point return SMS_ERR_UNSUPPORTED. */
sms_status sms_ctx_set_proposal(sms_ctx *ctx, sms_proposal *p, float defensive);

/* ------------------------------------------------------------- rendering */
/* Wavefront path tracer around the SMS solvers, the reference's sampling
 * integrators for this path:
 *   path          src/integrators/path.cpp:94-226
 *   path_sms_ss   src/integrators/path_sms_ss.cpp:69-251
 *   path_sms_ms   src/integrators/path_sms_ms.cpp:172-330
 * with the MonteCarloIntegrator parameters (src/librender/integrator.cpp:
 * 300-320), a perspective sensor (src/sensors/perspective.cpp) and a box
 * reconstruction filter (one pixel per sample, src/rfilters/box.cpp), for
 * scenes of diffuse, smooth dielectric and smooth conductor BSDFs, point
 * lights and sphere area lights.  Shading points on caustic receivers are
 * solved as one SMS batch per bounce by the context's estimator and config.
 *
 * Random numbers: path p = s * width * height + y * width + x (sample s of
 * pixel (x, y)) draws from PCG32 stream p (state seed `seed`) in the
 * reference's per-sample order: pixel position (2), wavelength (1), then per
 * bounce Russian roulette (1, past rr_depth), emitter sampling (2, when it
 * runs) and BSDF sampling (1 + 2).  The SMS call at bounce `depth` of path p
 * draws from stream p + depth * 2^48 of state seed sms_render_sms_seed(seed).
 * Images therefore do not depend on the wavefront size. */
typedef struct sms_camera {
    float   to_world[16];   /* row-major camera-to-world; camera space has x
                               left, y up, z forward (the reference's look_at) */
    float   fov;            /* field of view in degrees along fov_axis       */
    int32_t fov_axis;       /* SMS_FOV_*                                     */
    int32_t width, height;  /* film size in pixels                           */
    float   near_clip;      /* 1e-2 */
    float   far_clip;       /* 1e4  */
} sms_camera;
#define SMS_FOV_X        0
#define SMS_FOV_Y        1
#define SMS_FOV_DIAGONAL 2
#define SMS_FOV_SMALLER  3
#define SMS_FOV_LARGER   4

#define SMS_INTEGRATOR_PATH            0
#define SMS_INTEGRATOR_PATH_SMS_SS     1
#define SMS_INTEGRATOR_PATH_SMS_MS     2
#define SMS_INTEGRATOR_PATH_SMS_GLINTS 3   /* src/integrators/path_sms_glints.cpp:62-194 */
/* Plain path tracing restricted to the light paths path_sms_ss / path_sms_ms
 * account for (the paper's equal-time comparisons): src/integrators/
 * path_filtered_ss.cpp:36-181 and path_filtered_ms.cpp:36-206 (chain length
 * = the context's cfg.bounces). */
#define SMS_INTEGRATOR_PATH_FILTERED_SS 4
#define SMS_INTEGRATOR_PATH_FILTERED_MS 5
/* The paper's combined integrator (src/integrators/path_sms_teaser.cpp:60-81,
 * 120-320): single- and multi-scatter caustics at receivers with the
 * context's config (the "caustics_*" block), biased glints at glinty shapes
 * seen from the camera with options.glints (the "glints_*" block), and path
 * tracing filtered to the paths SMS does not handle (non_sms_paths_enabled). */
#define SMS_INTEGRATOR_PATH_SMS_TEASER 6
/* Its comparison integrator (src/integrators/path_filtered_teaser.cpp): path
 * tracing restricted like path_sms_teaser's caustics -- on a caster, emitter
 * samples and emitter hits count only when they complete the single-scatter
 * chain (caster, then a caustic single-scatter emitter) or the multi-scatter
 * chain of the context's cfg.bounces (multi_caustic_bounces) vertices, with
 * the scattering SMS solves; elsewhere only with non_sms_paths_enabled.  As
 * in the reference, an emitter hit completes either chain only when the
 * emitter is flagged caustic_emitter_multi_scatter (:380-393).  No glints. */
#define SMS_INTEGRATOR_PATH_FILTERED_TEASER 7
typedef struct sms_render_options {
    int32_t  integrator;                 /* SMS_INTEGRATOR_*                        */
    int32_t  max_depth;                  /* -1 = unbounded                          */
    int32_t  rr_depth;                   /* 5                                       */
    int32_t  spp;                        /* samples per pixel (1)                   */
    int32_t  disable_reflected_emitters; /* path_sms_ss (false)                     */
    int32_t  biased_mnee;                /* path_sms_ss (false)                     */
    uint64_t seed;                       /* 0                                       */
    uint32_t max_paths;                  /* paths per wavefront, 0 = 1,048,576      */
    float    glint_diff_scale_factor_clamp; /* 0: ray differentials of the camera are
                                           scaled by max(1/sqrt(spp), this)
                                           (src/librender/integrator.cpp:41,164-165) */
    uint32_t samples_per_pass;           /* 0 = spp; spp must be a multiple of it
                                            (integrator.cpp:35,61-68)              */
    float    timeout;                    /* seconds, <= 0: none.  Passes of
                                            samples_per_pass spp are rendered until
                                            the time is up; the image is the mean
                                            of the passes done (integrator.cpp:36,
                                            143-146: the reference stops at the
                                            block, here at the pass) */
    /* path_sms_teaser only (path_sms_teaser.cpp:60-81) */
    int32_t  caustics_enabled;           /* true                                    */
    int32_t  glints_enabled;             /* true                                    */
    int32_t  non_sms_paths_enabled;      /* true                                    */
    sms_config glints;                   /* glints_* (SMSConfig defaults); the
                                            glints always run the biased estimator
                                            (path_sms_teaser.cpp:347-350)          */
    /* the film's reconstruction filter: SMS_RFILTER_BOX (this struct's default;
       each pixel the mean of its samples) or SMS_RFILTER_GAUSSIAN (the
       reference film's default, src/rfilters/gaussian.cpp: stddev, radius
       4 stddev, tabulated like rfilter.cpp:9-20; every sample splats onto the
       pixels within the radius, imageblock.cpp:111-160, and each pixel is its
       weighted mean)                                                         */
    int32_t  rfilter;
    float    rfilter_stddev;             /* 0.5; Gaussian only, (0, 2]             */
} sms_render_options;
#define SMS_RFILTER_BOX      0
#define SMS_RFILTER_GAUSSIAN 1
void sms_render_options_default(sms_render_options *opt);

/* Samples per pixel of the context's last render (spp, or fewer after a
 * timeout). */
uint32_t sms_render_spp_done(const sms_ctx *ctx);

/* State seed of the SMS streams (SplitMix64 of the seed). */
uint64_t sms_render_sms_seed(uint64_t seed);

/* Render: image receives height x width RGB (row-major, y down, 3 floats per
 * pixel) = the mean of spp samples.  sms_render takes a host pointer and
 * returns when the image is there; sms_render_device takes a device pointer
 * and is asynchronous on the context stream apart from one small
 * device-to-host read per bounce (the number of SMS queries).
 * Unbiased MNEE (mnee_init without biased_mnee): path_sms_ss and path_sms_ms
 * add a BSDF-sampled caustic path when the deterministic MNEE walk from its
 * receiver does not find the same chain (path_sms_ss.cpp:207-241,
 * path_sms_ms.cpp:54-142, 323-360).
 *
 * path_sms_glints: camera rays carry ray differentials; at the first hit of
 * the glinty shape the glint estimator (the context's config) runs over the
 * pixel footprint, weighted by the sensor importance and MIS against a BSDF
 * sample inside the footprint, both with the LEAN-mapping density of the
 * footprint (manifold_glints.cpp:28-223, the LEAN mip pyramid of
 * src/librender/normalmap.cpp, include/mitsuba/render/lean.h); the
 * normal-mapped BSDF samples its nested BSDF in the frame of the bilinear
 * slope normal elsewhere (normalmap.cpp:118-135).
 * The LEAN pyramid (5 floats per texel over all levels, 4/3 x 20 bytes per
 * texel of the slope map) is built on the device at the first glint render. */
sms_status sms_render(sms_ctx *ctx, const sms_camera *cam, const sms_render_options *opt, float *image);
sms_status sms_render_device(sms_ctx *ctx, const sms_camera *cam, const sms_render_options *opt,
                             float *image_dev);

#ifdef __cplusplus
}
#endif
#endif /* SMS_GB300_H */
