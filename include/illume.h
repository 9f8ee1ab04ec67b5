/*
 * illume-gb300: C-ABI of the GB300 wavefront path tracer.
 *
 * Drop-in boundary for the reference renderer's render path (matthewshang/illume):
 *   HostScene(rapidjson::Document&)            src/scene/scene.h:11-28, src/scene/scene.cpp:11-99
 *   SceneRef(HostScene&)                       src/scene/sceneref.h:11-35 (host -> device copy)
 *   Renderer(json, HostScene&, spp, max_depth) src/renderer.h:8-25, src/renderer.cu:39-59
 *   Renderer::render_to_bitmap(Bitmap*)        src/renderer.cu:498-597
 *   Renderer::get_width / get_height           src/renderer.cu:599-607
 *   bitmap_new / bitmap_free / bitmap_save_to_png   src/bitmap.h:26-30
 *   CLI  illume <save> <scene> <spp> <maxdepth>     src/main.cu:14-43
 *
 * Conventions: every function that can fail returns an int status (ILLUME_OK = 0,
 * negative on error) and never exits or prints on the render path; the message of the
 * last failure on the calling thread is returned by illume_last_error(). Handles are
 * opaque. A context owns one CUDA stream on one device; it may be used from one host
 * thread at a time, and different contexts may be used concurrently. The library owns
 * device memory; callers own every host buffer they pass.
 */
#ifndef ILLUME_H
#define ILLUME_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ILLUME_ABI_VERSION 4

enum illume_status {
  ILLUME_OK = 0,
  ILLUME_ERR_INVALID = -1,     /* bad argument or handle */
  ILLUME_ERR_CUDA = -2,        /* CUDA runtime error (message has the CUDA string) */
  ILLUME_ERR_OOM = -3,         /* device or host allocation failed */
  ILLUME_ERR_IO = -4,          /* file could not be read or written */
  ILLUME_ERR_PARSE = -5,       /* malformed JSON or OBJ */
  ILLUME_ERR_BUDGET = -6,      /* request exceeds the context's HBM budget */
  ILLUME_ERR_TIMEOUT = -7,     /* a bounded device wait ran out */
  ILLUME_ERR_CANCELLED = -8,   /* job cancelled */
  ILLUME_ERR_UNSUPPORTED = -9, /* feature not available in this build */
  ILLUME_ERR_NOT_READY = -10,  /* job still running (illume_job_poll) */
  ILLUME_ERR_TRAVERSAL = -11   /* a BVH traversal stack overflowed: the render's outputs are
                                * written but rays may have missed hits (scene upload rejects
                                * trees deep enough for this, so it reports a defect) */
};

/* ---- enumerations shared with the JSON scene format ---- */
enum illume_material_type { /* src/material.h:12-20 */
  ILLUME_MAT_EMISSIVE = 0, ILLUME_MAT_LAMBERT = 1, ILLUME_MAT_REFLECTIVE = 2, ILLUME_MAT_REFRACTIVE = 3,
  ILLUME_MAT_ROUGHREFLECTIVE = 4, ILLUME_MAT_ROUGHREFRACTIVE = 5, ILLUME_MAT_CONDUCTOR = 6,
  ILLUME_MAT_ROUGHCONDUCTOR = 7, ILLUME_MAT_PLASTIC = 8
};
enum illume_texture_type { ILLUME_TEX_CONSTANT = 0, ILLUME_TEX_CHECKERBOARD = 1, ILLUME_TEX_BITMAP = 2 }; /* src/texture.h:8-11 */
enum illume_distribution { ILLUME_DIST_BECKMANN = 0, ILLUME_DIST_GGX = 1 };
enum illume_tonemapper { ILLUME_TONE_LINEAR = 0, ILLUME_TONE_REINHARD = 1, ILLUME_TONE_FILMIC = 2, ILLUME_TONE_UNCHARTED = 3 }; /* src/tonemapper.h:10-13 */
enum illume_intersector { ILLUME_ISECT_MT = 0, ILLUME_ISECT_WATERTIGHT = 1 };
/* WIDE4: 128-byte 4-wide nodes with FP32 child boxes, collapsed from the binary tree (the
 * default of illume_render_params_default). BINARY: 64-byte nodes holding both child
 * boxes. WIDE8: 80-byte 8-wide nodes with 8-bit quantised child boxes. WIDE8_PERSISTENT:
 * the same nodes traversed by a persistent kernel that schedules node and triangle steps
 * per warp. All four give the same closest hits. The 8-wide layout is built (on the host
 * cores) and uploaded when a render, trace, check or digest first asks for it, so the
 * first such call on a scene takes longer and must not be made under stream capture. */
enum illume_bvh_kind { ILLUME_BVH_BINARY = 0, ILLUME_BVH_WIDE8 = 1, ILLUME_BVH_WIDE8_PERSISTENT = 2, ILLUME_BVH_WIDE4 = 3 };
enum illume_accum_mode { ILLUME_ACCUM_FP32 = 0, ILLUME_ACCUM_KAHAN = 1, ILLUME_ACCUM_FP64 = 2 };
/* REFERENCE: paths find light only by BSDF sampling, as src/renderer.cu:183-386 (the
 * default; every parity test runs it). NEE: adds next-event estimation with multiple
 * importance sampling at lambert, rough conductor and rough dielectric reflection
 * vertices (environment map and emissive mesh triangles); same expectation, less noise. */
enum illume_estimator { ILLUME_ESTIMATOR_REFERENCE = 0, ILLUME_ESTIMATOR_NEE = 1 };

/* ---- reference output types: same layout as src/bitmap.h:6-20 ---- */
typedef struct { size_t red, green, blue; } illume_pixel;
typedef struct { illume_pixel* pixels; size_t width, height; } illume_bitmap;

typedef struct illume_context illume_context;
typedef struct illume_scene illume_scene;
typedef struct illume_renderer illume_renderer;

/* Flat, host-side description of a scene: what HostScene holds after parsing
 * (src/scene/scene.h:20-27), as plain arrays. Matrices are 3x4 row-major (the rows of
 * the reference's Matrix4 without the constant last row). Unused pointers may be NULL
 * when the matching count is zero. Per-mesh arrays index into the pooled arrays. */
typedef struct {
  /* meshes (src/primitives/mesh.h:18-33) */
  int32_t num_meshes;
  const int32_t* mesh_vertex_offset;  /* first vertex of each mesh in positions */
  const int32_t* mesh_num_vertices;
  const int32_t* mesh_tri_offset;     /* first triangle of each mesh in tris */
  const int32_t* mesh_num_tris;
  const int32_t* mesh_has_normals;    /* 0 = face normals (the JSON default) */
  const int32_t* mesh_has_texcoords;
  const int32_t* mesh_bvh_leaf_size;  /* bvh_items_per_node (JSON default 4) */
  const float* positions;             /* 3 per vertex */
  const float* normals;               /* 3 per vertex (read for meshes with normals) */
  const float* texcoords;             /* 2 per vertex (read for meshes with texcoords) */
  const int32_t* tris;                /* 3 per triangle, vertex indices local to the mesh */
  /* instances (src/primitives/mesh_instance.h:13-20) */
  int32_t num_instances;
  const int32_t* inst_mesh;
  const int32_t* inst_material;
  const float* inst_mat;              /* 12 per instance: object -> world */
  const float* inst_inv;              /* 12 per instance: world -> object */
  const float* inst_trans_inv;        /* 12 per instance: normal transform (transpose of inv) */
  /* spheres (src/primitives/sphere.h:11-17) */
  int32_t num_spheres;
  const float* sphere_center_radius;  /* 4 per sphere */
  const int32_t* sphere_material;
  /* materials (src/material.h:22-33) */
  int32_t num_materials;
  const int32_t* mat_type;            /* illume_material_type */
  const int32_t* mat_albedo_tex;
  const int32_t* mat_roughness_tex;
  const int32_t* mat_medium;          /* -1 = air */
  const int32_t* mat_distribution;    /* illume_distribution */
  const float* mat_ior;
  const float* mat_diffuse_fresnel;   /* plastic: Fresnel::diffuse_fresnel(1/ior, 1e6) */
  const float* mat_eta;               /* 3 per material */
  const float* mat_k;                 /* 3 per material */
  /* mediums (src/medium.h:8-14) */
  int32_t num_mediums;
  const float* med_absorption;        /* 3 per medium, already 1 - JSON value */
  const float* med_scattering;
  const float* med_g;
  const int32_t* med_active;
  /* textures (src/texture.h:13-48) */
  int32_t num_textures;
  const int32_t* tex_type;            /* illume_texture_type */
  const float* tex_color;             /* 3 per texture: constant colour / checker on colour */
  const float* tex_off;               /* 3 per texture: checker off colour */
  const float* tex_scale;             /* 2 per texture */
  const int32_t* tex_width;
  const int32_t* tex_height;
  const int32_t* tex_hdr;             /* 1 = float texels, bilinear; 0 = 8-bit texels, point */
  const int64_t* tex_texel_offset;    /* first float of each bitmap in texels */
  const float* texels;                /* RGBA, 4 floats per texel (8-bit texels as 0..255) */
  int32_t env_tex;                    /* environment texture, -1 = black */
  /* camera (src/camera.h:9-17) */
  float camera_transform[12];
  float camera_fov, camera_dof, camera_aperture;
  /* render_settings (src/renderer.cu:42-58) */
  int32_t width, height;
  float ray_bias;
  int32_t tonemapper;                 /* illume_tonemapper */
} illume_scene_desc;

/* Parameters of one render (Renderer's settings plus the GB300 extensions). */
typedef struct {
  int32_t width, height;      /* image size (scene default from render_settings) */
  int32_t spp;                /* samples per pixel */
  int32_t max_depth;          /* closest-hit queries per path */
  int32_t sample_begin;       /* first sample index (progressive / sharded renders) */
  float ray_bias;
  int32_t tonemapper;         /* illume_tonemapper */
  uint32_t seed, job;         /* Philox key */
  int32_t accum_mode;         /* illume_accum_mode */
  int32_t intersector;        /* illume_intersector */
  int32_t bvh_kind;           /* illume_bvh_kind */
  int32_t exact_hg;           /* 0 = reference Henyey-Greenstein sampler, 1 = exact */
  int32_t samples_per_pass;   /* samples of every pixel kept in flight per wavefront pass (0 = auto:
                               * min(spp, 128M paths / pixels), at least 1) */
  /* Nullable camera override, read when a renderer is created or a job is submitted: 12
   * floats of the camera-to-world rows (3x4, the layout of illume_scene_desc's
   * camera_transform), then fov (degrees), dof and aperture. NULL = the scene's camera. */
  const float* camera;
  int32_t trace_variant;      /* binary BVH: 0 = 64 registers, fused box tests, dynamic ray fetch,
                               * while-while traversal (default); 1 = compiler's register choice,
                               * grid-stride rays, leaves tested where met; 2 = variant 1 held to 64
                               * registers; 3 = variant 0 with leaves tested where met; 4 = variant
                               * 0 with lane refill. 4-wide BVH: 0 = at most 64 registers,
                               * near / far planes loaded by per-ray offsets, stack in local
                               * memory (default); 1 = four compare-swaps instead of five in
                               * the child ordering; 2 = lo / hi planes selected per child
                               * box; 3 = at most 80 registers; 4 = variant 0 with exact
                               * box-test reciprocals and the instances walked in index
                               * order (variant 0 takes the hardware's approximate
                               * reciprocal and, in scenes of 3 to 16 instances, visits
                               * the instances a ray enters nearest box entry first).
                               * 8-wide (ILLUME_BVH_WIDE8): 2 = the compiler's register
                               * choice (others: at most 64 registers). The persistent
                               * 8-wide layout ignores it. */
  int32_t shade_variant;      /* 0 = the measured best register bound (default), 1 = the
                               * compiler's choice, 2 / 3 / 4 = at most 80 / 72 / 64 registers */
  int32_t estimator;          /* illume_estimator */
  int32_t engines;            /* renderer: engines (path tables on their own streams) taking
                               * turns on the passes of a call, so that one pass's last bounces
                               * overlap the next passes; 0 = for a pass of 4M paths or more one
                               * per 16M paths, 2 to 4, else 1; at most 16 and at most the
                               * samples per pass.
                               * The image does not depend on it. The server ignores it
                               * (ILLUME_SERVER_LANES). */
  /* Path regeneration (no counterpart in the reference, whose passes hold one sample of
   * every pixel): with queue_slots > 0 and below a pass's paths, the wavefront queues hold
   * queue_slots rays, and each pass runs as a loop on the device (one graph launch: a
   * while node) in which new paths of the pass enter the queue as earlier ones end,
   * whenever the next queue holds at most regen_threshold x queue_slots rays (0 <=
   * regen_threshold <= 1; 1 = refill every iteration). 0 = every path of a pass starts
   * at once (the default). The image does not depend on either. A loop that reaches its
   * iteration bound (never expected) makes the render return ILLUME_ERR_TIMEOUT. */
  int32_t queue_slots;
  float regen_threshold;
  /* Order of a pass's camera rays in the queue (no counterpart in the reference): up to
   * ray_group samples of a pixel next to each other, pixels in 8x4 tiles, so that a warp's
   * rays start alike and stay alike for more bounces. 0 = the library's choice (16, the
   * fastest measured), 1 = one sample of every pixel after another. The image does not
   * depend on it. */
  int32_t ray_group;
} illume_render_params;

typedef struct {
  int64_t rays;               /* closest-hit queries, counted as src/renderer.cu:554 counts them */
  int64_t paths;
  double render_ms;           /* device time of the bounce loop (CUDA events) */
  double total_ms;            /* wall time of the call, uploads and downloads included */
  int64_t kernel_launches;    /* launches of this library's kernels during the call */
  int64_t h2d_bytes, d2h_bytes;
} illume_render_stats;

/* Hit record of the closest-hit test hook. */
typedef struct {
  float t;                    /* FLT_MAX on a miss */
  float u, v;                 /* barycentric weights of vertices 1 and 2 (mesh hits) */
  int32_t inst;               /* instance index, -1 if none */
  int32_t prim;               /* triangle index within the instance's mesh, -1 if none */
  int32_t sphere;             /* sphere index, -1 if none */
  int32_t pad[2];
} illume_hit;

/* ---- errors and version ---- */
const char* illume_last_error(void);
int illume_abi_version(void);

/* ---- context ---- */
int illume_context_create(int device, size_t hbm_budget_bytes, illume_context** out);
int illume_context_destroy(illume_context* ctx);
/* Where the BVHs of the scenes later made on this context are built (no counterpart in
 * the reference, whose tree is built on one host thread, src/accel/bvh.cpp:65-439):
 * HOST (the default) = binned SAH on the host cores; DEVICE = locally-ordered clustering
 * on the context's GPU (Morton order, then merges of mutual nearest neighbours within 16
 * positions), the leaves and node layouts made on the host from its tree. The two give
 * different trees and the same closest hits. A device build that fails or whose tree is
 * too deep for the traversal stacks is replaced by the host build
 * (illume_scene_build_info). Host-only scenes (no context) are always built on the host. */
enum illume_bvh_builder { ILLUME_BVH_BUILD_HOST = 0, ILLUME_BVH_BUILD_DEVICE = 1 };
int illume_context_set_bvh_builder(illume_context* ctx, int builder);
/* the context's CUDA stream (a cudaStream_t) */
void* illume_context_stream(illume_context* ctx);

/* ---- scenes: HostScene + SceneRef ---- */
/* Parse a scene file in the reference JSON format; relative "file" paths resolve
 * against base_dir (NULL = the current directory, as the reference does).
 * With ctx == NULL the three scene constructors build a host-only scene (parsed,
 * validated, BVHs built, nothing uploaded): it can be described and checked, not
 * rendered. */
int illume_scene_load_json(illume_context* ctx, const char* path, const char* base_dir, illume_scene** out);
int illume_scene_load_json_string(illume_context* ctx, const char* json, const char* base_dir, illume_scene** out);
int illume_scene_create(illume_context* ctx, const illume_scene_desc* desc, illume_scene** out);
/* Fill *out with pointers into the scene's host copy (valid while the scene lives). */
int illume_scene_describe(const illume_scene* scene, illume_scene_desc* out);
/* Device bytes held by the scene (geometry, BVHs, textures). */
int illume_scene_device_bytes(const illume_scene* scene, size_t* out);
/* Copies the scene's geometry to its device buffers again: triangles, vertex attributes,
 * every BVH layout, and the mesh / instance / sphere / material tables (what the
 * reference's SceneRef copies at the start of every render_to_bitmap,
 * src/scene/sceneref.cpp:9-122). Textures and light tables stay resident (the
 * reference creates its texture objects once, in HostScene). Synchronous. Returns the
 * bytes copied in *bytes (nullable). */
int illume_scene_upload(illume_scene* scene, size_t* bytes);
/* Checks the BVH invariants of every mesh (each triangle referenced exactly once, child
 * boxes inside their parent's, quantised boxes containing the exact boxes) and writes a
 * one-line summary per mesh (node counts, depths) into report. */
int illume_scene_check_bvh(const illume_scene* scene, char* report, size_t report_len);
/* Meshes of the scene whose BVHs came from the device build, and the wall time of the
 * scene's BVH construction (all meshes, cache hits included) in milliseconds. */
int illume_scene_build_info(const illume_scene* scene, int* device_meshes, double* build_ms);
/* Test hook: 64-bit FNV-1a digests of mesh `mesh`'s built layouts, in the order binary
 * nodes, 4-wide nodes, triangle records of both, 8-wide nodes with their triangle
 * records. Equal digests = bit-identical trees (the build's thread count, set by the
 * environment variable ILLUME_BUILD_THREADS, does not change them). */
int illume_scene_bvh_digest(const illume_scene* scene, int mesh, uint64_t out[4]);
/* Process-wide cache of mesh BVH builds, keyed by mesh content (vertex and index words):
 * scenes that share a mesh build it once. Not in the reference, which caches one BVH
 * file per OBJ path (src/accel/bvh.cpp:363-439). */
int illume_bvh_cache_stats(int64_t* entries, int64_t* bytes, int64_t* hits, int64_t* misses);
int illume_bvh_cache_clear(void);
int illume_scene_destroy(illume_scene* scene);

/* ---- renderer ---- */
/* Defaults of the reference: the scene's render_settings, seed 0, linear tonemap unless
 * the scene names another, FP32 accumulation, Beckmann as parsed. */
int illume_render_params_default(const illume_scene* scene, int spp, int max_depth, illume_render_params* out);
int illume_renderer_create(illume_context* ctx, illume_scene* scene, const illume_render_params* params,
                           illume_renderer** out);
int illume_renderer_destroy(illume_renderer* r);
int illume_renderer_get_width(const illume_renderer* r);
int illume_renderer_get_height(const illume_renderer* r);
/* Renderer::render_to_bitmap: full render and tonemap into a caller-allocated bitmap of
 * the renderer's size. */
int illume_render_to_bitmap(illume_renderer* r, illume_bitmap* bitmap, illume_render_stats* stats);
/* Render into host buffers (each nullable): mean linear radiance (W*H*3 floats), the
 * per-pixel sum and sum of squares of per-sample radiance (W*H*3 doubles each) and the
 * tonemapped RGB8 image (W*H*3 bytes). The sum follows accum_mode; the sum of squares is
 * an FP64 total of each pass's squares summed in FP32 (for variance estimates). */
int illume_render(illume_renderer* r, float* out_mean, double* out_sum, double* out_sumsq, uint8_t* out_rgb8,
                  illume_render_stats* stats);
/* Device-resident variant: runs the bounce loop only, leaving the accumulators on the
 * device (inputs already resident). Accumulates on top of earlier calls when
 * accumulate != 0. */
int illume_render_device(illume_renderer* r, int accumulate, illume_render_stats* stats);
/* Copies the device accumulators (sum, sumsq as in illume_render) to host buffers. */
int illume_renderer_read(illume_renderer* r, float* out_mean, double* out_sum, double* out_sumsq, uint8_t* out_rgb8);

/* Per-stage timing of one wavefront pass (samples_per_pass samples of every pixel),
 * launched kernel by kernel with CUDA events on the context stream. With count_visits,
 * the pass runs an instrumented trace kernel that counts node fetches and triangle
 * tests (its timings are then not representative). Accumulates into the renderer like
 * a progressive call. */
typedef struct {
  double raygen_ms, trace_ms, shade_ms, accumulate_ms;
  int64_t trace_launches, shade_launches;
  int64_t rays;
  int64_t node_fetches, tri_tests;   /* count_visits only */
  int64_t node_bytes, tri_bytes;     /* bytes of one node / one triangle record in the BVH used */
  int64_t lane_slots;                /* count_visits only: sum over the trace kernel's 32-ray warp
                                      * batches of 32 x the batch's most node fetches
                                      * (node_fetches / lane_slots = lane utilisation) */
} illume_profile;
int illume_renderer_profile(illume_renderer* r, int count_visits, illume_profile* out);

/* Render without allocating (no counterpart in the reference). For callers that cannot
 * allocate device memory at render time: hosts whose own pool owns all device memory,
 * and frame loops that must not stall on cudaMalloc/cudaFree. The wavefront queues live
 * in a fixed array inside the library (about 12 MB, reserved on every GPU that loads the
 * library until exit), which limits images to ILLUME_NOALLOC_MAX_PIXELS pixels; larger
 * images are rejected with ILLUME_ERR_INVALID. Renders params->spp samples (one per
 * pass, FP32 accumulation in sample order, accum_mode must be ILLUME_ACCUM_FP32) and
 * writes the per-pixel sum of radiance (3 floats per pixel) to the caller's device
 * buffer d_sum. Asynchronous on the context's stream. Takes the parameter checks of
 * illume_renderer_create; samples_per_pass and engines above 1, queue_slots above 0 and
 * the next-event estimator are rejected with ILLUME_ERR_UNSUPPORTED. The first call on a context looks
 * up the array's device address and caches it with the launch sizes; make it before any
 * stream capture. After a device reset (which invalidates every handle) the address is
 * looked up again. All calls share the array: calls whose GPU work overlaps race, so
 * order them on one stream. */
#define ILLUME_NOALLOC_MAX_PIXELS 65536
int illume_render_noalloc(illume_context* ctx, illume_scene* scene, const illume_render_params* params, float* d_sum);

/* ---- bitmap (src/bitmap.h:26-30) ---- */
illume_bitmap* illume_bitmap_new(size_t width, size_t height);
void illume_bitmap_free(illume_bitmap* bitmap);
int illume_bitmap_save_png(const illume_bitmap* bitmap, const char* path);
int illume_bitmap_save_ppm(const illume_bitmap* bitmap, const char* path);
int illume_save_pfm(const float* rgb, int width, int height, const char* path);

/* ---- test hooks ---- */
/* Closest hit of n rays (8 floats each: ox, oy, oz, unused, dx, dy, dz, unused; the
 * direction is used as given) against a scene, on the device; host buffers. */
int illume_trace_closest(illume_context* ctx, illume_scene* scene, const float* rays, int n, int intersector,
                         int bvh_kind, illume_hit* hits);
/* Same with device pointers, on the context's stream, no synchronisation. */
int illume_trace_closest_device(illume_context* ctx, illume_scene* scene, const float* d_rays, int n,
                                int intersector, int bvh_kind, illume_hit* d_hits);
/* BSDF sample / eval / pdf on the device for n tuples (host buffers). Each input tuple
 * is 16 floats: wi (3, pointing away from the surface), n (3), u1, u2, u3, roughness,
 * ior, eta.xyz, k, plastic diffuse-Fresnel term (0 = computed from ior); outputs are 16
 * floats: new_dir (3), weight (3), D, pdf_m, G, F, eval (f * cos, reflection), pdf_dir,
 * status (0 killed, 1 reflect, 2 transmit), 3 unused. The albedo is 1; conductors use
 * the one k for all three channels. */
int illume_bsdf_batch(illume_context* ctx, int material_type, int distribution, const float* inputs, int n,
                      float* outputs);

/* ---- batched and served rendering ----
 * Not in the reference, which renders one scene per call (src/renderer.cu:498-597).
 * Jobs with the same intersector and BVH layout share one wavefront job table: every
 * pass advances all running jobs, jobs are admitted while they run (continuous
 * batching), and each job's image is bit-identical to its render alone. */
typedef struct illume_server illume_server;
typedef int64_t illume_job_id;
/* max_jobs_in_flight: job-table rows (0 = 64). hbm_budget_bytes gates admission by the
 * server's device bytes (job accumulators and output staging plus the tables' path
 * buffers; scenes are the caller's and not counted); 0 = unlimited. */
int illume_server_create(illume_context* ctx, size_t hbm_budget_bytes, int max_jobs_in_flight, illume_server** out);
int illume_server_destroy(illume_server* s);
/* Queue a job (ILLUME_ERR_BUDGET if its footprint can never fit the budget). The
 * server ignores params->samples_per_pass and the binary-kernel variant word. */
int illume_job_submit(illume_server* s, illume_scene* scene, const illume_render_params* params, illume_job_id* out);
/* One scheduling round: wait for the passes the previous round launched and retire the
 * jobs they finished, admit what fits, compose the passes (jobs grouped by scene,
 * smallest remaining job first, slots shared by water-filling) and launch up to
 * ILLUME_SERVER_PASSES_PER_STEP wavefront passes (fewer if a job finishes sooner)
 * without waiting for them, so the device works while the caller does. A job's results
 * are ready (illume_job_poll) after the round that retires it; stats lag by a round.
 * *jobs_running = running + queued jobs afterwards (0 once everything is retired). */
int illume_server_step(illume_server* s, int* jobs_running);
/* ILLUME_OK when done (results copied to the nullable buffers), ILLUME_ERR_NOT_READY
 * otherwise. stats: rays of this job, paths, render_ms = submit-to-finish minus queue
 * wait (wall), total_ms = submit to finish (wall), kernel_launches of the passes the
 * job took part in. */
int illume_job_poll(illume_server* s, illume_job_id id, float* out_mean, uint8_t* out_rgb8, illume_render_stats* stats);
/* Cancels a queued or running job (its row and buffers are freed before the next pass);
 * a finished job keeps its results. */
int illume_job_cancel(illume_server* s, illume_job_id id);

typedef enum {
  ILLUME_SERVER_PATH_CAPACITY = 0,    /* path slots of each job table (default 33554432) */
  ILLUME_SERVER_PASSES_PER_STEP = 1,  /* passes per illume_server_step (default 1) */
  ILLUME_SERVER_AUTOTUNE = 2,         /* 1 = choose path slots and trace kernel from measured throughput */
  ILLUME_SERVER_TRACE_VARIANT = 3,    /* trace kernel variant (-1 = default) */
  ILLUME_SERVER_LANES = 4,            /* job tables per trace-kernel setting, each on its own
                                       * stream, whose passes overlap (1-16, default 4;
                                       * illume_render_batch uses 16); a table
                                       * is created only when every existing one has work */
  ILLUME_SERVER_QUEUE_SLOTS = 5,      /* path regeneration in every table: rays in flight
                                       * (0 = off, the default; see
                                       * illume_render_params.queue_slots) */
  ILLUME_SERVER_REGEN_THRESHOLD = 6   /* its refill threshold in thousandths (0-1000,
                                       * default 1000). The autotuner also tries
                                       * regeneration at a quarter of the path slots with
                                       * thresholds 1 and 1/4. */
} illume_server_option;
int illume_server_set_option(illume_server* s, int option, int64_t value);

typedef struct {
  int64_t rays;               /* closest-hit queries traced by all jobs */
  int64_t passes;             /* wavefront passes run */
  int64_t kernel_launches;
  int64_t jobs_done;
  double device_ms;           /* device time of the passes (CUDA events) */
  int64_t path_capacity;      /* path slots per table in use */
  int32_t trace_variant;      /* trace kernel variant in use */
  int32_t tuned;              /* 1 once the autotuner has chosen */
  int64_t device_bytes;       /* bytes the server holds on the device */
  int32_t queue_slots;        /* path regeneration in use: rays in flight per table (0 = off) */
  float regen_threshold;      /* and its refill threshold */
} illume_server_stats;
int illume_server_get_stats(const illume_server* s, illume_server_stats* out);

/* The server's split of `cap` path slots between n running jobs of npix[i] pixels with
 * left[i] samples to go (host only; exposed for tests and schedulers): per_pass[i] >= 1
 * samples of job i go into each pass, sum(per_pass[i] * npix[i]) <= cap.
 * ILLUME_ERR_BUDGET when one sample of every job does not fit. */
int illume_plan_pass_shares(int n, const int32_t* npix, const int32_t* left, int64_t cap, int32_t* per_pass);

/* The alias table (Walker) that the next-event estimator picks lights with, for n
 * non-negative weights (host only; exposed for tests; no counterpart in the reference,
 * which samples no lights): u in [0, 1) picks slot floor(u n), which keeps itself when
 * the fraction of u n is below keep[i] and becomes alias[i] otherwise, so that i comes
 * out with probability weights[i] / sum. ILLUME_ERR_INVALID when the weights sum to 0. */
int illume_alias_table(int n, const double* weights, float* keep, int32_t* alias);

/* Read bandwidth (GB/s) of a `bytes` buffer the device's L2 holds, swept `reps` times by
 * a grid-stride kernel with 16-byte loads that bypass L1 (measurement hook for the
 * traversal roofline, whose node and triangle data stay in L2; no counterpart in the
 * reference). Allocates and frees the buffer itself. */
int illume_measure_l2_read(illume_context* ctx, size_t bytes, int reps, double* gbs);

/* Renders n jobs together through one server (all submitted at once) and returns each
 * job's mean radiance (3 floats per pixel) and RGB8 in the nullable per-job buffers.
 * autotune: see ILLUME_SERVER_AUTOTUNE. batch_stats is nullable. */
int illume_render_batch(illume_context* ctx, int n, illume_scene* const* scenes, const illume_render_params* params,
                        float* const* out_mean, uint8_t* const* out_rgb8, illume_render_stats* job_stats,
                        int autotune, illume_server_stats* batch_stats);

#ifdef __cplusplus
}
#endif

#endif /* ILLUME_H */
