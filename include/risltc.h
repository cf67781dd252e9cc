/* risltc.h - C ABI of the GB300 implementation of risltc's per-pixel shading
 * path: RIS over polygonal lights with an LTC-integral target, projected
 * solid angle sampling of the chosen polygon, shadow-ray visibility and the
 * MIS combine.
 *
 * The first half repeats the reference's own host-side API verbatim (types,
 * enums and functions of src/polygonal_light.h, src/ltc_table.h,
 * src/noise_table.h and src/main.h), so C99 host code written against the
 * reference compiles unchanged.  The second half replaces what the reference
 * does through Vulkan (LTC texture upload, light buffer, acceleration
 * structure, the full-screen shading draw) with plain functions over host or
 * device pointers.
 *
 * Conventions: every function returns an int status (RISLTC_OK == 0) unless
 * it mirrors a reference function with another signature; no function prints,
 * aborts or traps.  A context is bound to one device and one CUDA stream and
 * is not thread-safe; distinct contexts may be used concurrently.  All device
 * work is stream-ordered.
 */
#ifndef RISLTC_H
#define RISLTC_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define EXTERN_C extern "C"
#else
#define EXTERN_C
#endif

/* ======================================================================== */
/* Reference API (verbatim)                                                 */
/* ======================================================================== */

/* src/polygonal_light.h:31-46 */
typedef enum sample_polygon_technique_e {
	sample_polygon_baseline,
	sample_polygon_area_turk,
	sample_polygon_projected_solid_angle,
	sample_polygon_projected_solid_angle_biased,
	sample_polygon_ltc_cp,
	sample_polygon_count
} sample_polygon_technique_t;

/* src/polygonal_light.h:52-67 */
typedef enum polygon_texturing_technique_e {
	polygon_texturing_none = 0,
	polygon_texturing_area = 1,
	polygon_texturing_portal = 2,
	polygon_texturing_ies_profile = 3,
	polygon_texturing_count,
	polygon_texturing_force_int = 0x7fffffff
} polygon_texturing_technique_t;

/* src/polygonal_light.h:73-99.  Host description of a convex polygonal
   light: Euler angles, scalings, translation and plane-space vertices in;
   world-space vertices, plane, area and radiance written by
   update_polygonal_light(). */
typedef struct polygonal_light_s {
	float rotation_angles[3];
	float scaling_x;
	float translation[3];
	float scaling_y;
	float radiant_flux[3];
	float inv_scaling_x;
	float surface_radiance[3];
	float inv_scaling_y;
	float plane[4];
	uint32_t vertex_count;
	polygon_texturing_technique_t texturing_technique;
	uint32_t texture_index;
	uint32_t padding_0;
	float rotation[3][4];
	float area, rcp_area;
	float padding_1[2];
	char* texture_file_path;
	float* vertices_plane_space;
	float* vertices_world_space;
} polygonal_light_t;

/* src/polygonal_light.h:104-111: the fixed part of one light in the
   shader's std140 light buffer. */
typedef struct polygonal_light_upload_s {
	float surface_radiance[3];
	float padding_1;
	float plane[4];
	uint32_t vertex_count;
	float padding_2[3];
} polygonal_light_upload_t;

/* src/polygonal_light.h:115-119 */
#define POLYGONAL_LIGHT_QUICKSAVE_SIZE (sizeof(float) * 20 + sizeof(uint32_t) * 2)
#define POLYGONAL_LIGHT_FIXED_CONSTANT_BUFFER_SIZE (sizeof(float) * 12)

/* src/main.h:59-77 */
typedef enum mis_heuristic_e {
	mis_heuristic_balance,
	mis_heuristic_power,
	mis_heuristic_weighted,
	mis_heuristic_optimal_clamped,
	mis_heuristic_optimal,
	mis_heuristic_count
} mis_heuristic_t;

/* src/main.h:79-84 */
typedef enum light_sampling_strategies_e { light_uniform, light_reservoir } light_sampling_strategies_t;

/* src/ltc_table.h:23-35 */
typedef struct ltc_constants_s {
	float fresnel_index_factor, fresnel_index_summand;
	float roughness_factor, roughness_summand;
	float inclination_factor, inclination_summand;
	float padding[2];
} ltc_constants_t;

/* src/noise_table.h:25-29 */
typedef struct noise_table_s {
	uint32_t random_seed;
} noise_table_t;

/* src/polygonal_light.c:27-41.  Like the reference, the return value is
   always 0 (it compares the count after assigning it). */
EXTERN_C int set_polygonal_light_vertex_count(polygonal_light_t* light, uint32_t vertex_count);
/* src/polygonal_light.c:44-98 */
EXTERN_C void update_polygonal_light(polygonal_light_t* light);
/* src/polygonal_light.c:101-110 */
EXTERN_C polygonal_light_t duplicate_polygonal_light(const polygonal_light_t* light);
/* src/polygonal_light.c:113-118 */
EXTERN_C void destroy_polygonal_light(polygonal_light_t* light);
/* src/noise_table.c:24-28 (VkBool32 animate_noise becomes uint32_t). */
EXTERN_C void set_noise_constants(uint32_t resolution_mask[2], uint32_t* texture_index_mask, uint32_t random_numbers[4],
                                  noise_table_t* noise, uint32_t animate_noise);

/* ======================================================================== */
/* GB300 replacement of the Vulkan-side path                                */
/* ======================================================================== */

enum risltc_status_e {
	RISLTC_OK = 0,
	RISLTC_ERROR_INVALID_ARGUMENT = 1,
	RISLTC_ERROR_VERTEX_COUNT = 2,
	RISLTC_ERROR_CUDA = 3,
	RISLTC_ERROR_TRAVERSAL_LIMIT = 4,
	RISLTC_ERROR_NON_FINITE = 5,
	RISLTC_ERROR_NO_DEVICE = 6,
	RISLTC_ERROR_OUT_OF_MEMORY = 7,
	RISLTC_ERROR_IO = 8,
	RISLTC_ERROR_UNSUPPORTED = 9,
	RISLTC_ERROR_TOO_LARGE = 10,
	RISLTC_ERROR_DEVICE_TIMEOUT = 11 /* a bounded device-side wait ran out (reported by risltc_ctx_check) */
};

/* Largest light vertex count (MAX_POLYGONAL_LIGHT_VERTEX_COUNT of
   main.c:181-204).  The reference's clipper covers 3..7 vertices; 8-vertex
   lights are clipped by the same rule extended by one vertex. */
#define RISLTC_MAX_LIGHT_VERTEX_COUNT 8

/* wang_random_number, src/math_utilities.h:50-57 */
EXTERN_C uint32_t risltc_wang_random_number(uint32_t seed);

/* std140 light buffer exactly as write_lights (src/main.c:456-490) builds it
   for the shader, except that every slot past vertex_count holds vertex 0
   (the reference writes it to slot vertex_count only and leaves the rest
   unwritten).  Calls update_polygonal_light() on each light.  data must hold
   count * (12 + 4 * max_vertex_count) floats. */
EXTERN_C int risltc_write_lights(float* data, polygonal_light_t* lights, uint32_t count, uint32_t max_vertex_count);
/* get_max_polygonal_light_vertex_count, src/main.c:183-189 (at least 3; no
   lights, or a null array, gives 3) */
EXTERN_C uint32_t risltc_max_light_vertex_count(const polygonal_light_t* lights, uint32_t count);

/* LTC table in FP32 (the reference keeps two UNORM16 texture arrays,
   src/ltc_table.h:41-57).  texels0: [fresnel][inclination][roughness][4] =
   (m00, -m02, m11, m20) of the normalised inverse fit; texels1: [...][2] =
   (m22, albedo). */
typedef struct risltc_ltc_table_s {
	uint32_t roughness_count, inclination_count, fresnel_count;
	uint32_t padding;
	float* texels0;
	float* texels1;
	ltc_constants_t constants;
} risltc_ltc_table_t;

/* The quantisation of load_ltc_table (src/ltc_table.c:82-116) and its
   constants (:184-192) without Vulkan.  fit holds fresnel_count slices of
   resolution^2 records of 5 floats (the records of fit<i>.dat after the
   uint64 resolution header).  quantize_unorm16 != 0 rounds every stored value
   to 16-bit UNORM as the reference's textures do. */
EXTERN_C int risltc_ltc_table_from_fit(risltc_ltc_table_t* table, const float* fit, uint32_t resolution,
                                       uint32_t fresnel_count, int quantize_unorm16);
/* Reads directory/fit<i>.dat for i < fresnel_count (load_ltc_table's files). */
EXTERN_C int risltc_load_ltc_table(risltc_ltc_table_t* table, const char* directory, uint32_t fresnel_count,
                                   int quantize_unorm16);
/* A smooth synthetic fit (positive diagonal, albedo in (0,1)) from a seed;
   stands in for the reference's fit files, which are not distributed. */
EXTERN_C int risltc_ltc_table_synthetic(risltc_ltc_table_t* table, uint64_t seed, uint32_t roughness_count,
                                        uint32_t inclination_count);
EXTERN_C void risltc_ltc_table_destroy(risltc_ltc_table_t* table);

/* Binary BVH over triangles, built on the host by binned SAH over
   references: a triangle whose box is large against the mean is cut into up
   to 8 pieces (early split clipping), each a reference to the whole triangle
   with the piece's box, at most 3 references per triangle in all.  Node =
   8 x 32-bit words {bmin.xyz, left_or_first, bmax.xyz, count}; count == 0
   marks an interior node with children left and left + 1; a leaf covers
   references [first, first + count) of the reordered triangle array
   (triangle_count references, 12 floats each {v0, 0, v1 - v0, 0, v2 - v0, 0},
   triangle_ids[k] the input triangle of reference k).  Every point of a
   triangle lies in the box of a leaf that references it, and boxes are
   widened by a relative 1e-6, so traversal never culls a box that holds a
   hit; any-hit answers equal a brute-force test of every triangle. */
typedef struct risltc_bvh_s {
	uint32_t node_count, triangle_count, depth;
	uint32_t padding;
	float* nodes;
	float* triangles;
	uint32_t* triangle_ids;
} risltc_bvh_t;
/* triangles: 9 floats per triangle (v0, v1, v2). */
EXTERN_C int risltc_bvh_build(risltc_bvh_t* bvh, const float* triangles, uint32_t triangle_count, uint32_t max_leaf_size);
EXTERN_C void risltc_bvh_destroy(risltc_bvh_t* bvh);

/* first_person_camera_t, src/camera.h:29-49 (48 bytes), as stored at the
   start of a quicksave file. */
typedef struct risltc_camera_s {
	float position_world_space[3];
	float rotation_z, rotation_x, vertical_fov;
	float near_plane, far_plane, speed;
	int32_t rotate_camera;
	float rotation_x_0, rotation_z_0;
} risltc_camera_t;

/* quick_load, src/main.c:76-125: reads a quicksave file (camera, then lights
   with their plane-space vertices and texture paths; legacy files with
   scaling_y <= 0 get scaling_y = scaling_x) and returns the lights with their
   derived members updated (update_polygonal_light).  camera may be NULL.
   Free the lights with risltc_destroy_lights.  RISLTC_ERROR_IO on a missing,
   short or implausible file. */
EXTERN_C int risltc_quick_load(const char* path, risltc_camera_t* camera, polygonal_light_t** lights,
                               uint32_t* light_count);
/* quick_save, src/main.c:45-71: writes the same format. */
EXTERN_C int risltc_quick_save(const char* path, const risltc_camera_t* camera, const polygonal_light_t* lights,
                               uint32_t light_count);
/* destroy_polygonal_light on each light, then frees the array. */
EXTERN_C void risltc_destroy_lights(polygonal_light_t* lights, uint32_t light_count);

/* Light clusters (no counterpart in the reference, which draws RIS
   candidates uniformly over all lights): k-means with k-means++ seeding of
   the lights' centres (centers: light_count x 3 floats) into cluster_count
   clusters, deterministic for a seed (double arithmetic, splitmix64).
   order (light_count entries) lists the lights cluster by cluster, ascending
   inside a cluster; cluster c holds order[offsets[c] .. offsets[c + 1])
   (offsets: cluster_count + 1 entries; a cluster may be empty). */
EXTERN_C int risltc_cluster_lights(const float* centers, uint32_t light_count, uint32_t cluster_count,
                                   uint64_t seed, uint32_t iterations, uint32_t* order, uint32_t* offsets);

/* Summaries of clusters (offsets as for risltc_cluster_lights, lights as the
   std140 rows of risltc_write_lights listed cluster by cluster): per cluster
   a bounding sphere (bounds: centre xyz = mean of the lights' vertices,
   radius rounded up) and the power (power: sum over its lights of the
   radiance's luminance times the polygon's area).  Used by
   risltc_scene_set_clusters. */
EXTERN_C int risltc_cluster_summaries(const float* lights_std140, uint32_t light_count, uint32_t max_vertex_count,
                                      const uint32_t* offsets, uint32_t cluster_count, float* bounds, float* power);

/* Run settings: render_settings_t (src/main.h:123-156) reduced to what the
   shading pass reads, plus the candidate count the reference hard-codes
   (shading_pass.frag.glsl:726, 32). */
typedef enum risltc_numerics_e {
	/* IEEE division and square root, no contraction, the project's own
	   transcendentals: bit-identical to the CPU oracle. */
	risltc_numerics_exact = 0,
	/* Hardware reciprocal square root, approximate division and
	   contraction in the RIS candidate evaluation, whose results only weight
	   the reservoir; the final PSA/MIS shading stays exact.  Faster; the
	   chosen light equals the exact path's for at least 99.9% of pixels, and
	   where it does the estimates agree within 1% relative at the 99th
	   percentile (the tested bounds). */
	risltc_numerics_fast = 1
} risltc_numerics_t;

typedef enum risltc_proposal_e {
	risltc_proposal_uniform = 0,  /* p = 1 / N (shading_pass.frag.glsl:733) */
	risltc_proposal_clusters = 1, /* cluster weights: power over distance with a cosine bound */
	risltc_proposal_learned = 2   /* cluster weights: softmax of a learned model's logits */
} risltc_proposal_t;

/* Tile shapes of the RIS candidate kernel: pixels per warp x candidates per
   pixel per chunk (the warp sorts each chunk's candidates by vertex count
   and evaluates them 32 at a time), or one thread per pixel with its
   candidates in sequence.  In exact numerics every shape gives the same
   results bit for bit; in fast numerics the binned shapes agree bit for bit
   and the per-pixel shape, whose multiply-adds the compiler contracts in
   its own way, agrees within the fast-numerics bounds.  risltc_autotune
   picks the fastest for a workload. */
typedef enum risltc_tile_e {
	risltc_tile_32x8 = 0, /* default */
	risltc_tile_16x8 = 1,
	risltc_tile_8x8 = 2,
	risltc_tile_32x4 = 3,
	risltc_tile_16x4 = 4,
	risltc_tile_per_pixel = 5,
	risltc_tile_count = 6
} risltc_tile_t;

typedef struct risltc_settings_s {
	sample_polygon_technique_t polygon_sampling_technique; /* ltc_cp or projected_solid_angle(_biased) */
	light_sampling_strategies_t light_sampling;
	mis_heuristic_t mis_heuristic;
	uint32_t candidate_count;   /* M */
	uint32_t sample_count;      /* SAMPLE_COUNT */
	uint32_t sample_count_light; /* LIGHT_SAMPLES */
	float mis_visibility_estimate;
	uint32_t fast_atan;
	uint32_t shadows;           /* trace shadow rays through the scene BVH */
	risltc_numerics_t numerics;
	/* Source of the RIS candidates (default configuration only): uniform
	   over all lights as in the reference, or the cluster proposal of
	   risltc_scene_set_clusters mixed with uniform sampling. */
	risltc_proposal_t proposal;
	float proposal_uniform_fraction; /* in (0, 1]: weight of the uniform part */
	risltc_tile_t tile;         /* candidate kernel tile shape (default configuration only) */
} risltc_settings_t;

/* specify_default_render_settings, src/main.c:220-236 (M = 32, shadows on;
   a null pointer is ignored) */
EXTERN_C void risltc_default_settings(risltc_settings_t* settings);

/* G-buffer: 17 planes of width*height floats in device memory (the fields
   of shading_data_t, src/shaders/brdfs.glsl:22-39): position xyz, normal xyz,
   outgoing xyz, lambert_outgoing, diffuse_albedo rgb, fresnel_0 rgb,
   roughness.  primitive (optional) marks background with 0xFFFFFFFF. */
#define RISLTC_GBUFFER_PLANES 17
typedef struct risltc_gbuffer_s {
	uint32_t width, height;
	const float* planes;
	const uint32_t* primitive;
} risltc_gbuffer_t;

/* The reservoir of reservoir.glsl:16-25 for the first light sample. */
typedef struct risltc_reservoir_s {
	int32_t light_index;
	float w_sum;
	float sample_value;
	uint32_t padding;
} risltc_reservoir_t;

typedef struct risltc_ctx_s risltc_ctx_t;
typedef struct risltc_scene_s risltc_scene_t;
typedef struct risltc_model_s risltc_model_t;

/* stream: a cudaStream_t, or NULL for the legacy default stream. */
EXTERN_C int risltc_ctx_create(risltc_ctx_t** ctx, int device, void* stream);
EXTERN_C void risltc_ctx_destroy(risltc_ctx_t* ctx);

/* Gives the scene's lights a cluster structure for the cluster proposal:
   cluster c holds lights offsets[c] .. offsets[c + 1] (the lights must be
   listed cluster by cluster, e.g. in the order of risltc_cluster_lights;
   offsets[0] = 0, offsets[cluster_count] = light_count, at most 1024
   clusters).  Derives each cluster's bounding sphere and power (luminance x
   area summed over its lights) and uploads them. */
EXTERN_C int risltc_scene_set_clusters(risltc_scene_t* scene, const uint32_t* offsets, uint32_t cluster_count);

/* The learned cluster proposal (no counterpart in the reference): an MLP
   from a shading point's position (centred and scaled by the model's input
   transform), normal, outgoing direction and roughness, encoded with six
   sine/cosine frequencies per input (144 features), through two hidden
   layers of 64 ReLU units to one logit per cluster; BF16 weights, FP32
   accumulation on the tensor cores.  q(cluster) = softmax(logits).
   Parameters: FP32, in the order W1 [64][144], b1 [64], W2 [64][64], b2 [64],
   W3 [clusters][64], b3 [clusters] (risltc_model_parameter_count floats). */
EXTERN_C uint32_t risltc_model_parameter_count(uint32_t cluster_count);
/* cluster_count: a multiple of 8, at most 1024.  Weights He-uniform from the
   seed (the output layer scaled by 0.1), biases zero. */
EXTERN_C int risltc_model_create(risltc_ctx_t* ctx, uint32_t cluster_count, uint64_t seed, risltc_model_t** model);
EXTERN_C void risltc_model_destroy(risltc_model_t* model);
EXTERN_C int risltc_model_set_params(risltc_model_t* model, const float* params);
EXTERN_C int risltc_model_get_params(const risltc_model_t* model, float* params);
/* Online training: while enabled, every risltc_shade call that uses this
   model for the learned proposal also trains it on its own RIS candidates
   (frame 0, every pixel_stride-th pixel, the phase following the noise
   seed): the candidates' weights p_hat / p give each cluster's share of the
   pixel's shading, the loss is its cross entropy with softmax(logits), and
   one Adam step (beta 0.9 / 0.999) with the given learning rate follows the
   call's kernels.  Defaults: off, 1e-3, 64. */
EXTERN_C int risltc_model_set_training(risltc_model_t* model, int enable, float learning_rate, uint32_t pixel_stride);
/* The training target's mix (default 0.5): with weight 1 - shadowed_weight
   the candidates' unshadowed per-cluster shares, with shadowed_weight the
   frame's final shaded estimate (with shadow rays) attributed to the chosen
   light's cluster, which makes the proposal learn visibility.  The shadowed
   part needs shadows on and one sample per technique. */
EXTERN_C int risltc_model_set_target_mix(risltc_model_t* model, float shadowed_weight);
/* How training steps run (flags, default 0): on the tensor cores (tcgen05,
   BF16 operands, FP32 accumulation) for every model (up to 256 clusters with
   all weight gradients accumulated in tensor memory, beyond that with the
   output layer in chunks of 128 clusters whose weight gradients are added to
   the gradient vector per tile).  RISLTC_TRAIN_CUDA_CORES: the FP32
   CUDA-core kernel for every model.  RISLTC_TRAIN_ACCUMULATE_ONLY: each
   training call adds its gradient to the model's gradient vector and takes
   no Adam step (risltc_model_apply_update takes it). */
#define RISLTC_TRAIN_CUDA_CORES 1u
#define RISLTC_TRAIN_ACCUMULATE_ONLY 2u
EXTERN_C int risltc_model_set_training_flags(risltc_model_t* model, uint32_t flags);
/* The accumulated gradient (risltc_model_parameter_count floats, host
   memory; synchronises the context's stream), reset to zero if clear. */
EXTERN_C int risltc_model_get_gradient(risltc_model_t* model, float* gradient, int clear);
/* One Adam step on the accumulated gradient, which it resets
   (stream-ordered on the context's stream). */
EXTERN_C int risltc_model_apply_update(risltc_model_t* model);
/* One RIS candidate of a pixel for risltc_model_train: the light drawn (an
   index into the scene's lights) and its RIS weight p_hat / p. */
typedef struct risltc_candidate_s {
	int32_t light;
	float weight;
} risltc_candidate_t;
/* One training step of the scene's model on caller-supplied candidates: the
 * step risltc_shade takes after a frame when training is on, with the frame's
 * candidates replaced by the caller's (no counterpart in the reference; for
 * callers that make their own RIS candidates, and for tests of the gradient).
 * Training pixels are i = phase + j * stride (phase < stride) of the G-buffer;
 * candidates (device, width * height * candidate_count records, pixel-major)
 * is read at training pixels only, candidates naming no light of the scene or
 * with a weight of 0 are skipped.  The target is each cluster's share of the
 * pixel's candidate weight (the scene's clusters, whose count must equal the
 * model's); with shaded (device, one float per pixel: the shaded estimate's
 * luminance) and reservoirs (device, the chosen light per pixel) the shadowed
 * part of risltc_model_set_target_mix is added.  The gradient of the mean
 * cross entropy over the training pixels is added to the model's gradient;
 * an Adam step follows unless RISLTC_TRAIN_ACCUMULATE_ONLY is set.  Runs on
 * the tensor cores or the CUDA cores as risltc_model_set_training_flags says.
 * Stream-ordered on the context's stream. */
EXTERN_C int risltc_model_train(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                                const risltc_candidate_t* candidates, uint32_t candidate_count, uint32_t stride,
                                uint32_t phase, const float* shaded, const risltc_reservoir_t* reservoirs);
/* Inputs: position (p - center) / half_extent. */
EXTERN_C int risltc_model_set_input_transform(risltc_model_t* model, const float center[3], float half_extent);
/* The model the scene's learned proposal uses (its cluster count must match
   the scene's clusters); NULL detaches.  The scene does not own it. */
EXTERN_C int risltc_scene_set_model(risltc_scene_t* scene, risltc_model_t* model);
/* The model's logits for every pixel of the G-buffer (device pointers;
   logits: width * height * cluster_count floats, pixel-major), stream-ordered. */
EXTERN_C int risltc_model_logits(risltc_ctx_t* ctx, const risltc_model_t* model, const risltc_gbuffer_t* gbuffer,
                                 float* logits);

/* A G-buffer producer for the synthetic heightfield scenes (the role of the
   reference's visibility pass and get_shading_data,
   shading_pass.frag.glsl:571-672, which rasterise meshes): a pinhole camera
   at `camera` looking at the origin (z up, vertical field of view fov_y in
   radians) sees the surface z = sum_w amplitude sin(fx x + fy y + phase);
   per pixel the first crossing (10 steps across the height band, then 12
   bisections), the gradient normal adapted into the view hemisphere, and a
   material hashed from (pixel, material_seed): roughness and per-channel
   albedo uniform in their ranges, F0 = fresnel_0.  planes: 17 x width x
   height floats and primitive: width x height (0 hit, 0xFFFFFFFF miss),
   device memory, stream-ordered. */
#define RISLTC_MAX_WAVES 16
typedef struct risltc_heightfield_s {
	float camera[3];
	float fov_y;
	uint32_t wave_count;
	float waves[RISLTC_MAX_WAVES][4];
	uint32_t material_seed;
	float roughness_min, roughness_max;
	float albedo_min, albedo_max;
	float fresnel_0;
} risltc_heightfield_t;
EXTERN_C int risltc_gbuffer_heightfield(risltc_ctx_t* ctx, const risltc_heightfield_t* heightfield, uint32_t width,
                                        uint32_t height, float* planes, uint32_t* primitive);

/* Uploads lights (the std140 buffer of risltc_write_lights), the LTC table
   and, if triangle_count > 0, builds and uploads the BVH of the occluders
   (9 floats per triangle; fewer than 2^28 triangles and 2^22 lights, else
   RISLTC_ERROR_TOO_LARGE; all finite, else RISLTC_ERROR_NON_FINITE).  All
   inputs are host memory. */
EXTERN_C int risltc_scene_create(risltc_ctx_t* ctx, const float* lights_std140, uint32_t light_count,
                                 uint32_t max_vertex_count, const risltc_ltc_table_t* ltc, const float* triangles,
                                 uint32_t triangle_count, risltc_scene_t** scene);
EXTERN_C void risltc_scene_destroy(risltc_scene_t* scene);

/* Sizes the context's scratch for frames of width x height pixels and
 * frame_count frames per call: 16 bytes per pixel and frame of reservoir
 * records between the candidate and shading kernels (used by the default
 * configuration: LTC-CP, light_reservoir, one light sample).  risltc_shade
 * grows the scratch itself when needed (device allocations: these records,
 * the candidate kernel's p_hat slots and, with shadow rays, the ray queue,
 * whose per-light counters depend on the scene) and configures each kernel
 * on its first launch.  After one call, later calls that need no more
 * scratch (no more pixels, frames, lights, candidates or clusters) make no
 * allocation and no configuration call; a default-configuration call made
 * after one such call can be captured into a CUDA graph. */
EXTERN_C int risltc_ctx_reserve(risltc_ctx_t* ctx, uint32_t width, uint32_t height, uint32_t frame_count);

/* Shades frame_count consecutive frames of the G-buffer (device pointers).
 * Frame f uses the noise constants of set_noise_constants(..., noise,
 * animate) called once per frame (noise->random_seed advances by
 * frame_count).  out_rgb (device, width*height*3 floats, may be NULL) gets the
 * mean over the frames; accum (device, width*height*3 doubles, may be NULL)
 * gets the per-frame results added in FP64; reservoirs (device, may be NULL)
 * gets the first frame's reservoir per pixel.  Stream-ordered; returns
 * RISLTC_ERROR_TRAVERSAL_LIMIT etc. only through risltc_ctx_check(). */
EXTERN_C int risltc_shade(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                          const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                          uint32_t frame_count, float* out_rgb, double* accum, risltc_reservoir_t* reservoirs);

/* One item of risltc_shade_batch: the arguments of one risltc_shade call. */
typedef struct risltc_batch_item_s {
	const risltc_scene_t* scene;
	risltc_gbuffer_t gbuffer;
	risltc_settings_t settings;
	noise_table_t* noise;
	uint32_t animate, frame_count;
	float* out_rgb;
	double* accum;
	risltc_reservoir_t* reservoirs;
} risltc_batch_item_t;

/* Streams the items of risltc_shade_batch run on, forked from the context's
   stream. */
#define RISLTC_BATCH_STREAMS 8

/* Shades several G-buffers (each with its own scene, settings and noise) in
 * one call; no counterpart in the reference, which draws one view at a time.
 * Each item gets its own share of the context's scratch.  When every item
 * uses the default configuration (LTC-CP, light_reservoir, one light sample
 * and one sample per technique, uniform candidates, shadows on a scene with
 * occluders) with the same numerics and a binned tile shape, the batch runs
 * as one launch per phase for all items (candidate, sample, ray grouping,
 * trace and resolve kernels over the items' concatenated work, in groups of
 * 16 items) on the context's stream; otherwise each item runs its own
 * kernels on one of RISLTC_BATCH_STREAMS streams forked from the context's
 * stream and joined back to it.  Either way small frames fill the GPU
 * together and the results equal the items' risltc_shade calls bit for bit.
 * All items are validated before any work; noise->random_seed of each item
 * advances by its frame_count.  The first call grows the scratch (and creates
 * the streams where needed); later calls with no larger items allocate
 * nothing, so a batch can be captured into one CUDA graph. */
EXTERN_C int risltc_shade_batch(risltc_ctx_t* ctx, const risltc_batch_item_t* items, uint32_t item_count);

/* Autotuner of the candidate kernel's tile shape: for every risltc_tile_t,
 * one untimed and `repeats` timed runs of the shading call that `settings`
 * describes (risltc_shade with these arguments, outputs discarded; the
 * noise seed is not advanced), timing the candidate kernel with CUDA events
 * on the context's stream.  Sets settings->tile to the fastest shape and, if
 * ms_per_tile is not NULL, stores each shape's mean time per call
 * (risltc_tile_count floats; settings that do not use the candidate kernel
 * leave settings->tile unchanged and store zeros).  Synchronises the
 * context's stream. */
EXTERN_C int risltc_autotune(risltc_ctx_t* ctx, const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                             risltc_settings_t* settings, const noise_table_t* noise, uint32_t frame_count,
                             uint32_t repeats, float* ms_per_tile);

/* The same for a batch: every shape is timed on the whole risltc_shade_batch
 * call (CUDA events on the context's stream around the fork and join), the
 * fastest is written to every item's settings.tile, and the items' noise
 * seeds are restored.  Synchronises the context's stream. */
EXTERN_C int risltc_autotune_batch(risltc_ctx_t* ctx, risltc_batch_item_t* items, uint32_t item_count,
                                   uint32_t repeats, float* ms_per_tile);

/* Same with host buffers: copies the G-buffer planes in, shades, copies
 * out_rgb back, synchronises and reports device errors.  This is the call a
 * host program makes per frame. */
EXTERN_C int risltc_shade_host(risltc_ctx_t* ctx, const risltc_scene_t* scene, uint32_t width, uint32_t height,
                               const float* gbuffer_planes, const uint32_t* primitive,
                               const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                               uint32_t frame_count, float* out_rgb);

/* Allocation-free shading, for callers that may not allocate device memory
 * while they render: a plugin inside a host application that owns the device
 * memory budget (a game engine or content-creation tool with its own
 * allocator), or a frame loop that must not stall other streams (cudaMalloc
 * and cudaFree synchronise the device).  Such a caller creates the scene once,
 * where allocation is allowed, and shades each frame here.  No counterpart in
 * the reference, which renders through Vulkan.
 *
 * Same arguments and results as risltc_shade for the default configuration
 * (LTC-CP technique, light_reservoir, one light sample; other settings return
 * RISLTC_ERROR_UNSUPPORTED), on the given CUDA stream (NULL: the legacy
 * default stream) of the current device, but without a context: the
 * reservoir records between the two kernels and the error word live in a
 * static device array of RISLTC_NOALLOC_MAX_PIXEL_FRAMES records (4 MiB),
 * which every GPU that loads the library holds until the process exits.
 * width * height * frame_count above that limit returns
 * RISLTC_ERROR_TOO_LARGE before any work.  The call waits for its stream to
 * finish and returns the kernels' error status.  The scene must have been
 * created on the current device; a scene of another device returns
 * RISLTC_ERROR_INVALID_ARGUMENT before any work.  The first call on each
 * device resolves the array's device address (cudaGetSymbolAddress) and keeps
 * it for the life of the process; make no call on a device after resetting
 * it (cudaDeviceReset).  All calls share the array: calls that overlap on the
 * GPU (other streams, other threads) race, so serialise them. */
#define RISLTC_NOALLOC_MAX_PIXEL_FRAMES 262144
EXTERN_C int risltc_shade_noalloc(const risltc_scene_t* scene, const risltc_gbuffer_t* gbuffer,
                                  const risltc_settings_t* settings, noise_table_t* noise, uint32_t animate,
                                  uint32_t frame_count, float* out_rgb, double* accum,
                                  risltc_reservoir_t* reservoirs, void* stream);

/* Any-hit shadow queries through the scene BVH: rays are 8 floats
   {origin xyz, t_min, direction xyz, t_max} in device memory; hits gets
   1 (occluded) or 0 per ray. */
EXTERN_C int risltc_trace_shadow(risltc_ctx_t* ctx, const risltc_scene_t* scene, const float* rays, uint32_t ray_count,
                                 uint32_t* hits);

/* Kernel timing with CUDA events on the context's stream.  Returns the time
 * of the shading calls made since the previous call of this function (at
 * most 64 calls are timed), split into RISLTC_PROFILE_PHASES phases:
 * phase_ms[0] the RIS candidate kernel (or the fused kernel), phase_ms[1] the
 * shading kernel (with its shadow rays, or up to queueing them), phase_ms[2]
 * the grouping of the shadow rays by light (bucket scan and scatter),
 * phase_ms[3] the shadow-ray traversal kernel and phase_ms[4] the resolve
 * kernel (0 where a phase is not a kernel of its own), and their number in
 * calls; then enables (enable != 0) or disables timing of the following
 * calls.  phase_ms and calls may be NULL.  Querying synchronises the
 * stream. */
#define RISLTC_PROFILE_PHASES 5
EXTERN_C int risltc_ctx_profile(risltc_ctx_t* ctx, int enable, float* phase_ms, uint32_t* calls);

/* The number of this library's own kernels launched through the context
 * since it was created (shading, proposal, training and query kernels;
 * memory copies and sets excluded). */
EXTERN_C int risltc_ctx_launch_count(const risltc_ctx_t* ctx, uint64_t* launches);

/* The shadow rays that the last risltc_shade call on the context traced
 * through its ray queue (the default configuration with shadows on: rays
 * grouped by light, then traced by the persistent kernel); 0 when that call
 * traced none that way.  Waits for the context's stream.  No counterpart in
 * the reference, whose ray queries run inside the fragment shader; the
 * shadow-ray rate of the benchmark (rays per second) comes from it. */
EXTERN_C int risltc_ctx_ray_count(risltc_ctx_t* ctx, uint32_t* rays);

/* Synchronises the context's stream and returns the first error recorded by
   a kernel since the last check (RISLTC_OK if none). */
EXTERN_C int risltc_ctx_check(risltc_ctx_t* ctx);

/* Fault injection for tests of the failure paths, made on the host: with
   RISLTC_FAULT_TENSOR_WAIT the next learned-proposal logits launch issues no
   tensor-core products, so its bounded waits (one second each) run out, the
   kernel records the timeout, frees its tensor memory and returns, and the
   next risltc_ctx_check reports RISLTC_ERROR_DEVICE_TIMEOUT; the context stays
   usable.  Nothing faults, traps or hangs. */
#define RISLTC_FAULT_TENSOR_WAIT 1u
/* The same for the next tensor-core training launch. */
#define RISLTC_FAULT_TRAIN_TENSOR_WAIT 2u
EXTERN_C int risltc_ctx_inject_fault(risltc_ctx_t* ctx, uint32_t faults);
EXTERN_C const char* risltc_status_string(int status);

#endif /* RISLTC_H */
