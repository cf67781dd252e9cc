/* oracle.h - interface of the CPU restatement of risltc's shading path.
 *
 * TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg use this library, as the checker.  The product never
 * links it.
 *
 * Data layouts are the ones the reference's shader consumes:
 *  - lights: the std140 light buffer of write_lights (main.c:456-490), 12 +
 *    4 * max_light_vertex_count floats per light (surface_radiance, pad,
 *    plane, vertex_count as uint32, pad x3, vertices_world_space with a pad
 *    float each).  Slots past vertex_count hold copies of vertex 0;
 *  - LTC tables: the two texture arrays of ltc_table.h:41-57 as FP32,
 *    [layer][height][width][4] and [layer][height][width][2];
 *  - G-buffer: 17 planes of width*height floats (shading_data_t of
 *    brdfs.glsl:22-39: position xyz, normal xyz, outgoing xyz,
 *    lambert_outgoing, diffuse_albedo rgb, fresnel_0 rgb, roughness);
 *  - occluders: 12 floats per triangle (v0, pad, v1 - v0, pad, v2 - v0, pad)
 *    and an optional binary BVH (8 words per node: bmin xyz,
 *    left_or_first, bmax xyz, count).
 */
#ifndef RISLTC_ORACLE_H
#define RISLTC_ORACLE_H
#include <stddef.h>
#include <stdint.h>

/* Values of sample_polygon_technique_t (polygonal_light.h:31-46),
   mis_heuristic_t (main.h:59-77) and light_sampling_strategies_t
   (main.h:79-84). */
enum {
	ORACLE_TECHNIQUE_BASELINE = 0,
	ORACLE_TECHNIQUE_AREA_TURK = 1,
	ORACLE_TECHNIQUE_PSA = 2,
	ORACLE_TECHNIQUE_PSA_BIASED = 3,
	ORACLE_TECHNIQUE_LTC_CP = 4
};
enum { ORACLE_MIS_BALANCE = 0, ORACLE_MIS_POWER, ORACLE_MIS_WEIGHTED, ORACLE_MIS_OPTIMAL_CLAMPED, ORACLE_MIS_OPTIMAL };
enum { ORACLE_LIGHT_UNIFORM = 0, ORACLE_LIGHT_RESERVOIR = 1 };

typedef struct oracle_scene_s {
	const float* lights;
	int32_t light_count;
	int32_t max_light_vertex_count;
	const float* ltc0;
	const float* ltc1;
	int32_t ltc_width, ltc_height, ltc_layers;
	float ltc_constants[6]; /* ltc_constants_t order, ltc_table.h:23-35 */
	const float* triangles;
	int32_t triangle_count;
	const float* bvh_nodes; /* NULL: brute-force shadow queries */
	int32_t bvh_node_count;
	/* Light clusters for the cluster proposal (lights listed cluster by
	   cluster): offsets (count + 1), each light's cluster, each cluster's
	   bounding sphere (centre xyz, radius) and power. */
	const uint32_t* cluster_offsets;
	const uint32_t* light_cluster;
	const float* cluster_bounds;
	const float* cluster_power;
	int32_t cluster_count;
} oracle_scene_t;

typedef struct oracle_settings_s {
	int32_t polygon_sampling_technique;
	int32_t light_sampling;
	int32_t mis_heuristic;
	int32_t candidate_count;
	int32_t sample_count;
	int32_t light_samples;
	float mis_visibility_estimate;
	int32_t fast_atan;
	/* 1: reproduce the reference's calculate_ltc over all array slots and its
	   8-vertex clip aliasing (for pinning against the reference itself). */
	int32_t reference_slots;
	/* 1: RIS candidates from the cluster proposal (risltc_proposal_clusters)
	   with the given uniform fraction and the frame's second noise number. */
	int32_t proposal;
	float proposal_uniform_fraction;
	uint32_t random_number_proposal;
} oracle_settings_t;

typedef struct oracle_gbuffer_s {
	int32_t width, height;
	const float* planes;
	const uint32_t* primitive; /* NULL: every pixel is covered */
} oracle_gbuffer_t;

typedef struct oracle_reservoir_s {
	int32_t light_index;
	int32_t pad;
	double w_sum;
	double sample_value;
} oracle_reservoir_t;

#ifdef __cplusplus
extern "C" {
#endif
int oracle_render_f32(const oracle_scene_t*, const oracle_settings_t*, const oracle_gbuffer_t*, uint32_t random_number_x,
                      int row_begin, int row_end, float* out_rgb, oracle_reservoir_t* out_reservoirs);
int oracle_render_pixels_f32(const oracle_scene_t*, const oracle_settings_t*, const oracle_gbuffer_t*,
                             uint32_t random_number_x, const uint32_t* pixels, size_t begin, size_t end, float* out_rgb,
                             oracle_reservoir_t* out_reservoirs);
int oracle_render_f64(const oracle_scene_t*, const oracle_settings_t*, const oracle_gbuffer_t*, uint32_t random_number_x,
                      int row_begin, int row_end, double* out_rgb, oracle_reservoir_t* out_reservoirs);
#ifdef __cplusplus
}
#endif
#endif
