/* Binary BVH over occluder triangles, built on the host with a binned SAH
 * over references made by early split clipping (below).
 *
 * Replaces the driver-built acceleration structure of the reference
 * (create_acceleration_structure, src/scene.c:142-400: one BLAS over all
 * triangles, opaque, no culling, PREFER_FAST_TRACE).  Layout: see risltc.h.
 * Children of an interior node are stored next to each other, so a node needs
 * one index; leaves reference a contiguous range of the reordered triangles.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "../../../include/risltc.h"

#define BVH_BINS 16
#define BVH_MAX_DEPTH 60
/* Early split clipping: references per triangle at most, box area (against
   the mean triangle box) above which a reference is cut, and the references
   at most, as a multiple of the triangles. */
#define BVH_SPLIT_PIECES 8
#define BVH_SPLIT_AREA 0.5f
#define BVH_SPLIT_BUDGET 3u
#define BVH_MAX_REFERENCES ((1u << 28) - 1u) /* leaf references keep 28 bits for the first index */

typedef struct {
	float lo[3], hi[3];
} box_t;

static void box_empty(box_t* b) {
	for (int a = 0; a != 3; ++a) {
		b->lo[a] = FLT_MAX;
		b->hi[a] = -FLT_MAX;
	}
}
static void box_grow_point(box_t* b, const float* p) {
	for (int a = 0; a != 3; ++a) {
		if (p[a] < b->lo[a]) b->lo[a] = p[a];
		if (p[a] > b->hi[a]) b->hi[a] = p[a];
	}
}
static void box_grow_box(box_t* b, const box_t* o) {
	for (int a = 0; a != 3; ++a) {
		if (o->lo[a] < b->lo[a]) b->lo[a] = o->lo[a];
		if (o->hi[a] > b->hi[a]) b->hi[a] = o->hi[a];
	}
}
static float box_area(const box_t* b) {
	float d[3];
	for (int a = 0; a != 3; ++a) d[a] = b->hi[a] > b->lo[a] ? b->hi[a] - b->lo[a] : 0.0f;
	return 2.0f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
}

typedef struct {
	uint32_t node, begin, end, depth;
} task_t;

/* Early split clipping (Ernst and Greiner, "Early split clipping for bounding
   volume hierarchies", 2007): a triangle whose box area is more than
   BVH_SPLIT_AREA times the mean is cut at the middle of its largest piece's
   longest box axis (the piece, a convex polygon, clipped against the plane
   on both sides) until every piece's box is small enough, it has
   BVH_SPLIT_PIECES pieces, or `room` references are used.  Each piece is a
   reference to the whole triangle with the piece's box.  The pieces cover the
   triangle, so a ray that hits it passes through one piece's box, reaches
   that leaf and tests the triangle: any-hit answers do not change (the node
   boxes' widening covers the rounding of the cut points).  Returns the
   number of references written. */
static uint32_t split_triangle(const float* tri, const box_t* box, float limit, uint32_t room, uint32_t id,
                               box_t* ref_box, uint32_t* ref_tri) {
	enum { kMaxVertices = 3 + BVH_SPLIT_PIECES };
	float poly[BVH_SPLIT_PIECES][kMaxVertices][3];
	int vertices[BVH_SPLIT_PIECES];
	box_t pbox[BVH_SPLIT_PIECES];
	uint32_t pieces = 1;
	for (int v = 0; v != 3; ++v)
		for (int a = 0; a != 3; ++a) poly[0][v][a] = tri[3 * v + a];
	vertices[0] = 3;
	pbox[0] = *box;
	if (room > BVH_SPLIT_PIECES) room = BVH_SPLIT_PIECES;
	while (pieces < room) {
		int k = -1;
		float largest = limit;
		for (uint32_t j = 0; j != pieces; ++j)
			if (box_area(&pbox[j]) > largest) {
				largest = box_area(&pbox[j]);
				k = (int) j;
			}
		if (k < 0) break;
		int ax = 0;
		for (int a = 1; a != 3; ++a)
			if (pbox[k].hi[a] - pbox[k].lo[a] > pbox[k].hi[ax] - pbox[k].lo[ax]) ax = a;
		const float mid = 0.5f * (pbox[k].lo[ax] + pbox[k].hi[ax]);
		float lo_side[kMaxVertices][3], hi_side[kMaxVertices][3];
		int nl = 0, nh = 0;
		const int n = vertices[k];
		for (int v = 0; v != n; ++v) {
			const float* p = poly[k][v];
			const float* q = poly[k][(v + 1) % n];
			const int p_lo = p[ax] <= mid, q_lo = q[ax] <= mid;
			if (p_lo)
				memcpy(lo_side[nl++], p, sizeof(float) * 3);
			else
				memcpy(hi_side[nh++], p, sizeof(float) * 3);
			if (p_lo != q_lo) {
				/* The edge crosses the plane: the cut point goes to both sides. */
				const float t = (mid - p[ax]) / (q[ax] - p[ax]);
				float x[3];
				for (int a = 0; a != 3; ++a) x[a] = p[a] + t * (q[a] - p[a]);
				x[ax] = mid;
				memcpy(lo_side[nl++], x, sizeof(x));
				memcpy(hi_side[nh++], x, sizeof(x));
			}
		}
		if (nl < 3 || nh < 3) break; /* the plane does not cut this piece */
		memcpy(poly[k], lo_side, sizeof(float) * 3 * (size_t) nl);
		memcpy(poly[pieces], hi_side, sizeof(float) * 3 * (size_t) nh);
		vertices[k] = nl;
		vertices[pieces] = nh;
		box_empty(&pbox[k]);
		for (int v = 0; v != nl; ++v) box_grow_point(&pbox[k], lo_side[v]);
		box_empty(&pbox[pieces]);
		for (int v = 0; v != nh; ++v) box_grow_point(&pbox[pieces], hi_side[v]);
		++pieces;
	}
	for (uint32_t j = 0; j != pieces; ++j) {
		ref_box[j] = pbox[j];
		ref_tri[j] = id;
	}
	return pieces;
}

int risltc_bvh_build(risltc_bvh_t* bvh, const float* tris, uint32_t count, uint32_t max_leaf_size) {
	if (!bvh || (!tris && count)) return RISLTC_ERROR_INVALID_ARGUMENT;
	memset(bvh, 0, sizeof(*bvh));
	if (count == 0) return RISLTC_OK;
	if (max_leaf_size < 1) max_leaf_size = 4;
	if (count > BVH_MAX_REFERENCES) return RISLTC_ERROR_INVALID_ARGUMENT;
	const uint32_t triangle_count = count;
	uint32_t room = count <= BVH_MAX_REFERENCES / BVH_SPLIT_BUDGET ? count * BVH_SPLIT_BUDGET : BVH_MAX_REFERENCES;
	box_t* tri_box = (box_t*) malloc(sizeof(box_t) * count);
	box_t* boxes = (box_t*) malloc(sizeof(box_t) * room);
	uint32_t* ref_tri = (uint32_t*) malloc(sizeof(uint32_t) * room);
	if (!tri_box || !boxes || !ref_tri) {
		free(tri_box);
		free(boxes);
		free(ref_tri);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	double mean_area = 0.0;
	for (uint32_t i = 0; i != count; ++i) {
		box_empty(&tri_box[i]);
		for (int v = 0; v != 3; ++v) box_grow_point(&tri_box[i], tris + 9 * (size_t) i + 3 * v);
		mean_area += box_area(&tri_box[i]);
	}
	const float limit = (float) (BVH_SPLIT_AREA * mean_area / count);
	count = 0;
	for (uint32_t i = 0; i != triangle_count; ++i) {
		/* Leave one reference for each triangle still to come. */
		const uint32_t left = room - count - (triangle_count - 1 - i);
		count += split_triangle(tris + 9 * (size_t) i, &tri_box[i], limit, left, i, boxes + count, ref_tri + count);
	}
	free(tri_box);
	/* The references (box, centroid, triangle) are reordered in place as the
	   build partitions them, so every pass over a node's range reads them in
	   sequence. */
	float* centroid = (float*) malloc(sizeof(float) * 3 * count);
	uint32_t capacity = 2 * count;
	float* nodes = (float*) malloc(sizeof(float) * 8 * (size_t) capacity);
	task_t* stack = (task_t*) malloc(sizeof(task_t) * (BVH_MAX_DEPTH + 4) * 2);
	if (!centroid || !nodes || !stack) {
		free(boxes);
		free(ref_tri);
		free(centroid);
		free(nodes);
		free(stack);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	for (uint32_t i = 0; i != count; ++i)
		for (int a = 0; a != 3; ++a) centroid[3 * i + a] = 0.5f * (boxes[i].lo[a] + boxes[i].hi[a]);
	uint32_t node_count = 1, max_depth = 0;
	int sp = 0;
	stack[sp++] = (task_t){0, 0, count, 0};
	while (sp) {
		task_t t = stack[--sp];
		if (t.depth > max_depth) max_depth = t.depth;
		box_t bounds, cbounds;
		box_empty(&bounds);
		box_empty(&cbounds);
		for (uint32_t i = t.begin; i != t.end; ++i) {
			box_grow_box(&bounds, &boxes[i]);
			box_grow_point(&cbounds, centroid + 3 * (size_t) i);
		}
		float* node = nodes + 8 * (size_t) t.node;
		/* Widen by a relative 1e-6 so traversal is conservative. */
		for (int a = 0; a != 3; ++a) {
			float ext = bounds.hi[a] - bounds.lo[a];
			float pad_lo = 1e-6f * (fabsf(bounds.lo[a]) + ext) + 1e-30f;
			float pad_hi = 1e-6f * (fabsf(bounds.hi[a]) + ext) + 1e-30f;
			node[a] = bounds.lo[a] - pad_lo;
			node[4 + a] = bounds.hi[a] + pad_hi;
		}
		uint32_t n = t.end - t.begin;
		int split_axis = -1, sah_leaf = 0;
		uint32_t split_bin = 0;
		if (n > max_leaf_size && t.depth < BVH_MAX_DEPTH) {
			float best = FLT_MAX;
			for (int a = 0; a != 3; ++a) {
				float lo = cbounds.lo[a], hi = cbounds.hi[a];
				if (!(hi > lo)) continue;
				float scale = (float) BVH_BINS / (hi - lo);
				box_t bin_box[BVH_BINS];
				uint32_t bin_count[BVH_BINS];
				for (int b = 0; b != BVH_BINS; ++b) {
					box_empty(&bin_box[b]);
					bin_count[b] = 0;
				}
				for (uint32_t i = t.begin; i != t.end; ++i) {
					int b = (int) ((centroid[3 * (size_t) i + a] - lo) * scale);
					b = b < 0 ? 0 : (b >= BVH_BINS ? BVH_BINS - 1 : b);
					bin_count[b]++;
					box_grow_box(&bin_box[b], &boxes[i]);
				}
				float right_area[BVH_BINS];
				uint32_t right_count[BVH_BINS];
				box_t acc;
				box_empty(&acc);
				uint32_t c = 0;
				for (int b = BVH_BINS - 1; b > 0; --b) {
					box_grow_box(&acc, &bin_box[b]);
					c += bin_count[b];
					right_area[b] = box_area(&acc);
					right_count[b] = c;
				}
				box_empty(&acc);
				c = 0;
				for (int b = 0; b < BVH_BINS - 1; ++b) {
					box_grow_box(&acc, &bin_box[b]);
					c += bin_count[b];
					if (c == 0 || right_count[b + 1] == 0) continue;
					float cost = box_area(&acc) * (float) c + right_area[b + 1] * (float) right_count[b + 1];
					if (cost < best) {
						best = cost;
						split_axis = a;
						split_bin = (uint32_t) b;
					}
				}
			}
			/* Leaf if splitting does not beat intersecting everything (with
			   traversal cost 1 relative to a triangle test), unless too big. */
			float leaf_cost = box_area(&bounds) * (float) n;
			if (split_axis >= 0 && best + box_area(&bounds) >= leaf_cost && n <= 4 * max_leaf_size) {
				split_axis = -1;
				sah_leaf = 1;
			}
		}
		uint32_t mid = t.begin;
		if (split_axis >= 0) {
			float lo = cbounds.lo[split_axis], hi = cbounds.hi[split_axis];
			float scale = (float) BVH_BINS / (hi - lo);
			uint32_t i = t.begin, j = t.end;
			while (i < j) {
				int b = (int) ((centroid[3 * (size_t) i + split_axis] - lo) * scale);
				b = b < 0 ? 0 : (b >= BVH_BINS ? BVH_BINS - 1 : b);
				if ((uint32_t) b <= split_bin) {
					++i;
				} else {
					--j;
					const box_t box = boxes[i];
					boxes[i] = boxes[j];
					boxes[j] = box;
					for (int a = 0; a != 3; ++a) {
						const float c = centroid[3 * (size_t) i + a];
						centroid[3 * (size_t) i + a] = centroid[3 * (size_t) j + a];
						centroid[3 * (size_t) j + a] = c;
					}
					const uint32_t tri = ref_tri[i];
					ref_tri[i] = ref_tri[j];
					ref_tri[j] = tri;
				}
			}
			mid = i;
			if (mid == t.begin || mid == t.end) split_axis = -1;
		}
		if (split_axis < 0 && !sah_leaf && n > max_leaf_size && t.depth < BVH_MAX_DEPTH) {
			/* Degenerate centroids: split by position in the list. */
			mid = t.begin + n / 2;
			split_axis = 3;
		}
		int32_t first, leaf_count;
		if (split_axis < 0) {
			first = (int32_t) t.begin;
			leaf_count = (int32_t) n;
		} else {
			uint32_t left = node_count;
			node_count += 2;
			first = (int32_t) left;
			leaf_count = 0;
			stack[sp++] = (task_t){left + 1, mid, t.end, t.depth + 1};
			stack[sp++] = (task_t){left, t.begin, mid, t.depth + 1};
		}
		memcpy(node + 3, &first, 4);
		memcpy(node + 7, &leaf_count, 4);
	}
	float* shrunk = (float*) realloc(nodes, sizeof(float) * 8 * node_count);
	bvh->nodes = shrunk ? shrunk : nodes;
	bvh->node_count = node_count;
	bvh->depth = max_depth;
	bvh->triangle_count = count;
	uint32_t* ids = (uint32_t*) realloc(ref_tri, sizeof(uint32_t) * count);
	bvh->triangle_ids = ids ? ids : ref_tri;
	bvh->triangles = (float*) malloc(sizeof(float) * 12 * (size_t) count);
	if (!bvh->triangles) {
		free(boxes);
		free(centroid);
		free(stack);
		risltc_bvh_destroy(bvh);
		return RISLTC_ERROR_OUT_OF_MEMORY;
	}
	for (uint32_t i = 0; i != count; ++i) {
		const float* t = tris + 9 * (size_t) bvh->triangle_ids[i];
		float* o = bvh->triangles + 12 * (size_t) i;
		for (int a = 0; a != 3; ++a) {
			o[a] = t[a];
			o[4 + a] = t[3 + a] - t[a];
			o[8 + a] = t[6 + a] - t[a];
		}
		o[3] = o[7] = o[11] = 0.0f;
	}
	free(boxes);
	free(centroid);
	free(stack);
	return RISLTC_OK;
}

void risltc_bvh_destroy(risltc_bvh_t* bvh) {
	if (!bvh) return;
	free(bvh->nodes);
	free(bvh->triangles);
	free(bvh->triangle_ids);
	memset(bvh, 0, sizeof(*bvh));
}
