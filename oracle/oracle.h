/* CPU oracle for the ray-query hot path — TEST INFRASTRUCTURE ONLY.
 *
 * A restatement, in plain C++17, of the reference ray tracer's acceleration
 * structures and ray queries (Alhajras/Raytracer-Data-structures,
 * project/raytracer/accelerators.h and main.cpp), plus the documented
 * restatements of the parts the reference leaves unfinished (Karras LBVH
 * topology and refit, Moller-Trumbore triangles, any-hit shadow queries).
 * Every function cites the reference lines it follows.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library.  The engine never links or calls it.
 *
 * Pinning: tests/test_oracle_golden.py checks this oracle against vectors
 * produced by the reference's own code (tests/golden/, generated by
 * tests/golden/make_golden.py through oracle/ref_dump.cpp).
 *
 * Data layouts are the engine's (include/rq.h) so that the oracle can check
 * the engine's exported structures directly:
 *   ray  : {org[3], tmin, dir[3], tmax}           32 B
 *   hit  : {t, prim, u, v}                         16 B, prim = 0xFFFFFFFF on miss
 *   BVH2 : n_internal nodes of 16 words
 *          [lx0 lx1 ly0 ly1 | rx0 rx1 ry0 ry1 | lz0 lz1 rz0 rz1 | left right nl nr]
 *          (l/r = child boxes, *0 = min, *1 = max).  A child c >= 0 is an
 *          internal node; c < 0 is a leaf holding slots [~c, ~c + n).
 *          order[slot] = primitive id.  With n_internal == 0 the root is one
 *          leaf holding every slot.
 *   KD   : the reference's 12-byte KdAccelNode words, depth-first order
 *          (accelerators.h:715-761).
 */
#ifndef RQ_ORACLE_H
#define RQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float org[3]; float tmin; float dir[3]; float tmax; } orc_ray_t;
typedef struct { float t; uint32_t prim; float u; float v; } orc_hit_t;

enum { ORC_TRIANGLES = 0, ORC_SPHERES = 1 };
enum { ORC_MODE_FAST = 0, ORC_MODE_REFERENCE = 1 };
enum { ORC_CLOSEST = 0, ORC_ANY = 1 };

/* ---- Morton codes (accelerators.h:374-394, 575-580) ---- */
uint32_t orc_expand_bits(uint32_t v);
uint32_t orc_morton3d(float x, float y, float z);
void orc_morton_spheres_ref(const float* sph, uint32_t n, uint32_t* codes);
void orc_morton_centroids(const float* centroids, uint32_t n, const float* lo, const float* hi,
                          uint32_t* codes);
/* The engine's cube normalisation (one scale, the largest extent). */
void orc_morton_centroids_cube(const float* centroids, uint32_t n, const float* lo, const float* hi,
                               uint32_t* codes);

/* ---- primitive preparation (engine definitions) ---- */
void orc_tri_prims(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt,
                   float* prims9, float* aabb6, float* centroid3);
void orc_sphere_prims(const float* sph, uint32_t n, float* aabb6, float* centroid3);
void orc_bounds3(const float* pts, uint32_t n, uint32_t stride, float* lo, float* hi);

/* ---- LBVH: stable sort, Karras topology, bottom-up refit ---- */
void orc_sort_pairs(const uint32_t* keys, uint32_t n, uint32_t* out_keys, uint32_t* out_vals);
void orc_karras(const uint32_t* sorted_codes, uint32_t n, int32_t* left, int32_t* right,
                int32_t* parent);
void orc_refit(uint32_t n, const int32_t* left, const int32_t* right, const float* slot_aabb6,
               float* nodes16, float* root_bounds6);
int orc_build_lbvh(const uint32_t* codes, const float* aabb6, uint32_t n, float* nodes16,
                   uint32_t* order, uint32_t* sorted_codes, float* root_bounds6);
/* The engine's RQ_LBVH_TREELETS pass (csrc/treelet.cu), in place on the 16-word
 * nodes of an LBVH with one primitive per leaf: post-order over the tree, at
 * each internal node the treelet of up to four leaves grown from it (largest
 * half area first, first of equals) is rebuilt with the topology of least sum
 * of internal half areas (dynamic program over leaf subsets, first minimum in
 * the engine's enumeration order), reusing the treelet's nodes (the root
 * first, then in expansion order, assigned to the chosen subsets in
 * decreasing subset order).  Nodes of more than 2048 leaves are left as they
 * are when there are more than 2048 of them (the engine's top-node block
 * capacity).  No reference counterpart. */
void orc_treelet_opt(float* nodes16, uint32_t n_internal);

/* ---- median BVH (constructBVHNew, accelerators.h:246-337) ---- */
/* compat = 0: the engine's deterministic rule; 1: replay of the reference's
 * std::partition / std::nth_element sequence.  Returns 1 if cap_order is too
 * small (n_slots tells the size), 2 if the reference would recurse forever. */
int orc_build_median(const float* aabb6, const float* centroid3, uint32_t n, int compat,
                     float* nodes16, uint32_t* order, uint32_t cap_order, uint32_t* n_slots,
                     uint32_t* n_internal, float* root_bounds6);

/* ---- KD tree (constructKDTreeNew / buildTree, accelerators.h:815-988) ---- */
int orc_kd_max_depth(uint32_t n);
int orc_build_kd(const float* aabb6, uint32_t n, int32_t max_depth, int32_t* nodes3,
                 uint32_t cap_nodes, uint32_t* n_nodes, int32_t* prim_idx, uint32_t cap_idx,
                 uint32_t* n_idx, float* root_bounds6);

/* ---- ray queries ---- */
/* FAST closest hit: the smallest t in (tmin, tmax) and, among primitives hit
 * at exactly that t, the smallest primitive id (independent of traversal
 * order).  REFERENCE: the reference's first closest in candidate order. */
/* prims: triangles = 9 floats per primitive id (v0, e1 = v1-v0, e2 = v2-v0);
 * spheres = 4 floats per primitive id (centre, radius).
 * counters (may be NULL): [0] += internal nodes visited, [1] += primitive tests. */
int orc_trace_bvh2(int kind, int mode, int query, const float* nodes16, uint32_t n_internal,
                   const float* root_bounds6, uint32_t n_prims, const uint32_t* order,
                   const float* prims, const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits,
                   uint8_t* occluded, uint64_t* counters, int nthreads);
/* boxIntersect's candidate lists (accelerators.h:668-690): counts[r] per ray,
 * the ids concatenated in ray order into ids (up to cap entries; may be
 * NULL).  Returns the total. */
uint64_t orc_candidates_bvh2(const float* nodes16, uint32_t n_internal, const float* root_bounds6, uint32_t n_prims,
                             const uint32_t* order, const orc_ray_t* rays, uint32_t nrays, uint32_t* counts,
                             uint32_t* ids, uint64_t cap);
int orc_trace_kd(int kind, int mode, int query, const int32_t* nodes3, uint32_t n_nodes,
                 const int32_t* prim_idx, const float* root_bounds6, const float* prims,
                 const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits, uint8_t* occluded,
                 uint64_t* counters, int nthreads);
/* Collapsed 4-wide BVH (the engine's node-width option).  Node = 32 words
 * [lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4] link[4] count[4]], made
 * from a BVH2 by merging every internal node at even depth with its internal
 * children; children in the order left.left, left.right, right.left,
 * right.right (a leaf child of the binary node stays one child); unused slots
 * have lo = +inf, hi = -inf, link 0 and count -1.  Nodes are numbered in binary-index order of the
 * even-depth nodes.  Returns the node count (nodes32 holds n_internal nodes). */
uint32_t orc_collapse_bvh4(const float* nodes16, uint32_t n_internal, float* nodes32);
/* FAST closest/any hit through it: the hit children are ordered by the key
 * (order-preserving bits of the entry distance with the low two bits
 * replaced by the slot); the first is visited next, the rest pushed last
 * first. */
int orc_trace_bvh4(int kind, int query, const float* nodes32, uint32_t n4, const float* root_bounds6,
                   uint32_t n_prims, const uint32_t* order, const float* prims, const orc_ray_t* rays,
                   uint32_t nrays, orc_hit_t* hits, uint8_t* occluded, uint64_t* counters, int nthreads);
int orc_trace_brute(int kind, int mode, int query, uint32_t n_prims, const float* prims,
                    const orc_ray_t* rays, uint32_t nrays, orc_hit_t* hits, uint8_t* occluded,
                    int nthreads);

/* ---- render step (main.cpp:503-566, 390-497) ---- */
void orc_jitter_mt19937(uint64_t count, double* out);
void orc_camera_rays_ref(uint32_t width, uint32_t height, uint32_t aa, const double* jitter,
                         orc_ray_t* rays);
void orc_shade_ref(const float* sph, const float* surface_rgb, const orc_ray_t* rays,
                   const orc_hit_t* hits, uint32_t n, int kd_mode, const uint8_t* kd_any,
                   float* rgb);
void orc_pixels_ref(const float* rgb, uint32_t npix, uint32_t aa, uint8_t* out);

/* ---- render of a view (the engine's rq_render; restated, no reference
 * counterpart beyond castRay's shading, main.cpp:390-497) ---- */
typedef struct {
  float eye[3], target[3], up[3], light[3], albedo[3], bg[3];
  float tan_half, ambient, mirror, bias;
  uint32_t width, height, spp, x0, y0, ww, wh, bounces;
  uint64_t seed;
} orc_view_t;
/* rays: ww*wh*spp camera rays; cw: 4 floats per ray (colour, weight). */
void orc_view_rays(const orc_view_t* v, orc_ray_t* rays, float* cw);
/* One depth: reads hits of `rays`, writes shadow rays and the next mirror
 * rays (into rays), updates cw, writes pend (4 floats per ray).  counters
 * (may be NULL): [0] += shadow rays, [1] += mirror rays. */
void orc_shade_hits(int kind, const float* verts, const uint32_t* idx, const float* sph,
                    const orc_view_t* v, uint64_t nray, int last, orc_ray_t* rays, const orc_hit_t* hits,
                    orc_ray_t* shadow, float* cw, float* pend, uint64_t* counters);
void orc_shadow_accum(uint64_t nray, const uint8_t* occluded, const float* pend, float* cw);
void orc_view_pixels(uint64_t npix, uint32_t spp, const float* cw, uint8_t* pixels, float* rgb);

#ifdef __cplusplus
}
#endif
#endif
