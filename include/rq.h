/*
 * rq.h — C ABI of the GB300 ray-query engine (acceleration-structure build +
 * ray traversal for sm_103a, one GPU).
 *
 * The engine replaces the hot path of the reference CPU ray tracer
 * (Alhajras/Raytracer-Data-structures, project/raytracer/): the builders
 * behind the Settings::dataStructure switch and the queries castRay makes
 * through them.  Every entry point below names the reference interface it
 * replaces.  Plain C types only: opaque handles, pointers and sizes.
 *
 * Conventions
 *  - Every call returns rq_status_t; no exception crosses the ABI.
 *    rq_last_error(ctx) describes the last failure on that context.
 *  - Device memory of scenes and acceleration structures is owned by the
 *    engine.  Caller buffers are host memory unless RQ_DEVICE_POINTERS is set
 *    in `flags`, in which case they are device pointers on the context's
 *    device.
 *  - Host-pointer calls are synchronous.  Device-pointer calls are enqueued
 *    on the context's stream (rq_set_stream) and return at once; device-side
 *    errors (traversal stack overflow, a bounded wait that gave up) are then
 *    reported by rq_synchronize.
 *  - A context is used by one host thread at a time; distinct contexts may be
 *    used concurrently.
 */
#ifndef RQ_H
#define RQ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RQ_ABI_VERSION 1

typedef enum rq_status_t {
  RQ_SUCCESS = 0,
  RQ_ERROR_INVALID_ARGUMENT = 1, /* null handle/pointer, size out of range, NaN input, bad index */
  RQ_ERROR_UNSUPPORTED = 2,      /* e.g. UNIFORM_GRID, declared but never built by the reference */
  RQ_ERROR_OUT_OF_MEMORY = 3,
  RQ_ERROR_CUDA = 4,             /* a CUDA runtime call failed; see rq_last_error */
  RQ_ERROR_STACK_OVERFLOW = 5,   /* a traversal stack would have overflowed; the ray was abandoned */
  RQ_ERROR_TIMEOUT = 6,          /* a bounded device-side wait gave up */
  RQ_ERROR_EMPTY_SCENE = 7,      /* zero primitives (undefined behaviour in the reference) */
  RQ_ERROR_NO_DEVICE = 8
} rq_status_t;

/* AccType, accelerators.h:21 — same names and values. */
typedef enum rq_acc_type_t {
  RQ_BVH = 0,          /* median/midpoint BVH, constructBVHNew accelerators.h:246 */
  RQ_KDTREE = 1,       /* SAH KD-tree, constructKDTreeNew accelerators.h:951 */
  RQ_UNIFORM_GRID = 2, /* declared by the reference, never implemented: RQ_ERROR_UNSUPPORTED */
  RQ_LBVH = 3,         /* Morton + radix sort + Karras + refit (cited at accelerators.h:371,568) */
  RQ_NONE = 4          /* brute force, castRay default branch main.cpp:373-387 */
} rq_acc_type_t;

/* SceneModel, settings.h:4 — same names and values. */
typedef enum rq_scene_model_t {
  RQ_IGEA = 0, RQ_ARMADILLO = 1, RQ_BUNNY = 2, RQ_BUNNIES = 3,
  RQ_TEST = 4, RQ_GRASS = 5, RQ_BUDDHA = 6, RQ_CITY = 7
} rq_scene_model_t;

/* Settings, settings.h:7-17: the reference's fields in the reference's order
 * with the reference's defaults (rq_settings_default), followed by engine
 * fields. */
typedef struct rq_settings_t {
  uint32_t width;             /* 640 */
  uint32_t height;            /* 480 */
  float fov;                  /* 90; the reference's render() ignores it and uses 30 (main.cpp:545) */
  float backgroundColor[3];   /* (1, 1, 1) */
  float bias;                 /* 1e-4 */
  uint32_t aa_samples;        /* 1 */
  int32_t dataStructure;      /* rq_acc_type_t, RQ_BVH */
  int32_t sceneModel;         /* rq_scene_model_t, RQ_BUNNY */
  /* ---- engine fields ---- */
  int32_t traversal;          /* rq_traversal_t, RQ_TRAVERSAL_FAST */
  int32_t morton;             /* rq_morton_t, RQ_MORTON_SCENE_BOUNDS */
  int32_t kd_max_depth;       /* <= 0: round(8 + 1.3 log2 N) as the reference (accelerators.h:958) */
  int32_t ray_sort;           /* rq_ray_sort_t: reorder large FAST batches for coherence */
  int32_t node_width;         /* rq_node_width_t: BVH node fan-out for FAST queries (RQ_BVH, RQ_LBVH) */
  int32_t scheduling;         /* rq_scheduling_t: how FAST binary-BVH queries map rays to threads */
  int32_t lbvh_quality;       /* rq_lbvh_quality_t: RQ_LBVH tree after the Karras build, RQ_LBVH_KARRAS */
  int32_t reserved[1];
} rq_settings_t;

/* How FAST queries on binary BVH structures map rays to GPU threads.  Speed
 * only: every ray walks the same nodes in the same order either way. */
typedef enum rq_scheduling_t {
  RQ_SCHEDULING_THREAD_PER_RAY = 0, /* each thread walks one ray at a time; warps take 32 rays at a time from a counter */
  RQ_SCHEDULING_LANE_REFILL = 1,    /* persistent warps refill finished lanes with new rays */
  RQ_SCHEDULING_SPECULATIVE = 2,    /* while-while walk that postpones leaves until the warp has one each */
  RQ_SCHEDULING_WARP_PACKET = 3,    /* the warp walks one shared stack (lane masks per entry): coherent rays */
  RQ_SCHEDULING_SHARED_TOP = 4      /* one thread per ray; the top 6 tree levels staged in shared memory per block */
} rq_scheduling_t;

/* Node fan-out of BVH structures (RQ_BVH, RQ_LBVH), fixed when the structure
 * is built.  RQ_NODE_WIDTH_4 adds a collapsed 4-wide copy of the binary tree
 * (every even-depth node merged with its internal children: one 128-byte
 * node holds up to four child boxes) that FAST queries walk instead.
 * RQ_NODE_WIDTH_8 adds a compressed 8-wide copy (every node at a depth
 * divisible by 3 holds its descendants three levels down: one 128-byte node
 * with eight child boxes quantised to bytes, rounded outward, and the children
 * placed by direction so each ray visits them in an order set by its
 * direction's signs).  Hits and occlusion bits are those of the binary tree;
 * REFERENCE queries and rq_accel_export_bvh2 keep using the binary nodes. */
typedef enum rq_node_width_t {
  RQ_NODE_WIDTH_2 = 0, /* binary nodes (2 is accepted too) */
  RQ_NODE_WIDTH_4 = 4,
  RQ_NODE_WIDTH_8 = 8
} rq_node_width_t;

/* The RQ_LBVH tree.  RQ_LBVH_KARRAS keeps the Karras radix-tree topology
 * over the sorted Morton codes.  RQ_LBVH_TREELETS then runs one bottom-up
 * pass of treelet restructuring (Karras and Aila 2013): at every internal node
 * the treelet of up to four leaves grown from it (largest-area internal leaf
 * expanded first) is rebuilt with the topology of least surface-area cost,
 * the tree's own nodes reused.  On the 998,000-triangle terrain the walks
 * visit about 10% fewer nodes.  Hits and occlusion bits do not change; the
 * exported topology does.  Single-structure builds only (rq_build_batched
 * keeps the Karras tree). */
typedef enum rq_lbvh_quality_t {
  RQ_LBVH_KARRAS = 0,
  RQ_LBVH_TREELETS = 1
} rq_lbvh_quality_t;

/* Ray reordering before FAST BVH2 traversal of batches of at least 65,536
 * rays.  Results are written in the caller's order either way and do not
 * change; only the speed does. */
typedef enum rq_ray_sort_t {
  RQ_RAY_SORT_NONE = 0,
  RQ_RAY_SORT_OCTANT_MORTON = 1,    /* direction octant, then 27-bit Morton code of the origin */
  RQ_RAY_SORT_ORIGIN_DIRECTION = 2, /* octant, 15-bit origin Morton code, 12-bit direction (|dx|, |dy|) */
  RQ_RAY_SORT_DIRECTION_ORIGIN = 3, /* octant, 12-bit direction, 15-bit origin Morton code */
  RQ_RAY_SORT_OCTANT_MORTON12 = 4,  /* octant, 12-bit origin Morton code: a 15-bit key, half the sort passes */
  RQ_RAY_SORT_OCTANT = 5,           /* direction octant only: a 3-bit key, one sort pass */
  RQ_RAY_SORT_OCTANT_MORTON3 = 6    /* octant, 3-bit origin Morton code (2x2x2 cells): one sort pass */
} rq_ray_sort_t;

/* How rays meet boxes and primitives. */
typedef enum rq_traversal_t {
  /* Reciprocal-direction slab test clipped to [tmin, closest hit], widened by
   * 1 + 2*gamma(3) so no box is lost to rounding; near child first; hits
   * limited to (tmin, tmax).  BVH and brute-force closest hit is the smallest
   * t and, among primitives hit at exactly that t, the smallest primitive id:
   * a result independent of the order of the walk (node width, scheduling,
   * ray reordering). */
  RQ_TRAVERSAL_FAST = 0,
  /* The reference's semantics: division slab test with no clipping
   * (accelerators.h:588-626), boxIntersect's pre-order candidate walk
   * (accelerators.h:668-690), castRay's closest selection (t0 < 0 -> t1,
   * strict <, main.cpp:343-358), kdtreeIntersect's any-hit
   * (accelerators.h:997-1086).  Reproduces the reference's pixels. */
  RQ_TRAVERSAL_REFERENCE = 1
} rq_traversal_t;

/* Centroid normalisation before morton3D. */
typedef enum rq_morton_t {
  RQ_MORTON_SCENE_BOUNDS = 0, /* (c - lo) / (hi - lo); lo/hi = vertex box (triangles) or centre box (spheres) */
  RQ_MORTON_REFERENCE = 1,    /* (c + 30) / 1000, accelerators.h:577 */
  /* (c - lo) / E with E = max over axes of (hi - lo): one scale for all axes,
   * which splits flat or elongated scenes into tighter boxes (on a 1M-triangle
   * terrain 16-22% fewer node visits per ray).  FAST results do not depend on
   * the tree (the closest-hit rule picks the same hit), so this is a speed
   * option for those queries. */
  RQ_MORTON_SCENE_CUBE = 2
} rq_morton_t;

/* Flags for calls that take caller buffers. */
#define RQ_DEVICE_POINTERS 0x1u

/* Ray, 32 bytes: the origin/direction pair castRay receives (main.cpp:291-298)
 * plus the query interval. */
typedef struct rq_ray_t {
  float org[3];
  float tmin;
  float dir[3];
  float tmax;
} rq_ray_t;

/* Closest hit, 16 bytes.  prim = RQ_MISS and t = tmax when nothing is hit.
 * u, v: barycentrics for triangles, 0 for spheres. */
typedef struct rq_hit_t {
  float t;
  uint32_t prim;
  float u;
  float v;
} rq_hit_t;

#define RQ_MISS 0xFFFFFFFFu

typedef struct rq_context* rq_ctx_t;
typedef struct rq_scene* rq_scene_t;
typedef struct rq_accel* rq_accel_t;

/* Description of a built structure, for the caller and for parity checks. */
typedef struct rq_accel_info_t {
  int32_t type;            /* rq_acc_type_t */
  int32_t prim_kind;       /* 0 triangles, 1 spheres */
  uint32_t n_prims;
  uint32_t n_nodes;        /* BVH2: internal nodes; KD: nodes */
  uint32_t n_slots;        /* BVH2: leaf slots; KD: primitive-index entries */
  uint32_t max_depth;      /* KD: depth limit used */
  float root_bounds[6];    /* min xyz, max xyz */
  uint64_t device_bytes;   /* device memory held by the structure */
  uint32_t node_width;     /* BVH2 structures: 2, or 4 with a collapsed 4-wide copy; else 0 */
  uint32_t n_wide_nodes;   /* nodes of the 4-wide copy */
} rq_accel_info_t;

/* ------------------------------------------------------------ lifecycle */

/* Defaults of settings.h:7-17 plus engine defaults. */
void rq_settings_default(rq_settings_t* s);

/* Replaces the implicit global state of main() (main.cpp:723-760).  Binds
 * `device` (a CUDA ordinal); settings may be NULL for defaults. */
rq_status_t rq_create(const rq_settings_t* settings, int device, rq_ctx_t* out);
rq_status_t rq_destroy(rq_ctx_t ctx);
rq_status_t rq_get_settings(rq_ctx_t ctx, rq_settings_t* out);
rq_status_t rq_set_settings(rq_ctx_t ctx, const rq_settings_t* settings);
/* All later work of the context goes to this cudaStream_t (passed as void*,
 * used as given: NULL is the CUDA legacy default stream).  A new context
 * starts on a non-blocking stream of its own. */
rq_status_t rq_set_stream(rq_ctx_t ctx, void* cuda_stream);
rq_status_t rq_synchronize(rq_ctx_t ctx);
const char* rq_last_error(rq_ctx_t ctx);
const char* rq_status_string(rq_status_t status);

/* ----------------------------------------------------------------- scenes */

/* Triangle mesh: verts = nv * 3 floats, idx = nt * 3 uint32 (the OBJ `v`/`f`
 * content the reference's loader, main.cpp:599-721, reads only as points).
 * Validated: finite vertices, indices < nv, nt > 0. */
rq_status_t rq_scene_create_triangles(rq_ctx_t ctx, const float* verts, uint32_t nv,
                                      const uint32_t* idx, uint32_t nt, uint32_t flags,
                                      rq_scene_t* out);
/* Spheres: n * (cx, cy, cz, r), the SceneObject list createScene_new builds
 * (main.cpp:677-692, 702-717); primitive id = position. */
rq_status_t rq_scene_create_spheres(rq_ctx_t ctx, const float* center_radius, uint32_t n,
                                    uint32_t flags, rq_scene_t* out);
/* Overwrite a scene's geometry with the same counts (dynamic scenes; follow
 * with rq_accel_rebuild): data = vertices (triangles) or spheres; idx = new
 * triangle indices, or NULL to keep them. */
rq_status_t rq_scene_update(rq_ctx_t ctx, rq_scene_t scene, const float* data, const uint32_t* idx,
                            uint32_t flags);
rq_status_t rq_scene_destroy(rq_scene_t scene);

/* ----------------------------------------------------------------- builds */

/* The dataStructure switch of main() (main.cpp:791-843):
 *   RQ_BVH    -> constructBVHNew (accelerators.h:246)
 *   RQ_KDTREE -> constructKDTreeNew (accelerators.h:951)
 *   RQ_LBVH   -> constructLBVHTree (accelerators.h:570), as a Karras LBVH
 *   RQ_NONE   -> no structure; queries test every primitive
 * Uses the context's settings (morton normalisation, kd_max_depth). */
rq_status_t rq_build(rq_ctx_t ctx, rq_scene_t scene, int32_t acc_type, rq_accel_t* out);
/* Rebuild in place from the (possibly updated) scene, reusing device memory. */
rq_status_t rq_accel_rebuild(rq_ctx_t ctx, rq_accel_t accel);
rq_status_t rq_accel_destroy(rq_accel_t accel);

/* Build one structure per scene.  RQ_LBVH builds the whole batch in one pass
 * of batched kernels (scene boxes, Morton codes, one segmented radix sort by
 * (scene, code), Karras topology, refit), the arrays of all scenes back to
 * back in one allocation that lives until the last of the returned
 * structures is destroyed; each structure equals the one rq_build would make
 * from its scene.  The scenes must all hold triangles or all spheres, with
 * fewer than 2^30 primitives together.  Other types are built scene by
 * scene.  out receives n handles.  No reference counterpart: the reference
 * builds one scene per run. */
rq_status_t rq_build_batched(rq_ctx_t ctx, const rq_scene_t* scenes, uint32_t n, int32_t acc_type,
                             rq_accel_t* out);
/* Rebuild all structures of one rq_build_batched call (same handles, same
 * order) in one pass, after rq_scene_update of any of its scenes.  Enqueued
 * on the context's stream without waiting.  It allocates nothing once one
 * build or rebuild has run with the same settings.node_width, so it can be
 * captured into a CUDA graph (rq_plan_create does). */
rq_status_t rq_accel_rebuild_batched(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n);
rq_status_t rq_accel_get_info(rq_accel_t accel, rq_accel_info_t* info);

/* Host copies of a built structure (layouts in the engine documentation):
 * BVH2 (RQ_BVH, RQ_LBVH): nodes = n_nodes * 16 words, order = n_slots ids,
 * sorted_codes = n_prims Morton codes in slot order (RQ_LBVH only; may be
 * NULL).  KD: nodes = n_nodes * 3 words in the reference's KdAccelNode
 * encoding (accelerators.h:715-742), prim_idx = n_slots ids. */
rq_status_t rq_accel_export_bvh2(rq_ctx_t ctx, rq_accel_t accel, float* nodes, uint32_t* order,
                                 uint32_t* sorted_codes);
rq_status_t rq_accel_export_kd(rq_ctx_t ctx, rq_accel_t accel, int32_t* nodes, int32_t* prim_idx);
/* The wide nodes of a structure built with RQ_NODE_WIDTH_4 or _8: n_nodes
 * receives the count; nodes (may be NULL) receives n_nodes * 32 words.
 * 4-wide: [lo.x[4] hi.x[4] lo.y[4] hi.y[4] lo.z[4] hi.z[4] link[4] count[4]];
 * a child with link >= 0 is a 4-wide node, link < 0 a leaf holding slots
 * [~link, ~link + count) of the binary tree's order; unused children have
 * count -1.  8-wide: [pm.x pm.y pm.z E] [qlo.x[8] qhi.x[8] as bytes] (y) (z)
 * [(link, count) x 8]: E packs three biased exponents (bits 0-23) and the
 * mask of used slots (bits 24-31); child plane = fma(2^(E_a - 127),
 * 1 + q * 2^-15, pm_a); count 0 -> 8-wide node `link`, count > 0 -> leaf of
 * slots [link, link + count).  No reference counterpart: the reference's
 * trees are binary. */
rq_status_t rq_accel_export_bvh4(rq_ctx_t ctx, rq_accel_t accel, float* nodes, uint32_t* n_nodes);

/* A BVH2 structure from host arrays in rq_accel_export_bvh2's layout (nodes =
 * n_nodes * 16 words, order = n_slots primitive ids of `scene`, root_bounds =
 * min xyz, max xyz), for trees built elsewhere or edited by the caller.  Every
 * link is checked to stay inside the arrays (internal child < n_nodes, leaf
 * slots within n_slots, counts >= 1) and every box to be finite; the shape
 * itself is not checked: a cycle makes queries end with
 * RQ_ERROR_INVALID_ARGUMENT ("malformed acceleration structure") once a walk
 * exceeds the steps a valid tree allows, and boxes that miss their primitives
 * lose those hits.  The structure reports type RQ_BVH, is walked with binary
 * nodes whatever settings.node_width says, and cannot be rebuilt
 * (rq_accel_rebuild: RQ_ERROR_UNSUPPORTED).  No reference counterpart: the
 * reference builds its trees in process (constructBVHNew, accelerators.h:246). */
rq_status_t rq_accel_import_bvh2(rq_ctx_t ctx, rq_scene_t scene, const float* nodes, uint32_t n_nodes,
                                 const uint32_t* order, uint32_t n_slots, const float* root_bounds,
                                 rq_accel_t* out);

/* Test hooks that make the engine's device-side guards fire on purpose,
 * without a fault, so a test can check the status a caller then sees and that
 * the context keeps working.  All fields 0 (the default) is normal operation.
 * No reference counterpart (the reference reports no errors at all,
 * main.cpp:656-660). */
typedef struct rq_debug_t {
  /* 1: in rq_sort_pairs of this context with at least 3,841 pairs, one tile
   * of the first digit pass waits on a device word that nothing ever sets; its
   * bounded wait gives up (some microseconds) and the call returns
   * RQ_ERROR_TIMEOUT with keys and values undefined. */
  uint32_t sort_stall;
  /* 1: FAST thread-per-ray binary-BVH queries (rq_trace_closest / any, BVH and
   * LBVH, node_width 2, scheduling THREAD_PER_RAY) run with a traversal
   * stack of 8 entries instead of 64, so trees deep enough along a ray end in
   * RQ_ERROR_STACK_OVERFLOW. */
  uint32_t small_stack;
} rq_debug_t;
/* debug may be NULL (all hooks off). */
rq_status_t rq_set_debug(rq_ctx_t ctx, const rq_debug_t* debug);

/* ---------------------------------------------------------------- queries */

/* Closest hit per ray: replaces boxIntersect + castRay's candidate loop
 * (accelerators.h:668-690, main.cpp:330-388). */
rq_status_t rq_trace_closest(rq_ctx_t ctx, rq_accel_t accel, const rq_ray_t* rays, uint32_t n,
                             rq_hit_t* hits, uint32_t flags);
/* Any hit within (tmin, tmax) per ray, one bit per ray (bit r%32 of word
 * r/32): replaces kdtreeIntersect (accelerators.h:997) and the shadow query
 * trace_more (main.cpp:235-245, a stub returning false). */
rq_status_t rq_trace_any(rq_ctx_t ctx, rq_accel_t accel, const rq_ray_t* rays, uint32_t n,
                         uint32_t* occluded_bits, uint32_t flags);

/* boxIntersect (accelerators.h:668-690) for a batch of rays: for each ray,
 * the ids of the primitives of every leaf the reference's walk reaches
 * (division slab test without clipping, left subtree before right), the list
 * castRay's candidate loop (main.cpp:335-358) then tests.  counts: n entries;
 * *total: their sum; ids (may be NULL: counts only): the lists concatenated
 * in ray order, ids_cap entries available (RQ_ERROR_INVALID_ARGUMENT when
 * fewer than *total, or when *total is 2^32 or more: split the rays; counts
 * and total are still written).  BVH
 * structures (RQ_BVH, RQ_LBVH); RQ_DEVICE_POINTERS for device buffers. */
rq_status_t rq_trace_candidates(rq_ctx_t ctx, rq_accel_t accel, const rq_ray_t* rays, uint32_t n, uint32_t* counts,
                                uint32_t* ids, uint64_t ids_cap, uint64_t* total, uint32_t flags);

/* One host-buffer query of rq_trace_queries. */
typedef struct rq_query_t {
  const rq_ray_t* rays;   /* host */
  uint32_t n;
  int32_t any;            /* 0: closest hits (rq_hit_t per ray) into out; 1: occlusion bits */
  void* out;              /* host */
  int32_t ray_sort;       /* rq_ray_sort_t for this query; -1: the context's setting */
  int32_t scheduling;     /* rq_scheduling_t for this query; -1: the context's setting */
} rq_query_t;
/* Several host-buffer queries on one structure in one call, with copies
 * and traversals overlapped across queries: queries run in the given order;
 * the first streams chunk by chunk when it has no ray order, the others (and
 * a first query with a ray order, whose order pays off only over the whole
 * batch) upload whole while earlier ones trace, each traced as one batch,
 * and download while later ones trace.  Uploads begin at once, overlapping
 * work already queued on the context's stream such as a rebuild.  Put the
 * query with the longest traversal first.  Results equal
 * rq_trace_closest / rq_trace_any per query; returns when every result is in
 * host memory.  Device memory: each query after the first keeps a buffer of
 * its rays and results (grow-only, per context). */
rq_status_t rq_trace_queries(rq_ctx_t ctx, rq_accel_t accel, const rq_query_t* queries, uint32_t n_queries);

/* The FAST closest/any query of rq_trace_closest / rq_trace_any that also
 * sums, over all rays, the internal nodes visited (counters[0]) and the
 * primitives tested (counters[1]): the inputs of the traversal byte model.
 * BVH2 structures (RQ_BVH, RQ_LBVH).  Synchronous; results go to `out`
 * (hits or occlusion bits) as in the plain calls. */
rq_status_t rq_trace_counters(rq_ctx_t ctx, rq_accel_t accel, const rq_ray_t* rays, uint32_t n,
                              int32_t any, void* out, uint64_t* counters, uint32_t flags);

/* ------------------------------------------------ many structures at once */

/* Rays of many structures in one persistent, work-stealing launch: rays
 * [ray_offsets[k], ray_offsets[k+1]) are traced against accels[k]
 * (ray_offsets: host array of n_accels + 1 non-decreasing entries, first 0).
 * any = 0: closest hits (16 B per ray) into out; any = 1: occlusion bits.
 * Results equal the one-structure FAST queries.  The structures must be BVH
 * structures (RQ_BVH, RQ_LBVH) of one primitive kind and node width.
 * RQ_DEVICE_POINTERS: rays and out are device buffers and the launch is
 * enqueued without waiting.  No reference counterpart. */
rq_status_t rq_trace_batched(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n_accels, const rq_ray_t* rays,
                             const uint32_t* ray_offsets, int32_t any, void* out, uint32_t flags);

/* A captured step over fixed device buffers, replayed as one CUDA graph:
 * [rq_accel_rebuild_batched of the batch] + the many-structure query of
 * rq_trace_batched.  rq_plan_create autotunes the query's launch shape
 * (block of 128 or 256 threads x shallow or deep traversal stack, each
 * without and with a per-scene ray order) by timing each on `rays`, drops
 * shapes whose stack overflows on these trees, then captures the step.  A
 * rebuilding plan (rebuild = 1) also tries every node width (binary,
 * collapsed 4-wide, compressed 8-wide) and leaves the batch's structures at
 * the width it picked.  rays and out are device buffers whose contents may
 * change between launches; the structures and scenes must outlive the plan.
 * rebuild = 1 needs accels to be the whole batch of one rq_build_batched
 * call.  No reference counterpart. */
typedef struct rq_plan* rq_plan_t;
typedef struct rq_plan_info_t {
  uint32_t block_threads;   /* chosen launch shape */
  uint32_t stack_entries;
  uint32_t graph_kernels;   /* kernels one launch replays */
  uint32_t n_rays;
  uint32_t rebuilds;        /* 1 when the step rebuilds the batch */
  float shape_ms[4];        /* query time of 128/shallow, 128/deep, 256/shallow, 256/deep; < 0: dropped */
  uint32_t ray_order;       /* 1 when the plan traces through a per-scene ray order (chosen by time) */
  float ordered_ms[4];      /* the same shapes with the ray order (keys + sort + query); < 0: not offered */
  uint32_t node_width;      /* node width the plan runs with (2, 4 or 8) */
  float width_ms[3];        /* best query time with node width 2 / 4 / 8; < 0: not tried */
} rq_plan_info_t;
rq_status_t rq_plan_create(rq_ctx_t ctx, const rq_accel_t* accels, uint32_t n_accels, int32_t rebuild,
                           const rq_ray_t* rays, const uint32_t* ray_offsets, int32_t any, void* out,
                           rq_plan_t* plan);
/* Enqueue one replay on the context's stream (no host synchronisation;
 * rq_synchronize reports device-side errors). */
rq_status_t rq_plan_launch(rq_plan_t plan);
rq_status_t rq_plan_get_info(rq_plan_t plan, rq_plan_info_t* info);
rq_status_t rq_plan_destroy(rq_plan_t plan);

/* Kernel launches the engine has made in this process, over all contexts. */
uint64_t rq_kernel_launch_count(void);

/* --------------------------------------------------- component kernels */

/* morton3D over centroids (accelerators.h:374-394, 575-580): codes for the
 * scene's primitives with the context's normalisation, in primitive order. */
rq_status_t rq_morton_codes(rq_ctx_t ctx, rq_scene_t scene, uint32_t* codes, uint32_t flags);
/* Stable LSD radix sort of (key, value) pairs on the low `key_bits` bits:
 * what radixSort (accelerators.h:348-369) intends (it sorts a by-value copy
 * and so has no effect).  In place. */
rq_status_t rq_sort_pairs(rq_ctx_t ctx, uint32_t* keys, uint32_t* values, uint32_t n,
                          uint32_t key_bits, uint32_t flags);

/* The same sort for callers that must not allocate device memory while they
 * run: a serving loop held to a fixed memory budget, code whose device memory
 * belongs to another allocator, or a latency-critical loop where cudaMalloc /
 * cudaFree would synchronize the device.  This entry point has no counterpart
 * in the reference.
 *  - keys and values are device pointers on the current device; no context is
 *    needed.  Work is enqueued on cuda_stream (NULL: the legacy default
 *    stream) and the call returns once the sort has finished on it.
 *  - No memory is allocated: the working memory is one fixed array of about
 *    9.5 MB that every GPU loading this library holds until the process exits.
 *    It bounds n to RQ_SORT_NOALLOC_MAX_PAIRS; larger n returns
 *    RQ_ERROR_INVALID_ARGUMENT.
 *  - Every call looks up the array's device address on the current device
 *    (cuda_stream must belong to that device: RQ_ERROR_INVALID_ARGUMENT
 *    otherwise).  The first call on a device may load the library's device
 *    code there; make that first call before any stream capture.
 *  - All calls on a device share the array, so calls that overlap on the GPU
 *    (other streams, other host threads) race and must be serialized by the
 *    caller.
 *  - RQ_ERROR_TIMEOUT (a bounded device-side wait gave up) leaves keys and
 *    values undefined: later digit passes still run and write into them. */
#define RQ_SORT_NOALLOC_MAX_PAIRS (1u << 20)
rq_status_t rq_sort_pairs_noalloc(uint32_t* keys, uint32_t* values, uint32_t n, uint32_t key_bits,
                                  void* cuda_stream);

/* ------------------------------------------------------------ render step */

/* render() (main.cpp:541-566) with castRay's shading (main.cpp:390-497) for
 * a sphere scene: pinhole camera at the origin looking down -z, fov 30,
 * aa_samples jittered samples per pixel, one point light at (0, 3, 30).
 * jitter: 2 doubles per sample in (y, x, sample) order; NULL draws the
 * reference's default-seeded mt19937 sequence.  surface_rgb: 3 floats per
 * sphere.  pixels: width*height*3 bytes of the P6 payload (main.cpp:516-528).
 * rgb_sum (may be NULL): per-pixel colour sums before quantisation. */
rq_status_t rq_render_reference(rq_ctx_t ctx, rq_accel_t accel, const rq_settings_t* settings,
                                const double* jitter, const float* surface_rgb, uint8_t* pixels,
                                float* rgb_sum);

/* ----------------------------------------------------- render of a view */

/* A pinhole view of any scene (triangles or spheres) with one point light.
 * The reference renders only its fixed sphere camera (rq_render_reference);
 * this generalises castRay's shading (main.cpp:390-497) to the triangle
 * workloads: per sample, at each hit, albedo * (ambient + visible * max(0,
 * N.L)) with a real shadow ray (the reference's trace_more is a stub), plus
 * optional mirror bounces; misses add settings.backgroundColor.  Normals face
 * the incoming ray; shadow and mirror rays start at P + settings.bias * N.
 * Sample s of pixel (x, y) is jittered by a counter-based generator of
 * (seed, (y * width + x) * spp + s), so a window reproduces the full image's
 * pixels exactly. */
typedef struct rq_view_t {
  float eye[3];
  float target[3];
  float up[3];
  float fov_deg;        /* vertical field of view, degrees */
  float light[3];       /* point light position */
  float albedo[3];      /* surface colour */
  float ambient;        /* added to max(0, N.L) at every hit */
  float mirror;         /* reflectance of the mirror bounces, 0..1 */
  uint32_t bounces;     /* mirror bounces after the camera hit */
  uint32_t window[4];   /* x0, y0, w, h inside width x height; w or h == 0: the whole image */
  uint64_t seed;        /* sample jitter */
} rq_view_t;

/* Render `view` with settings.width x height pixels and settings.aa_samples
 * samples per pixel through `accel` (any dataStructure; FAST or REFERENCE
 * traversal and the speed options of the context's settings).  pixels:
 * w*h*3 bytes (min(1, mean)*255, truncated, as write_into_file,
 * main.cpp:516-528); rgb (may be NULL): w*h*3 float means before
 * quantisation; ray_counts (may be NULL, host): camera rays, shadow rays and
 * mirror rays traced.  RQ_DEVICE_POINTERS: pixels and rgb are device
 * buffers and the call returns without waiting (ray_counts must then be
 * NULL).  No reference counterpart beyond the sphere render it generalises. */
rq_status_t rq_render(rq_ctx_t ctx, rq_accel_t accel, const rq_view_t* view, uint8_t* pixels, float* rgb,
                      uint64_t* ray_counts, uint32_t flags);

/* ------------------------------------------------------------ scene I/O */

/* Wavefront OBJ meshes (host only; no context or GPU needed).  rq_obj_load
 * reads `v x y z` records and `f` records with the v, v/vt, v/vt/vn or v//vn
 * corner forms, 1-based or negative (relative to the vertices read so far);
 * a polygon of k > 3 corners becomes k - 2 triangles around its first
 * corner; every other record (vn, vt, o, g, s, usemtl, mtllib, #) is
 * skipped.  A file without `f` records gives nt = 0 (a point cloud: the form
 * of the reference's models, which its loader, main.cpp:650-718, reads as
 * `v` records only).  verts (nv * 3 floats) and idx (nt * 3) are allocated by
 * the library; release them with rq_free.  Malformed records, out-of-range
 * corners and unreadable files: RQ_ERROR_INVALID_ARGUMENT. */
rq_status_t rq_obj_load(const char* path, float** verts, uint32_t* nv, uint32_t** idx, uint32_t* nt);
/* `v` records in the shortest form that reads back to the same float, then
 * 1-based `f` records. */
rq_status_t rq_obj_save(const char* path, const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt);
void rq_free(void* p);
/* createScene_new's model file (main.cpp:605-643): <dir>/<name>.obj for a
 * rq_scene_model_t (other values: test.obj), the name matched without regard
 * to case (the reference asks for "igea.obj"; its file is "Igea.obj").  out
 * receives the path (cap bytes including the terminating NUL). */
rq_status_t rq_model_path(const char* dir, int32_t scene_model, char* out, uint32_t cap);
/* createScene_new's spheres from a model file: each `v` record up to the
 * first other token becomes a sphere of radius 0.05 at v * 100 + shift, then
 * y - 10, z - 60 (shift = 20 * clone, for `clones` copies), followed by the
 * ground sphere of radius 100 (main.cpp:650-718).  spheres: n * 4 floats,
 * released with rq_free. */
rq_status_t rq_reference_spheres(const char* path, int32_t clones, float** spheres, uint32_t* n);

/* ------------------------------------------------------------ serving */

/* A serving loop: render requests against a library of triangle meshes,
 * served by a worker thread that owns its own context on `device`.
 *  - Admission: a request must name a registered mesh, and its camera rays
 *    (width * height * spp) must fit max_batch_rays; requests whose mesh
 *    cannot fit the HBM budget complete with RQ_ERROR_OUT_OF_MEMORY.
 *  - Residency: meshes are kept on the host; a request's mesh is uploaded and
 *    its LBVH built on first use, on a stream of its own beside the rendering.
 *    Resident scenes and structures and the wavefront buffers (112 bytes per
 *    camera sample in flight) stay within hbm_budget bytes by evicting the
 *    least recently used meshes that no step being formed or in flight needs
 *    (rebuilt when requested again).
 *  - Continuous batching (batching = 1): each step takes rows of the waiting
 *    requests in arrival order, up to step_rays camera rays and
 *    max_batch_requests requests; while others wait, one request takes at
 *    most half a step (a larger request is split by rows and finished in
 *    later steps); the step renders them as one wavefront (camera
 *    rays, one many-structure closest-hit query, shading, one many-structure
 *    shadow query, pixels, one download).  Two steps are in flight at once on
 *    two streams: requests that arrive while one step runs go into the next,
 *    which starts on the GPU beside it.  A request completes when its last
 *    rows land.  batching = 0 renders one whole request per step and waits
 *    for each step before the next.
 *  - A request renders exactly what rq_render renders for the same view with
 *    bounces = 0, settings.bias = 1e-4 and its width, height, spp and
 *    background, alone or among others.
 *  - Latency: from rq_server_submit until the pixels are in host memory.
 * The reference has no serving path; this is the engine's own. */
typedef struct rq_server* rq_server_t;
typedef struct rq_server_config_t {
  int32_t device;              /* CUDA ordinal */
  int32_t batching;            /* 1: continuous batching; 0: one request per step */
  uint64_t hbm_budget;         /* bytes of resident scenes + structures + wavefront buffers; 0: 80 GB */
  uint32_t max_batch_rays;     /* camera rays of one request at most; 0: 2^25 (below 2^31) */
  uint32_t max_batch_requests; /* requests (or parts of requests) per step; 0: 256 */
  uint32_t step_rays;          /* batching: camera rays per step; larger requests are split by rows; 0: 2^24 */
} rq_server_config_t;
typedef struct rq_request_t {
  uint32_t mesh_id;
  uint32_t width, height, spp;
  rq_view_t view;              /* window and bounces are ignored */
  float background[3];
  uint32_t keep_pixels;        /* 1: keep width*height*3 bytes for rq_server_wait */
} rq_request_t;
typedef struct rq_server_stats_t {
  uint64_t submitted, completed, rejected;
  uint64_t batches, builds, evictions;
  uint64_t camera_rays, shadow_rays;
  uint64_t resident_bytes, resident_meshes;
  double busy_s;               /* worker time spent in steps */
  double latency_ms_p50, latency_ms_p99, latency_ms_mean, latency_ms_max;
} rq_server_stats_t;
/* cfg may be NULL (device 0, batching on, defaults). */
rq_status_t rq_server_create(const rq_server_config_t* cfg, rq_server_t* out);
/* Register a mesh (copied; validated: finite vertices, indices < nv). */
rq_status_t rq_server_add_mesh(rq_server_t s, uint32_t mesh_id, const float* verts, uint32_t nv,
                               const uint32_t* idx, uint32_t nt);
rq_status_t rq_server_submit(rq_server_t s, const rq_request_t* req, uint64_t* ticket);
/* Wait for a request (timeout_s < 0: no limit; RQ_ERROR_TIMEOUT when it runs
 * out), copy its pixels when it kept them, and forget the ticket.  Returns
 * the request's status. */
rq_status_t rq_server_wait(rq_server_t s, uint64_t ticket, uint8_t* pixels, double timeout_s);
/* Wait until every submitted request has completed. */
rq_status_t rq_server_drain(rq_server_t s, double timeout_s);
rq_status_t rq_server_get_stats(rq_server_t s, rq_server_stats_t* out);
rq_status_t rq_server_reset_stats(rq_server_t s);
/* Last device-side or CUDA error the worker met (empty when none). */
const char* rq_server_last_error(rq_server_t s);
/* Stops the worker after its current step; drain first. */
rq_status_t rq_server_destroy(rq_server_t s);

#ifdef __cplusplus
}
#endif
#endif /* RQ_H */
