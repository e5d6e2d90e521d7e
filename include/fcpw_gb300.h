/*
 * fcpw_gb300 — C ABI of the GB300-native GPU query path for FCPW scenes.
 *
 * Every entry point takes plain pointers and sizes and returns an int status
 * (FCPWGB_OK on success). A human-readable message for the last failure on the
 * calling thread is available from fcpwgb_last_error().
 *
 * The record types below are byte-identical to the interop structs of the
 * reference GPU path (include/fcpw/gpu/bvh_interop_structures.h:14-28,55-162,
 * 730-774), so arrays built for the reference's GPUScene can be passed as-is.
 *
 * Threading: like the reference ("GPU queries are not thread-safe",
 * include/fcpw/fcpw_gpu.h:30) a scene handle must not be used from two host
 * threads at once. Different handles are independent.
 */
#ifndef FCPW_GB300_H
#define FCPW_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#define FCPWGB_ALIGN8 alignas(8)
#else
#define FCPWGB_ALIGN8 _Alignas(8)
#endif

/* ---------------------------------------------------------------- status */
#define FCPWGB_OK                   0
#define FCPWGB_ERR_INVALID_ARGUMENT 1
#define FCPWGB_ERR_CUDA             2
#define FCPWGB_ERR_NOT_TRANSFERRED  3
#define FCPWGB_ERR_UNSUPPORTED      4
#define FCPWGB_ERR_OUT_OF_MEMORY    5
#define FCPWGB_ERR_TRAVERSAL        6 /* a device traversal overflowed its stack or step budget */

/* FCPW_GPU_UINT_MAX, include/fcpw/gpu/bvh_interop_structures.h:10 */
#define FCPWGB_UINT_MAX 4294967295u

/* BVH flavours, same numbering as FCPW_BVH_TYPE (include/fcpw/fcpw_gpu.inl:3-6) */
#define FCPWGB_LINE_SEGMENT_BVH  1
#define FCPWGB_TRIANGLE_BVH      2
#define FCPWGB_LINE_SEGMENT_SNCH 3
#define FCPWGB_TRIANGLE_SNCH     4

/* AggregateType numbering (include/fcpw/utilities/scene_data.h:17-24) */
#define FCPWGB_AGGREGATE_BASELINE              0
#define FCPWGB_AGGREGATE_BVH_LONGEST_AXIS      1
#define FCPWGB_AGGREGATE_BVH_OVERLAP_SURFACE   2
#define FCPWGB_AGGREGATE_BVH_SURFACE_AREA      3
#define FCPWGB_AGGREGATE_BVH_OVERLAP_VOLUME    4
#define FCPWGB_AGGREGATE_BVH_VOLUME            5

/* ------------------------------------------------------- record layouts */
typedef struct { FCPWGB_ALIGN8 float x; float y; } fcpwgb_float2;        /* 8 B, align 8 */
typedef struct { float x, y, z; } fcpwgb_float3;                          /* 12 B */

typedef struct { fcpwgb_float3 pMin, pMax; } fcpwgb_bounding_box;         /* 24 B */
typedef struct { fcpwgb_float3 axis; float halfAngle, radius; } fcpwgb_bounding_cone; /* 20 B */

typedef struct {                                                          /* 32 B, GPUBvhNode */
    fcpwgb_bounding_box box;
    uint32_t nPrimitives;
    uint32_t offset;          /* leaf: first primitive; inner: right-child offset (left = i + 1) */
} fcpwgb_bvh_node;

typedef struct {                                                          /* 60 B, GPUSnchNode */
    fcpwgb_bounding_box box;
    fcpwgb_bounding_cone cone;
    uint32_t nPrimitives;
    uint32_t offset;
    uint32_t nSilhouettes;
    uint32_t silhouetteOffset;
} fcpwgb_snch_node;

typedef struct { fcpwgb_float3 pa, pb; uint32_t index; } fcpwgb_line_segment;      /* 28 B */
typedef struct { fcpwgb_float3 pa, pb, pc; uint32_t index; } fcpwgb_triangle;      /* 40 B */
typedef struct { fcpwgb_float3 p, n0, n1; uint32_t index, hasOneAdjacentFace; } fcpwgb_vertex; /* 44 B */
typedef struct { fcpwgb_float3 pa, pb, n0, n1; uint32_t index, hasOneAdjacentFace; } fcpwgb_edge; /* 56 B */

typedef struct { fcpwgb_float3 o, d, dInv; float tMax; } fcpwgb_ray;               /* 40 B, GPURay */
typedef struct { fcpwgb_float3 c; float r2; } fcpwgb_bounding_sphere;              /* 16 B */

typedef struct {                                                          /* 40 B, GPUInteraction */
    fcpwgb_float3 p;
    fcpwgb_float3 n;
    fcpwgb_float2 uv;
    float d;
    uint32_t index;
} fcpwgb_interaction;

/* ------------------------------------------------------------- library */
const char *fcpwgb_last_error(void);
const char *fcpwgb_version(void);
/* number of CUDA devices visible (0 when none); never fails */
int fcpwgb_device_count(void);
/* Testing aid, injected on the host: after the next `skip` growths of a
 * device buffer succeed, the `count` growths after them fail with
 * FCPWGB_ERR_OUT_OF_MEMORY without calling the allocator, leaving the buffer
 * as it was ((0, 0) clears the injection). No device call is made or
 * faulted. The reference has no counterpart (its allocation failures exit
 * the process, slang_rhi_utils.h:51-59). */
int fcpwgb_debug_fail_allocations(int skip, int count);

/* ------------------------------------------------ CPU-side BVH producer
 * Builds the binary SAH BVH on the host exactly as the reference's
 * Scene<DIM>::build(aggregateType, vectorize=false) does for a single object
 * (include/fcpw/fcpw.inl:796-867,1053-1126; include/fcpw/aggregates/bvh.inl:40-234),
 * including the leaf-order vertex renumbering (fcpw.inl:613-758) and, when
 * with_silhouettes is set, the SNCH silhouette references and bounding cones
 * (fcpw.inl:405-521, bvh.inl:236-425). dim is 2 (line segments, indices has
 * 2 ints per primitive) or 3 (triangles, 3 ints per primitive). positions has
 * dim floats per vertex in the caller's vertex order.
 */
typedef struct fcpwgb_cpu_bvh fcpwgb_cpu_bvh;

typedef struct {
    int dim;
    int bvh_type;            /* FCPWGB_*_BVH / FCPWGB_*_SNCH */
    uint32_t n_nodes;
    uint32_t n_leaves;
    uint32_t max_depth;
    uint32_t n_primitives;
    uint32_t n_silhouettes;  /* silhouette references (SNCH only) */
    uint32_t n_vertices;
} fcpwgb_bvh_info;

int fcpwgb_cpu_bvh_build(int dim, const float *positions, uint32_t n_vertices,
                         const int32_t *indices, uint32_t n_primitives,
                         int aggregate_type, int with_silhouettes,
                         fcpwgb_cpu_bvh **out);
void fcpwgb_cpu_bvh_destroy(fcpwgb_cpu_bvh *bvh);
int fcpwgb_cpu_bvh_info(const fcpwgb_cpu_bvh *bvh, fcpwgb_bvh_info *info);
/* Writes the flattened tree in the reference interop layouts
 * (extractBvhNodes / extractSnchNodes / extractTriangles / extractLineSegments /
 * extractSilhouetteEdges / extractSilhouetteVertices,
 * bvh_interop_structures.h:172-298). nodes receives n_nodes fcpwgb_bvh_node
 * (BVH) or fcpwgb_snch_node (SNCH); primitives n_primitives triangles or
 * segments; silhouettes n_silhouettes edges or vertices (may be NULL for BVH).
 * Any output pointer may be NULL to skip it. */
int fcpwgb_cpu_bvh_export(const fcpwgb_cpu_bvh *bvh, void *nodes, void *primitives,
                          void *silhouettes);
/* index_map[v] = leaf-order position of caller vertex v (PolygonSoup::indexMap,
 * -1 for unreferenced vertices); prim_vertices[k*dim + j] = caller vertex
 * index of corner j of the k-th primitive in leaf order; prim_index[k] =
 * original primitive index; sil_vertices[s*(dim+1) + j] = caller vertex index
 * j of silhouette reference s (SilhouetteEdge::indices[4] /
 * SilhouetteVertex::indices[3], -1 where a face is missing). */
int fcpwgb_cpu_bvh_export_topology(const fcpwgb_cpu_bvh *bvh, int32_t *index_map,
                                   int32_t *prim_vertices, uint32_t *prim_index,
                                   int32_t *sil_vertices);
/* Collapses the host tree into the wide layout the GPU fast path uses
 * (branching 2/4/8, child boxes at 32/16/8 bits; the record format is
 * documented in fcpw_gb300/csrc/wide.h). Call with nodes == NULL to query
 * *n_nodes and *node_bytes; then pass buffers of n_nodes * node_bytes bytes
 * and n_nodes * branching int32 (child_binary: binary node behind every slot,
 * -1 for an empty slot). leaf_size as in fcpwgb_traversal_config. Returns
 * FCPWGB_ERR_UNSUPPORTED when the tree cannot be encoded. */
int fcpwgb_cpu_bvh_export_wide(const fcpwgb_cpu_bvh *bvh, int branching, int bits, int leaf_size, void *nodes,
                               int32_t *child_binary, uint32_t *n_nodes, uint32_t *node_bytes);
/* updateObjectVertices (fcpw.inl:1129-1143): replaces the vertex positions
 * (caller vertex order) so that a following export yields the moved
 * primitives and silhouettes. The tree itself is left unchanged. */
int fcpwgb_cpu_bvh_update_positions(fcpwgb_cpu_bvh *bvh, const float *positions);

/* ------------------------------------------------------------ GPU scene
 * Replaces fcpw::GPUScene<DIM> (include/fcpw/fcpw_gpu.h:8-91). One scene owns
 * one CUDA stream and its device buffers, reused across calls. */
typedef struct fcpwgb_gpu_scene fcpwgb_gpu_scene;

/* GPUScene ctor, fcpw_gpu.h:12 (the shader directory has no meaning here). */
int fcpwgb_gpu_scene_create(int dim, int device, fcpwgb_gpu_scene **out);
void fcpwgb_gpu_scene_destroy(fcpwgb_gpu_scene *scene);

/* transferToGPU, fcpw_gpu.h:21 / bvh_interop_structures.h:694-728: uploads a
 * flattened binary tree in the interop layouts. prim_vertices (optional, may
 * be NULL) lists the caller vertex index of every primitive corner in leaf
 * order, which enables fcpwgb_gpu_scene_update_vertices_device. */
int fcpwgb_gpu_scene_transfer(fcpwgb_gpu_scene *scene, int bvh_type,
                              const void *nodes, uint32_t n_nodes,
                              const void *primitives, uint32_t n_primitives,
                              const void *silhouettes, uint32_t n_silhouettes,
                              const int32_t *prim_vertices, uint32_t n_vertices);
/* convenience: transferToGPU straight from a host-built BVH */
int fcpwgb_gpu_scene_transfer_cpu_bvh(fcpwgb_gpu_scene *scene, const fcpwgb_cpu_bvh *bvh);

/* ----------------------------------------- several objects, instances
 * Scene<DIM> with several objects and instance transforms
 * (setObjectCount / setObjectInstanceTransforms, fcpw.h:29-70; the build,
 * fcpw.inl:1053-1102: one BVH per object, a TransformedAggregate per instance,
 * core/primitive.h:289-478, and a top-level BVH over the instances). The
 * reference's GPU path takes single-object scenes only (fcpw_gpu.h:17-20);
 * here such scenes run on the GPU too.
 *
 * fcpwgb_cpu_instances_build: objects are host-built trees (one per object,
 * fcpwgb_cpu_bvh_build), borrowed until fcpwgb_gpu_scene_transfer_instanced
 * returns. Instance i uses object instance_objects[i]; transforms (may be
 * NULL) hold dim x (dim + 1) floats per instance, the rows of the affine map
 * [A | b] from object to world space (uniform scale, as the reference
 * requires); transformed (may be NULL: all, when transforms are given) marks
 * the instances that use their transform; an untransformed instance is the
 * object itself, like an object without instance transforms in the
 * reference. Instances are listed in the reference's order: objects in turn,
 * an object's transforms in turn. The top-level tree is built with the
 * aggregate type's heuristic over the instance boxes (the object's root box,
 * or its eight corners mapped and widened by FLT_EPSILON) and centroids (the
 * mean primitive centroid, mapped), as the reference builds it; a single
 * instance has no top-level tree. */
typedef struct fcpwgb_cpu_instances fcpwgb_cpu_instances;
int fcpwgb_cpu_instances_build(int dim, int aggregate_type, const fcpwgb_cpu_bvh *const *objects,
                               uint32_t n_objects, const uint32_t *instance_objects,
                               const float *transforms, const uint32_t *transformed,
                               uint32_t n_instances, fcpwgb_cpu_instances **out);
void fcpwgb_cpu_instances_destroy(fcpwgb_cpu_instances *instances);
/* The top-level tree (n_top_nodes fcpwgb_bvh_node, 0 for a single instance),
 * its leaf references (instance indices, one per instance in leaf order) and
 * per instance 24 floats: the 3 x 4 rows of t, then of its inverse (2D: the
 * z row and column are the identity's). Any output may be NULL. */
int fcpwgb_cpu_instances_export(const fcpwgb_cpu_instances *instances, void *top_nodes, uint32_t *top_refs,
                                float *instance_matrices, uint32_t *n_top_nodes);
/* transferToGPU for such a scene: every object's tree is uploaded as by
 * fcpwgb_gpu_scene_transfer_cpu_bvh, with the instances and the top-level
 * tree. Closest point and ray queries (the regular entry points, and the
 * _instanced ones below that also give each answer's instance) then walk the
 * top-level tree in the reference's CPU order, each instance's object in
 * object space on its 4-wide tree (the configured box precision; branching
 * does not apply), with FP32 results like the reference's. The other query
 * kinds, refit and exports refuse such a scene (FCPWGB_ERR_UNSUPPORTED). */
int fcpwgb_gpu_scene_transfer_instanced(fcpwgb_gpu_scene *scene, const fcpwgb_cpu_instances *instances);
/* instance_out (may be NULL): the instance of each answer, FCPWGB_UINT_MAX
 * where nothing was found; interactions hold world-space points and normals
 * and the primitive index within the instance's object */
int fcpwgb_find_closest_points_instanced(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                         fcpwgb_interaction *interactions, uint32_t *instance_out, uint32_t n,
                                         int record_normals);
int fcpwgb_find_closest_points_instanced_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                                fcpwgb_interaction *interactions, uint32_t *instance_out,
                                                uint32_t n, int record_normals, void *stream);
int fcpwgb_intersect_rays_instanced(fcpwgb_gpu_scene *scene, const fcpwgb_ray *rays,
                                    fcpwgb_interaction *interactions, uint32_t *instance_out, uint32_t n,
                                    int check_for_occlusion);
int fcpwgb_intersect_rays_instanced_device(fcpwgb_gpu_scene *scene, const fcpwgb_ray *rays,
                                           fcpwgb_interaction *interactions, uint32_t *instance_out, uint32_t n,
                                           int check_for_occlusion, void *stream);
/* Sphere sampling and closest silhouette points on a scene of several objects
 * or instances: the reference CPU's stochastic top-level descent with
 * aggregate leaves (include/fcpw/aggregates/bvh.inl:1140-1288; every instance
 * in the chosen leaf sampled with the current random number, one of those
 * that hit chosen uniformly) and its silhouette walk (bvh.inl:1435-1596), each
 * instance through TransformedAggregate (include/fcpw/core/primitive.h:392-466:
 * query and minimum radius to object space, the object's own tree, the answer
 * back to world space; a sample keeps its object-space pdf). Silhouette
 * queries need every object built with silhouettes, else every result keeps
 * its default record. instance_out (may be NULL) receives each answer's
 * instance (UINT_MAX when none). The regular fcpwgb_intersect_spheres* and
 * fcpwgb_find_closest_silhouette_points* entry points route here too. */
int fcpwgb_intersect_spheres_instanced(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                       const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out,
                                       uint32_t *instance_out, uint32_t n);
int fcpwgb_intersect_spheres_instanced_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                              const fcpwgb_float3 *rand_nums, fcpwgb_interaction *out,
                                              uint32_t *instance_out, uint32_t n, void *stream);
int fcpwgb_find_closest_silhouette_points_instanced(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                                    const uint32_t *flip, fcpwgb_interaction *out,
                                                    uint32_t *instance_out, uint32_t n, float squared_min_radius,
                                                    float precision);
int fcpwgb_find_closest_silhouette_points_instanced_device(fcpwgb_gpu_scene *scene,
                                                           const fcpwgb_bounding_sphere *spheres,
                                                           const uint32_t *flip, fcpwgb_interaction *out,
                                                           uint32_t *instance_out, uint32_t n,
                                                           float squared_min_radius, float precision, void *stream);
/* Refit of one object of an instanced scene without a new transfer
 * (Scene::updateObjectVertices + Scene::refit, include/fcpw/fcpw.inl:1146-1158,
 * bvh.inl:548-599): the object's tree is refit from the given records
 * (primitives / silhouettes in its leaf order, NULL = its device geometry as
 * it is; as fcpwgb_gpu_scene_refit), or from device vertex positions in the
 * object's own vertex order (as fcpwgb_gpu_scene_update_vertices_device, on
 * stream), then the top level: every instance's box is its object's new root
 * box mapped by its transform, and the top-level nodes are their unions. The
 * object is shared by all its instances. */
int fcpwgb_gpu_scene_refit_object(fcpwgb_gpu_scene *scene, uint32_t object, const void *primitives,
                                  const void *silhouettes);
int fcpwgb_gpu_scene_update_object_vertices_device(fcpwgb_gpu_scene *scene, uint32_t object, const float *positions,
                                                   uint32_t n_vertices, void *stream);
/* The device's top-level tree of an instanced scene (32 B interop nodes, leaf
 * references are instance indices): n_nodes receives the count, nodes (may be
 * NULL) the records; synchronous. No counterpart in the reference's GPU path. */
int fcpwgb_gpu_scene_export_top_nodes(fcpwgb_gpu_scene *scene, void *nodes, uint32_t *n_nodes);

/* Scene::build(AggregateType::Bvh, ...) + transferToGPU (fcpw.h:95,
 * fcpw_gpu.h:21) with the tree built on the device: a linear BVH over the
 * Morton codes of the primitive centroids (30-bit in 3D, 32-bit in 2D),
 * subtrees of at most max_leaf_size (1..15) primitives merged into leaves,
 * boxes widened by FLT_EPSILON per vertex as the host build does. The tree
 * differs from the host SAH build, so query results agree with it in
 * distance but may pick another primitive on ties; the scene is set up
 * through fcpwgb_gpu_scene_transfer (with prim_vertices, so device vertex
 * updates work). BVH only, no silhouettes. positions: n_vertices * dim
 * floats, indices: n_primitives * dim. The _device form takes device arrays
 * and builds on stream (NULL: the scene's stream); both return when the scene
 * is ready. */
int fcpwgb_gpu_scene_build(fcpwgb_gpu_scene *scene, const float *positions, uint32_t n_vertices,
                           const int32_t *indices, uint32_t n_primitives, uint32_t max_leaf_size);
/* Scene::build(aggregate_type, vectorize=false) + transferToGPU (fcpw.h:95,
 * fcpw_gpu.h:21) with the reference's binned SAH build (bvh.inl:1-234: 8
 * buckets, leaf <= 4, depth cut at 62; aggregate_type one of the Bvh_* types)
 * run on the device: the tree and the primitive order equal the host build's
 * (fcpwgb_cpu_bvh_build, and so the reference's) byte for byte. BVH only, no
 * silhouettes. Same arrays, streams and return as fcpwgb_gpu_scene_build. */
int fcpwgb_gpu_scene_build_sah(fcpwgb_gpu_scene *scene, const float *positions, uint32_t n_vertices,
                               const int32_t *indices, uint32_t n_primitives, int aggregate_type);
int fcpwgb_gpu_scene_build_sah_device(fcpwgb_gpu_scene *scene, const float *positions, uint32_t n_vertices,
                                      const int32_t *indices, uint32_t n_primitives, int aggregate_type,
                                      void *stream);
int fcpwgb_gpu_scene_build_device(fcpwgb_gpu_scene *scene, const float *positions, uint32_t n_vertices,
                                  const int32_t *indices, uint32_t n_primitives, uint32_t max_leaf_size,
                                  void *stream);

/* refit, fcpw_gpu.h:27 / bvh_interop_structures.h:891-934. When primitives
 * (and, for SNCH, silhouettes) are non-NULL they replace the device copies
 * first (updateGeometry=true); with NULL the device geometry is refit as is
 * (updateGeometry=false). Bottom-up in a single launch. Synchronous. */
int fcpwgb_gpu_scene_refit(fcpwgb_gpu_scene *scene, const void *primitives,
                           const void *silhouettes);
/* Device-side geometry update + refit for differentiable pipelines: positions
 * is a device array of n_vertices*dim floats in caller vertex order. The
 * primitive (and silhouette) records are regathered on the device and the
 * tree refit; asynchronous on stream (a cudaStream_t; NULL is the CUDA default stream). */
int fcpwgb_gpu_scene_update_vertices_device(fcpwgb_gpu_scene *scene, const float *positions,
                                            uint32_t n_vertices, void *stream);
/* No counterpart in the reference. The same update + refit as
 * fcpwgb_gpu_scene_update_vertices_device for callers that may not allocate
 * device memory: the call performs no cudaMalloc/cudaFree and no other
 * allocation; the refit's per-node arrival counters live in a static device
 * array of 2^20 32-bit words (4 MiB, held on every GPU that loads the library
 * until the process exits). Trees with more than 1,048,576 nodes are rejected
 * with FCPWGB_ERR_INVALID_ARGUMENT. Each call clears the counters it uses;
 * the array is shared by all calls on a device, so calls that overlap on the
 * GPU (other streams, scenes or threads) race and must be ordered by the
 * caller. The array's device address is looked up (and the code holding it
 * loaded, which is when the 4 MiB is reserved) while the scene is
 * transferred, not in this call; after a cudaDeviceReset the scene must be
 * transferred again, as for any of its device buffers. Status codes and
 * their order of checks are those of fcpwgb_gpu_scene_update_vertices_device.
 * Asynchronous on stream (NULL is the CUDA default stream). */
int fcpwgb_gpu_scene_update_vertices_device_static(fcpwgb_gpu_scene *scene, const float *positions,
                                                   uint32_t n_vertices, void *stream);
/* Testing aid (no counterpart in the reference): writes `word` into the first
 * n words of the static refit array on the scene's device, synchronously,
 * without allocating device memory; a test uses it to check that
 * fcpwgb_gpu_scene_update_vertices_device_static clears what it reads. */
int fcpwgb_debug_fill_static_scratch(fcpwgb_gpu_scene *scene, uint32_t word, uint32_t n);

/* Traversal variant used by the closest point entry points of a scene. With
 * branching 0 the transferred binary tree is traversed in the reference GPU
 * order (bvh.slang:395-502). With branching 2, 4 or 8 a wide tree is derived
 * from it (children of largest surface area expanded first) whose child boxes
 * are stored in 32-bit floats or conservatively quantised to 16 or 8 bits;
 * sort_queries reorders each batch spatially before traversal, persistent
 * runs one resident block set that fetches query chunks from a counter, and
 * precise recomputes the winning primitive's distance and point (and the
 * runner-up's within the FP32 rounding band) to within 1e-6 of FP64:
 * double-single arithmetic, FP64 where the projection is ill-conditioned;
 * for triangles in a second kernel after the traversal, for segments at its
 * end;
 * packet traverses the 32 (sorted) queries of a warp together, one record
 * load per warp and step, each query pruning with its own radius (with
 * persistent, one resident wave of blocks whose warps take the next 32
 * queries from a counter as soon as their packet is done); leaf_size > 0 collapses binary subtrees of at most that
 * many primitives (up to 15) into one wide leaf; short_stack is the number of
 * traversal-stack entries per thread kept in shared memory by the
 * one-thread-per-query schedules (0 or 16; the others in local memory);
 * threads_per_query > 1 answers each query with a group of that many
 * consecutive lanes (2, 4 or 8): the lanes split the child boxes of every
 * record and the primitives of every leaf and combine their candidates by
 * shuffles (not with packet; persistent is then ignored).
 * Defaults: {0, 32, 128, 1, 1, 1, 0, 0, 16, 1}. Results differ from the binary
 * order only on equidistant ties (and, with precise, by the FP32 rounding
 * removed). With branching > 0, closest silhouette points are answered by
 * warp packets on the binary SNCH tree (unless squared_min_radius > 0),
 * contains sorts its points spatially (sort_queries), and rays are sorted by
 * direction octant, then origin (sort_queries), except with persistent (and
 * not packet): a persistent wave of lanes then takes the rays in the
 * caller's order, each lane the next ray as soon as its own is done. */
typedef struct {
    int branching;     /* 0, 2, 4 or 8 */
    int bits;          /* 32, 16 or 8 */
    int block_size;    /* threads per block of the wide kernels (128) */
    int sort_queries;  /* 0 or 1 */
    int persistent;    /* 0 or 1 */
    int precise;       /* 0 or 1 */
    int packet;        /* 0 or 1 */
    int leaf_size;     /* 0 (binary leaves) or 1..15 */
    int short_stack;   /* 0 or 16 */
    int threads_per_query; /* 1, 2, 4 or 8 */
} fcpwgb_traversal_config;
int fcpwgb_gpu_scene_set_traversal(fcpwgb_gpu_scene *scene, const fcpwgb_traversal_config *config);
int fcpwgb_gpu_scene_get_traversal(const fcpwgb_gpu_scene *scene, fcpwgb_traversal_config *config);

/* ----- queries with HOST arrays (synchronous, as the reference) ----- */
/* findClosestPoints, fcpw_gpu.h:60-62. In precise mode on triangles with a
 * fast-path configuration (sorted queries, n >= 4096) and a page-locked
 * interactions array starting on a 16 B boundary, the records are written
 * into that array by the device directly; otherwise they are copied back. */
int fcpwgb_find_closest_points(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                               fcpwgb_interaction *interactions, uint32_t n, int record_normals);
/* intersect(rays), fcpw_gpu.h:38-40 */
int fcpwgb_intersect_rays(fcpwgb_gpu_scene *scene, const fcpwgb_ray *rays,
                          fcpwgb_interaction *interactions, uint32_t n, int check_for_occlusion);
/* intersect(spheres, randNums), fcpw_gpu.h:50-52 */
int fcpwgb_intersect_spheres(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                             const fcpwgb_float3 *rand_nums, fcpwgb_interaction *interactions,
                             uint32_t n);
/* findClosestSilhouettePoints, fcpw_gpu.h:73-76 */
int fcpwgb_find_closest_silhouette_points(fcpwgb_gpu_scene *scene,
                                          const fcpwgb_bounding_sphere *spheres,
                                          const uint32_t *flip_normal_orientation,
                                          fcpwgb_interaction *interactions, uint32_t n,
                                          float squared_min_radius, float precision);

/* ----- queries with DEVICE arrays: asynchronous on stream (a cudaStream_t, used as
 * given; NULL is the CUDA default stream, as for any CUDA runtime call).
 * Sphere arrays must start on a 16 B boundary, ray and interaction arrays on
 * an 8 B boundary, flag arrays on 4 B (cudaMalloc'd arrays and every element
 * of them do); otherwise FCPWGB_ERR_INVALID_ARGUMENT, before any launch. ----- */
int fcpwgb_find_closest_points_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                      fcpwgb_interaction *interactions, uint32_t n,
                                      int record_normals, void *stream);
int fcpwgb_intersect_rays_device(fcpwgb_gpu_scene *scene, const fcpwgb_ray *rays,
                                 fcpwgb_interaction *interactions, uint32_t n,
                                 int check_for_occlusion, void *stream);
int fcpwgb_intersect_spheres_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                    const fcpwgb_float3 *rand_nums,
                                    fcpwgb_interaction *interactions, uint32_t n, void *stream);
int fcpwgb_find_closest_silhouette_points_device(fcpwgb_gpu_scene *scene,
                                                 const fcpwgb_bounding_sphere *spheres,
                                                 const uint32_t *flip_normal_orientation,
                                                 fcpwgb_interaction *interactions, uint32_t n,
                                                 float squared_min_radius, float precision,
                                                 void *stream);

/* Runs the closest point query of the scene's current variant over device
 * spheres in counting mode and returns, synchronously, eight counters:
 * stats[0] = queries, stats[1] = popped (loaded) binary nodes, stats[2] =
 * expanded inner records, stats[3] = primitive tests (the last three summed
 * over all queries), stats[4] = record loads and stats[5] = primitive loads
 * of the warp-packet kernel (one per warp and step), stats[6..7] = 0. Used
 * to compute the algorithmic bytes of a launch; results are written to
 * interactions. */
int fcpwgb_closest_points_traversal_stats(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                          fcpwgb_interaction *interactions, uint32_t n, uint64_t stats[8]);

/* Like fcpwgb_closest_points_traversal_stats, it runs on the scene's own
 * stream and uses the scene's scratch arrays: the caller's earlier work on the
 * scene must have completed.
 * Runs fcpwgb_find_closest_silhouette_points_device's warp-packet path (a
 * fast-path configuration and squared_min_radius <= 0, else
 * FCPWGB_ERR_UNSUPPORTED) over device arrays in counting mode and returns,
 * synchronously: stats[0] = queries, stats[1] = warp steps at an inner node
 * (two 64 B child records loaded), stats[2] = warp steps at a leaf,
 * stats[3] = silhouette records loaded by warps, stats[4] = child tests and
 * stats[5] = silhouette tests of the queries (lanes), stats[6..7] = 0. Used
 * to compute the algorithmic bytes of a launch; results are written to
 * interactions. */
int fcpwgb_silhouette_traversal_stats(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                      const uint32_t *flip_normal_orientation, fcpwgb_interaction *interactions,
                                      uint32_t n, float squared_min_radius, float precision, uint64_t stats[8]);

/* ----- differentiation (no counterpart in the reference; needs a tree
 * transferred with prim_vertices). Device arrays, asynchronous on stream. ----- */
/* Backward of the unsigned closest point distance d(x) = |x - p(x, V)| from
 * the forward records of fcpwgb_find_closest_points_device: writes
 * grad_x = dL/dx (n x dim) and grad_vertices = dL/dV (n_vertices x dim, the
 * caller's vertex order), given grad_d = dL/dd. Queries without a hit or at
 * distance 0 contribute nothing. The vertex reduction is deterministic. */
int fcpwgb_closest_point_backward_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                         const fcpwgb_interaction *forward, const float *grad_d, uint32_t n,
                                         float *grad_x, float *grad_vertices, void *stream);
/* Backward of the ray hit distance t(o, dir, V) from the forward records of
 * fcpwgb_intersect_rays_device: writes dL/do, dL/ddir (n x dim) and dL/dV. */
int fcpwgb_ray_backward_device(fcpwgb_gpu_scene *scene, const fcpwgb_ray *rays, const fcpwgb_interaction *forward,
                               const float *grad_t, uint32_t n, float *grad_o, float *grad_dir,
                               float *grad_vertices, void *stream);

/* Kernel timing: when enabled, every closest point traversal launch of the
 * scene is bracketed by CUDA events recorded on its stream.
 * fcpwgb_gpu_scene_kernel_time synchronises on the recorded events and
 * returns (then clears) the summed duration in ms and the number of launches. */
int fcpwgb_gpu_scene_enable_kernel_timing(fcpwgb_gpu_scene *scene, int enable);
int fcpwgb_gpu_scene_kernel_time(fcpwgb_gpu_scene *scene, double *total_ms, uint32_t *launches);

/* Copies the scene's current (possibly refit) binary tree back to the host in
 * the interop layout it was transferred in (fcpwgb_bvh_node or
 * fcpwgb_snch_node records, n_nodes of them). Synchronous. */
int fcpwgb_gpu_scene_export_nodes(fcpwgb_gpu_scene *scene, void *nodes);
/* Sizes of the scene's binary tree: *info receives the fcpwgb_bvh_info fields
 * (dim, bvh_type, n_nodes, n_leaves, max_depth, n_primitives, n_silhouettes,
 * n_vertices), however the tree got there (transfer, file or GPU build). */
int fcpwgb_gpu_scene_info(fcpwgb_gpu_scene *scene, fcpwgb_bvh_info *info);

/* Reads and clears the device error word of the scene (stack overflow or
 * step budget exhausted in a traversal). Synchronises the scene stream. */
int fcpwgb_gpu_scene_check_errors(fcpwgb_gpu_scene *scene, uint32_t *error_word);

/* No counterpart in the reference: the FP64 closest distance of every query
 * (its centre; r2 is ignored) over ALL primitives of the scene, by brute
 * force, for measuring the distance error of any traversal variant. Device
 * arrays, asynchronous on stream; O(n x primitives), n <= 2^24. */
int fcpwgb_closest_distances_f64_device(fcpwgb_gpu_scene *scene, const fcpwgb_bounding_sphere *spheres,
                                        uint32_t n, double *distances, void *stream);

/* ----------------------------------------------------- scene files ----- */
/* No counterpart in the reference. A scene file holds a host-built tree in
 * the interop layouts (nodes, primitives, silhouettes), its topology, and the
 * wide trees of the n_wide given traversal configurations (branching, bits
 * and leaf_size are used), with a checksum. fcpwgb_gpu_scene_load uploads it
 * through the validating transfer and keeps the wide trees for the matching
 * configurations, so neither the CPU build nor the wide collapse runs. */
int fcpwgb_cpu_bvh_save(const fcpwgb_cpu_bvh *bvh, const char *path, const fcpwgb_traversal_config *wide,
                        uint32_t n_wide);
int fcpwgb_gpu_scene_load(fcpwgb_gpu_scene *scene, const char *path);
/* Reads and checks a scene file's header and checksum: the counts in info
 * (n_leaves and max_depth are 0), the number of wide trees in *n_wide. */
int fcpwgb_scene_file_info(const char *path, fcpwgb_bvh_info *info, uint32_t *n_wide);

/* ------------------------------------------- inside / line of sight ----- */
/* Scene<DIM>::contains and hasLineOfSight (fcpw.inl:1443-1460, 1501-1520;
 * Aggregate::contains / hasLineOfSight, core/primitive.h:173-207), CPU-only in
 * the reference, as GPU batches over the transferred binary tree with the
 * reference CPU arithmetic (results equal the reference's). contains: 1 when
 * rays from the point along +x and +y both cross the boundary an odd number
 * of times (a watertight boundary is assumed, as in the reference), else 0;
 * 2 when a ray had more than 64 hits. has_line_of_sight: 1 when the segment
 * from points_a[i] to points_b[i] hits no primitive. Points are 3 floats (z
 * ignored in 2D). Host arrays: synchronous; _device: asynchronous on stream. */
int fcpwgb_contains(fcpwgb_gpu_scene *scene, const fcpwgb_float3 *points, uint32_t n, uint32_t *result);
int fcpwgb_contains_device(fcpwgb_gpu_scene *scene, const fcpwgb_float3 *points, uint32_t n, uint32_t *result,
                           void *stream);
int fcpwgb_has_line_of_sight(fcpwgb_gpu_scene *scene, const fcpwgb_float3 *points_a,
                             const fcpwgb_float3 *points_b, uint32_t n, uint32_t *result);
int fcpwgb_has_line_of_sight_device(fcpwgb_gpu_scene *scene, const fcpwgb_float3 *points_a,
                                    const fcpwgb_float3 *points_b, uint32_t n, uint32_t *result, void *stream);

/* ------------------------------------------------- batches of scenes ----- */
/* No counterpart in the reference (its GPUScene holds one object). A batch
 * holds many scenes of uneven size; the closest points of all their query
 * sets are found by one persistent launch over a forest of wide trees,
 * replayed from a captured CUDA graph. Queries arrive grouped by scene: those
 * of scene s are spheres[query_offsets[s] .. query_offsets[s+1]) and their
 * interaction indices are primitive indices of scene s. Not thread-safe. */
typedef struct fcpwgb_gpu_batch fcpwgb_gpu_batch;
int fcpwgb_gpu_batch_create(int dim, int device, fcpwgb_gpu_batch **out);
void fcpwgb_gpu_batch_destroy(fcpwgb_gpu_batch *batch);
/* Copies the trees and primitives of n_scenes host-built BVHs (the handles
 * may be destroyed afterwards). */
int fcpwgb_gpu_batch_set_scenes(fcpwgb_gpu_batch *batch, const fcpwgb_cpu_bvh *const *bvhs, uint32_t n_scenes);
/* branching 2/4/8 and bits 8/16/32 (default 8 and 8), persistent, precise;
 * queries are always sorted. The forest is rebuilt on the next query when
 * branching or bits change. */
int fcpwgb_gpu_batch_set_traversal(fcpwgb_gpu_batch *batch, const fcpwgb_traversal_config *config);
int fcpwgb_gpu_batch_get_traversal(const fcpwgb_gpu_batch *batch, fcpwgb_traversal_config *config);
/* Graph replay on (default) or off: with it on, the first call with a given
 * set of arrays, query layout and traversal captures the call's work in a
 * CUDA graph and later identical calls launch that graph. */
int fcpwgb_gpu_batch_use_graph(fcpwgb_gpu_batch *batch, int on);
/* query_offsets: host array of n_offsets = n_scenes + 1 non-decreasing
 * entries, query_offsets[0] = 0. Device arrays, asynchronous on stream. */
int fcpwgb_gpu_batch_find_closest_points_device(fcpwgb_gpu_batch *batch, const fcpwgb_bounding_sphere *spheres,
                                                const uint32_t *query_offsets, uint32_t n_offsets,
                                                fcpwgb_interaction *interactions, int record_normals,
                                                void *stream);
/* Host arrays, synchronous. */
int fcpwgb_gpu_batch_find_closest_points(fcpwgb_gpu_batch *batch, const fcpwgb_bounding_sphere *spheres,
                                         const uint32_t *query_offsets, uint32_t n_offsets,
                                         fcpwgb_interaction *interactions, int record_normals);
/* Device arrays, synchronous: the eight counters of
 * fcpwgb_closest_points_traversal_stats for one batched launch. */
int fcpwgb_gpu_batch_traversal_stats(fcpwgb_gpu_batch *batch, const fcpwgb_bounding_sphere *spheres,
                                     const uint32_t *query_offsets, uint32_t n_offsets,
                                     fcpwgb_interaction *interactions, uint64_t stats[8]);
int fcpwgb_gpu_batch_info(const fcpwgb_gpu_batch *batch, uint32_t *n_scenes, uint32_t *n_wide_nodes,
                          uint32_t *n_primitives, uint32_t *n_sort_cells);
int fcpwgb_gpu_batch_check_errors(fcpwgb_gpu_batch *batch, uint32_t *error_word);

#ifdef __cplusplus
}
#endif
#endif /* FCPW_GB300_H */
