/*
 * mcgpu.h — C ABI of the GB300 marching-cubes library (libmcgpu.so).
 *
 * This is the drop-in boundary for model3d's MarchingCubesSearch path
 * (model3d/mc.go:45-49).  A host-language wrapper (a Go cgo binding, the
 * Python mirror in model3d_gb300/, or a C++ caller) serialises its Solid tree
 * into an array of mc_node records, the library lowers it to a device
 * program (CSG bytecode; collider meshes as the reference's BVH boxes plus a
 * ray grid of candidate triangles), runs corner classification, cube
 * classification, compaction and the edge bisection search on one GPU, and
 * returns an indexed mesh.
 *
 * Plain C types only: pointers and sizes.  Inputs are borrowed for the
 * duration of a call.  Solids that cannot be lowered return
 * MC_ERR_NOT_LOWERABLE; there is no CPU fallback.
 *
 * Threading: one mc_ctx per host thread.  Each context owns a CUDA stream
 * and grow-only device buffers; every call is synchronous on return.  Destroy
 * a context's solids before the context (mc_solid_destroy may run on any
 * thread); a solid that outlives its context is detached by mc_destroy and
 * can still be destroyed, but not used.
 */
#ifndef MCGPU_H
#define MCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */

typedef enum mc_status {
    MC_OK = 0,
    /* validateBounds panic "invalid bounds: ..." (model3d/bounder.go:48-52). */
    MC_ERR_INVALID_BOUNDS = 1,
    /* solidCache.FetchZ panic "solid is true outside of bounds" (model3d/mc.go:687-689). */
    MC_ERR_BOUNDS_INSIDE = 2,
    /* squareSpacer.LookupEdgePoint panic "vertex not on edge" (model3d/mc.go:659). */
    MC_ERR_NOT_ON_EDGE = 3,
    /* LookupEdgePoint computed an index past the spacer array; Go raises an
     * index-out-of-range runtime panic there (model3d/mc.go:655-656). */
    MC_ERR_EDGE_INDEX = 4,
    /* Malformed node array (bad child counts, unknown kind, bad mesh index). */
    MC_ERR_BAD_PROGRAM = 5,
    /* A node kind or mode that has no device lowering (e.g. an inset collider). */
    MC_ERR_NOT_LOWERABLE = 6,
    MC_ERR_OOM = 7,
    /* A bounded device-side wait ran out (never used to cover a fault). */
    MC_ERR_TIMEOUT = 8,
    MC_ERR_CUDA = 9,
    MC_ERR_ARG = 10,
    /* The spacer loop would not terminate (x += delta leaves x unchanged, or
     * delta <= 0 / NaN) or the grid exceeds the library's size limit. */
    MC_ERR_GRID = 11,
    /* The program exceeds a device limit (stack depth, leaf count). */
    MC_ERR_LIMIT = 12
} mc_status;

/* ---------------------------------------------------------------- the scene */

/* Node kinds.  Values are part of the ABI. */
enum {
    /* Leaves (n_children == 0). */
    MC_NODE_SPHERE = 1,    /* p = Center.xyz, Radius                (model3d/shapes.go:13-31)   */
    MC_NODE_RECT = 2,      /* p = MinVal.xyz, MaxVal.xyz            (model3d/shapes.go:145-173) */
    MC_NODE_CYLINDER = 3,  /* p = P1.xyz, P2.xyz, Radius            (model3d/shapes.go:542-598) */
    MC_NODE_CAPSULE = 4,   /* p = P1.xyz, P2.xyz, Radius            (model3d/shapes.go:348-368) */
    MC_NODE_TORUS = 5,     /* p = Center.xyz, Axis.xyz, Outer, Inner (model3d/shapes.go:1323-1365) */
    MC_NODE_COLLIDER = 6,  /* NewColliderSolid(collider) over triangle set `mesh`
                              (model3d/solid.go:247-305, collisions.go:119-212) */
    MC_NODE_METABALL = 7,  /* WeightedMetaballSolid(f, radiusThreshold, balls, weights)
                              (model3d/metaball.go:165-242): min/max = its bounds (the
                              outset box, computed by the caller as the reference does);
                              p = radiusThreshold, MC_FALLOFF_*, falloff parameter;
                              n_children MC_NODE_BALL records follow.  With no positive
                              weight the reference returns NewRect(Origin, Origin), and
                              so does the library. */
    MC_NODE_BALL = 8,      /* One metaball term (only as a child of MC_NODE_METABALL):
                              p[0] = weight; n_steps MC_XF_* records follow (the forward
                              transform of TransformMetaball / VecScaleMetaball, innermost
                              first, model3d/transform.go:319-414), then one SPHERE, RECT,
                              CYLINDER, CAPSULE or TORUS record whose MetaballField is
                              -SDF (shapes.go:100, :255, :466, :712, :1431). */
    /* Combinators. */
    MC_NODE_JOIN = 16,      /* JoinedSolid, n_children >= 1      (model3d/solid.go:71-98)    */
    MC_NODE_SUBTRACT = 17,  /* SubtractedSolid, children = Positive, Negative (solid.go:120-142) */
    MC_NODE_INTERSECT = 18, /* IntersectedSolid, n_children >= 1 (model3d/solid.go:144-172)  */
    MC_NODE_TRANSFORM = 19, /* TransformSolid(t, child): n_steps MC_XF_* records follow the node,
                               then the child (model3d/transform.go:240-247).  The steps are
                               the FORWARD transform t in JoinedTransform order; the library
                               computes t.Inverse() itself. */
    MC_NODE_CHECKED = 20,   /* CheckedFuncSolid(min, max, child.Contains), as made by
                               CacheSolidBounds / ForceSolidBounds (model3d/solid.go:46-50,
                               :294-318); one child. */
    /* Transform steps (only directly after a MC_NODE_TRANSFORM node). */
    MC_XF_TRANSLATE = 32,   /* p = Offset.xyz   (model3d/transform.go:40-58)   */
    MC_XF_SCALE = 33,       /* p = Scale        (model3d/transform.go:67-89)   */
    MC_XF_VECSCALE = 34,    /* p = Scale.xyz    (model3d/transform.go:100-118) */
    MC_XF_MATRIX = 35,      /* p = Matrix3, row-major (model3d/transform.go:127-157; Rotation
                               and Mirror are Matrix3 transforms as well) */
    /* Falloff functions of MC_NODE_METABALL (p[1]); p[2] is the parameter. */
    MC_FALLOFF_POWER = 1,   /* InversePowerMetaballFalloffFunc(p[2]), p[2] a positive integer
                               below 2^20: math.Pow(r, -p[2]), +Inf for r <= 0
                               (model3d/metaball.go:17-28; Linear..Quintic are 1..5) */
    MC_FALLOFF_WYVILL = 2   /* WyvillMetaballFalloffFunc(p[2]) (model3d/metaball.go:86-103).
                               Exponential and Gaussian falloffs call math.Exp, which Go
                               implements per architecture in assembly: not lowerable. */
};

/*
 * One record of the prefix-order serialisation of a Solid tree: a node, then
 * (for MC_NODE_TRANSFORM and MC_NODE_BALL) its n_steps transform-step records, then its
 * children, each serialised the same way.
 *
 * min/max are the node's Min()/Max() exactly as the host language computed
 * them; the library uses the root's bounds for the spacer and the bounds of
 * TRANSFORM / CHECKED / COLLIDER / METABALL nodes for their containment checks, so that
 * the grid is bit-identical to the caller's own newSquareSpacer.  The bounds
 * of other non-root nodes are not read and may be left zero.
 */
typedef struct mc_node {
    int32_t kind;
    int32_t n_children;
    int32_t n_steps;  /* MC_NODE_TRANSFORM / MC_NODE_BALL: number of MC_XF_* records that follow */
    int32_t mesh;     /* MC_NODE_COLLIDER: index into the mc_tri_set array */
    double min[3];
    double max[3];
    double p[12];
} mc_node;

/*
 * Triangle set behind a MC_NODE_COLLIDER.  tris holds n triangles of three
 * vertices of three float64 each (row-major, n x 9).
 *   grouped == 0: the collider is MeshToCollider(mesh) — the library applies
 *                 GroupTriangles to the given order (model3d/collisions.go:138-142);
 *   grouped == 1: the order is already grouped and the collider is
 *                 GroupedTrianglesToCollider(tris) (model3d/collisions.go:169-181).
 */
typedef struct mc_tri_set {
    const double* tris;
    int64_t n;
    int32_t grouped;
    int32_t reserved;
} mc_tri_set;

/* --------------------------------------------------------------- options */

enum {
    MC_PREC_FP64 = 0,          /* every predicate in FP64, reference operation order */
    MC_PREC_FP32_FILTERED = 1  /* FP32 predicate with a forward error bound; FP64 when it cannot decide */
};

typedef struct mc_opts {
    int32_t precision;  /* MC_PREC_* (default MC_PREC_FP32_FILTERED) */
    int32_t cull;       /* 1: per-tile bounding-box culling of leaves (default); 0: off */
    int32_t tile_y;     /* corner-tile height in y (0: tuned default) */
    int32_t tile_z;     /* corner-tile depth in z (0: tuned default) */
    int32_t interior;   /* 1: also record each vertex's interior point (MarchingCubesInterior,
                           model3d/mc.go:55-60) for mc_result_interior_copy; mc_search_device
                           and mc_search only (ignored by the batch call; the allocation-free
                           call returns MC_ERR_ARG) */
    int32_t z_begin;    /* z-slab of one solid: cube layers [z_begin, z_end) of the solid's */
    int32_t z_end;      /* grid, on corner planes z_begin..z_end (z_end == 0: the whole grid).
                           The spacer, LookupEdgePoint and the border check stay those of the
                           whole grid, so the slabs of a partition, meshed separately, give the
                           whole mesh once the vertices that two neighbouring slabs share (the
                           x and y edges of their common corner plane, equal bit for bit) are
                           merged.  mc_search_device / mc_search only (the batch and the
                           allocation-free calls return MC_ERR_ARG).  No counterpart in the
                           reference: its z-slab ring runs inside one call (mc.go:614-645). */
    int32_t reserved;
} mc_opts;

typedef struct mc_stats {
    int64_t nx, ny, nz;      /* spacer sizes */
    int64_t corners;         /* nx*ny*nz */
    int64_t vertices;        /* unique edge vertices */
    int64_t triangles;
    int64_t leaf_evals;      /* leaf predicate evaluations (classification + search) */
    int64_t escalations;     /* FP32 evaluations that fell back to FP64 */
    int64_t tiles;           /* corner tiles classified */
    int64_t tiles_const;     /* tiles decided without evaluating any leaf */
    int64_t bvh_nodes;       /* collider: BVH nodes whose box was tested */
    int64_t bvh_tris;        /* collider: ray-triangle tests */
    double ms_classify;      /* device time per phase (CUDA events on the context's stream) */
    double ms_count;         /* cube classification + prefix sums */
    double ms_emit;          /* vertex / triangle emission */
    double ms_search;        /* edge bisection */
    double ms_total;         /* first upload to last kernel, including the totals read-back */
    int64_t h2d_bytes;       /* host-to-device bytes of the call */
    int64_t d2h_bytes;       /* device-to-host bytes of the call (incl. the mesh for mc_search) */
    int64_t flops_classify;  /* float operations of the reference formulas of the leaves the */
    int64_t flops_search;    /* classification / search evaluated (Sphere 10, Rect 6, Cylinder and
                                Capsule 23, Torus 36 per evaluation; colliders and metaballs 0) */
} mc_stats;

/* Indexed mesh: vertices n_vertices x 3 float64, triangles n_triangles x 3
 * vertex indices in the lookup-table vertex order (model3d/mc.go:401-407). */
typedef struct mc_mesh {
    double* vertices;
    int32_t* triangles;
    int64_t n_vertices;
    int64_t n_triangles;
    mc_stats stats;
} mc_mesh;

typedef struct mc_ctx mc_ctx;
typedef struct mc_solid mc_solid;

/* ---------------------------------------------------------------- entries */

/* Reference panic text for a status (or a short description). */
const char* mc_status_string(mc_status s);

/* Detailed message of the last failing call on this context. */
const char* mc_last_error(const mc_ctx* ctx);

/* Create a context on CUDA device `device` (its own stream and buffers). */
mc_status mc_create(mc_ctx** out, int device);
void mc_destroy(mc_ctx* ctx);

/* Lower a serialised Solid tree (prefix order, see mc_node) to the device.
 * Replaces the dynamic Solid.Contains dispatch (model3d/solid.go:16-21). */
mc_status mc_solid_create(mc_ctx* ctx, const mc_node* nodes, size_t n_nodes,
                          const mc_tri_set* sets, size_t n_sets, mc_solid** out);
void mc_solid_destroy(mc_solid* solid);

/* Root Min()/Max() of a lowered solid. */
mc_status mc_solid_bounds(const mc_solid* solid, double min[3], double max[3]);

/* One axis of newSquareSpacer (model3d/mc.go:594-608): for x := lo - delta;
 * x <= hi + delta; x += delta.  Writes at most cap values, sets *n to the
 * full count.  MC_ERR_GRID if the loop would not terminate. */
mc_status mc_spacer_axis(double lo, double hi, double delta, double* out, int64_t cap,
                         int64_t* n);

/* Host-only: lower a node array as mc_solid_create does, without a GPU or a
 * context, and describe the program.  Returns the lowering's status
 * (MC_ERR_NOT_LOWERABLE, MC_ERR_BAD_PROGRAM, MC_ERR_LIMIT, ...) with its
 * message in err (err_cap bytes, may be 0).  No counterpart in the
 * reference: a binding can refuse an unlowerable solid before any device
 * work. */
typedef struct mc_program_info {
    int64_t n_ops;        /* postfix program words */
    int64_t n_leaves;     /* leaf predicates: primitives, colliders, metaballs */
    int64_t n_metaballs;  /* MC_NODE_METABALL leaves */
    int64_t n_balls;      /* their balls */
    int64_t n_boxes;      /* TRANSFORM / CHECKED box checks */
    int64_t n_colliders;  /* collider trees */
    int64_t max_stack;    /* deepest bit stack */
    double threshold;     /* f(radiusThreshold) of the first metaball, as the library computed it */
    double root_min[3];
    double root_max[3];
    uint64_t digest;      /* FNV-1a over the 64-bit words of every array of the lowered program, in a
                             fixed order: changes exactly when the bytes uploaded to the device change */
} mc_program_info;
mc_status mc_program_check(const mc_node* nodes, size_t n_nodes, const mc_tri_set* sets, size_t n_sets,
                           mc_program_info* info, char* err, size_t err_cap);

/* MarchingCubesSearch(s, delta, iters) (model3d/mc.go:45-49); iters == 0 is
 * MarchingCubes (model3d/mc.go:14-37).  The result is copied into host arrays
 * owned by the library; release them with mc_mesh_free.  opts may be NULL. */
mc_status mc_search(mc_ctx* ctx, const mc_solid* solid, double delta, int32_t iters,
                    const mc_opts* opts, mc_mesh* out);
void mc_mesh_free(mc_mesh* mesh);

/* Same as mc_search, but the mesh stays in device memory owned by the
 * context (valid until the next call on it); *n_vertices / *n_triangles and
 * *stats (may be NULL) are filled.  Once an earlier call on the context has
 * sized its mesh buffers, the call does not wait mid-way for the mesh's size:
 * if the mesh outgrew the buffers, the call runs again with waiting (same
 * result); stats then describe the second run. */
mc_status mc_search_device(mc_ctx* ctx, const mc_solid* solid, double delta, int32_t iters,
                           const mc_opts* opts, int64_t* n_vertices, int64_t* n_triangles,
                           mc_stats* stats);
/* Device pointers of the last mc_search_device result. */
mc_status mc_result_device(const mc_ctx* ctx, const double** vertices,
                           const int32_t** triangles);
/* Copy the last result into caller-provided host arrays (V*3, T*3). */
mc_status mc_result_copy(mc_ctx* ctx, double* vertices, int32_t* triangles);
/* The grid edge of each vertex of the last mc_search_device result: V keys
 * axis << 60 | z << 40 | y << 20 | x, the edge from corner (x, y, z) to the
 * next corner along axis (0 x, 1 y, 2 z; z counted from the slab's first
 * plane for a z-slab).  A triangle's three edges lie on one cube, the one
 * whose cube loop emitted it (mc.go:20-35).  No counterpart in the
 * reference: MarchingCubesFilter's block pruning (mc.go:83-148) is applied
 * on the host with it. */
mc_status mc_result_keys(mc_ctx* ctx, uint64_t* keys);
/* Interior points of the last mc_search_device run with opts->interior set:
 * V*3 float64, point i being the last inside point of vertex i's bisection
 * (the CoordMap of MarchingCubesInterior, model3d/mc.go:55-60, :191-198,
 * :252-255, keyed by vertex index).  MC_ERR_ARG if it was not requested. */
mc_status mc_result_interior_copy(mc_ctx* ctx, double* interior);
/* Mesh.Transform (model3d/mesh.go:643-645) of the last result's vertices, on
 * the device: every vertex becomes JoinedTransform(steps).Apply(vertex), or
 * its Inverse().Apply with inverse != 0 (transform.go:213-219; each step's
 * Inverse as in transform.go).  steps are n_steps MC_XF_* records.  With
 * TransformSolid of the same steps this is MarchingCubesConj
 * (model3d/mc.go:66-71). */
mc_status mc_result_transform(mc_ctx* ctx, const mc_node* steps, size_t n_steps, int32_t inverse);
/* EncodeSTL (model3d/export.go:20-66, fileformats/stl.go:27-58) of the last
 * result, encoded on the device: an 80-byte zero header, the triangle count
 * (uint32 LE), then per triangle the float32 casts of Triangle.Normal()
 * (primitives.go:27-33, float64 in the reference's operation order) and of
 * its three vertices, and two zero bytes -- 84 + 50 T bytes.  Triangles are
 * in this library's order (the reference writes them in its map order).
 * With out == NULL only *n_bytes is set; MC_ERR_ARG if cap is too small or
 * T does not fit in uint32. */
mc_status mc_result_stl(mc_ctx* ctx, uint8_t* out, size_t cap, size_t* n_bytes);

/* GroupTriangles (model3d/bvh.go:118-217) of the last result's triangles, on
 * the device: order[i] = the index of the triangle SaveGroupedSTL
 * (model3d/mesh.go:724-742) writes i-th.  The reference sorts a slice in Go
 * map order with an unstable sort; here each midpoint sort is stable over
 * the library's triangle order (ties keep that order).  order: T int32. */
mc_status mc_result_group(mc_ctx* ctx, int32_t* order);
/* SaveGroupedSTL's bytes (model3d/mesh.go:724-742: GroupTriangles, then
 * WriteSTL, model3d/export.go:28-60) of the last result, grouped and encoded
 * on the device.  Sizes and errors as mc_result_stl. */
mc_status mc_result_stl_grouped(mc_ctx* ctx, uint8_t* out, size_t cap, size_t* n_bytes);
/* The same two for a caller's indexed mesh (n_vertices x 3 float64,
 * n_triangles x 3 int32 vertex indices, checked on the host: MC_ERR_ARG for
 * an index outside [0, n_vertices)).  The mesh is copied to the device; the
 * last result is left as it was. */
mc_status mc_mesh_group(mc_ctx* ctx, const double* vertices, int64_t n_vertices, const int32_t* triangles,
                        int64_t n_triangles, int32_t* order);
mc_status mc_mesh_stl_grouped(mc_ctx* ctx, const double* vertices, int64_t n_vertices, const int32_t* triangles,
                              int64_t n_triangles, uint8_t* out, size_t cap, size_t* n_bytes);

/* Solid.Contains on the GPU for n points (n x 3 float64) -> out[i] in {0,1}.
 * Same device predicates and precision modes as mc_search. */
mc_status mc_contains(mc_ctx* ctx, const mc_solid* solid, const double* points, int64_t n,
                      const mc_opts* opts, uint8_t* out);

/* Batched search: n independent (solid, delta, iters) jobs meshed by one
 * persistent work-queue launch, replayed from a CUDA graph when the same
 * batch shape repeats.  outs[i] receives job i's mesh (free each with
 * mc_mesh_free).  Statuses per job go to job_status (may be NULL); the
 * return value is the first failing status. */
typedef struct mc_job {
    const mc_solid* solid;
    double delta;
    int32_t iters;
    int32_t reserved;
} mc_job;
mc_status mc_search_batch(mc_ctx* ctx, const mc_job* jobs, size_t n, const mc_opts* opts,
                          mc_mesh* outs, mc_status* job_status);

/* Autotuner for the corner-tile shape of the classification kernel: times
 * every candidate (tile_y, tile_z) on this solid and grid (CUDA events, best
 * of three), keeps the fastest in the context — later calls on the context
 * that leave tile_y / tile_z at 0 use it — and returns it in *best (may be
 * NULL) with its classification time in *best_ms (may be NULL).  Tuning
 * knob only: results are identical for every shape.  No counterpart in the
 * reference (its z-slab ring has no tile shape). */
mc_status mc_autotune(mc_ctx* ctx, const mc_solid* solid, double delta, int32_t iters,
                      const mc_opts* opts, mc_opts* best, double* best_ms);

/* Roofline denominators for this path on the context's GPU, measured with
 * micro-kernels: FP32 and FP64 FMA throughput (TFLOP/s, 2 flops per FMA)
 * and the read bandwidth of a buffer resident in L2 (GB/s).  Any output may
 * be NULL.  Measurement utility; no counterpart in the reference. */
mc_status mc_measure_peaks(mc_ctx* ctx, double* fp32_tflops, double* fp64_tflops, double* l2_read_gbs);

/* The 256-case lookup table the library uses (mcLookupTable,
 * model3d/mc.go:434-456): counts[c] triangles for case c, each as three
 * corner pairs tris[c][t][0..5]. */
mc_status mc_case_table(uint8_t counts[256], uint8_t tris[256][5][6]);

/*
 * Allocation-free MarchingCubesSearch, for callers that cannot allocate
 * device memory when they mesh: a process whose device memory belongs to
 * another allocator that hands the caller only its own buffers, or a
 * real-time loop that forbids cudaMalloc / cudaFree after start-up because
 * those calls can synchronise the whole device.  No counterpart in the
 * reference (it is a GPU-memory concern the Go code does not have).
 *
 * Same result as mc_search for CSG and metaball solids.  Solids with a
 * MC_NODE_COLLIDER node return MC_ERR_BAD_PROGRAM (a collider's tree and ray
 * grid are built from triangle sets this call does not take), and
 * opts->interior set returns MC_ERR_ARG.  Every intermediate array lives in
 * one file-scope device array of MC_NOALLOC_SCRATCH_BYTES, which every GPU
 * that loads the library holds until the process exits; the call makes no
 * cudaMalloc / cudaFree.  Inputs: the node array (host memory), delta,
 * iters, opts (may be NULL), the stream to run on (NULL: the legacy default
 * stream) on the current device.  Outputs: device buffers vertices
 * (vertex_cap x 3 float64) and triangles (triangle_cap x 3 int32), written in
 * the same layout as mc_search_device; *n_vertices / *n_triangles receive the
 * mesh size, also when the status is MC_ERR_LIMIT because a buffer is too
 * small (the caller can retry with larger buffers).  MC_ERR_LIMIT also means
 * that the grid, the program or the vertex keys do not fit the scratch array
 * (roughly beyond 400^3 corners), or that the folded program needs more
 * shared memory per block than the device offers.  When it returns
 * MC_ERR_LIMIT, no work of the call is left running on the GPU.
 *
 * The call uploads the program from host memory and waits on the stream
 * twice before it returns: once for the mesh size, once for the error words.
 *
 * The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress) and uploads the case table; make that first call
 * before any stream capture.  All calls share the scratch array, which
 * keeps the last call's contents (each call clears what must start at
 * zero): calls whose GPU work overlaps, from other threads or streams, race.
 */
#define MC_NOALLOC_SCRATCH_BYTES (64u << 20)
mc_status mc_search_noalloc(const mc_node* nodes, size_t n_nodes, double delta, int32_t iters,
                            const mc_opts* opts, void* stream, double* vertices,
                            int64_t vertex_cap, int32_t* triangles, int64_t triangle_cap,
                            int64_t* n_vertices, int64_t* n_triangles);

/* Library version string. */
const char* mc_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MCGPU_H */
