/*
 * psr.h - C ABI of the GB300 Poisson surface reconstruction path.
 *
 * Drop-in replacement for the data-parallel path of the reference's
 * SparseSurfelFusion::PoissonReconstruction (mesh/PoissonReconstruction.h:63-184):
 * oriented (optionally coloured) points in, triangle mesh out.  The reference's
 * compile-time configuration (base/GlobalConfigs.h) becomes a runtime psr_config; all
 * state lives in a handle (no process-global __constant__ state), every call returns a
 * status instead of exiting, and no call allocates device memory after psr_create.
 *
 * Plain C types only: pointers, sizes and a CUDA stream passed as void*.
 */
#ifndef PSR_PSR_H_
#define PSR_PSR_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PSR_ABI_VERSION 2

typedef enum psr_status {
    PSR_OK = 0,
    PSR_OUT_OF_CAPACITY = 1, /* a count exceeded its configured capacity */
    PSR_INVALID_INPUT = 2,   /* bad argument, empty cloud, non-finite coordinate */
    PSR_NONCONVERGED = 3,    /* CG hit its iteration limit above tolerance (informational) */
    PSR_DEVICE_TIMEOUT = 4,  /* a bounded device-side wait gave up */
    PSR_CUDA_ERROR = 5,      /* CUDA runtime error (message via psr_last_error) */
    PSR_PENDING = 6          /* psr_poll: the submitted reconstruction is still running */
} psr_status;

typedef enum psr_location { PSR_HOST = 0, PSR_DEVICE = 1 } psr_location;

/* Capacities and solver settings; replaces base/GlobalConfigs.h:7-53. */
typedef struct psr_config {
    int max_depth;             /* MAX_DEPTH_OCTREE (base/GlobalConfigs.h:34); 2..9 */
    int max_points;            /* MAX_SURFEL_COUNT (:7) */
    int max_triangles;         /* MAX_MESH_TRIANGLE_COUNT (:8) */
    int max_mesh_vertices;     /* MeshTriangleVertex capacity (mesh/ComputeTriangleIndices.cpp:32) */
    int max_nodes;             /* 0: 10 x max_points (TOTAL_NODEARRAY_MAX_COUNT, :42) */
    int max_subdivision_nodes; /* subdivision nodes built (0: 8 x max_points); a quarter of
                                  it bounds the nodes kept live */
    float bbox_scale;          /* 1.25 (mesh/BuildOctree.cpp:91) */
    int cg_max_iterations;     /* 10000 (mesh/solver/CGAlgorithm.cu:15) */
    float cg_tolerance;        /* 1e-5, absolute on ||r|| (mesh/solver/CGAlgorithm.cu:298) */
    int compute_colors;        /* per-vertex colour transfer (mesh/DrawMesh.cu:179-214) */
    int compute_normals;       /* per-vertex normals (mesh/DrawMesh.cu:102-177) */
    int device;                /* CUDA device ordinal */
    float laplacian_epsilon;   /* Laplacian entries with |value| <= this are dropped: 1e-6 as in
                                  mesh/solver/LaplacianSolver.cu:128-204; 0 keeps every entry
                                  (from depth 9 on the 1e-6 rule drops the stencil's edge and
                                  corner entries and leaves an indefinite system) */
    int concurrent_stages;     /* 1: the octree-only mesh records and the colour grid run on a
                                  second stream beside the solve (lower latency of one call);
                                  0: one chain (more throughput when many handles share the
                                  GPU, as in the served form) */
    int weld_vertices;         /* 1: vertices with bit-identical coordinates become one (the
                                  reference emits the vertices on the boundary of every
                                  subdivided region once per region,
                                  mesh/ComputeTriangleIndices.cu:1247-1282); representatives
                                  keep their order, triangles are renumbered, colours and
                                  normals come from the welded mesh.  0 (default): as the
                                  reference */
    int disable_graphs;        /* 0 (default): each (depth, options) pipeline is captured once
                                  into a CUDA graph and replayed; for depths 8 and 9 the graph
                                  solves the CG systems too large for a cluster's shared memory
                                  in a device loop (a while node; such a graph is profiled by
                                  Nsight Compute only as a whole).  1: kernels are issued one by
                                  one on every call, those systems on the clusters' global-memory
                                  path (meshes within the CG tolerance of the graph's; for
                                  inspection and per-kernel profiling) */
    int root_poly_capacity;    /* 0 (default): max(65536, nodes / 16).  Subdivision roots beyond
                                  this many evaluate the levels above them by walking their
                                  octree chain instead of from one cached polynomial per root
                                  (same mesh, slower) */
    int cg_residual_period;    /* CG iterative refinement: the true residual b - A x (exact
                                  products, double-float sums, FP64 norm) is evaluated every
                                  this many iterations and when the recursive residual reaches
                                  the tolerance; the CG restarts from it when it is above the
                                  tolerance and the floor of an FP32 solution (2^-20 ||b||).
                                  0 (default): every 32 iterations; -1: never (the reference's
                                  recursive residual only, mesh/solver/CGAlgorithm.cu:36-75) */
    int batch_clouds;          /* 0 or 1: one cloud per call.  K (2..64): the handle holds K
                                  complete workspaces and psr_submit_batch reconstructs up to K
                                  clouds of one depth with one launch of each kernel for all of
                                  them (the clouds' data never mix; each result equals the
                                  one-cloud call's).  Device memory: K x psr_memory_bytes of a
                                  one-cloud handle */
    int cg_cluster_ctas;       /* CTAs of the thread-block cluster that solves depth D (1..16;
                                  0: the largest the device schedules, 16 on GB300).  Fewer
                                  CTAs take more rows each: longer per call, less SM time, which
                                  is what many concurrent reconstructions share */
    int cg_cluster_ctas_fine;  /* the same for depths D-1 and D-2 (0: 8) */
} psr_config;

/* Oriented input cloud (the fields of DepthSurfel, base/CommonTypes.h:113-118, as SoA). */
typedef struct psr_points {
    const float* xyz;      /* 3 * count, x y z interleaved */
    const float* normals;  /* 3 * count */
    const uint8_t* rgb;    /* 3 * count, or NULL; colour = rgb / 255 */
    int count;
    int location;          /* psr_location of the three arrays */
} psr_points;

/* Per-call options. */
typedef struct psr_options {
    int depth;             /* octree depth of this call, <= max_depth (0: max_depth) */
    int cg_iterations;     /* > 0: per-depth iteration limit instead of cg_max_iterations */
} psr_options;

/* Output mesh: vertices in the normalised unit cube of the reference
 * (mesh/ComputeTriangleIndices.h:331-342); world = center + vertex * scale. */
typedef struct psr_mesh {
    float* vertices;       /* 3 * vertex_capacity */
    int32_t* triangles;    /* 3 * triangle_capacity */
    float* colors;         /* 3 * vertex_capacity, or NULL */
    float* normals;        /* 3 * vertex_capacity, or NULL */
    int vertex_capacity;
    int triangle_capacity;
    int location;          /* psr_location of the output arrays */
    int vertex_count;      /* out */
    int triangle_count;    /* out */
    float center[3];       /* out: bounding-box origin */
    float scale;           /* out: bounding-box edge (1.25 x largest extent) */
} psr_mesh;

/* Counts of the last reconstruction. */
typedef struct psr_stats {
    int points, unique_leaves, nodes, depth;
    int level_count[10];
    int vertices, edges, faces;
    int crossings, triangles;
    int subdivision_roots, subdivision_nodes;
    int mesh_vertices, mesh_triangles;
    int cg_iterations[10];
    double cg_residual[10]; /* ||r|| of the recursive residual at the end of each depth's CG
                               (the reference's stopping quantity) */
    float iso_value;
    unsigned error_bits;
    float stage_ms[6];     /* octree, field, solve, mesh, transfer, total (device time) */
    int kernel_launches;   /* kernels launched by the call (CUDA-graph kernel nodes) */
    int graph_replay;      /* 1 when the call replayed a captured CUDA graph */
    float cg_kernel_ms;    /* device time of the CG kernel alone (part of stage_ms[2]) */
    float cg_depth_ms[10]; /* device time of each depth's CG (depths solve concurrently) */
    double cg_true_residual[10]; /* ||b - A x|| of each depth at its last true-residual
                                    evaluation (exact products, FP64 norm); -1: none */
    int cg_residual_checks[10];  /* true-residual evaluations of each depth's CG */
    int cg_restarts[10];         /* refinement restarts from the true residual */
} psr_stats;

typedef struct psr_handle psr_handle;

/* Fills the reference defaults. */
psr_status psr_config_default(psr_config* cfg);

/* Allocates every device buffer from the capacities (replaces the constructor,
 * mesh/PoissonReconstruction.cpp:10-30, and ComputeVectorField::BuildInnerProductTable,
 * mesh/ComputeVectorField.cpp:77-121). */
psr_status psr_create(const psr_config* cfg, psr_handle** out);

psr_status psr_destroy(psr_handle* h);

/* One reconstruction (replaces SolvePoissionReconstructionMesh,
 * mesh/PoissonReconstruction.cpp:195-245, and the mesh read-back of DrawRebuildMesh,
 * :248-252).  `stream` is a cudaStream_t or NULL for the handle's own stream.  The call
 * returns once the mesh counts are known and the mesh has been written. */
psr_status psr_reconstruct(psr_handle* h, const psr_points* points, const psr_options* options,
                           psr_mesh* mesh, void* stream);

/* Served form (no counterpart in the reference, which blocks): psr_submit enqueues the
 * same work as psr_reconstruct on `stream` and returns without waiting; one
 * reconstruction per handle is in flight at a time.  `points` may be released once the
 * work has run (device inputs are read by the GPU, host inputs are copied from the host
 * asynchronously: keep them alive and pinned until completion); `mesh` must stay valid
 * until completion.  Device-resident outputs are written by the GPU; host outputs are
 * copied when the completion is collected.  psr_poll returns PSR_PENDING while the GPU
 * is still working, else collects the result (counts, stats, status) exactly like
 * psr_reconstruct would have; psr_wait blocks until then.  Many handles, each with its
 * own stream, give concurrent reconstructions driven from one host thread. */
psr_status psr_submit(psr_handle* h, const psr_points* points, const psr_options* options, psr_mesh* mesh,
                      void* stream);
psr_status psr_poll(psr_handle* h);
psr_status psr_wait(psr_handle* h);

/* Normals of an unoriented cloud (replaces the PCL step the reference runs before the path,
 * CalculatePointCloudNormal, mesh/PoissonReconstruction.cpp:137-161: NormalEstimationOMP,
 * k = 10 nearest neighbours, viewpoint (0, 0, 0)): for every point the eigenvector of the
 * smallest eigenvalue of its 10 nearest samples' covariance (itself included), flipped
 * towards `viewpoint` (NULL: the origin); NaN when the cloud has fewer than 3 points.
 * xyz and normals are count x 3 floats, both on the device or both on the host
 * (`location`); count <= max_points.  Blocks until the normals are written; uses the
 * handle's scratch (no reconstruction in flight on the handle). */
psr_status psr_estimate_normals(psr_handle* h, const float* xyz, int count, psr_location location, float* normals,
                                const float* viewpoint, void* stream);

/* Multi-cloud form (no counterpart in the reference, which reconstructs one cloud per
 * blocking call, mesh/PoissonReconstruction.cpp:195-245): enqueues the reconstruction of
 * `count` clouds (1 <= count <= batch_clouds) on `stream` and returns without waiting.
 * Every kernel of the pipeline is launched once for all of them, cloud i in workspace slot
 * i; options (depth, iterations) are shared, and the clouds must agree on having colours
 * (points[i].rgb) and on the outputs asked for (meshes[i].colors / normals).  Completion is
 * collected with psr_poll / psr_wait, which fill meshes[i] like psr_reconstruct does and
 * return PSR_OK when every cloud succeeded; psr_get_batch_result gives each cloud's status
 * and statistics.  psr_reconstruct_batch submits and waits. */
psr_status psr_submit_batch(psr_handle* h, const psr_points* points, int count, const psr_options* options,
                            psr_mesh* meshes, void* stream);
psr_status psr_reconstruct_batch(psr_handle* h, const psr_points* points, int count, const psr_options* options,
                                 psr_mesh* meshes, void* stream);
/* Status and statistics of cloud `index` of the last completed call (index 0 for a one-cloud
 * call); `out` may be NULL.  Returns PSR_INVALID_INPUT, leaving `out` untouched, when the
 * last completed call had no cloud `index` (or no call has completed yet). */
psr_status psr_get_batch_result(const psr_handle* h, int index, psr_stats* out);

/* Input adaptor: device array of `count` DepthSurfel records (base/CommonTypes.h:113-118,
 * 64 bytes each) -> device SoA arrays for psr_points: xyz and normals (3 * count floats),
 * and rgb (3 * count bytes, round(255 * ColorAndTime.xyz) clamped) unless rgb is NULL.
 * Replaces getCoordinateAndNormalKernel (mesh/BuildOctree.cu:135-143); enqueued on
 * `stream` (a cudaStream_t or NULL), no host wait. */
psr_status psr_surfels_to_points(const void* surfels, int count, float* xyz, float* normals, uint8_t* rgb,
                                 void* stream);

/* Device memory held by the handle (bytes), for admission under a memory budget. */
psr_status psr_memory_bytes(const psr_handle* h, size_t* bytes);

psr_status psr_get_stats(const psr_handle* h, psr_stats* out);

/* Copies an internal device array of the last reconstruction to host memory (testing
 * and inspection); "name@k" names cloud k's array after a multi-cloud call.  Returns the
 * byte size in *bytes; dst may be NULL to query it. */
psr_status psr_debug_array(psr_handle* h, const char* name, void* dst, size_t dst_bytes, size_t* bytes);

/* Point ordering without any device allocation (no counterpart in the reference).
 * For callers that cannot call cudaMalloc at all (a caller-owned memory pool or arena,
 * a host process whose allocator must see every byte, a real-time loop that may not
 * allocate): normalises the cloud exactly like psr_reconstruct, computes each point's
 * Morton code at `depth` (1..9) and stably sorts by it.  `xyz` (3 * count floats),
 * `codes` and `order` (count uint32 each: sorted codes, original index of each sorted
 * point) are device pointers owned by the caller.  All scratch lives in a fixed
 * file-scope device array (about 9 MB, on every device that loads the library, until
 * exit), so at most 1,048,576 points per call (PSR_OUT_OF_CAPACITY above that).  Calls
 * share that array: calls whose GPU work overlaps race.  The first call on a device
 * looks up the array's address with that device current.  Every call synchronises
 * `stream` (a cudaStream_t or NULL) and returns after its work there has completed, so
 * it must not be called while any stream of the device is being captured. */
psr_status psr_morton_sort_noalloc(const float* xyz, int count, int depth, float bbox_scale, uint32_t* codes,
                                   uint32_t* order, void* stream);

const char* psr_status_string(psr_status s);
const char* psr_last_error(const psr_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* PSR_PSR_H_ */
