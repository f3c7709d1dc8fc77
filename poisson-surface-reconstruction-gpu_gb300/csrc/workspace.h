// Device workspace of one reconstruction handle.  Every buffer is allocated once at
// handle creation from the configured capacities; a reconstruction never allocates.
//
// HBM layout (structure of arrays, one array per field):
//   points   : sorted positions / scaled normals / colours, 3 x N floats each
//   nodes    : key, pidx, pnum, parent, first_child, didx, dnum, depth, enc (int32 x M),
//              centre (3 x M floats), neighbour table [27][M] int32,
//              vertex / edge / face back-pointers [8|12|6][M] int32
//   build    : level-by-level staging arrays used while the octree is assembled
//   mesh     : vertex / edge / face records, implicit values, output vertices/triangles
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include "primitives.cuh"

namespace psr {

struct Caps {
    int points;        // N cap
    int nodes;         // M cap (all depths)
    int dnodes;        // D-level node cap
    int vertices;      // octree vertex records
    int edges;         // D-level edge records
    int faces;         // face records
    int sub_nodes;     // subdivision-space nodes (all groups of one reconstruction)
    int sub_dnodes;    // live D-level subdivision cells
    int sub_live;      // live subdivision nodes of all depths
    int mesh_vertices; // output vertex cap
    int mesh_tris;     // output triangle cap
    int scan_tiles;    // tiles of the largest scan
};

// mesh-stage scratch
struct MeshBufs {
    int* ov_group;             // [8][cap.nodes]: group whose root redirects this child slot
    int* ov_sub;               // [8][cap.nodes]: root slot inside that group
    int* groups;               // group records (see mesh.cu)
    int max_groups;
    unsigned* edge_of_dnode;   // sub-edge prefix per live depth-D cell
    unsigned* tri_of_dnode;    // sub-triangle prefix per live depth-D cell
    unsigned* group_cross0;    // per group: crossing prefix at its first sub edge
    int* parts;                // per output part: vertex start / count, triangle start / count
    unsigned* kept_prefix;     // per staged vertex: kept vertices before it
    int* misc;                 // [0] parts, [1] staged vertices, [2] staged triangles
};

struct Workspace {
    int batch = 1;          // clouds of the launches being issued (the grids' y extent)
    int cg_ctas = 0;        // CTAs of the depth-D CG cluster (0: the largest the device runs, 16)
    int cg_ctas_fine = 0;   // CTAs of each depth-(D-1), (D-2) CG cluster (0: 8)
    MeshBufs mb;
    Caps cap;
    int depth;
    Counters* cnt;          // device
    Counters* cnt_host;     // pinned mirror for the final read-back
    ScanScratch scan;
    ScanScratch scan_aux;   // scans issued on the geometry stream (aux2) while `scan` is in use
    SortScratch sort;
    unsigned* scan_total;   // device scratch (points into cnt)

    // input staging (device copies of host inputs, or caller's device pointers)
    float* in_xyz;
    float* in_nrm;
    uint8_t* in_rgb;

    // sort
    unsigned *code, *sidx;

    // sorted points (SoA)
    float *px, *py, *pz, *nx, *ny, *nz, *cr, *cg, *cb;
    int* point2node;        // D-level local index of each sorted point
    int* puid;              // unique-leaf id of each sorted point
    unsigned* ucode;        // unique leaf codes
    int* ufirst;            // first sorted point of each unique leaf (+ sentinel)
    int* uslot;             // D-level slot of each unique leaf
    unsigned* uaddr;        // group address of each unique leaf

    // level build staging (levels D, D-1, ..., 0 appended in that order)
    int *tkey, *tpidx, *tpnum, *tdidx, *tdnum, *tchild;
    int* tparent_slot;      // per group of 8: slot of its father one level up
    int *gkey, *gpidx, *gpnum, *gdidx, *gdnum;   // per-group aggregates of the current level
    unsigned* gaddr;

    // final node arrays
    int *key, *pidx, *pnum, *parent, *first_child, *didx, *dnum, *ndepth, *enc;
    float *ctr_x, *ctr_y, *ctr_z;
    int* neigh;             // [27][cap.nodes]
    int* node_vtx;          // [8][cap.nodes]
    int* node_edge;         // [12][cap.nodes]
    int* node_face;         // [6][cap.nodes]

    // function tables (FP64, res x res) and per-depth stencil coefficients
    int res;
    float* dff;             // d/dx F_i . F_j rounded to float (index i + res * j)
    float* stencil;         // [D+1][27] Laplacian coefficients (0 where dropped)
    float stencil_host[(kMaxDepth + 1) * 27];   // the same on the host

    // field / solve
    float* vfield;          // 3 x dnodes (SoA: x block, y block, z block)
    float* divg;            // M
    float* xsol;            // M
    cudaEvent_t ev_cg = nullptr;   // recorded right after the CG kernel (stage timing)
    unsigned ev_flags = 0;         // flags of the stage-timing event records (external in a capture)
    float *cg_r, *cg_p, *cg_q, *cg_ap;   // residual, two direction buffers, A p
    int* cg_blk;            // CG block table: 64 same-depth nodes per sibling group
    CgLoopState* cg_loop;   // [D+1]: device-loop CG state per depth
    double* cg_loop_part;   // [D+1][kLoopMaxBlocks]: its per-block partial sums
    unsigned* cg_loop_ctl;  // loop control of a launch (passes, listed units; cloud 0's copy)
    double* cg_partial;     // scratch: divergence chunk sums (float pairs, 8 bytes each)
    float* point_val;       // N
    float* pv_coef;         // [27][cap.dnodes / 8 + 64]: per depth-(D-1) node, Bernstein coefficients
    double* iso_partial;

    // mesh geometry
    unsigned char* vmask;   // per node: owned corner mask (8 bits)
    unsigned short* emask16;   // per D node: owned edge mask (12 bits)
    unsigned char* fmask;   // per node: owned face mask (6 bits)
    float *v_x, *v_y, *v_z; // vertex positions
    int *v_owner, *v_kind, *v_depth;
    int *e_owner, *e_kind;
    int *f_owner, *f_kind, *f_hasparent;
    float* vvalue;          // implicit value - iso at every vertex
    unsigned* e_cross;      // per edge: staged vertex index of its crossing (exclusive scan)
    int* cube_class;        // per D node
    int* face_hit;          // per face: surface-edge intersection

    // subdivision
    int* sub_root;          // node index of each root (node order)
    int* sub_root_depth;
    int* root_group;        // per subdivision root: its group
    int* root_self;         // per root: the octree node it stands for
    float* root_poly;       // [28][cap_poly]: per root, Bernstein coefficients of the levels up to it
    int cap_poly;
    // subdivision candidates in compact slots (SoA, capacity cap.sub_nodes)
    int *c_vnode, *c_key, *c_group, *c_parent, *c_jump, *c_depth;
    float *c_cx, *c_cy, *c_cz;
    int* c_neigh;           // [27][cap.sub_nodes]
    int* c_live;            // live slots, depth after depth (capacity cap.sub_live)
    float* c_poly;          // [28][cap.sub_live]: per live entry, its Bernstein coefficients, sum |y|
    unsigned char* c_touch; // per live entry: faces of its root's cell its cell lies on
    // live depth-D cells (capacity cap.sub_dnodes)
    int* lv_vnode;          // virtual index, ascending
    int* lv_nb;             // [27][cap.sub_dnodes]: live index of each same-depth neighbour
    int *s_vtx, *s_edge;    // [8|12][cap.sub_dnodes]
    unsigned char* s_vmask;
    unsigned short* s_emask;
    float *sv_x, *sv_y, *sv_z;
    int *sv_owner, *sv_kind;
    float* sv_value;
    int *se_owner, *se_kind;
    unsigned* se_cross;
    int* s_cube_class;

    // output (device)
    float* mesh_v;          // 3 x mesh_vertices
    int* mesh_t;            // 3 x mesh_tris
    float* mesh_c;          // colours
    float* mesh_n;          // normals
    double* nacc;           // per output vertex normal accumulator (3 doubles)
    int* vcount;            // per output vertex triangle count
    int* cell_start;        // sample grid for the colour search
    int* colour_far;        // (vertex, bound) pairs the near colour search left
    int* colour_far2;       // those the coarser search left (trees of depth 8 and 9)
    // vertex welding (allocated only when the handle welds)
    int* weld_table = nullptr;   // hash slots: a vertex of the class, then its smallest index
    unsigned weld_mask = 0;      // slots - 1 (a power of two >= 2 x mesh vertex capacity)
    int* weld_slot = nullptr;    // slot of every vertex's class
    int* weld_newid = nullptr;   // welded number of every representative
    float* weld_v = nullptr;     // compacted positions

    // staging for the two-phase insertion of each mesh part
    float* part_v;          // 3 x cap
    int* part_t;
    int part_cap_v, part_cap_t;

    int* d_params;          // [0] point count of the current call (written before each run)

    cudaStream_t stream;
    cudaStream_t aux = nullptr;         // second stream for work forked off `stream`
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaStream_t aux2 = nullptr;        // third stream: octree-only mesh records beside the solve
    cudaEvent_t ev_fork2 = nullptr, ev_join2 = nullptr;
    cudaStream_t aux3 = nullptr;        // fourth stream: the CG of depths D-1 and D-2
    cudaEvent_t ev_join3 = nullptr;
    cudaStream_t aux4 = nullptr;        // fifth stream: the device-loop CG of large depths
    cudaEvent_t ev_join4 = nullptr;
    cudaStream_t loop_body = nullptr;   // captures the body graph of the device loop
    int num_sms;
};

// sample grid of the colour search: 2^g cells per axis (128^3: a few samples per surface
// cell at 200k points)
constexpr int kColourGridLevel = 7;

// launch grid for the clouds of the batch being issued (gx blocks for one cloud)
#define PSR_GRID(ws, gx) dim3(::psr::cloud_blocks((ws).batch, (gx)), (ws).batch)

// the clouds of the next launches (every scan scratch copy carries the count too)
inline void set_batch(Workspace& ws, int clouds) {
    ws.batch = clouds;
    ws.scan.batch = clouds;
    ws.scan_aux.batch = clouds;
    ws.sort.scan.batch = clouds;
}

// grid of a grid-stride kernel over `work` items: enough blocks, at most 8 per SM
inline int grid_for(const Workspace& ws, long long work) {
    long long g = (work + kBlock - 1) / kBlock;
    long long cap = (long long)ws.num_sms * 8;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// stage entry points (each issues kernels on ws.stream; no host synchronisation)
cudaError_t octree_build(Workspace& ws);
void prepare_launch_configs(Workspace& ws);
cudaError_t field_build(Workspace& ws);
// res_period: true residual every res_period CG iterations and at convergence (0: only at
// convergence, < 0: never)
cudaError_t solve_build(Workspace& ws, int cg_mode, int cg_iters, float cg_tol, int cg_max_iter, int res_period);
cudaError_t mesh_geometry(Workspace& ws);   // vertex / edge / face records (octree only)
cudaError_t mesh_build(Workspace& ws);      // values, marching cubes, subdivision, compaction
cudaError_t transfer_prepare(Workspace& ws, int with_colour);   // sample grid (points only)
cudaError_t transfer_build(Workspace& ws, int with_colour, int with_normals);

}  // namespace psr
