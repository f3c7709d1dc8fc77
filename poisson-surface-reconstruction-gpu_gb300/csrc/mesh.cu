// Stage (d): vertex / edge / face arrays, marching cubes at the finest depth, subdivision
// of coarser leaves that carry surface, and compaction of the output mesh.
//
// Reference: mesh/BuildMeshGeometry.cu:42-546 and mesh/ComputeTriangleIndices.cu:346-2194.
// The reference processes each coarse subdivision root in its own host iteration and the
// finer roots in one host iteration per depth, temporarily redirecting the parent's child
// pointer to the subdivided copy.  Here every root group (one coarse root, or all finer
// roots of one depth) owns a region of one subdivision-space array and an overlay of the
// redirected child pointers that only its own lookups see, so all groups run in one
// batched pass with the same results as the sequential reference.
#include "workspace.h"
#include "tables.cuh"

PSR_DEFINE_CONST_TABLES(upload_tables_mesh)

namespace psr {

__device__ __forceinline__ float sqdist3(float ax, float ay, float az, float bx, float by, float bz) {
    float dx = __fsub_rn(ax, bx), dy = __fsub_rn(ay, by), dz = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// values behind N 1-based vertex pointers, every load issued before any check (a pointer
// <= 0 is a broken record: it reads entry 0, yields 1.0f and flags the error)
template <int N>
__device__ __forceinline__ void ptr_values(const float* vals, const int (&p)[N], float (&v)[N], unsigned* err) {
#pragma unroll
    for (int q = 0; q < N; ++q) v[q] = vals[p[q] > 0 ? p[q] - 1 : 0];
    bool bad = false;
#pragma unroll
    for (int q = 0; q < N; ++q)
        if (p[q] <= 0) { v[q] = 1.0f; bad = true; }
    if (bad) atomicOr(err, kErrInvalid);
}

__device__ __forceinline__ void decode3m(int e, int depth, int& ix, int& iy, int& iz) {
    const int o1 = 1 << (depth + 1);
    ix = e & (o1 - 1);
    iy = (e >> (depth + 1)) & (o1 - 1);
    iz = e >> (2 * (depth + 1));
}

// vertex slot of a neighbour centre relative to a vertex (mesh/BuildMeshGeometry.cu:133-144)
__device__ __forceinline__ int vertex_slot(float ncx, float ncy, float ncz, float vx, float vy, float vz) {
    int idx = 0;
    if (__fsub_rn(ncx, vx) < 0) idx |= 1;
    if (__fsub_rn(ncz, vz) < 0) idx |= 4;
    if (__fsub_rn(ncy, vy) < 0) idx += (idx & 1) ? 1 : 3;
    return idx;
}

__device__ __forceinline__ void edge_center(float cx, float cy, float cz, int e, float hw, float out[3]) {
    const int orient = e >> 2;
    const int off[2] = {e & 1, (e & 2) >> 1};
    const float c[3] = {cx, cy, cz};
    int dim = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int m = 0;
        if (orient != a) { m = 2 * off[dim] - 1; dim++; }
        out[a] = __fadd_rn(c[a], (float)m * hw);
    }
}

// Same-depth cells around a vertex, an edge or a face.  Neighbour slot k of a node is the
// same-depth cell at offset (k/9 - 1, (k/3)%3 - 1, k%3 - 1).  Node centres, corners and
// edge / face midpoints are dyadic, so the reference's test "centre within one cell width
// of the point" is exact, and it holds for precisely these cells: the 8 cells whose offset
// is 0 or the corner's side on every axis, the 4 around an edge, the 2 across a face.
// Ownership (smallest key among those cells) and the back-pointers are evaluated on these
// slots only, with the reference's slot numbering derived from the same offsets.
__device__ __forceinline__ int nslot(int ax, int ay, int az) { return 9 * (ax + 1) + 3 * (ay + 1) + (az + 1); }

// corner q: + side on x if bit 0, y if bit 1, z if bit 2
__device__ __forceinline__ void corner_sides(int q, int& mx, int& my, int& mz) {
    mx = (q & 1) ? 1 : -1;
    my = (q & 2) ? 1 : -1;
    mz = (q & 4) ? 1 : -1;
}
__device__ __forceinline__ unsigned vertex_cells(int q) {
    int mx, my, mz;
    corner_sides(q, mx, my, mz);
    unsigned m = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) m |= 1u << nslot((j & 1) ? mx : 0, (j & 2) ? my : 0, (j & 4) ? mz : 0);
    return m;
}
// edge e: axis e >> 2; the two other axes (increasing order) at sides 2 (e & 1) - 1 and
// 2 ((e >> 1) & 1) - 1
__device__ __forceinline__ void edge_offset(int e, int j, int a[3]) {
    const int orient = e >> 2;
    const int m[2] = {2 * (e & 1) - 1, 2 * ((e >> 1) & 1) - 1};
    int dim = 0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
        a[ax] = 0;
        if (ax != orient) { a[ax] = ((j >> dim) & 1) ? m[dim] : 0; dim++; }
    }
}
__device__ __forceinline__ unsigned edge_cells(int e) {
    unsigned m = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        int a[3];
        edge_offset(e, j, a);
        m |= 1u << nslot(a[0], a[1], a[2]);
    }
    return m;
}
__device__ __forceinline__ unsigned face_cells(int f) {
    int a[3] = {0, 0, 0};
    a[f >> 1] = 2 * (f & 1) - 1;
    return (1u << 13) | (1u << nslot(a[0], a[1], a[2]));
}
// vertex_slot() of the cell at offset a for corner sides m (centre minus corner is
// (2 a - m) half widths on every axis)
__device__ __forceinline__ int vertex_slot_of(int ax, int ay, int az, int mx, int my, int mz) {
    int idx = 0;
    if (2 * ax - mx < 0) idx |= 1;
    if (2 * az - mz < 0) idx |= 4;
    if (2 * ay - my < 0) idx += (idx & 1) ? 1 : 3;
    return idx;
}
// edge slot of the cell at offset a around edge e (mesh/BuildMeshGeometry.cu:255-268)
__device__ __forceinline__ int edge_slot_of(int e, const int a[3]) {
    const int orient = e >> 2;
    const int m[2] = {2 * (e & 1) - 1, 2 * ((e >> 1) & 1) - 1};
    int idx = orient << 2, dim = 0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
        if (ax != orient) { if (2 * a[ax] - m[dim] < 0) idx |= 1 << dim; dim++; }
    return idx;
}

// ------------------------------------------------------------------------------------
// octree vertex / edge / face records
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_mesh_reset(const Counters* c, int* node_vtx, int* node_edge,
                                                       int* node_face, int* ov_group, int* ov_sub, size_t stride) {
    PSR_CLOUD(c, node_vtx, node_edge, node_face, ov_group, ov_sub);
    const int M = c->n_nodes;
    PSR_GRID_STRIDE(i, M) {
        for (int k = 0; k < 8; ++k) node_vtx[(size_t)k * stride + i] = 0;
        for (int k = 0; k < 12; ++k) node_edge[(size_t)k * stride + i] = 0;
        for (int k = 0; k < 6; ++k) node_face[(size_t)k * stride + i] = 0;
        for (int k = 0; k < 8; ++k) { ov_group[(size_t)k * stride + i] = -1; ov_sub[(size_t)k * stride + i] = -1; }
    }
}

// vertex ownership (initVertexOwner, mesh/BuildMeshGeometry.cu:42-101): a node owns a
// corner when no other cell around it has a smaller key
__global__ void __launch_bounds__(kBlock) k_vertex_owner(const Counters* c, const int* key, const int* neigh,
                                                         size_t stride, unsigned char* vmask) {
    PSR_CLOUD(c, key, neigh, vmask);
    const int M = c->n_nodes;
    PSR_GRID_STRIDE(i, M) {
        const int myk = key[i];
        unsigned smaller = 0;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            if (k == 13) continue;
            const int nb = neigh[(size_t)k * stride + i];
            if (nb != -1 && key[nb] < myk) smaller |= 1u << k;
        }
        unsigned m = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) if (!(smaller & vertex_cells(q))) m |= 1u << q;
        vmask[i] = (unsigned char)m;
    }
}

struct PopcLoad8 {
    const unsigned char* m;
    __device__ unsigned operator()(int i) const { return __popc((unsigned)m[i]); }
    __device__ void rebase() { PSR_CLOUD(m); }   // to cloud blockIdx.y
};

struct VertexStore {
    const unsigned char* vmask;
    const int* ndepth;
    const float *cx, *cy, *cz;
    float *vx, *vy, *vz;
    int *vowner, *vkind, *vdepth;
    int cap;
    unsigned* err;
    __device__ void operator()(int i, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        if ((int)(pre + cnt) > cap) { atomicOr(err, kErrCapacity); return; }
        const unsigned m = vmask[i];
        const int d = ndepth[i];
        const float hw = 1.0f / (float)(1 << (d + 1));
        int o = (int)pre;
        for (int q = 0; q < 8; ++q) {
            if (!((m >> q) & 1)) continue;
            vx[o] = __fadd_rn(cx[i], (float)(2 * (q & 1) - 1) * hw);
            vy[o] = __fadd_rn(cy[i], (float)(2 * ((q >> 1) & 1) - 1) * hw);
            vz[o] = __fadd_rn(cz[i], (float)(2 * ((q >> 2) & 1) - 1) * hw);
            vowner[o] = i;
            vkind[o] = q;
            vdepth[o] = d;
            ++o;
        }
    }
    __device__ void rebase() { PSR_CLOUD(vmask, ndepth, cx, cy, cz, vx, vy, vz, vowner, vkind, vdepth, err); }   // to cloud blockIdx.y
};

// maintainVertexNodePointer (mesh/BuildMeshGeometry.cu:108-147)
__global__ void __launch_bounds__(kBlock) k_vertex_maintain(const Counters* c, const int* neigh, size_t stride,
                                                            const int* vowner, const int* vkind, int* node_vtx) {
    PSR_CLOUD(c, neigh, vowner, vkind, node_vtx);
    const int V = c->n_vertices;
    PSR_GRID_STRIDE(v, V) {
        const int ow = vowner[v];
        int mx, my, mz;
        corner_sides(vkind[v], mx, my, mz);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ax = (j & 1) ? mx : 0, ay = (j & 2) ? my : 0, az = (j & 4) ? mz : 0;
            const int nb = neigh[(size_t)nslot(ax, ay, az) * stride + ow];
            if (nb != -1) node_vtx[(size_t)vertex_slot_of(ax, ay, az, mx, my, mz) * stride + nb] = v + 1;
        }
    }
}

// edge ownership for D-level nodes (initEdgeArray, mesh/BuildMeshGeometry.cu:149-220)
__global__ void __launch_bounds__(kBlock) k_edge_owner(const Counters* c, int depth, const int* key, const int* neigh,
                                                       size_t stride, unsigned short* emask) {
    PSR_CLOUD(c, key, neigh, emask);
    const int md = c->level_count[depth];
    const int b = c->level_base[depth];
    PSR_GRID_STRIDE(o, md) {
        const int i = b + o;
        const int myk = key[i];
        unsigned smaller = 0;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            if (k == 13 || k == 0 || k == 2 || k == 6 || k == 8 || k == 18 || k == 20 || k == 24 || k == 26)
                continue;   // corner-diagonal cells touch no edge
            const int nb = neigh[(size_t)k * stride + i];
            if (nb != -1 && key[nb] < myk) smaller |= 1u << k;
        }
        unsigned m = 0;
#pragma unroll
        for (int e = 0; e < 12; ++e) if (!(smaller & edge_cells(e))) m |= 1u << e;
        emask[o] = (unsigned short)m;
    }
}

struct PopcLoad16 {
    const unsigned short* m;
    __device__ unsigned operator()(int i) const { return __popc((unsigned)m[i]); }
    __device__ void rebase() { PSR_CLOUD(m); }   // to cloud blockIdx.y
};

struct EdgeStore {
    const unsigned short* emask;
    const int* base_ptr;   // first D-level node
    int *eowner, *ekind;
    int cap;
    unsigned* err;
    __device__ void operator()(int o, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        if ((int)(pre + cnt) > cap) { atomicOr(err, kErrCapacity); return; }
        const unsigned m = emask[o];
        const int i = *base_ptr + o;
        int q = (int)pre;
        for (int e = 0; e < 12; ++e)
            if ((m >> e) & 1) { eowner[q] = i; ekind[q] = e; ++q; }
    }
    __device__ void rebase() { PSR_CLOUD(emask, base_ptr, eowner, ekind, err); }   // to cloud blockIdx.y
};

// maintainEdgeNodePointer (mesh/BuildMeshGeometry.cu:222-280)
__global__ void __launch_bounds__(kBlock) k_edge_maintain(const Counters* c, const int* neigh, size_t stride,
                                                          const int* eowner, const int* ekind, int* node_edge) {
    PSR_CLOUD(c, neigh, eowner, ekind, node_edge);
    const int E = c->n_edges;
    PSR_GRID_STRIDE(ei, E) {
        const int ow = eowner[ei], kind = ekind[ei];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int a[3];
            edge_offset(kind, j, a);
            const int nb = neigh[(size_t)nslot(a[0], a[1], a[2]) * stride + ow];
            if (nb != -1) node_edge[(size_t)edge_slot_of(kind, a) * stride + nb] = ei + 1;
        }
    }
}

// face ownership (initFaceArray, mesh/BuildMeshGeometry.cu:282-354)
__global__ void __launch_bounds__(kBlock) k_face_owner(const Counters* c, const int* key, const int* neigh,
                                                       size_t stride, unsigned char* fmask) {
    PSR_CLOUD(c, key, neigh, fmask);
    const int M = c->n_nodes;
    PSR_GRID_STRIDE(i, M) {
        const int myk = key[i];
        unsigned m = 0;
#pragma unroll
        for (int f = 0; f < 6; ++f) {
            int a[3] = {0, 0, 0};
            a[f >> 1] = 2 * (f & 1) - 1;
            const int nb = neigh[(size_t)nslot(a[0], a[1], a[2]) * stride + i];
            if (!(nb != -1 && key[nb] < myk)) m |= 1u << f;
        }
        fmask[i] = (unsigned char)m;
    }
}

struct FaceStore {
    const unsigned char* fmask;
    const int* key;
    const int* ndepth;
    const int* parent;
    int depth;
    int *fowner, *fkind, *fhas;
    int cap;
    unsigned* err;
    __device__ void operator()(int i, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        if ((int)(pre + cnt) > cap) { atomicOr(err, kErrCapacity); return; }
        const unsigned m = fmask[i];
        const int d = ndepth[i];
        const int son = (key[i] >> (3 * (depth - d))) & 7;
        int q = (int)pre;
        for (int f = 0; f < 6; ++f) {
            if (!((m >> f) & 1)) continue;
            fowner[q] = i;
            fkind[q] = f;
            fhas[q] = (parent[i] == -1) ? -1 : ((__ldg(&g_tab.parent_face_kind[son][f]) != -1) ? 1 : -1);
            ++q;
        }
    }
    __device__ void rebase() { PSR_CLOUD(fmask, key, ndepth, parent, fowner, fkind, fhas, err); }   // to cloud blockIdx.y
};

// maintainFaceNodePointer (mesh/BuildMeshGeometry.cu:356-400)
__global__ void __launch_bounds__(kBlock) k_face_maintain(const Counters* c, const int* neigh, size_t stride,
                                                          const int* fowner, const int* fkind, int* node_face) {
    PSR_CLOUD(c, neigh, fowner, fkind, node_face);
    const int F = c->n_faces;
    PSR_GRID_STRIDE(fi, F) {
        const int ow = fowner[fi], kind = fkind[fi];
        const int orient = kind >> 1, m = 2 * (kind & 1) - 1;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            int a[3] = {0, 0, 0};
            a[orient] = j ? m : 0;
            const int nb = neigh[(size_t)nslot(a[0], a[1], a[2]) * stride + ow];
            if (nb != -1) node_face[(size_t)((orient << 1) + (2 * a[orient] - m < 0 ? 1 : 0)) * stride + nb] = fi + 1;
        }
    }
}

// ------------------------------------------------------------------------------------
// implicit values at the octree vertices (mesh/ComputeTriangleIndices.cu:346-399)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float node_terms(int node, float val, float qx, float qy, float qz, int depth,
                                            const int* neigh, size_t stride, const int* enc, const float* x) {
    return level_terms(node, val, qx, qy, qz, depth, neigh, stride, enc, x);
}

__global__ void __launch_bounds__(kBlock) k_vertex_values(const Counters* c, int depth, const float* vx,
                                                          const float* vy, const float* vz, const int* vowner,
                                                          const int* vkind, const int* vdepth, const int* neigh,
                                                          size_t stride, const int* parent, const int* first_child,
                                                          const int* enc, const float* x, float* vvalue) {
    PSR_CLOUD(c, vx, vy, vz, vowner, vkind, vdepth, neigh, parent, first_child, enc, x, vvalue);
    const int V = c->n_vertices;
    const float iso = c->iso;
    PSR_GRID_STRIDE(v, V) {
        float val = 0.0f;
        const int ow = vowner[v];
        if (ow > 0) {
            // The chain: the owner, its ancestors up to the root, then the owner's
            // descendants of child kind ec down to depth D.  Software-pipelined: the next
            // node's neighbour row, code, parent and first child are read while the current
            // node's values are in flight; terms are added in chain order as before.
            const float qx = vx[v], qy = vy[v], qz = vz[v];
            const int ec = __ldg(&g_tab.children_vertex_kind[vkind[v]]);
            int d = vdepth[v];
            const int fc_ow = first_child[ow];
            bool up = true;
            int nbs[27];
#pragma unroll
            for (int k = 0; k < 27; ++k) nbs[k] = neigh[(size_t)k * stride + ow];
            int e = enc[ow], par = parent[ow], fcn = fc_ow;
            while (true) {
                float xv[27];
#pragma unroll
                for (int k = 0; k < 27; ++k) xv[k] = x[nbs[k] >= 0 ? nbs[k] : 0];
                int nx;
                if (up && par != -1) {
                    nx = par;
                } else {
                    const int f = up ? fc_ow : fcn;
                    up = false;
                    nx = (d < depth && f != -1) ? f + ec : -1;
                    if (nx != -1) ++d;
                }
                int nb2[27];
                int e2 = 0, par2 = -1, fc2 = -1;
                const int n0 = (nx != -1) ? nx : 0;
#pragma unroll
                for (int k = 0; k < 27; ++k) nb2[k] = neigh[(size_t)k * stride + n0];
                e2 = enc[n0];
                par2 = parent[n0];
                fc2 = first_child[n0];
                val = terms_from(e, nbs, xv, val, qx, qy, qz, depth);
                if (nx == -1) break;
#pragma unroll
                for (int k = 0; k < 27; ++k) nbs[k] = nb2[k];
                e = e2;
                par = par2;
                fcn = fc2;
            }
        }
        vvalue[v] = __fsub_rn(val, iso);
    }
}

// ------------------------------------------------------------------------------------
// marching cubes at depth D (mesh/ComputeTriangleIndices.cu:401-526)
// ------------------------------------------------------------------------------------
__device__ __forceinline__ void interp_point(float p1x, float p1y, float p1z, float p2x, float p2y, float p2z, int dim,
                                             float v1, float v2, float* out) {
    out[0] = p1x; out[1] = p1y; out[2] = p1z;
    const float a1 = (dim == 0) ? p1x : (dim == 1) ? p1y : p1z;   // selects: no local array
    const float a2 = (dim == 0) ? p2x : (dim == 1) ? p2y : p2z;
    float pivot = __fdiv_rn(v1, __fsub_rn(v1, v2));
    float other = __fsub_rn(1.0f, pivot);
    out[dim] = __fadd_rn(__fmul_rn(a2, pivot), __fmul_rn(a1, other));
}

struct CrossLoad {
    const int* eowner;
    const int* ekind;
    const int* node_vtx;
    size_t stride;
    const float* vvalue;
    unsigned* err;
    __device__ unsigned operator()(int e) const {
        const int ow = eowner[e], kind = ekind[e];
        const int p[2] = {node_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][0]) * stride + ow],
                          node_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][1]) * stride + ow]};
        float ab[2];
        ptr_values(vvalue, p, ab, err);
        const float a = ab[0], b = ab[1];
        return (__fmul_rn(a, b) <= 0.0f) ? 1u : 0u;
    }
    __device__ void rebase() { PSR_CLOUD(eowner, ekind, node_vtx, vvalue, err); }   // to cloud blockIdx.y
};

struct CrossStore {
    const int* eowner;
    const int* ekind;
    const int* node_vtx;
    size_t stride;
    const float* vvalue;
    const float *vx, *vy, *vz;
    unsigned* ecross;   // per edge: staged vertex index (valid when the edge crosses)
    float* part_v;      // staged vertices (3 floats each)
    int voff;
    int cap;
    unsigned* err;
    __device__ void operator()(int e, unsigned pre, unsigned flag) const {
        ecross[e] = pre;
        if (!flag) return;
        const int at = voff + (int)pre;
        if (at >= cap) { atomicOr(err, kErrCapacity); return; }
        const int ow = eowner[e], kind = ekind[e];
        const int v1 = node_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][0]) * stride + ow] - 1;
        const int v2 = node_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][1]) * stride + ow] - 1;
        if (v1 < 0 || v2 < 0) return;   // only reachable for a malformed tree (flagged in the load)
        interp_point(vx[v1], vy[v1], vz[v1], vx[v2], vy[v2], vz[v2], kind >> 2, vvalue[v1], vvalue[v2],
                     &part_v[3 * (size_t)at]);
    }
    __device__ void rebase() { PSR_CLOUD(eowner, ekind, node_vtx, vvalue, vx, vy, vz, ecross, part_v, err); }   // to cloud blockIdx.y
};

struct CubeLoad {
    const int* node_vtx;
    size_t stride;
    const int* base_ptr;
    const float* vvalue;
    int* cube_class;
    unsigned* err;
    __device__ unsigned operator()(int o) const {
        const int i = *base_ptr + o;
        int p[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) p[q] = node_vtx[(size_t)q * stride + i];
        float vq[8];
        ptr_values(vvalue, p, vq, err);
        int cls = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (vq[q] < 0.0f) cls |= 1 << q;
        cube_class[o] = cls;
        return (unsigned)__ldg(&g_tab.mc_count[cls]);
    }
    __device__ void rebase() { PSR_CLOUD(node_vtx, base_ptr, vvalue, cube_class, err); }   // to cloud blockIdx.y
};

// emits the triangles of a D-level cube and marks surface-edge intersections on faces,
// propagating them to the parent faces (generateTrianglePos, :476-526)
struct CubeStore {
    const int* cube_class;
    const int* base_ptr;
    const int* node_edge;
    const int* node_face;
    size_t stride;
    const unsigned* ecross;
    const int* parent;
    const int* fhas;
    int* face_hit;
    int* part_t;
    int toff;
    int cap;
    unsigned* err;
    __device__ void operator()(int o, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        const int i = *base_ptr + o;
        const int cls = cube_class[o];
        const unsigned long long tri = __ldg(&g_tab.mc_tri[cls]);
        unsigned used = 0;
        for (int t = 0; t < (int)cnt; ++t) {
            const int at = toff + (int)pre + t;
            for (int a = 0; a < 3; ++a) {
                const int e = (int)((tri >> (4 * (3 * t + a))) & 0xF);
                used |= 1u << e;
                const int ei = node_edge[(size_t)e * stride + i] - 1;
                if (at < cap) part_t[3 * (size_t)at + a] = (ei >= 0) ? (int)ecross[ei] : -1;
            }
            if (at >= cap) atomicOr(err, kErrCapacity);
        }
        for (int f = 0; f < 6; ++f) {
            unsigned mark = 0;
            for (int j = 0; j < 4; ++j) mark |= (used >> c_tab.face_edges[f][j]) & 1u;
            if (!mark) continue;
            int pn = parent[i];
            int cf = node_face[(size_t)f * stride + i] - 1;
            if (cf < 0) continue;
            face_hit[cf] = 1;
            int guard = 0;
            while (fhas[cf] != -1 && pn >= 0 && guard++ < 32) {
                cf = node_face[(size_t)f * stride + pn] - 1;
                if (cf < 0) break;
                pn = parent[pn];
                face_hit[cf] = 1;
            }
        }
    }
    __device__ void rebase() { PSR_CLOUD(cube_class, base_ptr, node_edge, node_face, ecross, parent, fhas, face_hit, part_t, err); }   // to cloud blockIdx.y
};

// ------------------------------------------------------------------------------------
// subdivision roots (ProcessLeafNodesAtOtherDepth :555-587, selection :1284-1346)
// ------------------------------------------------------------------------------------
struct RootLoad {
    const int* node_vtx;
    const int* node_face;
    size_t stride;
    const float* vvalue;
    const int* face_hit;
    const int* first_child;
    unsigned* err;
    __device__ unsigned operator()(int i) const {
        // all reads first (the cell's 8 corner values, 6 faces and their flags), then the tests
        int p[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) p[q] = node_vtx[(size_t)q * stride + i];
        int fp[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) fp[f] = node_face[(size_t)f * stride + i] - 1;
        int fh[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) fh[f] = face_hit[fp[f] >= 0 ? fp[f] : 0];
        const int fc = first_child[i];
        float vq[8];
        ptr_values(vvalue, p, vq, err);
        const float s = (vq[0] < 0.0f) ? -1.0f : 1.0f;
        int ht = 0;
#pragma unroll
        for (int q = 1; q < 8; ++q)
            if (__fmul_rn(s, vq[q]) < 0.0f) ht = 1;
        int hi = 0;
#pragma unroll
        for (int f = 0; f < 6; ++f)
            if (fp[f] >= 0 && fh[f]) hi = 1;
        return (fc == -1 && (ht || hi)) ? 1u : 0u;
    }
    __device__ void rebase() { PSR_CLOUD(node_vtx, node_face, vvalue, face_hit, first_child, err); }   // to cloud blockIdx.y
};
struct RootStore {
    int* sub_root;
    int cap;
    unsigned* err;
    __device__ void operator()(int i, unsigned pre, unsigned f) const {
        if (!f) return;
        if ((int)pre >= cap) { atomicOr(err, kErrCapacity); return; }
        sub_root[pre] = i;
    }
    __device__ void rebase() { PSR_CLOUD(sub_root, err); }   // to cloud blockIdx.y
};

// Group table.  Group record (ints): 0 root depth, 1 first root, 2 root count,
// 3 virtual node offset, 4 virtual node count.  Coarse roots (depth < D - 4) are one group each; the finer roots
// of one depth form one group (mesh/ComputeTriangleIndices.cu:1475-1799, :1801-2194).
constexpr int kGroupRec = 8;

struct GroupFlagLoad {
    const int* sub_root;
    const int* ndepth;
    int finer;
    __device__ unsigned operator()(int r) const {
        const int rd = ndepth[sub_root[r]];
        if (r == 0 || rd < finer) return 1u;
        return (ndepth[sub_root[r - 1]] != rd) ? 1u : 0u;
    }
    __device__ void rebase() { PSR_CLOUD(sub_root, ndepth); }   // to cloud blockIdx.y
};
struct GroupFlagStore {
    int* root_group;
    int* groups;
    int max_groups;
    unsigned* err;
    __device__ void operator()(int r, unsigned pre, unsigned v) const {
        const int g = (int)(pre + v) - 1;
        root_group[r] = g;
        if (v) {
            if (g >= max_groups) { atomicOr(err, kErrCapacity); return; }
            groups[(size_t)g * kGroupRec + 1] = r;
        }
    }
    __device__ void rebase() { PSR_CLOUD(root_group, groups, err); }   // to cloud blockIdx.y
};

__global__ void k_group_count(Counters* c, const unsigned* total, int max_groups) {
    PSR_CLOUD(c, total);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int ng = (int)*total;
        if (ng > max_groups) { atomicOr(&c->error, kErrCapacity); ng = 0; }
        c->n_groups = ng;
    }
}

// per-group sizes (thread per group)
__global__ void __launch_bounds__(kBlock) k_group_sizes(Counters* c, int depth, const int* sub_root,
                                                        const int* ndepth, int* groups) {
    PSR_CLOUD(c, sub_root, ndepth, groups);
    const int ng = c->n_groups;
    const int R = c->n_subroots;
    PSR_GRID_STRIDE(g, ng) {
        int* G = groups + (size_t)g * kGroupRec;
        const int first = G[1];
        const int next = (g + 1 < ng) ? groups[(size_t)(g + 1) * kGroupRec + 1] : R;
        const int rd = ndepth[sub_root[first]];
        const long long n = next - first;
        long long per = 0, dper = 1;
        for (int d = rd; d <= depth; ++d) { per += dper; if (d < depth) dper *= 8; }
        const long long nodes = per * n;
        G[0] = rd;
        G[2] = (int)n;
        if (nodes > 0x3fffffffLL) atomicOr(&c->error, kErrCapacity);
        G[4] = nodes > 0x3fffffffLL ? 0x3fffffff : (int)nodes;
    }
}

struct GroupFieldLoad {
    const int* groups;
    int field;
    __device__ unsigned operator()(int g) const { return (unsigned)groups[(size_t)g * kGroupRec + field]; }
    __device__ void rebase() { PSR_CLOUD(groups); }   // to cloud blockIdx.y
};
struct GroupFieldStore {
    int* groups;
    int field;
    __device__ void operator()(int g, unsigned pre, unsigned) const { groups[(size_t)g * kGroupRec + field] = (int)pre; }
    __device__ void rebase() { PSR_CLOUD(groups); }   // to cloud blockIdx.y
};

// the virtual numbering of all groups must fit beside the octree indices (na + index)
__global__ void k_group_totals(Counters* c, const unsigned* node_total, int na) {
    PSR_CLOUD(c, node_total);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const unsigned nt = *node_total;
        if (nt > 0x7fffffffu - (unsigned)na) {
            atomicOr(&c->error, kErrCapacity);
            c->n_groups = 0;
        }
    }
}

// per root: its depth, the octree node it stands for, and the redirected child slot of
// its parent (overlay)
__global__ void __launch_bounds__(kBlock) k_root_overlay(const Counters* c, int depth, const int* sub_root,
                                                         const int* ndepth, const int* key, const int* parent,
                                                         const int* neigh, const int* root_group, const int* groups,
                                                         int* sub_root_depth, int* root_self, int* ov_group,
                                                         int* ov_sub, size_t stride) {
    PSR_CLOUD(c, sub_root, ndepth, key, parent, neigh, root_group, groups, sub_root_depth, root_self, ov_group, ov_sub);
    const int R = c->n_subroots;
    const int ng = c->n_groups;
    PSR_GRID_STRIDE(r, R) {
        const int node = sub_root[r];
        const int rd = ndepth[node];
        sub_root_depth[r] = rd;
        const int self = neigh[(size_t)13 * stride + node];   // its neighs[13] in the reference
        root_self[r] = (self == -1) ? node : self;
        const int g = root_group[r];
        if (g < 0 || g >= ng) continue;
        const int q = r - groups[(size_t)g * kGroupRec + 1];
        const int son = (key[node] >> (3 * (depth - rd))) & 7;
        const int pa = parent[node];
        if (pa >= 0) {
            ov_group[(size_t)son * stride + pa] = g;
            ov_sub[(size_t)son * stride + pa] = q;
        }
    }
}

// ---- subdivision, breadth-first over live nodes ----------------------------------------
// Virtual numbering (singleRebuildArray :599-635 / wholeRebuildArray :1110-1168): group g
// owns the virtual sub nodes G[3] .. G[3] + G[4] - 1, level by level from its root depth rd
// (its n roots) to D; node (q, rel) of level d sits at G[3] + off_d + q 8^(d-rd) + rel (rel:
// the Morton code below root q).  Neighbour tables hold octree nodes (< na), na + virtual
// index for sub nodes, or -1.  Only candidates are stored, in compact slots: at depth d the
// 8 children of every live node of depth d-1, in order, then the roots of depth d.  Both
// parts are in virtual order (groups are ordered by root depth), so the live depth-D cells,
// which carry all records from here on, come out in the reference's order.
__device__ __forceinline__ int sub_level_off(int rd, int n, int d) {
    int off = 0, cnt = n;
    for (int e = rd; e < d; ++e) { off += cnt; cnt *= 8; }
    return off;
}

// per-depth candidate bookkeeping (Counters::sub_*): [d] for depth d; one lane per depth
__global__ void k_sub_setup(Counters* c, int depth, const int* sub_root_depth, int cap_nodes) {
    PSR_CLOUD(c, sub_root_depth);
    const int d = threadIdx.x;
    const int R = c->n_subroots;
    __shared__ int s_end[kMaxDepth + 2];
    if (d <= depth + 1) {
        int lo = 0, hi = R;   // first root deeper than d (roots are in depth order)
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (sub_root_depth[mid] <= d) lo = mid + 1;
            else hi = mid;
        }
        s_end[d] = lo;
    }
    __syncthreads();
    if (d <= depth + 1) {
        const int start = (d > 0) ? s_end[d - 1] : 0;
        c->sub_rstart[d] = start;
        c->sub_nroots[d] = (c->n_groups > 0) ? s_end[d] - start : 0;
        c->sub_cand[d] = 0;
        c->sub_cbase[d] = 0;
        c->sub_lbase[d] = 0;
        c->sub_nlive[d] = 0;
    }
    __syncthreads();
    if (d == 0) {
        if (c->sub_nroots[1] > cap_nodes) atomicOr(&c->error, kErrCapacity);
        else c->sub_cand[1] = c->sub_nroots[1];
        c->n_sub_nodes = 0;
        c->n_sub_dnodes = 0;
    }
}

struct SubArrays {
    int *vnode, *key, *group, *parent, *jump, *depth;   // parent: slot, or -2 - octree parent
    float *cx, *cy, *cz;
    int* neigh;   // [27][cap]
    size_t cstride;
    int* live;    // live slots, depth after depth
    float* poly;  // [28][cap_live]: per live entry, Bernstein coefficients of its levels, sum |y|
    unsigned char* touch;   // per live entry: faces of its root's cell it lies on (bits x-, x+, y-, y+, z-, z+)
    int* lv_vnode;   // virtual index of each live depth-D cell
    int cap_nodes, cap_live, cap_live_d;
    __device__ void rebase() { PSR_CLOUD(vnode, key, group, parent, jump, depth, cx, cy, cz, neigh, live, poly, touch, lv_vnode); }   // to cloud blockIdx.y
};

// ---- certain-sign cells -------------------------------------------------------------
// Subdivision replaces a coarse leaf that carries surface by all of its depth-D cells, but
// the surface crosses few of them.  A cell where F - iso provably keeps one sign has no
// crossing edge and no triangle, so it needs no vertex, edge or cube record, and its
// subtree is never built.  The test below is conservative, so the mesh is unchanged.
//
// On the closed cell of a sub node s at depth d, F is the sum over the levels l <= d of the
// 27 neighbour terms y_k B_k of s's ancestor at l (y = 0 for absent nodes and for sub nodes
// that are not roots), provided no octree node deeper than d reaches the cell: that holds
// when none of s's 27 neighbours is an octree node with children.  B_k = b(x) b(y) b(z) with
// b(t) = 4/3 (3/4 - t^2) for |t| < 1/2 and 2/3 (3/2 - |t|)^2 for |t| < 3/2 (t in level
// widths from the translate's centre).  The knots of a level-l translate lie on level-l cell
// boundaries and the cell of s lies inside one level-l cell, so on it every translate is a
// single quadratic and F is a tensor-product quadratic.  Written in the Bernstein basis of
// the cell, F's 27 coefficients bound its values there (convex hull), so all coefficients
// above iso (below iso) make the sign certain.  With s in [-1, 1] across the cell, a
// translate is q(s) = b + g s + k/2 s^2 (b, g = h b', k = h^2 b'' at the centre, h the half
// width), whose Bernstein coefficients are b - g + k/2, b - k/2, b + g + k/2.
// Float vertex values are sums of the same nonzero terms (at most 27 (D+1)), within
// ~1.7e-5 sum |y| of the exact value; the float coefficients here are as close; the test
// keeps a margin of 1e-4 (sum |y| + |iso|).

// value carried by a sub-node neighbour (na + virtual index) of group G: its root's octree
// node for a root (it stands for that node), else nothing (x = 0 in subdivision space)
__device__ __forceinline__ int sub_value_node(int v, int na, const int* G, const int* root_self) {
    const int local = v - na - G[3];
    return ((unsigned)local < (unsigned)G[2]) ? root_self[G[1] + local] : -1;
}

// Levels up to a root's depth are the same for every cell below that root: their sum is one
// tensor-product quadratic on the root's cell, kept as its 27 Bernstein coefficients
// (root_poly[k][r], k < 27; [27][r]: sum |y| of those levels).  A cell inside it takes
// them by Bernstein subdivision: with the cell at [a, b] of the root's unit interval, the
// new coefficients are the blossom values P(a, a), P(a, b), P(b, b) -- convex weights, exact
// for these dyadic a, b.
__global__ void __launch_bounds__(kBlock) k_root_poly(const Counters* c, int depth, const int* sub_root,
                                                      const int* ndepth, const float* ctr_x, const float* ctr_y,
                                                      const float* ctr_z, const int* neigh, size_t stride,
                                                      const int* parent, const int* enc, const float* x,
                                                      float* root_poly, int cap_poly) {
    PSR_CLOUD(c, sub_root, ndepth, ctr_x, ctr_y, ctr_z, neigh, parent, enc, x, root_poly);
    const int R = c->n_subroots < cap_poly ? c->n_subroots : cap_poly;
    PSR_GRID_STRIDE(r, R) {
        const int node = sub_root[r];
        const int rd = ndepth[node];
        const float qx = ctr_x[node], qy = ctr_y[node], qz = ctr_z[node];
        float C[27];
#pragma unroll
        for (int k = 0; k < 27; ++k) C[k] = 0.0f;
        float mag = 0.0f, y[27];
        for (int now = node; now >= 0; now = parent[now]) {
            int ox, oy, oz;
            decode_fn_index(enc[now], depth, ox, oy, oz);
            const int l = ilog2_dev(ox + 1);
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int v = neigh[(size_t)k * stride + now];
                y[k] = (v >= 0) ? x[v] : 0.0f;
            }
            sign_level(y, ox, oy, oz, qx, qy, qz, __int_as_float((126 + l - rd) << 23), C, mag);
        }
#pragma unroll
        for (int k = 0; k < 27; ++k) root_poly[(size_t)k * cap_poly + r] = C[k];
        root_poly[(size_t)27 * cap_poly + r] = mag;
    }
}

// blossom matrix of [a, b] (rows: new coefficients, columns: old)
__device__ __forceinline__ void blossom3(float a, float b, float (&M)[3][3]) {
    const float a1 = 1.0f - a, b1 = 1.0f - b;
    M[0][0] = a1 * a1; M[0][1] = 2.0f * a * a1;     M[0][2] = a * a;
    M[1][0] = a1 * b1; M[1][1] = a1 * b + a * b1;   M[1][2] = a * b;
    M[2][0] = b1 * b1; M[2][1] = 2.0f * b * b1;     M[2][2] = b * b;
}

// C += the root polynomial P subdivided to the cell at Morton code rel (m levels below it)
__device__ __forceinline__ void add_subdivided(const float* P, size_t pstride, unsigned rel, int m, float (&C)[27]) {
    int i3[3] = {0, 0, 0};
    for (int j = 0; j < m; ++j)
#pragma unroll
        for (int a = 0; a < 3; ++a) i3[a] |= (int)((rel >> (3 * j + 2 - a)) & 1u) << j;
    const float inv = __int_as_float((127 - m) << 23);   // 2^-m
    float Mx[3][3], My[3][3], Mz[3][3];
    blossom3((float)i3[0] * inv, (float)(i3[0] + 1) * inv, Mx);
    blossom3((float)i3[1] * inv, (float)(i3[1] + 1) * inv, My);
    blossom3((float)i3[2] * inv, (float)(i3[2] + 1) * inv, Mz);
    float p[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) p[k] = __ldg(P + (size_t)k * pstride);   // written by an earlier launch
    float T1[27], T2[27];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int jk = 0; jk < 9; ++jk)
            T1[a * 9 + jk] = fmaf(Mx[a][0], p[jk], fmaf(Mx[a][1], p[9 + jk], Mx[a][2] * p[18 + jk]));
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                T2[a * 9 + bb * 3 + k] = fmaf(My[bb][0], T1[a * 9 + k],
                                              fmaf(My[bb][1], T1[a * 9 + 3 + k], My[bb][2] * T1[a * 9 + 6 + k]));
#pragma unroll
    for (int ab3 = 0; ab3 < 9; ++ab3)
#pragma unroll
        for (int gg = 0; gg < 3; ++gg)
            C[ab3 * 3 + gg] += fmaf(Mz[gg][0], T2[ab3 * 3], fmaf(Mz[gg][1], T2[ab3 * 3 + 1], Mz[gg][2] * T2[ab3 * 3 + 2]));
}

// Coefficients of a live node are kept (per live entry): a child's levels above its own are
// its parent's polynomial restricted to the child's octant (Bernstein subdivision, convex
// weights: the float error grows by a few ulp of the coefficients per level, inside the
// margin), so a candidate adds at most its own level.  A root starts from root_poly, or,
// beyond its capacity, from the walk over its octree chain.
__device__ __forceinline__ void root_coefficients(int r, int root_node, int rd, float qx, float qy, float qz,
                                                  int depth, const int* neigh, size_t stride, const int* parent,
                                                  const int* enc, const float* x, const float* root_poly,
                                                  int cap_poly, float (&C)[27], float& mag) {
    if (r < cap_poly) {
#pragma unroll
        for (int k = 0; k < 27; ++k) C[k] = root_poly[(size_t)k * cap_poly + r];
        mag = root_poly[(size_t)27 * cap_poly + r];
        return;
    }
#pragma unroll
    for (int k = 0; k < 27; ++k) C[k] = 0.0f;
    mag = 0.0f;
    float y[27];
    for (int now = root_node; now >= 0; now = parent[now]) {
        int ox, oy, oz;
        decode_fn_index(enc[now], depth, ox, oy, oz);
        const int l = ilog2_dev(ox + 1);
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            const int v = neigh[(size_t)k * stride + now];
            y[k] = (v >= 0) ? x[v] : 0.0f;
        }
        sign_level(y, ox, oy, oz, qx, qy, qz, __int_as_float((126 + l - rd) << 23), C, mag);
    }
}

// per-thread hand-over of a candidate's coefficients (28), face bits and virtual index
// from the scan's load to its store
__device__ __forceinline__ float* sub_poly_stash() {
    __shared__ float s_stash[30 * kBlock];
    return s_stash;
}

// faces of the root's cell that child `ch` (x = 4, y = 2, z = 1) of a cell with face bits
// pt lies on: a face its parent lies on, on the child's side
__device__ __forceinline__ unsigned child_touch(unsigned pt, int ch) {
    const unsigned side = ((ch & 4) ? 2u : 1u) | ((ch & 2) ? 8u : 4u) | ((ch & 1) ? 32u : 16u);
    return pt & side;
}

// One candidate of depth d (computeRebuildNeighbor :669-696 for its neighbours): its record,
// its neighbours and its sign test; returns 1 when it stays live.
struct SubLevelLoad {
    const Counters* c;
    int d, depth, na;
    const int* groups;
    const int* sub_root;
    const int* root_group;
    const int* root_self;
    const int* key;
    const int* neigh;
    size_t stride;
    const int* first_child;
    const int* parent;
    const int* ov_group;
    const int* ov_sub;
    const int* enc;
    const float* x;
    const float* root_poly;
    int cap_poly;
    SubArrays A;
    __device__ unsigned operator()(int i) const {
        const int nl_prev = c->sub_nlive[d - 1];
        if (i < 8 * nl_prev) {
            // A child on no face of its root's cell is interior: its levels are its parent's,
            // restricted to its octant, with nothing of its own or deeper; test that first
            // (the same test as below, without touching any record)
            const int pl = c->sub_lbase[d - 1] + (i >> 3);
            if (child_touch(A.touch[pl], i & 7) == 0u) {
                float C[27];
#pragma unroll
                for (int kk = 0; kk < 27; ++kk) C[kk] = 0.0f;
                add_subdivided(A.poly + pl, (size_t)A.cap_live, (unsigned)(i & 7), 1, C);
                const float mag = A.poly[(size_t)27 * A.cap_live + pl];
                float lo = C[0], hi = C[0];
#pragma unroll
                for (int kk = 1; kk < 27; ++kk) { lo = fminf(lo, C[kk]); hi = fmaxf(hi, C[kk]); }
                const float iso = c->iso;
                const float margin = 1e-4f * (mag + fabsf(iso));
                if (lo - iso > margin || hi - iso < -margin) return 0u;   // certain sign
            }
        }
        const int slot = c->sub_cbase[d] + i;
        int g, vnode, k, pslot, pa;   // pa: parent as a neighbour-table entry
        float cc[3];
        if (i < 8 * nl_prev) {
            pslot = A.live[c->sub_lbase[d - 1] + (i >> 3)];
            const int ch = i & 7;
            g = A.group[pslot];
            const int* G = groups + (size_t)g * kGroupRec;
            const int pl = A.vnode[pslot] - G[3] - sub_level_off(G[0], G[2], d - 1);
            vnode = G[3] + sub_level_off(G[0], G[2], d) + 8 * pl + ch;
            k = A.key[pslot] | (ch << (3 * (depth - d)));
            const float w = __int_as_float((126 - d) << 23);   // 2^-(d+1)
            cc[0] = (ch & 4) ? __fadd_rn(A.cx[pslot], w) : __fsub_rn(A.cx[pslot], w);
            cc[1] = (ch & 2) ? __fadd_rn(A.cy[pslot], w) : __fsub_rn(A.cy[pslot], w);
            cc[2] = (ch & 1) ? __fadd_rn(A.cz[pslot], w) : __fsub_rn(A.cz[pslot], w);
            pa = na + A.vnode[pslot];
        } else {
            const int r = c->sub_rstart[d] + (i - 8 * nl_prev);
            g = root_group[r];
            const int* G = groups + (size_t)g * kGroupRec;
            vnode = G[3] + (r - G[1]);
            const int root_node = sub_root[r];
            k = key[root_node];
            cc[0] = cc[1] = cc[2] = 0.5f;
            float w = 0.25f;
            for (int l = depth - 1; l >= depth - d; --l) {
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    if ((k >> (3 * l + 2 - a)) & 1) cc[a] = __fadd_rn(cc[a], w);
                    else cc[a] = __fsub_rn(cc[a], w);
                }
                w = __fdiv_rn(w, 2.0f);
            }
            pslot = -1;
            pa = parent[root_node];
        }
        const int* G = groups + (size_t)g * kGroupRec;
        const bool at_root_depth = (d == G[0]);
        const int local = vnode - G[3] - sub_level_off(G[0], G[2], d);
        const int off_prev = (d > G[0]) ? sub_level_off(G[0], G[2], d - 1) : 0;
        const int off_cur = sub_level_off(G[0], G[2], d);
        int contrib = 0;
        bool deeper = false;   // an octree neighbour with children reaches below depth d
        const int son = (k >> (3 * (depth - d))) & 7;
        // Position inside the root's cell: rel = the Morton code of the node's L = d - rd
        // levels below its root (x = bit 2, y = bit 1, z = bit 0 of every triple).  A
        // neighbour inside the same root's cell is the node at the shifted code in the same
        // root's block (dilated-integer +-1 per axis); only neighbours outside the root's
        // cell need the parent-based look-up.
        const unsigned lmask = (1u << (3 * (d - G[0]))) - 1u;
        const unsigned rel = (unsigned)local & lmask;
        unsigned cmp[3][3];
        bool ok[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const unsigned M = (0x24924924u >> a) & lmask;   // x, y, z bit positions
            const unsigned u = 4u >> a;
            const unsigned cm = rel & M;
            cmp[a][0] = (cm - u) & M;
            cmp[a][1] = cm;
            cmp[a][2] = ((cm | ~M) + u) & M;
            ok[a][0] = cm != 0u;
            ok[a][1] = true;
            ok[a][2] = cm != M;
        }
        const int r = G[1] + (int)((unsigned)local >> (3 * (d - G[0])));
        // An interior node (below its root, all 27 neighbours inside the root's cell) has only
        // zero-valued sub nodes around it and nothing deeper: it is tested before anything is
        // built.  Other nodes are built first (the test may read their own level).  Only live
        // nodes are referred to later (children, value chains), so a node dropped here needs
        // nothing else.
        const bool interior = ok[0][0] && ok[0][2] && ok[1][0] && ok[1][2] && ok[2][0] && ok[2][2];
        // values of the own level's neighbours, read as each neighbour is found: below its
        // root only octree neighbours carry one (deeper subdivision nodes are never roots).
        // Every array read in the loop is written by earlier launches only: read-only loads
        // let the 27 look-up chains overlap instead of waiting behind each A.neigh store
        float y[27];
#pragma unroll
        for (int kk = 0; kk < 27; ++kk) y[kk] = 0.0f;
        if (!interior) {
            // Three slabs of 9 neighbours, each in three rounds of independent loads (all
            // addresses clamped to valid entries, results selected afterwards): the parent's
            // neighbour row; the redirect, child and first-child entries of those neighbours;
            // the values and grandchildren of the neighbours found
            const bool has_row = pslot >= 0 || pa >= 0;
            const int* rowp = (pslot >= 0) ? A.neigh + pslot : neigh + (pa >= 0 ? pa : 0);
            const size_t rstride = (pslot >= 0) ? A.cstride : stride;
#pragma unroll
            for (int ix = 0; ix < 3; ++ix) {
                int np[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int kk = 9 * ix + q;
                    int lp, lc;
                    nb_lut(son, kk, lp, lc);
                    const int t = __ldg(rowp + (size_t)lp * rstride);
                    np[q] = has_row ? t : -1;
                }
                int og[9], fc[9], os[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int kk = 9 * ix + q;
                    int lp, lc;
                    nb_lut(son, kk, lp, lc);
                    const int n0 = (np[q] >= 0 && np[q] < na) ? np[q] : 0;
                    og[q] = __ldg(ov_group + (size_t)lc * stride + n0);
                    os[q] = __ldg(ov_sub + (size_t)lc * stride + n0);
                    fc[q] = __ldg(first_child + n0);
                }
                int vv[9];
                bool plain_oct[9];
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int kk = 9 * ix + q;
                    const int iy = (kk / 3) % 3, iz = kk % 3;
                    int lp, lc;
                    nb_lut(son, kk, lp, lc);
                    int v = -1;
                    plain_oct[q] = false;
                    if (ok[0][ix] && ok[1][iy] && ok[2][iz]) {
                        const unsigned relk = cmp[0][ix] | cmp[1][iy] | cmp[2][iz];
                        v = na + vnode + (int)relk - (int)rel;
                        if (at_root_depth) contrib = 1;   // the node itself, a root
                    } else {
                        const int n = np[q];
                        if (n != -1) {
                            if (n < na) {
                                if (og[q] == g) {
                                    // redirected child pointer of this group's root
                                    v = na + G[3] + os[q];
                                } else {
                                    v = (fc[q] == -1) ? -1 : fc[q] + lc;
                                    plain_oct[q] = true;
                                }
                            } else {
                                // a sub node of depth d - 1 in this group: its children are
                                // at 8 x its index in level d
                                v = na + G[3] + off_cur + 8 * (n - na - G[3] - off_prev) + lc;
                            }
                        }
                        // a contributing neighbour is an octree node or a root; the subdivision
                        // nodes at a group's root depth are exactly its roots, and deeper ones
                        // are never roots
                        if (v >= 0 && (v < na || at_root_depth)) contrib = 1;
                    }
                    vv[q] = v;
                }
#pragma unroll
                for (int q = 0; q < 9; ++q) {
                    const int v = vv[q];
                    const bool oct = v >= 0 && v < na;
                    const int v0 = oct ? v : 0;
                    const float xv = __ldg(x + v0);
                    const int gc = __ldg(first_child + v0);
                    if (plain_oct[q] && v >= 0 && d < depth && gc != -1) deeper = true;
                    if (oct && !at_root_depth) y[9 * ix + q] = xv;
                }
#pragma unroll
                for (int q = 0; q < 9; ++q) A.neigh[(size_t)(9 * ix + q) * A.cstride + slot] = vv[q];
            }
        }
        const int prec = (pslot >= 0) ? pslot : -2 - pa;
        // nearest contributing node on the path to the root (itself when it contributes;
        // roots always do): lets the value chains skip non-contributing levels in one hop
        const int jump = contrib ? slot : ((pslot >= 0) ? __ldg(A.jump + pslot) : slot);
        // Bernstein coefficients of the levels up to d on the node's cell
        float C[27], mag;
        if (at_root_depth) {
            root_coefficients(r, sub_root[r], d, cc[0], cc[1], cc[2], depth, neigh, stride, parent, enc, x,
                              root_poly, cap_poly, C, mag);
        } else {
            const int pl = c->sub_lbase[d - 1] + (i >> 3);   // the parent's live entry
#pragma unroll
            for (int kk = 0; kk < 27; ++kk) C[kk] = 0.0f;
            add_subdivided(A.poly + pl, (size_t)A.cap_live, (unsigned)(i & 7), 1, C);
            mag = __ldg(A.poly + (size_t)27 * A.cap_live + pl);
            if (contrib) {   // its own level (octree neighbours; never for an interior node)
                const float sc = (float)(1 << d);
                const int base = (1 << d) - 1;
                sign_level(y, base + (int)__fmul_rn(cc[0], sc), base + (int)__fmul_rn(cc[1], sc),
                           base + (int)__fmul_rn(cc[2], sc), cc[0], cc[1], cc[2], 0.5f, C, mag);
            }
            if (!deeper) {
                float lo = C[0], hi = C[0];
#pragma unroll
                for (int kk = 1; kk < 27; ++kk) { lo = fminf(lo, C[kk]); hi = fmaxf(hi, C[kk]); }
                const float iso = c->iso;
                const float margin = 1e-4f * (mag + fabsf(iso));
                if (lo - iso > margin || hi - iso < -margin) return 0u;   // certain sign
            }
        }
        float* stash = sub_poly_stash();
#pragma unroll
        for (int kk = 0; kk < 27; ++kk) stash[kk * kBlock + threadIdx.x] = C[kk];
        stash[27 * kBlock + threadIdx.x] = mag;
        const unsigned touch = at_root_depth ? 0x3fu
                                             : child_touch(__ldg(A.touch + c->sub_lbase[d - 1] + (i >> 3)), i & 7);
        stash[28 * kBlock + threadIdx.x] = __uint_as_float(touch);
        stash[29 * kBlock + threadIdx.x] = __int_as_float(vnode);
        if (interior) {
#pragma unroll
            for (int kk = 0; kk < 27; ++kk) {
                const int ix = kk / 9, iy = (kk / 3) % 3, iz = kk % 3;
                const unsigned relk = cmp[0][ix] | cmp[1][iy] | cmp[2][iz];
                A.neigh[(size_t)kk * A.cstride + slot] = na + vnode + (int)relk - (int)rel;
            }
        }
        A.depth[slot] = d;
        A.cx[slot] = cc[0];
        A.cy[slot] = cc[1];
        A.cz[slot] = cc[2];
        A.parent[slot] = prec;
        A.jump[slot] = jump;
        A.vnode[slot] = vnode;
        A.key[slot] = k;
        A.group[slot] = g;
        return 1u;
    }
    __device__ void rebase() { PSR_CLOUD(c, groups, sub_root, root_group, root_self, key, neigh, first_child, parent, ov_group, ov_sub, enc, x, root_poly, A); }   // to cloud blockIdx.y
};
struct SubLevelStore {
    Counters* c;
    int d, depth;
    SubArrays A;
    unsigned* err;
    __device__ void operator()(int i, unsigned pre, unsigned live) const {
        if (!live) return;
        const int at = c->sub_lbase[d] + (int)pre;
        if (at >= A.cap_live) { atomicOr(err, kErrCapacity); return; }
        const int slot = c->sub_cbase[d] + i;
        A.live[at] = slot;
        const float* stash = sub_poly_stash();
#pragma unroll
        for (int k = 0; k < 28; ++k) A.poly[(size_t)k * A.cap_live + at] = stash[k * kBlock + threadIdx.x];
        A.touch[at] = (unsigned char)__float_as_uint(stash[28 * kBlock + threadIdx.x]);
        if (d == depth) {
            if ((int)pre >= A.cap_live_d) { atomicOr(err, kErrCapacity); return; }
            A.lv_vnode[pre] = __float_as_int(stash[29 * kBlock + threadIdx.x]);
        }
    }
    // chains the counts: candidates of depth d + 1 = 8 x live of depth d + roots of d + 1
    __device__ void done(unsigned total) const {
        const int nl = (int)total;
        c->sub_nlive[d] = nl;
        const int cend = c->sub_cbase[d] + c->sub_cand[d];
        if (d < depth) {
            const long long nc = 8LL * nl + c->sub_nroots[d + 1];
            c->sub_cbase[d + 1] = cend;
            c->sub_lbase[d + 1] = c->sub_lbase[d] + nl;
            if (cend + nc > (long long)A.cap_nodes || c->sub_lbase[d] + nl > A.cap_live) {
                atomicOr(err, kErrCapacity);
                c->sub_cand[d + 1] = 0;
            } else {
                c->sub_cand[d + 1] = (int)nc;
            }
        } else {
            // live cells beyond either capacity were not stored (and flagged)
            int n = nl;
            if (n > A.cap_live_d) n = A.cap_live_d;
            if (n > A.cap_live - c->sub_lbase[d]) n = A.cap_live - c->sub_lbase[d];
            c->n_sub_nodes = cend;
            c->n_sub_dnodes = n;
        }
    }
    __device__ void rebase() { PSR_CLOUD(c, A, err); }   // to cloud blockIdx.y
};

// index of virtual node v among the live depth-D cells (sorted), or -1
__device__ __forceinline__ int live_index(const int* lv_vnode, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (lv_vnode[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return (lo < n && lv_vnode[lo] == v) ? lo : -1;
}

// per live depth-D cell: the live index of each same-depth sub neighbour (-1: none, an
// octree node, or a cell with a certain sign); one thread per (cell, slot)
__global__ void __launch_bounds__(kBlock) k_sub_live_neigh(const Counters* c, int depth, SubArrays A,
                                                           int* lv_nb, size_t dstride, int na) {
    PSR_CLOUD(c, A, lv_nb);
    const int nl = c->n_sub_dnodes;
    const int lb = c->sub_lbase[depth];
    const long long n = 27LL * nl;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const int L = (int)(t / 27), k = (int)(t - 27LL * L);
        const int v = A.neigh[(size_t)k * A.cstride + A.live[lb + L]];
        lv_nb[(size_t)k * dstride + L] = (k == 13) ? L : ((v >= na) ? live_index(A.lv_vnode, nl, v - na) : -1);
    }
}

// vertex ownership among the live depth-D cells (initSubdivideVertexOwner :698-763): a corner
// is owned by the smallest-key live cell around it.  Cells with a certain sign take no part:
// every corner of a live cell still gets exactly one record, the records of crossing edges
// keep their owners (every cell around a crossing edge has a sign change, so is live), and a
// vertex value does not depend on the cell that evaluates it (the same nonzero terms in the
// same order), so the mesh is unchanged.
__global__ void __launch_bounds__(kBlock) k_sub_vertex_owner(const Counters* c, int depth, SubArrays A,
                                                             const int* lv_nb, size_t dstride,
                                                             unsigned char* s_vmask) {
    PSR_CLOUD(c, A, lv_nb, s_vmask);
    const int nl = c->n_sub_dnodes;
    const int lb = c->sub_lbase[depth];
    PSR_GRID_STRIDE(L, nl) {
        const int myk = A.key[A.live[lb + L]];
        unsigned smaller = 0;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            if (k == 13) continue;
            const int nb = lv_nb[(size_t)k * dstride + L];
            if (nb >= 0 && A.key[A.live[lb + nb]] < myk) smaller |= 1u << k;
        }
        unsigned m = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) if (!(smaller & vertex_cells(q))) m |= 1u << q;
        s_vmask[L] = (unsigned char)m;
    }
}

struct SubVertexStore {
    const unsigned char* vmask;
    const Counters* c;
    int depth;
    SubArrays A;
    float *vx, *vy, *vz;
    int *vowner, *vkind;
    int cap;
    unsigned* err;
    __device__ void operator()(int L, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        if ((int)(pre + cnt) > cap) { atomicOr(err, kErrCapacity); return; }
        const int s = A.live[c->sub_lbase[depth] + L];
        const unsigned m = vmask[L];
        const float hw = 1.0f / (float)(1 << (depth + 1));
        int q = (int)pre;
        for (int k = 0; k < 8; ++k) {
            if (!((m >> k) & 1)) continue;
            vx[q] = __fadd_rn(A.cx[s], (float)(2 * (k & 1) - 1) * hw);
            vy[q] = __fadd_rn(A.cy[s], (float)(2 * ((k >> 1) & 1) - 1) * hw);
            vz[q] = __fadd_rn(A.cz[s], (float)(2 * ((k >> 2) & 1) - 1) * hw);
            vowner[q] = L;
            vkind[q] = k;
            ++q;
        }
    }
    __device__ void rebase() { PSR_CLOUD(vmask, c, A, vx, vy, vz, vowner, vkind, err); }   // to cloud blockIdx.y
};

// maintainSubdivideVertexNodePointer (:765-810): s_vtx indexed by live cell
__global__ void __launch_bounds__(kBlock) k_sub_vertex_maintain(const Counters* c, const int* lv_nb,
                                                                size_t dstride, const int* vowner, const int* vkind,
                                                                int* s_vtx) {
    PSR_CLOUD(c, lv_nb, vowner, vkind, s_vtx);
    const int V = c->n_sub_vertices;
    PSR_GRID_STRIDE(v, V) {
        const int ow = vowner[v];
        int mx, my, mz;
        corner_sides(vkind[v], mx, my, mz);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int ax = (j & 1) ? mx : 0, ay = (j & 2) ? my : 0, az = (j & 4) ? mz : 0;
            const int nb = lv_nb[(size_t)nslot(ax, ay, az) * dstride + ow];
            if (nb >= 0) s_vtx[(size_t)vertex_slot_of(ax, ay, az, mx, my, mz) * dstride + nb] = v + 1;
        }
    }
}

// edge ownership among the live depth-D cells (initSubdivideEdgeArray :812-886)
__global__ void __launch_bounds__(kBlock) k_sub_edge_owner(const Counters* c, int depth, SubArrays A,
                                                           const int* lv_nb, size_t dstride,
                                                           unsigned short* s_emask) {
    PSR_CLOUD(c, A, lv_nb, s_emask);
    const int nl = c->n_sub_dnodes;
    const int lb = c->sub_lbase[depth];
    PSR_GRID_STRIDE(L, nl) {
        const int myk = A.key[A.live[lb + L]];
        unsigned smaller = 0;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
            if (k == 13 || k == 0 || k == 2 || k == 6 || k == 8 || k == 18 || k == 20 || k == 24 || k == 26)
                continue;   // corner-diagonal cells touch no edge
            const int nb = lv_nb[(size_t)k * dstride + L];
            if (nb >= 0 && A.key[A.live[lb + nb]] < myk) smaller |= 1u << k;
        }
        unsigned m = 0;
#pragma unroll
        for (int e = 0; e < 12; ++e) if (!(smaller & edge_cells(e))) m |= 1u << e;
        s_emask[L] = (unsigned short)m;
    }
}

struct SubEdgeStore {
    const unsigned short* emask;
    int *eowner, *ekind;
    unsigned* edge_of_live;   // sub-edge prefix per live cell (for the part table)
    int cap;
    unsigned* err;
    __device__ void operator()(int L, unsigned pre, unsigned cnt) const {
        edge_of_live[L] = pre;
        if (!cnt) return;
        if ((int)(pre + cnt) > cap) { atomicOr(err, kErrCapacity); return; }
        const unsigned m = emask[L];
        int q = (int)pre;
        for (int e = 0; e < 12; ++e)
            if ((m >> e) & 1) { eowner[q] = L; ekind[q] = e; ++q; }
    }
    __device__ void rebase() { PSR_CLOUD(emask, eowner, ekind, edge_of_live, err); }   // to cloud blockIdx.y
};

// maintainSubdivideEdgeNodePointer (:888-949)
__global__ void __launch_bounds__(kBlock) k_sub_edge_maintain(const Counters* c, const int* lv_nb, size_t dstride,
                                                              const int* eowner, const int* ekind, int* s_edge) {
    PSR_CLOUD(c, lv_nb, eowner, ekind, s_edge);
    const int E = c->n_sub_edges;
    PSR_GRID_STRIDE(ei, E) {
        const int ow = eowner[ei], kind = ekind[ei];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int a[3];
            edge_offset(kind, j, a);
            const int nb = lv_nb[(size_t)nslot(a[0], a[1], a[2]) * dstride + ow];
            if (nb >= 0) s_edge[(size_t)edge_slot_of(kind, a) * dstride + nb] = ei + 1;
        }
    }
}

// implicit values of subdivision vertices (:956-1038): x = 0 inside subdivision space,
// a root stands for the octree node it replaces (same depth and position).  Every
// neighbour of a level is a same-depth cell, so its function index is the level node's
// own plus the slot offset.  A subdivision node's own index comes from its centre
// ((off + 1/2) / 2^d exactly).  The value is the sum, level after level from the owner's
// nearest contributing node up to the root and then 27 neighbour terms in slot order, of
// ((x Fx) Fy) Fz.  Eight lanes per vertex (four vertices per warp, whose chains of
// dependent loads overlap): the group's first lane finds the levels (subdivision nodes
// through the jump links, then the octree ancestors), the lanes evaluate the 3 basis values
// per axis of each level and form the terms in parallel, and the first lane adds them in
// that order (absent neighbours as +0, which leaves such a sum unchanged): the chain's
// dependent loads are paid once per level instead of once per term.
constexpr int kSvLanes = 8;
constexpr int kSvBlock = 128;
constexpr int kSvGroups = kSvBlock / kSvLanes;
constexpr int kSvMaxLevels = kMaxDepth + 1;
__global__ void __launch_bounds__(kSvBlock) k_sub_vertex_values(const Counters* c, int depth, const float* vx,
                                                                const float* vy, const float* vz, const int* vowner,
                                                                const int* neigh, size_t stride, const int* parent,
                                                                const int* groups, const int* root_self, SubArrays A,
                                                                const int* enc, const float* x, float* vvalue, int na) {
    PSR_CLOUD(c, vx, vy, vz, vowner, neigh, parent, groups, root_self, A, enc, x, vvalue);
    __shared__ int s_node[kSvGroups][kSvMaxLevels];   // slot (subdivision) or octree node
    __shared__ int s_o[kSvGroups][kSvMaxLevels][3];   // function index of the level's node
    __shared__ float s_t[kSvGroups][kSvMaxLevels * 27];
    __shared__ float s_b[kSvGroups][kSvMaxLevels][9];  // a level's 3 basis values per axis
    const int V = c->n_sub_vertices;
    const float iso = c->iso;
    const int lb = c->sub_lbase[depth];
    const int gl = threadIdx.x & (kSvLanes - 1), w = threadIdx.x / kSvLanes;
    const unsigned gmask = 0xffu << (threadIdx.x & 24);   // the group's lanes in its warp
    for (int v = blockIdx.x * kSvGroups + w; v < V; v += gridDim.x * kSvGroups) {
        const float qx = vx[v], qy = vy[v], qz = vz[v];
        const int own = A.live[lb + vowner[v]];
        const int* G = groups + (size_t)A.group[own] * kGroupRec;
        int nsub = 0, nlev = 0;
        if (gl == 0) {
            // levels whose 27 neighbours are all zero-valued subdivision nodes add nothing:
            // the jump links skip them
            int sn = A.jump[own], now = -1;
            while (nsub < kSvMaxLevels) {
                s_node[w][nsub++] = sn;
                const int p = A.parent[sn];
                if (p < 0) { now = -2 - p; break; }
                sn = A.jump[p];
            }
            nlev = nsub;
            for (; now != -1 && nlev < kSvMaxLevels; now = parent[now]) s_node[w][nlev++] = now;
        }
        nsub = __shfl_sync(gmask, nsub, 0, kSvLanes);
        nlev = __shfl_sync(gmask, nlev, 0, kSvLanes);
        __syncwarp(gmask);
        for (int l = gl; l < nlev; l += kSvLanes) {
            const int nd = s_node[w][l];
            int ox, oy, oz;
            if (l < nsub) {
                const int d = A.depth[nd];
                const float sc = (float)(1 << d);
                const int base = (1 << d) - 1;
                ox = base + (int)__fmul_rn(A.cx[nd], sc);
                oy = base + (int)__fmul_rn(A.cy[nd], sc);
                oz = base + (int)__fmul_rn(A.cz[nd], sc);
            } else {
                decode_fn_index(enc[nd], depth, ox, oy, oz);
            }
            s_o[w][l][0] = ox;
            s_o[w][l][1] = oy;
            s_o[w][l][2] = oz;
        }
        __syncwarp(gmask);
        // the 27 translates of a level share 3 basis values per axis: 9 evaluations per level
        for (int t = gl; t < nlev * 9; t += kSvLanes) {
            const int l = t / 9, r = t - 9 * l, a = r / 3;
            s_b[w][l][r] = basis32(s_o[w][l][a] - 1 + (r - 3 * a), a == 0 ? qx : (a == 1 ? qy : qz));
        }
        __syncwarp(gmask);
        for (int t = gl; t < nlev * 27; t += kSvLanes) {
            const int l = t / 27, k = t - 27 * l;
            const int nd = s_node[w][l];
            int nb = (l < nsub) ? A.neigh[(size_t)k * A.cstride + nd] : neigh[(size_t)k * stride + nd];
            if (nb >= na) nb = sub_value_node(nb, na, G, root_self);
            float term = 0.0f;
            if (nb >= 0) {
                const float bxk = s_b[w][l][k / 9];
                const float byk = s_b[w][l][3 + (k / 3) % 3];
                const float bzk = s_b[w][l][6 + k % 3];
                term = __fmul_rn(__fmul_rn(__fmul_rn(x[nb], bxk), byk), bzk);
            }
            s_t[w][t] = term;
        }
        __syncwarp(gmask);
        if (gl == 0) {
            float val = 0.0f;
            for (int l = 0; l < nlev; ++l) {
#pragma unroll
                for (int k = 0; k < 27; ++k) val = __fadd_rn(val, s_t[w][l * 27 + k]);
            }
            vvalue[v] = __fsub_rn(val, iso);
        }
        __syncwarp(gmask);
    }
}

struct SubCrossLoad {
    const int* eowner;   // live cell owning the edge
    const int* ekind;
    const int* s_vtx;
    size_t dstride;
    const float* vvalue;
    unsigned* err;
    __device__ unsigned operator()(int e) const {
        const int dn = eowner[e];
        const int kind = ekind[e];
        const int p[2] = {s_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][0]) * dstride + dn],
                          s_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][1]) * dstride + dn]};
        float ab[2];
        ptr_values(vvalue, p, ab, err);
        const float a = ab[0], b = ab[1];
        return (__fmul_rn(a, b) <= 0.0f) ? 1u : 0u;
    }
    __device__ void rebase() { PSR_CLOUD(eowner, ekind, s_vtx, vvalue, err); }   // to cloud blockIdx.y
};
struct SubCrossStore {
    const int* eowner;
    const int* ekind;
    const int* s_vtx;
    size_t dstride;
    const float* vvalue;
    const float *vx, *vy, *vz;
    unsigned* ecross;
    float* part_v;
    const int* voff_ptr;
    int cap;
    unsigned* err;
    __device__ void operator()(int e, unsigned pre, unsigned flag) const {
        ecross[e] = pre;
        if (!flag) return;
        const int at = *voff_ptr + (int)pre;
        if (at >= cap) { atomicOr(err, kErrCapacity); return; }
        const int dn = eowner[e];
        const int kind = ekind[e];
        const int v1 = s_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][0]) * dstride + dn] - 1;
        const int v2 = s_vtx[(size_t)__ldg(&g_tab.edge_vertex[kind][1]) * dstride + dn] - 1;
        if (v1 < 0 || v2 < 0) return;
        interp_point(vx[v1], vy[v1], vz[v1], vx[v2], vy[v2], vz[v2], kind >> 2, vvalue[v1], vvalue[v2],
                     &part_v[3 * (size_t)at]);
    }
    __device__ void rebase() { PSR_CLOUD(eowner, ekind, s_vtx, vvalue, vx, vy, vz, ecross, part_v, voff_ptr, err); }   // to cloud blockIdx.y
};

struct SubCubeLoad {
    const int* s_vtx;
    size_t dstride;
    const float* vvalue;
    int* cube_class;
    unsigned* err;
    __device__ unsigned operator()(int L) const {
        int p[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) p[q] = s_vtx[(size_t)q * dstride + L];
        float vq[8];
        ptr_values(vvalue, p, vq, err);
        int cls = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (vq[q] < 0.0f) cls |= 1 << q;
        cube_class[L] = cls;
        return (unsigned)__ldg(&g_tab.mc_count[cls]);
    }
    __device__ void rebase() { PSR_CLOUD(s_vtx, vvalue, cube_class, err); }   // to cloud blockIdx.y
};

// triangles of a live cell; indices relative to its group's first crossing
struct SubCubeStore {
    const int* cube_class;
    const int* s_edge;
    size_t dstride;
    const unsigned* ecross;
    const unsigned* group_cross0;   // per group: crossing prefix at its first edge
    const Counters* c;
    int depth;
    SubArrays A;
    int* part_t;
    const int* toff_ptr;
    int cap;
    unsigned* err;
    __device__ void operator()(int L, unsigned pre, unsigned cnt) const {
        if (!cnt) return;
        const int g = A.group[A.live[c->sub_lbase[depth] + L]];
        const unsigned base = group_cross0[g];
        const int cls = cube_class[L];
        const unsigned long long tri = __ldg(&g_tab.mc_tri[cls]);
        for (int t = 0; t < (int)cnt; ++t) {
            const int at = *toff_ptr + (int)pre + t;
            if (at >= cap) { atomicOr(err, kErrCapacity); continue; }
            for (int a = 0; a < 3; ++a) {
                const int e = (int)((tri >> (4 * (3 * t + a))) & 0xF);
                const int ei = s_edge[(size_t)e * dstride + L] - 1;
                part_t[3 * (size_t)at + a] = (ei >= 0) ? (int)(ecross[ei] - base) : -1;
            }
        }
    }
    __device__ void rebase() { PSR_CLOUD(cube_class, s_edge, ecross, group_cross0, c, A, part_t, toff_ptr, err); }   // to cloud blockIdx.y
};

// first live index at or after virtual node v
__device__ __forceinline__ int live_lower_bound(const int* lv_vnode, int n, int v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (lv_vnode[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// per-group first sub edge / first crossing / first triangle -> part table
// parts: [0] main, [1 + g] group g.  part record: vstart, vcount, tstart, tcount
__global__ void k_part_table(Counters* c, int depth, const int* groups, const int* lv_vnode,
                             const unsigned* edge_of_live, const unsigned* ecross_sub, const unsigned* tri_of_live,
                             unsigned* group_cross0, int* parts) {
    PSR_CLOUD(c, groups, lv_vnode, edge_of_live, ecross_sub, tri_of_live, group_cross0, parts);
    const int ng = c->n_groups;
    const int nE = c->n_sub_edges;
    const int nl = c->n_sub_dnodes;
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        parts[0] = 0;
        parts[1] = c->n_cross;
        parts[2] = 0;
        parts[3] = c->n_tri;
    }
    PSR_GRID_STRIDE(g, ng) {   // one thread per group (independent entries)
        const int* G = groups + (size_t)g * kGroupRec;
        const int v0 = G[3] + sub_level_off(G[0], G[2], depth);
        const int v1 = G[3] + G[4];
        // first sub edge of the group = edge prefix at its first live cell
        const int L0 = live_lower_bound(lv_vnode, nl, v0);
        const int L1 = live_lower_bound(lv_vnode, nl, v1);
        const int e0 = (L0 < nl) ? (int)edge_of_live[L0] : nE;
        const int e1 = (L1 < nl) ? (int)edge_of_live[L1] : nE;
        const unsigned x0 = (e0 < nE) ? ecross_sub[e0] : (unsigned)c->n_sub_cross;
        const unsigned x1 = (e1 < nE) ? ecross_sub[e1] : (unsigned)c->n_sub_cross;
        const unsigned t0 = (L0 < nl) ? tri_of_live[L0] : (unsigned)c->n_sub_tri;
        const unsigned t1 = (L1 < nl) ? tri_of_live[L1] : (unsigned)c->n_sub_tri;
        group_cross0[g] = x0;
        int* P = parts + 4 * (size_t)(g + 1);
        P[0] = c->n_cross + (int)x0;
        P[1] = (int)(x1 - x0);
        P[2] = c->n_tri + (int)t0;
        P[3] = (int)(t1 - t0);
    }
}

// ------------------------------------------------------------------------------------
// insertion (insertTriangle :1247-1282): drop vertices with |x| < 1e-6, offset triangle
// indices by the vertices kept before the part, drop triangles out of the part's range
// ------------------------------------------------------------------------------------
struct KeepVertexLoad {
    const float* part_v;
    __device__ unsigned operator()(int v) const { return (fabsf(part_v[3 * (size_t)v]) < 1e-6f) ? 0u : 1u; }
    __device__ void rebase() { PSR_CLOUD(part_v); }   // to cloud blockIdx.y
};
struct KeepVertexStore {
    const float* part_v;
    float* mesh_v;
    unsigned* kept_prefix;
    int cap;
    unsigned* err;
    __device__ void operator()(int v, unsigned pre, unsigned keep) const {
        kept_prefix[v] = pre;
        if (!keep) return;
        if ((int)pre >= cap) { atomicOr(err, kErrCapacity); return; }
        mesh_v[3 * (size_t)pre] = part_v[3 * (size_t)v];
        mesh_v[3 * (size_t)pre + 1] = part_v[3 * (size_t)v + 1];
        mesh_v[3 * (size_t)pre + 2] = part_v[3 * (size_t)v + 2];
    }
    __device__ void rebase() { PSR_CLOUD(part_v, mesh_v, kept_prefix, err); }   // to cloud blockIdx.y
};

__device__ __forceinline__ int find_part(const int* parts, int np, int t) {
    int lo = 0, hi = np - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (parts[4 * mid + 2] <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

struct KeepTriLoad {
    const int* part_t;
    const int* parts;
    const int* np_ptr;
    __device__ unsigned operator()(int t) const {
        const int p = find_part(parts, *np_ptr, t);
        const int vc = parts[4 * p + 1];
        for (int a = 0; a < 3; ++a) {
            int l = part_t[3 * (size_t)t + a];
            if (l < 0 || l >= vc) return 0u;
        }
        return 1u;
    }
    __device__ void rebase() { PSR_CLOUD(part_t, parts, np_ptr); }   // to cloud blockIdx.y
};
struct KeepTriStore {
    const int* part_t;
    const int* parts;
    const int* np_ptr;
    const unsigned* kept_prefix;
    const int* n_staged_v;
    const int* n_kept_v;
    int* mesh_t;
    int cap;
    unsigned* err;
    __device__ void operator()(int t, unsigned pre, unsigned keep) const {
        if (!keep) return;
        if ((int)pre >= cap) { atomicOr(err, kErrCapacity); return; }
        const int p = find_part(parts, *np_ptr, t);
        const int vs = parts[4 * p];
        const int prev = (vs < *n_staged_v) ? (int)kept_prefix[vs] : *n_kept_v;
        for (int a = 0; a < 3; ++a) mesh_t[3 * (size_t)pre + a] = part_t[3 * (size_t)t + a] + prev;
    }
    __device__ void rebase() { PSR_CLOUD(part_t, parts, np_ptr, kept_prefix, n_staged_v, n_kept_v, mesh_t, err); }   // to cloud blockIdx.y
};

__global__ void k_count_parts(Counters* c, int* n_parts, int* n_staged_v, int* n_staged_t, int cap_v, int cap_t) {
    PSR_CLOUD(c, n_parts, n_staged_v, n_staged_t);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *n_parts = 1 + c->n_groups;
        int nv = c->n_cross + c->n_sub_cross, nt = c->n_tri + c->n_sub_tri;
        if (nv > cap_v || nt > cap_t) atomicOr(&c->error, kErrCapacity);
        *n_staged_v = nv < cap_v ? nv : cap_v;
        *n_staged_t = nt < cap_t ? nt : cap_t;
    }
}

// Vertex, edge and face records of the octree: they need only the octree, so they are
// issued on their own stream beside the divergence and the solve (ws.stream, ws.scan and
// the scan total are the caller's for that stream).
cudaError_t mesh_geometry_impl(Workspace& ws, const MeshBufs& mb, unsigned* total) {
    cudaStream_t s = ws.stream;
    const int D = ws.depth;
    Counters* c = ws.cnt;
    unsigned* err = &c->error;
    const size_t stride = (size_t)ws.cap.nodes;
    const int gm = grid_for(ws, ws.cap.nodes);
    cudaError_t e;
    k_mesh_reset<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.node_vtx, ws.node_edge, ws.node_face, mb.ov_group, mb.ov_sub, stride);
    // vertices
    k_vertex_owner<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.key, ws.neigh, stride, ws.vmask);
    e = launch_scan<1>(PopcLoad8{ws.vmask},
                    VertexStore{ws.vmask, ws.ndepth, ws.ctr_x, ws.ctr_y, ws.ctr_z, ws.v_x, ws.v_y, ws.v_z, ws.v_owner,
                                ws.v_kind, ws.v_depth, ws.cap.vertices, err},
                    &c->n_nodes, 0, ws.scan, total, err, s, ScanCount{&c->n_vertices, ws.cap.vertices});
    if (e != cudaSuccess) return e;
    k_vertex_maintain<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.neigh, stride, ws.v_owner, ws.v_kind, ws.node_vtx);
    // edges (D level)
    k_edge_owner<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, D, ws.key, ws.neigh, stride, ws.emask16);
    e = launch_scan<1>(PopcLoad16{ws.emask16},
                    EdgeStore{ws.emask16, &c->level_base[D], ws.e_owner, ws.e_kind, ws.cap.edges, err},
                    &c->level_count[D], 0, ws.scan, total, err, s, ScanCount{&c->n_edges, ws.cap.edges});
    if (e != cudaSuccess) return e;
    k_edge_maintain<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.neigh, stride, ws.e_owner, ws.e_kind, ws.node_edge);
    // faces
    k_face_owner<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.key, ws.neigh, stride, ws.fmask);
    e = launch_scan<1>(PopcLoad8{ws.fmask},
                    FaceStore{ws.fmask, ws.key, ws.ndepth, ws.parent, D, ws.f_owner, ws.f_kind, ws.f_hasparent,
                              ws.cap.faces, err},
                    &c->n_nodes, 0, ws.scan, total, err, s, ScanCount{&c->n_faces, ws.cap.faces});
    if (e != cudaSuccess) return e;
    k_face_maintain<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, ws.neigh, stride, ws.f_owner, ws.f_kind, ws.node_face);
    return cudaGetLastError();
}

cudaError_t mesh_build_impl(Workspace& ws, const MeshBufs& mb) {
    cudaStream_t s = ws.stream;
    const int D = ws.depth;
    Counters* c = ws.cnt;
    unsigned* err = &c->error;
    unsigned* total = (unsigned*)&c->scan_total;
    const size_t stride = (size_t)ws.cap.nodes;
    const int gm = grid_for(ws, ws.cap.nodes);
    cudaError_t e;
    // implicit values
    k_vertex_values<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, D, ws.v_x, ws.v_y, ws.v_z, ws.v_owner, ws.v_kind, ws.v_depth, ws.neigh,
                                          stride, ws.parent, ws.first_child, ws.enc, ws.xsol, ws.vvalue);
    // crossings -> staged vertices of the main part
    e = launch_scan<1>(CrossLoad{ws.e_owner, ws.e_kind, ws.node_vtx, stride, ws.vvalue, err},
                    CrossStore{ws.e_owner, ws.e_kind, ws.node_vtx, stride, ws.vvalue, ws.v_x, ws.v_y, ws.v_z,
                               ws.e_cross, ws.part_v, 0, ws.part_cap_v, err},
                    &c->n_edges, 0, ws.scan, total, err, s, ScanCount{&c->n_cross, ws.part_cap_v});
    if (e != cudaSuccess) return e;
    // face hits must start cleared
    fill_words((unsigned*)ws.face_hit, 0u, ws.cap.faces, ws.batch, s);
    e = launch_scan<1>(CubeLoad{ws.node_vtx, stride, &c->level_base[D], ws.vvalue, ws.cube_class, err},
                    CubeStore{ws.cube_class, &c->level_base[D], ws.node_edge, ws.node_face, stride, ws.e_cross,
                              ws.parent, ws.f_hasparent, ws.face_hit, ws.part_t, 0, ws.part_cap_t, err},
                    &c->level_count[D], 0, ws.scan, total, err, s, ScanCount{&c->n_tri, ws.part_cap_t});
    if (e != cudaSuccess) return e;
    // subdivision roots among nodes of depth < D
    e = launch_scan<1>(RootLoad{ws.node_vtx, ws.node_face, stride, ws.vvalue, ws.face_hit, ws.first_child, err},
                    RootStore{ws.sub_root, ws.cap.nodes, err}, &c->level_base[D], 0, ws.scan, total, err, s, ScanCount{&c->n_subroots, ws.cap.nodes});
    if (e != cudaSuccess) return e;
    // subdivision groups
    e = launch_scan(GroupFlagLoad{ws.sub_root, ws.ndepth, D - 4},
                    GroupFlagStore{ws.root_group, mb.groups, mb.max_groups, err}, &c->n_subroots, 0, ws.scan,
                    total, err, s, ScanCount{}, 1);
    if (e != cudaSuccess) return e;
    k_group_count<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, total, mb.max_groups);
    k_group_sizes<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, D, ws.sub_root, ws.ndepth, mb.groups);
    e = launch_scan(GroupFieldLoad{mb.groups, 4}, GroupFieldStore{mb.groups, 3}, &c->n_groups, 0, ws.scan, total, err,
                    s, ScanCount{}, 1);
    if (e != cudaSuccess) return e;
    k_group_totals<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, total, ws.cap.nodes);
    k_root_overlay<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, D, ws.sub_root, ws.ndepth, ws.key, ws.parent, ws.neigh, ws.root_group,
                                         mb.groups, ws.sub_root_depth, ws.root_self, mb.ov_group, mb.ov_sub, stride);
    return cudaGetLastError();
}

// Subdivision nodes appear in neighbour tables as cap.nodes + virtual index: every such
// number is larger than any octree index, which is all the kernels compare against.
cudaError_t mesh_build_sub(Workspace& ws, const MeshBufs& mb) {
    cudaStream_t s = ws.stream;
    const int D = ws.depth;
    Counters* c = ws.cnt;
    unsigned* err = &c->error;
    unsigned* total = (unsigned*)&c->scan_total;
    const size_t stride = (size_t)ws.cap.nodes;
    const size_t dstride = (size_t)ws.cap.sub_dnodes;
    const int na = ws.cap.nodes;
    // kernels over live depth-D cells and the scans of the subdivision: sized for a few
    // thousand live cells (one block per SM, grid-stride beyond) up to depth 7; the trees of
    // depth 8 and 9 have hundreds of thousands to millions, four blocks per SM
    const int gl = D >= 8 ? 4 * ws.num_sms : ws.num_sms;
    const int sbps = D >= 8 ? 4 : 1;
    cudaError_t e;
    SubArrays A{ws.c_vnode, ws.c_key, ws.c_group, ws.c_parent, ws.c_jump, ws.c_depth, ws.c_cx, ws.c_cy, ws.c_cz,
                ws.c_neigh, (size_t)ws.cap.sub_nodes, ws.c_live, ws.c_poly, ws.c_touch, ws.lv_vnode,
                ws.cap.sub_nodes, ws.cap.sub_live, ws.cap.sub_dnodes};
    k_sub_setup<<<PSR_GRID(ws, 1), 32, 0, s>>>(c, D, ws.sub_root_depth, ws.cap.sub_nodes);   // kMaxDepth + 2 <= 32 lanes
    k_root_poly<<<PSR_GRID(ws, grid_for(ws, ws.cap_poly)), kBlock, 0, s>>>(c, D, ws.sub_root, ws.ndepth, ws.ctr_x, ws.ctr_y,
                                                             ws.ctr_z, ws.neigh, stride, ws.parent, ws.enc, ws.xsol,
                                                             ws.root_poly, ws.cap_poly);
    // depth after depth: candidates (children of the live nodes above, then the roots of this
    // depth), their neighbours and sign tests; the live ones are compacted in order
    for (int d = 1; d <= D; ++d) {
        e = launch_scan<1>(SubLevelLoad{c, d, D, na, mb.groups, ws.sub_root, ws.root_group, ws.root_self, ws.key,
                                        ws.neigh, stride, ws.first_child, ws.parent, mb.ov_group, mb.ov_sub, ws.enc,
                                        ws.xsol, ws.root_poly, ws.cap_poly, A},
                           SubLevelStore{c, d, D, A, err}, &c->sub_cand[d], 0, ws.scan, total, err, s, ScanCount{},
                           sbps);
        if (e != cudaSuccess) return e;
    }
    // the live depth-D cells carry every record from here on, indexed by their live index
    k_sub_live_neigh<<<PSR_GRID(ws, 2 * gl), kBlock, 0, s>>>(c, D, A, ws.lv_nb, dstride, na);
    // s_vtx / s_edge need no clearing: every slot of a live cell is written by the owner of
    // that vertex / edge
    k_sub_vertex_owner<<<PSR_GRID(ws, gl), kBlock, 0, s>>>(c, D, A, ws.lv_nb, dstride, ws.s_vmask);
    e = launch_scan<2>(PopcLoad8{ws.s_vmask},
                       SubVertexStore{ws.s_vmask, c, D, A, ws.sv_x, ws.sv_y, ws.sv_z, ws.sv_owner, ws.sv_kind,
                                      8 * ws.cap.sub_dnodes, err},
                       &c->n_sub_dnodes, 0, ws.scan, total, err, s, ScanCount{&c->n_sub_vertices, 8 * ws.cap.sub_dnodes},
                       sbps);
    if (e != cudaSuccess) return e;
    k_sub_vertex_maintain<<<PSR_GRID(ws, gl), kBlock, 0, s>>>(c, ws.lv_nb, dstride, ws.sv_owner, ws.sv_kind, ws.s_vtx);
    k_sub_edge_owner<<<PSR_GRID(ws, gl), kBlock, 0, s>>>(c, D, A, ws.lv_nb, dstride, ws.s_emask);
    e = launch_scan<2>(PopcLoad16{ws.s_emask},
                       SubEdgeStore{ws.s_emask, ws.se_owner, ws.se_kind, mb.edge_of_dnode, 12 * ws.cap.sub_dnodes, err},
                       &c->n_sub_dnodes, 0, ws.scan, total, err, s, ScanCount{&c->n_sub_edges, 12 * ws.cap.sub_dnodes},
                       sbps);
    if (e != cudaSuccess) return e;
    k_sub_edge_maintain<<<PSR_GRID(ws, gl), kBlock, 0, s>>>(c, ws.lv_nb, dstride, ws.se_owner, ws.se_kind, ws.s_edge);
    k_sub_vertex_values<<<PSR_GRID(ws, 16 * ws.num_sms), kSvBlock, 0, s>>>(
        c, D, ws.sv_x, ws.sv_y, ws.sv_z, ws.sv_owner, ws.neigh, stride, ws.parent, mb.groups, ws.root_self, A, ws.enc,
        ws.xsol, ws.sv_value, na);
    // crossings: staged after the main part's vertices
    e = launch_scan<2>(SubCrossLoad{ws.se_owner, ws.se_kind, ws.s_vtx, dstride, ws.sv_value, err},
                       SubCrossStore{ws.se_owner, ws.se_kind, ws.s_vtx, dstride, ws.sv_value, ws.sv_x, ws.sv_y,
                                     ws.sv_z, ws.se_cross, ws.part_v, &c->n_cross, ws.part_cap_v, err},
                       &c->n_sub_edges, 0, ws.scan, total, err, s, ScanCount{&c->n_sub_cross, ws.part_cap_v}, sbps);
    if (e != cudaSuccess) return e;
    // triangle prefix per live cell
    e = launch_scan<2>(SubCubeLoad{ws.s_vtx, dstride, ws.sv_value, ws.s_cube_class, err},
                       StoreExclusive{mb.tri_of_dnode}, &c->n_sub_dnodes, 0, ws.scan, total, err, s,
                       ScanCount{&c->n_sub_tri, ws.part_cap_t}, sbps);
    if (e != cudaSuccess) return e;
    k_part_table<<<PSR_GRID(ws, grid_for(ws, 1 << 16)), kBlock, 0, s>>>(c, D, mb.groups, ws.lv_vnode, mb.edge_of_dnode, ws.se_cross,
                                                          mb.tri_of_dnode, mb.group_cross0, mb.parts);
    e = launch_scan<2>(SubCubeLoad{ws.s_vtx, dstride, ws.sv_value, ws.s_cube_class, err},
                       SubCubeStore{ws.s_cube_class, ws.s_edge, dstride, ws.se_cross, mb.group_cross0, c, D, A,
                                    ws.part_t, &c->n_tri, ws.part_cap_t, err},
                       &c->n_sub_dnodes, 0, ws.scan, total, err, s, ScanCount{}, sbps);
    if (e != cudaSuccess) return e;
    // insertion of all parts
    int* n_parts = mb.misc;
    int* n_staged_v = mb.misc + 1;
    int* n_staged_t = mb.misc + 2;
    k_count_parts<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, n_parts, n_staged_v, n_staged_t, ws.part_cap_v, ws.part_cap_t);
    e = launch_scan(KeepVertexLoad{ws.part_v},
                    KeepVertexStore{ws.part_v, ws.mesh_v, mb.kept_prefix, ws.cap.mesh_vertices, err}, n_staged_v, 0,
                    ws.scan, total, err, s, ScanCount{&c->n_mesh_vertices, ws.cap.mesh_vertices}, sbps);
    if (e != cudaSuccess) return e;
    e = launch_scan<1>(KeepTriLoad{ws.part_t, mb.parts, n_parts},
                    KeepTriStore{ws.part_t, mb.parts, n_parts, mb.kept_prefix, n_staged_v, &c->n_mesh_vertices,
                                 ws.mesh_t, ws.cap.mesh_tris, err},
                    n_staged_t, 0, ws.scan, total, err, s, ScanCount{&c->n_mesh_triangles, ws.cap.mesh_tris}, sbps);
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

}  // namespace psr

namespace psr {
cudaError_t mesh_geometry(Workspace& ws) {
    return mesh_geometry_impl(ws, ws.mb, (unsigned*)&ws.cnt->scan_total_aux);
}

cudaError_t mesh_build(Workspace& ws) {
    cudaError_t e = mesh_build_impl(ws, ws.mb);
    if (e != cudaSuccess) return e;
    return mesh_build_sub(ws, ws.mb);
}
}  // namespace psr
