// Vertex welding of the output mesh (optional; off by default).  The reference appends the
// vertices of every subdivided region to the mesh on their own, so a vertex on the boundary
// between regions is emitted once per region (mesh/ComputeTriangleIndices.cu:1247-1282,
// insertTriangle); parity with it keeps those copies.  With welding on, vertices whose three
// coordinates are bit-identical become one: the copy with the smallest index represents the
// class, representatives keep their order, and every triangle corner is renumbered.  The
// result equals a stable first-occurrence unique over the coordinate bit patterns and does
// not depend on thread timing.  It runs before the colour / normal transfer, so those are
// computed on the welded mesh.
//
// Device steps: an open-addressing hash table over the coordinate bits (each vertex finds or
// claims the slot of its class), an atomicMin per slot that leaves the class's smallest
// index in it, one scan over "is its own representative" giving the new numbering and the
// compacted vertices, then a pass that renumbers the triangles and copies the vertices back.
#include "workspace.h"

namespace psr {

__device__ __forceinline__ unsigned weld_hash(unsigned x, unsigned y, unsigned z) {
    unsigned h = x * 0x9e3779b1u;
    h ^= (y + 0x7f4a7c15u) * 0x85ebca77u;
    h = (h << 13) | (h >> 19);
    h ^= (z + 0x165667b1u) * 0xc2b2ae3du;
    h ^= h >> 16;
    h *= 0x7feb352du;
    h ^= h >> 15;
    return h;
}

__device__ __forceinline__ bool weld_same(const unsigned* vb, int a, int b) {
    return vb[3 * (size_t)a] == vb[3 * (size_t)b] && vb[3 * (size_t)a + 1] == vb[3 * (size_t)b + 1] &&
           vb[3 * (size_t)a + 2] == vb[3 * (size_t)b + 2];
}

// every vertex finds the slot of its class or claims an empty one (table starts at -1);
// at most `mask + 1` probes, the table being at least twice the vertex capacity
__global__ void __launch_bounds__(kBlock) k_weld_insert(Counters* c, const float* mv, int* table, unsigned mask,
                                                        int* slot) {
    PSR_CLOUD(c, mv, table, slot);
    const int V = c->n_mesh_vertices;
    const unsigned* vb = reinterpret_cast<const unsigned*>(mv);
    PSR_GRID_STRIDE(v, V) {
        unsigned h = weld_hash(vb[3 * (size_t)v], vb[3 * (size_t)v + 1], vb[3 * (size_t)v + 2]) & mask;
        int found = -1;
        for (unsigned probe = 0; probe <= mask; ++probe) {
            int cur = table[h];
            if (cur < 0) {
                cur = atomicCAS(&table[h], -1, v);
                if (cur < 0) { found = (int)h; break; }
            }
            if (weld_same(vb, cur, v)) { found = (int)h; break; }
            h = (h + 1) & mask;
        }
        if (found < 0) {   // a full table: only reachable past the vertex capacity
            atomicOr(&c->error, kErrCapacity);
            found = 0;
        }
        slot[v] = found;
    }
}

// the smallest index of each class into its slot (any member's index is there already)
__global__ void __launch_bounds__(kBlock) k_weld_min(const Counters* c, const int* slot, int* table) {
    PSR_CLOUD(c, slot, table);
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(v, V) atomicMin(&table[slot[v]], v);
}

struct WeldLoad {
    const int* table;
    const int* slot;
    __device__ unsigned operator()(int v) const { return table[slot[v]] == v ? 1u : 0u; }
    __device__ void rebase() { PSR_CLOUD(table, slot); }   // to cloud blockIdx.y
};

// representatives: new number and a compacted copy of the position
struct WeldStore {
    const float* mv;
    float* out_v;
    int* newid;
    __device__ void operator()(int v, unsigned pre, unsigned keep) const {
        if (!keep) return;
        newid[v] = (int)pre;
        out_v[3 * (size_t)pre] = mv[3 * (size_t)v];
        out_v[3 * (size_t)pre + 1] = mv[3 * (size_t)v + 1];
        out_v[3 * (size_t)pre + 2] = mv[3 * (size_t)v + 2];
    }
    __device__ void rebase() { PSR_CLOUD(mv, out_v, newid); }   // to cloud blockIdx.y
};

// triangle corners -> the new number of their class's representative; welded positions back
// into the mesh array; the vertex count becomes the welded one
__global__ void __launch_bounds__(kBlock) k_weld_apply(Counters* c, const int* table, const int* slot,
                                                       const int* newid, const float* wv, float* mv, int* mt) {
    PSR_CLOUD(c, table, slot, newid, wv, mv, mt);
    const int V = c->n_mesh_vertices;
    const int W = c->n_weld;
    const int T3 = 3 * c->n_mesh_triangles;
    PSR_GRID_STRIDE(i, max(T3, 3 * W)) {
        if (i < T3) {
            const int v = mt[i];
            if (v >= 0 && v < V) mt[i] = newid[table[slot[v]]];
        }
        if (i < 3 * W) mv[i] = wv[i];
    }
}

__global__ void k_weld_count(Counters* c) {
    PSR_CLOUD(c);
    if (threadIdx.x == 0 && blockIdx.x == 0) c->n_mesh_vertices = c->n_weld;
}

cudaError_t weld_build(Workspace& ws) {
    if (!ws.weld_table) return cudaSuccess;
    cudaStream_t s = ws.stream;
    Counters* c = ws.cnt;
    cudaError_t e = fill_words((unsigned*)ws.weld_table, 0xffffffffu, (long long)ws.weld_mask + 1, ws.batch, s);
    if (e != cudaSuccess) return e;
    const int g = grid_for(ws, ws.cap.mesh_vertices);
    k_weld_insert<<<PSR_GRID(ws, g), kBlock, 0, s>>>(c, ws.mesh_v, ws.weld_table, ws.weld_mask, ws.weld_slot);
    k_weld_min<<<PSR_GRID(ws, g), kBlock, 0, s>>>(c, ws.weld_slot, ws.weld_table);
    e = launch_scan(WeldLoad{ws.weld_table, ws.weld_slot}, WeldStore{ws.mesh_v, ws.weld_v, ws.weld_newid},
                    &c->n_mesh_vertices, 0, ws.scan, (unsigned*)&c->scan_total, &c->error, s,
                    ScanCount{&c->n_weld, ws.cap.mesh_vertices}, 1);
    if (e != cudaSuccess) return e;
    k_weld_apply<<<PSR_GRID(ws, grid_for(ws, 3 * ws.cap.mesh_tris)), kBlock, 0, s>>>(c, ws.weld_table, ws.weld_slot,
                                                                       ws.weld_newid, ws.weld_v, ws.mesh_v,
                                                                       ws.mesh_t);
    k_weld_count<<<PSR_GRID(ws, 1), 32, 0, s>>>(c);
    return cudaGetLastError();
}

}  // namespace psr
