// Per-vertex colour and normal transfer onto the output mesh.
//
// Colour (mesh/DrawMesh.cu:179-214): the 4 nearest samples of each mesh vertex (the
// reference searches all samples; here a uniform grid over the Morton-sorted samples
// finds the same exact 4 nearest, ties resolved towards the lower sample index), blended
// with weights proportional to the squared distance (a reference quirk kept as is).
// Normals (mesh/DrawMesh.cu:102-177): unweighted average of the unit normals of the
// incident triangles, normalised.
#include "workspace.h"
#include "tables.cuh"

PSR_DEFINE_CONST_TABLES(upload_tables_transfer)

namespace psr {

constexpr int kGridLevel = 6;   // 64^3 cells

__device__ __forceinline__ unsigned morton3(int x, int y, int z, int g) {
    unsigned m = 0;
    for (int l = 0; l < g; ++l)
        m |= (((unsigned)(x >> l) & 1u) << (3 * l + 2)) | (((unsigned)(y >> l) & 1u) << (3 * l + 1)) |
             (((unsigned)(z >> l) & 1u) << (3 * l));
    return m;
}

__device__ __forceinline__ unsigned point_cell(int i, int depth, int g, int bD, const int* key,
                                               const int* point2node) {
    return (unsigned)key[bD + point2node[i]] >> (3 * (depth - g));
}

// cell_start[m] = first sorted sample whose cell code is >= m, for m in [0, 8^g]
__global__ void __launch_bounds__(kBlock) k_cell_starts(const Counters* c, int depth, int g, const int* key,
                                                        const int* point2node, int* cell_start) {
    const int n = c->n_points;
    const int bD = c->level_base[depth];
    const int ncell = 1 << (3 * g);
    PSR_GRID_STRIDE(i, n + 1) {
        const int cur = (i < n) ? (int)point_cell(i, depth, g, bD, key, point2node) : ncell;
        const int prev = (i > 0) ? (int)point_cell(i - 1, depth, g, bD, key, point2node) : -1;
        for (int m = prev + 1; m <= cur && m <= ncell; ++m) cell_start[m] = i;
    }
}

__global__ void __launch_bounds__(kBlock) k_colour(const Counters* c, int g, const float* mv, const float* px,
                                                   const float* py, const float* pz, const float* cr, const float* cg,
                                                   const float* cb, const int* cell_start, float* out) {
    const int V = c->n_mesh_vertices;
    const int G = 1 << g;
    PSR_GRID_STRIDE(v, V) {
        const float qx = mv[3 * (size_t)v], qy = mv[3 * (size_t)v + 1], qz = mv[3 * (size_t)v + 2];
        float bd[4] = {1e6f, 1e6f, 1e6f, 1e6f};
        int bi[4] = {0, 0, 0, 0};
        const int cx = min(max((int)floorf(qx * G), 0), G - 1);
        const int cy = min(max((int)floorf(qy * G), 0), G - 1);
        const int cz = min(max((int)floorf(qz * G), 0), G - 1);
        for (int r = 0; r <= G; ++r) {
            for (int a = cx - r; a <= cx + r; ++a) {
                if (a < 0 || a >= G) continue;
                for (int b = cy - r; b <= cy + r; ++b) {
                    if (b < 0 || b >= G) continue;
                    for (int z = cz - r; z <= cz + r; ++z) {
                        if (z < 0 || z >= G) continue;
                        if (max(abs(a - cx), max(abs(b - cy), abs(z - cz))) != r) continue;
                        const unsigned m = morton3(a, b, z, g);
                        for (int i = cell_start[m]; i < cell_start[m + 1]; ++i) {
                            const float dx = __fsub_rn(qx, px[i]), dy = __fsub_rn(qy, py[i]), dz = __fsub_rn(qz, pz[i]);
                            const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                            if (d2 < bd[3] || (d2 == bd[3] && i < bi[3])) {
                                int k = 3;
                                while (k > 0 && (d2 < bd[k - 1] || (d2 == bd[k - 1] && i < bi[k - 1]))) {
                                    bd[k] = bd[k - 1];
                                    bi[k] = bi[k - 1];
                                    --k;
                                }
                                bd[k] = d2;
                                bi[k] = i;
                            }
                        }
                    }
                }
            }
            const float lim = (float)r / (float)G;
            if (bd[3] < 1e6f && bd[3] < lim * lim) break;
        }
        const float sum = bd[0] + bd[1] + bd[2] + bd[3];
        const float inv = (sum > 0.0f) ? 1.0f / sum : 0.0f;
        float o[3] = {0.f, 0.f, 0.f};
        for (int k = 0; k < 4; ++k) {
            const float w = bd[k] * inv;   // weight grows with the squared distance
            o[0] += cr[bi[k]] * w;
            o[1] += cg[bi[k]] * w;
            o[2] += cb[bi[k]] * w;
        }
        out[3 * (size_t)v] = o[0];
        out[3 * (size_t)v + 1] = o[1];
        out[3 * (size_t)v + 2] = o[2];
    }
}

__global__ void __launch_bounds__(kBlock) k_normals_zero(const Counters* c, double* acc, int* cnt) {
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(v, V) {
        acc[3 * (size_t)v] = acc[3 * (size_t)v + 1] = acc[3 * (size_t)v + 2] = 0.0;
        cnt[v] = 0;
    }
}

__global__ void __launch_bounds__(kBlock) k_triangle_normals(const Counters* c, const float* mv, const int* mt,
                                                             double* acc, int* cnt) {
    const int T = c->n_mesh_triangles;
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(t, T) {
        const int i0 = mt[3 * (size_t)t], i1 = mt[3 * (size_t)t + 1], i2 = mt[3 * (size_t)t + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= V || i1 >= V || i2 >= V) continue;
        const float ox = mv[3 * (size_t)i0], oy = mv[3 * (size_t)i0 + 1], oz = mv[3 * (size_t)i0 + 2];
        const float ax = mv[3 * (size_t)i1] - ox, ay = mv[3 * (size_t)i1 + 1] - oy, az = mv[3 * (size_t)i1 + 2] - oz;
        const float bx = mv[3 * (size_t)i2] - ox, by = mv[3 * (size_t)i2 + 1] - oy, bz = mv[3 * (size_t)i2 + 2] - oz;
        float nx = ay * bz - az * by, ny = az * bx - ax * bz, nz = ax * by - ay * bx;
        const float l = sqrtf(nx * nx + ny * ny + nz * nz);
        if (l == 0.0f) { nx = ny = nz = 0.0f; }
        else { nx /= l; ny /= l; nz /= l; }
        const int ids[3] = {i0, i1, i2};
        for (int k = 0; k < 3; ++k) {
            atomicAdd(&acc[3 * (size_t)ids[k]], (double)nx);
            atomicAdd(&acc[3 * (size_t)ids[k] + 1], (double)ny);
            atomicAdd(&acc[3 * (size_t)ids[k] + 2], (double)nz);
            atomicAdd(&cnt[ids[k]], 1);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_vertex_normals(const Counters* c, const double* acc, const int* cnt,
                                                           float* out) {
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(v, V) {
        const int n = cnt[v];
        float x = 0.f, y = 0.f, z = 0.f;
        if (n > 0) {
            x = (float)acc[3 * (size_t)v] / n;
            y = (float)acc[3 * (size_t)v + 1] / n;
            z = (float)acc[3 * (size_t)v + 2] / n;
            const float l = sqrtf(x * x + y * y + z * z);
            if (l > 0.0f) { x /= l; y /= l; z /= l; }
            else { x = y = z = 0.0f; }
        }
        out[3 * (size_t)v] = x;
        out[3 * (size_t)v + 1] = y;
        out[3 * (size_t)v + 2] = z;
    }
}

cudaError_t transfer_build(Workspace& ws, int with_colour, int with_normals) {
    cudaStream_t s = ws.stream;
    const int grid = ws.num_sms * 8;
    const int D = ws.depth;
    if (with_colour) {
        const int g = D < kGridLevel ? D : kGridLevel;
        int* cell_start = ws.cell_start;   // (1 << 3g) + 1 entries
        k_cell_starts<<<grid, kBlock, 0, s>>>(ws.cnt, D, g, ws.key, ws.point2node, cell_start);
        k_colour<<<grid, kBlock, 0, s>>>(ws.cnt, g, ws.mesh_v, ws.px, ws.py, ws.pz, ws.cr, ws.cg, ws.cb, cell_start,
                                         ws.mesh_c);
    }
    if (with_normals) {
        double* acc = ws.nacc;
        k_normals_zero<<<grid, kBlock, 0, s>>>(ws.cnt, acc, ws.vcount);
        k_triangle_normals<<<grid, kBlock, 0, s>>>(ws.cnt, ws.mesh_v, ws.mesh_t, acc, ws.vcount);
        k_vertex_normals<<<grid, kBlock, 0, s>>>(ws.cnt, acc, ws.vcount, ws.mesh_n);
    }
    return cudaGetLastError();
}

}  // namespace psr
