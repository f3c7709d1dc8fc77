// Stage (b): B-spline vector-field splat at the finest depth and per-node divergence.
//
// Vector field (mesh/ComputeVectorField.cu:61-100): for every D-level node o
//     V[o] = sum_{27 neighbours nb} sum_{points p in nb} B(p - c_o) n_p,
// B the separable normalised quadratic B-spline of width 2^-D, evaluated in the node's
// local coordinate (the reference expands shifted polynomials in float, which loses
// ~1e-4 relative accuracy at depth 7; the value is the same function).
// Divergence (mesh/ComputeNodesDivergence.cu:25-136): for every node o
//     div[o] = sum_{27 neighbours nb} sum_{D-level l under nb} V[l] . dff(o, l)
// with float terms (table entries rounded to float, as the reference's kernel does)
// accumulated as float pairs (TwoSum, ~44 bits; GB300's FP64 rate is far below FP32), in
// a fixed order.  The
// reference's coarse-depth host loop (one node at a time, :159-207) is replaced by one
// chunked reduction over all coarse nodes.
#include "workspace.h"
#include "tables.cuh"

PSR_DEFINE_CONST_TABLES(upload_tables_field)

namespace psr {

__device__ __forceinline__ float bspline32(float t) {
    const float kF43 = 1.33333337306976318359375f;
    const float kF23 = 0.666666686534881591796875f;
    float a = fabsf(t);
    if (a < 0.5f) return __fmul_rn(__fsub_rn(0.75f, __fmul_rn(t, t)), kF43);
    if (a < 1.5f) { float u = __fsub_rn(1.5f, a); return __fmul_rn(__fmul_rn(u, u), kF23); }
    return 0.0f;
}

// 8 lanes per D-level node (4 nodes per warp): the 27 neighbours' sample ranges are
// flattened over the group's lanes (a group scan gives the range offsets), every lane
// accumulates its samples' weighted normals and a butterfly over the group combines the
// lanes (fixed order).
constexpr int kVfLanes = 8;
constexpr int kVfGroups = kBlock / kVfLanes;
__global__ void __launch_bounds__(kBlock) k_vector_field(const Counters* c, int depth, const float* px, const float* py,
                                                         const float* pz, const float* nx, const float* ny,
                                                         const float* nz, const int* pidx, const int* pnum,
                                                         const float* cx, const float* cy, const float* cz,
                                                         const int* neigh, size_t stride, float* vx, float* vy,
                                                         float* vz) {
    PSR_CLOUD(c, px, py, pz, nx, ny, nz, pidx, pnum, cx, cy, cz, neigh, vx, vy, vz);
    __shared__ int s_off[kVfGroups][28];
    __shared__ int s_base[kVfGroups][27];
    const int md = c->level_count[depth];
    const int b = c->level_base[depth];
    const float s = (float)(1 << depth);
    const int lane = threadIdx.x & (kVfLanes - 1);
    const int gib = threadIdx.x / kVfLanes;
    const unsigned gmask = 0xffu << (threadIdx.x & 24);   // the group's lanes in its warp
    const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kVfLanes;
    const int ngroups = (gridDim.x * blockDim.x) / kVfLanes;
    for (int o = group; o < md; o += ngroups) {
        const int i = b + o;
        const float ox = cx[i], oy = cy[i], oz = cz[i];
        int running = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int k = lane + kVfLanes * r;
            int cnt = 0, base = 0;
            if (k < 27) {
                const int nb = neigh[(size_t)k * stride + i];
                if (nb >= 0) { base = pidx[nb]; cnt = pnum[nb]; }
            }
            int incl = cnt;
#pragma unroll
            for (int q = 1; q < kVfLanes; q <<= 1) {
                const int y = __shfl_up_sync(gmask, incl, q, kVfLanes);
                if (lane >= q) incl += y;
            }
            if (k < 27) {
                s_off[gib][k] = running + incl - cnt;
                s_base[gib][k] = base;
            }
            running += __shfl_sync(gmask, incl, kVfLanes - 1, kVfLanes);
        }
        if (lane == 0) s_off[gib][27] = running;
        __syncwarp(gmask);
        float ax = 0.f, ay = 0.f, az = 0.f;
        int k = 0;
        for (int t = lane; t < running; t += kVfLanes) {
            while (s_off[gib][k + 1] <= t) ++k;
            const int p = s_base[gib][k] + (t - s_off[gib][k]);
            const float w = bspline32((px[p] - ox) * s) * bspline32((py[p] - oy) * s) * bspline32((pz[p] - oz) * s);
            ax = fmaf(w, nx[p], ax);
            ay = fmaf(w, ny[p], ay);
            az = fmaf(w, nz[p], az);
        }
#pragma unroll
        for (int q = kVfLanes / 2; q > 0; q >>= 1) {
            ax += __shfl_xor_sync(gmask, ax, q);
            ay += __shfl_xor_sync(gmask, ay, q);
            az += __shfl_xor_sync(gmask, az, q);
        }
        if (lane == 0) {
            vx[o] = ax;
            vy[o] = ay;
            vz[o] = az;
        }
        __syncwarp(gmask);
    }
}

__device__ __forceinline__ void decode3(int e, int depth, int& ix, int& iy, int& iz) {
    const int o1 = 1 << (depth + 1);
    ix = e & (o1 - 1);
    iy = (e >> (depth + 1)) & (o1 - 1);
    iz = e >> (2 * (depth + 1));
}

// contribution of D-level leaves [l0, l1) to node o's divergence
__device__ __forceinline__ FF div_terms(int l0, int l1, int step, int ox, int oy, int oz, int depth, int res,
                                        int bD, const int* enc, const float* vx, const float* vy, const float* vz,
                                        const float* dff) {
    FF acc = ff_zero();
    for (int l = l0; l < l1; l += step) {
        int lx, ly, lz;
        decode3(enc[bD + l], depth, lx, ly, lz);
        const float ux = dff[(size_t)ox + (size_t)res * lx];
        const float uy = dff[(size_t)oy + (size_t)res * ly];
        const float uz = dff[(size_t)oz + (size_t)res * lz];
        float t = __fmul_rn(vx[l], ux);
        t = fmaf(vy[l], uy, t);
        t = fmaf(vz[l], uz, t);
        acc = ff_add_float(acc, t);
    }
    return acc;
}

// Depth-D nodes: every neighbour holds exactly one depth-D leaf (itself), so a node's
// divergence has at most 27 terms; one thread per node sums them in slot order.
__global__ void __launch_bounds__(kBlock) k_div_leaf(const Counters* c, int depth, int res, const int* enc,
                                                     const int* neigh, size_t stride, const float* vx,
                                                     const float* vy, const float* vz, const float* dff,
                                                     float* divg) {
    PSR_CLOUD(c, enc, neigh, vx, vy, vz, dff, divg);
    const int bD = c->level_base[depth];
    const int MD = c->level_count[depth];
    PSR_GRID_STRIDE(o, MD) {
        const int i = bD + o;
        int ox, oy, oz;
        decode3(enc[i], depth, ox, oy, oz);
        FF acc = ff_zero();
#pragma unroll 9
        for (int k = 0; k < 27; ++k) {
            const int nb = neigh[(size_t)k * stride + i];
            if (nb < 0) continue;
            int lx, ly, lz;
            decode3(enc[nb], depth, lx, ly, lz);
            const int l = nb - bD;
            const float ux = dff[(size_t)ox + (size_t)res * lx];
            const float uy = dff[(size_t)oy + (size_t)res * ly];
            const float uz = dff[(size_t)oz + (size_t)res * lz];
            float t = __fmul_rn(vx[l], ux);
            t = fmaf(vy[l], uy, t);
            t = fmaf(vz[l], uz, t);
            acc = ff_add_float(acc, t);
        }
        divg[i] = ff_to_float(acc);
    }
}

// One warp per node for depths dsplit .. D-1.  The (neighbour, leaf) pairs of the node are
// flattened over the lanes: lane k < 27 holds neighbour k's leaf range, a warp scan gives
// the range offsets, and term t belongs to the last neighbour whose offset is <= t.  A
// depth-D node has at most 27 terms (one leaf per neighbour): one pass, 27 lanes busy.
__global__ void __launch_bounds__(kBlock) k_div_fine(const Counters* c, int depth, int dsplit, int res,
                                                     const int* enc, const int* didx, const int* dnum,
                                                     const int* neigh, size_t stride, const float* vx,
                                                     const float* vy, const float* vz, const float* dff,
                                                     float* divg) {
    PSR_CLOUD(c, enc, didx, dnum, neigh, vx, vy, vz, dff, divg);
    __shared__ int s_off[kBlock / 32][33];
    __shared__ int s_base[kBlock / 32][32];
    const int b0 = c->level_base[dsplit];
    const int bD = c->level_base[depth];
    const int M = bD;   // depth-D nodes: k_div_leaf
    const int lane = lane_id();
    const int wib = threadIdx.x >> 5;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = b0 + warp; i < M; i += nwarps) {
        int ox, oy, oz;
        decode3(enc[i], depth, ox, oy, oz);
        int cnt = 0, base = 0;
        if (lane < 27) {
            const int nb = neigh[(size_t)lane * stride + i];
            if (nb >= 0) { cnt = dnum[nb]; base = didx[nb]; }
        }
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        s_off[wib][lane] = incl - cnt;   // exclusive offset of neighbour `lane`
        s_base[wib][lane] = base;
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        __syncwarp();
        FF acc = ff_zero();
        int k = 0;
        for (int t = lane; t < total; t += 32) {
            while (k < 26 && s_off[wib][k + 1] <= t) ++k;   // terms are visited in increasing order
            const int l = s_base[wib][k] + (t - s_off[wib][k]);
            int lx, ly, lz;
            decode3(enc[bD + l], depth, lx, ly, lz);
            const float ux = dff[(size_t)ox + (size_t)res * lx];
            const float uy = dff[(size_t)oy + (size_t)res * ly];
            const float uz = dff[(size_t)oz + (size_t)res * lz];
            float tt = __fmul_rn(vx[l], ux);
            tt = fmaf(vy[l], uy, tt);
            tt = fmaf(vz[l], uz, tt);
            acc = ff_add_float(acc, tt);
        }
        acc = ff_warp_sum(acc);
        if (lane == 0) divg[i] = ff_to_float(acc);
        __syncwarp();
    }
}

constexpr int kDivChunk = 512;

// chunk count of every coarse node (depth < dsplit)
struct DivChunkLoad {
    const int* neigh;
    size_t stride;
    const int* dnum;
    __device__ unsigned operator()(int i) const {
        unsigned n = 0;
        for (int k = 0; k < 27; ++k) {
            int nb = neigh[(size_t)k * stride + i];
            if (nb >= 0) n += (unsigned)((dnum[nb] + kDivChunk - 1) / kDivChunk);
        }
        return n;
    }
    __device__ void rebase() { PSR_CLOUD(neigh, dnum); }   // to cloud blockIdx.y
};

__global__ void k_div_chunk_count(Counters* c, int dsplit, const unsigned* total, int cap, int* n_items) {
    PSR_CLOUD(c, total, n_items);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int n = (int)*total;
        if (n > cap) { atomicOr(&c->error, kErrCapacity); n = 0; }
        *n_items = n;
    }
}

// one warp per chunk: partial sum of up to kDivChunk leaves of one neighbour of one node
__global__ void __launch_bounds__(kBlock) k_div_chunks(const Counters* c, int depth, int dsplit, int res,
                                                       const int* n_items_ptr, const unsigned* item_start,
                                                       const int* enc, const int* didx, const int* dnum,
                                                       const int* neigh, size_t stride, const float* vx,
                                                       const float* vy, const float* vz, const float* dff,
                                                       FF* partial) {
    PSR_CLOUD(c, n_items_ptr, item_start, enc, didx, dnum, neigh, vx, vy, vz, dff, partial);
    const int n_nodes = c->level_base[dsplit];
    const int n_items = *n_items_ptr;
    const int bD = c->level_base[depth];
    const int lane = lane_id();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int it = warp; it < n_items; it += nwarps) {
        // node owning this item: last node with item_start <= it
        int lo = 0, hi = n_nodes - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if ((int)item_start[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo;
        int rem = it - (int)item_start[i];
        int nb = -1, ch = 0;
        for (int k = 0; k < 27; ++k) {
            int q = neigh[(size_t)k * stride + i];
            if (q < 0) continue;
            int nc = (dnum[q] + kDivChunk - 1) / kDivChunk;
            if (rem < nc) { nb = q; ch = rem; break; }
            rem -= nc;
        }
        FF acc = ff_zero();
        if (nb >= 0) {
            int ox, oy, oz;
            decode3(enc[i], depth, ox, oy, oz);
            const int l0 = didx[nb] + ch * kDivChunk;
            const int l1 = min(didx[nb] + dnum[nb], l0 + kDivChunk);
            acc = div_terms(l0 + lane, l1, 32, ox, oy, oz, depth, res, bD, enc, vx, vy, vz, dff);
        }
        acc = ff_warp_sum(acc);
        if (lane == 0) partial[it] = acc;
    }
}

__global__ void __launch_bounds__(kBlock) k_div_coarse_reduce(const Counters* c, int dsplit, const unsigned* item_start,
                                                              const int* n_items_ptr, const FF* partial,
                                                              float* divg) {
    PSR_CLOUD(c, item_start, n_items_ptr, partial, divg);
    const int n_nodes = c->level_base[dsplit];
    const int n_items = *n_items_ptr;
    PSR_GRID_STRIDE(i, n_nodes) {
        int a = (int)item_start[i];
        int b = (i + 1 < n_nodes) ? (int)item_start[i + 1] : n_items;
        FF s = ff_zero();
        for (int t = a; t < b; ++t) s = ff_add(s, partial[t]);
        divg[i] = ff_to_float(s);
    }
}

cudaError_t field_build(Workspace& ws) {
    cudaStream_t s = ws.stream;
    const int D = ws.depth;
    Counters* c = ws.cnt;
    const size_t stride = (size_t)ws.cap.nodes;
    float* vx = ws.vfield;
    float* vy = ws.vfield + ws.cap.dnodes;
    float* vz = ws.vfield + 2 * (size_t)ws.cap.dnodes;
    k_vector_field<<<PSR_GRID(ws, ws.num_sms * 8), kBlock, 0, s>>>(c, D, ws.px, ws.py, ws.pz, ws.nx, ws.ny, ws.nz,
                                                                    ws.pidx, ws.pnum, ws.ctr_x, ws.ctr_y, ws.ctr_z,
                                                                    ws.neigh, stride, vx, vy, vz);
    const int dsplit = D >= 2 ? D - 2 : 0;
    cudaError_t e = cudaSuccess;
    if (dsplit > 0) {
        // The coarse depths' chunked divergence runs on the second stream beside k_div_fine
        // (both only read the vector field); it issues the only scan meanwhile.
        // item_start / n_items / partial live in the (otherwise idle) CG scratch.
        cudaStream_t a2 = ws.aux;
        e = cudaEventRecord(ws.ev_fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(a2, ws.ev_fork, 0);
        if (e != cudaSuccess) return e;
        unsigned* item_start = (unsigned*)ws.cg_r;
        int* n_items = (int*)&c->n_groups;
        unsigned* total = (unsigned*)&c->scan_total;
        e = launch_scan(DivChunkLoad{ws.neigh, stride, ws.dnum}, StoreExclusive{item_start}, &c->level_base[dsplit],
                        0, ws.scan, total, &c->error, a2, ScanCount{}, 1);
        if (e != cudaSuccess) return e;
        const int item_cap = ws.cap.nodes;   // partial buffer holds cap.nodes float pairs
        k_div_chunk_count<<<PSR_GRID(ws, 1), 1, 0, a2>>>(c, dsplit, total, item_cap, n_items);
        FF* partial = reinterpret_cast<FF*>(ws.cg_partial);
        k_div_chunks<<<PSR_GRID(ws, ws.num_sms * 8), kBlock, 0, a2>>>(c, D, dsplit, ws.res, n_items, item_start, ws.enc, ws.didx,
                                                        ws.dnum, ws.neigh, stride, vx, vy, vz, ws.dff, partial);
        k_div_coarse_reduce<<<PSR_GRID(ws, grid_for(ws, 1 << 16)), kBlock, 0, a2>>>(c, dsplit, item_start, n_items, partial,
                                                                     ws.divg);
        e = cudaEventRecord(ws.ev_join, a2);
        if (e != cudaSuccess) return e;
    }
    k_div_fine<<<PSR_GRID(ws, ws.num_sms * 8), kBlock, 0, s>>>(c, D, dsplit, ws.res, ws.enc, ws.didx, ws.dnum, ws.neigh, stride, vx,
                                                 vy, vz, ws.dff, ws.divg);
    k_div_leaf<<<PSR_GRID(ws, ws.num_sms * 8), kBlock, 0, s>>>(c, D, ws.res, ws.enc, ws.neigh, stride, vx, vy, vz, ws.dff, ws.divg);
    if (dsplit > 0) {
        e = cudaStreamWaitEvent(s, ws.ev_join, 0);
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

}  // namespace psr
