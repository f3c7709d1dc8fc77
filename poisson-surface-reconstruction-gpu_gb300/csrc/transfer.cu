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

// cell_start[m] = first sorted sample whose cell code is >= m, for m in [0, 8^g]: the
// exclusive prefix sum of the samples per cell.  k_cell_count counts them (the table
// starts zeroed; the samples are Morton-sorted, so the last sample of a cell's run adds
// the run's length), then one scan turns the counts into starts in place.
__global__ void __launch_bounds__(kBlock) k_cell_count(Counters* c, int depth, int g, const int* key,
                                                       const int* point2node, int* count) {
    PSR_CLOUD(c, key, point2node, count);
    const int n = c->n_points;
    const int bD = c->level_base[depth];
    if (blockIdx.x == 0 && threadIdx.x == 0) c->n_colour_cells = (1 << (3 * g)) + 1;
    PSR_GRID_STRIDE(i, n) {
        const unsigned m = point_cell(i, depth, g, bD, key, point2node);
        if (i + 1 < n && point_cell(i + 1, depth, g, bD, key, point2node) == m) continue;
        int lo = 0, hi = i;   // first sample of the run ending at i
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (point_cell(mid, depth, g, bD, key, point2node) < m) lo = mid + 1;
            else hi = mid;
        }
        count[m] = i + 1 - lo;
    }
}

// (d, i) lexicographic order: smaller squared distance first, then lower sample index
__device__ __forceinline__ bool knn_less(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

// insert (d, i) into a sorted 4-list held in registers
__device__ __forceinline__ void knn_insert(float (&bd)[4], int (&bi)[4], float d, int i) {
    if (!knn_less(d, i, bd[3], bi[3])) return;
    if (knn_less(d, i, bd[2], bi[2])) {
        bd[3] = bd[2]; bi[3] = bi[2];
        if (knn_less(d, i, bd[1], bi[1])) {
            bd[2] = bd[1]; bi[2] = bi[1];
            if (knn_less(d, i, bd[0], bi[0])) {
                bd[1] = bd[0]; bi[1] = bi[0];
                bd[0] = d; bi[0] = i;
            } else { bd[1] = d; bi[1] = i; }
        } else { bd[2] = d; bi[2] = i; }
    } else { bd[3] = d; bi[3] = i; }
}

// the warp's 4 nearest from the lanes' sorted 4-lists (sample sets disjoint between lanes):
// four rounds of a warp-wide minimum of the lanes' heads under the (d, i) order, the lane
// holding the minimum popping its head; every lane ends with the same 4
__device__ __forceinline__ void knn_warp_merge(const float (&bd)[4], const int (&bi)[4], float (&md)[4],
                                               int (&mi)[4]) {
    float hd[4] = {bd[0], bd[1], bd[2], bd[3]};
    int hi[4] = {bi[0], bi[1], bi[2], bi[3]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        float d = hd[0];
        int i = hi[0];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, d, o);
            const int oi = __shfl_xor_sync(0xffffffffu, i, o);
            if (knn_less(od, oi, d, i)) { d = od; i = oi; }
        }
        md[r] = d;
        mi[r] = i;
        if (hd[0] == d && hi[0] == i) {   // this lane's head was taken
            hd[0] = hd[1]; hi[0] = hi[1];
            hd[1] = hd[2]; hi[1] = hi[2];
            hd[2] = hd[3]; hi[2] = hi[3];
            hd[3] = 1e6f; hi[3] = 0x7fffffff;
        }
    }
}

__device__ __forceinline__ void knn_visit(float qx, float qy, float qz, const float* px, const float* py,
                                          const float* pz, int i, float (&bd)[4], int (&bi)[4]) {
    const float dx = __fsub_rn(qx, px[i]), dy = __fsub_rn(qy, py[i]), dz = __fsub_rn(qz, pz[i]);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    knn_insert(bd, bi, d2, i);
}

// the same, keeping only samples that precede (d4, i4), the 4th nearest found so far: the
// others cannot be among the 4 nearest
__device__ __forceinline__ void knn_visit_below(float qx, float qy, float qz, const float* px, const float* py,
                                                const float* pz, int i, float d4, int i4, float (&bd)[4],
                                                int (&bi)[4]) {
    const float dx = __fsub_rn(qx, px[i]), dy = __fsub_rn(qy, py[i]), dz = __fsub_rn(qz, pz[i]);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    if (knn_less(d2, i, d4, i4)) knn_insert(bd, bi, d2, i);
}

// colour of a vertex from its 4 nearest (fewer than 4 samples: the reference's unfilled
// slots, distance 1e6 and sample 0); weights grow with the squared distance
__device__ __forceinline__ void colour_blend(const float (&md)[4], const int (&mi)[4], const float* cr,
                                             const float* cg, const float* cb, float* out) {
    const float sum = md[0] + md[1] + md[2] + md[3];
    const float inv = (sum > 0.0f) ? 1.0f / sum : 0.0f;
    float o[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 4; ++k) {
        const int idx = (mi[k] == 0x7fffffff) ? 0 : mi[k];
        const float w = md[k] * inv;
        o[0] += cr[idx] * w;
        o[1] += cg[idx] * w;
        o[2] += cb[idx] * w;
    }
    out[0] = o[0];
    out[1] = o[1];
    out[2] = o[2];
}

// bits of v (< 1024) to every third bit
__device__ __forceinline__ unsigned spread3(unsigned v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Near pass, 8 lanes per mesh vertex: the samples of the 3x3x3 block of finest-level
// cells around the vertex's cell (every sample outside it is at least one cell width
// away), spread over the group's lanes (flattened over the 27 cell ranges), each lane
// keeping a sorted 4-list, merged by warp-minimum rounds within the group.  When 4 were
// found and the 4th is closer than one width they are the exact 4 nearest and the colour
// is written; otherwise the vertex goes to the far list for the wide search (k_colour_far).
constexpr int kNearLanes = 8;
constexpr int kNearGroups = kBlock / kNearLanes;
constexpr int kNearCoarseCap = 512;   // samples the coarser pass scans per vertex at most
// The same search one or two levels coarser (g < gt, the table's level: cell m of level g
// is the range of table entries m << 3 (gt - g) .. (m + 1) << 3 (gt - g)) serves the vertices
// a finer pass left (`in`: (vertex, bound) pairs, *in_count of them), when their block holds
// at most `cap` samples; the ones it does not settle go on to `out` with the smaller bound.
__global__ void __launch_bounds__(kBlock) k_colour_near(Counters* c, int g, int gt, const float* mv, const float* px,
                                                        const float* py, const float* pz, const float* cr,
                                                        const float* cg, const float* cb, const int* cell_start,
                                                        const int* in, const int* in_count, int cap, int* far,
                                                        int* far_count, float* out) {
    PSR_CLOUD(c, mv, px, py, pz, cr, cg, cb, cell_start, in, in_count, far, far_count, out);
    __shared__ int s_off[kNearGroups][28];
    __shared__ int s_base[kNearGroups][27];
    const int V = in ? *in_count : c->n_mesh_vertices;
    const int G = 1 << g;
    const int shift = 3 * (gt - g);
    const float w = 1.0f / (float)G;
    const int lane = threadIdx.x & (kNearLanes - 1);
    const int gib = threadIdx.x / kNearLanes;
    const unsigned gmask = 0xffu << (threadIdx.x & 24);   // the group's lanes in its warp
    const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kNearLanes;
    const int ngroups = (gridDim.x * blockDim.x) / kNearLanes;
    for (int t = group; t < V; t += ngroups) {
        const int v = in ? in[2 * (size_t)t] : t;
        const float prev = in ? __int_as_float(in[2 * (size_t)t + 1]) : 1e6f;
        const float qx = mv[3 * (size_t)v], qy = mv[3 * (size_t)v + 1], qz = mv[3 * (size_t)v + 2];
        const int cx = min(max((int)floorf(qx * G), 0), G - 1);
        const int cy = min(max((int)floorf(qy * G), 0), G - 1);
        const int cz = min(max((int)floorf(qz * G), 0), G - 1);
        // cells k = lane + 8 r, offsets in k order
        int running = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int k = lane + kNearLanes * r;
            int cnt = 0, base = 0;
            if (k < 27) {
                const int a = cx + k / 9 - 1, b = cy + (k / 3) % 3 - 1, z = cz + k % 3 - 1;
                if (a >= 0 && a < G && b >= 0 && b < G && z >= 0 && z < G) {
                    const unsigned m = (spread3((unsigned)a) << 2) | (spread3((unsigned)b) << 1) | spread3((unsigned)z);
                    base = cell_start[(size_t)m << shift];
                    cnt = cell_start[(size_t)(m + 1) << shift] - base;
                }
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < kNearLanes; o <<= 1) {
                const int y = __shfl_up_sync(gmask, incl, o, kNearLanes);
                if (lane >= o) incl += y;
            }
            if (k < 27) {
                s_off[gib][k] = running + incl - cnt;
                s_base[gib][k] = base;
            }
            running += __shfl_sync(gmask, incl, kNearLanes - 1, kNearLanes);
        }
        if (lane == 0) s_off[gib][27] = running;
        __syncwarp(gmask);
        if (cap > 0 && running > cap) {   // a crowded block: left to the wide search as it is
            if (lane == 0) {
                const int slot = atomicAdd(far_count, 1);
                far[2 * (size_t)slot] = v;
                far[2 * (size_t)slot + 1] = __float_as_int(prev);
            }
            continue;
        }
        float bd[4] = {1e6f, 1e6f, 1e6f, 1e6f};
        int bi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
        int k = 0;
        for (int t = lane; t < running; t += kNearLanes) {
            while (s_off[gib][k + 1] <= t) ++k;   // flattened index -> cell (increasing)
            knn_visit(qx, qy, qz, px, py, pz, s_base[gib][k] + (t - s_off[gib][k]), bd, bi);
        }
        __syncwarp(gmask);
        // the group's 4 nearest: four rounds of the minimum head, its lane popping it
        float md[4];
        int mi[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float d = bd[0];
            int i = bi[0];
#pragma unroll
            for (int o = kNearLanes / 2; o > 0; o >>= 1) {
                const float od = __shfl_xor_sync(gmask, d, o);
                const int oi = __shfl_xor_sync(gmask, i, o);
                if (knn_less(od, oi, d, i)) { d = od; i = oi; }
            }
            md[r] = d;
            mi[r] = i;
            if (bd[0] == d && bi[0] == i) {
                bd[0] = bd[1]; bi[0] = bi[1];
                bd[1] = bd[2]; bi[1] = bi[2];
                bd[2] = bd[3]; bi[2] = bi[3];
                bd[3] = 1e6f; bi[3] = 0x7fffffff;
            }
        }
        if (lane == 0) {
            if (mi[3] != 0x7fffffff && md[3] < w * w) colour_blend(md, mi, cr, cg, cb, &out[3 * (size_t)v]);
            else {   // (vertex, the 4th squared distance found so far: an upper bound, 1e6 if none)
                const int slot = atomicAdd(far_count, 1);
                far[2 * (size_t)slot] = v;
                far[2 * (size_t)slot + 1] = __float_as_int(mi[3] != 0x7fffffff ? fminf(md[3], prev) : prev);
            }
        }
    }
}

// bits 0, 3, 6, ... of v gathered into the low bits (the inverse of spread3)
__device__ __forceinline__ unsigned compact3(unsigned v) {
    v &= 0x09249249u;
    v = (v | (v >> 2)) & 0x030c30c3u;
    v = (v | (v >> 4)) & 0x0300f00fu;
    v = (v | (v >> 8)) & 0x030000ffu;
    v = (v | (v >> 16)) & 0x3ffu;
    return v;
}

// the sorted 4-list of the union of two sorted 4-lists over disjoint sample sets: four
// rounds, each taking the smaller head and shifting that list (registers only)
__device__ __forceinline__ void knn_merge4(float (&md)[4], int (&mi)[4], const float (&ld)[4], const int (&li)[4]) {
    float ad[4] = {md[0], md[1], md[2], md[3]}, bd[4] = {ld[0], ld[1], ld[2], ld[3]};
    int ai[4] = {mi[0], mi[1], mi[2], mi[3]}, bi[4] = {li[0], li[1], li[2], li[3]};
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const bool take_b = knn_less(bd[0], bi[0], ad[0], ai[0]);
        md[r] = take_b ? bd[0] : ad[0];
        mi[r] = take_b ? bi[0] : ai[0];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            ad[q] = take_b ? ad[q] : ad[q + 1];
            ai[q] = take_b ? ai[q] : ai[q + 1];
            bd[q] = take_b ? bd[q + 1] : bd[q];
            bi[q] = take_b ? bi[q + 1] : bi[q];
        }
        ad[3] = take_b ? ad[3] : 1e6f;
        ai[3] = take_b ? ai[3] : 0x7fffffff;
        bd[3] = take_b ? 1e6f : bd[3];
        bi[3] = take_b ? 0x7fffffff : bi[3];
    }
}

// Far pass, one warp per vertex of the far list: a branch-and-bound descent of the grid's
// cell hierarchy.  The samples are Morton-sorted, so the samples of a cell at any level
// g <= gmax form one contiguous range, read from the level-gmax table at codes shifted by
// 3 (gmax - g); the children of cell m are cells 8m .. 8m + 7 one level finer.  Expanding
// a node, the lanes 0..7 take its children: a child that is a finest-level cell or holds
// at most kFarLeaf samples is scanned at once, together with its leaf siblings (their
// samples flattened over the lanes, each lane keeping a sorted 4-list of the samples ahead
// of the warp's 4th nearest so far, merged by warp-minimum rounds into the warp's 4 nearest
// only when some lane holds one); the other non-empty children are pushed onto a per-warp
// stack, nearest box first.  A node whose box is farther than the bound (the 4th nearest
// so far, or the near passes' 4th distance when smaller, with 1e-4 relative slack) is
// skipped: a sample's float distance is at least its cell box's (the sample lies in the
// closed box and rounding is monotone).  So the result is the exact 4 nearest under the
// (distance, index) order, whatever the distance.  The stack holds at most 7 siblings per
// level plus 8 children: 7 gmax + 9 entries.
constexpr int kFarWarps = kBlock / 32;
constexpr int kFarLeaf = 128;
constexpr int kFarStack = 64;
static_assert(7 * kColourGridLevel + 9 <= kFarStack, "descent stack");

__global__ void __launch_bounds__(kBlock) k_colour_far(const Counters* c, int gmax, const float* mv,
                                                       const float* px, const float* py, const float* pz,
                                                       const float* cr, const float* cg, const float* cb,
                                                       const int* cell_start, const int* far, const int* far_count,
                                                       float* out) {
    PSR_CLOUD(c, mv, px, py, pz, cr, cg, cb, cell_start, far, far_count, out);
    __shared__ int s_node[kFarWarps][kFarStack];    // (level << 24) | cell code
    __shared__ float s_dist[kFarWarps][kFarStack];  // squared distance to the cell's box
    __shared__ int s_loff[kFarWarps][9];            // leaf children scanned together: offsets
    __shared__ int s_lbase[kFarWarps][8];           //   in the flattened range, first samples
    const int nfar = *far_count;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    int* stk = s_node[wib];
    float* sdist = s_dist[wib];
    int* loff = s_loff[wib];
    int* lbase = s_lbase[wib];
    for (int t = gw; t < nfar; t += nw) {
        const int v = far[2 * (size_t)t];
        const float bound = __int_as_float(far[2 * (size_t)t + 1]);
        const float qx = mv[3 * (size_t)v], qy = mv[3 * (size_t)v + 1], qz = mv[3 * (size_t)v + 2];
        // the warp's 4 nearest so far, the same in every lane (1e6: a slot not yet filled;
        // every squared distance in the unit cube is below 3)
        float md[4] = {1e6f, 1e6f, 1e6f, 1e6f};
        int mi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
        if (lane == 0) {
            stk[0] = 0;   // the root: level 0, code 0
            sdist[0] = 0.0f;
        }
        __syncwarp();
        int top = 1;
        while (top > 0) {
            --top;
            const int node = stk[top];
            const float nd = sdist[top];
            __syncwarp();   // every lane has read the entry before the slot is reused
            const float lim = fminf(bound, md[3]) * 1.0001f;
            if (nd > lim) continue;
            const int g = node >> 24;
            const unsigned m = (unsigned)node & 0xffffffu;
            if (g == 0) {   // a small cloud: the root itself is a leaf
                const int s1 = cell_start[(size_t)1 << (3 * gmax)];
                if (s1 <= kFarLeaf) {
                    float bd[4] = {1e6f, 1e6f, 1e6f, 1e6f};
                    int bi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
                    for (int j = lane; j < s1; j += 32) knn_visit(qx, qy, qz, px, py, pz, j, bd, bi);
                    float ld[4];
                    int li[4];
                    knn_warp_merge(bd, bi, ld, li);
                    knn_merge4(md, mi, ld, li);
                    continue;
                }
            }
            // lanes 0..7: child (g + 1, 8 m + lane), its samples and box distance
            const int gc = g + 1;
            const unsigned child = (m << 3) | (unsigned)(lane & 7);
            const int cshift = 3 * (gmax - gc);
            bool keep = false, leaf = false;
            float d2 = 0.0f;
            int n0 = 0, cnt = 0;
            if (lane < 8) {
                n0 = cell_start[(size_t)child << cshift];
                cnt = cell_start[(size_t)(child + 1) << cshift] - n0;
                const float w = 1.0f / (float)(1 << gc);
                const int a = (int)compact3(child >> 2), b = (int)compact3(child >> 1), z = (int)compact3(child);
                const float gx = fmaxf(fmaxf(__fsub_rn(a * w, qx), __fsub_rn(qx, (a + 1) * w)), 0.0f);
                const float gy = fmaxf(fmaxf(__fsub_rn(b * w, qy), __fsub_rn(qy, (b + 1) * w)), 0.0f);
                const float gz = fmaxf(fmaxf(__fsub_rn(z * w, qz), __fsub_rn(qz, (z + 1) * w)), 0.0f);
                d2 = __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
                keep = cnt > 0 && !(d2 > lim);
                leaf = gc == gmax || cnt <= kFarLeaf;
            }
            if (__any_sync(0xffffffffu, keep && leaf)) {
                // the kept leaf children's samples, flattened over the lanes
                const int lc = (keep && leaf) ? cnt : 0;
                int incl = lc;
#pragma unroll
                for (int o = 1; o < 8; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                if (lane < 8) {
                    loff[lane] = incl - lc;
                    lbase[lane] = n0;
                }
                const int total = __shfl_sync(0xffffffffu, incl, 7);
                if (lane == 0) loff[8] = total;
                __syncwarp();
                float bd[4] = {1e6f, 1e6f, 1e6f, 1e6f};
                int bi[4] = {0x7fffffff, 0x7fffffff, 0x7fffffff, 0x7fffffff};
                int k = 0;
                for (int f = lane; f < total; f += 32) {
                    while (loff[k + 1] <= f) ++k;   // flattened index -> child (increasing)
                    knn_visit_below(qx, qy, qz, px, py, pz, lbase[k] + (f - loff[k]), md[3], mi[3], bd, bi);
                }
                // merged only when some lane found a sample that enters the 4 nearest so far
                // (each lane's list is sorted: its head decides; most batches of a far
                // search bring none)
                if (__any_sync(0xffffffffu, knn_less(bd[0], bi[0], md[3], mi[3]))) {
                    float ld[4];
                    int li[4];
                    knn_warp_merge(bd, bi, ld, li);
                    knn_merge4(md, mi, ld, li);
                }
                __syncwarp();   // the offsets are read before the next expansion rewrites them
            }
            // the kept inner children: rank by box distance (ties: lower child), pushed in
            // reverse so the nearest is popped next
            const bool push = keep && !leaf;
            const unsigned pm = __ballot_sync(0xffffffffu, push);
            int rank = 0;
#pragma unroll
            for (int o = 0; o < 8; ++o) {
                const float od = __shfl_sync(0xffffffffu, d2, o);
                if (((pm >> o) & 1u) && (od < d2 || (od == d2 && o < lane))) ++rank;
            }
            const int np = __popc(pm);
            if (push) {
                stk[top + np - 1 - rank] = (gc << 24) | (int)child;
                sdist[top + np - 1 - rank] = d2;
            }
            top += np;
            __syncwarp();
        }
        if (lane == 0) colour_blend(md, mi, cr, cg, cb, &out[3 * (size_t)v]);
        __syncwarp();   // the stack is rewritten for the next vertex
    }
}

__global__ void __launch_bounds__(kBlock) k_normals_zero(const Counters* c, double* acc, int* cnt) {
    PSR_CLOUD(c, acc, cnt);
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(v, V) {
        acc[3 * (size_t)v] = acc[3 * (size_t)v + 1] = acc[3 * (size_t)v + 2] = 0.0;
        cnt[v] = 0;
    }
}

// a b - c d within 1.5 ulp (Kahan's difference of products: fma recovers the rounding error
// of c d), so a sliver triangle's cross product keeps its direction instead of cancelling
__device__ __forceinline__ float diff_of_products(float a, float b, float c, float d) {
    const float w = __fmul_rn(c, d);
    const float e = fmaf(-c, d, w);
    const float f = fmaf(a, b, -w);
    return f + e;
}

__global__ void __launch_bounds__(kBlock) k_triangle_normals(const Counters* c, const float* mv, const int* mt,
                                                             double* acc, int* cnt) {
    PSR_CLOUD(c, mv, mt, acc, cnt);
    const int T = c->n_mesh_triangles;
    const int V = c->n_mesh_vertices;
    PSR_GRID_STRIDE(t, T) {
        const int i0 = mt[3 * (size_t)t], i1 = mt[3 * (size_t)t + 1], i2 = mt[3 * (size_t)t + 2];
        if (i0 < 0 || i1 < 0 || i2 < 0 || i0 >= V || i1 >= V || i2 >= V) continue;
        const float ox = mv[3 * (size_t)i0], oy = mv[3 * (size_t)i0 + 1], oz = mv[3 * (size_t)i0 + 2];
        const float ax = mv[3 * (size_t)i1] - ox, ay = mv[3 * (size_t)i1 + 1] - oy, az = mv[3 * (size_t)i1 + 2] - oz;
        const float bx = mv[3 * (size_t)i2] - ox, by = mv[3 * (size_t)i2 + 1] - oy, bz = mv[3 * (size_t)i2 + 2] - oz;
        float nx = diff_of_products(ay, bz, az, by), ny = diff_of_products(az, bx, ax, bz),
              nz = diff_of_products(ax, by, ay, bx);
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
    PSR_CLOUD(c, acc, cnt, out);
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

// sample grid of the colour search: needs only the sorted samples, so it runs beside the solve
cudaError_t transfer_prepare(Workspace& ws, int with_colour) {
    if (!with_colour) return cudaSuccess;
    const int D = ws.depth;
    const int g = D < kColourGridLevel ? D : kColourGridLevel;
    cudaError_t e = fill_words((unsigned*)ws.cell_start, 0u, ((long long)1 << (3 * g)) + 1, ws.batch, ws.stream);
    if (e != cudaSuccess) return e;
    k_cell_count<<<PSR_GRID(ws, ws.num_sms * 4), kBlock, 0, ws.stream>>>(ws.cnt, D, g, ws.key, ws.point2node, ws.cell_start);
    unsigned* table = reinterpret_cast<unsigned*>(ws.cell_start);
    Counters* c = ws.cnt;
    return launch_scan(LoadArray{table}, StoreExclusive{table}, &c->n_colour_cells, 0, ws.scan,
                       (unsigned*)&c->scan_total_aux, &c->error, ws.stream, ScanCount{}, 2);
}

cudaError_t transfer_build(Workspace& ws, int with_colour, int with_normals) {
    cudaStream_t s = ws.stream;
    const int grid = ws.num_sms * 8;
    const int D = ws.depth;
    if (with_colour) {
        const int g = D < kColourGridLevel ? D : kColourGridLevel;
        int* cell_start = ws.cell_start;   // (1 << 3g) + 1 entries, from transfer_prepare
        k_colour_near<<<PSR_GRID(ws, grid), kBlock, 0, s>>>(ws.cnt, g, g, ws.mesh_v, ws.px, ws.py, ws.pz, ws.cr, ws.cg,
                                                          ws.cb, cell_start, nullptr, nullptr, 0, ws.colour_far,
                                                          &ws.cnt->n_colour_far, ws.mesh_c);
        // the vertices it leaves: the same search two levels coarser (a sparse cloud's
        // vertices find their 4 samples there), then the wide search for the rest
        const int* far_list = ws.colour_far;
        const int* far_count = &ws.cnt->n_colour_far;
        if (D >= 8) {
            k_colour_near<<<PSR_GRID(ws, grid), kBlock, 0, s>>>(ws.cnt, g - 2, g, ws.mesh_v, ws.px, ws.py, ws.pz, ws.cr,
                                                              ws.cg, ws.cb, cell_start, ws.colour_far,
                                                              &ws.cnt->n_colour_far, kNearCoarseCap, ws.colour_far2,
                                                              &ws.cnt->n_colour_far2, ws.mesh_c);
            far_list = ws.colour_far2;
            far_count = &ws.cnt->n_colour_far2;
        }
        k_colour_far<<<PSR_GRID(ws, ws.num_sms * 8), kBlock, 0, s>>>(ws.cnt, g, ws.mesh_v, ws.px, ws.py, ws.pz, ws.cr,
                                                                   ws.cg, ws.cb, cell_start, far_list, far_count,
                                                                   ws.mesh_c);
    }
    if (with_normals) {
        double* acc = ws.nacc;
        k_normals_zero<<<PSR_GRID(ws, grid), kBlock, 0, s>>>(ws.cnt, acc, ws.vcount);
        k_triangle_normals<<<PSR_GRID(ws, grid), kBlock, 0, s>>>(ws.cnt, ws.mesh_v, ws.mesh_t, acc, ws.vcount);
        k_vertex_normals<<<PSR_GRID(ws, grid), kBlock, 0, s>>>(ws.cnt, acc, ws.vcount, ws.mesh_n);
    }
    return cudaGetLastError();
}

}  // namespace psr
