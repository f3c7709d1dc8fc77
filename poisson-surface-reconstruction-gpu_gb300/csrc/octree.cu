// Stage (a): normalisation, Morton encoding, radix sort, unique leaves, level-by-level
// octree with full 8-sibling groups, node information and the 27-neighbour table.
//
// Follows mesh/BuildOctree.cu / BuildOctree.cpp:75-194 of the reference (including its
// documented quirks) with a structure-of-arrays layout and device-resident counts.
#include "workspace.h"
#include "tables.cuh"

PSR_DEFINE_CONST_TABLES(upload_tables_octree)

namespace psr {

// ------------------------------------------------------------------------------------
// bounding box (mesh/BuildOctree.cu:51-133) and normalisation parameters (:619-631)
// ------------------------------------------------------------------------------------
__global__ void k_reset_counters(Counters* c, const int* params) {
    PSR_CLOUD(c, params);
    static_assert(sizeof(Counters) % 4 == 0, "Counters is cleared word by word");
    unsigned* w = (unsigned*)c;
    for (int i = threadIdx.x; i < (int)(sizeof(Counters) / 4); i += blockDim.x) w[i] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
        c->n_points = params[0];
        for (int a = 0; a < 3; ++a) {
            // The reference seeds its reduction (padding threads, mesh/BuildOctree.cu:66-73)
            // and its host finish (mesh/BuildOctree.cpp:87-88) with -1e6 / 1e6, which gives a
            // wrong box when every coordinate of an axis lies beyond 1e6 in magnitude (a
            // georeferenced scan).  Seeding with -FLT_MAX / FLT_MAX gives the reference's box
            // for every other input and the true box for those.
            ((int*)c->bbox_max)[a] = float_to_ordered(-FLT_MAX);
            ((int*)c->bbox_min)[a] = float_to_ordered(FLT_MAX);
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_bbox(const float* xyz, const float* nrm, Counters* c) {
    PSR_CLOUD(xyz, nrm, c);
    const int n = c->n_points;
    float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    bool bad = false;
    PSR_GRID_STRIDE(i, n) {
        for (int a = 0; a < 3; ++a) {
            float v = xyz[3 * (size_t)i + a];
            float w = nrm[3 * (size_t)i + a];
            if (!isfinite(v) || !isfinite(w)) bad = true;
            mx[a] = mx[a] < v ? v : mx[a];
            mn[a] = mn[a] > v ? v : mn[a];
        }
    }
    for (int a = 0; a < 3; ++a) {
        for (int o = 16; o > 0; o >>= 1) {
            mx[a] = fmaxf(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
            mn[a] = fminf(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
        }
    }
    if (__any_sync(0xffffffffu, bad) && lane_id() == 0) atomicOr(&c->error, kErrInvalid);
    // block reduction, then one set of atomics per block
    __shared__ float s_mx[3][kBlock / 32], s_mn[3][kBlock / 32];
    const int w = threadIdx.x >> 5;
    if (lane_id() == 0)
        for (int a = 0; a < 3; ++a) { s_mx[a][w] = mx[a]; s_mn[a][w] = mn[a]; }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int a = threadIdx.x;
        float bmx = s_mx[a][0], bmn = s_mn[a][0];
        for (int q = 1; q < kBlock / 32; ++q) { bmx = fmaxf(bmx, s_mx[a][q]); bmn = fminf(bmn, s_mn[a][q]); }
        atomicMax(&((int*)c->bbox_max)[a], float_to_ordered(bmx));
        atomicMin(&((int*)c->bbox_min)[a], float_to_ordered(bmn));
    }
}

__global__ void k_bbox_finalize(Counters* c, float scale) {
    PSR_CLOUD(c);
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float mx[3], mn[3];
    for (int a = 0; a < 3; ++a) {
        mx[a] = ordered_to_float(((int*)c->bbox_max)[a]);
        mn[a] = ordered_to_float(((int*)c->bbox_min)[a]);
        c->bbox_max[a] = mx[a];
        c->bbox_min[a] = mn[a];
    }
    float edge = 1.0f;
    float ctr[3];
    for (int a = 0; a < 3; ++a) {
        float ext = __fsub_rn(mx[a], mn[a]);
        if (a == 0 || edge < ext) edge = ext;
        ctr[a] = __fdiv_rn(__fadd_rn(mx[a], mn[a]), 2.0f);
    }
    edge = __fmul_rn(edge, __fmul_rn(scale, 1.0f));
    for (int a = 0; a < 3; ++a) ctr[a] = __fsub_rn(ctr[a], __fdiv_rn(edge, 2.0f));
    for (int a = 0; a < 3; ++a) c->center[a] = ctr[a];
    c->max_edge = edge;
    if (!(edge > 0.0f)) atomicOr(&c->error, kErrInvalid);
}

__device__ __forceinline__ float normalise_coord(float v, float ctr, float edge) {
    // (p - c) * 1.0f / maxEdge evaluated left to right (mesh/BuildOctree.cu:149)
    return __fdiv_rn(__fmul_rn(__fsub_rn(v, ctr), 1.0f), edge);
}

// Morton code of a normalised point (mesh/BuildOctree.cu:167-208); bit 3l+2 = x of level
// D-l, so the code equals the reference key's upper 32 bits.
__global__ void __launch_bounds__(kBlock) k_encode(const float* xyz, const Counters* c, int depth,
                                                   unsigned* code, unsigned* sidx) {
    PSR_CLOUD(xyz, c, code, sidx);
    const int n = c->n_points;
    const float c0 = c->center[0], c1 = c->center[1], c2 = c->center[2], e = c->max_edge;
    PSR_GRID_STRIDE(i, n) {
        float p[3] = {normalise_coord(xyz[3 * (size_t)i], c0, e), normalise_coord(xyz[3 * (size_t)i + 1], c1, e),
                      normalise_coord(xyz[3 * (size_t)i + 2], c2, e)};
        unsigned k = 0;
        float cc[3] = {0.5f, 0.5f, 0.5f};
        float w = 0.25f;
        for (int l = depth - 1; l >= 0; --l) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if (p[a] > cc[a]) { k |= 1u << (3 * l + 2 - a); cc[a] = __fadd_rn(cc[a], w); }
                else cc[a] = __fsub_rn(cc[a], w);
            }
            w = __fdiv_rn(w, 2.0f);
        }
        code[i] = k;
        sidx[i] = (unsigned)i;
    }
}

// Gather the sorted points, scale the normals to 2^(D+1) (mesh/BuildOctree.cu:152-164)
// and flag the first point of every unique leaf.
__global__ void __launch_bounds__(kBlock) k_gather(const float* xyz, const float* nrm, const uint8_t* rgb,
                                                   const unsigned* scode, const unsigned* sidx, const Counters* c,
                                                   int depth, float* px, float* py, float* pz, float* nx, float* ny,
                                                   float* nz, float* cr, float* cg, float* cb, unsigned* head) {
    PSR_CLOUD(xyz, nrm, rgb, scode, sidx, c, px, py, pz, nx, ny, nz, cr, cg, cb, head);
    const int n = c->n_points;
    const float c0 = c->center[0], c1 = c->center[1], c2 = c->center[2], e = c->max_edge;
    const float nscale = (float)(2 << depth);
    PSR_GRID_STRIDE(i, n) {
        const size_t o = sidx[i];
        px[i] = normalise_coord(xyz[3 * o], c0, e);
        py[i] = normalise_coord(xyz[3 * o + 1], c1, e);
        pz[i] = normalise_coord(xyz[3 * o + 2], c2, e);
        float a = nrm[3 * o], b = nrm[3 * o + 1], d = nrm[3 * o + 2];
        float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(d, d)));
        // reference quirk: a normal no longer than 1e-6 is multiplied by its length
        if (len > 1e-6f) len = __fdiv_rn(1.0f, len);
        len = __fmul_rn(len, nscale);
        nx[i] = __fmul_rn(a, len);
        ny[i] = __fmul_rn(b, len);
        nz[i] = __fmul_rn(d, len);
        if (rgb) {
            cr[i] = __fdiv_rn((float)rgb[3 * o], 255.0f);
            cg[i] = __fdiv_rn((float)rgb[3 * o + 1], 255.0f);
            cb[i] = __fdiv_rn((float)rgb[3 * o + 2], 255.0f);
        } else {
            cr[i] = cg[i] = cb[i] = 0.0f;
        }
        head[i] = (i == 0 || scode[i] != scode[i - 1]) ? 1u : 0u;
    }
}

// scan over leaf heads: point -> unique leaf id, unique leaf -> code / first point
struct HeadStore {
    const unsigned* scode;
    int* puid;
    unsigned* ucode;
    int* ufirst;
    __device__ void operator()(int i, unsigned pre, unsigned v) const {
        int u = (int)(pre + v) - 1;
        puid[i] = u;
        if (v) { ucode[u] = scode[i]; ufirst[u] = i; }
    }
    __device__ void rebase() { PSR_CLOUD(scode, puid, ucode, ufirst); }   // to cloud blockIdx.y
};

__global__ void k_after_unique(Counters* c, int* ufirst, const unsigned* total) {
    PSR_CLOUD(c, ufirst, total);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        c->n_unique = (int)*total;
        ufirst[c->n_unique] = c->n_points;
    }
}

// D-level groups: 8 slots for every new parent code (mesh/BuildOctree.cu:267-280)
struct LeafGroupLoad {
    const unsigned* ucode;
    __device__ unsigned operator()(int u) const {
        return (u == 0) ? 0u : (((ucode[u - 1] >> 3) != (ucode[u] >> 3)) ? 8u : 0u);
    }
    __device__ void rebase() { PSR_CLOUD(ucode); }   // to cloud blockIdx.y
};

__global__ void k_after_leaf_groups(Counters* c, const unsigned* total, int depth, int node_cap) {
    PSR_CLOUD(c, total);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int md = (int)*total + 8;
        if (c->n_unique == 0) md = 0;
        c->level_tmp_off[depth] = 0;
        if (md > node_cap) { atomicOr(&c->error, kErrCapacity); md = 0; }
        c->level_count[depth] = md;
        c->n_groups = md;   // bound for the leaf placement
    }
}

// level initialisation: D level gets dnum = 1, didx = slot (:294-300), others zero
__global__ void __launch_bounds__(kBlock) k_init_level(const Counters* c, int d, int depth, int* tkey, int* tpidx,
                                                       int* tpnum, int* tdidx, int* tdnum, int* tchild) {
    PSR_CLOUD(c, tkey, tpidx, tpnum, tdidx, tdnum, tchild);
    const int m = c->level_count[d];
    const int off = c->level_tmp_off[d];
    PSR_GRID_STRIDE(i, m) {
        tkey[off + i] = 0;
        tpidx[off + i] = 0;
        tpnum[off + i] = 0;
        tdidx[off + i] = (d == depth) ? i : 0;
        tdnum[off + i] = (d == depth) ? 1 : 0;
        tchild[off + i] = -1;
    }
}

// place unique leaves in their groups (:282-292) and map points to leaves (:302-313)
__global__ void __launch_bounds__(kBlock) k_place_leaves(const Counters* c, const unsigned* ucode, const int* ufirst,
                                                         const unsigned* uaddr, int* uslot, int* tkey, int* tpidx,
                                                         int* tpnum) {
    PSR_CLOUD(c, ucode, ufirst, uaddr, uslot, tkey, tpidx, tpnum);
    const int u_n = c->n_unique;
    PSR_GRID_STRIDE(u, u_n) {
        int s = (int)uaddr[u] + (int)(ucode[u] & 7u);
        uslot[u] = s;
        if (s >= c->n_groups) continue;   // capacity overflow (flagged); n_groups holds M_D here
        tkey[s] = (int)ucode[u];
        tpidx[s] = ufirst[u];
        tpnum[s] = ufirst[u + 1] - ufirst[u];
    }
}
__global__ void __launch_bounds__(kBlock) k_point2node(const Counters* c, const int* puid, const int* uslot,
                                                       int* point2node) {
    PSR_CLOUD(c, puid, uslot, point2node);
    const int n = c->n_points;
    PSR_GRID_STRIDE(i, n) point2node[i] = uslot[puid[i]];
}

// per-group aggregation into the father (mesh/BuildOctree.cu:323-357)
__global__ void __launch_bounds__(kBlock) k_group_aggregate(Counters* c, int d, int depth, const int* tkey,
                                                            const int* tpidx, const int* tpnum, const int* tdidx,
                                                            const int* tdnum, int* gkey, int* gpidx, int* gpnum,
                                                            int* gdidx, int* gdnum) {
    PSR_CLOUD(c, tkey, tpidx, tpnum, tdidx, tdnum, gkey, gpidx, gpnum, gdidx, gdnum);
    const int m = c->level_count[d];
    const int off = c->level_tmp_off[d];
    const int G = m / 8;
    if (blockIdx.x == 0 && threadIdx.x == 0) c->n_groups = G;
    const int sh = 3 * (depth - d);
    PSR_GRID_STRIDE(g, G) {
        int fk = 0, pn = 0, pi = 0x7fffffff, dn = 0, di = 0x7fffffff;
        for (int j = 0; j < 8; ++j) {
            int t = off + 8 * g + j;
            int pnum = tpnum[t], dnum = tdnum[t], didx = tdidx[t];
            if (pnum == 0) {
                if (dnum != 0) { dn += dnum; di = min(di, didx); }
            } else {
                fk = tkey[t] & ~(7 << sh);
                pn += pnum;
                pi = min(pi, tpidx[t]);
                dn += dnum;
                di = min(di, didx);
            }
        }
        gkey[g] = fk;
        gpidx[g] = pi;
        gpnum[g] = pn;
        gdidx[g] = di;
        gdnum[g] = dn;
    }
}

// father groups one level up (mesh/BuildOctree.cu:359-375, scan :796-799)
struct FatherGroupLoad {
    const int* gkey;
    int sh2;
    __device__ unsigned operator()(int g) const {
        return (g == 0) ? 0u : (((gkey[g - 1] >> sh2) != (gkey[g] >> sh2)) ? 8u : 0u);
    }
    __device__ void rebase() { PSR_CLOUD(gkey); }   // to cloud blockIdx.y
};

__global__ void k_after_father_groups(Counters* c, int d, const unsigned* total, int node_cap) {
    PSR_CLOUD(c, total);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int m = (d > 1) ? (int)*total + 8 : 1;
        int off = c->level_tmp_off[d] + c->level_count[d];
        c->level_count[d - 1] = m;
        c->level_tmp_off[d - 1] = off;
        if (off + m > node_cap) { atomicOr(&c->error, kErrCapacity); c->level_count[d - 1] = 0; }
    }
}

// place fathers (mesh/BuildOctree.cu:377-390): record the father slot of every group
__global__ void __launch_bounds__(kBlock) k_place_fathers(const Counters* c, int d, int depth, const int* gkey,
                                                          const int* gpidx, const int* gpnum, const int* gdidx,
                                                          const int* gdnum, const unsigned* gaddr, int* tkey,
                                                          int* tpidx, int* tpnum, int* tdidx, int* tdnum, int* tchild,
                                                          int* tparent_slot) {
    PSR_CLOUD(c, gkey, gpidx, gpnum, gdidx, gdnum, gaddr, tkey, tpidx, tpnum, tdidx, tdnum, tchild, tparent_slot);
    const int G = c->n_groups;
    const int off_parent = c->level_tmp_off[d - 1];
    const int off_group = c->level_tmp_off[d] / 8;
    const int sh3 = 3 * (depth - d + 1);
    PSR_GRID_STRIDE(g, G) {
        int s = (int)gaddr[g] + ((gkey[g] >> sh3) & 7);
        if (s >= c->level_count[d - 1]) continue;   // capacity overflow (flagged)
        int t = off_parent + s;
        tkey[t] = gkey[g];
        tpidx[t] = gpidx[g];
        tpnum[t] = gpnum[g];
        tdidx[t] = gdidx[g];
        tdnum[t] = gdnum[g];
        tchild[t] = 8 * g;   // level-local address of the child group
        tparent_slot[off_group + g] = s;
    }
}

// ---- coarse levels in one CTA --------------------------------------------------------
// The levels near the root hold few nodes, so their per-level passes (group aggregate,
// father-group scan, level set-up, father placement) run inside one 1024-thread CTA with
// block barriers between steps instead of five launches per level.  Same arithmetic as
// the per-level kernels above.
constexpr int kLevelBlock = 1024;

// inclusive block scan of one value per thread (1024 threads); returns the block total
__device__ __forceinline__ unsigned block_inclusive_scan_1024(unsigned v, unsigned* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    if (lane == 31) s_warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        unsigned w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        s_warp[lane] = w;   // inclusive warp totals
    }
    __syncthreads();
    const unsigned r = v + (warp > 0 ? s_warp[warp - 1] : 0u);
    const unsigned total = s_warp[31];
    __syncthreads();
    s_warp[32] = total;
    return r;
}

__global__ void __launch_bounds__(kLevelBlock) k_levels_block(Counters* c, int dtop, int depth, int* tkey, int* tpidx,
                                                              int* tpnum, int* tdidx, int* tdnum, int* tchild,
                                                              int* tparent_slot, int* gkey, int* gpidx, int* gpnum,
                                                              int* gdidx, int* gdnum, unsigned* gaddr, int node_cap) {
    PSR_CLOUD(c, tkey, tpidx, tpnum, tdidx, tdnum, tchild, tparent_slot, gkey, gpidx, gpnum, gdidx, gdnum, gaddr);
    __shared__ unsigned s_warp[33];
    const int t = threadIdx.x;
    for (int d = dtop; d >= 1; --d) {
        const int m = c->level_count[d];
        const int off = c->level_tmp_off[d];
        const int G = m / 8;
        const int sh = 3 * (depth - d);
        // (1) sibling groups of level d -> father candidates
        for (int g = t; g < G; g += kLevelBlock) {
            int fk = 0, pn = 0, pi = 0x7fffffff, dn = 0, di = 0x7fffffff;
            for (int j = 0; j < 8; ++j) {
                const int q = off + 8 * g + j;
                const int pnum = tpnum[q], dnum = tdnum[q], didx = tdidx[q];
                if (pnum == 0) {
                    if (dnum != 0) { dn += dnum; di = min(di, didx); }
                } else {
                    fk = tkey[q] & ~(7 << sh);
                    pn += pnum;
                    pi = min(pi, tpidx[q]);
                    dn += dnum;
                    di = min(di, didx);
                }
            }
            gkey[g] = fk;
            gpidx[g] = pi;
            gpnum[g] = pn;
            gdidx[g] = di;
            gdnum[g] = dn;
        }
        __syncthreads();
        // (2) inclusive scan of "new father group" flags (8 per new group of level d-1)
        const int sh2 = 3 * (depth - d + 2);
        unsigned carry = 0;
        for (int b = 0; b < G; b += kLevelBlock) {
            const int g = b + t;
            const unsigned f = (g < G && g > 0) ? (((gkey[g - 1] >> sh2) != (gkey[g] >> sh2)) ? 8u : 0u) : 0u;
            const unsigned incl = block_inclusive_scan_1024(f, s_warp);
            if (g < G) gaddr[g] = carry + incl;
            carry += s_warp[32];
            __syncthreads();
        }
        // (3) size and offset of level d-1
        int m1 = (d > 1) ? (int)carry + 8 : 1;
        const int off1 = off + m;
        if (off1 + m1 > node_cap) {
            if (t == 0) atomicOr(&c->error, kErrCapacity);
            m1 = 0;
        }
        if (t == 0) {
            c->level_count[d - 1] = m1;
            c->level_tmp_off[d - 1] = off1;
            c->n_groups = G;
        }
        for (int i = t; i < m1; i += kLevelBlock) {
            tkey[off1 + i] = 0;
            tpidx[off1 + i] = 0;
            tpnum[off1 + i] = 0;
            tdidx[off1 + i] = 0;
            tdnum[off1 + i] = 0;
            tchild[off1 + i] = -1;
        }
        __syncthreads();
        // (4) fathers into their slots of level d-1
        const int off_group = off / 8;
        const int sh3 = 3 * (depth - d + 1);
        for (int g = t; g < G; g += kLevelBlock) {
            const int sl = (int)gaddr[g] + ((gkey[g] >> sh3) & 7);
            if (sl >= m1) continue;   // capacity overflow (flagged)
            const int q = off1 + sl;
            tkey[q] = gkey[g];
            tpidx[q] = gpidx[g];
            tpnum[q] = gpnum[g];
            tdidx[q] = gdidx[g];
            tdnum[q] = gdnum[g];
            tchild[q] = 8 * g;
            tparent_slot[off_group + g] = sl;
        }
        __syncthreads();
    }
}

// 27-neighbour tables of levels 1..dmax in one CTA (levels in order: a level reads its
// parents' table)
__global__ void __launch_bounds__(kLevelBlock) k_neighbours_block(const Counters* c, int dmax, int depth,
                                                                  const int* key, const int* parent,
                                                                  const int* first_child, int* neigh, size_t stride) {
    PSR_CLOUD(c, key, parent, first_child, neigh);
    for (int d = 1; d <= dmax; ++d) {
        const int m = c->level_count[d];
        const int b = c->level_base[d];
        for (int li = threadIdx.x; li < m; li += kLevelBlock) {
            const int i = b + li;
            const int son = (key[i] >> (3 * (depth - d))) & 7;
            const int pa = parent[i];
            // every read before the first store: the look-ups overlap
            int v[27];
            child_neighbours(son, [&](int j) { return neigh[(size_t)j * stride + pa]; },
                             [&](int n) { return first_child[n]; }, v);
#pragma unroll
            for (int k = 0; k < 27; ++k) neigh[(size_t)k * stride + i] = v[k];
        }
        __syncthreads();
    }
}

__global__ void k_levels_done(Counters* c, int depth) {
    PSR_CLOUD(c);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        int b = 0;
        for (int d = 0; d <= depth; ++d) {
            c->level_base[d] = b;
            b += c->level_count[d];
        }
        c->n_nodes = b;
    }
}

// Final node records (mesh/BuildOctree.cu:392-488, :552-586, :514-550).
__global__ void __launch_bounds__(kBlock) k_finalize_nodes(const Counters* c, int depth, const int* tkey,
                                                           const int* tpidx, const int* tpnum, const int* tdidx,
                                                           const int* tdnum, const int* tchild,
                                                           const int* tparent_slot, int* key, int* pidx, int* pnum,
                                                           int* parent, int* first_child, int* didx, int* dnum,
                                                           int* ndepth, int* enc, float* cx, float* cy, float* cz) {
    PSR_CLOUD(c, tkey, tpidx, tpnum, tdidx, tdnum, tchild, tparent_slot, key, pidx, pnum, parent, first_child, didx, dnum, ndepth, enc, cx, cy, cz);
    const int M = c->n_nodes;
    PSR_GRID_STRIDE(i, M) {
        int d = 0;
        while (d < depth && i >= c->level_base[d + 1]) ++d;
        const int li = i - c->level_base[d];
        const int off = c->level_tmp_off[d];
        const int t = off + li;
        int k, pi, pn, dn, di, par, fc;
        pn = tpnum[t];
        dn = tdnum[t];
        if (d == 0) {
            k = tkey[t];
            pi = tpidx[t];
            di = tdidx[t];
            par = -1;
            fc = 1;   // root children are 1..8 (:403-410)
        } else {
            const int sh = 3 * (depth - d);
            const int g = li >> 3, j = li & 7;
            const int gs = off + 8 * g;
            int v = 0;
            while (v < 8 && tpnum[gs + v] == 0) ++v;
            if (v == 8) v = 0;   // cannot happen: every group holds a non-empty node
            k = (tkey[gs + v] & ~(7 << sh)) | (j << sh);
            int nowP = tpidx[gs + v], nowD = tdidx[gs + v];
            for (int q = 0; q < j; ++q) { nowP += tpnum[gs + q]; nowD += tdnum[gs + q]; }
            pi = nowP;
            di = (d == depth) ? tdidx[t] : nowD;
            // reference quirk: the first non-empty node of the group passes its parent to
            // all siblings, and a node at level-local index 0 never had its parent set
            const int lp = (g == 0 && v == 0) ? 0 : tparent_slot[off / 8 + g];
            par = c->level_base[d - 1] + lp;
            fc = (pn != 0 && d < depth) ? c->level_base[d + 1] + tchild[t] : -1;
        }
        key[i] = k;
        pidx[i] = pi;
        pnum[i] = pn;
        parent[i] = par;
        first_child[i] = fc;
        didx[i] = di;
        dnum[i] = dn;
        ndepth[i] = d;
        float cc[3] = {0.5f, 0.5f, 0.5f};
        float w = 0.25f;
        for (int l = depth - 1; l >= depth - d; --l) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                if ((k >> (3 * l + 2 - a)) & 1) cc[a] = __fadd_rn(cc[a], w);
                else cc[a] = __fsub_rn(cc[a], w);
            }
            w = __fdiv_rn(w, 2.0f);
        }
        cx[i] = cc[0];
        cy[i] = cc[1];
        cz[i] = cc[2];
        int e = ((1 << d) - 1) * (1 + (1 << (depth + 1)) + (1 << (2 * (depth + 1))));
        for (int l = d; l >= 1; --l) {
            int sx = (k >> (3 * (depth - l) + 2)) & 1;
            int sy = (k >> (3 * (depth - l) + 1)) & 1;
            int sz = (k >> (3 * (depth - l))) & 1;
            e += sx * (1 << (d - l)) + sy * (1 << (d - l)) * (1 << (depth + 1)) +
                 sz * (1 << (d - l)) * (1 << (2 * (depth + 1)));
        }
        enc[i] = e;
    }
}

// 27-neighbour table of one depth (mesh/BuildOctree.cu:490-512), stored [27][cap]
__global__ void __launch_bounds__(kBlock) k_neighbours(const Counters* c, int d, int depth, const int* key,
                                                       const int* parent, const int* first_child, int* neigh,
                                                       size_t stride) {
    PSR_CLOUD(c, key, parent, first_child, neigh);
    const int m = c->level_count[d];
    const int b = c->level_base[d];
    PSR_GRID_STRIDE(li, m) {
        const int i = b + li;
        const int son = (key[i] >> (3 * (depth - d))) & 7;
        const int pa = parent[i];
        int v[27];
        child_neighbours(son, [&](int j) { return neigh[(size_t)j * stride + pa]; },
                         [&](int n) { return first_child[n]; }, v);
#pragma unroll
        for (int k = 0; k < 27; ++k) neigh[(size_t)k * stride + i] = v[k];
    }
}

__global__ void k_root_neighbours(int* neigh, size_t stride) {
    PSR_CLOUD(neigh);
    int k = threadIdx.x;
    if (k < 27) neigh[(size_t)k * stride] = (k == 13) ? 0 : -1;
}

// points -> Morton codes of the reference's normalised coordinates at `depth`, sorted with
// their input indices (the octree's first steps; the normal estimation stage uses them on
// their own).  n_points and the bounding-box seeds must be set.
cudaError_t encode_sort_points(Workspace& ws, const float* xyz, int depth, const unsigned** scode,
                               const unsigned** sidx) {
    cudaStream_t s = ws.stream;
    Counters* c = ws.cnt;
    const int gp = grid_for(ws, ws.cap.points);
    k_bbox<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(xyz, xyz, c);
    k_bbox_finalize<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, 1.25f);
    k_encode<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(xyz, c, depth, ws.code, ws.sidx);
    bool alt = false;
    cudaError_t e = radix_sort_pairs(ws.code, ws.sidx, &c->n_points, 3 * depth, ws.sort, &c->error, s, &alt);
    if (e != cudaSuccess) return e;
    *scode = alt ? ws.sort.keys_alt : ws.code;
    *sidx = alt ? ws.sort.vals_alt : ws.sidx;
    return cudaGetLastError();
}

cudaError_t octree_build(Workspace& ws) {
    cudaStream_t s = ws.stream;
    const int D = ws.depth;
    Counters* c = ws.cnt;
    unsigned* err = &c->error;
    unsigned* total = (unsigned*)&c->scan_total;
    const int gp = grid_for(ws, ws.cap.points);
    k_reset_counters<<<PSR_GRID(ws, 1), 256, 0, s>>>(c, ws.d_params);
    k_bbox<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(ws.in_xyz, ws.in_nrm, c);
    k_bbox_finalize<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, 1.25f);
    k_encode<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(ws.in_xyz, c, D, ws.code, ws.sidx);
    bool alt = false;
    cudaError_t e = radix_sort_pairs(ws.code, ws.sidx, &c->n_points, 3 * D, ws.sort, err, s, &alt);
    if (e != cudaSuccess) return e;
    const unsigned* scode = alt ? ws.sort.keys_alt : ws.code;
    const unsigned* sidx = alt ? ws.sort.vals_alt : ws.sidx;
    unsigned* head = alt ? ws.code : ws.sort.keys_alt;   // free buffer of N words
    k_gather<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(ws.in_xyz, ws.in_nrm, ws.in_rgb, scode, sidx, c, D, ws.px, ws.py, ws.pz, ws.nx,
                                   ws.ny, ws.nz, ws.cr, ws.cg, ws.cb, head);
    e = launch_scan(LoadArray{head}, HeadStore{scode, ws.puid, ws.ucode, ws.ufirst}, &c->n_points, 0, ws.scan, total,
                    err, s, ScanCount{}, 1);
    if (e != cudaSuccess) return e;
    k_after_unique<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, ws.ufirst, total);
    e = launch_scan(LeafGroupLoad{ws.ucode}, StoreInclusive{ws.uaddr}, &c->n_unique, 0, ws.scan, total, err, s,
                    ScanCount{}, 1);
    if (e != cudaSuccess) return e;
    k_after_leaf_groups<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, total, D, ws.cap.dnodes);
    const int gn = grid_for(ws, ws.cap.dnodes);
    k_init_level<<<PSR_GRID(ws, gn), kBlock, 0, s>>>(c, D, D, ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.tchild);
    k_place_leaves<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(c, ws.ucode, ws.ufirst, ws.uaddr, ws.uslot, ws.tkey, ws.tpidx, ws.tpnum);
    k_point2node<<<PSR_GRID(ws, gp), kBlock, 0, s>>>(c, ws.puid, ws.uslot, ws.point2node);
    // levels D .. dfuse+1 level by level across the GPU, the small levels near the root in
    // one CTA
    const int dfuse = D - 3;
    for (int d = D; d >= 1 && d > dfuse; --d) {
        const int gg = grid_for(ws, ws.cap.dnodes / 8 + 1);
        k_group_aggregate<<<PSR_GRID(ws, gg), kBlock, 0, s>>>(c, d, D, ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.gkey,
                                                ws.gpidx, ws.gpnum, ws.gdidx, ws.gdnum);
        e = launch_scan(FatherGroupLoad{ws.gkey, 3 * (D - d + 2)}, StoreInclusive{ws.gaddr}, &c->n_groups, 0, ws.scan,
                        total, err, s, ScanCount{}, 1);
        if (e != cudaSuccess) return e;
        k_after_father_groups<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, d, total, ws.cap.nodes);
        k_init_level<<<PSR_GRID(ws, gg), kBlock, 0, s>>>(c, d - 1, D, ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.tchild);
        k_place_fathers<<<PSR_GRID(ws, gg), kBlock, 0, s>>>(c, d, D, ws.gkey, ws.gpidx, ws.gpnum, ws.gdidx, ws.gdnum, ws.gaddr,
                                              ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.tchild,
                                              ws.tparent_slot);
    }
    if (dfuse >= 1)
        k_levels_block<<<PSR_GRID(ws, 1), kLevelBlock, 0, s>>>(c, dfuse, D, ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.tchild,
                                                 ws.tparent_slot, ws.gkey, ws.gpidx, ws.gpnum, ws.gdidx, ws.gdnum,
                                                 ws.gaddr, ws.cap.nodes);
    k_levels_done<<<PSR_GRID(ws, 1), 1, 0, s>>>(c, D);
    const int gm = grid_for(ws, ws.cap.nodes);
    k_finalize_nodes<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, D, ws.tkey, ws.tpidx, ws.tpnum, ws.tdidx, ws.tdnum, ws.tchild,
                                           ws.tparent_slot, ws.key, ws.pidx, ws.pnum, ws.parent, ws.first_child,
                                           ws.didx, ws.dnum, ws.ndepth, ws.enc, ws.ctr_x, ws.ctr_y, ws.ctr_z);
    const size_t stride = (size_t)ws.cap.nodes;
    k_root_neighbours<<<PSR_GRID(ws, 1), 32, 0, s>>>(ws.neigh, stride);
    if (dfuse >= 1)
        k_neighbours_block<<<PSR_GRID(ws, 1), kLevelBlock, 0, s>>>(c, dfuse, D, ws.key, ws.parent, ws.first_child, ws.neigh, stride);
    for (int d = (dfuse >= 1 ? dfuse + 1 : 1); d <= D; ++d)
        k_neighbours<<<PSR_GRID(ws, gm), kBlock, 0, s>>>(c, d, D, ws.key, ws.parent, ws.first_child, ws.neigh, stride);
    return cudaGetLastError();
}

}  // namespace psr
