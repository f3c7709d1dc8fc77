// Common device definitions for the Poisson reconstruction kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>
#include <cstdio>

namespace psr {

constexpr int kMaxDepth = 9;      // the encoded function index packs 3 x (D+1) bits in int32
constexpr int kBlock = 256;

// Device error word bits (read back by the host after a run).
enum : unsigned {
    kErrSpinTimeout = 1u,   // a bounded wait gave up
    kErrCapacity = 2u,      // a device-side count exceeded its buffer capacity
    kErrInvalid = 4u,       // non-finite input
};

// Device-resident counts: every kernel reads its problem size from here, so the whole
// pipeline can be replayed from a CUDA graph without host round trips.
struct Counters {
    int n_points;
    int n_unique;
    int n_groups;                 // scratch: group count of the level being built
    int level_count[kMaxDepth + 1];
    int level_base[kMaxDepth + 1];
    int level_tmp_off[kMaxDepth + 1];   // offset of each level inside the build buffer
    int n_nodes;
    int n_vertices, n_edges, n_faces;
    int n_cross, n_tri;
    int n_subroots;
    // subdivision, per depth d: candidates, their first compact slot, the first entry of
    // the depth's live list, live nodes, first root index and roots of depth d
    int sub_cand[kMaxDepth + 2], sub_cbase[kMaxDepth + 2], sub_lbase[kMaxDepth + 2];
    int sub_nlive[kMaxDepth + 2], sub_rstart[kMaxDepth + 2], sub_nroots[kMaxDepth + 2];
    int n_sub_nodes;              // subdivision nodes built (candidates of all depths)
    int n_sub_dnodes;             // live depth-D subdivision cells
    int n_sub_vertices, n_sub_edges, n_sub_cross, n_sub_tri;
    int n_mesh_vertices, n_mesh_triangles;
    int n_colour_far;             // mesh vertices whose 4 nearest samples the near pass left
    int n_colour_far2;            //   and of those, the ones the coarser pass left
    int n_colour_cells;           // entries of the colour cell table
    int n_weld;                   // mesh vertices left by welding
    int scan_total;               // scratch total written by scans
    int scan_total_aux;           // the same for scans issued on the geometry stream
    unsigned error;
    float bbox_min[3], bbox_max[3];
    float center[3];
    float max_edge;
    double iso_sum;
    float iso;
    int cg_iters[kMaxDepth + 1];
    double cg_rr[kMaxDepth + 1];      // recursive r.r at the end of each depth's CG (FP64)
    double cg_rr_true[kMaxDepth + 1]; // r.r of the last true residual b - A x (-1: none)
    int cg_checks[kMaxDepth + 1];     // true-residual evaluations of each depth's CG
    int cg_restarts[kMaxDepth + 1];   // refinement restarts from the true residual
    unsigned long long cg_depth_ns[kMaxDepth + 1];   // device time of each depth's CG
};

// State of one depth's CG when it runs as a device loop (a CUDA-graph while node whose
// body launches one kernel per step over the whole GPU): the scalars the cluster solver
// keeps in shared memory, in global memory between the kernels of an iteration.
struct CgLoopState {
    double rr, rr_prev, pap, floor2, rr_true;
    float alpha, beta;
    int go, check, replace, checks, restarts;
    int active;              // the depth runs in the device loop (else a cluster solves it)
    int it;                  // iterations done
    unsigned ticket;         // blocks of the current kernel done (last-block reductions)
    unsigned long long t0;   // global timer at the start of the solve
    unsigned long long t1;   // global timer at the end of its last step
};
constexpr int kLoopMaxBlocks = 2048;   // virtual blocks of one depth of the device loop (partials)

// Look-up tables shared by the kernels (values derived in tables.cpp).
struct ConstTables {
    int lut_parent[8][27];
    int lut_child[8][27];
    int edge_vertex[12][2];
    int face_edges[6][4];
    int parent_face_kind[8][6];
    int children_vertex_kind[8];
    unsigned long long mc_tri[256];
    int mc_count[256];
};

// ---- multi-cloud launches --------------------------------------------------------------
// A batch handle keeps one complete workspace per cloud.  The workspaces sit in one
// reserved address range, slot k at k * kCloudStride from slot 0, so a workspace pointer
// of cloud 0 plus k * kCloudStride is the same buffer of cloud k.  Every kernel of the
// pipeline is launched once for all the clouds of a batch with gridDim.y = clouds, and
// first moves each of its workspace pointers (PSR_CLOUD) to cloud blockIdx.y; a one-cloud
// launch has blockIdx.y = 0 and keeps them.  Null pointers (absent optional inputs) stay
// null.  The range is aligned to kMaxBatchClouds * kCloudStride, so bits 35..40 of a
// workspace address are its slot.
constexpr unsigned long long kCloudStride = 1ull << 35;   // 32 GiB of address space per cloud
constexpr int kMaxBatchClouds = 64;
// words of the device loop's control block (pass and unit counts, the unit list, its
// virtual-block offsets)
constexpr int kLoopControlWords = 3 + 2 * kMaxBatchClouds * (kMaxDepth + 1);

// blocks along x of a launch over `clouds` clouds whose one-cloud launch has gx blocks:
// about twice the one-cloud grid in total (each cloud's blocks stride over its work), at
// least one block per cloud
inline int cloud_blocks(int clouds, int gx) {
    if (clouds <= 1) return gx;
    const int g = (2 * gx + clouds - 1) / clouds;
    return g < 1 ? 1 : (g < gx ? g : gx);
}

#ifdef __CUDACC__
template <class T>
__device__ __forceinline__ void cloud_rebase_one(T*& p) {
#ifdef PSR_CLOUD_CHECK
    // diagnostic builds: a pointer handed to a multi-cloud launch must be slot 0's
    if (blockIdx.y != 0 && p && ((((unsigned long long)p) >> 35) & (kMaxBatchClouds - 1)) != 0) {
        if (threadIdx.x == 0 && blockIdx.x == 0)
            printf("PSR_CLOUD_CHECK: cloud %u got a pointer outside slot 0: %p\n", blockIdx.y, (const void*)p);
        return;
    }
#endif
    if (p) p = (T*)((const char*)p + (unsigned long long)blockIdx.y * kCloudStride);
}
template <class S>
__device__ __forceinline__ auto cloud_rebase_one(S& s) -> decltype(s.rebase(), void()) {
    s.rebase();
}
template <class... T>
__device__ __forceinline__ void cloud_rebase(T&... p) {
    (cloud_rebase_one(p), ...);
}
#define PSR_CLOUD(...) ::psr::cloud_rebase(__VA_ARGS__)

#define PSR_GRID_STRIDE(i, n) for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += gridDim.x * blockDim.x)

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// ordered-int encoding of floats for atomic min / max
__device__ __forceinline__ int float_to_ordered(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ordered_to_float(int i) {
    return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff);
}

__device__ __forceinline__ int ilog2_dev(int v) { return 31 - __clz(v); }

// Normalised quadratic B-spline of the 1-D function index `idx` (centre (o+1/2)/2^d,
// width 2^-d) at x.  Operation order is fixed (no contraction) so the host mirror in
// the oracle reproduces it bit for bit.
__device__ __forceinline__ float basis32(int idx, float x) {
    const float kF43 = 1.33333337306976318359375f;
    const float kF23 = 0.666666686534881591796875f;
    int d = ilog2_dev(idx + 1);
    int off = idx + 1 - (1 << d);
    float s = (float)(1 << d);
    // (off + 1/2) / 2^d: the quotient by a power of two is exact, so it is the product with 2^-d
    float c = __fmul_rn(__fadd_rn((float)off, 0.5f), __int_as_float((127 - d) << 23));
    float t = __fmul_rn(__fsub_rn(x, c), s);
    float a = fabsf(t);
    if (a < 0.5f) return __fmul_rn(__fsub_rn(0.75f, __fmul_rn(t, t)), kF43);
    if (a < 1.5f) { float u = __fsub_rn(1.5f, a); return __fmul_rn(__fmul_rn(u, u), kF23); }
    return 0.0f;
}

// Function index of a node at tree depth `depth` packed as (D+1)-bit fields x | y | z.
__device__ __forceinline__ void decode_fn_index(int e, int depth, int& ix, int& iy, int& iz) {
    const int o1 = 1 << (depth + 1);
    ix = e & (o1 - 1);
    iy = (e >> (depth + 1)) & (o1 - 1);
    iz = e >> (2 * (depth + 1));
}

// Neighbour slot k (9 ox + 3 oy + oz) of child `son` (x = 4, y = 2, z = 1) seen from its
// parent: the parent's neighbour slot holding that cell's parent (lp) and the cell's child
// slot there (lc) -- the table of mesh/BuildOctree.cu:20-42 evaluated arithmetically.
__device__ __forceinline__ void nb_lut(int son, int k, int& lp, int& lc) {
    const int qx = ((son >> 2) & 1) + k / 9 - 1;
    const int qy = ((son >> 1) & 1) + (k / 3) % 3 - 1;
    const int qz = (son & 1) + k % 3 - 1;
    lp = 9 * ((qx >= 0) + (qx > 1)) + 3 * ((qy >= 0) + (qy > 1)) + ((qz >= 0) + (qz > 1));
    lc = 4 * ((qx + 2) & 1) + 2 * ((qy + 2) & 1) + ((qz + 2) & 1);
}

// The 27 same-depth neighbours of child `son` (x = bit 2) of a node, the child of the same
// slot order as nb_lut: per axis they lie in two of the parent's neighbours (the parent's -1
// and 0 for a lower child, 0 and +1 for an upper one), so 8 parent-row reads and 8
// first-child reads, all independent, give the 27 (children of a missing neighbour, or of a
// childless one, are -1).  `row(j)` reads entry j (0..26) of the parent's neighbour row;
// `first(n)` reads first_child[n].  The picks below use compile-time indices only.
template <class Row, class First>
__device__ __forceinline__ void child_neighbours(int son, Row row, First first, int (&v)[27]) {
    const int sx = (son >> 2) & 1, sy = (son >> 1) & 1, sz = son & 1;
    int F[2][2][2];
#pragma unroll
    for (int jx = 0; jx < 2; ++jx)
#pragma unroll
        for (int jy = 0; jy < 2; ++jy)
#pragma unroll
            for (int jz = 0; jz < 2; ++jz) F[jx][jy][jz] = row(9 * (sx + jx) + 3 * (sy + jy) + (sz + jz));
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int& f = F[j >> 2][(j >> 1) & 1][j & 1];
        f = (f == -1) ? -1 : first(f);
    }
    // offset d per axis (0, 1, 2 for -1, 0, +1): parent column 0, 1 - s, 1
    int Gx[3][2][2];
#pragma unroll
    for (int jy = 0; jy < 2; ++jy)
#pragma unroll
        for (int jz = 0; jz < 2; ++jz) {
            Gx[0][jy][jz] = F[0][jy][jz];
            Gx[1][jy][jz] = sx ? F[0][jy][jz] : F[1][jy][jz];
            Gx[2][jy][jz] = F[1][jy][jz];
        }
    int Gy[3][3][2];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int jz = 0; jz < 2; ++jz) {
            Gy[a][0][jz] = Gx[a][0][jz];
            Gy[a][1][jz] = sy ? Gx[a][0][jz] : Gx[a][1][jz];
            Gy[a][2][jz] = Gx[a][1][jz];
        }
#pragma unroll
    for (int k = 0; k < 27; ++k) {
        const int a = k / 9, b = (k / 3) % 3, cz = k % 3;
        const int g = (cz == 0) ? Gy[a][b][0] : (cz == 2) ? Gy[a][b][1] : (sz ? Gy[a][b][0] : Gy[a][b][1]);
        // child bit per axis: (s + d - 1) & 1
        const int lc = 4 * ((sx + a + 1) & 1) + 2 * ((sy + b + 1) & 1) + ((sz + cz + 1) & 1);
        v[k] = (g == -1) ? -1 : g + lc;
    }
}

// Terms of one level of an implicit-function chain: the 27 same-depth neighbours nb of
// `node`, each adding ((x[nb] * Fx) * Fy) * Fz in slot order.  A neighbour's function
// index is the node's own plus the slot offset, so the 81 basis values come from 9.
__device__ __forceinline__ float terms_from(int encv, const int (&nbs)[27], const float (&xv)[27], float val,
                                            float qx, float qy, float qz, int depth) {
    int ox, oy, oz;
    decode_fn_index(encv, depth, ox, oy, oz);
    float bx[3], by[3], bz[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        bx[j] = basis32(ox - 1 + j, qx);
        by[j] = basis32(oy - 1 + j, qy);
        bz[j] = basis32(oz - 1 + j, qz);
    }
#pragma unroll
    for (int k = 0; k < 27; ++k) {
        if (nbs[k] == -1) continue;
        float t = __fmul_rn(xv[k], bx[k / 9]);
        t = __fmul_rn(t, by[(k / 3) % 3]);
        t = __fmul_rn(t, bz[k % 3]);
        val = __fadd_rn(val, t);
    }
    return val;
}

__device__ __forceinline__ float level_terms(int node, float val, float qx, float qy, float qz, int depth,
                                             const int* neigh, size_t stride, const int* enc, const float* x) {
    const int e = enc[node];
    int nbs[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) nbs[k] = neigh[(size_t)k * stride + node];
    // every value read at once (a missing neighbour reads entry 0 and adds nothing)
    float xv[27];
#pragma unroll
    for (int k = 0; k < 27; ++k) xv[k] = x[nbs[k] >= 0 ? nbs[k] : 0];
    return terms_from(e, nbs, xv, val, qx, qy, qz, depth);
}

// ---- Bernstein form of the implicit function on a cell --------------------------------
// On a cell inside one cell of level l, every level-l translate b((x - c) 2^l) is a single
// quadratic piece; with s in [-1, 1] across the cell (half width h) it is
// q(s) = b + g s + k/2 s^2 (b, g = h b', k = h^2 b'' at the cell centre), whose Bernstein
// coefficients are b - g + k/2, b - k/2, b + g + k/2.  A sum of tensor-product translates
// is then a tensor-product quadratic given by its 27 Bernstein coefficients.
// Bernstein coefficients on the cell of the translate `idx` (hs = h 2^l: half width in
// level widths; x the cell centre)
__device__ __forceinline__ void basis_bernstein(int idx, float x, float hs, float (&q)[3]) {
    const int l = ilog2_dev(idx + 1);
    const int off = idx + 1 - (1 << l);
    const float c = __fmul_rn(__fadd_rn((float)off, 0.5f), __int_as_float((127 - l) << 23));
    const float t = __fmul_rn(__fsub_rn(x, c), (float)(1 << l));
    const float a = fabsf(t);
    float b, g, k2;
    if (a < 0.5f) {
        b = (0.75f - t * t) * (4.0f / 3.0f);
        g = -(8.0f / 3.0f) * t * hs;
        k2 = -(4.0f / 3.0f) * hs * hs;
    } else if (a < 1.5f) {
        const float u = 1.5f - a;
        b = u * u * (2.0f / 3.0f);
        g = copysignf((4.0f / 3.0f) * u * hs, -t);
        k2 = (2.0f / 3.0f) * hs * hs;
    } else {
        b = 0.0f;
        g = 0.0f;
        k2 = 0.0f;
    }
    q[0] = b - g + k2;
    q[1] = b - k2;
    q[2] = b + g + k2;
}

// adds one level (ancestor function indices ox, oy, oz; its 27 values y) to the cell's
// Bernstein coefficients C[alpha][beta][gamma] (x, y, z), separably
__device__ __forceinline__ void sign_level(const float (&y)[27], int ox, int oy, int oz, float qx, float qy,
                                           float qz, float hs, float (&C)[27], float& mag) {
    float X[3][3], Y[3][3], Z[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        basis_bernstein(ox - 1 + j, qx, hs, X[j]);
        basis_bernstein(oy - 1 + j, qy, hs, Y[j]);
        basis_bernstein(oz - 1 + j, qz, hs, Z[j]);
    }
    float ab = 0.0f;
#pragma unroll
    for (int k = 0; k < 27; ++k) ab += fabsf(y[k]);
    mag += ab;
    // T1[a][j][k] = sum_i X[i][a] y[i][j][k]
    float T1[27];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int jk = 0; jk < 9; ++jk)
            T1[a * 9 + jk] = fmaf(X[0][a], y[jk], fmaf(X[1][a], y[9 + jk], X[2][a] * y[18 + jk]));
    // T2[a][b][k] = sum_j Y[j][b] T1[a][j][k]
    float T2[27];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int bb = 0; bb < 3; ++bb)
#pragma unroll
            for (int k = 0; k < 3; ++k)
                T2[a * 9 + bb * 3 + k] = fmaf(Y[0][bb], T1[a * 9 + k],
                                              fmaf(Y[1][bb], T1[a * 9 + 3 + k], Y[2][bb] * T1[a * 9 + 6 + k]));
    // C[a][b][g] += sum_k Z[k][g] T2[a][b][k]
#pragma unroll
    for (int ab3 = 0; ab3 < 9; ++ab3)
#pragma unroll
        for (int gg = 0; gg < 3; ++gg)
            C[ab3 * 3 + gg] += fmaf(Z[0][gg], T2[ab3 * 3], fmaf(Z[1][gg], T2[ab3 * 3 + 1], Z[2][gg] * T2[ab3 * 3 + 2]));
}

// ---- float-float ("double-float") accumulation ---------------------------------------
// GB300 executes FP64 at a small fraction of its FP32 rate, so sums that need more than
// FP32 precision are carried as an unevaluated pair hi + lo of floats (|lo| <= ulp(hi)/2):
// Knuth's TwoSum for the error of an addition, Dekker's FastTwoSum to renormalise, and
// the fused multiply-add for the exact error of a product (Dekker's TwoProduct).
// About 44 significant bits; the order of operations is fixed, so sums are deterministic.
struct FF {
    float hi, lo;
};

__device__ __forceinline__ FF ff_zero() { return FF{0.0f, 0.0f}; }

__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bv = __fsub_rn(s, a.hi);
    const float av = __fsub_rn(s, bv);
    float e = __fadd_rn(__fsub_rn(a.hi, av), __fsub_rn(b.hi, bv));   // a.hi + b.hi = s + e exactly
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, e);
    return FF{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ FF ff_add_float(FF a, float b) { return ff_add(a, FF{b, 0.0f}); }

// exact product of two floats as a float pair
__device__ __forceinline__ FF ff_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return FF{p, fmaf(a, b, -p)};
}

__device__ __forceinline__ FF ff_shfl_xor(FF v, int o) {
    return FF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// warp-wide sum (butterfly; every lane ends with the same value)
__device__ __forceinline__ FF ff_warp_sum(FF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_xor(v, o));
    return v;
}

__device__ __forceinline__ float ff_to_float(FF a) { return __fadd_rn(a.hi, a.lo); }

// the pair as one FP64 value (hi and lo are floats, so each converts exactly)
__device__ __forceinline__ double ff_to_double(FF a) { return (double)a.hi + (double)a.lo; }

// FP64 warp-wide sum (butterfly; IEEE addition is commutative, so every lane ends with the
// same value, in a fixed order)
__device__ __forceinline__ double dbl_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// a / b rounded to float: float quotient of the leading parts, then one correction step
// with the remainder a - q b evaluated with fused multiply-adds
__device__ __forceinline__ float ff_div(FF a, FF b) {
    const float q = __fdiv_rn(a.hi, b.hi);
    float r = fmaf(-q, b.hi, a.hi);   // exact: a.hi - q * b.hi
    r = __fadd_rn(r, a.lo);
    r = fmaf(-q, b.lo, r);
    return __fadd_rn(q, __fdiv_rn(r, b.hi));
}

#endif  // __CUDACC__

// Iteration limit of every device-side wait; exceeding it sets kErrSpinTimeout.
constexpr int kSpinLimit = 1 << 22;

}  // namespace psr
