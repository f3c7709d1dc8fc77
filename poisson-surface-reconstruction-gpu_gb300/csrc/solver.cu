// Stage (c): per-depth Laplacian conjugate gradients and the iso-value.
//
// System of depth d (mesh/solver/LaplacianSolver.cu:27-74,120-267): rows are the nodes of
// depth d, columns their same-depth neighbours, entry ff_x ff_y ff_z (d2_x + d2_y + d2_z)
// stored in FP32 and dropped when |value| <= 1e-6.  Same-depth entries depend only on
// the neighbour offset, so the operator is applied matrix-free from a 27-entry stencil
// per depth and the neighbour table.  Right-hand side: the divergence of the depth.
//
// CG (mesh/solver/CGAlgorithm.cu:10-80): x0 = 0, r0 = b, stops when r.r <= tol^2 or after
// max_iter iterations (or after a fixed count).  All depths are independent; they are
// solved together in concurrent launches of thread-block clusters (see k_cg_cluster).
// Precision: the operator, the vectors and the updates are FP32; the dot products and
// residual norms are FP64 quantities (exact products, double-float sums within a warp, FP64
// sums across warps and CTAs, in a fixed order).  Every res_period iterations and when the
// recursive residual reaches the tolerance, the true residual b - A x of the current x is
// evaluated (exact products, double-float sums, FP64 norm); it drives iterative refinement:
// the CG restarts from it when it is above both the tolerance and the floor an FP32
// solution can reach (2^-20 ||b||) and the recursive residual has converged or drifted.
//
// Iso-value (:269-305): mean of the implicit function at the sample points, evaluated in
// FP32 per point and averaged in FP64.
#include <cooperative_groups.h>
#include <vector>
#include "workspace.h"
#include "tables.cuh"

PSR_DEFINE_CONST_TABLES(upload_tables_solver)

namespace cg = cooperative_groups;

namespace psr {

// ---- per-depth CG ---------------------------------------------------------------------
// Every depth is an independent system.  The two finest depths (most rows, most
// iterations) get one thread-block cluster each (k_cg_cluster: cluster barriers, sums
// through distributed shared memory); the coarser depths get one CTA each (k_cg_cta,
// launched concurrently on a second stream).  Both run the same solver body: a cluster
// of one CTA is a CTA.
//
// Reductions: every product enters exactly (fma: TwoProduct) into a per-thread float pair,
// warp butterflies sum the pairs (FF arithmetic on the FP32 pipes), one warp per CTA sums
// the 32 warp partials in FP64 and writes the CTA's sum to its shared memory, and after
// the barrier one warp of every CTA sums the CTAs' values in FP64 in a fixed order, so
// every CTA holds the same result.  GB300 executes FP64 at a small fraction of its FP32
// rate (an FP64 add per element cost 2.4 us per reduction against 0.3 us for the
// cluster barrier), so FP64 arithmetic is kept to the 32 + 16 values of the cross-warp
// and cross-CTA steps; the in-warp pairs carry about 44 bits, more than the reference's
// float-rounded products summed in double (mesh/solver/CGAlgorithm.cu:106-133).  The
// scalars of an iteration (alpha, beta, the continue flag) are computed once, by the
// thread that finishes the sum, and read by every thread from shared memory.  The
// partial buffers alternate between two slots, so a slot is only rewritten after a
// barrier that follows its reads.
//
// True residual (iterative refinement): every res_period iterations, and when the
// recursive r.r reaches tol^2, each row's b - sum_k st_k x[nb_k] is evaluated with exact
// products and float-pair sums (staged in the A p buffer) and its FP64 norm is taken.  With
// the reference's absolute tolerance (1e-5) and right-hand sides of norm ~1e7, the FP32
// recursion ends with a true residual near 1e-7 ||b||, below what an FP32 x can resolve
// (2^-20 ||b||, 16 ulps of b); refinement restarts the CG from the true residual only
// above that floor (and the tolerance), when the recursive residual has converged or has
// drifted below the true one by more than 2x in norm, at most kCgMaxRefine times and while
// each restart cuts the true r.r fourfold.  Replacing r periodically while keeping the
// direction was tried and fails at this scale: beta = r_true.r_true / r_old.r_old mixes a
// true residual at the FP32 floor with a recursive one far below it and the iteration
// stalls (it ran to the 10,000-iteration cap on the depth-3 system of the superquadric).
//
// One iteration costs two barriers: the direction update p = r + beta p is fused into the
// operator application (a row's neighbours rebuild their p values from r and the
// previous p), so the FP32 operations per element are the textbook loop's:
//   p_k = fma(beta, p_{k-1}, r_k)   Ap = sum_k st_k p_k[nb]   alpha = rr / (p.Ap)
//   x = fma(alpha, p, x)            r = fma(-alpha, Ap, r)    beta = rr_new / rr
// Missing neighbours contribute fma(st_k, 0, y) = y, the same as skipping them.
//
// Resident path (depth >= 1 and at most kCgSmemRows rows per CTA): each CTA owns a
// contiguous, sibling-group aligned chunk of rows and keeps (r_k, p_{k-1}) in shared
// memory (two buffers alternating per iteration), plus A p and x.  The operator is
// applied per sibling group: the 8 children of one parent have all their 27-neighbours
// inside one 4x4x4 block of same-depth nodes, listed once per group in the block table
// (k_cg_blocks).  Each lane of a warp (4 groups of 8 siblings) fetches 8 block entries
// (local shared memory or a remote CTA's through distributed shared memory), the group's
// 64 p values go to a per-warp shared block, and each lane applies its 27-point stencil
// from there.  Otherwise (the root, or more rows than fit) the vectors live in global
// memory and the neighbour table is read row by row.
constexpr int kCgcBlock = 1024;
constexpr int kCgWarps = kCgcBlock / 32;
constexpr int kCgSmemRows = 7168;
constexpr size_t kCgRowBytes = 2 * sizeof(float2) + 2 * sizeof(float);   // r/p x2, A p, x
// per-warp shared block of 4 sibling groups: group gi at gi * 80 + {0, 18, 8, 26}[gi]
// floats, so the 4 groups start in banks 0, 2, 8, 10 and the 32 lanes' stencil reads (at
// sibling offsets {0,1,4,5,16,17,20,21} + a common neighbour offset) hit 32 distinct banks
constexpr int kCgWarpBlockFloats = 352;
constexpr size_t kCgBlockBytes = (size_t)kCgWarps * kCgWarpBlockFloats * sizeof(float);
constexpr size_t kCgSmemBytes = (size_t)kCgSmemRows * kCgRowBytes + kCgBlockBytes;
static_assert(kCgSmemRows % 32 == 0, "whole warp slots");

constexpr int kCgMaxRefine = 4;

// Workspace pointers of the CG; a multi-cloud launch moves them to the CTA's cloud (a
// copy in registers: the launch parameters below stay where the launch put them).
struct CgcVec {
    const Counters* c;
    Counters* cw;
    const int* neigh;
    const int* blk;     // block table: 64 entries per sibling group of depth >= 1
    const float* stencil;
    const float* b;
    float* x;
    float* r;
    float* pa;
    float* pb;
    float* ap;
    __device__ void rebase() { PSR_CLOUD(c, cw, neigh, blk, stencil, b, x, r, pa, pb, ap); }
};

// a workspace pointer of cloud 0 moved to cloud k (null stays null)
template <class T>
__device__ __forceinline__ T* at_cloud(T* p, int k) {
    return p ? (T*)((const char*)p + (unsigned long long)k * kCloudStride) : p;
}

struct CgcArgs {
    CgcVec v;
    int depth;
    int first;          // depth of cluster / CTA 0; unit u solves depth first - u
    size_t stride;
    float tol2;
    int max_iter;
    int res_period;     // > 0: true residual every res_period iterations; 0: only at
                        // convergence; < 0: never (the recursive residual alone)
    unsigned loop_mask; // depths the device loop solves when they do not fit the cluster
    float stp[3][27];   // stencils of units 0..2 of k_cg_cluster (depth first - u)
};

// The resident path holds a depth when its cluster's chunk of rows fits a CTA's shared
// memory (the last row is the zero row); the root never does.
__device__ __forceinline__ int cg_chunk(int m, int nblk) { return ((m + nblk - 1) / nblk + 7) & ~7; }
__device__ __forceinline__ bool cg_fits_resident(int d, int m, int nblk) {
    return d >= 1 && cg_chunk(m, nblk) < kCgSmemRows;
}

struct CgcShared {
    FF warp[kCgWarps];
    double slot[2];
    double rr;          // r.r of the recursive residual (FP64)
    double rr_prev;     // the same one iteration earlier
    double pap;
    double floor2;      // (2^-20 ||b||)^2: what the true residual of an FP32 solution can reach
    double rr_true;     // r.r of the last true residual (-1: none yet)
    float alpha, beta;
    int go;             // the iteration continues
    int check;          // the true residual is due
    int replace;        // the true residual replaces r (a refinement restart)
    int checks;         // true-residual evaluations
    int restarts;       // refinement restarts
    float st[27];
};
static_assert(kCgWarps == 32, "one FP64 lane per warp partial");
static_assert(kCgSmemBytes + sizeof(CgcShared) <= 227 * 1024, "shared memory of one CTA");

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Sum of every thread's `v` over the cluster (FP64).  Thread 0 hands the sum to `post`,
// which sets the shared scalars the next step reads; every thread sees them when this
// returns.  Contains the cluster barrier; identical in every CTA.
template <class Post>
__device__ __forceinline__ void cgc_allreduce(cg::cluster_group& cl, CgcShared& sh, int& buf, FF v, Post post) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = ff_warp_sum(v);
    if (lane == 0) sh.warp[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const double w = dbl_warp_sum(ff_to_double(sh.warp[lane]));
        if (lane == 0) sh.slot[buf] = w;
    }
    cl.sync();
    if (warp == 0) {
        const unsigned nb = cl.num_blocks();
        double w = 0.0;
        if ((unsigned)lane < nb) w = *cl.map_shared_rank(&sh.slot[buf], (unsigned)lane);
        w = dbl_warp_sum(w);
        if (lane == 0) post(w);
    }
    buf ^= 1;
    __syncthreads();
}

// After the r.r reduction of an iteration (thread 0): beta, the continue flag and whether
// the true residual is due.  `it` is the iteration just completed.
// The step scalars are quotients of the FP64 sums rounded to float and divided in FP32 (within
// 1.5 ulp of the FP64 quotient rounded to float): an FP64 division on the one thread that
// finishes the sums sits on every iteration's critical path, and GB300 divides in FP64
// slowly.
__device__ __forceinline__ float cg_quot(double num, double den) {
    return den != 0.0 ? __fdiv_rn((float)num, (float)den) : 0.0f;
}

template <class St, class Ar>
__device__ __forceinline__ void cg_after_rr(St& sh, const Ar& a, double w, int it) {
    sh.beta = cg_quot(w, sh.rr);
    sh.rr_prev = sh.rr;
    sh.rr = w;
    const bool conv = !((float)w > a.tol2);   // the reference compares a float r.r (CGAlgorithm.cu:36)
    const bool more = sh.pap != 0.0 && it + 1 <= a.max_iter;
    sh.go = !conv && more;
    sh.check = a.res_period >= 0 && sh.pap != 0.0 &&
               (conv || (a.res_period > 0 && it % a.res_period == 0 && more));
}

// After the true-residual reduction (thread 0).  The CG restarts from the true residual
// (beta = 0: one cycle of iterative refinement) when that residual is above both the
// tolerance and the floor an FP32 solution can reach, and either the recursive residual
// has converged or has drifted more than 2x (in norm) below the true one; at most
// kCgMaxRefine restarts, each one reducing the true r.r at least fourfold.  `it` is the
// next iteration's number.
template <class St, class Ar>
__device__ __forceinline__ void cg_after_true(St& sh, const Ar& a, double w, int it) {
    ++sh.checks;
    const double target = fmax((double)a.tol2, sh.floor2);
    const bool drift = w > 4.0 * fmax(sh.rr, sh.floor2);
    const bool falling = sh.rr_true < 0.0 || w < 0.25 * sh.rr_true;
    sh.replace = w > target && (!sh.go || drift) && sh.restarts < kCgMaxRefine && it <= a.max_iter && falling;
    if (sh.replace) {
        ++sh.restarts;
        sh.beta = 0.0f;
        sh.go = 1;
        sh.rr = w;
    }
    sh.rr_true = w;
}

// Start of a solve (thread 0): r0 = b, so r.r is also ||b||^2.
template <class St, class Ar>
__device__ __forceinline__ void cg_start(St& sh, const Ar& a, double w) {
    sh.rr = w;
    sh.beta = 0.0f;
    sh.go = ((float)w > a.tol2) && a.max_iter >= 1;
    sh.floor2 = w * 0x1p-40;
    sh.rr_true = -1.0;
    sh.checks = 0;
    sh.restarts = 0;
    sh.replace = 0;
}

// Per-depth results of a finished solve (thread 0 of cluster CTA 0).
template <class St>
__device__ __forceinline__ void cg_report(const CgcVec& v, int d, const St& sh) {
    v.cw->cg_rr[d] = sh.rr;
    v.cw->cg_rr_true[d] = sh.rr_true;
    v.cw->cg_checks[d] = sh.checks;
    v.cw->cg_restarts[d] = sh.restarts;
}

// position of neighbour k (9 ox + 3 oy + oz) of sibling s (x = 4, y = 2, z = 1) in the
// group's 4x4x4 block (16 bx + 4 by + bz)
__host__ __device__ constexpr int cg_kpos(int k) { return 16 * (k / 9) + 4 * ((k / 3) % 3) + (k % 3); }
__device__ __forceinline__ int cg_spos(int s) { return 16 * ((s >> 2) & 1) + 4 * ((s >> 1) & 1) + (s & 1); }

// Block table of every sibling group (depth >= 1; group G = rows 1 + 8G .. 8 + 8G):
// block position (bx, by, bz) holds neighbour (ox, oy, oz) of sibling (cx, cy, cz) with
// b = c + o, taking c = 1 on an axis where b >= 2, else 0.  Stored transposed: table
// entry j of a group is position (j & 7) * 8 + (j >> 3), so lane s of a group reads its
// 8 positions s, s + 8, ... as two contiguous int4.
__global__ void __launch_bounds__(kBlock) k_cg_blocks(const Counters* c, const int* neigh, size_t stride,
                                                      int* blk) {
    PSR_CLOUD(c, neigh, blk);
    const int ngroups = (c->n_nodes - 1) >> 3;
    PSR_GRID_STRIDE(t, ngroups * 64) {
        const int G = t >> 6, j = t & 63;
        const int pos = ((j & 7) << 3) | (j >> 3);
        const int bx = pos >> 4, by = (pos >> 2) & 3, bz = pos & 3;
        const int cx = bx >= 2, cy = by >= 2, cz = bz >= 2;
        const int k = 9 * (bx - cx) + 3 * (by - cy) + (bz - cz);
        const int sib = 4 * cx + 2 * cy + cz;
        blk[t] = neigh[(size_t)k * stride + 1 + 8 * G + sib];
    }
}

struct CgUnit {
    int d, row0, row1;
};

// (r, p) pair at byte offset `off` of the `cur` buffer of cluster CTA `rank`: the shared
// address of this CTA's buffer mapped into that CTA's window (mapa), then one
// distributed-shared-memory load
__device__ __forceinline__ float2 cg_ld_pair(unsigned cur_sa, unsigned desc) {
    unsigned ra;
    float2 v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(cur_sa + (desc & 0xffffffu)), "r"(desc >> 24));
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(ra));
    return v;
}
constexpr int kCgZeroRow = kCgSmemRows - 1;   // kept (0, 0) in both buffers: absent neighbours

// x of the row whose (r, p) pair a descriptor addresses: the x array holds one float per
// row, so the row's byte offset in the pair buffer halves
__device__ __forceinline__ float cg_ld_x(unsigned x_sa, unsigned desc) {
    unsigned ra;
    float v;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(x_sa + ((desc & 0xffffffu) >> 1)), "r"(desc >> 24));
    asm volatile("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(ra));
    return v;
}

// Resident path.  CTA k of the cluster owns rows [row0 + k*chunk, row0 + (k+1)*chunk).
// U >= 0: the cluster unit whose stencil is a launch parameter (a.stp[U]), read as a
// constant operand of the FMAs; U < 0: the stencil staged in shared memory.
template <int U>
__device__ __forceinline__ void cgc_resident(cg::cluster_group& cl, CgcShared& sh, const CgcArgs& a,
                                             const CgcVec& v, const CgUnit& u, int chunk, float2* rp0, float2* rp1, float* sap,
                                             float* sx, float* sblk) {
    const unsigned me = cl.block_rank();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int m = u.row1 - u.row0;
    const int mlo = u.row0 + (int)me * chunk;
    const int nloc = max(0, min(chunk, m - (int)me * chunk));
    const int nslot = (nloc + 31) >> 5;
    const int gi = lane >> 3, sib = lane & 7;
    const int spos = cg_spos(sib);
    float* myblk = sblk + warp * kCgWarpBlockFloats + gi * 80 + ((0x1a081200 >> (gi * 8)) & 0xff);
    const int gbase = (mlo - 1) >> 3;   // block-table group of local row 0
    // g / chunk = umulhi(g, ceil(2^32 / chunk)): exact while g * (magic * chunk - 2^32) < 2^32,
    // true here (g < 2^17 rows, chunk <= kCgSmemRows)
    const unsigned chunk_magic = chunk > 0 ? (unsigned)((0x100000000ull + (unsigned)chunk - 1) / (unsigned)chunk) : 0u;
    // The block table of this CTA's groups becomes descriptors, once: (CTA rank << 24) |
    // byte offset of the row inside that CTA's buffer (the zero row for an absent cell), so
    // an iteration reads a neighbour with one mapped load instead of locating its owner.
    // Only this CTA reads these groups' entries; the barrier below publishes them.
    int* blkw = const_cast<int*>(v.blk);
    for (int t = threadIdx.x; t < nloc * 8; t += kCgcBlock) {
        const size_t at = (size_t)gbase * 64 + t;
        const int nb = blkw[at];
        const int gl = nb - mlo;
        const int g = nb - u.row0;
        unsigned desc = (me << 24) | (unsigned)(kCgZeroRow * 8);
        if ((unsigned)gl < (unsigned)nloc) {
            desc = (me << 24) | (unsigned)(gl * 8);
        } else if (nb >= 0 && (unsigned)g < (unsigned)m) {
            const int owner = (int)__umulhi((unsigned)g, chunk_magic);   // g / chunk
            desc = ((unsigned)owner << 24) | (unsigned)((g - owner * chunk) * 8);
        }
        blkw[at] = (int)desc;
    }
    if (threadIdx.x == 0) {
        rp0[kCgZeroRow] = make_float2(0.0f, 0.0f);
        rp1[kCgZeroRow] = make_float2(0.0f, 0.0f);
        sx[kCgZeroRow] = 0.0f;
    }
    // r0 = b, p_{-1} = 0, x0 = 0
    FF acc = ff_zero();
    for (int l = threadIdx.x; l < nloc; l += kCgcBlock) {
        const float bi = v.b[mlo + l];
        rp0[l] = make_float2(bi, 0.0f);
        sx[l] = 0.0f;
        acc = ff_add(acc, ff_prod(bi, bi));
    }
    int buf = 0;
    cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_start(sh, a, w); });
    bool ran = false;
    float2* cur = rp0;
    float2* nxt = rp1;
    int it = 1;
    while (sh.go) {
        const float beta = sh.beta;
        // (A) own p_k, A p_k from the neighbours' (r_k, p_{k-1}), p.Ap
        acc = ff_zero();
        // the block-table entries of the warp's next slot are loaded while the current
        // slot is processed (they do not change between iterations)
        int4 q0 = make_int4(-1, -1, -1, -1), q1 = q0;
        if (warp < nslot && warp * 32 + lane < nloc) {
            const int4* bp = reinterpret_cast<const int4*>(v.blk + (size_t)(gbase + ((warp * 32 + lane) >> 3)) * 64 + sib * 8);
            q0 = bp[0];
            q1 = bp[1];
        }
        const unsigned cur_sa = (unsigned)__cvta_generic_to_shared(cur);
        for (int sl = warp; sl < nslot; sl += kCgWarps) {
            const int l = sl * 32 + lane;
            const bool mine = l < nloc;   // whole groups: a group is all in or all out
            const int ids[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
            const int ln = l + kCgWarps * 32;
            if (ln < nloc) {
                const int4* bp = reinterpret_cast<const int4*>(v.blk + (size_t)(gbase + (ln >> 3)) * 64 + sib * 8);
                q0 = bp[0];
                q1 = bp[1];
            }
            if (mine) {
                // 8 independent mapped loads (own buffer, a peer's, or the zero row)
                float2 vals[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) vals[e] = cg_ld_pair(cur_sa, (unsigned)ids[e]);
#pragma unroll
                for (int e = 0; e < 8; ++e) myblk[e * 8 + sib] = fmaf(beta, vals[e].y, vals[e].x);
            }
            __syncwarp();
            if (mine) {
                float y = 0.0f;
#pragma unroll
                for (int k = 0; k < 27; ++k) y = fmaf(U >= 0 ? a.stp[U < 0 ? 0 : U][k] : sh.st[k], myblk[spos + cg_kpos(k)], y);
                const float2 own = cur[l];
                const float pi = fmaf(beta, own.y, own.x);
                nxt[l].y = pi;
                sap[l] = y;
                acc = ff_add(acc, ff_prod(pi, y));
            }
            __syncwarp();
        }
        cgc_allreduce(cl, sh, buf, acc, [&](double w) {
            sh.pap = w;
            sh.alpha = cg_quot(sh.rr, w);
        });
        const float alpha = sh.alpha;
        // (B) x and r, r.r
        acc = ff_zero();
        for (int sl = warp; sl < nslot; sl += kCgWarps) {
            const int l = sl * 32 + lane;
            if (l < nloc) {
                const float pi = nxt[l].y;
                sx[l] = fmaf(alpha, pi, sx[l]);
                const float ri = fmaf(-alpha, sap[l], cur[l].x);
                nxt[l].x = ri;
                acc = ff_add(acc, ff_prod(ri, ri));
            }
        }
        cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_after_rr(sh, a, w, it); });
        ran = true;
        if (me == 0 && threadIdx.x == 0) v.cw->cg_iters[u.d] = it;
        float2* t = cur;
        cur = nxt;
        nxt = t;
        ++it;
        if (sh.check) {
            // (C) true residual b - A x of the current x from the neighbours' x (the barrier
            // of the last reduction published every CTA's x), with exact products and
            // float-pair sums; staged in the A p buffer, which holds nothing live here
            acc = ff_zero();
            const unsigned x_sa = (unsigned)__cvta_generic_to_shared(sx);
            for (int sl = warp; sl < nslot; sl += kCgWarps) {
                const int l = sl * 32 + lane;
                const bool mine = l < nloc;
                if (mine) {
                    const int4* bp = reinterpret_cast<const int4*>(v.blk + (size_t)(gbase + (l >> 3)) * 64 + sib * 8);
                    const int4 d0 = bp[0], d1 = bp[1];
                    const int ids[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
                    float vals[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) vals[e] = cg_ld_x(x_sa, (unsigned)ids[e]);
#pragma unroll
                    for (int e = 0; e < 8; ++e) myblk[e * 8 + sib] = vals[e];
                }
                __syncwarp();
                if (mine) {
                    FF y = ff_zero();
#pragma unroll
                    for (int k = 0; k < 27; ++k)
                        y = ff_add(y, ff_prod(U >= 0 ? a.stp[U < 0 ? 0 : U][k] : sh.st[k], myblk[spos + cg_kpos(k)]));
                    const float ri = ff_to_float(ff_add(FF{v.b[mlo + l], 0.0f}, FF{-y.hi, -y.lo}));
                    sap[l] = ri;
                    acc = ff_add(acc, ff_prod(ri, ri));
                }
                __syncwarp();
            }
            cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_after_true(sh, a, w, it); });
            if (sh.replace) {   // refinement restart: CG continues from the true residual
                for (int l = threadIdx.x; l < nloc; l += kCgcBlock) cur[l].x = sap[l];
                cl.sync();      // before any CTA reads a neighbour's new r
            }
        }
    }
    for (int l = threadIdx.x; l < nloc; l += kCgcBlock) {
        v.x[mlo + l] = sx[l];
        v.r[mlo + l] = cur[l].x;
    }
    if (ran && me == 0 && threadIdx.x == 0) cg_report(v, u.d, sh);
}

// Global-memory path (any size, any depth).
__device__ __forceinline__ void cgc_global(cg::cluster_group& cl, CgcShared& sh, const CgcArgs& a,
                                           const CgcVec& v, const CgUnit& u) {
    const int tid = cl.block_rank() * blockDim.x + threadIdx.x;
    const int nthr = cl.num_blocks() * blockDim.x;
    FF acc = ff_zero();
    for (int i = u.row0 + tid; i < u.row1; i += nthr) {
        const float bi = v.b[i];
        v.r[i] = bi;
        v.pa[i] = 0.0f;
        v.x[i] = 0.0f;
        acc = ff_add(acc, ff_prod(bi, bi));
    }
    int buf = 0;
    cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_start(sh, a, w); });
    bool ran = false;
    const float* pprev = v.pa;
    float* pcur = v.pb;
    int it = 1;
    while (sh.go) {
        const float beta = sh.beta;
        acc = ff_zero();
        for (int i = u.row0 + tid; i < u.row1; i += nthr) {
            const float pi = fmaf(beta, pprev[i], v.r[i]);
            float y = 0.0f;
#pragma unroll 9
            for (int k = 0; k < 27; ++k) {
                const int nb = __ldg(&v.neigh[(size_t)k * a.stride + i]);
                if (nb >= 0) y = fmaf(sh.st[k], fmaf(beta, pprev[nb], v.r[nb]), y);
            }
            pcur[i] = pi;
            v.ap[i] = y;
            acc = ff_add(acc, ff_prod(pi, y));
        }
        cgc_allreduce(cl, sh, buf, acc, [&](double w) {
            sh.pap = w;
            sh.alpha = cg_quot(sh.rr, w);
        });
        const float alpha = sh.alpha;
        acc = ff_zero();
        for (int i = u.row0 + tid; i < u.row1; i += nthr) {
            v.x[i] = fmaf(alpha, pcur[i], v.x[i]);
            const float ri = fmaf(-alpha, v.ap[i], v.r[i]);
            v.r[i] = ri;
            acc = ff_add(acc, ff_prod(ri, ri));
        }
        cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_after_rr(sh, a, w, it); });
        ran = true;
        if (cl.block_rank() == 0 && threadIdx.x == 0) v.cw->cg_iters[u.d] = it;
        float* t = const_cast<float*>(pprev);
        pprev = pcur;
        pcur = t;
        ++it;
        if (sh.check) {
            // true residual r = b - A x (the barrier of the last reduction published x)
            acc = ff_zero();
            for (int i = u.row0 + tid; i < u.row1; i += nthr) {
                FF y = ff_zero();
                for (int k = 0; k < 27; ++k) {
                    const int nb = __ldg(&v.neigh[(size_t)k * a.stride + i]);
                    if (nb >= 0) y = ff_add(y, ff_prod(sh.st[k], v.x[nb]));
                }
                const float ri = ff_to_float(ff_add(FF{v.b[i], 0.0f}, FF{-y.hi, -y.lo}));
                v.ap[i] = ri;   // staged; A p holds nothing live here
                acc = ff_add(acc, ff_prod(ri, ri));
            }
            cgc_allreduce(cl, sh, buf, acc, [&](double w) { cg_after_true(sh, a, w, it); });
            if (sh.replace) {   // refinement restart: CG continues from the true residual
                for (int i = u.row0 + tid; i < u.row1; i += nthr) v.r[i] = v.ap[i];
                cl.sync();
            }
        }
    }
    if (ran && cl.block_rank() == 0 && threadIdx.x == 0) cg_report(v, u.d, sh);
}

// one depth per cluster (a CTA when the launch has no cluster dimension); kClusterUnits:
// the unit's stencil is a launch parameter
template <bool kClusterUnits>
__device__ __forceinline__ void cg_unit_body(const CgcArgs& a, const CgcVec& v, int unit) {
    cg::cluster_group cl = cg::this_cluster();
    __shared__ CgcShared sh;
    extern __shared__ float4 cg_dyn[];
    const unsigned long long t_start = global_ns();
    CgUnit u;
    u.d = a.first - unit;
    u.row0 = v.c->level_base[u.d];
    u.row1 = (u.d < a.depth) ? v.c->level_base[u.d + 1] : v.c->n_nodes;
    if (threadIdx.x < 27) sh.st[threadIdx.x] = v.stencil[u.d * 27 + threadIdx.x];
    __syncthreads();
    const int nblk = (int)cl.num_blocks();
    const int m = u.row1 - u.row0;
    const int chunk = cg_chunk(m, nblk);   // sibling-group aligned
    const bool fits = cg_fits_resident(u.d, m, nblk);   // uniform over the cluster
    if (!fits && ((a.loop_mask >> u.d) & 1u)) return;    // the device loop solves this depth
    if (fits) {
        float2* rp0 = reinterpret_cast<float2*>(cg_dyn);
        float2* rp1 = rp0 + kCgSmemRows;
        float* sap = reinterpret_cast<float*>(rp1 + kCgSmemRows);
        float* sx = sap + kCgSmemRows;
        float* sblk = sx + kCgSmemRows;
        if (kClusterUnits && unit == 0) cgc_resident<0>(cl, sh, a, v, u, chunk, rp0, rp1, sap, sx, sblk);
        else if (kClusterUnits && unit == 1) cgc_resident<1>(cl, sh, a, v, u, chunk, rp0, rp1, sap, sx, sblk);
        else if (kClusterUnits && unit == 2) cgc_resident<2>(cl, sh, a, v, u, chunk, rp0, rp1, sap, sx, sblk);
        else cgc_resident<-1>(cl, sh, a, v, u, chunk, rp0, rp1, sap, sx, sblk);
    } else {
        cgc_global(cl, sh, a, v, u);
    }
    cl.sync();   // no CTA exits while others may still read its shared memory
    if (cl.block_rank() == 0 && threadIdx.x == 0) v.cw->cg_depth_ns[u.d] = global_ns() - t_start;
}

__global__ void __launch_bounds__(kCgcBlock) k_cg_cluster(CgcArgs a) {
    cg::cluster_group cl = cg::this_cluster();
    CgcVec v = a.v;
    v.rebase();
    cg_unit_body<true>(a, v, (int)(blockIdx.x / cl.num_blocks()));
}

__global__ void __launch_bounds__(kCgcBlock) k_cg_cta(CgcArgs a) {
    CgcVec v = a.v;
    v.rebase();
    cg_unit_body<false>(a, v, (int)blockIdx.x);
}

// ---- device-loop CG: the depths too large for a cluster's shared memory -----------------
// A depth whose cluster chunk does not fit shared memory (cg_fits_resident false) is solved
// by a loop of whole-GPU kernels inside a CUDA-graph while node.  Body, per pass: twice the
// true residual when it is due (k_cgl_true), p and A p with p.Ap (k_cgl_spmv), x and r with
// r.r (k_cgl_update); then one thread lists the (depth, cloud) units that go on and ends
// the loop when none does (k_cgl_control).  The iteration, the decisions after each
// reduction and the precision (exact products, float-pair sums in a thread and a warp, FP64
// across warps and blocks, in a fixed order) are the cluster solver's; the scalars live in
// a CgLoopState per depth.  Each unit's work is split over virtual blocks, one per
// kLoopRowsPerSplit rows, which the launch's blocks take in turn over the listed units, so
// the sums keep one order whatever the number of clouds, and units that are done cost
// nothing.  Every reduction
// ends in the last virtual block to finish (a ticket counter after a fence), which sums the
// virtual blocks' partials in order; every virtual block has read the state before it
// takes its ticket, so the last one may clear a flag the kernel acted on.  The loop ends
// after at most max_iter iterations per depth; no block waits on another.
// Operator: the block-table gathers of the resident path (8 per row: each lane of a warp
// loads its sibling group's 8 block entries, the group's 64 values go to a per-warp shared
// block, the 27-point stencil reads them there), from global memory.
constexpr int kLoopBlock = 256;
constexpr int kLoopWarps = kLoopBlock / 32;
constexpr int kLoopUnroll = 2;   // CG iterations per pass of the while node's body
static_assert(kLoopMaxBlocks >= 1, "partials per unit");

struct CgLoopArgs {
    CgcVec v;            // cloud 0's workspace
    CgLoopState* st;     // per depth (cloud 0)
    double* part;        // per depth: kLoopMaxBlocks partial sums (cloud 0)
    unsigned* ctl;       // CgLoopControl (cloud 0 only)
    int first;           // unit z solves depth first - z
    int units, clouds;
    int ctas[kMaxDepth + 1];   // CTAs of the cluster launch that owns each depth
    unsigned loop_mask;
    float tol2;
    int max_iter;
    int res_period;
};

// Loop control of a launch: body passes run so far, the units (cloud << 8 | z) the next
// pass works on, and the first virtual block of each (vstart[count]: their total).
struct CgLoopControl {
    unsigned passes;
    unsigned count;
    unsigned list[kMaxBatchClouds * (kMaxDepth + 1)];
    unsigned vstart[kMaxBatchClouds * (kMaxDepth + 1) + 1];
};
static_assert(sizeof(CgLoopControl) == sizeof(unsigned) * kLoopControlWords, "control block words");
constexpr int kLoopRowsPerSplit = 1024;   // rows per virtual block (below 2M rows)

// virtual blocks of a unit of m rows: one per kLoopRowsPerSplit rows, at most
// kLoopMaxBlocks (the sums' order depends on m alone)
__device__ __forceinline__ unsigned loop_split(int m) {
    const int v = (m + kLoopRowsPerSplit - 1) / kLoopRowsPerSplit;
    return (unsigned)(v < 1 ? 1 : (v > kLoopMaxBlocks ? kLoopMaxBlocks : v));
}

struct LoopUnit {
    int d, row0, m, bx, split;
    CgcVec v;
    CgLoopState* st;
    double* part;
};

// virtual block vb of the listed units: its unit (cloud's workspace) and index in the unit
__device__ __forceinline__ LoopUnit loop_unit(const CgLoopArgs& a, const CgLoopControl* ctl, int vb) {
    int lo = 0, hi = (int)ctl->count - 1;   // the unit i with vstart[i] <= vb < vstart[i + 1]
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((int)ctl->vstart[mid] <= vb) lo = mid;
        else hi = mid - 1;
    }
    const unsigned e = ctl->list[lo];
    const int k = (int)(e >> 8), z = (int)(e & 255u);
    LoopUnit u;
    u.bx = vb - (int)ctl->vstart[lo];
    u.split = (int)(ctl->vstart[lo + 1] - ctl->vstart[lo]);
    u.d = a.first - z;
    u.v = a.v;
    u.v.c = at_cloud(a.v.c, k); u.v.cw = at_cloud(a.v.cw, k); u.v.neigh = at_cloud(a.v.neigh, k);
    u.v.blk = at_cloud(a.v.blk, k); u.v.stencil = at_cloud(a.v.stencil, k); u.v.b = at_cloud(a.v.b, k);
    u.v.x = at_cloud(a.v.x, k); u.v.r = at_cloud(a.v.r, k); u.v.pa = at_cloud(a.v.pa, k);
    u.v.pb = at_cloud(a.v.pb, k); u.v.ap = at_cloud(a.v.ap, k);
    u.row0 = u.v.c->level_base[u.d];
    u.m = u.v.c->level_count[u.d];
    u.st = at_cloud(a.st, k) + u.d;
    u.part = at_cloud(a.part, k) + (size_t)u.d * kLoopMaxBlocks;
    return u;
}

// Sum of every thread's `v` over the unit's virtual blocks (FP64).  Returns true in the
// block that finishes the sum, with the sum in `w` of thread 0 (the ticket is back at zero).
__device__ __forceinline__ bool loop_reduce(FF v, const LoopUnit& u, double& w) {
    const int split = u.split;
    __shared__ double s_w[kLoopWarps];
    __shared__ int s_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = ff_warp_sum(v);
    if (lane == 0) s_w[warp] = ff_to_double(v);
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int k = 0; k < kLoopWarps; ++k) b += s_w[k];
        u.part[u.bx] = b;
        __threadfence();
        s_last = atomicAdd(&u.st->ticket, 1u) == (unsigned)split - 1;
    }
    __syncthreads();
    const bool last = s_last;
    if (last) {
        __threadfence();
        if (warp == 0) {
            double t = 0.0;
            for (int k = lane; k < split; k += 32) t += __ldcg(&u.part[k]);
            t = dbl_warp_sum(t);
            if (lane == 0) {
                w = t;
                u.st->ticket = 0u;
            }
        }
    }
    __syncthreads();   // s_w and s_last are reused by the next virtual block
    return last;
}

// One thread, before the loop: which depths of which clouds the loop solves (the others
// are marked inactive), listed for the first pass.
__global__ void k_cgl_plan(CgLoopArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    CgLoopControl* ctl = reinterpret_cast<CgLoopControl*>(a.ctl);
    unsigned n = 0;
    ctl->vstart[0] = 0u;
    for (int k = 0; k < a.clouds; ++k) {
        const Counters* c = at_cloud(a.v.c, k);
        CgLoopState* st = at_cloud(a.st, k);
        for (int z = 0; z < a.units; ++z) {
            const int d = a.first - z;
            const bool active = ((a.loop_mask >> d) & 1u) && !cg_fits_resident(d, c->level_count[d], a.ctas[d]);
            st[d].active = active;
            st[d].go = 0;
            st[d].check = 0;
            st[d].replace = 0;
            st[d].it = 0;
            if (active) {
                ctl->list[n] = ((unsigned)k << 8) | (unsigned)z;
                ctl->vstart[n + 1] = ctl->vstart[n] + loop_split(c->level_count[d]);
                ++n;
            }
        }
    }
    ctl->count = n;
    ctl->passes = 0u;
}

// r0 = b, p_{-1} = 0 (buffer pa), x0 = 0 for the listed depths
__global__ void __launch_bounds__(kLoopBlock) k_cgl_init(CgLoopArgs a) {
    const CgLoopControl* ctl = reinterpret_cast<const CgLoopControl*>(a.ctl);
    const int nv = (int)ctl->vstart[ctl->count];
    for (int vb = blockIdx.x; vb < nv; vb += gridDim.x) {
        const LoopUnit u = loop_unit(a, ctl, vb);
        FF acc = ff_zero();
        for (int i = u.bx * kLoopBlock + threadIdx.x; i < u.m; i += u.split * kLoopBlock) {
            const float bi = u.v.b[u.row0 + i];
            u.v.r[u.row0 + i] = bi;
            u.v.pa[u.row0 + i] = 0.0f;
            u.v.x[u.row0 + i] = 0.0f;
            acc = ff_add(acc, ff_prod(bi, bi));
        }
        double w = 0.0;
        if (loop_reduce(acc, u, w) && threadIdx.x == 0) {
            cg_start(*u.st, a, w);
            u.st->t0 = global_ns();
            u.st->t1 = u.st->t0;
        }
    }
}

// the sibling group's block-table entries of lane (l, sib)
__device__ __forceinline__ const int4* loop_blk(const LoopUnit& u, int l, int sib) {
    return reinterpret_cast<const int4*>(u.v.blk + (size_t)(((u.row0 - 1) >> 3) + (l >> 3)) * 64 + sib * 8);
}

// True residual b - A x when due (exact products, float-pair sums), staged in the direction
// buffer the next iteration writes, and the refinement decision.
__global__ void __launch_bounds__(kLoopBlock) k_cgl_true(CgLoopArgs a) {
    const CgLoopControl* ctl = reinterpret_cast<const CgLoopControl*>(a.ctl);
    __shared__ float s_st[27];
    __shared__ float sblk[kLoopWarps * kCgWarpBlockFloats];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gi = lane >> 3, sib = lane & 7;
    const int spos = cg_spos(sib);
    float* myblk = sblk + warp * kCgWarpBlockFloats + gi * 80 + ((0x1a081200 >> (gi * 8)) & 0xff);
    const int nv = (int)ctl->vstart[ctl->count];
    for (int vb = blockIdx.x; vb < nv; vb += gridDim.x) {
        const LoopUnit u = loop_unit(a, ctl, vb);
        if (!u.st->check) continue;   // uniform over the block
        const int next = u.st->it + 1;
        float* stage = (next & 1) ? u.v.pb : u.v.pa;
        if (threadIdx.x < 27) s_st[threadIdx.x] = u.v.stencil[u.d * 27 + threadIdx.x];
        __syncthreads();
        const int nslot = (u.m + 31) >> 5;
        FF acc = ff_zero();
        for (int sl = u.bx * kLoopWarps + warp; sl < nslot; sl += u.split * kLoopWarps) {
            const int l = sl * 32 + lane;
            const bool mine = l < u.m;   // whole groups: a group is all in or all out
            if (mine) {
                const int4* bp = loop_blk(u, l, sib);
                const int4 q0 = bp[0], q1 = bp[1];
                const int ids[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
                float vals[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) vals[e] = ids[e] >= 0 ? u.v.x[ids[e]] : 0.0f;
#pragma unroll
                for (int e = 0; e < 8; ++e) myblk[e * 8 + sib] = vals[e];
            }
            __syncwarp();
            if (mine) {
                FF y = ff_zero();
#pragma unroll
                for (int k = 0; k < 27; ++k) y = ff_add(y, ff_prod(s_st[k], myblk[spos + cg_kpos(k)]));
                const float ri = ff_to_float(ff_add(FF{u.v.b[u.row0 + l], 0.0f}, FF{-y.hi, -y.lo}));
                stage[u.row0 + l] = ri;
                acc = ff_add(acc, ff_prod(ri, ri));
            }
            __syncwarp();
        }
        double w = 0.0;
        if (loop_reduce(acc, u, w) && threadIdx.x == 0) {
            cg_after_true(*u.st, a, w, next);
            u.st->check = 0;
            u.st->t1 = global_ns();
        }
    }
}

// p_k = r + beta p_{k-1}, A p_k, p.Ap.  Iteration it = st->it + 1 takes p_{k-1} from pa when
// it is odd, from pb when it is even, and writes p_k to the other buffer.  After a
// refinement restart (beta = 0) r is the true residual staged in that other buffer: each row
// takes it into r, and p_k = fma(0, p_{k-1}, r) is that residual itself, so the rows that
// overwrite the staged values with their p_k write the values already there.
__global__ void __launch_bounds__(kLoopBlock) k_cgl_spmv(CgLoopArgs a) {
    const CgLoopControl* ctl = reinterpret_cast<const CgLoopControl*>(a.ctl);
    __shared__ float s_st[27];
    __shared__ float sblk[kLoopWarps * kCgWarpBlockFloats];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gi = lane >> 3, sib = lane & 7;
    const int spos = cg_spos(sib);
    float* myblk = sblk + warp * kCgWarpBlockFloats + gi * 80 + ((0x1a081200 >> (gi * 8)) & 0xff);
    const int nv = (int)ctl->vstart[ctl->count];
    for (int vb = blockIdx.x; vb < nv; vb += gridDim.x) {
        const LoopUnit u = loop_unit(a, ctl, vb);
        if (!u.st->go) continue;   // uniform over the block
        const int it = u.st->it + 1;
        const float beta = u.st->beta;
        const bool restart = u.st->replace != 0;
        const float* pprev = (it & 1) ? u.v.pa : u.v.pb;
        float* pcur = (it & 1) ? u.v.pb : u.v.pa;
        const float* rsrc = restart ? pcur : u.v.r;
        if (threadIdx.x < 27) s_st[threadIdx.x] = u.v.stencil[u.d * 27 + threadIdx.x];
        __syncthreads();
        const int nslot = (u.m + 31) >> 5;
        FF acc = ff_zero();
        for (int sl = u.bx * kLoopWarps + warp; sl < nslot; sl += u.split * kLoopWarps) {
            const int l = sl * 32 + lane;
            const bool mine = l < u.m;
            if (mine) {
                const int4* bp = loop_blk(u, l, sib);
                const int4 q0 = bp[0], q1 = bp[1];
                const int ids[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
                float vals[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) vals[e] = ids[e] >= 0 ? fmaf(beta, pprev[ids[e]], rsrc[ids[e]]) : 0.0f;
#pragma unroll
                for (int e = 0; e < 8; ++e) myblk[e * 8 + sib] = vals[e];
            }
            __syncwarp();
            if (mine) {
                float y = 0.0f;
#pragma unroll
                for (int k = 0; k < 27; ++k) y = fmaf(s_st[k], myblk[spos + cg_kpos(k)], y);
                const float pi = myblk[spos + cg_kpos(13)];   // the row itself
                if (restart) u.v.r[u.row0 + l] = pi;
                pcur[u.row0 + l] = pi;
                u.v.ap[u.row0 + l] = y;
                acc = ff_add(acc, ff_prod(pi, y));
            }
            __syncwarp();
        }
        double w = 0.0;
        if (loop_reduce(acc, u, w) && threadIdx.x == 0) {
            u.st->pap = w;
            u.st->alpha = cg_quot(u.st->rr, w);
            u.st->replace = 0;
        }
    }
}

// x = x + alpha p, r = r - alpha A p, r.r and the decisions after it
__global__ void __launch_bounds__(kLoopBlock) k_cgl_update(CgLoopArgs a) {
    const CgLoopControl* ctl = reinterpret_cast<const CgLoopControl*>(a.ctl);
    const int nv = (int)ctl->vstart[ctl->count];
    for (int vb = blockIdx.x; vb < nv; vb += gridDim.x) {
        const LoopUnit u = loop_unit(a, ctl, vb);
        if (!u.st->go) continue;   // uniform over the block
        const int it = u.st->it + 1;
        const float alpha = u.st->alpha;
        const float* pcur = (it & 1) ? u.v.pb : u.v.pa;
        FF acc = ff_zero();
        for (int i = u.bx * kLoopBlock + threadIdx.x; i < u.m; i += u.split * kLoopBlock) {
            const int row = u.row0 + i;
            u.v.x[row] = fmaf(alpha, pcur[row], u.v.x[row]);
            const float ri = fmaf(-alpha, u.v.ap[row], u.v.r[row]);
            u.v.r[row] = ri;
            acc = ff_add(acc, ff_prod(ri, ri));
        }
        double w = 0.0;
        if (loop_reduce(acc, u, w) && threadIdx.x == 0) {
            cg_after_rr(*u.st, a, w, it);
            u.st->it = it;
            u.st->t1 = global_ns();
            u.v.cw->cg_iters[u.d] = it;
        }
    }
}

// One thread, last in the body: lists the units with an iteration or a true residual
// pending for the next pass and continues the loop while there is one.  Whatever the states
// say, it stops after max_iter + kCgMaxRefine + 2 passes (each depth iterates at most
// max_iter times, at least once per pass while it goes on, and its checks ride on those
// passes plus one after the last iteration) and then marks every cloud's counters as timed
// out.
__global__ void k_cgl_control(CgLoopArgs a, cudaGraphConditionalHandle cond) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    CgLoopControl* ctl = reinterpret_cast<CgLoopControl*>(a.ctl);
    const unsigned n0 = ctl->count;
    unsigned n = 0;
    for (unsigned i = 0; i < n0; ++i) {   // in place: entry n <= i is written after i is read
        const unsigned e = ctl->list[i];
        const unsigned sp = ctl->vstart[i + 1] - ctl->vstart[i];
        const CgLoopState& q = at_cloud(a.st, (int)(e >> 8))[a.first - (int)(e & 255u)];
        if (q.go || q.check) {
            ctl->list[n] = e;
            ctl->vstart[n + 1] = ctl->vstart[n] + sp;
            ++n;
        }
    }
    const unsigned passes = ++ctl->passes;
    if (n > 0 && passes > (unsigned)a.max_iter + kCgMaxRefine + 2u) {
        n = 0;
        ctl->vstart[0] = 0u;
        for (int k = 0; k < a.clouds; ++k) atomicOr(&at_cloud(a.v.cw, k)->error, kErrSpinTimeout);
    }
    ctl->count = n;
    cudaGraphSetConditional(cond, n > 0 ? 1u : 0u);
}

// after the loop: the per-depth results the cluster solver reports (one thread per unit)
__global__ void k_cgl_finish(CgLoopArgs a) {
    if (threadIdx.x != 0) return;
    const int k = (int)blockIdx.y, d = a.first - (int)blockIdx.z;
    const CgLoopState& q = at_cloud(a.st, k)[d];
    if (!q.active) return;
    CgcVec v = a.v;
    v.cw = at_cloud(a.v.cw, k);
    if (q.it > 0) cg_report(v, d, q);
    v.cw->cg_depth_ns[d] = q.t1 - q.t0;
}

// ---- implicit function at the sample points and the iso-value ----------------------
__device__ __forceinline__ void decode3s(int e, int depth, int& ix, int& iy, int& iz) {
    const int o1 = 1 << (depth + 1);
    ix = e & (o1 - 1);
    iy = (e >> (depth + 1)) & (o1 - 1);
    iz = e >> (2 * (depth + 1));
}

// Implicit value at a sample point: the 27 neighbour terms ((x * Fx) * Fy) * Fz of every
// level of its chain (its depth-D node and that node's ancestors).  The levels up to D-1
// are summed first, as soon as their systems are solved, beside the depth-D CG: on the cell
// of a depth-(D-1) node they form one tensor-product quadratic (k_point_poly: its 27
// Bernstein coefficients, one thread per node), evaluated at each sample of the cell
// (k_point_values_coarse; the partial sum is kept in `out`).  The depth-D terms are added
// after the depth-D CG (k_point_values).  The iso-value is the FP64 mean of these float
// values.
__global__ void __launch_bounds__(kBlock) k_point_poly(const Counters* c, int depth, const float* ctr_x,
                                                       const float* ctr_y, const float* ctr_z, const int* neigh,
                                                       size_t stride, const int* parent, const int* enc,
                                                       const float* x, float* coef, size_t cstride) {
    PSR_CLOUD(c, ctr_x, ctr_y, ctr_z, neigh, parent, enc, x, coef);
    const int d1 = depth - 1;
    const int n = c->level_count[d1];
    const int b = c->level_base[d1];
    PSR_GRID_STRIDE(a, n) {
        const int node = b + a;
        const float qx = ctr_x[node], qy = ctr_y[node], qz = ctr_z[node];
        float C[27], y[27], mag = 0.0f;
#pragma unroll
        for (int k = 0; k < 27; ++k) C[k] = 0.0f;
        for (int now = node; now >= 0; now = parent[now]) {
            int ox, oy, oz;
            decode3s(enc[now], depth, ox, oy, oz);
            const int l = ilog2_dev(ox + 1);
#pragma unroll
            for (int k = 0; k < 27; ++k) {
                const int v = neigh[(size_t)k * stride + now];
                y[k] = (v >= 0) ? x[v] : 0.0f;
            }
            sign_level(y, ox, oy, oz, qx, qy, qz, __int_as_float((127 + l - depth) << 23), C, mag);   // h 2^l
        }
#pragma unroll
        for (int k = 0; k < 27; ++k) coef[(size_t)k * cstride + a] = C[k];
    }
}

__global__ void __launch_bounds__(kBlock) k_point_values_coarse(const Counters* c, int depth, const float* px,
                                                                const float* py, const float* pz,
                                                                const int* point2node, const int* parent,
                                                                const float* ctr_x, const float* ctr_y,
                                                                const float* ctr_z, const float* coef,
                                                                size_t cstride, float* out) {
    PSR_CLOUD(c, px, py, pz, point2node, parent, ctr_x, ctr_y, ctr_z, coef, out);
    const int n = c->n_points;
    const int bD = c->level_base[depth];
    const int b1 = c->level_base[depth - 1];
    const float inv2h = (float)(1 << (depth - 1));   // 1 / (2 h) of a depth-(D-1) cell
    PSR_GRID_STRIDE(i, n) {
        const int node = parent[bD + point2node[i]];
        const int a = node - b1;
        // position in the cell, u in [0, 1] per axis (cell from centre - h to centre + h)
        const float hh = 0.5f / inv2h;
        const float ux = (px[i] - (ctr_x[node] - hh)) * inv2h;
        const float uy = (py[i] - (ctr_y[node] - hh)) * inv2h;
        const float uz = (pz[i] - (ctr_z[node] - hh)) * inv2h;
        const float wx[3] = {(1.0f - ux) * (1.0f - ux), 2.0f * ux * (1.0f - ux), ux * ux};
        const float wy[3] = {(1.0f - uy) * (1.0f - uy), 2.0f * uy * (1.0f - uy), uy * uy};
        const float wz[3] = {(1.0f - uz) * (1.0f - uz), 2.0f * uz * (1.0f - uz), uz * uz};
        float val = 0.0f;
#pragma unroll
        for (int k = 0; k < 27; ++k)
            val = fmaf(wx[k / 9] * wy[(k / 3) % 3] * wz[k % 3], coef[(size_t)k * cstride + a], val);
        out[i] = val;
    }
}

// The sample values are summed in chunks of kBlock points (chunk_sums[chunk]), then the
// chunks in order: the iso-value's summation order depends only on the point count, not on
// the launch's grid, so a cloud gets the same iso-value alone and in a multi-cloud launch.
__global__ void __launch_bounds__(kBlock) k_point_values(const Counters* c, int depth, const float* px,
                                                         const float* py, const float* pz, const int* point2node,
                                                         const int* neigh, size_t stride, const int* enc,
                                                         const float* x, float* out, double* chunk_sums) {
    PSR_CLOUD(c, px, py, pz, point2node, neigh, enc, x, out, chunk_sums);
    __shared__ double s_w[kBlock / 32];
    const int n = c->n_points;
    const int bD = c->level_base[depth];
    const int nchunks = (n + kBlock - 1) / kBlock;
    for (int ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        const int i = ch * kBlock + threadIdx.x;
        double acc = 0.0;
        if (i < n) {
            const float v = level_terms(bD + point2node[i], out[i], px[i], py[i], pz[i], depth, neigh, stride, enc, x);
            out[i] = v;
            acc = (double)v;
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane_id() == 0) s_w[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0;
            for (int w = 0; w < kBlock / 32; ++w) sum += s_w[w];
            chunk_sums[ch] = sum;
        }
        __syncthreads();
    }
}

__global__ void k_iso_finalize(Counters* c, const double* chunk_sums) {
    PSR_CLOUD(c, chunk_sums);
    __shared__ double s_w[32];
    const int nchunks = (c->n_points + kBlock - 1) / kBlock;
    double s = 0.0;
    for (int b = threadIdx.x; b < nchunks; b += blockDim.x) s += chunk_sums[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane_id() == 0) s_w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_w[w];
        c->iso_sum = t;
        c->iso = (c->n_points > 0) ? (float)(t / (double)c->n_points) : 0.0f;
    }
}

static int g_cg_cluster = 0;

// launch geometry that needs device queries (done once, outside any stream capture):
// the largest cluster (16, else 8) the device can schedule for the CG kernel
void prepare_launch_configs(Workspace& ws) {
    if (g_cg_cluster == 0) {
        int size = 8;
        if (cudaFuncSetAttribute(k_cg_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCgSmemBytes) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_cg_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCgSmemBytes) !=
                cudaSuccess)
            return;   // left unset: the CG launch reports the error
        if (cudaFuncSetAttribute(k_cg_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess) {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(16);
            cfg.blockDim = dim3(kCgcBlock);
            cfg.dynamicSmemBytes = kCgSmemBytes;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = 16;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, (void*)k_cg_cluster, &cfg) == cudaSuccess && nclusters >= 2)
                size = 16;
        }
        (void)cudaGetLastError();
        g_cg_cluster = size;
    }
    (void)scan_grid(1 << 20);
}

// one cluster (or CTA) per depth and cloud: x spans the depths, y the clouds of the batch
static cudaError_t launch_cg(void (*kernel)(CgcArgs), CgcArgs& a, int grid, int cluster, int clouds, cudaStream_t s) {
    void* args[] = {&a};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid, clouds);
    cfg.blockDim = dim3(kCgcBlock);
    cfg.dynamicSmemBytes = kCgSmemBytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelExC(&cfg, (const void*)kernel, args);
}

// The device loop of the depths in L.loop_mask (units first .. first - units + 1), issued
// on ws.aux4 while that stream is being captured: the initialisation kernel, then a while
// node added to the captured graph, whose body is captured on ws.loop_body, then the report
// kernel.  The body runs once even when no depth needs it (the control kernel then ends
// the loop), so one graph serves every cloud size.
static cudaError_t launch_cg_loop(Workspace& ws, CgLoopArgs& L) {
    // the launches' blocks (8 resident blocks of 256 threads per SM) take the listed units'
    // virtual blocks in turn
    const int grid = 8 * ws.num_sms;
    cudaStream_t s = ws.aux4;
    k_cgl_plan<<<1, 32, 0, s>>>(L);
    k_cgl_init<<<grid, kLoopBlock, 0, s>>>(L);
    cudaError_t e = cudaGetLastError();
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t graph = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t ndeps = 0;
    if (e == cudaSuccess) e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &graph, &deps, nullptr, &ndeps);
    if (e == cudaSuccess && cs != cudaStreamCaptureStatusActive) e = cudaErrorStreamCaptureUnsupported;
    if (e != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> dep(deps, deps + ndeps);
    cudaGraphConditionalHandle cond = 0;
    e = cudaGraphConditionalHandleCreate(&cond, graph, 1, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) return e;
    cudaGraphNodeParams np = {};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = cond;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t loop = nullptr;
    e = cudaGraphAddNode(&loop, graph, dep.data(), nullptr, dep.size(), &np);
    if (e != cudaSuccess) return e;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t b = ws.loop_body;
    e = cudaStreamBeginCaptureToGraph(b, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    for (int rep = 0; rep < kLoopUnroll; ++rep) {   // a depth that is done skips the rest of the pass
        k_cgl_true<<<grid, kLoopBlock, 0, b>>>(L);
        k_cgl_spmv<<<grid, kLoopBlock, 0, b>>>(L);
        k_cgl_update<<<grid, kLoopBlock, 0, b>>>(L);
    }
    k_cgl_control<<<1, 32, 0, b>>>(L, cond);
    cudaError_t el = cudaGetLastError();
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(b, &captured);
    if (e == cudaSuccess) e = el;
    if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(s, &loop, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return e;
    k_cgl_finish<<<dim3(1, ws.batch, L.units), 32, 0, s>>>(L);
    return cudaGetLastError();
}

cudaError_t solve_build(Workspace& ws, int cg_mode, int cg_iters, float cg_tol, int cg_max_iter, int res_period) {
    cudaStream_t s = ws.stream;
    if (g_cg_cluster == 0) prepare_launch_configs(ws);
    const int D = ws.depth;
    CgcArgs a;
    a.v.c = ws.cnt;
    a.v.cw = ws.cnt;
    a.depth = D;
    a.v.neigh = ws.neigh;
    a.v.blk = ws.cg_blk;
    a.stride = (size_t)ws.cap.nodes;
    a.v.stencil = ws.stencil;
    a.v.b = ws.divg;
    a.v.x = ws.xsol;
    a.v.r = ws.cg_r;
    a.v.pa = ws.cg_p;
    a.v.pb = ws.cg_q;
    a.v.ap = ws.cg_ap;
    a.tol2 = cg_tol * cg_tol;
    // a fixed iteration count replaces the reference's max_iter (10000); the tolerance
    // test of the loop is kept (mesh/solver/CGAlgorithm.cu:36)
    a.max_iter = (cg_mode == 1 && cg_iters > 0) ? cg_iters : cg_max_iter;
    a.res_period = res_period;
    k_cg_blocks<<<PSR_GRID(ws, grid_for(ws, 1 << 20)), kBlock, 0, s>>>(ws.cnt, ws.neigh, (size_t)ws.cap.nodes, ws.cg_blk);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // The finest depths (D, D-1, and D-2 from depth 5 on; never the root) on clusters: depth
    // D on the widest cluster, D-1 and D-2 (fewer rows, done well before depth D) on clusters
    // of at most 8 CTAs, on a third stream, so that they hold fewer SMs; the rest one CTA
    // each, on the second stream.  All three run concurrently.
    const int ncl = D < 2 ? D : (D >= 5 ? 3 : 2);
    const int ncta = D - ncl + 1;
    int cl1 = ws.cg_ctas > 0 ? ws.cg_ctas : g_cg_cluster;
    if (cl1 > g_cg_cluster) cl1 = g_cg_cluster;
    int cl2 = ws.cg_ctas_fine > 0 ? ws.cg_ctas_fine : 8;
    if (cl2 > g_cg_cluster) cl2 = g_cg_cluster;
    // Depths 5 .. D may outgrow their cluster's shared memory (depths up to 4 have at most
    // 4,096 rows).  For trees of depth 8 and 9, whose finest depths usually do, a captured
    // graph solves those depths by the device loop, which decides per run from the row
    // counts.  Shallower trees, and pipelines issued directly (no graph), leave them to the
    // global-memory path of their cluster: their depths fit the clusters up to dense clouds
    // of millions of points, and a graph holding a while node cannot be profiled kernel by
    // kernel (Nsight Compute profiles such a graph only as a whole).
    const int loop_units = (ws.ev_flags == cudaEventRecordExternal && D >= 8) ? D - 4 : 0;
    a.loop_mask = 0u;
    for (int z = 0; z < loop_units; ++z) a.loop_mask |= 1u << (D - z);
    e = cudaEventRecord(ws.ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ws.aux, ws.ev_fork, 0);
    if (e == cudaSuccess && ncl > 1) e = cudaStreamWaitEvent(ws.aux3, ws.ev_fork, 0);
    if (e == cudaSuccess && loop_units > 0) {
        e = cudaStreamWaitEvent(ws.aux4, ws.ev_fork, 0);
        CgLoopArgs L;
        L.v = a.v;
        L.st = ws.cg_loop;
        L.part = ws.cg_loop_part;
        L.ctl = ws.cg_loop_ctl;
        L.first = D;
        L.units = loop_units;
        L.clouds = ws.batch;
        for (int d = 0; d <= kMaxDepth; ++d) L.ctas[d] = (d == D) ? cl1 : (d >= D - ncl + 1 ? cl2 : 1);
        L.loop_mask = a.loop_mask;
        L.tol2 = a.tol2;
        L.max_iter = a.max_iter;
        L.res_period = a.res_period;
        if (e == cudaSuccess) e = launch_cg_loop(ws, L);
        if (e == cudaSuccess) e = cudaEventRecord(ws.ev_join4, ws.aux4);
        // the coarse sample values and the depth-D terms wait for every depth's solution
        if (e == cudaSuccess) e = cudaStreamWaitEvent(ws.aux, ws.ev_join4, 0);
    }
    if (e == cudaSuccess && ncta > 0) {
        CgcArgs b = a;
        b.first = D - ncl;
        e = launch_cg(k_cg_cta, b, ncta, 1, ws.batch, ws.aux);   // clusters of one CTA
    }
    if (e != cudaSuccess) return e;
    auto set_stencils = [&](CgcArgs& q) {
        for (int u = 0; u < 3; ++u)
            for (int k = 0; k < 27; ++k)
                q.stp[u][k] = (q.first - u >= 0) ? ws.stencil_host[(q.first - u) * 27 + k] : 0.0f;
    };
    if (ncl > 1) {
        CgcArgs b = a;
        b.first = D - 1;
        set_stencils(b);
        e = launch_cg(k_cg_cluster, b, (ncl - 1) * cl2, cl2, ws.batch, ws.aux3);
        if (e == cudaSuccess) e = cudaEventRecord(ws.ev_join3, ws.aux3);
        if (e != cudaSuccess) return e;
    }
    // the coarser levels' part of the sample values, as soon as every depth below D is
    // solved, beside the depth-D CG
    if (ncl > 1) e = cudaStreamWaitEvent(ws.aux, ws.ev_join3, 0);
    if (e == cudaSuccess) {
        const size_t cstride = (size_t)ws.cap.dnodes / 8 + 64;
        k_point_poly<<<PSR_GRID(ws, ws.num_sms * 4), kBlock, 0, ws.aux>>>(ws.cnt, D, ws.ctr_x, ws.ctr_y, ws.ctr_z, ws.neigh,
                                                            (size_t)ws.cap.nodes, ws.parent, ws.enc, ws.xsol,
                                                            ws.pv_coef, cstride);
        k_point_values_coarse<<<PSR_GRID(ws, ws.num_sms * 4), kBlock, 0, ws.aux>>>(ws.cnt, D, ws.px, ws.py, ws.pz, ws.point2node,
                                                                     ws.parent, ws.ctr_x, ws.ctr_y, ws.ctr_z,
                                                                     ws.pv_coef, cstride, ws.point_val);
        e = cudaEventRecord(ws.ev_join, ws.aux);
    }
    if (e != cudaSuccess) return e;
    if (ncl > 0) {
        a.first = D;
        set_stencils(a);
        e = launch_cg(k_cg_cluster, a, cl1, cl1, ws.batch, s);
        if (e != cudaSuccess) return e;
    }
    if (ws.ev_cg) {
        e = cudaEventRecordWithFlags(ws.ev_cg, s, ws.ev_flags);
        if (e != cudaSuccess) return e;
    }
    e = cudaStreamWaitEvent(s, ws.ev_join, 0);
    if (e != cudaSuccess) return e;
    // iso-value: the depth-D terms complete the sample values
    const int nb = ws.num_sms * 4;
    k_point_values<<<PSR_GRID(ws, nb), kBlock, 0, s>>>(ws.cnt, ws.depth, ws.px, ws.py, ws.pz, ws.point2node, ws.neigh,
                                         (size_t)ws.cap.nodes, ws.enc, ws.xsol, ws.point_val, ws.iso_partial);
    k_iso_finalize<<<PSR_GRID(ws, 1), 256, 0, s>>>(ws.cnt, ws.iso_partial);
    return cudaGetLastError();
}

}  // namespace psr
