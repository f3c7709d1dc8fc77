// Normals of an unoriented point cloud (the reference's PCL step ahead of the path,
// mesh/PoissonReconstruction.cpp:137-161: pcl::NormalEstimationOMP with a kd-tree and
// k = 10 nearest neighbours, viewpoint at the origin).  PCL's published algorithm: the k
// nearest samples of a point (itself included), their centroid and covariance, the
// eigenvector of the smallest eigenvalue as the normal, flipped when it points away from
// the viewpoint.  Fewer than 3 points give no normal (NaN).
//
// Here: the points are Morton-sorted on a 128^3 grid of the reference's normalised
// coordinates (the octree encoder and radix sort), a cell -> first point table is built
// by a scan, and the exact k nearest of every point are found like the colour search's:
// an 8-lane near pass over the 3x3x3 cell block (exact when the k-th is within one cell
// width), then one block per remaining point over coarser levels and shells.  Neighbour
// distances are compared in normalised coordinates (a uniform scale of the input), ties
// towards the lower sorted index.  The 3x3 eigenproblem is solved in FP64.
#include "workspace.h"

namespace psr {

constexpr int kNrmK = 10;            // neighbours (the reference's setKSearch(10))
constexpr int kNrmGridLevel = 7;     // 128^3 cells
constexpr int kNrmLanes = 8;
constexpr int kNrmGroups = kBlock / kNrmLanes;
constexpr int kNrmMaxShell = 12;

__device__ __forceinline__ bool nrm_less(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

// insert (d, i) into a sorted K-list
template <int K>
__device__ __forceinline__ void nrm_insert(float (&bd)[K], int (&bi)[K], float d, int i) {
    if (!nrm_less(d, i, bd[K - 1], bi[K - 1])) return;
    bd[K - 1] = d;
    bi[K - 1] = i;
#pragma unroll
    for (int q = K - 1; q > 0; --q) {
        if (nrm_less(bd[q], bi[q], bd[q - 1], bi[q - 1])) {
            const float td = bd[q]; bd[q] = bd[q - 1]; bd[q - 1] = td;
            const int ti = bi[q]; bi[q] = bi[q - 1]; bi[q - 1] = ti;
        }
    }
}

// the K smallest of the sorted K-lists of `width` lanes (disjoint sets; width lanes
// aligned inside the warp, mask = those lanes): K rounds of the minimum head, the lane
// holding it popping it; every lane of the group ends with the same K
template <int K>
__device__ __forceinline__ void nrm_group_merge(float (&bd)[K], int (&bi)[K], float (&md)[K], int (&mi)[K],
                                                unsigned mask, int width) {
#pragma unroll
    for (int r = 0; r < K; ++r) {
        float d = bd[0];
        int i = bi[0];
        for (int o = width / 2; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(mask, d, o);
            const int oi = __shfl_xor_sync(mask, i, o);
            if (nrm_less(od, oi, d, i)) { d = od; i = oi; }
        }
        md[r] = d;
        mi[r] = i;
        if (bd[0] == d && bi[0] == i) {
#pragma unroll
            for (int q = 0; q < K - 1; ++q) { bd[q] = bd[q + 1]; bi[q] = bi[q + 1]; }
            bd[K - 1] = 1e30f;
            bi[K - 1] = 0x7fffffff;
        }
    }
}

__device__ __forceinline__ unsigned nrm_spread3(unsigned v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}
__device__ __forceinline__ unsigned nrm_morton(int a, int b, int z) {
    return (nrm_spread3((unsigned)a) << 2) | (nrm_spread3((unsigned)b) << 1) | nrm_spread3((unsigned)z);
}

__device__ __forceinline__ void nrm_visit(float qx, float qy, float qz, const float* px, const float* py,
                                          const float* pz, int i, float (&bd)[kNrmK], int (&bi)[kNrmK]) {
    const float dx = __fsub_rn(qx, px[i]), dy = __fsub_rn(qy, py[i]), dz = __fsub_rn(qz, pz[i]);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    nrm_insert<kNrmK>(bd, bi, d2, i);
}

__global__ void k_nrm_reset(Counters* c, int n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    c->n_points = n;
    c->error = 0u;
    c->n_colour_far = 0;
    for (int a = 0; a < 3; ++a) {
        ((int*)c->bbox_max)[a] = float_to_ordered(-FLT_MAX);
        ((int*)c->bbox_min)[a] = float_to_ordered(FLT_MAX);
    }
}

// sorted points in the reference's normalised coordinates ((p - c) * 1 / maxEdge, the
// octree encoder's), whose level-7 cells are their Morton codes
__global__ void __launch_bounds__(kBlock) k_nrm_gather(const Counters* c, const float* xyz, const unsigned* sidx,
                                                       float* px, float* py, float* pz) {
    const int n = c->n_points;
    const float c0 = c->center[0], c1 = c->center[1], c2 = c->center[2], e = c->max_edge;
    PSR_GRID_STRIDE(i, n) {
        const size_t s = sidx[i];
        px[i] = __fdiv_rn(__fmul_rn(__fsub_rn(xyz[3 * s], c0), 1.0f), e);
        py[i] = __fdiv_rn(__fmul_rn(__fsub_rn(xyz[3 * s + 1], c1), 1.0f), e);
        pz[i] = __fdiv_rn(__fmul_rn(__fsub_rn(xyz[3 * s + 2], c2), 1.0f), e);
    }
}

// run length of every occupied cell at the run's last point (the table starts zeroed);
// one scan then turns counts into first points
__global__ void __launch_bounds__(kBlock) k_nrm_cells(Counters* c, const unsigned* scode, int* count) {
    const int n = c->n_points;
    if (blockIdx.x == 0 && threadIdx.x == 0) c->n_colour_cells = (1 << (3 * kNrmGridLevel)) + 1;
    PSR_GRID_STRIDE(i, n) {
        const unsigned m = scode[i];
        if (i + 1 < n && scode[i + 1] == m) continue;
        int lo = 0, hi = i;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (scode[mid] < m) lo = mid + 1;
            else hi = mid;
        }
        count[m] = i + 1 - lo;
    }
}

// Near pass, 8 lanes per point: the points of the 3x3x3 block of level-7 cells around the
// point's cell; exact when K were found and the K-th is closer than one cell width (every
// point outside the block is at least one width away), else the point goes to the far list
__global__ void __launch_bounds__(kBlock) k_nrm_near(Counters* c, const unsigned* scode, const float* px,
                                                     const float* py, const float* pz, const int* cell_start,
                                                     int* nbr, int* far) {
    __shared__ int s_off[kNrmGroups][28];
    __shared__ int s_base[kNrmGroups][27];
    const int n = c->n_points;
    const int G = 1 << kNrmGridLevel;
    const float w = 1.0f / (float)G;
    const int lane = threadIdx.x & (kNrmLanes - 1);
    const int gib = threadIdx.x / kNrmLanes;
    const unsigned gmask = 0xffu << (threadIdx.x & 24);
    const int group = (blockIdx.x * blockDim.x + threadIdx.x) / kNrmLanes;
    const int ngroups = (gridDim.x * blockDim.x) / kNrmLanes;
    for (int p = group; p < n; p += ngroups) {
        const float qx = px[p], qy = py[p], qz = pz[p];
        // the point's cell from its code (x = bit 2 of every triple)
        const unsigned code = scode[p];
        int cxyz[3] = {0, 0, 0};
#pragma unroll
        for (int l = 0; l < kNrmGridLevel; ++l)
#pragma unroll
            for (int a = 0; a < 3; ++a) cxyz[a] |= (int)((code >> (3 * l + 2 - a)) & 1u) << l;
        int running = 0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int k = lane + kNrmLanes * r;
            int cnt = 0, base = 0;
            if (k < 27) {
                const int a = cxyz[0] + k / 9 - 1, b = cxyz[1] + (k / 3) % 3 - 1, z = cxyz[2] + k % 3 - 1;
                if (a >= 0 && a < G && b >= 0 && b < G && z >= 0 && z < G) {
                    const unsigned m = nrm_morton(a, b, z);
                    base = cell_start[m];
                    cnt = cell_start[m + 1] - base;
                }
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < kNrmLanes; o <<= 1) {
                const int y = __shfl_up_sync(gmask, incl, o, kNrmLanes);
                if (lane >= o) incl += y;
            }
            if (k < 27) {
                s_off[gib][k] = running + incl - cnt;
                s_base[gib][k] = base;
            }
            running += __shfl_sync(gmask, incl, kNrmLanes - 1, kNrmLanes);
        }
        if (lane == 0) s_off[gib][27] = running;
        __syncwarp(gmask);
        float bd[kNrmK];
        int bi[kNrmK];
#pragma unroll
        for (int q = 0; q < kNrmK; ++q) { bd[q] = 1e30f; bi[q] = 0x7fffffff; }
        int k = 0;
        for (int t = lane; t < running; t += kNrmLanes) {
            while (s_off[gib][k + 1] <= t) ++k;
            nrm_visit(qx, qy, qz, px, py, pz, s_base[gib][k] + (t - s_off[gib][k]), bd, bi);
        }
        __syncwarp(gmask);
        float md[kNrmK];
        int mi[kNrmK];
        nrm_group_merge<kNrmK>(bd, bi, md, mi, gmask, kNrmLanes);
        if (lane == 0) {
            // fewer than K points in the whole cloud: all of them are the neighbours
            const bool all_found = mi[kNrmK - 1] != 0x7fffffff || running == n;
            if (all_found && (md[kNrmK - 1] < w * w || running == n)) {
#pragma unroll
                for (int q = 0; q < kNrmK; ++q) nbr[(size_t)p * kNrmK + q] = mi[q];
            } else {
                far[atomicAdd(&c->n_colour_far, 1)] = p;
            }
        }
    }
}

// the block's K nearest from its threads' sorted K-lists (left as they are: the shell pass
// goes on inserting into them): each warp merges its lanes, then warp 0 merges the warps'
// results; every thread gets them
__device__ __forceinline__ void nrm_block_merge(const float (&bd)[kNrmK], const int (&bi)[kNrmK],
                                                float (&md)[kNrmK], int (&mi)[kNrmK], float* s_cd, int* s_ci) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    constexpr int kCand = (kBlock / 32) * kNrmK;
    float wd[kNrmK], td[kNrmK];
    int wi[kNrmK], ti[kNrmK];
#pragma unroll
    for (int q = 0; q < kNrmK; ++q) { td[q] = bd[q]; ti[q] = bi[q]; }
    nrm_group_merge<kNrmK>(td, ti, wd, wi, 0xffffffffu, 32);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < kNrmK; ++q) {
            s_cd[warp * kNrmK + q] = wd[q];
            s_ci[warp * kNrmK + q] = wi[q];
        }
    }
    __syncthreads();
    if (warp == 0) {
        float cd[kNrmK];
        int ci[kNrmK];
#pragma unroll
        for (int q = 0; q < kNrmK; ++q) { cd[q] = 1e30f; ci[q] = 0x7fffffff; }
        for (int t = lane; t < kCand; t += 32) nrm_insert<kNrmK>(cd, ci, s_cd[t], s_ci[t]);
        nrm_group_merge<kNrmK>(cd, ci, wd, wi, 0xffffffffu, 32);
    }
    __syncthreads();   // every warp has read the candidates before they are replaced
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < kNrmK; ++q) {
            s_cd[q] = wd[q];
            s_ci[q] = wi[q];
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < kNrmK; ++q) {
        md[q] = s_cd[q];
        mi[q] = s_ci[q];
    }
    __syncthreads();
}

// Far pass, one block per far point: the 3x3x3 block of cells at level g, then the shell
// of cells up to the radius that bounds the K-th nearest (cells farther than it skipped),
// restarting one level coarser when the K-th is not found or the shell would be too wide
__global__ void __launch_bounds__(kBlock) k_nrm_far(const Counters* c, const float* px, const float* py,
                                                    const float* pz, const int* cell_start, const int* far,
                                                    int* nbr) {
    __shared__ int s_off[28];
    __shared__ int s_base[27];
    __shared__ float s_cd[(kBlock / 32) * kNrmK];
    __shared__ int s_ci[(kBlock / 32) * kNrmK];
    const int n = c->n_points;
    const int nfar = c->n_colour_far;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int t = blockIdx.x; t < nfar; t += gridDim.x) {
        const int p = far[t];
        const float qx = px[p], qy = py[p], qz = pz[p];
        float md[kNrmK];
        int mi[kNrmK];
        for (int g = kNrmGridLevel; g >= 0; --g) {
            const int G = 1 << g;
            const int shift = 3 * (kNrmGridLevel - g);
            const int cx = min(max((int)floorf(qx * G), 0), G - 1);
            const int cy = min(max((int)floorf(qy * G), 0), G - 1);
            const int cz = min(max((int)floorf(qz * G), 0), G - 1);
            if (warp == 0) {
                int cnt = 0, base = 0;
                if (lane < 27) {
                    const int a = cx + lane / 9 - 1, b = cy + (lane / 3) % 3 - 1, z = cz + lane % 3 - 1;
                    if (a >= 0 && a < G && b >= 0 && b < G && z >= 0 && z < G) {
                        const unsigned m = nrm_morton(a, b, z);
                        base = cell_start[(size_t)m << shift];
                        cnt = cell_start[(size_t)(m + 1) << shift] - base;
                    }
                }
                int incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += y;
                }
                if (lane < 27) {
                    s_off[lane] = incl - cnt;
                    s_base[lane] = base;
                }
                if (lane == 26) s_off[27] = incl;
            }
            __syncthreads();
            const int total = s_off[27];
            float bd[kNrmK];
            int bi[kNrmK];
#pragma unroll
            for (int q = 0; q < kNrmK; ++q) { bd[q] = 1e30f; bi[q] = 0x7fffffff; }
            int k = 0;
            for (int i = tid; i < total; i += kBlock) {
                while (s_off[k + 1] <= i) ++k;
                nrm_visit(qx, qy, qz, px, py, pz, s_base[k] + (i - s_off[k]), bd, bi);
            }
            nrm_block_merge(bd, bi, md, mi, s_cd, s_ci);
            if (total == n || g == 0) break;                // every point seen
            if (mi[kNrmK - 1] == 0x7fffffff) continue;      // fewer than K in the block
            const float w = 1.0f / (float)G;
            if (md[kNrmK - 1] < w * w) break;
            int R = (int)(sqrtf(md[kNrmK - 1]) * (float)G) + 1;
            while (!(md[kNrmK - 1] < __fmul_rn(R * w, R * w))) ++R;
            if (R > kNrmMaxShell) continue;
            const int side = 2 * R + 1;
            const int ncell = side * side * side;
            for (int i = tid; i < ncell; i += kBlock) {
                const int ta = i / (side * side), tr = i - ta * side * side;
                const int tb = tr / side, tz = tr - tb * side;
                const int a = cx - R + ta, b = cy - R + tb, z = cz - R + tz;
                if (a < 0 || a >= G || b < 0 || b >= G || z < 0 || z >= G) continue;
                if (max(abs(a - cx), max(abs(b - cy), abs(z - cz))) <= 1) continue;
                const float gx = fmaxf(fmaxf(__fsub_rn(a * w, qx), __fsub_rn(qx, (a + 1) * w)), 0.0f);
                const float gy = fmaxf(fmaxf(__fsub_rn(b * w, qy), __fsub_rn(qy, (b + 1) * w)), 0.0f);
                const float gz = fmaxf(fmaxf(__fsub_rn(z * w, qz), __fsub_rn(qz, (z + 1) * w)), 0.0f);
                const float mind2 = __fadd_rn(__fadd_rn(__fmul_rn(gx, gx), __fmul_rn(gy, gy)), __fmul_rn(gz, gz));
                if (mind2 > md[kNrmK - 1] * 1.0001f) continue;
                const unsigned m = nrm_morton(a, b, z);
                const int s0 = cell_start[(size_t)m << shift], s1 = cell_start[(size_t)(m + 1) << shift];
                for (int j = s0; j < s1; ++j) nrm_visit(qx, qy, qz, px, py, pz, j, bd, bi);
            }
            nrm_block_merge(bd, bi, md, mi, s_cd, s_ci);
            break;
        }
        if (tid == 0) {
#pragma unroll
            for (int q = 0; q < kNrmK; ++q) nbr[(size_t)p * kNrmK + q] = mi[q];
        }
    }
}

// eigenvector of the smallest eigenvalue of the symmetric 3x3 matrix (a00 a01 a02; a11 a12;
// a22): eigenvalues from the characteristic cubic (trigonometric form), the vector as the
// longest cross product of two rows of A - lambda I
__device__ __forceinline__ void nrm_smallest_eigvec(double a00, double a01, double a02, double a11, double a12,
                                                    double a22, double (&v)[3]) {
    const double scale = fmax(fmax(fmax(fabs(a00), fabs(a01)), fmax(fabs(a02), fabs(a11))), fmax(fabs(a12), fabs(a22)));
    if (!(scale > 0.0)) { v[0] = v[1] = v[2] = 0.0; return; }
    a00 /= scale; a01 /= scale; a02 /= scale; a11 /= scale; a12 /= scale; a22 /= scale;
    const double q = (a00 + a11 + a22) / 3.0;
    const double b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const double p2 = (b00 * b00 + b11 * b11 + b22 * b22 + 2.0 * (a01 * a01 + a02 * a02 + a12 * a12)) / 6.0;
    double lambda = q;
    if (p2 > 0.0) {
        const double p = sqrt(p2);
        const double det = b00 * (b11 * b22 - a12 * a12) - a01 * (a01 * b22 - a12 * a02) + a02 * (a01 * a12 - b11 * a02);
        double r = det / (2.0 * p * p2);
        r = fmin(fmax(r, -1.0), 1.0);
        const double phi = acos(r) / 3.0;
        lambda = q + 2.0 * p * cos(phi + 2.0943951023931954923);   // the smallest root
    }
    const double r0[3] = {a00 - lambda, a01, a02};
    const double r1[3] = {a01, a11 - lambda, a12};
    const double r2[3] = {a02, a12, a22 - lambda};
    const double c01[3] = {r0[1] * r1[2] - r0[2] * r1[1], r0[2] * r1[0] - r0[0] * r1[2], r0[0] * r1[1] - r0[1] * r1[0]};
    const double c02[3] = {r0[1] * r2[2] - r0[2] * r2[1], r0[2] * r2[0] - r0[0] * r2[2], r0[0] * r2[1] - r0[1] * r2[0]};
    const double c12[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2], r1[0] * r2[1] - r1[1] * r2[0]};
    const double n01 = c01[0] * c01[0] + c01[1] * c01[1] + c01[2] * c01[2];
    const double n02 = c02[0] * c02[0] + c02[1] * c02[1] + c02[2] * c02[2];
    const double n12 = c12[0] * c12[0] + c12[1] * c12[1] + c12[2] * c12[2];
    double b0 = c01[0], b1 = c01[1], b2 = c01[2], nb = n01;
    if (n02 > nb) { b0 = c02[0]; b1 = c02[1]; b2 = c02[2]; nb = n02; }
    if (n12 > nb) { b0 = c12[0]; b1 = c12[1]; b2 = c12[2]; nb = n12; }
    if (!(nb > 0.0)) { v[0] = v[1] = v[2] = 0.0; return; }
    const double inv = 1.0 / sqrt(nb);
    v[0] = b0 * inv;
    v[1] = b1 * inv;
    v[2] = b2 * inv;
}

// normal of every point: centroid and covariance of its neighbours (FP64), the smallest
// eigenvector, flipped towards the viewpoint (in input coordinates), written in input order
__global__ void __launch_bounds__(kBlock) k_nrm_pca(const Counters* c, const float* px, const float* py,
                                                    const float* pz, const float* xyz, const unsigned* sidx,
                                                    const int* nbr, float vpx, float vpy, float vpz, float* out) {
    const int n = c->n_points;
    const float nan = __int_as_float(0x7fc00000);
    PSR_GRID_STRIDE(p, n) {
        int cnt = 0;
        double sx = 0, sy = 0, sz = 0, sxx = 0, sxy = 0, sxz = 0, syy = 0, syz = 0, szz = 0;
#pragma unroll
        for (int q = 0; q < kNrmK; ++q) {
            const int j = nbr[(size_t)p * kNrmK + q];
            if (j < 0 || j >= n) continue;
            const double x = px[j], y = py[j], z = pz[j];
            ++cnt;
            sx += x; sy += y; sz += z;
            sxx += x * x; sxy += x * y; sxz += x * z; syy += y * y; syz += y * z; szz += z * z;
        }
        const size_t s = sidx[p];
        float nv[3] = {nan, nan, nan};
        if (cnt >= 3) {
            const double inv = 1.0 / cnt;
            const double mx = sx * inv, my = sy * inv, mz = sz * inv;
            double v[3];
            nrm_smallest_eigvec(sxx * inv - mx * mx, sxy * inv - mx * my, sxz * inv - mx * mz, syy * inv - my * my,
                                syz * inv - my * mz, szz * inv - mz * mz, v);
            if (v[0] != 0.0 || v[1] != 0.0 || v[2] != 0.0) {
                const double cosv = (vpx - xyz[3 * s]) * v[0] + (vpy - xyz[3 * s + 1]) * v[1] + (vpz - xyz[3 * s + 2]) * v[2];
                const double sg = (cosv < 0.0) ? -1.0 : 1.0;
                nv[0] = (float)(sg * v[0]);
                nv[1] = (float)(sg * v[1]);
                nv[2] = (float)(sg * v[2]);
            }
        }
        out[3 * s] = nv[0];
        out[3 * s + 1] = nv[1];
        out[3 * s + 2] = nv[2];
    }
}

cudaError_t encode_sort_points(Workspace& ws, const float* xyz, int depth, const unsigned** scode,
                               const unsigned** sidx);

// normals of the n points at xyz (device, 3 floats each) into out (device), on ws.stream;
// uses the workspace's point, node-neighbour and colour scratch (no reconstruction runs
// on the handle meanwhile)
cudaError_t normals_build(Workspace& ws, const float* xyz, int n, float* out, float vpx, float vpy, float vpz) {
    cudaStream_t s = ws.stream;
    Counters* c = ws.cnt;
    k_nrm_reset<<<1, 1, 0, s>>>(c, n);
    const unsigned *scode = nullptr, *sidx = nullptr;
    cudaError_t e = encode_sort_points(ws, xyz, kNrmGridLevel, &scode, &sidx);
    if (e != cudaSuccess) return e;
    const int gp = grid_for(ws, n);
    k_nrm_gather<<<gp, kBlock, 0, s>>>(c, xyz, sidx, ws.px, ws.py, ws.pz);
    e = cudaMemsetAsync(ws.cell_start, 0, sizeof(int) * (((size_t)1 << (3 * kNrmGridLevel)) + 1), s);
    if (e != cudaSuccess) return e;
    k_nrm_cells<<<gp, kBlock, 0, s>>>(c, scode, ws.cell_start);
    unsigned* table = reinterpret_cast<unsigned*>(ws.cell_start);
    e = launch_scan(LoadArray{table}, StoreExclusive{table}, &c->n_colour_cells, 0, ws.scan,
                    (unsigned*)&c->scan_total, &c->error, s, ScanCount{}, 2);
    if (e != cudaSuccess) return e;
    int* nbr = ws.neigh;           // K per point (the neighbour table is free before a reconstruction)
    int* far = ws.point2node;      // points left to the wide search
    k_nrm_near<<<ws.num_sms * 8, kBlock, 0, s>>>(c, scode, ws.px, ws.py, ws.pz, ws.cell_start, nbr, far);
    k_nrm_far<<<2 * ws.num_sms, kBlock, 0, s>>>(c, ws.px, ws.py, ws.pz, ws.cell_start, far, nbr);
    k_nrm_pca<<<gp, kBlock, 0, s>>>(c, ws.px, ws.py, ws.pz, xyz, sidx, nbr, vpx, vpy, vpz, out);
    return cudaGetLastError();
}

}  // namespace psr
