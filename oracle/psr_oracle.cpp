// CPU oracle for the Poisson surface reconstruction path.
//
// TEST INFRASTRUCTURE ONLY.  This file restates, sequentially and on the host, the
// reference pipeline (RKGalaxy-Luo/Poisson-Surface-Reconstruction-GPU) so that the CUDA
// implementation can be checked against it.  Only the test suite, the smoke check and
// the CPU-baseline leg of the benchmark load it; the product never does.
//
// Fidelity:
//  * integer / index work (Morton keys, node arrays, neighbour tables, vertex / edge /
//    face ownership, marching-cubes topology, subdivision) follows the reference kernels
//    step by step, quirks included (each quirk is marked "reference quirk");
//  * floating-point stages are computed in FP64 on the same discretisation (same basis,
//    same tables, same per-depth systems), using exact B-spline inner products;
//  * a float "mirror" of the implicit-function evaluation and of the edge interpolation
//    reproduces the GPU kernels' operation order so that mesh topology can be compared
//    bit for bit given the GPU's own solution vector.
// Where the reference reads uninitialised or stale memory the oracle implements the
// intended semantics and counts the event (see ub_events).
//
// Parity pin: the B-spline tables are pinned against the reference's own host table
// code (mesh/FunctionData.h) by tests/golden; all other stages are pinned by
// known-answer tests only (the reference ships no tests or golden outputs).
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fopenmp -shared -fPIC (see the package
// build script).  Plain C ABI at the bottom for ctypes.

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../poisson-surface-reconstruction-gpu_gb300/csrc/mc_tables.inc"

namespace oracle {

// ---------------------------------------------------------------------------------
// Lookup tables derived from geometry (the reference hard-codes the same values:
// mesh/BuildOctree.cu:20-42, mesh/ComputeTriangleIndices.cu:31-38,317-322,
// mesh/BuildMeshGeometry.cu:19-26).
// ---------------------------------------------------------------------------------
struct Luts {
    int lut_parent[8][27];
    int lut_child[8][27];
    int edge_vertex[12][2];   // marching-cubes corner pair of each cube edge
    int face_edges[6][4];
    int parent_face_kind[8][6];
    int children_vertex_kind[8];
    Luts() {
        // neighbour index i = 9*ox + 3*oy + oz, o in {0,1,2} for offsets -1,0,+1;
        // child key bits: x = 4, y = 2, z = 1 (mesh/BuildOctree.cu:167-208).
        for (int s = 0; s < 8; ++s) {
            int cp[3] = {(s >> 2) & 1, (s >> 1) & 1, s & 1};
            for (int i = 0; i < 27; ++i) {
                int o[3] = {i / 9, (i / 3) % 3, i % 3};
                int pidx = 0, cidx = 0;
                for (int a = 0; a < 3; ++a) {
                    int q = cp[a] + o[a] - 1;           // -1..2
                    int po = (q < 0) ? 0 : (q > 1 ? 2 : 1);
                    int cc = (q + 2) & 1;
                    pidx = pidx * 3 + po;
                    cidx = cidx * 2 + cc;
                }
                lut_parent[s][i] = pidx;
                lut_child[s][i] = cidx;
            }
        }
        // Cube corner numbering used by the node vertex slots (counter-clockwise in the
        // x/y plane, z low then high): 0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0) 4..7 same
        // with z = 1 (mesh/BuildMeshGeometry.cu:133-144).  Edges as in the reference
        // table mesh/ComputeTriangleIndices.cu:37.
        static const int ev[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 3}, {1, 2},
                                      {4, 7}, {5, 6}, {0, 4}, {1, 5}, {3, 7}, {2, 6}};
        static const int fe[6][4] = {{4, 6, 8, 10}, {5, 7, 9, 11}, {0, 2, 8, 9},
                                     {1, 3, 10, 11}, {0, 1, 4, 5}, {2, 3, 6, 7}};
        // parent face kind: mesh/BuildMeshGeometry.cu:19-26 (row 7 carries a stray 0 in
        // column 0, reproduced).
        static const int pfk[8][6] = {{0, -1, 2, -1, 4, -1}, {-1, 1, 2, -1, 4, -1},
                                      {0, -1, -1, 3, 4, -1}, {-1, 1, -1, 3, 4, -1},
                                      {0, -1, 2, -1, -1, 5}, {-1, 1, 2, -1, -1, 5},
                                      {0, -1, -1, 3, -1, 5}, {0, 1, -1, 3, -1, 5}};
        static const int cvk[8] = {0, 1, 3, 2, 4, 5, 7, 6};
        memcpy(edge_vertex, ev, sizeof(ev));
        memcpy(face_edges, fe, sizeof(fe));
        memcpy(parent_face_kind, pfk, sizeof(pfk));
        memcpy(children_vertex_kind, cvk, sizeof(cvk));
    }
};
static const Luts L;

static int mc_tri_edge(int cube, int k) {  // k-th edge index of case `cube`
    return (int)((kMcTrianglesInit[cube] >> (4 * k)) & 0xF);
}

// ---------------------------------------------------------------------------------
// Basis function: quadratic B-spline (box * box * box) normalised to F(0) = 1,
// i.e. PPolynomial<2>::GaussianApproximation() / F(0)  (math/PPolynomial.h:568-582,
// mesh/ComputeVectorField.cpp:81-95).
//   F(t) = 1 - 4/3 t^2          |t| < 1/2
//          2/3 (3/2 - |t|)^2    1/2 <= |t| < 3/2
// 1-D function index i (BinaryNode, mesh/BinaryNode.h:25-58): depth d = floor(log2(i+1)),
// offset o = i + 1 - 2^d, centre (o + 1/2) / 2^d, width 2^-d.
// ---------------------------------------------------------------------------------
static inline int ilog2(int v) { int d = -1; while (v) { v >>= 1; ++d; } return d; }

static inline double F64(double t) {
    double a = std::fabs(t);
    if (a < 0.5) return 1.0 - (4.0 / 3.0) * t * t;
    if (a < 1.5) { double u = 1.5 - a; return (2.0 / 3.0) * u * u; }
    return 0.0;
}
static inline double dF64(double t) {
    double a = std::fabs(t);
    if (a < 0.5) return -(8.0 / 3.0) * t;
    if (a < 1.5) { double u = 1.5 - a; double g = (4.0 / 3.0) * u; return t > 0 ? -g : g; }
    return 0.0;
}
static inline double basis64(int idx, double x) {
    int d = ilog2(idx + 1);
    int off = idx + 1 - (1 << d);
    double s = (double)(1 << d);
    double c = ((double)off + 0.5) / s;
    return F64((x - c) * s);
}

// Float mirror of the device evaluation (same operation order, no contraction).
static const float kF43 = 1.33333337306976318359375f;   // nearest float to 4/3
static const float kF23 = 0.666666686534881591796875f;  // nearest float to 2/3
static inline float basis32(int idx, float x) {
    int d = ilog2(idx + 1);
    int off = idx + 1 - (1 << d);
    float s = (float)(1 << d);
    float c = ((float)off + 0.5f) / s;
    float t = (x - c) * s;
    float a = std::fabs(t);
    if (a < 0.5f) { float tt = t * t; float q = 0.75f - tt; return q * kF43; }
    if (a < 1.5f) { float u = 1.5f - a; float uu = u * u; return uu * kF23; }
    return 0.0f;
}

// Exact inner products of 1-D basis functions over the union of breakpoints, 3-point
// Gauss-Legendre per piece (exact up to degree 5).
struct Tables {
    int res = 0;
    std::vector<double> ff, dff, d2;   // index i + res * j  (mesh/FunctionData.h:134-190)
    void build(int depth) {
        res = (1 << (depth + 1)) - 1;
        ff.assign((size_t)res * res, 0.0);
        dff.assign((size_t)res * res, 0.0);
        d2.assign((size_t)res * res, 0.0);
        static const double gx[3] = {-0.7745966692414833770, 0.0, 0.7745966692414833770};
        static const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
        for (int i = 0; i < res; ++i) {
            int di = ilog2(i + 1), oi = i + 1 - (1 << di);
            double wi = 1.0 / (1 << di), ci = (oi + 0.5) * wi;
            for (int j = 0; j < res; ++j) {
                int dj = ilog2(j + 1), oj = j + 1 - (1 << dj);
                double wj = 1.0 / (1 << dj), cj = (oj + 0.5) * wj;
                double lo = std::max(ci - 1.5 * wi, cj - 1.5 * wj);
                double hi = std::min(ci + 1.5 * wi, cj + 1.5 * wj);
                if (lo >= hi) continue;
                double bp[12];
                int nb = 0;
                for (int k = 0; k < 4; ++k) {
                    double a = ci + (k - 1.5) * wi, b = cj + (k - 1.5) * wj;
                    if (a > lo && a < hi) bp[nb++] = a;
                    if (b > lo && b < hi) bp[nb++] = b;
                }
                bp[nb++] = lo;
                bp[nb++] = hi;
                for (int a = 1; a < nb; ++a)   // insertion sort of <= 10 breakpoints
                    for (int b = a; b > 0 && bp[b - 1] > bp[b]; --b) std::swap(bp[b - 1], bp[b]);
                double sff = 0, sdf = 0, sd2 = 0;
                for (int k = 0; k + 1 < nb; ++k) {
                    double a = bp[k], b = bp[k + 1];
                    if (b <= a) continue;
                    double h = 0.5 * (b - a), m = 0.5 * (a + b);
                    for (int q = 0; q < 3; ++q) {
                        double x = m + h * gx[q];
                        double ti = (x - ci) / wi, tj = (x - cj) / wj;
                        double Fi = F64(ti), Fj = F64(tj);
                        double dFi = dF64(ti) / wi, dFj = dF64(tj) / wj;
                        sff += gw[q] * h * Fi * Fj;
                        sdf += gw[q] * h * dFi * Fj;
                        sd2 += gw[q] * h * dFi * dFj;
                    }
                }
                size_t k = (size_t)i + (size_t)res * j;
                ff[k] = sff;
                dff[k] = sdf;
                d2[k] = sd2;
            }
        }
    }
};

// ---------------------------------------------------------------------------------
// Mesh-side records (mesh/OctNode.cuh:79-106)
// ---------------------------------------------------------------------------------
struct VertexRec { float pos[3]; int owner, kind, depth; int nodes[8]; int nnodes; };
struct EdgeRec { int kind, owner; int nodes[4]; int nnodes; };
struct FaceRec { int kind, owner, has_parent_face; int nodes[2]; int nnodes; };

struct Options {
    int depth = 7;
    int cg_iters = 0;          // > 0: replaces the maximum iteration count per depth
    double cg_tol = 1e-5;      // absolute tolerance on ||r|| (mesh/solver/CGAlgorithm.cu:298)
    int cg_max_iter = 10000;   // mesh/solver/CGAlgorithm.cu:15
    int stop_after = 99;       // 1 octree, 2 field, 3 solve, 4 mesh, 5 colour
    int tri_cap = 1000000;     // MAX_MESH_TRIANGLE_COUNT (base/GlobalConfigs.h:8)
    int vert_cap = 300000;     // MeshTriangleVertex capacity (ComputeTriangleIndices.cpp:32)
    double lap_eps = (double)1e-6f;   // entries with |L| <= lap_eps are dropped (EPSILON, device::eps)
};

struct State {
    Options opt;
    int N = 0, D = 0, M = 0;
    int ub_events = 0;         // reference reads of uninitialised / stale memory hit
    float bbox_center[3] = {0, 0, 0}, bbox_edge = 0;
    // points, sorted by Morton key, normalised to the unit cube
    std::vector<long long> sorted_keys;
    std::vector<float> pos, color;
    std::vector<double> nrm;   // normal scaled to 2^(D+1) (FP64)
    std::vector<int> point2node;
    std::vector<int> base, count;
    // node arrays
    std::vector<int> key, pidx, pnum, parent, didx, dnum, depth, enc;
    std::vector<int> children, neighs;   // 8 and 27 per node
    std::vector<float> center;            // 3 per node
    Tables tab;
    // field / solve
    std::vector<double> vfield, div, x, point_chi;
    std::vector<int> cg_iters;
    std::vector<double> cg_resid;
    double iso = 0;
    // mesh geometry
    std::vector<VertexRec> verts;
    std::vector<EdgeRec> edges;
    std::vector<FaceRec> faces;
    std::vector<int> node_vertices, node_edges, node_faces;
    std::vector<double> vvalue;
    std::vector<int> has_triangle, has_intersection;
    std::vector<int> sub_roots;          // node index of each subdivision root, in order
    std::vector<int> sub_root_depth;
    std::vector<float> mesh_v;            // 3 per output vertex (unit cube)
    std::vector<int> mesh_t;              // 3 per output triangle
    std::vector<int> mesh_stage_v, mesh_stage_t;   // counts per insertion (0 = main)
    int status = 0;                       // 0 ok, 1 capacity exceeded, 2 invalid input
    std::vector<float> vcolor, vnormal;
    // mirror-mode intermediates
    std::vector<float> vvalue32;
    std::vector<int> cube_class;          // per D-level node
    std::vector<int> edge_cross;          // per edge
};

// ---------------------------------------------------------------------------------
// Octree build: mesh/BuildOctree.cpp:75-194, mesh/BuildOctree.cu
// ---------------------------------------------------------------------------------
static int build_octree(State& S, const float* xyz, const float* nrm, const float* rgb, int n) {
    const int D = S.opt.depth;
    S.D = D;
    S.N = n;
    // bounding box (mesh/BuildOctree.cu:51-133, host finish :121-133).  The reference seeds
    // with -1e6 / 1e6 (mesh/BuildOctree.cpp:87-88, BuildOctree.cu:66-73); -FLT_MAX / FLT_MAX
    // gives the same box unless every coordinate of an axis lies beyond 1e6 in magnitude,
    // where the reference's box is wrong and this one is the true box.
    float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX}, mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    for (int i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            float v = xyz[3 * i + a];
            mx[a] = mx[a] < v ? v : mx[a];
            mn[a] = mn[a] > v ? v : mn[a];
        }
    // mesh/BuildOctree.cu:619-631
    float maxEdge = 1.0f, c[3];
    for (int a = 0; a < 3; ++a) {
        if (a == 0 || maxEdge < (mx[a] - mn[a])) maxEdge = mx[a] - mn[a];
        c[a] = (mx[a] + mn[a]) / 2.0f;
    }
    maxEdge *= 1.25f * 1.0f;
    for (int a = 0; a < 3; ++a) c[a] -= maxEdge / 2.0f;
    for (int a = 0; a < 3; ++a) S.bbox_center[a] = c[a];
    S.bbox_edge = maxEdge;
    // normalise (mesh/BuildOctree.cu:144-165) and encode (:167-208)
    std::vector<float> p(3 * (size_t)n);
    std::vector<double> nn(3 * (size_t)n);
    std::vector<long long> keys(n);
    const double nscale = (double)(2 << D);
    for (int i = 0; i < n; ++i) {
        for (int a = 0; a < 3; ++a) p[3 * i + a] = (xyz[3 * i + a] - c[a]) * 1.0f / maxEdge;
        double l = std::sqrt((double)nrm[3 * i] * nrm[3 * i] + (double)nrm[3 * i + 1] * nrm[3 * i + 1] +
                             (double)nrm[3 * i + 2] * nrm[3 * i + 2]);
        // reference quirk: a normal shorter than 1e-6 is scaled by its length instead
        // of its inverse length
        double s = (l > (double)1e-6f) ? 1.0 / l : l;
        s *= nscale;
        for (int a = 0; a < 3; ++a) nn[3 * i + a] = nrm[3 * i + a] * s;
        long long k = 0;
        float cc[3] = {0.5f, 0.5f, 0.5f};
        float w = 0.25f;
        for (int lvl = D - 1; lvl >= 0; --lvl) {
            for (int a = 0; a < 3; ++a) {
                if (p[3 * i + a] > cc[a]) { k |= 1ll << (3 * lvl + 34 - a); cc[a] += w; }
                else cc[a] -= w;
            }
            w /= 2.0f;
        }
        keys[i] = k + i;
    }
    // sort by the full key (= stable sort on the code) (mesh/BuildOctree.cu:654-660)
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int a, int b) { return keys[a] < keys[b]; });
    S.sorted_keys.resize(n);
    S.pos.resize(3 * (size_t)n);
    S.nrm.resize(3 * (size_t)n);
    S.color.assign(3 * (size_t)n, 0.0f);
    for (int i = 0; i < n; ++i) {
        int o = order[i];
        // low 32 bits replaced by the sorted index (mesh/BuildOctree.cu:210-221)
        S.sorted_keys[i] = (keys[o] & ~((1ll << 32) - 1)) + i;
        for (int a = 0; a < 3; ++a) {
            S.pos[3 * i + a] = p[3 * o + a];
            S.nrm[3 * i + a] = nn[3 * o + a];
            if (rgb) S.color[3 * i + a] = rgb[3 * o + a];
        }
    }
    // unique leaves (mesh/BuildOctree.cu:223-265)
    std::vector<int> ukey, upidx, upnum, ufirst;
    for (int i = 0; i < n; ++i) {
        int hi = (int)(S.sorted_keys[i] >> 32);
        if (i == 0 || hi != (int)(S.sorted_keys[i - 1] >> 32)) {
            ukey.push_back(hi);
            upidx.push_back(i);
            ufirst.push_back(i);
        }
    }
    const int U = (int)ukey.size();
    for (int u = 0; u < U; ++u) upnum.push_back((u + 1 < U ? upidx[u + 1] : n) - upidx[u]);
    // node numbers / addresses (mesh/BuildOctree.cu:267-280, :715-733)
    std::vector<int> naddr(U);
    {
        int run = 0;
        for (int u = 0; u < U; ++u) {
            int v = (u == 0) ? 0 : (((ukey[u - 1] >> 3) != (ukey[u] >> 3)) ? 8 : 0);
            run += v;
            naddr[u] = run;
        }
    }
    // per-level arrays, built from depth D upwards
    struct Level {
        std::vector<int> key, pidx, pnum, parent, didx, dnum, children;  // children 8/node
    };
    std::vector<Level> lv(D + 1);
    std::vector<int> count(D + 1, 0), base(D + 1, 0);
    auto init_level = [](Level& l, int m) {
        l.key.assign(m, 0); l.pidx.assign(m, 0); l.pnum.assign(m, 0); l.parent.assign(m, 0);
        l.didx.assign(m, 0); l.dnum.assign(m, 0); l.children.assign(8 * (size_t)m, 0);
    };
    int MD = (U > 0 ? naddr[U - 1] : 0) + 8;
    init_level(lv[D], MD);
    std::vector<int> addr_full(MD, 0);
    S.point2node.assign(n, -1);
    for (int u = 0; u < U; ++u) {    // mesh/BuildOctree.cu:282-292
        int s = naddr[u] + (ukey[u] & 7);
        lv[D].key[s] = ukey[u];
        lv[D].pidx[s] = upidx[u];
        lv[D].pnum[s] = upnum[u];
        addr_full[s] = naddr[u];
        S.point2node[ufirst[u]] = s;
    }
    for (int s = 0; s < MD; ++s) { lv[D].dnum[s] = 1; lv[D].didx[s] = s; }   // :294-300
    for (int i = 0; i < n; ++i) {   // :302-313 (backward fill)
        int j = i;
        int v = S.point2node[j];
        while (v == -1) { --j; v = S.point2node[j]; }
        S.point2node[i] = v;
    }
    // levels D .. 1 (mesh/BuildOctree.cu:763-841)
    int cur = MD;
    for (int d = D; d >= 1; --d) {
        count[d] = cur;
        int G = cur / 8;
        Level& L1 = lv[d];
        std::vector<int> gk(G, 0), gpidx(G, INT_MAX), gpnum(G, 0), gdidx(G, INT_MAX), gdnum(G, 0),
            gch(8 * (size_t)G, 0);
        const int sh = 3 * (D - d);
        for (int i = 0; i < cur; ++i) {   // :323-357
            if (L1.pnum[i] == 0) {
                int first = i - i % 8, v = first;
                for (int k = 0; k < 8; ++k) { v = first + k; if (L1.pnum[v] != 0) break; }
                int f = addr_full[v] / 8;
                if (L1.dnum[i] != 0) {
                    gdnum[f] += L1.dnum[i];
                    gdidx[f] = std::min(gdidx[f], L1.didx[i]);
                }
            } else {
                int fk = L1.key[i] & ~(7 << sh);
                int f = addr_full[i] / 8;
                int son = (L1.key[i] >> sh) & 7;
                gk[f] = fk;
                gpnum[f] += L1.pnum[i];
                gpidx[f] = std::min(gpidx[f], L1.pidx[i]);
                gdnum[f] += L1.dnum[i];
                gdidx[f] = std::min(gdidx[f], L1.didx[i]);
                gch[8 * (size_t)f + son] = i;
            }
        }
        // parent-level group addresses (:359-375 with depth-1, :796-799)
        std::vector<int> gaddr(G);
        {
            const int sh2 = 3 * (D - (d - 1) + 1);
            int run = 0;
            for (int g = 0; g < G; ++g) {
                int v = (g == 0) ? 0 : (((gk[g - 1] >> sh2) != (gk[g] >> sh2)) ? 8 : 0);
                run += v;
                gaddr[g] = run;
            }
        }
        if (d > 1) {
            int prev = gaddr[G - 1] + 8;
            init_level(lv[d - 1], prev);
            Level& L0 = lv[d - 1];
            if ((int)addr_full.size() < prev) addr_full.resize(prev, 0);
            const int sh3 = 3 * (D - d + 1);
            for (int g = 0; g < G; ++g) {   // :377-390
                int idx = gaddr[g] + ((gk[g] >> sh3) & 7);
                L0.key[idx] = gk[g];
                L0.pidx[idx] = gpidx[g];
                L0.pnum[idx] = gpnum[g];
                L0.didx[idx] = gdidx[g];
                L0.dnum[idx] = gdnum[g];
                for (int k = 0; k < 8; ++k) L0.children[8 * (size_t)idx + k] = gch[8 * (size_t)g + k];
                addr_full[idx] = gaddr[g];
                for (int k = 0; k < 8; ++k) {
                    int ch = gch[8 * (size_t)g + k];
                    // reference quirk: a child at level-local index 0 is treated as absent
                    // and keeps parent 0 (mesh/BuildOctree.cu:386)
                    if (ch != 0) L1.parent[ch] = idx;
                }
            }
            cur = prev;
        } else {
            init_level(lv[0], 1);
            lv[0].key[0] = gk[0];
            lv[0].pidx[0] = gpidx[0];
            lv[0].pnum[0] = gpnum[0];
            lv[0].didx[0] = gdidx[0];
            lv[0].dnum[0] = gdnum[0];
            for (int k = 0; k < 8; ++k) lv[0].children[k] = gch[k];
            cur = 1;
        }
    }
    count[0] = 1;
    base[0] = 0;
    for (int d = 1; d <= D; ++d) base[d] = base[d - 1] + count[d - 1];
    const int M = base[D] + count[D];
    S.M = M;
    S.base = base;
    S.count = count;
    // concatenate (mesh/BuildOctree.cu:843-859)
    S.key.assign(M, 0); S.pidx.assign(M, 0); S.pnum.assign(M, 0); S.parent.assign(M, 0);
    S.didx.assign(M, 0); S.dnum.assign(M, 0); S.children.assign(8 * (size_t)M, 0);
    S.depth.assign(M, 0); S.center.assign(3 * (size_t)M, 0.0f); S.enc.assign(M, 0);
    S.neighs.assign(27 * (size_t)M, 0);
    for (int d = 0; d <= D; ++d)
        for (int i = 0; i < count[d]; ++i) {
            int g = base[d] + i;
            S.key[g] = lv[d].key[i]; S.pidx[g] = lv[d].pidx[i]; S.pnum[g] = lv[d].pnum[i];
            S.parent[g] = lv[d].parent[i]; S.didx[g] = lv[d].didx[i]; S.dnum[g] = lv[d].dnum[i];
            for (int k = 0; k < 8; ++k) S.children[8 * (size_t)g + k] = lv[d].children[8 * (size_t)i + k];
            S.depth[g] = d;
        }
    // global parent / children (mesh/BuildOctree.cu:392-424)
    for (int i = 0; i < M; ++i) {
        if (S.pnum[i] == 0) continue;
        int d = S.depth[i];
        if (i == 0) {
            S.parent[0] = -1;
            for (int k = 0; k < 8; ++k) S.children[k] = k + 1;
        } else {
            S.parent[i] += base[d - 1];
            if (d < D)
                for (int k = 0; k < 8; ++k)
                    if (S.children[8 * (size_t)i + k] != 0) S.children[8 * (size_t)i + k] += base[d + 1];
        }
    }
    // empty siblings (mesh/BuildOctree.cu:426-488)
    for (int g0 = 1; g0 < M; g0 += 8) {
        int v = 0, nowP = 0, nowD = 0, cp = 0;
        for (v = 0; v < 8; ++v)
            if (S.pnum[g0 + v] != 0) { nowP = S.pidx[g0 + v]; nowD = S.didx[g0 + v]; cp = S.parent[g0 + v]; break; }
        if (v == 8) { S.ub_events++; v = 0; }
        int d = S.depth[g0];
        const int sh = 3 * (D - d);
        int baseKey = S.key[g0 + v] - (S.key[g0 + v] & (7 << sh));
        for (int j = 0; j < 8; ++j) {
            int x = g0 + j;
            if (S.pnum[x] == 0) {
                for (int k = 0; k < 8; ++k) S.children[8 * (size_t)x + k] = -1;
            } else {
                int bp = INT_MIN;
                for (int k = 0; k < 8; ++k)
                    if (S.children[8 * (size_t)x + k] > 0) { bp = S.children[8 * (size_t)x + k] - k; break; }
                if (d != D && bp == INT_MIN) {
                    // reference reads an uninitialised register here; the intended first
                    // child slot is the start of the child group at level d+1
                    S.ub_events++;
                    bp = base[d + 1];
                }
                for (int k = 0; k < 8; ++k) S.children[8 * (size_t)x + k] = (d != D) ? bp + k : -1;
            }
            S.key[x] = baseKey + (j << sh);
            S.pidx[x] = nowP;
            nowP += S.pnum[x];
            if (d != D) { S.didx[x] = nowD; nowD += S.dnum[x]; }
            S.parent[x] = cp;
        }
    }
    // depth and centre (mesh/BuildOctree.cu:552-586)
    for (int i = 0; i < M; ++i) {
        int d = S.depth[i];
        float cc[3] = {0.5f, 0.5f, 0.5f};
        float w = 0.25f;
        for (int l = D - 1; l >= D - d; --l) {
            for (int a = 0; a < 3; ++a) {
                if ((S.key[i] >> (3 * l + 2 - a)) & 1) cc[a] += w;
                else cc[a] -= w;
            }
            w /= 2;
        }
        for (int a = 0; a < 3; ++a) S.center[3 * (size_t)i + a] = cc[a];
    }
    // neighbours (mesh/BuildOctree.cu:490-512, :870-892)
    for (int k = 0; k < 27; ++k) S.neighs[k] = (k == 13) ? 0 : -1;
    for (int d = 1; d <= D; ++d)
        for (int i = base[d]; i < base[d] + count[d]; ++i) {
            int son = (S.key[i] >> (3 * (D - d))) & 7;
            int pa = S.parent[i];
            for (int k = 0; k < 27; ++k) {
                int np = S.neighs[27 * (size_t)pa + L.lut_parent[son][k]];
                S.neighs[27 * (size_t)i + k] = (np != -1) ? S.children[8 * (size_t)np + L.lut_child[son][k]] : -1;
            }
        }
    // encoded function index (mesh/BuildOctree.cu:514-550)
    for (int i = 0; i < M; ++i) {
        int d = S.depth[i];
        int idx = ((1 << d) - 1) * (1 + (1 << (D + 1)) + (1 << (2 * (D + 1))));
        for (int l = d; l >= 1; --l) {
            int sx = (S.key[i] >> (3 * (D - l) + 2)) & 1;
            int sy = (S.key[i] >> (3 * (D - l) + 1)) & 1;
            int sz = (S.key[i] >> (3 * (D - l))) & 1;
            idx += sx * (1 << (d - l)) + sy * (1 << (d - l)) * (1 << (D + 1)) +
                   sz * (1 << (d - l)) * (1 << (2 * (D + 1)));
        }
        S.enc[i] = idx;
    }
    return 0;
}

static inline void decode(const State& S, int e, int& ix, int& iy, int& iz) {
    const int o1 = 1 << (S.D + 1), o2 = 1 << (2 * (S.D + 1));
    ix = e % o1;
    iy = (e / o1) % o1;
    iz = e / o2;
}

// ---------------------------------------------------------------------------------
// Vector field (mesh/ComputeVectorField.cu:61-100) and divergence
// (mesh/ComputeNodesDivergence.cu:25-136), FP64.
// ---------------------------------------------------------------------------------
static void compute_field(State& S) {
    const int D = S.D, MD = S.count[D], bD = S.base[D];
    S.vfield.assign(3 * (size_t)MD, 0.0);
    const double s = (double)(1 << D);
#pragma omp parallel for schedule(dynamic, 256)
    for (int o = 0; o < MD; ++o) {
        int node = bD + o;
        int ix, iy, iz;
        decode(S, S.enc[node], ix, iy, iz);   // equals getFunctionIdxNode for depth D
        double cc[3];
        int id3[3] = {ix, iy, iz};
        for (int a = 0; a < 3; ++a) {
            int off = id3[a] + 1 - (1 << D);
            cc[a] = (off + 0.5) / s;
        }
        double v[3] = {0, 0, 0};
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)node + k];
            if (nb == -1) continue;
            for (int j = 0; j < S.pnum[nb]; ++j) {
                int p = S.pidx[nb] + j;
                double w = F64((S.pos[3 * p] - cc[0]) * s) * F64((S.pos[3 * p + 1] - cc[1]) * s) *
                           F64((S.pos[3 * p + 2] - cc[2]) * s);
                for (int a = 0; a < 3; ++a) v[a] += w * S.nrm[3 * p + a];
            }
        }
        for (int a = 0; a < 3; ++a) S.vfield[3 * (size_t)o + a] = v[a];
    }
    S.div.assign(S.M, 0.0);
    const int res = S.tab.res;
    const int bDl = S.base[D];
#pragma omp parallel for schedule(dynamic, 64)
    for (int o = 0; o < S.M; ++o) {
        int ox, oy, oz;
        decode(S, S.enc[o], ox, oy, oz);
        double acc = 0;
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)o + k];
            if (nb == -1) continue;
            for (int j = 0; j < S.dnum[nb]; ++j) {
                int l = S.didx[nb] + j;
                int lx, ly, lz;
                decode(S, S.enc[bDl + l], lx, ly, lz);
                acc += S.vfield[3 * (size_t)l] * S.tab.dff[(size_t)ox + (size_t)res * lx] +
                       S.vfield[3 * (size_t)l + 1] * S.tab.dff[(size_t)oy + (size_t)res * ly] +
                       S.vfield[3 * (size_t)l + 2] * S.tab.dff[(size_t)oz + (size_t)res * lz];
            }
        }
        S.div[o] = acc;
    }
}

// ---------------------------------------------------------------------------------
// Per-depth Laplacian and CG (mesh/solver/LaplacianSolver.cu:27-74,120-267,
// mesh/solver/CGAlgorithm.cu:10-80), FP64.
// ---------------------------------------------------------------------------------
static void solve(State& S) {
    const int D = S.D, res = S.tab.res;
    S.x.assign(S.M, 0.0);
    S.cg_iters.assign(D + 1, 0);
    S.cg_resid.assign(D + 1, 0.0);
    for (int d = 0; d <= D; ++d) {
        const int b = S.base[d], m = S.count[d];
        std::vector<int> rp(m + 1, 0), ci;
        std::vector<double> va;
        ci.reserve(27 * (size_t)m);
        va.reserve(27 * (size_t)m);
        for (int r = 0; r < m; ++r) {
            int o = b + r;
            int ox, oy, oz;
            decode(S, S.enc[o], ox, oy, oz);
            for (int k = 0; k < 27; ++k) {
                int nb = S.neighs[27 * (size_t)o + k];
                if (nb == -1) continue;
                int nx, ny, nz;
                decode(S, S.enc[nb], nx, ny, nz);
                size_t sx = (size_t)ox * res + nx, sy = (size_t)oy * res + ny, sz = (size_t)oz * res + nz;
                double e = S.tab.ff[sx] * S.tab.ff[sy] * S.tab.ff[sz] * (S.tab.d2[sx] + S.tab.d2[sy] + S.tab.d2[sz]);
                if (std::fabs(e) > S.opt.lap_eps) { ci.push_back(nb - b); va.push_back((double)(float)e); }
            }
            rp[r + 1] = (int)ci.size();
        }
        std::vector<double> xx(m, 0.0), rr(m), pp(m, 0.0), ap(m, 0.0);
        for (int r = 0; r < m; ++r) rr[r] = S.div[b + r];
        auto dot = [&](const std::vector<double>& a, const std::vector<double>& c) {
            double s = 0;
            for (int i = 0; i < m; ++i) s += a[i] * c[i];
            return s;
        };
        double r1 = dot(rr, rr), r0 = 0;
        // the reference keeps r.r in a float and compares it with the float tol * tol
        // (mesh/solver/CGAlgorithm.cu:19,36); a fixed iteration count replaces max_iter
        const float tolf = (float)S.opt.cg_tol;
        const double tol2 = (double)(tolf * tolf);
        const int maxit = S.opt.cg_iters > 0 ? S.opt.cg_iters : S.opt.cg_max_iter;
        int k = 1;
        while ((double)(float)r1 > tol2 && k <= maxit) {
            if (k > 1) { double be = r0 != 0 ? r1 / r0 : 0.0; for (int i = 0; i < m; ++i) pp[i] = rr[i] + be * pp[i]; }
            else pp = rr;
            for (int i = 0; i < m; ++i) {
                double s = 0;
                for (int q = rp[i]; q < rp[i + 1]; ++q) s += va[q] * pp[ci[q]];
                ap[i] = s;
            }
            double pap = dot(pp, ap);
            if (pap == 0) break;
            double a = r1 / pap;
            for (int i = 0; i < m; ++i) { xx[i] += a * pp[i]; rr[i] -= a * ap[i]; }
            r0 = r1;
            r1 = dot(rr, rr);
            ++k;
        }
        S.cg_iters[d] = k - 1;
        S.cg_resid[d] = std::sqrt(std::max(r1, 0.0));
        for (int r = 0; r < m; ++r) S.x[b + r] = xx[r];
    }
}

// implicit function at a point, FP64 (mesh/solver/LaplacianSolver.cu:85-118)
template <typename XT>
static double chi64_chain(const State& S, const XT* x, int node, const double p[3]) {
    double val = 0;
    while (node != -1) {
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)node + k];
            if (nb == -1) continue;
            int ix, iy, iz;
            decode(S, S.enc[nb], ix, iy, iz);
            val += (double)x[nb] * basis64(ix, p[0]) * basis64(iy, p[1]) * basis64(iz, p[2]);
        }
        node = S.parent[node];
    }
    return val;
}

static void iso_value(State& S) {
    const int bD = S.base[S.D];
    S.point_chi.assign(S.N, 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < S.N; ++i) {
        double p[3] = {S.pos[3 * i], S.pos[3 * i + 1], S.pos[3 * i + 2]};
        S.point_chi[i] = chi64_chain(S, S.x.data(), bD + S.point2node[i], p);
    }
    double s = 0;
    for (int i = 0; i < S.N; ++i) s += S.point_chi[i];
    S.iso = S.N ? s / S.N : 0.0;
}

// ---------------------------------------------------------------------------------
// Vertex / edge / face arrays (mesh/BuildMeshGeometry.cu:42-400)
// ---------------------------------------------------------------------------------
static inline float sqdist(const float* a, const float* b) {
    float dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;   // exact for the dyadic positions involved
}

// centre of node i as the kernels see it through neighs[13]; when the reference would
// read an uninitialised centre (neighs[13] == -1) the node's own centre is used.
static const float* self_center(State& S, int i) {
    if (S.neighs[27 * (size_t)i + 13] == -1) S.ub_events++;
    return &S.center[3 * (size_t)i];
}

static void build_geometry(State& S) {
    const int M = S.M, D = S.D;
    // vertices
    S.node_vertices.assign(8 * (size_t)M, 0);
    S.verts.clear();
    for (int i = 0; i < M; ++i) {
        int d = S.depth[i];
        float hw = 1.0f / (1 << (d + 1)), w = 1.0f / (1 << d), w2 = w * w;
        const float* nc = self_center(S, i);
        float vp[8][3];
        for (int c = 0; c < 8; ++c) {
            vp[c][0] = nc[0] + (2 * (c & 1) - 1) * hw;
            vp[c][1] = nc[1] + (2 * ((c & 2) >> 1) - 1) * hw;
            vp[c][2] = nc[2] + (2 * ((c & 4) >> 2) - 1) * hw;
        }
        for (int c = 0; c < 8; ++c) {
            int okey = INT_MAX, oidx = -1;
            for (int k = 0; k < 27; ++k) {
                int nb = S.neighs[27 * (size_t)i + k];
                if (nb == -1) continue;
                if ((double)sqdist(vp[c], &S.center[3 * (size_t)nb]) < (double)w2 && okey > S.key[nb]) {
                    okey = S.key[nb];
                    oidx = nb;
                }
            }
            if (oidx == i) {
                VertexRec v{};
                memcpy(v.pos, vp[c], sizeof(v.pos));
                v.owner = i; v.kind = c; v.depth = d; v.nnodes = 0;
                S.verts.push_back(v);
            }
        }
    }
    for (int vi = 0; vi < (int)S.verts.size(); ++vi) {   // maintainVertexNodePointer :108-147
        VertexRec& v = S.verts[vi];
        int ow = v.owner, d = S.depth[ow];
        float w = 1.0f / (1 << d), w2 = w * w;
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)ow + k];
            if (nb == -1) continue;
            const float* c = &S.center[3 * (size_t)nb];
            if ((double)sqdist(v.pos, c) < (double)w2) {
                v.nodes[v.nnodes++] = nb;
                int idx = 0;
                if (c[0] - v.pos[0] < 0) idx |= 1;
                if (c[2] - v.pos[2] < 0) idx |= 4;
                if (c[1] - v.pos[1] < 0) idx += (idx & 1) ? 1 : 3;
                S.node_vertices[8 * (size_t)nb + idx] = vi + 1;
            }
        }
    }
    // edges, D-level nodes only (:149-280)
    S.node_edges.assign(12 * (size_t)M, 0);
    S.edges.clear();
    const int bD = S.base[D], MD = S.count[D];
    auto edge_center = [](const float* nc, int e, float hw, float out[3]) {
        int orient = e >> 2;
        int off[2] = {e & 1, (e & 2) >> 1};
        int dim = 0;
        for (int a = 0; a < 3; ++a) {
            int m = 0;
            if (orient != a) { m = 2 * off[dim] - 1; dim++; }
            out[a] = nc[a] + m * hw;
        }
    };
    for (int o = 0; o < MD; ++o) {
        int i = bD + o;
        float hw = 1.0f / (1 << (D + 1)), w = 1.0f / (1 << D), w2 = w * w;
        const float* nc = self_center(S, i);
        for (int e = 0; e < 12; ++e) {
            float ec[3];
            edge_center(nc, e, hw, ec);
            int okey = INT_MAX, oidx = -1;
            for (int k = 0; k < 27; ++k) {
                int nb = S.neighs[27 * (size_t)i + k];
                if (nb == -1) continue;
                if ((double)sqdist(ec, &S.center[3 * (size_t)nb]) < (double)w2 && okey > S.key[nb]) {
                    okey = S.key[nb];
                    oidx = nb;
                }
            }
            if (oidx == i) {
                EdgeRec r{};
                r.kind = e; r.owner = i; r.nnodes = 0;
                S.edges.push_back(r);
            }
        }
    }
    for (int ei = 0; ei < (int)S.edges.size(); ++ei) {
        EdgeRec& r = S.edges[ei];
        int ow = r.owner;
        float hw = 1.0f / (1 << (D + 1)), w = 1.0f / (1 << D), w2 = w * w;
        const float* nc = self_center(S, ow);
        float ec[3];
        edge_center(nc, r.kind, hw, ec);
        int orient = r.kind >> 2;
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)ow + k];
            if (nb == -1) continue;
            const float* c = &S.center[3 * (size_t)nb];
            if ((double)sqdist(ec, c) < (double)w2) {
                if (r.nnodes < 4) r.nodes[r.nnodes] = nb;
                r.nnodes++;
                int idx = orient << 2, dim = 0;
                for (int a = 0; a < 3; ++a)
                    if (orient != a) { if (c[a] - ec[a] < 0) idx |= (1 << dim); dim++; }
                S.node_edges[12 * (size_t)nb + idx] = ei + 1;
            }
        }
    }
    // faces, all nodes (:282-400)
    S.node_faces.assign(6 * (size_t)M, 0);
    S.faces.clear();
    for (int i = 0; i < M; ++i) {
        int d = S.depth[i];
        float hw = 1.0f / (1 << (d + 1)), w = 1.0f / (1 << d), w2 = w * w;
        const float* nc = self_center(S, i);
        int son = (S.key[i] >> (3 * (D - d))) & 7;
        for (int f = 0; f < 6; ++f) {
            float fc[3] = {nc[0], nc[1], nc[2]};
            fc[f >> 1] += (2 * (f & 1) - 1) * hw;
            int okey = INT_MAX, oidx = -1;
            for (int k = 0; k < 27; ++k) {
                int nb = S.neighs[27 * (size_t)i + k];
                if (nb == -1) continue;
                if ((double)sqdist(fc, &S.center[3 * (size_t)nb]) < (double)w2 && okey > S.key[nb]) {
                    okey = S.key[nb];
                    oidx = nb;
                }
            }
            if (oidx == i) {
                FaceRec r{};
                r.kind = f; r.owner = i; r.nnodes = 0;
                if (S.parent[i] == -1) r.has_parent_face = -1;
                else r.has_parent_face = (L.parent_face_kind[son][f] != -1) ? 1 : -1;
                S.faces.push_back(r);
            }
        }
    }
    for (int fi = 0; fi < (int)S.faces.size(); ++fi) {
        FaceRec& r = S.faces[fi];
        int ow = r.owner, d = S.depth[ow];
        float hw = 1.0f / (1 << (d + 1)), w = 1.0f / (1 << d), w2 = w * w;
        const float* nc = self_center(S, ow);
        float fc[3] = {nc[0], nc[1], nc[2]};
        int orient = r.kind >> 1;
        fc[orient] += (2 * (r.kind & 1) - 1) * hw;
        for (int k = 0; k < 27; ++k) {
            int nb = S.neighs[27 * (size_t)ow + k];
            if (nb == -1) continue;
            const float* c = &S.center[3 * (size_t)nb];
            if ((double)sqdist(fc, c) < (double)w2) {
                if (r.nnodes < 2) r.nodes[r.nnodes] = nb;
                r.nnodes++;
                int idx = orient << 1;
                if (c[orient] - fc[orient] < 0) idx++;
                S.node_faces[6 * (size_t)nb + idx] = fi + 1;
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Marching cubes (mesh/ComputeTriangleIndices.cu) — templated on the value type:
// double for the FP64 oracle, float for the mirror of the device evaluation.
// ---------------------------------------------------------------------------------
template <typename T> struct Eval;
template <> struct Eval<double> {
    static double basis(int idx, double x) { return basis64(idx, x); }
    static double term(double xv, double fx, double fy, double fz) { return xv * fx * fy * fz; }
    static double add(double a, double b) { return a + b; }
};
template <> struct Eval<float> {
    static float basis(int idx, float x) { return basis32(idx, x); }
    static float term(float xv, float fx, float fy, float fz) {
        float t = xv * fx; t = t * fy; t = t * fz; return t;
    }
    static float add(float a, float b) { return a + b; }
};

// One insertion of a vertex buffer + triangle buffer (insertTriangle, :1247-1282).
template <typename T>
static bool insert_triangles(State& S, const std::vector<float>& vb, const std::vector<int>& tb) {
    int prev = (int)(S.mesh_v.size() / 3);
    int nv = (int)(vb.size() / 3), nt = (int)(tb.size() / 3);
    int kept_v = 0;
    std::vector<float> addv;
    for (int i = 0; i < nv; ++i) {
        if (std::fabs(vb[3 * i]) < 1e-6f) continue;   // markValidMeshVertexIndex :1170-1181
        addv.insert(addv.end(), vb.begin() + 3 * i, vb.begin() + 3 * i + 3);
        kept_v++;
    }
    std::vector<int> addt;
    for (int i = 0; i < nt; ++i) {
        int t[3];
        bool ok = true;
        for (int a = 0; a < 3; ++a) {
            t[a] = tb[3 * i + a] + prev;
            if (t[a] < 0 || t[a] >= nv + prev) ok = false;
        }
        if (ok) addt.insert(addt.end(), t, t + 3);
    }
    if (prev + kept_v > S.opt.vert_cap || (int)(S.mesh_t.size() / 3) + (int)(addt.size() / 3) > S.opt.tri_cap) {
        S.status = 1;
        return false;
    }
    S.mesh_v.insert(S.mesh_v.end(), addv.begin(), addv.end());
    S.mesh_t.insert(S.mesh_t.end(), addt.begin(), addt.end());
    S.mesh_stage_v.push_back(kept_v);
    S.mesh_stage_t.push_back((int)(addt.size() / 3));
    return true;
}

template <typename T>
static inline void interp(const float* p1, const float* p2, int dim, T v1, T v2, float* out) {
    for (int a = 0; a < 3; ++a) out[a] = p1[a];
    T pivot = v1 / (v1 - v2);
    T other = (T)1 - pivot;
    T a = (T)p2[dim] * pivot;
    T b = (T)p1[dim] * other;
    out[dim] = (float)(a + b);
}

// Subdivision-space node (EasyOctNode, mesh/OctNode.cuh:44-77)
struct SubNode {
    int key, parent;
    int children[8];
    int neighs[27];
    int vertices[8];
    int edges[12];
};

template <typename T>
struct MeshRun {
    State& S;
    const T* x;
    T iso;
    std::vector<int> ch;      // working copy of the children array (modified by subdivision)
    explicit MeshRun(State& s, const T* xx, T is) : S(s), x(xx), iso(is), ch(s.children) {}

    // implicit value at an octree vertex (ComputeVertexImplicitFunctionValueKernel :346-399)
    T vertex_value(const VertexRec& v) {
        typedef Eval<T> E;
        T val = 0;
        int now = v.owner;
        const int D = S.D;
        if (now > 0) {
            T p[3] = {(T)v.pos[0], (T)v.pos[1], (T)v.pos[2]};
            auto node_sum = [&](int node) {
                for (int k = 0; k < 27; ++k) {
                    int nb = S.neighs[27 * (size_t)node + k];
                    if (nb == -1) continue;
                    int ix, iy, iz;
                    decode(S, S.enc[nb], ix, iy, iz);
                    val = E::add(val, E::term((T)x[nb], E::basis(ix, p[0]), E::basis(iy, p[1]), E::basis(iz, p[2])));
                }
            };
            while (now != -1) { node_sum(now); now = S.parent[now]; }
            now = v.owner;
            int d = v.depth;
            int ec = L.children_vertex_kind[v.kind];
            while (d < D) {
                d++;
                now = S.children[8 * (size_t)now + ec];
                if (now == -1) break;
                node_sum(now);
            }
        }
        return val - iso;
    }

    void run() {
        const int D = S.D, M = S.M, bD = S.base[D], MD = S.count[D];
        S.mesh_v.clear(); S.mesh_t.clear(); S.mesh_stage_v.clear(); S.mesh_stage_t.clear();
        S.status = 0;
        // Step 1: vertex values
        std::vector<T> vv(S.verts.size());
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < (int)S.verts.size(); ++i) vv[i] = vertex_value(S.verts[i]);
        if (sizeof(T) == 8) { S.vvalue.assign(vv.begin(), vv.end()); }
        else { S.vvalue32.resize(vv.size()); for (size_t i = 0; i < vv.size(); ++i) S.vvalue32[i] = (float)vv[i]; }
        // Step 2: crossing edges (:401-422) and addresses
        const int E = (int)S.edges.size();
        std::vector<int> vexn(E), vexa(E);
        S.edge_cross.assign(E, 0);
        int run = 0;
        for (int e = 0; e < E; ++e) {
            const EdgeRec& r = S.edges[e];
            int v1 = S.node_vertices[8 * (size_t)r.owner + L.edge_vertex[r.kind][0]] - 1;
            int v2 = S.node_vertices[8 * (size_t)r.owner + L.edge_vertex[r.kind][1]] - 1;
            vexn[e] = (vv[v1] * vv[v2] <= 0) ? 1 : 0;
            S.edge_cross[e] = vexn[e];
            vexa[e] = run;
            run += vexn[e];
        }
        const int nvex = run;
        // Step 3: cube classes (:424-438)
        std::vector<int> trin(MD), tria(MD);
        S.cube_class.assign(MD, 0);
        run = 0;
        for (int o = 0; o < MD; ++o) {
            int node = bD + o, cls = 0;
            for (int c = 0; c < 8; ++c)
                if (vv[S.node_vertices[8 * (size_t)node + c] - 1] < 0) cls |= 1 << c;
            S.cube_class[o] = cls;
            trin[o] = kMcTriangleCountInit[cls];
            tria[o] = run;
            run += trin[o];
        }
        const int ntri = run;
        // Step 4: intersection points (:440-474)
        std::vector<float> vbuf(3 * (size_t)nvex);
        for (int e = 0; e < E; ++e) {
            if (!vexn[e]) continue;
            const EdgeRec& r = S.edges[e];
            int v1 = S.node_vertices[8 * (size_t)r.owner + L.edge_vertex[r.kind][0]] - 1;
            int v2 = S.node_vertices[8 * (size_t)r.owner + L.edge_vertex[r.kind][1]] - 1;
            interp<T>(S.verts[v1].pos, S.verts[v2].pos, r.kind >> 2, vv[v1], vv[v2], &vbuf[3 * (size_t)vexa[e]]);
        }
        // Step 5: triangles + face intersection marks (:476-526)
        std::vector<int> tbuf(3 * (size_t)ntri);
        std::vector<int> hsi(S.faces.size(), 0);
        for (int o = 0; o < MD; ++o) {
            int node = bD + o, cls = S.cube_class[o];
            int ehv[12] = {0};
            for (int t = 0; t < trin[o]; ++t)
                for (int a = 0; a < 3; ++a) {
                    int e = mc_tri_edge(cls, 3 * t + a);
                    ehv[e] = 1;
                    tbuf[3 * (size_t)(tria[o] + t) + a] = vexa[S.node_edges[12 * (size_t)node + e] - 1];
                }
            for (int f = 0; f < 6; ++f) {
                int mark = 0;
                for (int j = 0; j < 4; ++j) mark |= ehv[L.face_edges[f][j]];
                if (!mark) continue;
                int pn = S.parent[node];
                int cf = S.node_faces[6 * (size_t)node + f] - 1;
                hsi[cf] = 1;
                while (S.faces[cf].has_parent_face != -1) {
                    cf = S.node_faces[6 * (size_t)pn + f] - 1;
                    pn = S.parent[pn];
                    hsi[cf] = 1;
                }
            }
        }
        if (!insert_triangles<T>(S, vbuf, tbuf)) return;
        // Step 6: leaves at coarser depths (:555-587) and subdivision roots (:1284-1346)
        S.has_triangle.assign(bD, 0);
        S.has_intersection.assign(bD, 0);
        S.sub_roots.clear();
        S.sub_root_depth.clear();
        for (int i = 0; i < bD; ++i) {
            int s = (vv[S.node_vertices[8 * (size_t)i] - 1] < 0) ? -1 : 1, ht = 0;
            for (int c = 1; c < 8; ++c)
                if (s * vv[S.node_vertices[8 * (size_t)i + c] - 1] < 0) { ht = 1; break; }
            int hi = 0;
            for (int f = 0; f < 6; ++f)
                if (hsi[S.node_faces[6 * (size_t)i + f] - 1]) { hi = 1; break; }
            S.has_triangle[i] = ht;
            S.has_intersection[i] = hi;
            bool leaf = true;
            for (int k = 0; k < 8; ++k) if (S.children[8 * (size_t)i + k] != -1) leaf = false;
            if (leaf && (ht || hi)) {
                int self = S.neighs[27 * (size_t)i + 13];
                if (self == -1) { S.ub_events++; self = i; }
                S.sub_roots.push_back(i);
                S.sub_root_depth.push_back(S.depth[self]);
            }
        }
        // Step 7: coarser roots one at a time (:1475-1799)
        const int finer = D - 4;   // MAX_DEPTH_OCTREE - COARSER_DIVERGENCE_LEVEL_NUM
        int coarse_depth_seen = -1;
        for (size_t r = 0; r < S.sub_roots.size(); ++r) {
            int rd = S.sub_root_depth[r];
            if (rd >= finer) break;
            if (coarse_depth_seen != -1 && coarse_depth_seen != rd) {
                // reference quirk: the per-depth subtree offsets are recomputed from stale
                // values once roots of a second depth appear (:1512-1514); the intended
                // offsets are used here.
                S.ub_events++;
            }
            coarse_depth_seen = rd;
            if (!coarse_root(r)) return;
        }
        // Step 8: finer roots batched per depth (:1801-2194)
        for (int d = std::max(finer, 0); d < D; ++d) {
            std::vector<int> roots;
            for (size_t r = 0; r < S.sub_roots.size(); ++r)
                if (S.sub_root_depth[r] == d) roots.push_back((int)r);
            if (roots.empty()) continue;
            if (!finer_batch(d, roots)) return;
        }
    }

    // ---- subdivision helpers -------------------------------------------------------
    // neighbours of a subdivision-space node (computeRebuildNeighbor :669-696)
    void rebuild_neighbours(std::vector<SubNode>& A, int idx, int d) {
        const int NA = S.M;
        SubNode& n = A[idx];
        int son = (n.key >> (3 * (S.D - d))) & 7;
        for (int k = 0; k < 27; ++k) {
            int pa = n.parent, np;
            if (pa < NA) np = S.neighs[27 * (size_t)pa + L.lut_parent[son][k]];
            else np = A[pa - NA].neighs[L.lut_parent[son][k]];
            if (np != -1) {
                if (np < NA) n.neighs[k] = ch[8 * (size_t)np + L.lut_child[son][k]];
                else n.neighs[k] = A[np - NA].children[L.lut_child[son][k]];
            } else n.neighs[k] = -1;
        }
    }

    // marching cubes inside subdivision space; `lvl_off` / `lvl_cnt` delimit the D-level
    // nodes; `replace(nb)` maps a subdivision-space neighbour to an octree node or -1
    template <typename Rep>
    bool sub_mc(std::vector<SubNode>& A, std::vector<float>& Actr, int lvl_off, int lvl_cnt, Rep replace,
                bool stop_if_no_vertex) {
        const int NA = S.M, D = S.D;
        typedef Eval<T> E;
        const float hw = 1.0f / (1 << (D + 1)), w = 1.0f / (1 << D), w2 = w * w;
        auto nctr = [&](int nb) -> const float* {
            return nb < NA ? &S.center[3 * (size_t)nb] : &Actr[3 * (size_t)(nb - NA)];
        };
        // vertices (initSubdivideVertexOwner :698-763)
        std::vector<VertexRec> sv;
        for (int o = 0; o < lvl_cnt; ++o) {
            int off = lvl_off + o;
            const SubNode& n = A[off];
            const float* nc = &Actr[3 * (size_t)(n.neighs[13] - NA)];
            float vp[8][3];
            for (int c = 0; c < 8; ++c) {
                vp[c][0] = nc[0] + (2 * (c & 1) - 1) * hw;
                vp[c][1] = nc[1] + (2 * ((c & 2) >> 1) - 1) * hw;
                vp[c][2] = nc[2] + (2 * ((c & 4) >> 2) - 1) * hw;
            }
            for (int c = 0; c < 8; ++c) {
                int okey = INT_MAX, oidx = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = n.neighs[k];
                    if (nb == -1 || nb < NA) continue;
                    if ((double)sqdist(vp[c], nctr(nb)) < (double)w2) {
                        int nk = A[nb - NA].key;
                        if (okey > nk) { okey = nk; oidx = nb; }
                    }
                }
                if (oidx == NA + off) {
                    VertexRec v{};
                    memcpy(v.pos, vp[c], sizeof(v.pos));
                    v.owner = oidx; v.kind = c; v.depth = D; v.nnodes = 0;
                    sv.push_back(v);
                }
            }
        }
        if (sv.empty()) return false;   // :1571-1574 / :1970-1981
        for (int vi = 0; vi < (int)sv.size(); ++vi) {   // :765-810
            VertexRec& v = sv[vi];
            const SubNode& n = A[v.owner - NA];
            for (int k = 0; k < 27; ++k) {
                int nb = n.neighs[k];
                if (nb == -1) continue;
                const float* c = nctr(nb);
                if ((double)sqdist(v.pos, c) < (double)w2) {
                    int idx = 0;
                    if (c[0] - v.pos[0] < 0) idx |= 1;
                    if (c[2] - v.pos[2] < 0) idx |= 4;
                    if (c[1] - v.pos[1] < 0) idx += (idx & 1) ? 1 : 3;
                    if (nb >= NA) A[nb - NA].vertices[idx] = vi + 1;
                }
            }
        }
        // edges (:812-949)
        std::vector<EdgeRec> se;
        for (int o = 0; o < lvl_cnt; ++o) {
            int off = lvl_off + o;
            const SubNode& n = A[off];
            const float* nc = &Actr[3 * (size_t)(n.neighs[13] - NA)];
            for (int e = 0; e < 12; ++e) {
                float ec[3];
                int orient = e >> 2, of[2] = {e & 1, (e & 2) >> 1}, dim = 0;
                for (int a = 0; a < 3; ++a) {
                    int m = 0;
                    if (orient != a) { m = 2 * of[dim] - 1; dim++; }
                    ec[a] = nc[a] + m * hw;
                }
                int okey = INT_MAX, oidx = -1;
                for (int k = 0; k < 27; ++k) {
                    int nb = n.neighs[k];
                    if (nb == -1 || nb < NA) continue;
                    if ((double)sqdist(ec, nctr(nb)) < (double)w2) {
                        int nk = A[nb - NA].key;
                        if (okey > nk) { okey = nk; oidx = nb; }
                    }
                }
                if (oidx == off + NA) { EdgeRec r{}; r.kind = e; r.owner = oidx; se.push_back(r); }
            }
        }
        if (se.empty()) return false;   // :1615-1619 / :2018-2030
        for (int ei = 0; ei < (int)se.size(); ++ei) {
            EdgeRec& r = se[ei];
            const SubNode& n = A[r.owner - NA];
            const float* nc = nctr(n.neighs[13]);
            float ec[3];
            int orient = r.kind >> 2, of[2] = {r.kind & 1, (r.kind & 2) >> 1}, dim = 0;
            for (int a = 0; a < 3; ++a) {
                int m = 0;
                if (orient != a) { m = 2 * of[dim] - 1; dim++; }
                ec[a] = nc[a] + m * hw;
            }
            for (int k = 0; k < 27; ++k) {
                int nb = n.neighs[k];
                if (nb == -1) continue;
                const float* c = nctr(nb);
                if ((double)sqdist(ec, c) < (double)w2) {
                    int idx = orient << 2, dd = 0;
                    for (int a = 0; a < 3; ++a)
                        if (orient != a) { if (c[a] - ec[a] < 0) idx |= (1 << dd); dd++; }
                    if (nb >= NA) A[nb - NA].edges[idx] = ei + 1;
                }
            }
        }
        // implicit values (:956-1038): x = 0 inside subdivision space
        std::vector<T> svv(sv.size());
        for (int vi = 0; vi < (int)sv.size(); ++vi) {
            const VertexRec& v = sv[vi];
            T val = 0;
            int now = v.owner;
            T p[3] = {(T)v.pos[0], (T)v.pos[1], (T)v.pos[2]};
            if (now > 0) {
                while (now != -1) {
                    for (int k = 0; k < 27; ++k) {
                        int nb = (now < NA) ? S.neighs[27 * (size_t)now + k] : A[now - NA].neighs[k];
                        if (nb == -1) continue;
                        nb = replace(nb);
                        if (nb < 0 || nb >= NA) continue;
                        int ix, iy, iz;
                        decode(S, S.enc[nb], ix, iy, iz);
                        val = E::add(val, E::term((T)x[nb], E::basis(ix, p[0]), E::basis(iy, p[1]), E::basis(iz, p[2])));
                    }
                    now = (now < NA) ? S.parent[now] : A[now - NA].parent;
                }
            }
            svv[vi] = val - iso;
        }
        // crossings / cubes / points / triangles (:1040-1096, :528-553)
        const int SE = (int)se.size();
        std::vector<int> vexn(SE, 0), vexa(SE, 0);
        int run = 0;
        for (int e = 0; e < SE; ++e) {
            const SubNode& n = A[se[e].owner - NA];
            int v1 = n.vertices[L.edge_vertex[se[e].kind][0]] - 1;
            int v2 = n.vertices[L.edge_vertex[se[e].kind][1]] - 1;
            vexn[e] = (svv[v1] * svv[v2] <= 0) ? 1 : 0;
            vexa[e] = run;
            run += vexn[e];
        }
        const int nvex = run;
        if (nvex == 0 && stop_if_no_vertex) return false;
        std::vector<int> trin(lvl_cnt), tria(lvl_cnt), cls(lvl_cnt);
        run = 0;
        for (int o = 0; o < lvl_cnt; ++o) {
            const SubNode& n = A[lvl_off + o];
            int c = 0;
            for (int k = 0; k < 8; ++k) if (svv[n.vertices[k] - 1] < 0) c |= 1 << k;
            cls[o] = c;
            trin[o] = kMcTriangleCountInit[c];
            tria[o] = run;
            run += trin[o];
        }
        const int ntri = run;
        std::vector<float> vbuf(3 * (size_t)nvex);
        for (int e = 0; e < SE; ++e) {
            if (!vexn[e]) continue;
            const SubNode& n = A[se[e].owner - NA];
            int v1 = n.vertices[L.edge_vertex[se[e].kind][0]] - 1;
            int v2 = n.vertices[L.edge_vertex[se[e].kind][1]] - 1;
            interp<T>(sv[v1].pos, sv[v2].pos, se[e].kind >> 2, svv[v1], svv[v2], &vbuf[3 * (size_t)vexa[e]]);
        }
        std::vector<int> tbuf(3 * (size_t)ntri);
        for (int o = 0; o < lvl_cnt; ++o) {
            const SubNode& n = A[lvl_off + o];
            for (int t = 0; t < trin[o]; ++t)
                for (int a = 0; a < 3; ++a) {
                    int e = mc_tri_edge(cls[o], 3 * t + a);
                    tbuf[3 * (size_t)(tria[o] + t) + a] = vexa[n.edges[e] - 1];
                }
        }
        return insert_triangles<T>(S, vbuf, tbuf) || S.status == 0;
    }

    static void node_center(int key, int d, int D, float out[3]) {
        out[0] = out[1] = out[2] = 0.5f;
        float w = 0.25f;
        for (int l = D - 1; l >= D - d; --l) {
            for (int a = 0; a < 3; ++a) {
                if ((key >> (3 * l + 2 - a)) & 1) out[a] += w;
                else out[a] -= w;
            }
            w /= 2;
        }
    }

    bool coarse_root(size_t r) {
        const int D = S.D, NA = S.M;
        int node = S.sub_roots[r];
        int rd = S.sub_root_depth[r];
        int root_index = S.neighs[27 * (size_t)node + 13];
        if (root_index == -1) root_index = node;
        int rparent = S.parent[node], rkey = S.key[node];
        int rson = (rkey >> (3 * (D - rd))) & 7;
        int size = 0;
        std::vector<int> lvl_off(D + 2, 0), lvl_cnt(D + 2, 0);
        for (int d = rd, c = 1; d <= D; ++d, c <<= 3) { lvl_off[d] = size; lvl_cnt[d] = c; size += c; }
        std::vector<SubNode> A(size);
        std::vector<float> Actr(3 * (size_t)size);
        memset(A.data(), 0, sizeof(SubNode) * A.size());
        ch[8 * (size_t)rparent + rson] = NA;
        A[0].parent = rparent;
        for (int idx = 0; idx < size; ++idx) {   // singleRebuildArray :599-635
            int d = rd;
            while (!(idx >= lvl_off[d] && idx < lvl_off[d] + lvl_cnt[d])) d++;
            int rel = idx - lvl_off[d];
            if (d < D) for (int k = 0; k < 8; ++k) A[idx].children[k] = NA + lvl_off[d + 1] + (rel << 3) + k;
            else for (int k = 0; k < 8; ++k) A[idx].children[k] = -1;
            if (idx != 0) A[idx].parent = NA + lvl_off[d - 1] + (rel >> 3);
            A[idx].key = rkey | (rel << (3 * (D - d)));
            node_center(A[idx].key, d, D, &Actr[3 * (size_t)idx]);
        }
        for (int d = rd; d <= D; ++d)
            for (int i = 0; i < lvl_cnt[d]; ++i) rebuild_neighbours(A, lvl_off[d] + i, d);
        auto rep = [&](int nb) { return nb == NA ? root_index : nb; };
        bool ok = sub_mc(A, Actr, lvl_off[D], lvl_cnt[D], rep, true);
        ch[8 * (size_t)rparent + rson] = root_index;
        return S.status == 0 || ok;
    }

    bool finer_batch(int rd, const std::vector<int>& roots) {
        const int D = S.D, NA = S.M;
        const int n = (int)roots.size();
        std::vector<int> lvl_off(D + 2, 0), lvl_cnt(D + 2, 0);
        int size = 0;
        for (int d = 1; d <= D; ++d) {
            lvl_cnt[d] = (d >= rd) ? n << (3 * (d - rd)) : 0;
            lvl_off[d] = size;
            size += lvl_cnt[d];
        }
        std::vector<SubNode> A(size);
        memset(A.data(), 0, sizeof(SubNode) * A.size());
        std::vector<float> Actr(3 * (size_t)size, 0.0f);
        std::vector<int> replace_id(size, 0), is_root(size, 0);
        for (int q = 0; q < n; ++q) {   // wholeRebuildArray :1110-1168
            int node = S.sub_roots[roots[q]];
            int now = lvl_off[rd] + q;
            SubNode& rn = A[now];
            rn.key = S.key[node];
            rn.parent = S.parent[node];
            for (int k = 0; k < 8; ++k) { rn.children[k] = ch[8 * (size_t)node + k]; rn.vertices[k] = S.node_vertices[8 * (size_t)node + k]; }
            for (int k = 0; k < 27; ++k) rn.neighs[k] = S.neighs[27 * (size_t)node + k];
            for (int k = 0; k < 12; ++k) rn.edges[k] = S.node_edges[12 * (size_t)node + k];
            int rid = rn.neighs[13];
            if (rid == -1) rid = node;
            rn.neighs[13] = NA + now;
            replace_id[now] = rid;
            is_root[now] = 1;
            node_center(rn.key, rd, D, &Actr[3 * (size_t)now]);
            int son = (rn.key >> (3 * (D - rd))) & 7;
            ch[8 * (size_t)rn.parent + son] = NA + now;   // not restored by the reference
            int per = 1;
            for (int d = rd + 1; d <= D; ++d) {
                int cnow = lvl_off[d] + q * per * 8;
                for (int j = 0; j < per * 8; j += 8) {
                    int pidx = lvl_off[d - 1] + q * per + j / 8;
                    int pg = A[pidx].neighs[13];
                    int pk = A[pidx].key;
                    for (int k = 0; k < 8; ++k) {
                        int t = cnow + j + k;
                        A[t].parent = pg;
                        A[t].key = pk | (k << (3 * (D - d)));
                        A[t].neighs[13] = NA + t;
                        replace_id[t] = rid;
                        node_center(A[t].key, d, D, &Actr[3 * (size_t)t]);
                        A[pidx].children[k] = NA + t;
                    }
                }
                per *= 8;
            }
        }
        for (int d = std::max(D - 4, 0); d <= D; ++d)
            for (int i = 0; i < lvl_cnt[d]; ++i) rebuild_neighbours(A, lvl_off[d] + i, d);
        auto rep = [&](int nb) {
            if (nb >= NA && is_root[nb - NA]) return replace_id[nb - NA];
            return nb;
        };
        bool ok = sub_mc(A, Actr, lvl_off[D], lvl_cnt[D], rep, false);
        return ok || S.status == 0;
    }
};

// colour / normal transfer (mesh/DrawMesh.cu:102-214).  The reference searches all
// samples per vertex; the oracle finds the same exact 4 nearest samples (ties towards the
// lower sample index) through a uniform grid.
static void transfer(State& S) {
    const int V = (int)(S.mesh_v.size() / 3), T = (int)(S.mesh_t.size() / 3);
    S.vcolor.assign(3 * (size_t)V, 0.0f);
    S.vnormal.assign(3 * (size_t)V, 0.0f);
    const int G = 64;
    auto cell = [&](float v) { int c = (int)std::floor(v * G); return c < 0 ? 0 : (c >= G ? G - 1 : c); };
    std::vector<int> start((size_t)G * G * G + 1, 0), items(S.N);
    for (int i = 0; i < S.N; ++i) {
        size_t c = ((size_t)cell(S.pos[3 * i]) * G + cell(S.pos[3 * i + 1])) * G + cell(S.pos[3 * i + 2]);
        start[c + 1]++;
    }
    for (size_t c = 0; c < (size_t)G * G * G; ++c) start[c + 1] += start[c];
    {
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (int i = 0; i < S.N; ++i) {
            size_t c = ((size_t)cell(S.pos[3 * i]) * G + cell(S.pos[3 * i + 1])) * G + cell(S.pos[3 * i + 2]);
            items[fill[c]++] = i;
        }
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int v = 0; v < V; ++v) {
        const float* q = &S.mesh_v[3 * (size_t)v];
        float bd[4] = {1e6f, 1e6f, 1e6f, 1e6f};
        int bi[4] = {0, 0, 0, 0};
        int cq[3] = {cell(q[0]), cell(q[1]), cell(q[2])};
        for (int r = 0; r <= G; ++r) {
            // all samples within distance r/G of q have been visited after ring r
            if (r > 0) {
                double lim = (double)(r - 1) / G;
                if (bd[3] < 1e6f && (double)bd[3] < lim * lim) break;
            }
            for (int a = cq[0] - r; a <= cq[0] + r; ++a)
                for (int b = cq[1] - r; b <= cq[1] + r; ++b)
                    for (int c = cq[2] - r; c <= cq[2] + r; ++c) {
                        if (a < 0 || b < 0 || c < 0 || a >= G || b >= G || c >= G) continue;
                        if (std::max(std::abs(a - cq[0]), std::max(std::abs(b - cq[1]), std::abs(c - cq[2]))) != r) continue;
                        size_t cc = ((size_t)a * G + b) * G + c;
                        for (int t = start[cc]; t < start[cc + 1]; ++t) {
                            int i = items[t];
                            float dx = q[0] - S.pos[3 * i], dy = q[1] - S.pos[3 * i + 1], dz = q[2] - S.pos[3 * i + 2];
                            float d2 = dx * dx + dy * dy + dz * dz;
                            if (d2 < bd[3] || (d2 == bd[3] && i < bi[3])) {
                                int k = 3;
                                while (k > 0 && (d2 < bd[k - 1] || (d2 == bd[k - 1] && i < bi[k - 1]))) {
                                    bd[k] = bd[k - 1]; bi[k] = bi[k - 1]; --k;
                                }
                                bd[k] = d2; bi[k] = i;
                            }
                        }
                    }
        }
        double sum = (double)bd[0] + bd[1] + bd[2] + bd[3];
        double inv = sum > 0 ? 1.0 / sum : 0.0;
        for (int a = 0; a < 3; ++a) {
            double c = 0;
            // reference quirk: weights proportional to the squared distance
            for (int k = 0; k < 4; ++k) c += S.color[3 * (size_t)bi[k] + a] * (bd[k] * inv);
            S.vcolor[3 * (size_t)v + a] = (float)c;
        }
    }
    std::vector<double> acc(3 * (size_t)V, 0.0);
    std::vector<int> cnt(V, 0);
    for (int t = 0; t < T; ++t) {
        const int* tr = &S.mesh_t[3 * (size_t)t];
        double o[3], a[3], b[3];
        for (int k = 0; k < 3; ++k) {
            o[k] = S.mesh_v[3 * (size_t)tr[0] + k];
            a[k] = S.mesh_v[3 * (size_t)tr[1] + k] - o[k];
            b[k] = S.mesh_v[3 * (size_t)tr[2] + k] - o[k];
        }
        double nx = a[1] * b[2] - a[2] * b[1], ny = a[2] * b[0] - a[0] * b[2], nz = a[0] * b[1] - a[1] * b[0];
        double l = std::sqrt(nx * nx + ny * ny + nz * nz);
        if (l > 0) { nx /= l; ny /= l; nz /= l; } else { nx = ny = nz = 0; }
        for (int k = 0; k < 3; ++k) {
            acc[3 * (size_t)tr[k]] += nx; acc[3 * (size_t)tr[k] + 1] += ny; acc[3 * (size_t)tr[k] + 2] += nz;
            cnt[tr[k]]++;
        }
    }
    for (int v = 0; v < V; ++v) {
        if (!cnt[v]) continue;
        double x = acc[3 * (size_t)v] / cnt[v], y = acc[3 * (size_t)v + 1] / cnt[v], z = acc[3 * (size_t)v + 2] / cnt[v];
        double l = std::sqrt(x * x + y * y + z * z);
        if (l > 0) { x /= l; y /= l; z /= l; }
        S.vnormal[3 * (size_t)v] = (float)x; S.vnormal[3 * (size_t)v + 1] = (float)y; S.vnormal[3 * (size_t)v + 2] = (float)z;
    }
}

}  // namespace oracle

// ---------------------------------------------------------------------------------
// C ABI for ctypes
// ---------------------------------------------------------------------------------
using namespace oracle;

struct OracleHandle {
    State S;
    double lap_eps = (double)1e-6f;
    std::map<std::string, std::vector<char>> scratch;
    Tables given;            // tables supplied by the caller (res 0: none)
};

extern "C" {

void* oro_create(void) { return new OracleHandle(); }
void oro_destroy(void* h) { delete (OracleHandle*)h; }

// Drop threshold of the Laplacian entries for the following runs (the reference's 1e-6
// by default; 0 keeps every entry).
void oro_set_lap_eps(void* h, double eps) { ((OracleHandle*)h)->lap_eps = eps; }

// Tables for the following runs instead of the exact integrals: `count` entries (i, j) of
// <F,F>, <F',F>, <F',F'> (every other entry zero) for runs whose depth gives this `res`
// (2^(depth+1) - 1).  Used to solve on the reference's own tables (mesh/FunctionData.h
// setDotTables, float polynomial arithmetic).  res = 0 goes back to the exact tables.
void oro_set_tables(void* hp, int res, int count, const int* i, const int* j, const double* ff, const double* dff,
                    const double* d2) {
    OracleHandle* h = (OracleHandle*)hp;
    Tables& t = h->given;
    t.res = res;
    t.ff.assign((size_t)res * res, 0.0);
    t.dff.assign((size_t)res * res, 0.0);
    t.d2.assign((size_t)res * res, 0.0);
    for (int k = 0; k < count; ++k) {
        const size_t at = (size_t)i[k] + (size_t)res * j[k];
        t.ff[at] = ff[k];
        t.dff[at] = dff[k];
        t.d2[at] = d2[k];
    }
}

// Runs the pipeline up to `stop_after` (1 octree, 2 field, 3 solve, 4 mesh, 5 colour).
// cg_iters > 0 selects a fixed iteration count per depth; otherwise CG stops when
// ||r|| <= cg_tol or after cg_max_iter iterations.  Returns 0, 1 (capacity) or 2.
int oro_run(void* hp, const float* xyz, const float* nrm, const float* rgb, int n, int depth, int cg_iters,
            double cg_tol, int cg_max_iter, int stop_after, int vert_cap, int tri_cap) {
    OracleHandle* h = (OracleHandle*)hp;
    State& S = h->S;
    S = State();
    S.opt.depth = depth;
    S.opt.cg_iters = cg_iters;
    S.opt.cg_tol = cg_tol;
    S.opt.cg_max_iter = cg_max_iter;
    S.opt.stop_after = stop_after;
    S.opt.lap_eps = h->lap_eps;
    if (vert_cap > 0) S.opt.vert_cap = vert_cap;
    if (tri_cap > 0) S.opt.tri_cap = tri_cap;
    if (n <= 0 || depth < 2 || depth > 9) return 2;
    build_octree(S, xyz, nrm, rgb, n);
    if (stop_after <= 1) return 0;
    if (h->given.res == (1 << (depth + 1)) - 1) S.tab = h->given;
    else S.tab.build(depth);
    compute_field(S);
    if (stop_after <= 2) return 0;
    solve(S);
    iso_value(S);
    if (stop_after <= 3) return 0;
    build_geometry(S);
    MeshRun<double> mr(S, S.x.data(), S.iso);
    mr.run();
    if (S.status) return S.status;
    if (stop_after <= 4) return 0;
    transfer(S);
    return 0;
}

// Re-runs the marching-cubes stage in float, mirroring the device evaluation order,
// with a caller-supplied solution vector (M floats) and iso-value.  Requires a prior
// oro_run with stop_after >= 3 on the same input.
int oro_run_mesh32(void* hp, const float* x, float iso) {
    OracleHandle* h = (OracleHandle*)hp;
    State& S = h->S;
    if (S.verts.empty()) build_geometry(S);
    MeshRun<float> mr(S, x, iso);
    mr.run();
    if (S.status) return S.status;
    transfer(S);
    return 0;
}

// The oracle's derived look-up tables, flattened in the order lut_parent, lut_child,
// edge_vertex, face_edges, children_vertex_kind, parent_face_kind (536 ints).
int oro_luts(int* out) {
    int k = 0;
    for (int s = 0; s < 8; ++s) for (int i = 0; i < 27; ++i) out[k++] = L.lut_parent[s][i];
    for (int s = 0; s < 8; ++s) for (int i = 0; i < 27; ++i) out[k++] = L.lut_child[s][i];
    for (int e = 0; e < 12; ++e) for (int j = 0; j < 2; ++j) out[k++] = L.edge_vertex[e][j];
    for (int f = 0; f < 6; ++f) for (int j = 0; j < 4; ++j) out[k++] = L.face_edges[f][j];
    for (int c = 0; c < 8; ++c) out[k++] = L.children_vertex_kind[c];
    for (int s = 0; s < 8; ++s) for (int f = 0; f < 6; ++f) out[k++] = L.parent_face_kind[s][f];
    return k;
}

// Implicit function (FP64) of an arbitrary solution vector at the sorted points.
int oro_point_values(void* hp, const float* x, double* out) {
    State& S = ((OracleHandle*)hp)->S;
    const int bD = S.base[S.D];
    for (int i = 0; i < S.N; ++i) {
        double p[3] = {S.pos[3 * i], S.pos[3 * i + 1], S.pos[3 * i + 2]};
        out[i] = chi64_chain(S, x, bD + S.point2node[i], p);
    }
    return 0;
}

// Named array access: elem 0 int32, 1 float32, 2 float64, 3 int64.
int oro_get(void* hp, const char* name, void** data, long long* count, int* elem) {
    OracleHandle* h = (OracleHandle*)hp;
    State& S = h->S;
    std::string nm(name);
    auto I = [&](std::vector<int>& v) { *data = v.data(); *count = (long long)v.size(); *elem = 0; return 0; };
    auto Fv = [&](std::vector<float>& v) { *data = v.data(); *count = (long long)v.size(); *elem = 1; return 0; };
    auto Dv = [&](std::vector<double>& v) { *data = v.data(); *count = (long long)v.size(); *elem = 2; return 0; };
    if (nm == "sorted_keys") { *data = S.sorted_keys.data(); *count = (long long)S.sorted_keys.size(); *elem = 3; return 0; }
    if (nm == "pos") return Fv(S.pos);
    if (nm == "color") return Fv(S.color);
    if (nm == "nrm") return Dv(S.nrm);
    if (nm == "point2node") return I(S.point2node);
    if (nm == "base") return I(S.base);
    if (nm == "count") return I(S.count);
    if (nm == "key") return I(S.key);
    if (nm == "pidx") return I(S.pidx);
    if (nm == "pnum") return I(S.pnum);
    if (nm == "parent") return I(S.parent);
    if (nm == "didx") return I(S.didx);
    if (nm == "dnum") return I(S.dnum);
    if (nm == "depth") return I(S.depth);
    if (nm == "enc") return I(S.enc);
    if (nm == "children") return I(S.children);
    if (nm == "neighs") return I(S.neighs);
    if (nm == "center") return Fv(S.center);
    if (nm == "vfield") return Dv(S.vfield);
    if (nm == "div") return Dv(S.div);
    if (nm == "x") return Dv(S.x);
    if (nm == "point_chi") return Dv(S.point_chi);
    if (nm == "cg_iters") return I(S.cg_iters);
    if (nm == "cg_resid") return Dv(S.cg_resid);
    if (nm == "ff") return Dv(S.tab.ff);
    if (nm == "dff") return Dv(S.tab.dff);
    if (nm == "d2") return Dv(S.tab.d2);
    if (nm == "node_vertices") return I(S.node_vertices);
    if (nm == "node_edges") return I(S.node_edges);
    if (nm == "node_faces") return I(S.node_faces);
    if (nm == "vvalue") return Dv(S.vvalue);
    if (nm == "vvalue32") return Fv(S.vvalue32);
    if (nm == "cube_class") return I(S.cube_class);
    if (nm == "edge_cross") return I(S.edge_cross);
    if (nm == "has_triangle") return I(S.has_triangle);
    if (nm == "has_intersection") return I(S.has_intersection);
    if (nm == "sub_roots") return I(S.sub_roots);
    if (nm == "sub_root_depth") return I(S.sub_root_depth);
    if (nm == "mesh_v") return Fv(S.mesh_v);
    if (nm == "mesh_t") return I(S.mesh_t);
    if (nm == "mesh_stage_v") return I(S.mesh_stage_v);
    if (nm == "mesh_stage_t") return I(S.mesh_stage_t);
    if (nm == "vcolor") return Fv(S.vcolor);
    if (nm == "vnormal") return Fv(S.vnormal);
    // packed records
    auto pack = [&](const char* k, std::vector<int> v) {
        std::vector<char>& buf = h->scratch[k];
        buf.resize(v.size() * sizeof(int));
        memcpy(buf.data(), v.data(), buf.size());
        *data = buf.data(); *count = (long long)v.size(); *elem = 0;
        return 0;
    };
    if (nm == "vertex_rec") {   // owner, kind, depth per vertex
        std::vector<int> v;
        for (auto& r : S.verts) { v.push_back(r.owner); v.push_back(r.kind); v.push_back(r.depth); }
        return pack("vertex_rec", v);
    }
    if (nm == "vertex_pos") {
        std::vector<char>& buf = h->scratch["vertex_pos"];
        buf.resize(S.verts.size() * 3 * sizeof(float));
        float* f = (float*)buf.data();
        for (size_t i = 0; i < S.verts.size(); ++i) memcpy(f + 3 * i, S.verts[i].pos, 3 * sizeof(float));
        *data = buf.data(); *count = (long long)S.verts.size() * 3; *elem = 1;
        return 0;
    }
    if (nm == "edge_rec") {
        std::vector<int> v;
        for (auto& r : S.edges) { v.push_back(r.owner); v.push_back(r.kind); }
        return pack("edge_rec", v);
    }
    if (nm == "face_rec") {
        std::vector<int> v;
        for (auto& r : S.faces) { v.push_back(r.owner); v.push_back(r.kind); v.push_back(r.has_parent_face); }
        return pack("face_rec", v);
    }
    if (nm == "scalars") {   // iso, bbox centre xyz, bbox edge, ub_events, M, N, status
        std::vector<char>& buf = h->scratch["scalars"];
        buf.resize(9 * sizeof(double));
        double* d = (double*)buf.data();
        d[0] = S.iso; d[1] = S.bbox_center[0]; d[2] = S.bbox_center[1]; d[3] = S.bbox_center[2];
        d[4] = S.bbox_edge; d[5] = S.ub_events; d[6] = S.M; d[7] = S.N; d[8] = S.status;
        *data = buf.data(); *count = 9; *elem = 2;
        return 0;
    }
    return -1;
}

}  // extern "C"
