// Host-side tables: neighbour / marching-cubes look-up tables and the B-spline
// inner-product tables of the reconstruction basis.
//
// Basis (mesh/FunctionData.h:83-125 with PPolynomial<2>::GaussianApproximation,
// math/PPolynomial.h:568-582): the quadratic B-spline box*box*box normalised to F(0) = 1,
//     F(t) = 1 - 4/3 t^2 (|t| < 1/2),  2/3 (3/2 - |t|)^2 (1/2 <= |t| < 3/2),  0 otherwise,
// placed at every BinaryNode index i: depth d = floor(log2(i + 1)), offset o = i + 1 - 2^d,
// centre (o + 1/2) 2^-d, width 2^-d.  The tables hold the exact integrals
//     ff(i, j) = \int F_i F_j,  dff(i, j) = \int F_i' F_j,  d2(i, j) = \int F_i' F_j'
// (index i + res * j, res = 2^(D+1) - 1), the quantities the reference tabulates in
// mesh/FunctionData.h:134-190 with float polynomial arithmetic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "psr_common.cuh"
#include "mc_tables.inc"

namespace psr {

void fill_const_tables(ConstTables* t) {
    memset(t, 0, sizeof(*t));
    // neighbour look-ups: neighbour k = 9 ox + 3 oy + oz (offsets -1, 0, +1 -> 0, 1, 2);
    // child slot bits x = 4, y = 2, z = 1 (same convention as mesh/BuildOctree.cu:20-42)
    for (int s = 0; s < 8; ++s) {
        const int cp[3] = {(s >> 2) & 1, (s >> 1) & 1, s & 1};
        for (int k = 0; k < 27; ++k) {
            const int o[3] = {k / 9, (k / 3) % 3, k % 3};
            int pn = 0, ch = 0;
            for (int a = 0; a < 3; ++a) {
                int q = cp[a] + o[a] - 1;
                pn = pn * 3 + (q < 0 ? 0 : (q > 1 ? 2 : 1));
                ch = ch * 2 + ((q + 2) & 1);
            }
            t->lut_parent[s][k] = pn;
            t->lut_child[s][k] = ch;
        }
    }
    static const int ev[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 3}, {1, 2},
                                  {4, 7}, {5, 6}, {0, 4}, {1, 5}, {3, 7}, {2, 6}};
    static const int fe[6][4] = {{4, 6, 8, 10}, {5, 7, 9, 11}, {0, 2, 8, 9},
                                 {1, 3, 10, 11}, {0, 1, 4, 5}, {2, 3, 6, 7}};
    static const int pfk[8][6] = {{0, -1, 2, -1, 4, -1}, {-1, 1, 2, -1, 4, -1},
                                  {0, -1, -1, 3, 4, -1}, {-1, 1, -1, 3, 4, -1},
                                  {0, -1, 2, -1, -1, 5}, {-1, 1, 2, -1, -1, 5},
                                  {0, -1, -1, 3, -1, 5}, {0, 1, -1, 3, -1, 5}};
    static const int cvk[8] = {0, 1, 3, 2, 4, 5, 7, 6};
    memcpy(t->edge_vertex, ev, sizeof(ev));
    memcpy(t->face_edges, fe, sizeof(fe));
    memcpy(t->parent_face_kind, pfk, sizeof(pfk));
    memcpy(t->children_vertex_kind, cvk, sizeof(cvk));
    for (int c = 0; c < 256; ++c) {
        t->mc_tri[c] = kMcTrianglesInit[c];
        t->mc_count[c] = kMcTriangleCountInit[c];
    }
}

namespace {

inline double bspline(double t) {
    double a = std::fabs(t);
    if (a < 0.5) return 1.0 - (4.0 / 3.0) * t * t;
    if (a < 1.5) return (2.0 / 3.0) * (1.5 - a) * (1.5 - a);
    return 0.0;
}
inline double bspline_d(double t) {
    double a = std::fabs(t);
    if (a < 0.5) return -(8.0 / 3.0) * t;
    if (a < 1.5) return (t > 0 ? -1.0 : 1.0) * (4.0 / 3.0) * (1.5 - a);
    return 0.0;
}
struct Fn {
    double c, w;
};
inline Fn fn_of(int idx) {
    int d = 0;
    while ((1 << (d + 1)) <= idx + 1) ++d;
    int off = idx + 1 - (1 << d);
    Fn f;
    f.w = std::ldexp(1.0, -d);
    f.c = (off + 0.5) * f.w;
    return f;
}

// exact integrals of the products over the common support: the integrands are
// polynomials of degree <= 4 between consecutive breakpoints, so 3-point Gauss-Legendre
// per piece is exact
void integrals(const Fn& a, const Fn& b, double& ff, double& dff, double& d2) {
    ff = dff = d2 = 0.0;
    double lo = std::max(a.c - 1.5 * a.w, b.c - 1.5 * b.w);
    double hi = std::min(a.c + 1.5 * a.w, b.c + 1.5 * b.w);
    if (!(lo < hi)) return;
    std::vector<double> bp = {lo, hi};
    for (int k = 0; k < 4; ++k) {
        double u = a.c + (k - 1.5) * a.w, v = b.c + (k - 1.5) * b.w;
        if (u > lo && u < hi) bp.push_back(u);
        if (v > lo && v < hi) bp.push_back(v);
    }
    std::sort(bp.begin(), bp.end());
    static const double gx[3] = {-0.77459666924148337704, 0.0, 0.77459666924148337704};
    static const double gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    for (size_t k = 0; k + 1 < bp.size(); ++k) {
        double h = 0.5 * (bp[k + 1] - bp[k]), m = 0.5 * (bp[k + 1] + bp[k]);
        if (h <= 0) continue;
        for (int q = 0; q < 3; ++q) {
            double x = m + h * gx[q];
            double ta = (x - a.c) / a.w, tb = (x - b.c) / b.w;
            double Fa = bspline(ta), Fb = bspline(tb);
            double dFa = bspline_d(ta) / a.w, dFb = bspline_d(tb) / b.w;
            ff += gw[q] * h * Fa * Fb;
            dff += gw[q] * h * dFa * Fb;
            d2 += gw[q] * h * dFa * dFb;
        }
    }
}

}  // namespace

// d/dx-product table (full res x res; only pairs with overlapping support are non-zero)
void build_dff_table(int depth, std::vector<double>& dff) {
    const int res = (1 << (depth + 1)) - 1;
    dff.assign((size_t)res * res, 0.0);
    std::vector<Fn> f(res);
    for (int i = 0; i < res; ++i) f[i] = fn_of(i);
    for (int i = 0; i < res; ++i)
        for (int j = 0; j < res; ++j) {
            if (std::fabs(f[i].c - f[j].c) >= 1.5 * (f[i].w + f[j].w)) continue;
            double a, b, c;
            integrals(f[i], f[j], a, b, c);
            dff[(size_t)i + (size_t)res * j] = b;
        }
}

// Same-depth Laplacian stencil (mesh/solver/LaplacianSolver.cu:27-74): entry for the
// neighbour at offset (ox, oy, oz) of a node at depth d is
//     ff_x ff_y ff_z (d2_x + d2_y + d2_z)
// evaluated in FP64 and stored as FP32; entries with |value| <= 1e-6 are dropped.  Same
// depth pairs only depend on the offset, so one coefficient per (depth, neighbour) is
// exact.  Returns (D+1) x 27 floats.
void build_stencil(int depth, std::vector<float>& st, double eps) {
    st.assign((size_t)(depth + 1) * 27, 0.0f);
    for (int d = 0; d <= depth; ++d) {
        // representative node well inside the unit interval (or the only node at d = 0)
        int n = 1 << d;
        int off = n / 2;
        double ff[3], d2[3];
        bool ok[3];
        for (int o = 0; o < 3; ++o) {
            int o2 = off + o - 1;
            ok[o] = (o2 >= 0 && o2 < n);
            ff[o] = d2[o] = 0.0;
            if (!ok[o]) {
                // the neighbour exists only for d >= 1; evaluate the offset pair explicitly
                Fn a{(off + 0.5) / n, 1.0 / n}, b{(o2 + 0.5) / n, 1.0 / n};
                double x, y, z;
                integrals(a, b, x, y, z);
                ff[o] = x; d2[o] = z;
                continue;
            }
            Fn a = fn_of(n - 1 + off), b = fn_of(n - 1 + o2);
            double x, y, z;
            integrals(a, b, x, y, z);
            ff[o] = x;
            d2[o] = z;
        }
        for (int k = 0; k < 27; ++k) {
            int ox = k / 9, oy = (k / 3) % 3, oz = k % 3;
            double v = ff[ox] * ff[oy] * ff[oz] * (d2[ox] + d2[oy] + d2[oz]);
            st[(size_t)d * 27 + k] = (std::fabs(v) > eps) ? (float)v : 0.0f;
        }
    }
}

}  // namespace psr
