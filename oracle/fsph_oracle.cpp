/*
 * fsph_oracle.cpp -- CPU ORACLE of the fluid step.  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, by __graft_entry__.smoke() as the checker, and by the
 * CPU-baseline leg of bench.py.  The product (libfsph.so) never links,
 * loads or calls it.
 *
 * A restatement of the reference's CPU fluid path, templated on the storage
 * precision T:
 *   T = float  : the reference's own arithmetic -- float particle arrays and
 *                float accumulators (RXREAL), per-pair geometry and kernel
 *                values in double (the reference's Vec3 / rx_kernel.h).
 *   T = double : the same algorithm entirely in double (the FP64 oracle used
 *                to report the error of every FP32 result).
 *
 * Followed, function by function:
 *   kernels        rx_kernel.h:29-80 (poly6), 133-203 (spiky gradient), 236-324 (visc Laplacian)
 *   rest density   rx_sph_pbd.cpp:1035-1049 (calRestDensity)
 *   derivation     rx_sph_pbd.cpp:102-201 (rxPBDSPH::Initialize), rx_sph_cpu.cpp:92-166
 *   neighbours     rx_nnsearch.h:454-515 (GetNN / getNeighborsInCell): the set
 *                  {j : fl32(|xi-xj|^2 in double) <= fl32(h*h)}, self included
 *   walls          rx_sph_solid.cpp:44-108 (AABB_point_dist), 244-262 (GetDistanceR),
 *                  rx_sph_pbd.cpp:1374-1398 (calCollisionSolid: position only)
 *   WCSPH          rx_sph_cpu.cpp:323-380 (Update), 495-552 (calDensity),
 *                  558-656 (calForce), 1040-1077 (integrate)
 *   PBF            rx_sph_pbd.cpp:377-484 (Update), 599-646 (calDensity),
 *                  651-689 (calForceExtAndVisc), 699-914 (calScalingFactor, with the
 *                  k = i self term), 925-1026 (calPositionCorrection, s_corr with dt^2),
 *                  1409-1446 (integrate)
 *   XSPH           rx_pbdsph_kernel.cu:1090-1162 (xsphVisocosity; GPU-only in the reference)
 *   vorticity      absent from the reference (only a flag, rx_ps.h:161); restated from
 *                  Macklin & Mueller, "Position Based Fluids", SIGGRAPH 2013, eq. 15-16,
 *                  which rx_sph.h:1281 cites.
 *
 * Deliberate, documented choices where the reference is ambiguous:
 *   - neighbour lists are kept in ascending particle index (the reference's
 *     within-cell order depends on an unstable std::sort, rx_nnsearch.h:257);
 *   - the convergence error may be the one-sided GPU form or the two-sided
 *     CPU form (fsph_params.error_mode);
 *   - the iteration count reported is the number of constraint iterations
 *     executed (the reference's g_iIterations is one less when the loop ends
 *     by its early break, rx_sph_pbd.cpp:456-459).
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/fsph.h"

namespace {

const double kPi = 3.14159265358979323846;

struct V3 {
    double x, y, z;
};
inline V3 v3(double a, double b, double c) { return V3{a, b, c}; }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator*(double s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
inline V3 operator/(V3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

/* Kernel coefficients and values (rx_kernel.h): the coefficient is computed
 * in double from the float radius, as the reference's Initialize does. */
struct Kern {
    double h, aw, ag, al;
    explicit Kern(double h_) : h(h_) {
        aw = 315.0 / (64.0 * kPi * std::pow(h, 9.0));
        ag = -45.0 / (kPi * std::pow(h, 6.0));
        al = 45.0 / (kPi * std::pow(h, 6.0));
    }
    double W(double r) const {
        if (r >= 0.0 && r <= h) { double q = h * h - r * r; return aw * q * q * q; }
        return 0.0;
    }
    /* scalar s with grad W = s * rij */
    double G(double r) const {
        if (r > 0.0 && r <= h) { double q = h - r; return ag * q * q / r; }
        return 0.0;
    }
    double L(double r) const {
        if (r > 0.0 && r <= h) return al * (h - r);
        return 0.0;
    }
};

template <class T>
inline void acc_add(T &a, double term) { a = (T)((double)a + term); }

/* Triangle-mesh obstacles, the reference's GPU rule (rxPBDSPH_GPU::
 * SetPolygonObstacle / setPolysToCell, rx_sph_pbd_gpu.cpp:2051-2200, 2367-2410;
 * pbdsphIntegrateWithPolygon / calCollisionPolygonPB, rx_pbdsph_kernel.cu:
 * 916-1030; intersectSegmentTriangle, rx_cu_common.cu:891-975), restated in
 * T arithmetic, one rounding per operation: the triangles are binned into the
 * cells of the reference's GPU grid that they intersect; a segment x0 -> x1
 * is tested against the triangles of the cells of x0 and of x1, in that order
 * (both, even when equal), each in ascending triangle index, and a crossing
 * from a triangle's front side moves x1 back to that side with the velocity
 * component into the triangle removed (restitution 0).  Zero-area triangles
 * are skipped. */
template <class T>
struct PolyMesh {
    struct P3 {
        T x, y, z;
    };
    static P3 sub(P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; }
    static P3 add(P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; }
    static P3 scl(P3 a, T s) { return P3{a.x * s, a.y * s, a.z * s}; }
    static T dot(P3 a, P3 b) {
        T s = a.x * b.x;
        s = s + a.y * b.y;
        return s + a.z * b.z;
    }
    static P3 crs(P3 a, P3 b) { return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
    static T len(P3 a) { return std::sqrt(dot(a, a)); }
    static P3 unit(P3 a) {
        T l = len(a);
        return P3{a.x / l, a.y / l, a.z / l};
    }

    int nt = 0;
    std::vector<P3> V;                 /* vertices, rounded to float as stored */
    std::vector<int> tri;              /* 3 per triangle */
    std::vector<unsigned int> start, end, idx;
    double org[3] = {0, 0, 0};
    T orgT[3] = {0, 0, 0}, cw = 0;
    int g[3] = {1, 1, 1};

    /* separating axes of a triangle against the cube [-0.5, 0.5]^3 */
    static bool overlap(const double v[3][3]) {
        for (int a = 0; a < 3; ++a) {
            double mn = std::min(v[0][a], std::min(v[1][a], v[2][a]));
            double mx = std::max(v[0][a], std::max(v[1][a], v[2][a]));
            if (mn > 0.5 || mx < -0.5) return false;
        }
        double e[3][3];
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) e[k][a] = v[(k + 1) % 3][a] - v[k][a];
        for (int k = 0; k < 3; ++k)
            for (int a = 0; a < 3; ++a) {
                double ax[3] = {0, 0, 0};
                ax[(a + 1) % 3] = -e[k][(a + 2) % 3];
                ax[(a + 2) % 3] = e[k][(a + 1) % 3];
                double mn = 1e300, mx = -1e300;
                for (int j = 0; j < 3; ++j) {
                    double q = ax[0] * v[j][0] + ax[1] * v[j][1] + ax[2] * v[j][2];
                    mn = std::min(mn, q);
                    mx = std::max(mx, q);
                }
                double r = 0.5 * (std::fabs(ax[0]) + std::fabs(ax[1]) + std::fabs(ax[2]));
                if (mn > r || mx < -r) return false;
            }
        double nr[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                        e[0][0] * e[1][1] - e[0][1] * e[1][0]};
        double dp = nr[0] * v[0][0] + nr[1] * v[0][1] + nr[2] * v[0][2];
        return std::fabs(dp) <= 0.5 * (std::fabs(nr[0]) + std::fabs(nr[1]) + std::fabs(nr[2]));
    }

    /* vertices as stored (floats), triangles, the grid over the box grown by
     * 1 % (rx_sph_pbd_gpu.cpp:248-262, 1986-2011) */
    void set(const float *v3f, int nv, const int *t, int ntri, const fsph_params &P) {
        nt = ntri;
        V.resize(nv);
        for (int k = 0; k < nv; ++k) V[k] = P3{(T)v3f[3 * k], (T)v3f[3 * k + 1], (T)v3f[3 * k + 2]};
        tri.assign(t, t + 3 * (size_t)ntri);
        double lo[3], ws[3];
        for (int a = 0; a < 3; ++a) {
            double size = P.box_max[a] - P.box_min[a];
            lo[a] = P.box_min[a] - 0.5 * 0.01 * size;
            double hi = lo[a] + size * (1.0 + 0.01);
            ws[a] = hi - lo[a];
        }
        double h = (double)P.h;
        double max_axis = std::max(ws[0], std::max(ws[1], ws[2]));
        int d = (int)(std::log(max_axis / h) / std::log(2.0) + 0.5);
        int m = (int)(std::pow(2.0, (double)d) + 0.5);
        double cwd = max_axis / m;
        float cwf = (float)cwd;
        cw = (T)cwf;
        for (int a = 0; a < 3; ++a) {
            org[a] = lo[a];
            orgT[a] = (T)(float)lo[a];
            g[a] = (int)(ws[a] / cwd) + 1;
        }
        double L = (double)cwf;
        size_t ncell = (size_t)g[0] * g[1] * g[2];
        start.assign(ncell, 0xffffffffu);
        end.assign(ncell, 0u);
        std::vector<std::vector<unsigned int>> per(ncell);
        for (int i = 0; i < ntri; ++i) {
            double P0[3][3];
            for (int j = 0; j < 3; ++j) {
                const float *q = v3f + 3 * (size_t)t[3 * i + j];
                for (int a = 0; a < 3; ++a) P0[j][a] = (double)q[a];
            }
            int l0[3], h0[3];
            for (int a = 0; a < 3; ++a) {
                double b0 = std::min(P0[0][a], std::min(P0[1][a], P0[2][a])) - org[a];
                double b1 = std::max(P0[0][a], std::max(P0[1][a], P0[2][a])) - org[a];
                double f0 = std::max(std::min(b0 / L, (double)g[a]), -1.0), f1 = std::max(std::min(b1 / L, (double)g[a]), -1.0);
                l0[a] = std::min(std::max((int)f0, 0), g[a] - 1);
                h0[a] = std::min(std::max((int)f1, 0), g[a] - 1);
            }
            for (int x = l0[0]; x <= h0[0]; ++x)
                for (int y = l0[1]; y <= h0[1]; ++y)
                    for (int z = l0[2]; z <= h0[2]; ++z) {
                        double cen[3] = {org[0] + (x + 0.5) * L, org[1] + (y + 0.5) * L, org[2] + (z + 0.5) * L};
                        double vc[3][3];
                        for (int j = 0; j < 3; ++j)
                            for (int a = 0; a < 3; ++a) vc[j][a] = (P0[j][a] - cen[a]) / L;
                        if (overlap(vc)) per[((size_t)z * g[1] + y) * g[0] + x].push_back((unsigned int)i);
                    }
        }
        idx.clear();
        for (size_t c = 0; c < ncell; ++c) {
            if (per[c].empty()) continue;
            start[c] = (unsigned int)idx.size();
            idx.insert(idx.end(), per[c].begin(), per[c].end());
            end[c] = (unsigned int)idx.size();
        }
    }

    size_t cell(P3 x) const {
        T xs[3] = {x.x, x.y, x.z};
        int c[3];
        for (int a = 0; a < 3; ++a) {
            T f = std::floor((xs[a] - orgT[a]) / cw);
            f = std::max(std::min(f, (T)g[a]), (T)-1);
            int k = (int)f;
            c[a] = k < 0 ? 0 : (k >= g[a] ? g[a] - 1 : k);
        }
        return ((size_t)c[2] * g[1] + c[1]) * g[0] + c[0];
    }

    static int seg_tri(P3 P0, P3 P1, P3 V0, P3 V1, P3 V2, P3 &I, P3 &n) {
        P3 u = sub(V1, V0), v = sub(V2, V0);
        P3 c = crs(u, v);
        if (dot(c, c) == (T)0) return -1;
        n = unit(c);
        P3 dir = sub(P1, P0);
        T a = dot(n, sub(P0, V0));
        T b = dot(n, dir);
        if ((double)std::fabs(b) < 1e-10) return a == (T)0 ? 2 : 0;
        T r = -a / b;
        if (r < (T)0 || std::fabs(a) > std::fabs(b) || b > (T)0) return 0;
        I = add(P0, scl(dir, r));
        T uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
        P3 w = sub(I, V0);
        T wu = dot(w, u), wv = dot(w, v);
        T D = uv * uv - uu * vv;
        T s = (uv * wv - vv * wu) / D;
        if (s < (T)0 || s > (T)1) return 0;
        T t = (uv * wu - uu * wv) / D;
        if (t < (T)0 || s + t > (T)1) return 0;
        return 1;
    }

    /* x0, x1, v in double from the caller; rounded to T first */
    void collide(V3 x0d, V3 &x1d, V3 &vd, T dt) const {
        P3 x0{(T)x0d.x, (T)x0d.y, (T)x0d.z}, x1{(T)x1d.x, (T)x1d.y, (T)x1d.z}, v{(T)vd.x, (T)vd.y, (T)vd.z};
        const size_t cells[2] = {cell(x0), cell(x1)};
        for (int k = 0; k < 2; ++k) {
            if (start[cells[k]] == 0xffffffffu) continue;
            for (unsigned int j = start[cells[k]]; j < end[cells[k]]; ++j) {
                const int t = (int)idx[j];
                P3 cp, n;
                if (seg_tri(x0, x1, V[tri[3 * t]], V[tri[3 * t + 1]], V[tri[3 * t + 2]], cp, n) != 1) continue;
                T d = len(sub(x1, cp));
                n = unit(n);
                P3 vr = scl(scl(n, (T)-1), dot(n, v));
                T l = len(sub(x1, x0));
                x1 = add(cp, scl(vr, (dt * d) / l));
                v = add(v, vr);
            }
        }
        x1d = v3((double)x1.x, (double)x1.y, (double)x1.z);
        vd = v3((double)v.x, (double)v.y, (double)v.z);
    }
};

template <class T>
struct Solver {
    fsph_params P;
    int n = 0;
    std::vector<T> pos, vel, ppos, pvel, frc, dens, pres, lam, dp, vort;
    std::vector<int> noff, nidx; /* neighbour CSR */
    /* static boundary particles: positions, volumes psi_b, lambda_b, and the
     * boundary-boundary, fluid-boundary and boundary-fluid neighbour CSRs */
    int nb = 0;
    std::vector<T> bpos, bvol, blam;
    std::vector<int> bb_off, bb_idx, fb_off, fb_idx, bf_off, bf_idx;
    Kern K;
    /* analytic obstacles: type (0 box, 1 sphere), centre, half extents,
     * world -> local rotation (rows), sphere radius */
    struct Obs {
        int type;
        double cen[3], ext[3], R[3][3], rad;
    };
    std::vector<Obs> obs;
    /* triangle-mesh obstacles (see PolyMesh) */
    PolyMesh<T> mesh;
    int last_iters = 0;
    double last_err1 = 0, last_err2 = 0, last_errmax = 0;

    explicit Solver(const fsph_params &p) : P(p), K(p.h) {}

    void resize(int n_) {
        n = n_;
        pos.assign(4 * (size_t)n, 0); vel.assign(4 * (size_t)n, 0);
        ppos.assign(4 * (size_t)n, 0); pvel.assign(4 * (size_t)n, 0);
        frc.assign(4 * (size_t)n, 0); dp.assign(4 * (size_t)n, 0); vort.assign(4 * (size_t)n, 0);
        dens.assign(n, 0); pres.assign(n, 0); lam.assign(n, 0);
    }

    V3 at(const std::vector<T> &a, int i) const {
        return v3((double)a[4 * (size_t)i], (double)a[4 * (size_t)i + 1], (double)a[4 * (size_t)i + 2]);
    }

    /* Neighbour sets on positions p (rx_nnsearch.h:454-515): every j with
     * fl(|xi - xj|^2) <= fl(h*h), the squared distance evaluated in double and
     * rounded to T.  Binning uses cells of width >= h, so the 27 cells around
     * a particle hold every candidate; lists are ascending in j. */
    void neighbors(const std::vector<T> &p) {
        const T hT = (T)P.h;
        const T h2 = hT * hT;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                double v = (double)p[4 * (size_t)i + k];
                lo[k] = std::min(lo[k], v); hi[k] = std::max(hi[k], v);
            }
        const double cw = (double)P.h * 1.0001;
        int g[3];
        for (int k = 0; k < 3; ++k) g[k] = std::max(1, (int)std::floor((hi[k] - lo[k]) / cw) + 1);
        const size_t C = (size_t)g[0] * g[1] * g[2];
        std::vector<int> cnt(C + 1, 0), cellOf(n), order(n);
        auto cell3 = [&](int i, int c[3]) {
            for (int k = 0; k < 3; ++k) {
                int v = (int)std::floor(((double)p[4 * (size_t)i + k] - lo[k]) / cw);
                c[k] = std::min(std::max(v, 0), g[k] - 1);
            }
        };
        for (int i = 0; i < n; ++i) {
            int c[3]; cell3(i, c);
            cellOf[i] = (int)(((size_t)c[2] * g[1] + c[1]) * g[0] + c[0]);
            cnt[cellOf[i] + 1]++;
        }
        for (size_t c = 0; c < C; ++c) cnt[c + 1] += cnt[c];
        {
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            for (int i = 0; i < n; ++i) order[fill[cellOf[i]]++] = i;
        }
        std::vector<std::vector<int>> lists(n);
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < n; ++i) {
            int c[3]; cell3(i, c);
            V3 xi = at(p, i);
            std::vector<int> &L = lists[i];
            for (int dz = -1; dz <= 1; ++dz)
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        int z = c[2] + dz, y = c[1] + dy, x = c[0] + dx;
                        if (x < 0 || y < 0 || z < 0 || x >= g[0] || y >= g[1] || z >= g[2]) continue;
                        size_t cc = ((size_t)z * g[1] + y) * g[0] + x;
                        for (int s = cnt[cc]; s < cnt[cc + 1]; ++s) {
                            int j = order[s];
                            V3 d = xi - at(p, j);
                            T d2 = (T)dot(d, d);
                            if (d2 <= h2) L.push_back(j);
                        }
                    }
            std::sort(L.begin(), L.end());
        }
        noff.assign(n + 1, 0);
        for (int i = 0; i < n; ++i) noff[i + 1] = noff[i] + (int)lists[i].size();
        nidx.resize(noff[n]);
        for (int i = 0; i < n; ++i) std::copy(lists[i].begin(), lists[i].end(), nidx.begin() + noff[i]);
    }

    /* For every point i of a (na points): the points j of b (nbp points)
     * with fl(|a_i - b_j|^2) <= fl(h*h), ascending j -- the criterion of
     * rxNNGrid::GetNN(pos, ...) (rx_nnsearch.h:454-515) between two sets. */
    void cross_sets(const std::vector<T> &a, int na, const std::vector<T> &b, int nbp, std::vector<int> &off,
               std::vector<int> &idx) const {
        const T hT = (T)P.h;
        const T h2 = hT * hT;
        off.assign(na + 1, 0);
        idx.clear();
        if (nbp == 0 || na == 0) return;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int j = 0; j < nbp; ++j)
            for (int k = 0; k < 3; ++k) {
                double v = (double)b[4 * (size_t)j + k];
                lo[k] = std::min(lo[k], v); hi[k] = std::max(hi[k], v);
            }
        const double cw = (double)P.h * 1.0001;
        int g[3];
        for (int k = 0; k < 3; ++k) g[k] = std::max(1, (int)std::floor((hi[k] - lo[k]) / cw) + 1);
        const size_t C = (size_t)g[0] * g[1] * g[2];
        std::vector<int> cnt(C + 1, 0), cellOf(nbp), order(nbp);
        for (int j = 0; j < nbp; ++j) {
            int c[3];
            for (int k = 0; k < 3; ++k)
                c[k] = std::min(std::max((int)std::floor(((double)b[4 * (size_t)j + k] - lo[k]) / cw), 0), g[k] - 1);
            cellOf[j] = (int)(((size_t)c[2] * g[1] + c[1]) * g[0] + c[0]);
            cnt[cellOf[j] + 1]++;
        }
        for (size_t c = 0; c < C; ++c) cnt[c + 1] += cnt[c];
        {
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            for (int j = 0; j < nbp; ++j) order[fill[cellOf[j]]++] = j;
        }
        std::vector<std::vector<int>> lists(na);
#pragma omp parallel for schedule(dynamic, 256)
        for (int i = 0; i < na; ++i) {
            V3 xi = v3((double)a[4 * (size_t)i], (double)a[4 * (size_t)i + 1], (double)a[4 * (size_t)i + 2]);
            long long c0[3];
            double xs[3] = {xi.x, xi.y, xi.z};
            for (int k = 0; k < 3; ++k) c0[k] = (long long)std::floor((xs[k] - lo[k]) / cw);
            std::vector<int> &L = lists[i];
            for (long long z = c0[2] - 1; z <= c0[2] + 1; ++z)
                for (long long y = c0[1] - 1; y <= c0[1] + 1; ++y)
                    for (long long x = c0[0] - 1; x <= c0[0] + 1; ++x) {
                        if (x < 0 || y < 0 || z < 0 || x >= g[0] || y >= g[1] || z >= g[2]) continue;
                        size_t cc = ((size_t)z * g[1] + y) * g[0] + x;
                        for (int s = cnt[cc]; s < cnt[cc + 1]; ++s) {
                            int j = order[s];
                            V3 d = xi - v3((double)b[4 * (size_t)j], (double)b[4 * (size_t)j + 1],
                                           (double)b[4 * (size_t)j + 2]);
                            T d2 = (T)dot(d, d);
                            if (d2 <= h2) L.push_back(j);
                        }
                    }
            std::sort(L.begin(), L.end());
        }
        for (int i = 0; i < na; ++i) off[i + 1] = off[i] + (int)lists[i].size();
        idx.resize(off[na]);
        for (int i = 0; i < na; ++i) std::copy(lists[i].begin(), lists[i].end(), idx.begin() + off[i]);
    }

    V3 bat(int b) const { return at(bpos, b); }

    /* Static boundary particles and their volumes psi_b = m / sum_b' m W(r_bb')
     * (rxPBDSPH::calBoundaryVolumes, rx_sph_pbd.cpp:1061-1090), float
     * accumulation of the double kernel values as in the reference. */
    void set_boundary(const float *b4, int count) {
        nb = count;
        bpos.assign(4 * (size_t)nb, 0);
        for (size_t k = 0; k < 4 * (size_t)nb; ++k) bpos[k] = (T)b4[k];
        bvol.assign(nb, 0);
        blam.assign(nb, 0);
        cross_sets(bpos, nb, bpos, nb, bb_off, bb_idx);
        const T m = (T)P.mass;
        for (int i = 0; i < nb; ++i) {
            T mw = 0;
            for (int s = bb_off[i]; s < bb_off[i + 1]; ++s) {
                V3 d = bat(bb_idx[s]) - bat(i);
                T r = (T)std::sqrt(dot(d, d));
                acc_add(mw, (double)m * K.W((double)r));
            }
            bvol[i] = m / mw;
        }
    }

    /* rho0 psi_b / m of boundary particle b, in float as the reference forms it */
    T bscale(int b) const { return (T)P.rest_dens * bvol[b] / (T)P.mass; }

    /* sum_b rho0 psi_b W(|x_i - x_b|) over the boundary neighbours of fluid i
     * (rx_sph_pbd.cpp:624-644) */
    T boundary_density(const V3 &xi, int i) const {
        T brho = 0;
        for (int s = fb_off[i]; s < fb_off[i + 1]; ++s) {
            int b = fb_idx[s];
            V3 d = bat(b) - xi;
            T r = (T)std::sqrt(dot(d, d));
            acc_add(brho, (double)((T)P.rest_dens * bvol[b]) * K.W((double)r));
        }
        return brho;
    }

    /* Box-wall projection keeping the particle radius from every face
     * (rxSolidBox::GetDistanceR -> AABB_point_dist with sgn = 1, contact =
     * pos + n |d|).  Velocity is left unchanged: the reflection is commented
     * out in the reference (rx_sph_pbd.cpp:1392). */
    /* Obstacle projection, the rule of collisionPointBox / collisionPointSphere
     * with calCollisionSolidPB (rx_cu_common.cu:748-831, rx_pbdsph_kernel.cu:
     * 863-911): a point inside a box (in its rotated frame) moves to the
     * nearest face (ties x, y, z), inside a sphere radially to its surface.
     * The reference's CPU path sets obstacles up as rxSolid objects whose
     * particle-radius handling is inverted for obstacles (AABB_point_dist with
     * sgn = -1, rx_sph_solid.cpp:44-108), so the GPU rule is the one restated. */
    V3 obstacles(V3 x) const {
        for (const Obs &o : obs) {
            V3 l = x - v3(o.cen[0], o.cen[1], o.cen[2]);
            if (o.type == 1) {
                double ll = std::sqrt(dot(l, l));
                if (ll < o.rad && ll > 0.0) x = v3(o.cen[0], o.cen[1], o.cen[2]) + (o.rad / ll) * l;
                continue;
            }
            double cp[3], li[3] = {l.x, l.y, l.z};
            for (int r = 0; r < 3; ++r) cp[r] = o.R[r][0] * li[0] + o.R[r][1] * li[1] + o.R[r][2] * li[2];
            double t[3];
            for (int k = 0; k < 3; ++k) t[k] = std::fabs(cp[k]) - o.ext[k];
            if (t[0] < 0.0 && t[1] < 0.0 && t[2] < 0.0) {
                double a[3] = {-t[0], -t[1], -t[2]};
                int ax = (a[0] <= a[1] && a[0] <= a[2]) ? 0 : ((a[1] <= a[0] && a[1] <= a[2]) ? 1 : 2);
                cp[ax] = cp[ax] > 0.0 ? o.ext[ax] : -o.ext[ax];
                double w[3];
                for (int r = 0; r < 3; ++r) w[r] = o.R[0][r] * cp[0] + o.R[1][r] * cp[1] + o.R[2][r] * cp[2];
                x = v3(o.cen[0] + w[0], o.cen[1] + w[1], o.cen[2] + w[2]);
            }
        }
        return x;
    }

    V3 wall(V3 pos) const {
        if (!obs.empty()) pos = obstacles(pos);
        const double r = (double)(T)P.particle_radius;
        double cen[3], sl[3];
        for (int k = 0; k < 3; ++k) {
            cen[k] = 0.5 * (P.box_max[k] + P.box_min[k]);
            sl[k] = 0.5 * (P.box_max[k] - P.box_min[k]);
        }
        double sp[3] = {pos.x - cen[0], pos.y - cen[1], pos.z - cen[2]};
        double d0[6];
        int out = 0, last = -1;
        for (int k = 0; k < 3; ++k) {
            d0[2 * k] = (sp[k] - r) - (-sl[k]);
            if (d0[2 * k] < 0.0) { out |= 1 << (2 * k); last = 2 * k; }
            d0[2 * k + 1] = sl[k] - (sp[k] + r);
            if (d0[2 * k + 1] < 0.0) { out |= 1 << (2 * k + 1); last = 2 * k + 1; }
        }
        if (!out) return pos; /* inside: contact only when d == 0, which is pos itself */
        int c = __builtin_popcount(out);
        double p[3] = {pos.x, pos.y, pos.z};
        if (c == 1) {
            int ax = last / 2;
            double nrm = (last % 2 == 0) ? 1.0 : -1.0; /* inward face normal */
            p[ax] = p[ax] + nrm * std::fabs(d0[last]);
            return v3(p[0], p[1], p[2]);
        }
        double x[3] = {0, 0, 0};
        for (int k = 0; k < 3; ++k) {
            if (out & (1 << (2 * k))) x[k] = d0[2 * k];
            else if (out & (1 << (2 * k + 1))) x[k] = -d0[2 * k + 1];
        }
        double nx = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        double u[3] = {x[0] / nx, x[1] / nx, x[2] / nx};
        for (int k = 0; k < 3; ++k) p[k] = p[k] + (-u[k]) * std::fabs(-nx);
        return v3(p[0], p[1], p[2]);
    }

    /* v += dt a; x += dt v; walls (rxPBDSPH::integrate / rxSPH::integrate). */
    void integrate(const std::vector<T> &x0, const std::vector<T> &v0, const std::vector<T> &a0,
                   std::vector<T> &x1, std::vector<T> &v1, T dt) {
        for (int i = 0; i < n; ++i) {
            V3 x = at(x0, i), v = at(v0, i), a = at(a0, i);
            const V3 xo = x;
            v = v + (double)dt * a;
            x = x + (double)dt * v;
            if (mesh.nt) mesh.collide(xo, x, v, dt); /* in T arithmetic from the rounded end points */
            x = wall(x);
            size_t b = 4 * (size_t)i;
            x1[b] = (T)x.x; x1[b + 1] = (T)x.y; x1[b + 2] = (T)x.z;
            v1[b] = (T)v.x; v1[b + 1] = (T)v.y; v1[b + 2] = (T)v.z;
        }
    }

    /* rho_i = sum_j m W(r_ij), self included. */
    void density(const std::vector<T> &p, std::vector<T> &rho) {
        if (nb) cross_sets(p, n, bpos, nb, fb_off, fb_idx);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(p, i);
            T acc = 0;
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                V3 d = xi - at(p, nidx[s]);
                T r = (T)std::sqrt(dot(d, d));
                acc_add(acc, (double)(T)P.mass * K.W((double)r));
            }
            if (nb) acc = acc + boundary_density(xi, i);
            rho[i] = acc;
        }
    }

    /* ---------------- PBF ---------------- */
    /* a_i = mu sum_{j != i} m (v_j - v_i) / rho_i lapW(r) + g (rx_sph_pbd.cpp:651-689). */
    void ext_visc(const std::vector<T> &p, const std::vector<T> &v, const std::vector<T> &rho,
                  std::vector<T> &f) {
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(p, i), vi = at(v, i);
            V3 fev = v3(0, 0, 0);
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                int j = nidx[s];
                if (j == i) continue;
                V3 d = xi - at(p, j), vji = at(v, j) - vi;
                T r = (T)std::sqrt(dot(d, d));
                fev = fev + ((double)(T)P.mass * K.L((double)r)) * (vji / (double)rho[i]);
            }
            V3 force = (double)(T)P.viscosity * fev;
            force = force + v3((double)(T)P.gravity[0], (double)(T)P.gravity[1], (double)(T)P.gravity[2]);
            size_t b = 4 * (size_t)i;
            acc_add(f[b], force.x); acc_add(f[b + 1], force.y); acc_add(f[b + 2], force.z);
        }
    }

    /* lambda_i = -C_i / (sum_k |grad_k C_i|^2 + eps), C_i = rho_i / rho0 - 1,
     * with the k = i term |sum_j grad W_ij / rho0|^2 (rx_sph_pbd.cpp:699-914). */
    void lambda_pass(const std::vector<T> &p) {
        const double r0 = (double)(T)P.rest_dens;
        if (nb) cross_sets(p, n, bpos, nb, fb_off, fb_idx);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(p, i);
            T rho = 0;
            V3 gsum = v3(0, 0, 0);
            T sd = 0;
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                int j = nidx[s];
                V3 d = xi - at(p, j);
                T r = (T)std::sqrt(dot(d, d));
                acc_add(rho, (double)(T)P.mass * K.W((double)r));
                V3 g = (K.G((double)r) * d) / r0;
                gsum = gsum + g;
                if (j != i) acc_add(sd, dot(g, g));
            }
            acc_add(sd, dot(gsum, gsum));
            if (nb) {
                /* boundary density and |grad C|^2 terms (rx_sph_pbd.cpp:728-748,
                 * 795-818), each boundary neighbour counted once as in
                 * rx_pbdsph_kernel.cu:577-664 */
                rho = rho + boundary_density(xi, i);
                for (int s = fb_off[i]; s < fb_off[i + 1]; ++s) {
                    int b = fb_idx[s];
                    V3 d = xi - bat(b);
                    T r = (T)std::sqrt(dot(d, d));
                    V3 g = ((double)bscale(b) * K.G((double)r) * d) / r0;
                    acc_add(sd, dot(g, g));
                }
            }
            T C = (T)((double)rho / r0) - (T)1;
            if (P.clamp_constraint && C < (T)0) C = (T)0;
            dens[i] = rho;
            lam[i] = (T)(-(double)C / ((double)sd + (double)(T)P.epsilon));
        }
        if (nb) boundary_lambda(p);
    }

    /* lambda_b of every boundary particle from its fluid neighbours at the
     * current positions and its boundary neighbours (rx_sph_pbd.cpp:825-913;
     * fluid neighbours found on the current positions as in
     * rx_pbdsph_kernel.cu:666-735). */
    void boundary_lambda(const std::vector<T> &p) {
        const double r0 = (double)(T)P.rest_dens;
        cross_sets(bpos, nb, p, n, bf_off, bf_idx);
#pragma omp parallel for schedule(static)
        for (int b = 0; b < nb; ++b) {
            V3 xb = bat(b);
            T brho = 0;
            for (int s = bf_off[b]; s < bf_off[b + 1]; ++s) {
                V3 d = at(p, bf_idx[s]) - xb;
                T r = (T)std::sqrt(dot(d, d));
                acc_add(brho, (double)(T)P.mass * K.W((double)r));
            }
            for (int s = bb_off[b]; s < bb_off[b + 1]; ++s) {
                int c = bb_idx[s];
                V3 d = bat(c) - xb;
                T r = (T)std::sqrt(dot(d, d));
                acc_add(brho, (double)((T)P.rest_dens * bvol[c]) * K.W((double)r));
            }
            T C = (T)((double)brho / r0) - (T)1;
            if (P.clamp_constraint && C < (T)0) C = (T)0;
            T sd = 0;
            for (int s = bf_off[b]; s < bf_off[b + 1]; ++s) {
                V3 d = xb - at(p, bf_idx[s]);
                T r = (T)std::sqrt(dot(d, d));
                V3 g = (K.G((double)r) * d) / r0;
                acc_add(sd, dot(g, g));
            }
            for (int s = bb_off[b]; s < bb_off[b + 1]; ++s) {
                int c = bb_idx[s];
                V3 d = xb - bat(c);
                T r = (T)std::sqrt(dot(d, d));
                V3 g = ((double)bscale(c) * K.G((double)r) * d) / r0;
                acc_add(sd, dot(g, g));
            }
            blam[b] = (T)(-(double)C / ((double)sd + (double)(T)P.epsilon));
        }
    }

    /* dp_i = sum_j (lambda_i + lambda_j + s_corr) grad W_ij / rho0,
     * s_corr = -k (W(r)/W(q h))^n dt^2 (rx_sph_pbd.cpp:925-1026). */
    void correction_pass(const std::vector<T> &p, T dt) {
        const double r0 = (double)(T)P.rest_dens;
        const T dq = (T)P.ap_q * (T)P.h;
        const T wq = (T)K.W((double)dq);
        if (nb) cross_sets(p, n, bpos, nb, fb_off, fb_idx);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(p, i);
            V3 acc = v3(0, 0, 0);
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                int j = nidx[s];
                V3 d = xi - at(p, j);
                T r = (T)std::sqrt(dot(d, d));
                if ((double)r > (double)(T)P.h) continue;
                T sc = 0;
                if (P.use_ap) {
                    T ww = (T)(K.W((double)r) / (double)wq);
                    sc = (T)(-(double)(T)P.ap_k * std::pow((double)ww, (double)(T)P.ap_n)) * dt * dt;
                }
                T coef = lam[i] + lam[j] + sc;
                acc = acc + ((double)coef * K.G((double)r) / r0) * d;
            }
            if (nb) {
                /* boundary terms (rx_sph_pbd.cpp:977-1019): lambda_b, and s_corr
                 * of rho0 psi_b / m scaled W */
                V3 accb = v3(0, 0, 0);
                for (int s = fb_off[i]; s < fb_off[i + 1]; ++s) {
                    int bj = fb_idx[s];
                    V3 d = xi - bat(bj);
                    T r = (T)std::sqrt(dot(d, d));
                    if ((double)r > (double)(T)P.h) continue;
                    T sc = 0;
                    if (P.use_ap) {
                        T ww = (T)((double)bscale(bj) * K.W((double)r) / (double)wq);
                        sc = (T)(-(double)(T)P.ap_k * std::pow((double)ww, (double)(T)P.ap_n)) * dt * dt;
                    }
                    T coef = lam[i] + blam[bj] + sc;
                    accb = accb + ((double)coef * K.G((double)r) / r0) * d;
                }
                acc = acc + accb;
            }
            size_t b = 4 * (size_t)i;
            dp[b] = (T)acc.x; dp[b + 1] = (T)acc.y; dp[b + 2] = (T)acc.z; dp[b + 3] = 0;
        }
    }

    void errors(double &e1, double &e2, double &emax) const {
        const double r0 = (double)(T)P.rest_dens;
        double s1 = 0, s2 = 0, m = 0;
        for (int i = 0; i < n; ++i) {
            double e = ((double)dens[i] - r0) / r0;
            s1 += e > 0 ? e : 0.0;
            s2 += std::fabs(e);
            m = std::max(m, std::fabs(e));
        }
        e1 = n ? s1 / n : 0.0; e2 = n ? s2 / n : 0.0; emax = m;
    }

    /* One PBF step (rxPBDSPH::Update, rx_sph_pbd.cpp:377-484) plus the XSPH
     * and vorticity extensions.  fixed_iters > 0 runs exactly that many
     * iterations instead of the tolerance loop.  Returns iterations executed. */
    int pbf_step(T dt, int fixed_iters) {
        std::fill(frc.begin(), frc.end(), (T)0);
        neighbors(pos);
        density(pos, dens);
        ext_visc(pos, vel, dens, frc);
        integrate(pos, vel, frc, ppos, pvel, dt);

        int it = 0;
        double e1 = 1, e2 = 1, em = 1;
        for (;;) {
            neighbors(ppos);
            lambda_pass(ppos);
            correction_pass(ppos, dt);
            for (size_t k = 0; k < ppos.size(); ++k) { ppos[k] += dp[k]; pvel[k] = 0; frc[k] = 0; }
            integrate(ppos, pvel, frc, ppos, pvel, dt);
            errors(e1, e2, em);
            ++it;
            double err = (P.error_mode == FSPH_ERR_TWO_SIDED) ? e2 : e1;
            if (fixed_iters > 0) {
                if (it >= fixed_iters) break;
                continue;
            }
            /* loop test of rx_sph_pbd.cpp:425,456 restated on the executed count */
            if (it >= P.max_iter) break;
            if (err <= (double)P.eta && it >= std::max(P.min_iter, 1)) break;
        }
        last_iters = it; last_err1 = e1; last_err2 = e2; last_errmax = em;

        /* v = (x* - x) / dt, x = x* (rx_sph_pbd.cpp:464-471) */
        for (size_t k = 0; k < pos.size(); ++k) {
            vel[k] = (ppos[k] - pos[k]) / dt;
            pos[k] = ppos[k];
        }
        if (P.xsph_c != 0.0f || P.vort_eps != 0.0f) finalize_extensions(dt);
        return it;
    }

    /* XSPH (rx_pbdsph_kernel.cu:1090-1162) and vorticity confinement
     * (Macklin & Mueller 2013, eq. 15-16, with the SPH curl weighted by the
     * neighbour volume m / rho_j, which the paper leaves to its eps), both
     * evaluated on the velocities v = (x* - x)/dt and the densities of the
     * last lambda pass:
     *   w_i   = sum_j (m / rho_j)(v_j - v_i) x grad_j W(x_i - x_j),  grad_j = -grad_i
     *   eta_i = sum_j (m / rho_j) (|w_j| - |w_i|) grad_i W(x_i - x_j)
     *   N_i   = eta_i / |eta_i|,  f_i = eps (N_i x w_i)
     *   v_i  <- v_i + c sum_j (m / rho_j)(v_j - v_i) W(r_ij) + dt f_i        */
    void finalize_extensions(T dt) {
        neighbors(pos);
        const double m = (double)(T)P.mass;
        std::vector<T> vnew(vel);
        std::vector<double> wmag(n, 0.0);
        std::vector<V3> w(n);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(pos, i), vi = at(vel, i);
            V3 om = v3(0, 0, 0), xs = v3(0, 0, 0);
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                int j = nidx[s];
                if (j == i) continue;
                V3 d = xi - at(pos, j);
                T r = (T)std::sqrt(dot(d, d));
                V3 vij = at(vel, j) - vi;
                V3 gi = K.G((double)r) * d;
                om = om + (m / (double)dens[j]) * cross(vij, -1.0 * gi);
                xs = xs + (m / (double)dens[j] * K.W((double)r)) * vij;
            }
            w[i] = om;
            wmag[i] = std::sqrt(dot(om, om));
            size_t b = 4 * (size_t)i;
            vnew[b] = (T)(vi.x + (double)(T)P.xsph_c * xs.x);
            vnew[b + 1] = (T)(vi.y + (double)(T)P.xsph_c * xs.y);
            vnew[b + 2] = (T)(vi.z + (double)(T)P.xsph_c * xs.z);
            vort[b] = (T)om.x; vort[b + 1] = (T)om.y; vort[b + 2] = (T)om.z; vort[b + 3] = 0;
        }
        if (P.vort_eps != 0.0f) {
#pragma omp parallel for schedule(static)
            for (int i = 0; i < n; ++i) {
                V3 xi = at(pos, i);
                V3 eta = v3(0, 0, 0);
                for (int s = noff[i]; s < noff[i + 1]; ++s) {
                    int j = nidx[s];
                    if (j == i) continue;
                    V3 d = xi - at(pos, j);
                    T r = (T)std::sqrt(dot(d, d));
                    eta = eta + ((m / (double)dens[j]) * (wmag[j] - wmag[i]) * K.G((double)r)) * d;
                }
                double en = std::sqrt(dot(eta, eta));
                if (en > 1e-30) {
                    V3 N = eta / en;
                    V3 f = (double)(T)P.vort_eps * cross(N, w[i]);
                    size_t b = 4 * (size_t)i;
                    vnew[b] = (T)((double)vnew[b] + (double)dt * f.x);
                    vnew[b + 1] = (T)((double)vnew[b + 1] + (double)dt * f.y);
                    vnew[b + 2] = (T)((double)vnew[b + 2] + (double)dt * f.z);
                }
            }
        }
        vel.swap(vnew);
    }

    /* The density field on a lattice for meshing (rxPBDSPH::CalImplicitField
     * -> GetImplicit -> CalColorField, rx_sph_pbd.cpp:2024-2108): node (i, j, k)
     * at minp + (i, j, k) d (double), 0 outside the simulation range (the
     * box grown by 1 %, rx_sph_pbd.cpp:188-196), else sum_j m W(r_j) over the
     * particles with fl(|x - x_j|^2) <= fl(h h), r_j = fl(sqrt(Dist2)),
     * accumulated in T; out[k nx ny + j nx + i]. */
    void density_grid(const int nn[3], const double minp[3], const double dd[3], float *out) const {
        double lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            const double size = P.box_max[a] - P.box_min[a];
            lo[a] = P.box_min[a] - 0.5 * 0.01 * size;
            hi[a] = lo[a] + size * (1.0 + 0.01);
        }
        const T hT = (T)P.h;
        const T h2 = hT * hT;
        const double cw = (double)P.h * 1.0001;
        int g[3];
        for (int a = 0; a < 3; ++a) g[a] = std::max(1, (int)std::floor((hi[a] - lo[a]) / cw) + 1);
        const size_t C = (size_t)g[0] * g[1] * g[2];
        std::vector<int> cnt(C + 1, 0), cellOf(n), order(n);
        auto cell3 = [&](const double x[3], int c[3]) {
            for (int a = 0; a < 3; ++a) c[a] = std::min(std::max((int)std::floor((x[a] - lo[a]) / cw), 0), g[a] - 1);
        };
        for (int i = 0; i < n; ++i) {
            double x[3] = {(double)pos[4 * (size_t)i], (double)pos[4 * (size_t)i + 1], (double)pos[4 * (size_t)i + 2]};
            int c[3];
            cell3(x, c);
            cellOf[i] = (int)(((size_t)c[2] * g[1] + c[1]) * g[0] + c[0]);
            cnt[cellOf[i] + 1]++;
        }
        for (size_t c = 0; c < C; ++c) cnt[c + 1] += cnt[c];
        {
            std::vector<int> fill(cnt.begin(), cnt.end() - 1);
            for (int i = 0; i < n; ++i) order[fill[cellOf[i]]++] = i;
        }
        const double m = (double)(T)P.mass;
        const long long tot = (long long)nn[0] * nn[1] * nn[2];
#pragma omp parallel for schedule(static)
        for (long long t = 0; t < tot; ++t) {
            const int i = (int)(t % nn[0]), j = (int)((t / nn[0]) % nn[1]), k = (int)(t / ((long long)nn[0] * nn[1]));
            const double x[3] = {minp[0] + i * dd[0], minp[1] + j * dd[1], minp[2] + k * dd[2]};
            T c = 0;
            bool inside = true;
            for (int a = 0; a < 3; ++a) inside = inside && x[a] >= lo[a] && x[a] <= hi[a];
            if (inside) {
                int cc[3];
                cell3(x, cc);
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int z = cc[2] + dz, y = cc[1] + dy, xx = cc[0] + dx;
                            if (xx < 0 || y < 0 || z < 0 || xx >= g[0] || y >= g[1] || z >= g[2]) continue;
                            const size_t cell = ((size_t)z * g[1] + y) * g[0] + xx;
                            for (int s = cnt[cell]; s < cnt[cell + 1]; ++s) {
                                const int q = order[s];
                                const V3 dv = v3(x[0], x[1], x[2]) - at(pos, q);
                                const T d2 = (T)dot(dv, dv);
                                if (d2 <= h2) {
                                    const T r = (T)std::sqrt((double)d2);
                                    acc_add(c, m * K.W((double)r));
                                }
                            }
                        }
            }
            out[t] = (float)c;
        }
    }

    /* ---------------- WCSPH ---------------- */
    /* p = k (rho - rho0); a_i = -sum m (p_i/rho_i^2 + p_j/rho_j^2) gradW
     *   + mu sum m (v_j - v_i)/rho_j lapW + g (rx_sph_cpu.cpp:558-656). */
    void sph_forces(const std::vector<T> &p, const std::vector<T> &v) {
        const T r0 = (T)P.rest_dens;
        for (int i = 0; i < n; ++i) pres[i] = (T)P.gas_k * (dens[i] - r0);
#pragma omp parallel for schedule(static)
        for (int i = 0; i < n; ++i) {
            V3 xi = at(p, i), vi = at(v, i);
            T prsi = pres[i] / (dens[i] * dens[i]);
            V3 fp = v3(0, 0, 0), fev = v3(0, 0, 0);
            for (int s = noff[i]; s < noff[i + 1]; ++s) {
                int j = nidx[s];
                if (j == i) continue;
                V3 d = xi - at(p, j), vji = at(v, j) - vi;
                T r = (T)std::sqrt(dot(d, d));
                T prsj = pres[j] / (dens[j] * dens[j]);
                fp = fp + ((double)(T)P.mass * (double)(prsi + prsj) * K.G((double)r)) * d;
                fev = fev + ((double)(T)P.mass * K.L((double)r)) * (vji / (double)dens[j]);
            }
            V3 force = (-1.0 * fp) + (double)(T)P.viscosity * fev +
                       v3((double)(T)P.gravity[0], (double)(T)P.gravity[1], (double)(T)P.gravity[2]);
            size_t b = 4 * (size_t)i;
            frc[b] = (T)force.x; frc[b + 1] = (T)force.y; frc[b + 2] = (T)force.z; frc[b + 3] = 0;
        }
    }

    void sph_step(T dt) {
        neighbors(pos);
        density(pos, dens);
        sph_forces(pos, vel);
        integrate(pos, vel, frc, pos, vel, dt);
    }
};

template <class T>
struct Handle {
    Solver<T> s;
    explicit Handle(const fsph_params &p) : s(p) {}
};

template <class T>
void set_obstacles(Solver<T> *S, const double *rec, int n) {
    S->obs.clear();
    const double d2r = 3.14159265358979323846 / 180.0;
    for (int k = 0; k < n; ++k) {
        const double *q = rec + 11 * (size_t)k;
        typename Solver<T>::Obs ob{};
        ob.type = (int)q[0];
        for (int a = 0; a < 3; ++a) {
            ob.cen[a] = q[1 + a];
            ob.ext[a] = q[4 + a];
        }
        ob.rad = q[10];
        /* EulerToMatrix (rx_sph_commons.h:185-210): degrees, (pitch, yaw, roll) */
        const double cp = std::cos(q[7] * d2r), sp = std::sin(q[7] * d2r);
        const double cy = std::cos(q[8] * d2r), sy = std::sin(q[8] * d2r);
        const double cr = std::cos(q[9] * d2r), sr = std::sin(q[9] * d2r);
        const double cc = cy * cr, cs = cy * sr, sc = sy * cr, ss = sy * sr;
        const double m[3][3] = {{cc + sp * ss, cs - sp * sc, -sy * cp}, {-cp * sr, cp * cr, -sp},
                                {sc - sp * cs, ss + sp * cc, cy * cp}};
        std::memcpy(ob.R, m, sizeof(m));
        S->obs.push_back(ob);
    }
}

template <class T>
void load4(std::vector<T> &dst, const float *src, int n) {
    for (size_t k = 0; k < 4 * (size_t)n; ++k) dst[k] = src ? (T)src[k] : (T)0;
}
template <class T>
void store(float *dst, const std::vector<T> &src) {
    for (size_t k = 0; k < src.size(); ++k) dst[k] = (float)src[k];
}

}  // namespace

extern "C" {

/* precision: 0 = float (reference arithmetic), 1 = double (FP64 oracle).
 * The handle is a tagged pointer to a Solver<float> or Solver<double>. */
struct fsph_orc {
    int prec;
    void *s;
};

void fsph_orc_threads(int t) {
#ifdef _OPENMP
    omp_set_num_threads(t > 0 ? t : 1);
#else
    (void)t;
#endif
}

fsph_orc *fsph_orc_create(const fsph_params *p, int prec, int n) {
    fsph_orc *o = new fsph_orc{prec, nullptr};
    if (prec) { auto *s = new Solver<double>(*p); s->resize(n); o->s = s; }
    else { auto *s = new Solver<float>(*p); s->resize(n); o->s = s; }
    return o;
}

void fsph_orc_destroy(fsph_orc *o) {
    if (!o) return;
    if (o->prec) delete (Solver<double> *)o->s; else delete (Solver<float> *)o->s;
    delete o;
}

#define ORC_DISPATCH(o, expr)                                   \
    do {                                                        \
        if ((o)->prec) { auto *S = (Solver<double> *)(o)->s; expr; } \
        else { auto *S = (Solver<float> *)(o)->s; expr; }        \
    } while (0)

void fsph_orc_set(fsph_orc *o, const float *pos4, const float *vel4) {
    ORC_DISPATCH(o, { load4(S->pos, pos4, S->n); load4(S->vel, vel4, S->n); });
}

/* Static boundary particles (float4 positions); computes their volumes. */
void fsph_orc_set_boundary(fsph_orc *o, const float *bpos4, int nb) {
    ORC_DISPATCH(o, S->set_boundary(bpos4, nb));
}

/* which: 0 volume psi_b, 1 lambda_b of the last lambda pass (nb floats) */
void fsph_orc_get_boundary(fsph_orc *o, int which, float *out) {
    ORC_DISPATCH(o, {
        if (which == 0) store(out, S->bvol);
        else store(out, S->blam);
    });
}

/* which: 0 pos, 1 vel, 2 dens, 3 lambda, 4 dp, 5 predicted pos, 6 force, 7 pressure, 8 vorticity */
void fsph_orc_get(fsph_orc *o, int which, float *out) {
    ORC_DISPATCH(o, {
        switch (which) {
        case 0: store(out, S->pos); break;
        case 1: store(out, S->vel); break;
        case 2: store(out, S->dens); break;
        case 3: store(out, S->lam); break;
        case 4: store(out, S->dp); break;
        case 5: store(out, S->ppos); break;
        case 6: store(out, S->frc); break;
        case 7: store(out, S->pres); break;
        case 8: store(out, S->vort); break;
        }
    });
}

/* Returns iterations; errs[0..2] = one-sided, two-sided, max error. */
int fsph_orc_pbf_step(fsph_orc *o, float dt, int fixed_iters, double *errs) {
    int it = 0;
    ORC_DISPATCH(o, {
        it = S->pbf_step(dt, fixed_iters);
        if (errs) { errs[0] = S->last_err1; errs[1] = S->last_err2; errs[2] = S->last_errmax; }
    });
    return it;
}

void fsph_orc_sph_step(fsph_orc *o, float dt) { ORC_DISPATCH(o, S->sph_step(dt)); }

/* Analytic obstacles: n records of 11 doubles -- type (0 box, 1 sphere),
 * centre xyz, half extents xyz, Euler angles in degrees (pitch, yaw, roll;
 * EulerToMatrix, rx_sph_commons.h:185-210), sphere radius. */
void fsph_orc_set_obstacles(fsph_orc *o, const double *rec, int n) {
    if (o->prec) set_obstacles((Solver<double> *)o->s, rec, n);
    else set_obstacles((Solver<float> *)o->s, rec, n);
}

/* Triangle-mesh obstacles: nv float vertices (xyz), nt triangles (3 ints);
 * replaces any mesh set before. */
void fsph_orc_set_polygons(fsph_orc *o, const float *vrts, int nv, const int *tris, int nt) {
    ORC_DISPATCH(o, S->mesh.set(vrts, nv, tris, nt, S->P));
}

/* The mesh collision alone: x1 and v (float4 stride) updated from x0 -> x1. */
extern "C++" template <class T>
void polygon_collide(Solver<T> *S, const float *x0, float *x1, float *v, int n, float dt) {
    for (int i = 0; i < n; ++i) {
        const size_t b = 4 * (size_t)i;
        V3 a = v3(x0[b], x0[b + 1], x0[b + 2]);
        V3 c = v3(x1[b], x1[b + 1], x1[b + 2]);
        V3 w = v3(v[b], v[b + 1], v[b + 2]);
        if (S->mesh.nt) S->mesh.collide(a, c, w, (T)dt);
        x1[b] = (float)c.x; x1[b + 1] = (float)c.y; x1[b + 2] = (float)c.z;
        v[b] = (float)w.x; v[b + 1] = (float)w.y; v[b + 2] = (float)w.z;
    }
}
void fsph_orc_polygon_collide(fsph_orc *o, const float *x0, float *x1, float *v, int n, float dt) {
    if (o->prec) polygon_collide((Solver<double> *)o->s, x0, x1, v, n, dt);
    else polygon_collide((Solver<float> *)o->s, x0, x1, v, n, dt);
}

/* rxPBDSPH::CalImplicitField of the current positions (see Solver::density_grid). */
void fsph_orc_density_grid(fsph_orc *o, const int *nn, const double *minp, const double *d, float *out) {
    ORC_DISPATCH(o, S->density_grid(nn, minp, d, out));
}

/* The solid projection (obstacles, then the box walls) of n points. */
void fsph_orc_project(fsph_orc *o, const float *pos4, int n, float *out4) {
    ORC_DISPATCH(o, {
        for (int i = 0; i < n; ++i) {
            V3 x = v3(pos4[4 * (size_t)i], pos4[4 * (size_t)i + 1], pos4[4 * (size_t)i + 2]);
            x = S->wall(x);
            out4[4 * (size_t)i] = (float)x.x; out4[4 * (size_t)i + 1] = (float)x.y;
            out4[4 * (size_t)i + 2] = (float)x.z; out4[4 * (size_t)i + 3] = 0.0f;
        }
    });
}

/* XSPH + vorticity confinement alone (the end of pbf_step) on the given
 * positions, velocities and densities: velocity after both, and omega. */
void fsph_orc_finalize_ext(fsph_orc *o, const float *pos4, const float *vel4, const float *dens, float dt,
                           float *vel_out4, float *vort4) {
    ORC_DISPATCH(o, {
        load4(S->pos, pos4, S->n);
        load4(S->vel, vel4, S->n);
        for (int i = 0; i < S->n; ++i) S->dens[i] = dens[i];
        S->finalize_extensions(dt);
        store(vel_out4, S->vel);
        store(vort4, S->vort);
    });
}

/* Neighbour CSR of the given positions (ascending indices). */
long long fsph_orc_neighbors(fsph_orc *o, const float *pos4, int *offsets, int *idx, long long cap) {
    long long total = 0;
    ORC_DISPATCH(o, {
        load4(S->ppos, pos4, S->n);
        S->neighbors(S->ppos);
        for (int i = 0; i <= S->n; ++i) offsets[i] = S->noff[i];
        total = (long long)S->nidx.size();
        for (long long k = 0; k < total && k < cap; ++k) idx[k] = S->nidx[k];
    });
    return total;
}

void fsph_orc_pbf_lambda(fsph_orc *o, const float *pos4, float *dens, float *lam) {
    ORC_DISPATCH(o, {
        load4(S->ppos, pos4, S->n);
        S->neighbors(S->ppos);
        S->lambda_pass(S->ppos);
        store(dens, S->dens); store(lam, S->lam);
    });
}

void fsph_orc_pbf_correction(fsph_orc *o, const float *pos4, const float *lam, float dt, float *dp4) {
    ORC_DISPATCH(o, {
        load4(S->ppos, pos4, S->n);
        for (int i = 0; i < S->n; ++i) S->lam[i] = lam[i];
        S->neighbors(S->ppos);
        S->correction_pass(S->ppos, dt);
        store(dp4, S->dp);
    });
}

void fsph_orc_sph_forces(fsph_orc *o, const float *pos4, const float *vel4, float *dens, float *pres, float *acc4) {
    ORC_DISPATCH(o, {
        load4(S->pos, pos4, S->n); load4(S->vel, vel4, S->n);
        S->neighbors(S->pos);
        S->density(S->pos, S->dens);
        S->sph_forces(S->pos, S->vel);
        store(dens, S->dens); store(pres, S->pres); store(acc4, S->frc);
    });
}

/* Predict (density + ext/visc + integrate) only, the PBF pre-pass. */
void fsph_orc_pbf_predict(fsph_orc *o, float dt, float *dens, float *frc4, float *ppos4, float *pvel4) {
    ORC_DISPATCH(o, {
        std::fill(S->frc.begin(), S->frc.end(), 0);
        S->neighbors(S->pos);
        S->density(S->pos, S->dens);
        S->ext_visc(S->pos, S->vel, S->dens, S->frc);
        S->integrate(S->pos, S->vel, S->frc, S->ppos, S->pvel, dt);
        store(dens, S->dens); store(frc4, S->frc); store(ppos4, S->ppos); store(pvel4, S->pvel);
    });
}

double fsph_orc_kernel(int which, double r, double h) {
    Kern K(h);
    switch (which) {
    case 0: return K.W(r);
    case 1: return K.G(r);
    case 2: return K.L(r);
    }
    return 0.0;
}

/* Rest density by calRestDensity (rx_sph_pbd.cpp:1035-1049): poly6 sum over a
 * cubic lattice of spacing l around the origin, in float accumulation. */
double fsph_orc_lattice_density(double h, double mass, double spacing) {
    Kern K((float)h);
    float r0 = 0.0f;
    const float l = (float)spacing;
    int nn = (int)std::ceil((float)h / l) + 1;
    for (int x = -nn; x <= nn; ++x)
        for (int y = -nn; y <= nn; ++y)
            for (int z = -nn; z <= nn; ++z) {
                double r = std::sqrt((double)(x * l) * (x * l) + (double)(y * l) * (y * l) + (double)(z * l) * (z * l));
                r0 = (float)((double)r0 + (double)(float)mass * K.W(r));
            }
    return r0;
}

void fsph_orc_wall(const fsph_params *p, const double *pos, double *out) {
    Solver<double> s(*p);
    V3 q = s.wall(v3(pos[0], pos[1], pos[2]));
    out[0] = q.x; out[1] = q.y; out[2] = q.z;
}

}  // extern "C"
