// ORACLE — test infrastructure only (tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py may load it; the product never does).
//
// CPU restatement (FP64, OpenMP) of the reference's injective-deformation
// Newton step: surface extraction, neo-Hookean tet energy/gradient/projected
// Hessian, IPC constraint set with the reference's spatial hash, barrier
// energy/gradient/projected Hessian, additive CCD step size, min distance and
// kappa initialisation. The Newton loop itself is in oracle/newton.py.
//
// Parity status: UNPINNED. The reference has no tests or golden vectors and
// cannot be compiled in this environment (Eigen, Boost, CHOLMOD, Kokkos are
// absent). This file follows the cited reference lines; it is validated by
// analytic known-answer cases and finite-difference checks.
#include <cstdio>
#include <cstring>
#include <cstdint>
#include <cmath>
#include <vector>
#include <map>
#include <set>
#include <array>
#include <unordered_map>
#include <algorithm>
#include "geom.hpp"
#include "deriv.hpp"
#include "shell.hpp"

using namespace ora;

namespace {

// ---------------------------------------------------------------------------
// symmetric eigen-decomposition (cyclic Jacobi) and PSD projection.
// Restates makePD (Math/UTILS.h:10-27): if the smallest eigenvalue is >= 0
// the matrix is left unchanged; otherwise negative eigenvalues are set to 0
// and the matrix is rebuilt from its eigenvectors.
// ---------------------------------------------------------------------------
void jacobi_eigen(int n, const double* A, double* w, double* V) {
    std::vector<double> a(A, A + n * n);
    for (int i = 0; i < n * n; ++i) V[i] = 0;
    for (int i = 0; i < n; ++i) V[i * n + i] = 1;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += a[i * n + j] * a[i * n + j];
                if (i != j) off += a[i * n + j] * a[i * n + j];
            }
        if (off <= 1e-30 * tot || off == 0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = a[p * n + q];
                if (apq == 0) continue;
                double app = a[p * n + p], aqq = a[q * n + q];
                double theta = (aqq - app) / (2 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) w[i] = a[i * n + i];
}

void make_pd(int n, double* A) {
    double w[12], V[144];
    jacobi_eigen(n, A, w, V);
    double wmin = w[0];
    for (int i = 1; i < n; ++i) wmin = std::min(wmin, w[i]);
    if (wmin >= 0) return;
    for (int i = 0; i < n; ++i) w[i] = std::max(w[i], 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            double s = 0;
            for (int k = 0; k < n; ++k) s += V[i * n + k] * w[k] * V[j * n + k];
            A[i * n + j] = s;
        }
}

// ---------------------------------------------------------------------------
// 3x3 helpers (row-major double[9]); F(i,j) = F[i*3+j]
// ---------------------------------------------------------------------------
double det3(const double* F) {
    return F[0] * (F[4] * F[8] - F[5] * F[7]) - F[1] * (F[3] * F[8] - F[5] * F[6]) + F[2] * (F[3] * F[7] - F[4] * F[6]);
}
void cofactor3(const double* F, double* C) {
    C[0] = F[4] * F[8] - F[5] * F[7];
    C[1] = F[5] * F[6] - F[3] * F[8];
    C[2] = F[3] * F[7] - F[4] * F[6];
    C[3] = F[2] * F[7] - F[1] * F[8];
    C[4] = F[0] * F[8] - F[2] * F[6];
    C[5] = F[1] * F[6] - F[0] * F[7];
    C[6] = F[1] * F[5] - F[2] * F[4];
    C[7] = F[2] * F[3] - F[0] * F[5];
    C[8] = F[0] * F[4] - F[1] * F[3];
}

// SVD F = U diag(sigma) V^T with det(U) = det(V) = 1 (sigma[2] takes the sign
// of det F), from the eigen-decomposition of F^T F, like
// Math/SINGULAR_VALUE_DECOMPOSITION.h:23-177.
void svd3(const double* F, double* U, double* sigma, double* V) {
    double FtF[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) FtF[i * 3 + j] = F[0 * 3 + i] * F[0 * 3 + j] + F[1 * 3 + i] * F[1 * 3 + j] + F[2 * 3 + i] * F[2 * 3 + j];
    double w[3], Vt[9];
    jacobi_eigen(3, FtF, w, Vt);
    int order[3] = {0, 1, 2};
    std::sort(order, order + 3, [&](int a, int b) { return w[a] > w[b]; });
    for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) V[r * 3 + c] = Vt[r * 3 + order[c]];
    if (det3(V) < 0)
        for (int r = 0; r < 3; ++r) V[r * 3 + 2] = -V[r * 3 + 2];
    // U columns = F v_c / |F v_c|, Gram-Schmidt, last column by cross product
    double FV[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) FV[r * 3 + c] = F[r * 3 + 0] * V[0 * 3 + c] + F[r * 3 + 1] * V[1 * 3 + c] + F[r * 3 + 2] * V[2 * 3 + c];
    V3 u0{FV[0], FV[3], FV[6]}, u1{FV[1], FV[4], FV[7]};
    double s0 = std::sqrt(sq(u0));
    u0 = (1.0 / s0) * u0;
    u1 = u1 - dot(u1, u0) * u0;
    double n1 = std::sqrt(sq(u1));
    if (n1 > 1e-300) u1 = (1.0 / n1) * u1;
    else {
        V3 t = std::fabs(u0.x) < 0.9 ? V3{1, 0, 0} : V3{0, 1, 0};
        u1 = cross(u0, t);
        u1 = (1.0 / std::sqrt(sq(u1))) * u1;
    }
    V3 u2 = cross(u0, u1);
    double Ua[9] = {u0.x, u1.x, u2.x, u0.y, u1.y, u2.y, u0.z, u1.z, u2.z};
    std::memcpy(U, Ua, sizeof(Ua));
    // sigma_c = u_c . F v_c
    for (int c = 0; c < 3; ++c) sigma[c] = U[0 * 3 + c] * FV[0 * 3 + c] + U[1 * 3 + c] * FV[1 * 3 + c] + U[2 * 3 + c] * FV[2 * 3 + c];
}

// F = Ds * IB (FEM/DEFORMATION_GRADIENT.h:112-144)
void deformation_gradient(const double* X, const int* t, const double* IB, double* F) {
    const double* x0 = X + 3 * t[0];
    double Ds[9];
    for (int m = 0; m < 3; ++m) {
        const double* xm = X + 3 * t[m + 1];
        for (int i = 0; i < 3; ++i) Ds[i * 3 + m] = xm[i] - x0[i];
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) F[i * 3 + j] = Ds[i * 3 + 0] * IB[0 * 3 + j] + Ds[i * 3 + 1] * IB[1 * 3 + j] + Ds[i * 3 + 2] * IB[2 * 3 + j];
}

// The two means of the CCD hash in the reference's own order
// (SPATIAL_HASH.h:455-475).
//
// eigen_sum: `eLen.mean()` is Eigen's sum() / size(). For a dense double
// vector on an AVX build (the reference compiles with -mavx2,
// CMakeLists.txt:20) Eigen's redux (Eigen/src/Core/Redux.h,
// LinearVectorizedTraversal, storage 32-byte aligned) keeps two 4-lane
// accumulators: lane l of the first sums items l, l+8, l+16, ... and lane l
// of the second items 4+l, 12+l, ... over the first 8*floor(n/8) items; the
// accumulators are added lane by lane, one more 4-item packet is added when
// n mod 8 >= 4, the four lanes are reduced by the AVX predux as
// (l0 + l2) + (l1 + l3) (Eigen 3.3/3.4), and the last n mod 4 items are added
// one at a time. Fewer than 4 items are summed left to right.
double eigen_sum(const double* x, long n) {
    if (n <= 0) return 0.0;
    const long aligned = n & ~3L, aligned2 = n & ~7L;
    double res;
    if (aligned == 0) {
        res = x[0];
        for (long i = 1; i < n; ++i) res += x[i];
        return res;
    }
    double p0[4] = {x[0], x[1], x[2], x[3]};
    if (aligned > 4) {
        double p1[4] = {x[4], x[5], x[6], x[7]};
        for (long i = 8; i < aligned2; i += 8)
            for (int l = 0; l < 4; ++l) {
                p0[l] += x[i + l];
                p1[l] += x[i + 4 + l];
            }
        for (int l = 0; l < 4; ++l) p0[l] += p1[l];
        if (aligned > aligned2)
            for (int l = 0; l < 4; ++l) p0[l] += x[aligned2 + l];
    }
    res = (p0[0] + p0[2]) + (p0[1] + p0[3]);
    for (long i = aligned; i < n; ++i) res += x[i];
    return res;
}

// pSize: the reference's serial loop, |dir_x| + |dir_y| + |dir_z| of every
// surface node in node order into one accumulator.
double serial_sum(const double* x, long n) {
    double s = 0.0;
    for (long i = 0; i < n; ++i) s += x[i];
    return s;
}

// ---------------------------------------------------------------------------
// Spatial hash, restating Grid/SPATIAL_HASH.h
// ---------------------------------------------------------------------------
struct SpatialHash {
    V3 lbc;
    double inv;
    int vc[3];
    long vc01;
    int surfEdgeStart, surfTriStart;
    std::unordered_map<long, std::vector<int>> voxel;
    std::vector<std::vector<long>> occ;  // CCD occupancy of points and edges

    void axis_index(V3 p, int* a) const {
        a[0] = (int)std::floor((p.x - lbc.x) * inv);
        a[1] = (int)std::floor((p.y - lbc.y) * inv);
        a[2] = (int)std::floor((p.z - lbc.z) * inv);
    }
    long vidx(int ix, int iy, int iz) const { return ix + (long)iy * vc[0] + (long)iz * vc01; }

    void finish_grid(V3 lo, V3 hi, double voxelSize) {
        lbc = lo;
        double range[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
        inv = 1.0 / voxelSize;
        long vcl[3];
        for (int d = 0; d < 3; ++d) vcl[d] = std::max<long>((long)std::ceil(range[d] * inv), 1);
        double amt = (double)vcl[0] * (double)vcl[1] * (double)vcl[2];
        if (amt > 1e9) {  // SPATIAL_HASH.h:74-78
            voxelSize *= std::pow(amt / 1.0e9, 1.0 / 3);
            inv = 1.0 / voxelSize;
        }
        for (int d = 0; d < 3; ++d) vc[d] = std::max((int)std::ceil(range[d] * inv), 1);
        if (std::min(vc[0], std::min(vc[1], vc[2])) <= 0) {
            double rmax = std::max(range[0], std::max(range[1], range[2]));
            inv = 1.0 / (rmax * 1.01);
            vc[0] = vc[1] = vc[2] = 1;
        }
        vc01 = (long)vc[0] * vc[1];
    }

    // CCS build: SPATIAL_HASH.h:28-213
    void build_ccs(int V, const double* X, int nN, const int* nodes, int nE, const int* edges, int nT, const int* tris) {
        double voxelSize = 1.0;
        if (nE) {
            std::vector<double> len(nE);
            for (int e = 0; e < nE; ++e) len[e] = std::sqrt(sq(v3(X + 3 * edges[2 * e]) - v3(X + 3 * edges[2 * e + 1])));
            voxelSize *= eigen_sum(len.data(), nE) / (double)nE;
        }
        V3 lo = v3(X), hi = v3(X);
        for (int i = 1; i < V; ++i) {
            V3 p = v3(X + 3 * i);
            lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
            hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
        }
        finish_grid(lo, hi, voxelSize);
        surfEdgeStart = nN;
        surfTriStart = nN + nE;
        std::vector<std::array<int, 3>> ai(V);
        for (int s = 0; s < nN; ++s) axis_index(v3(X + 3 * nodes[s]), ai[nodes[s]].data());
        voxel.clear();
        for (int s = 0; s < nN; ++s) {
            auto& a = ai[nodes[s]];
            voxel[vidx(a[0], a[1], a[2])].push_back(s);
        }
        auto add_box = [&](const int* vs, int k, int id) {
            int mn[3], mx[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = mx[d] = ai[vs[0]][d];
                for (int j = 1; j < k; ++j) {
                    mn[d] = std::min(mn[d], ai[vs[j]][d]);
                    mx[d] = std::max(mx[d], ai[vs[j]][d]);
                }
            }
            for (int iz = mn[2]; iz <= mx[2]; ++iz)
                for (int iy = mn[1]; iy <= mx[1]; ++iy)
                    for (int ix = mn[0]; ix <= mx[0]; ++ix) voxel[vidx(ix, iy, iz)].push_back(id);
        };
        for (int e = 0; e < nE; ++e) add_box(edges + 2 * e, 2, e + surfEdgeStart);
        for (int t = 0; t < nT; ++t) add_box(tris + 3 * t, 3, t + surfTriStart);
    }

    void query_box(V3 lo, V3 hi, int* mn, int* mx) const {
        axis_index(lo, mn);
        axis_index(hi, mx);
        for (int d = 0; d < 3; ++d) {
            mn[d] = std::max(mn[d], 0);
            mx[d] = std::min(mx[d], vc[d] - 1);
        }
    }

    // Query_Point_For_Triangles: SPATIAL_HASH.h:215-241
    void query_point_tris(V3 p, double r, std::vector<int>& out) const {
        int mn[3], mx[3];
        query_box(p - V3{r, r, r}, p + V3{r, r, r}, mn, mx);
        std::set<int> s;
        for (int iz = mn[2]; iz <= mx[2]; ++iz)
            for (int iy = mn[1]; iy <= mx[1]; ++iy)
                for (int ix = mn[0]; ix <= mx[0]; ++ix) {
                    auto it = voxel.find(vidx(ix, iy, iz));
                    if (it == voxel.end()) continue;
                    for (int id : it->second)
                        if (id >= surfTriStart) s.insert(id - surfTriStart);
                }
        out.assign(s.begin(), s.end());
    }
    // Query_Edge_For_Edges: SPATIAL_HASH.h:243-291
    void query_edge_edges(V3 a, V3 b, double r, int eIq, std::vector<int>& out) const {
        V3 lo{std::min(a.x, b.x) - r, std::min(a.y, b.y) - r, std::min(a.z, b.z) - r};
        V3 hi{std::max(a.x, b.x) + r, std::max(a.y, b.y) + r, std::max(a.z, b.z) + r};
        int mn[3], mx[3];
        query_box(lo, hi, mn, mx);
        out.clear();
        for (int iz = mn[2]; iz <= mx[2]; ++iz)
            for (int iy = mn[1]; iy <= mx[1]; ++iy)
                for (int ix = mn[0]; ix <= mx[0]; ++ix) {
                    auto it = voxel.find(vidx(ix, iy, iz));
                    if (it == voxel.end()) continue;
                    for (int id : it->second)
                        if (id >= surfEdgeStart && id < surfTriStart && id - surfEdgeStart > eIq) out.push_back(id - surfEdgeStart);
                }
        std::sort(out.begin(), out.end());
        out.erase(std::unique(out.begin(), out.end()), out.end());
    }

    // CCD build: SPATIAL_HASH.h:432-622 (including the span cap at :466-482)
    void build_ccd(const double* X, int nN, const int* nodes, int nE, const int* edges, int nT, const int* tris,
                   const double* dir, double& curMaxStepSize, double thickness) {
        double voxelSize = 1.0;
        if (nE) {
            std::vector<double> len(nE);
            for (int e = 0; e < nE; ++e) len[e] = std::sqrt(sq(v3(X + 3 * edges[2 * e]) - v3(X + 3 * edges[2 * e + 1])));
            voxelSize *= eigen_sum(len.data(), nE) / (double)nE;
        }
        std::vector<double> ad(3 * (size_t)nN);
        for (int s = 0; s < nN; ++s)
            for (int d = 0; d < 3; ++d) ad[3 * s + d] = std::fabs(dir[3 * nodes[s] + d]);
        double pSize = serial_sum(ad.data(), 3L * nN) / (double)(nN * 3);
        double spanSize = curMaxStepSize * pSize / voxelSize;
        if (spanSize > 1) curMaxStepSize /= spanSize;

        std::vector<V3> SV(nN), SVt(nN);
        std::unordered_map<int, int> v2s;
        for (int s = 0; s < nN; ++s) {
            int v = nodes[s];
            v2s[v] = s;
            SV[s] = v3(X + 3 * v);
            SVt[s] = {X[3 * v] + curMaxStepSize * dir[3 * v], X[3 * v + 1] + curMaxStepSize * dir[3 * v + 1],
                      X[3 * v + 2] + curMaxStepSize * dir[3 * v + 2]};
        }
        V3 lo = SV[0], hi = SV[0];
        for (int s = 0; s < nN; ++s) {
            for (V3 p : {SV[s], SVt[s]}) {
                lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
                hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
            }
        }
        double ht = thickness / 2;
        lo = lo - V3{ht, ht, ht};
        hi = hi + V3{ht, ht, ht};
        finish_grid(lo, hi, voxelSize);
        surfEdgeStart = nN;
        surfTriStart = nN + nE;
        std::vector<std::array<int, 3>> mnA(nN), mxA(nN);
        for (int s = 0; s < nN; ++s) {
            V3 mnc{std::min(SV[s].x, SVt[s].x) - ht, std::min(SV[s].y, SVt[s].y) - ht, std::min(SV[s].z, SVt[s].z) - ht};
            V3 mxc{std::max(SV[s].x, SVt[s].x) + ht, std::max(SV[s].y, SVt[s].y) + ht, std::max(SV[s].z, SVt[s].z) + ht};
            axis_index(mnc, mnA[s].data());
            axis_index(mxc, mxA[s].data());
        }
        voxel.clear();
        occ.assign(surfTriStart, {});
        auto fill = [&](const int* mn, const int* mx, std::vector<long>& o) {
            for (int iz = mn[2]; iz <= mx[2]; ++iz)
                for (int iy = mn[1]; iy <= mx[1]; ++iy)
                    for (int ix = mn[0]; ix <= mx[0]; ++ix) o.push_back(vidx(ix, iy, iz));
        };
        for (int s = 0; s < nN; ++s) fill(mnA[s].data(), mxA[s].data(), occ[s]);
        for (int e = 0; e < nE; ++e) {
            int a = v2s[edges[2 * e]], b = v2s[edges[2 * e + 1]];
            int mn[3], mx[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(mnA[a][d], mnA[b][d]);
                mx[d] = std::max(mxA[a][d], mxA[b][d]);
            }
            fill(mn, mx, occ[e + surfEdgeStart]);
        }
        for (int i = 0; i < surfTriStart; ++i)
            for (long vx : occ[i]) voxel[vx].push_back(i);
        for (int t = 0; t < nT; ++t) {
            int a = v2s[tris[3 * t]], b = v2s[tris[3 * t + 1]], c = v2s[tris[3 * t + 2]];
            int mn[3], mx[3];
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(mnA[a][d], std::min(mnA[b][d], mnA[c][d]));
                mx[d] = std::max(mxA[a][d], std::max(mxA[b][d], mxA[c][d]));
            }
            std::vector<long> o;
            fill(mn, mx, o);
            for (long vx : o) voxel[vx].push_back(t + surfTriStart);
        }
    }
    // Query_Point_For_Primitives (triangles only) SPATIAL_HASH.h:624-647
    void ccd_point_tris(int s, std::vector<int>& out) const {
        std::set<int> st;
        for (long vx : occ[s]) {
            auto it = voxel.find(vx);
            if (it == voxel.end()) continue;
            for (int id : it->second)
                if (id >= surfTriStart) st.insert(id - surfTriStart);
        }
        out.assign(st.begin(), st.end());
    }
    // Query_Edge_For_Edges(int) SPATIAL_HASH.h:650-662
    void ccd_edge_edges(int e, std::vector<int>& out) const {
        std::set<int> st;
        for (long vx : occ[e + surfEdgeStart]) {
            auto it = voxel.find(vx);
            if (it == voxel.end()) continue;
            for (int id : it->second)
                if (id >= surfEdgeStart && id < surfTriStart && id - surfEdgeStart > e) st.insert(id - surfEdgeStart);
        }
        out.assign(st.begin(), st.end());
    }
};

inline bool aabb_far(const double* lo_a, const double* hi_a, const double* lo_b, const double* hi_b, double dist) {
    for (int d = 0; d < 3; ++d)
        if (lo_a[d] - hi_b[d] > dist || lo_b[d] - hi_a[d] > dist) return true;
    return false;
}
inline void box_of(std::initializer_list<V3> ps, double* lo, double* hi) {
    bool first = true;
    for (V3 p : ps) {
        double a[3] = {p.x, p.y, p.z};
        for (int d = 0; d < 3; ++d) {
            if (first) lo[d] = hi[d] = a[d];
            else { lo[d] = std::min(lo[d], a[d]); hi[d] = std::max(hi[d], a[d]); }
        }
        first = false;
    }
}

// ---- ACCD (Math/Distance/CCD.h:279-395); iteration cap added (flagged)
const long ACCD_MAX_ITERS = 1000000;

bool accd_pt(V3 p, V3 t0, V3 t1, V3 t2, V3 dp, V3 dt0, V3 dt1, V3 dt2, double eta, double thickness, double& toc, int* capped) {
    V3 mov = 0.25 * (((dt0 + dt1) + dt2) + dp);
    // CCD.h:291 divides by 4; multiplication by 0.25 is exact and identical
    dt0 = dt0 - mov; dt1 = dt1 - mov; dt2 = dt2 - mov; dp = dp - mov;
    double m2 = std::max(sq(dt0), std::max(sq(dt1), sq(dt2)));
    double maxDispMag = std::sqrt(sq(dp)) + std::sqrt(m2);
    if (maxDispMag == 0) return false;
    double th2 = thickness * thickness;
    double dist2_cur = d_PT_unclassified(p, t0, t1, t2);
    double dist_cur = std::sqrt(dist2_cur);
    double gap = eta * (dist2_cur - th2) / (dist_cur + thickness);
    double toc_prev = toc;
    toc = 0;
    for (long it = 0;; ++it) {
        if (it >= ACCD_MAX_ITERS) { *capped = 1; return true; }
        double tocLB = (1 - eta) * (dist2_cur - th2) / ((dist_cur + thickness) * maxDispMag);
        p = p + tocLB * dp; t0 = t0 + tocLB * dt0; t1 = t1 + tocLB * dt1; t2 = t2 + tocLB * dt2;
        dist2_cur = d_PT_unclassified(p, t0, t1, t2);
        dist_cur = std::sqrt(dist2_cur);
        if (toc != 0 && ((dist2_cur - th2) / (dist_cur + thickness) < gap)) break;
        toc += tocLB;
        if (toc > toc_prev) return false;
    }
    return true;
}

bool accd_ee(V3 ea0, V3 ea1, V3 eb0, V3 eb1, V3 dea0, V3 dea1, V3 deb0, V3 deb1, double eta, double thickness, double& toc, int* capped) {
    V3 mov = 0.25 * (((dea0 + dea1) + deb0) + deb1);
    dea0 = dea0 - mov; dea1 = dea1 - mov; deb0 = deb0 - mov; deb1 = deb1 - mov;
    double maxDispMag = std::sqrt(std::max(sq(dea0), sq(dea1))) + std::sqrt(std::max(sq(deb0), sq(deb1)));
    if (maxDispMag == 0) return false;
    double th2 = thickness * thickness;
    auto eval = [&](double& d2, double& dF) {
        d2 = d_EE_unclassified(ea0, ea1, eb0, eb1);
        dF = d2 - th2;
        if (dF <= 0) {
            d2 = std::min(std::min(sq(ea0 - eb0), sq(ea0 - eb1)), std::min(sq(ea1 - eb0), sq(ea1 - eb1)));
            dF = d2 - th2;
        }
    };
    double dist2_cur, dFunc;
    eval(dist2_cur, dFunc);
    double dist_cur = std::sqrt(dist2_cur);
    double gap = eta * dFunc / (dist_cur + thickness);
    double toc_prev = toc;
    toc = 0;
    for (long it = 0;; ++it) {
        if (it >= ACCD_MAX_ITERS) { *capped = 1; return true; }
        double tocLB = (1 - eta) * dFunc / ((dist_cur + thickness) * maxDispMag);
        ea0 = ea0 + tocLB * dea0; ea1 = ea1 + tocLB * dea1; eb0 = eb0 + tocLB * deb0; eb1 = eb1 + tocLB * deb1;
        eval(dist2_cur, dFunc);
        dist_cur = std::sqrt(dist2_cur);
        if (toc != 0 && (dFunc / (dist_cur + thickness) < gap)) break;
        toc += tocLB;
        if (toc > toc_prev) return false;
    }
    return true;
}

// constraint record -> stencil vertices and kind, following the sign
// encoding of FEM/IPC.h:202-250, 439-547, 652.
struct Stencil {
    int kind;      // 0 PP, 1 PE, 2 PT, 3 EE, 4 EE mollified, 5 PE mollified, 6 PP mollified
    int v[4];      // vertex ids in derivative order
    int nv;
    double mult;   // multiplicity (PP/PE merged)
};

Stencil decode(const int* c) {
    Stencil s{};
    s.mult = 1;
    if (c[0] >= 0) {
        if (c[3] >= 0 && c[2] >= 0) { s.kind = 3; s.v[0] = c[0]; s.v[1] = c[1]; s.v[2] = c[2]; s.v[3] = c[3]; s.nv = 4; }
        else if (c[3] >= 0) { s.kind = 4; s.v[0] = c[0]; s.v[1] = c[1]; s.v[2] = -c[2] - 1; s.v[3] = c[3]; s.nv = 4; }
        else if (c[2] >= 0) { s.kind = 5; s.v[0] = c[0]; s.v[1] = -c[3] - 1; s.v[2] = c[1]; s.v[3] = c[2]; s.nv = 4; }
        else { s.kind = 6; s.v[0] = c[0]; s.v[1] = -c[2] - 1; s.v[2] = c[1]; s.v[3] = -c[3] - 1; s.nv = 4; }
    } else {
        s.v[0] = -c[0] - 1;
        if (c[3] >= 0) { s.kind = 2; s.v[1] = c[1]; s.v[2] = c[2]; s.v[3] = c[3]; s.nv = 4; }
        else if (c[2] >= 0) { s.kind = 1; s.v[1] = c[1]; s.v[2] = c[2]; s.nv = 3; s.mult = -c[3]; }
        else { s.kind = 0; s.v[1] = c[1]; s.nv = 2; s.mult = -c[3]; }
    }
    return s;
}

// raw distance of a constraint (Compute_Min_Dist2, IPC.h:2288-2384)
double constraint_dist2(const Stencil& s, const double* X) {
    V3 a = v3(X + 3 * s.v[0]), b = v3(X + 3 * s.v[1]);
    switch (s.kind) {
        case 0: return d_PP(a, b);
        case 1: return d_PE(a, b, v3(X + 3 * s.v[2]));
        case 2: return d_PT(a, b, v3(X + 3 * s.v[2]), v3(X + 3 * s.v[3]));
        case 3: case 4: return d_EE(a, b, v3(X + 3 * s.v[2]), v3(X + 3 * s.v[3]));
        case 5: return d_PE(a, v3(X + 3 * s.v[2]), v3(X + 3 * s.v[3]));
        default: return d_PP(a, v3(X + 3 * s.v[2]));
    }
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Surface extraction: Find_Surface_TriMesh (Utils/MESHIO.h:485-544) +
// Find_Surface_Primitives_And_Compute_Area (Utils/MESHIO.h:768-834).
// Returns 0, or -1 if a capacity is too small. Outputs are in the reference's
// order: triangles in std::map<Triplet> order, edges in std::map<(i,j)> order
// with the orientation of the first triangle that adds them, nodes ascending.
// ---------------------------------------------------------------------------
int ora_surface(int V, int T, const int* tets, const double* X, int capTri, int capEdge,
                int* nTri, int* tris, int* nEdge, int* edges, int* nNode, int* nodes,
                double* BTArea, double* BEArea, double* BNArea) {
    std::map<std::array<int, 3>, int> tri2Tet;
    for (int t = 0; t < T; ++t) {
        const int* e = tets + 4 * t;
        tri2Tet[{e[0], e[2], e[1]}] = t;
        tri2Tet[{e[0], e[3], e[2]}] = t;
        tri2Tet[{e[0], e[1], e[3]}] = t;
        tri2Tet[{e[1], e[2], e[3]}] = t;
    }
    std::vector<std::array<int, 3>> Tri;
    for (auto& kv : tri2Tet) {
        const auto& k = kv.first;
        if (tri2Tet.count({k[2], k[1], k[0]}) || tri2Tet.count({k[1], k[0], k[2]}) || tri2Tet.count({k[0], k[2], k[1]})) continue;
        Tri.push_back(k);
    }
    if ((int)Tri.size() > capTri) return -1;
    std::map<std::array<int, 2>, double> edgeSet;
    std::vector<double> nodeArea(V, 0.0);
    std::vector<double> triArea;
    for (auto& t : Tri) {
        V3 v0 = v3(X + 3 * t[0]), v1 = v3(X + 3 * t[1]), v2 = v3(X + 3 * t[2]);
        double A = 0.5 * std::sqrt(sq(cross(v1 - v0, v2 - v0)));
        triArea.push_back(A);
        int pairs[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
        for (auto& pr : pairs) {
            auto it = edgeSet.find({pr[1], pr[0]});
            if (it == edgeSet.end()) edgeSet[{pr[0], pr[1]}] += A / 3;
            else it->second += A / 3;
        }
        nodeArea[t[0]] += A / 3; nodeArea[t[1]] += A / 3; nodeArea[t[2]] += A / 3;
    }
    if ((int)edgeSet.size() > capEdge) return -1;
    *nTri = (int)Tri.size();
    for (size_t i = 0; i < Tri.size(); ++i) {
        for (int d = 0; d < 3; ++d) tris[3 * i + d] = Tri[i][d];
        BTArea[i] = triArea[i] / 2;
    }
    int ne = 0;
    for (auto& kv : edgeSet) {
        edges[2 * ne] = kv.first[0]; edges[2 * ne + 1] = kv.first[1];
        BEArea[ne] = kv.second / 2;
        ++ne;
    }
    *nEdge = ne;
    int nn = 0;
    for (int v = 0; v < V; ++v)
        if (nodeArea[v] != 0) { nodes[nn] = v; BNArea[nn] = nodeArea[v]; ++nn; }
    *nNode = nn;
    return 0;
}

// Compute_Vol_And_Inv_Basis (FEM/DEFORMATION_GRADIENT.h:38-76)
void ora_tet_rest(int T, const int* tets, const double* X, double* IB, double* vol) {
    for (int t = 0; t < T; ++t) {
        const int* e = tets + 4 * t;
        double B[9];
        for (int m = 0; m < 3; ++m)
            for (int i = 0; i < 3; ++i) B[i * 3 + m] = X[3 * e[m + 1] + i] - X[3 * e[0] + i];
        double J = det3(B);
        vol[t] = J / 6.0;
        double C[9];
        cofactor3(B, C);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) IB[9 * t + i * 3 + j] = C[j * 3 + i] / J;
    }
}

// NEOHOOKEAN_FUNCTOR::Compute_Psi (Physics/NEOHOOKEAN.h:78-93) plus the
// inversion check of FEM/Shell/INC_POTENTIAL.h:98-108. Returns 1 when every
// det F > 0 (energy written), 0 otherwise.
int ora_tet_energy(int T, const int* tets, const double* X, const double* IB, const double* vol,
                   const double* lam, const double* mu, double w, double* E) {
    std::vector<double> psi(T);
    int bad = 0;
#pragma omp parallel for reduction(+ : bad)
    for (int t = 0; t < T; ++t) {
        double F[9], U[9], S[3], Vv[9];
        deformation_gradient(X, tets + 4 * t, IB + 9 * t, F);
        if (det3(F) <= 0) { bad += 1; psi[t] = 0; continue; }
        svd3(F, U, S, Vv);
        double s2 = S[0] * S[0] + S[1] * S[1] + S[2] * S[2];
        double lp = std::log(S[0] * S[1] * S[2]);
        double e = mu[t] / 2.0 * (s2 - 3) - (mu[t] - lam[t] / 2.0 * lp) * lp;  // NEOHOOKEAN.h:136-142
        psi[t] = e * w * vol[t];
    }
    if (bad) return 0;
    double s = 0;
    for (int t = 0; t < T; ++t) s += psi[t];
    *E = s;
    return 1;
}

// Compute_First_PiolaKirchoff_Stress (NEOHOOKEAN.h:100-109) scattered by
// Elem_To_Node / DF_Div_DX_Mult (FEM/ELEM_TO_NODE.h:90-120, 231-257).
void ora_tet_gradient(int V, int T, const int* tets, const double* X, const double* IB, const double* vol,
                      const double* lam, const double* mu, double w, double* g) {
    std::vector<double> ge(12 * (size_t)T);
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        double F[9], C[9];
        deformation_gradient(X, tets + 4 * t, IB + 9 * t, F);
        double J = det3(F);
        cofactor3(F, C);
        double lJ = std::log(J);
        double P[9];
        for (int k = 0; k < 9; ++k) {
            double FinvT = C[k] / J;
            P[k] = w * vol[t] * (mu[t] * (F[k] - FinvT) + lam[t] * lJ * FinvT);
        }
        const double* B = IB + 9 * t;
        double* r = ge.data() + 12 * (size_t)t;
        for (int m = 0; m < 3; ++m)
            for (int d = 0; d < 3; ++d) r[3 * (m + 1) + d] = B[m * 3 + 0] * P[d * 3 + 0] + B[m * 3 + 1] * P[d * 3 + 1] + B[m * 3 + 2] * P[d * 3 + 2];
        for (int d = 0; d < 3; ++d) r[d] = -r[3 + d] - r[6 + d] - r[9 + d];
    }
    for (int t = 0; t < T; ++t)
        for (int a = 0; a < 4; ++a)
            for (int d = 0; d < 3; ++d) g[3 * tets[4 * t + a] + d] += ge[12 * (size_t)t + 3 * a + d];
}

// Compute_First_PiolaKirchoff_Stress_Derivative (NEOHOOKEAN.h:116-133) ->
// Compute_DP_Div_DF (NEOHOOKEAN.h:191-300) -> 12x12 element Hessian
// (ELEM_TO_NODE.h:122-229 contracts dP/dF with dF/dx). Output row-major
// 12x12 per tet, vertex-major (vertex a, coord d) -> row 3a+d.
void ora_tet_hessian(int T, const int* tets, const double* X, const double* IB, const double* vol,
                     const double* lam, const double* mu, double w, int project, double* H) {
#pragma omp parallel for
    for (int t = 0; t < T; ++t) {
        double F[9], U[9], S[3], Vm[9];
        deformation_gradient(X, tets + 4 * t, IB + 9 * t, F);
        svd3(F, U, S, Vm);
        double u = mu[t], l = lam[t], ww = w * vol[t];
        double lp = std::log(S[0] * S[1] * S[2]);
        double dE[3], A[9];
        for (int i = 0; i < 3; ++i) {
            double inv = 1.0 / S[i];
            dE[i] = u * (S[i] - inv) + l * inv * lp;
        }
        for (int i = 0; i < 3; ++i) {
            double inv2 = 1.0 / S[i] / S[i];
            A[i * 3 + i] = u * (1.0 + inv2) - l * inv2 * (lp - 1.0);
        }
        A[1] = A[3] = l / S[0] / S[1];
        A[5] = A[7] = l / S[1] / S[2];
        A[2] = A[6] = l / S[2] / S[0];
        if (project) make_pd(3, A);
        double middle = u - l * lp;
        double left[3] = {(u + middle / S[0] / S[1]) / 2.0, (u + middle / S[1] / S[2]) / 2.0, (u + middle / S[2] / S[0]) / 2.0};
        double Bm[3][4];
        for (int c = 0; c < 3; ++c) {
            int cp = (c + 1) % 3;
            double right = dE[c] + dE[cp];
            double ss = S[c] + S[cp];
            const double eps = 1.0e-6;
            right /= (ss < eps) ? 2 * eps : 2 * ss;
            double b[4] = {left[c] + right, left[c] - right, left[c] - right, left[c] + right};
            if (project) make_pd(2, b);
            for (int k = 0; k < 4; ++k) Bm[c][k] = b[k];
        }
        // M in the rotated basis, index a*3+b <-> (U column a, V column b)
        double M[81] = {0};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) M[(i * 4) * 9 + j * 4] = ww * A[i * 3 + j];
        M[1 * 9 + 1] = ww * Bm[0][0]; M[1 * 9 + 3] = ww * Bm[0][1]; M[3 * 9 + 1] = ww * Bm[0][2]; M[3 * 9 + 3] = ww * Bm[0][3];
        M[5 * 9 + 5] = ww * Bm[1][0]; M[5 * 9 + 7] = ww * Bm[1][1]; M[7 * 9 + 5] = ww * Bm[1][2]; M[7 * 9 + 7] = ww * Bm[1][3];
        M[2 * 9 + 2] = ww * Bm[2][3]; M[2 * 9 + 6] = ww * Bm[2][2]; M[6 * 9 + 2] = ww * Bm[2][1]; M[6 * 9 + 6] = ww * Bm[2][0];
        // dP/dF[ij][rs] with ij = j*3+i (column-major F), NEOHOOKEAN.h:274-300
        double K[81];
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i)
                for (int s = 0; s < 3; ++s)
                    for (int r = 0; r < 3; ++r) {
                        double acc = 0;
                        for (int a = 0; a < 3; ++a)
                            for (int b = 0; b < 3; ++b)
                                for (int c = 0; c < 3; ++c)
                                    for (int d = 0; d < 3; ++d) {
                                        double m = M[(a * 3 + b) * 9 + c * 3 + d];
                                        if (m == 0) continue;
                                        acc += m * U[i * 3 + a] * Vm[j * 3 + b] * U[r * 3 + c] * Vm[s * 3 + d];
                                    }
                        K[(j * 3 + i) * 9 + s * 3 + r] = acc;
                    }
        // dF(i,j)/dx(vertex m+1, d) = delta_id IB(m, j); vertex 0 = -sum
        const double* B = IB + 9 * t;
        double G[9][12];  // G[ij][3a+d]
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) {
                double* row = G[j * 3 + i];
                for (int k = 0; k < 12; ++k) row[k] = 0;
                double sum = 0;
                for (int m = 0; m < 3; ++m) {
                    row[3 * (m + 1) + i] = B[m * 3 + j];
                    sum += B[m * 3 + j];
                }
                row[i] = -sum;
            }
        double* He = H + 144 * (size_t)t;
        for (int p = 0; p < 12; ++p)
            for (int q = 0; q < 12; ++q) {
                double acc = 0;
                for (int x = 0; x < 9; ++x) {
                    if (G[x][p] == 0) continue;
                    for (int y = 0; y < 9; ++y) acc += G[x][p] * K[x * 9 + y] * G[y][q];
                }
                He[p * 12 + q] = acc;
            }
    }
}

// ---------------------------------------------------------------------------
// Compute_Constraint_Set, 3D branch (FEM/IPC.h:143-661), for tet surfaces
// (no rods, particles or stitch exclusions). dbc[v] != 0 marks Dirichlet
// nodes. Writes up to cap constraints (int4) and stencil info (weight,
// inflated dHat2); returns the count, or -(count) if cap was too small.
// ---------------------------------------------------------------------------
int ora_constraint_set(int V, const double* X, const double* X0, int nN, const int* nodes, int nE, const int* edges,
                       int nT, const int* tris, const unsigned char* dbc, double dHat2, double thickness, int cap,
                       int* cons, double* info) {
    SpatialHash sh;
    sh.build_ccs(V, X, nN, nodes, nE, edges, nT, tris);
    double dHat = std::sqrt(dHat2) + thickness;
    double dHat2i = dHat * dHat;
    typedef std::array<int, 4> C4;
    std::vector<std::vector<C4>> csPT(nN), csEE(nE);
#pragma omp parallel for schedule(dynamic, 64)
    for (int s = 0; s < nN; ++s) {
        int vI = nodes[s];
        V3 p = v3(X + 3 * vI);
        std::vector<int> cand;
        sh.query_point_tris(p, dHat, cand);
        for (int f : cand) {
            const int* t = tris + 3 * f;
            if (vI == t[0] || vI == t[1] || vI == t[2]) continue;
            if (dbc[vI] && dbc[t[0]] && dbc[t[1]] && dbc[t[2]]) continue;
            V3 t0 = v3(X + 3 * t[0]), t1 = v3(X + 3 * t[1]), t2 = v3(X + 3 * t[2]);
            double plo[3] = {p.x, p.y, p.z}, tlo[3], thi[3];
            box_of({t0, t1, t2}, tlo, thi);
            if (aabb_far(plo, plo, tlo, thi, dHat)) continue;  // CCD.h:149-165
            double d;
            C4 c;
            switch (type_PT(p, t0, t1, t2)) {
                case 0: d = d_PP(p, t0); c = {-vI - 1, t[0], -1, -1}; break;
                case 1: d = d_PP(p, t1); c = {-vI - 1, t[1], -1, -1}; break;
                case 2: d = d_PP(p, t2); c = {-vI - 1, t[2], -1, -1}; break;
                case 3: d = d_PE(p, t0, t1); c = {-vI - 1, t[0], t[1], -1}; break;
                case 4: d = d_PE(p, t1, t2); c = {-vI - 1, t[1], t[2], -1}; break;
                case 5: d = d_PE(p, t2, t0); c = {-vI - 1, t[2], t[0], -1}; break;
                default: d = d_PT(p, t0, t1, t2); c = {-vI - 1, t[0], t[1], t[2]}; break;
            }
            if (d < dHat2i) csPT[s].push_back(c);
        }
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int eI = 0; eI < nE; ++eI) {
        const int* mi = edges + 2 * eI;
        V3 ea0 = v3(X + 3 * mi[0]), ea1 = v3(X + 3 * mi[1]);
        std::vector<int> cand;
        sh.query_edge_edges(ea0, ea1, dHat, eI, cand);
        for (int eJ : cand) {
            const int* mj = edges + 2 * eJ;
            if (mi[0] == mj[0] || mi[0] == mj[1] || mi[1] == mj[0] || mi[1] == mj[1] || eI > eJ) continue;
            if (dbc[mi[0]] && dbc[mi[1]] && dbc[mj[0]] && dbc[mj[1]]) continue;
            V3 eb0 = v3(X + 3 * mj[0]), eb1 = v3(X + 3 * mj[1]);
            double alo[3], ahi[3], blo[3], bhi[3];
            box_of({ea0, ea1}, alo, ahi);
            box_of({eb0, eb1}, blo, bhi);
            if (aabb_far(alo, ahi, blo, bhi, dHat)) continue;  // CCD.h:167-185
            double cn = ee_cross_norm2(ea0, ea1, eb0, eb1);
            double eps_x = ee_mollifier_threshold(v3(X0 + 3 * mi[0]), v3(X0 + 3 * mi[1]), v3(X0 + 3 * mj[0]), v3(X0 + 3 * mj[1]));
            bool mol = cn < eps_x;
            double d;
            C4 c;
            int a0 = mi[0], a1 = mi[1], b0 = mj[0], b1 = mj[1];
            switch (type_EE(ea0, ea1, eb0, eb1)) {  // IPC.h:434-554
                case 0: d = d_PP(ea0, eb0); c = mol ? C4{a0, b0, -a1 - 1, -b1 - 1} : C4{-a0 - 1, b0, -1, -1}; break;
                case 1: d = d_PP(ea0, eb1); c = mol ? C4{a0, b1, -a1 - 1, -b0 - 1} : C4{-a0 - 1, b1, -1, -1}; break;
                case 2: d = d_PE(ea0, eb0, eb1); c = mol ? C4{a0, b0, b1, -a1 - 1} : C4{-a0 - 1, b0, b1, -1}; break;
                case 3: d = d_PP(ea1, eb0); c = mol ? C4{a1, b0, -a0 - 1, -b1 - 1} : C4{-a1 - 1, b0, -1, -1}; break;
                case 4: d = d_PP(ea1, eb1); c = mol ? C4{a1, b1, -a0 - 1, -b0 - 1} : C4{-a1 - 1, b1, -1, -1}; break;
                case 5: d = d_PE(ea1, eb0, eb1); c = mol ? C4{a1, b0, b1, -a0 - 1} : C4{-a1 - 1, b0, b1, -1}; break;
                case 6: d = d_PE(eb0, ea0, ea1); c = mol ? C4{b0, a0, a1, -b1 - 1} : C4{-b0 - 1, a0, a1, -1}; break;
                case 7: d = d_PE(eb1, ea0, ea1); c = mol ? C4{b1, a0, a1, -b0 - 1} : C4{-b1 - 1, a0, a1, -1}; break;
                default: d = d_EE(ea0, ea1, eb0, eb1); c = mol ? C4{a0, a1, -b0 - 1, b1} : C4{a0, a1, b0, b1}; break;
            }
            if (d < dHat2i) csEE[eI].push_back(c);
        }
    }
    // merge duplicate regular PP/PE with multiplicity (IPC.h:599-654)
    std::vector<C4> out;
    std::map<C4, int> counter;
    for (auto& v : csPT)
        for (auto& c : v) {
            if (c[3] < 0) ++counter[c];
            else out.push_back(c);
        }
    for (auto& v : csEE)
        for (auto& c : v) {
            if (c[0] < 0) ++counter[c];
            else out.push_back(c);
        }
    for (auto& kv : counter) out.push_back({kv.first[0], kv.first[1], kv.first[2], -kv.second});
    int n = (int)out.size();
    if (n > cap) return -n;
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 4; ++k) cons[4 * i + k] = out[i][k];
        info[2 * i] = 1.0;  // IPC.h:656-660: no area weighting for offset IPC
        info[2 * i + 1] = dHat2i;
    }
    return n;
}

// Compute_Barrier (FEM/IPC.h:742-941), 3D branch
double ora_barrier_energy(int C, const int* cons, const double* info, const double* X, const double* X0,
                          double dHat2, double kappa, double thickness) {
    double th2 = thickness * thickness;
    dHat2 += 2 * std::sqrt(dHat2) * thickness;
    std::vector<double> b(C);
    for (int i = 0; i < C; ++i) {
        Stencil s = decode(cons + 4 * i);
        double d = constraint_dist2(s, X) - th2;
        if (d <= 0) return NAN;
        double e = barrier(d, dHat2, kappa);
        if (s.kind >= 4) {
            double eps_x = ee_mollifier_threshold(v3(X0 + 3 * s.v[0]), v3(X0 + 3 * s.v[1]), v3(X0 + 3 * s.v[2]), v3(X0 + 3 * s.v[3]));
            e *= ee_mollifier(ee_cross_norm2(v3(X + 3 * s.v[0]), v3(X + 3 * s.v[1]), v3(X + 3 * s.v[2]), v3(X + 3 * s.v[3])), eps_x);
        }
        if (s.kind <= 1 && cons[4 * i + 3] < -1) e *= -cons[4 * i + 3];
        b[i] = e * info[2 * i];
    }
    double E = 0;
    for (int i = 0; i < C; ++i) E += b[i];
    return E;
}

// per-constraint local gradient and Hessian of the (weighted) barrier term,
// over the constraint's stencil (Compute_Barrier_Gradient IPC.h:943-1256,
// Compute_Barrier_Hessian IPC.h:1258-1731).
static void barrier_local(const Stencil& s, const double* X, const double* X0, double dHat2, double kappa, double th2,
                          double weight, double* g, double* H, int* nv) {
    V3 x[4];
    for (int k = 0; k < 4; ++k) x[k] = (k < s.nv) ? v3(X + 3 * s.v[k]) : V3{0, 0, 0};
    double d, dg[12], dH[144];
    int nd;  // distance stencil size
    if (s.kind == 0 || s.kind == 6) {
        V3 b = (s.kind == 0) ? x[1] : x[2];
        d = d_PP(x[0], b); nd = 2;
        dPP_grad_hess(x[0], b, dg, H ? dH : nullptr);
    } else if (s.kind == 1 || s.kind == 5) {
        V3 e0 = (s.kind == 1) ? x[1] : x[2], e1 = (s.kind == 1) ? x[2] : x[3];
        d = d_PE(x[0], e0, e1); nd = 3;
        dPE_grad_hess(x[0], e0, e1, dg, H ? dH : nullptr);
    } else if (s.kind == 2) {
        d = d_PT(x[0], x[1], x[2], x[3]); nd = 4;
        dPT_grad_hess(x[0], x[1], x[2], x[3], dg, H ? dH : nullptr);
    } else {
        d = d_EE(x[0], x[1], x[2], x[3]); nd = 4;
        dEE_grad_hess(x[0], x[1], x[2], x[3], dg, H ? dH : nullptr);
    }
    d -= th2;
    double bg = barrier_g(d, dHat2, kappa), bh = barrier_h(d, dHat2, kappa);
    if (s.kind <= 3) {
        double m = s.mult * weight;
        int n = 3 * s.nv;
        *nv = s.nv;
        for (int i = 0; i < n; ++i) g[i] = m * bg * dg[i];
        if (H)
            for (int i = 0; i < n; ++i)
                for (int j = 0; j < n; ++j) H[i * n + j] = m * (bh * dg[i] * dg[j] + bg * dH[i * n + j]);
        return;
    }
    // mollified: E = e(x) b(d(x)); distance stencil embedded in 12 via map
    *nv = 4;
    double bv = barrier(d, dHat2, kappa);
    double eps_x = ee_mollifier_threshold(v3(X0 + 3 * s.v[0]), v3(X0 + 3 * s.v[1]), v3(X0 + 3 * s.v[2]), v3(X0 + 3 * s.v[3]));
    double e = ee_mollifier(ee_cross_norm2(x[0], x[1], x[2], x[3]), eps_x);
    double eg[12], eH[144];
    mollifier_grad_hess(x[0], x[1], x[2], x[3], eps_x, eg, H ? eH : nullptr);
    int map[4];  // distance-stencil slot -> 12 slot (vertex index in edgeVInd)
    if (s.kind == 4) { map[0] = 0; map[1] = 1; map[2] = 2; map[3] = 3; }
    else if (s.kind == 5) { map[0] = 0; map[1] = 2; map[2] = 3; }
    else { map[0] = 0; map[1] = 2; }
    double dg12[12] = {0};
    for (int a = 0; a < nd; ++a)
        for (int k = 0; k < 3; ++k) dg12[3 * map[a] + k] = dg[3 * a + k];
    for (int i = 0; i < 12; ++i) g[i] = weight * (e * bg * dg12[i] + bv * eg[i]);
    if (!H) return;
    double dH12[144] = {0};
    for (int a = 0; a < nd; ++a)
        for (int b = 0; b < nd; ++b)
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) dH12[(3 * map[a] + k) * 12 + 3 * map[b] + l] = dH[(3 * a + k) * (3 * nd) + 3 * b + l];
    for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j)
            H[i * 12 + j] = weight * (bg * (dg12[i] * eg[j] + eg[i] * dg12[j]) + bv * eH[i * 12 + j] +
                                      e * bh * dg12[i] * dg12[j] + e * bg * dH12[i * 12 + j]);
}

void ora_barrier_gradient(int C, const int* cons, const double* info, const double* X, const double* X0,
                          double dHat2, double kappa, double thickness, double* g) {
    double th2 = thickness * thickness;
    dHat2 += 2 * std::sqrt(dHat2) * thickness;
    for (int i = 0; i < C; ++i) {
        Stencil s = decode(cons + 4 * i);
        double gl[12];
        int nv;
        barrier_local(s, X, X0, dHat2, kappa, th2, info[2 * i], gl, nullptr, &nv);
        for (int a = 0; a < nv; ++a)
            for (int k = 0; k < 3; ++k) g[3 * s.v[a] + k] += gl[3 * a + k];
    }
}

// dense local Hessians (PSD-projected when project != 0): H is C*144
// (row-major nv*3 square packed at the front), verts is C*4 (-1 unused).
void ora_barrier_hessian(int C, const int* cons, const double* info, const double* X, const double* X0,
                         double dHat2, double kappa, double thickness, int project, int* verts, double* H) {
    double th2 = thickness * thickness;
    dHat2 += 2 * std::sqrt(dHat2) * thickness;
#pragma omp parallel for
    for (int i = 0; i < C; ++i) {
        Stencil s = decode(cons + 4 * i);
        double gl[12];
        int nv;
        double* Hl = H + 144 * (size_t)i;
        barrier_local(s, X, X0, dHat2, kappa, th2, info[2 * i], gl, Hl, &nv);
        if (project) make_pd(3 * nv, Hl);
        for (int a = 0; a < 4; ++a) verts[4 * i + a] = (a < nv) ? s.v[a] : -1;
    }
}

// Compute_Min_Dist2 (FEM/IPC.h:2246-2388): raw squared distances per
// constraint and min - thickness^2.
double ora_min_dist2(int C, const int* cons, const double* X, double thickness, double* dist2) {
    double mn = INFINITY;
    for (int i = 0; i < C; ++i) {
        dist2[i] = constraint_dist2(decode(cons + 4 * i), X);
        mn = std::min(mn, dist2[i]);
    }
    return mn - thickness * thickness;
}

// Compute_Intersection_Free_StepSize, 3D tet-surface branch
// (FEM/IPC.h:1879-2244). alpha is in/out. Returns 0 ok, 1 if an ACCD loop hit
// the iteration cap (alpha still conservative), -1 on a zero step (the
// reference exits the process there, IPC.h:2014-2031).
int ora_ccd_stepsize(int nN, const int* nodes, int nE, const int* edges, int nT, const int* tris,
                     const unsigned char* dbc, const double* X, const double* dir, double thickness, double* alpha) {
    SpatialHash sh;
    double stepSize = *alpha;
    sh.build_ccd(X, nN, nodes, nE, edges, nT, tris, dir, stepSize, thickness);
    const double eta = 0.1;
    std::vector<double> aPT(nN, stepSize);
    int capped = 0, zero = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : capped, zero)
    for (int s = 0; s < nN; ++s) {
        int vI = nodes[s];
        V3 p = v3(X + 3 * vI), dp = v3(dir + 3 * vI);
        std::vector<int> cand;
        sh.ccd_point_tris(s, cand);
        for (int f : cand) {
            const int* t = tris + 3 * f;
            if (vI == t[0] || vI == t[1] || vI == t[2]) continue;
            if (dbc[vI] && dbc[t[0]] && dbc[t[1]] && dbc[t[2]]) continue;
            V3 t0 = v3(X + 3 * t[0]), t1 = v3(X + 3 * t[1]), t2 = v3(X + 3 * t[2]);
            V3 dt0 = v3(dir + 3 * t[0]), dt1 = v3(dir + 3 * t[1]), dt2 = v3(dir + 3 * t[2]);
            double plo[3], phi[3], tlo[3], thi[3];
            box_of({p, p + dp}, plo, phi);
            box_of({t0, t1, t2, t0 + dt0, t1 + dt1, t2 + dt2}, tlo, thi);
            if (aabb_far(plo, phi, tlo, thi, thickness)) continue;  // CCD.h:187-211
            double la = aPT[s];
            int cp = 0;
            if (accd_pt(p, t0, t1, t2, dp, dt0, dt1, dt2, eta, thickness, la, &cp)) {
                if (aPT[s] > la) aPT[s] = la;
            }
            capped |= cp;
            if (la == 0) zero = 1;
        }
    }
    if (zero) return -1;
    for (double a : aPT) stepSize = std::min(stepSize, a);
    std::vector<double> aEE(nE, stepSize);
#pragma omp parallel for schedule(dynamic, 64) reduction(| : capped, zero)
    for (int eI = 0; eI < nE; ++eI) {
        const int* mi = edges + 2 * eI;
        V3 ea0 = v3(X + 3 * mi[0]), ea1 = v3(X + 3 * mi[1]);
        V3 dea0 = v3(dir + 3 * mi[0]), dea1 = v3(dir + 3 * mi[1]);
        std::vector<int> cand;
        sh.ccd_edge_edges(eI, cand);
        for (int eJ : cand) {
            const int* mj = edges + 2 * eJ;
            if (mi[0] == mj[0] || mi[0] == mj[1] || mi[1] == mj[0] || mi[1] == mj[1] || eI > eJ) continue;
            if (dbc[mi[0]] && dbc[mi[1]] && dbc[mj[0]] && dbc[mj[1]]) continue;
            V3 eb0 = v3(X + 3 * mj[0]), eb1 = v3(X + 3 * mj[1]);
            V3 deb0 = v3(dir + 3 * mj[0]), deb1 = v3(dir + 3 * mj[1]);
            double alo[3], ahi[3], blo[3], bhi[3];
            box_of({ea0, ea1, ea0 + dea0, ea1 + dea1}, alo, ahi);
            box_of({eb0, eb1, eb0 + deb0, eb1 + deb1}, blo, bhi);
            if (aabb_far(alo, ahi, blo, bhi, thickness)) continue;  // CCD.h:213-235
            double la = aEE[eI];
            int cp = 0;
            if (accd_ee(ea0, ea1, eb0, eb1, dea0, dea1, deb0, deb1, eta, thickness, la, &cp)) {
                if (aEE[eI] > la) aEE[eI] = la;
            }
            capped |= cp;
        }
    }
    for (double a : aEE) stepSize = std::min(stepSize, a);
    *alpha = stepSize;
    return capped ? 1 : 0;
}

// Initialize_EIPC<T, false> as called by Initialize_OIPC
// (FEM/Shell/DISCRETE_SHELL.h:555-577): kappa from the mean of diag(M).
double ora_kappa_init(double meanMassDiag, double dHat2, double stiffMult, double* kappaMax) {
    double H_b = barrier_h(1.0e-16, dHat2, 1.0);
    double k = stiffMult * 1.0e11 * meanMassDiag * 3 / (4.0e-16 * H_b);
    *kappaMax = 100 * k;
    return k;
}

// raw distance-function access for known-answer and FD tests
int ora_type_pt(const double* p, const double* t0, const double* t1, const double* t2) { return type_PT(v3(p), v3(t0), v3(t1), v3(t2)); }
// extend-add of a multifrontal update matrix into its parent front, lower
// triangle only. The front (order m = k + r) is held as three column-major
// blocks F11 (k x k), F21 (r x k), F22 (r x r); U (mu x mu, column-major)
// goes to the front positions li (ascending): F[li[i], li[j]] += U[i, j] for
// i >= j. Used by the oracle's sparse Cholesky (oracle/cholesky.py).
void ora_extend_add(double* F11, double* F21, double* F22, long k, long r, const double* U, long mu, const long* li) {
    for (long j = 0; j < mu; ++j) {
        const long c = li[j];
        const double* Uc = U + j * mu;
        if (c < k) {
            long i = j;
            for (; i < mu && li[i] < k; ++i) F11[c * k + li[i]] += Uc[i];
            for (; i < mu; ++i) F21[c * r + (li[i] - k)] += Uc[i];
        } else {
            double* Fc = F22 + (c - k) * r - k;
            for (long i = j; i < mu; ++i) Fc[li[i]] += Uc[i];
        }
    }
}

// the classifier's three (s, t) edge parameters (DISTANCE_TYPE.h:46,54,62),
// all computed, for tests of the 2x2 LDLT solve
void ora_pt_params(const double* p, const double* t0, const double* t1, const double* t2, double* st) {
    V3 P = v3(p), A = v3(t0), B = v3(t1), Cc = v3(t2);
    V3 n = cross(B - A, Cc - A);
    pt_param(B - A, n, P, A, st[0], st[1]);
    pt_param(Cc - B, n, P, B, st[2], st[3]);
    pt_param(A - Cc, n, P, Cc, st[4], st[5]);
}
int ora_type_ee(const double* a0, const double* a1, const double* b0, const double* b1) { return type_EE(v3(a0), v3(a1), v3(b0), v3(b1)); }
double ora_dist_pt_unclassified(const double* p, const double* t0, const double* t1, const double* t2) { return d_PT_unclassified(v3(p), v3(t0), v3(t1), v3(t2)); }
double ora_dist_ee_unclassified(const double* a0, const double* a1, const double* b0, const double* b1) { return d_EE_unclassified(v3(a0), v3(a1), v3(b0), v3(b1)); }
void ora_dist_derivs(int kind, const double* x, double* d, double* g, double* H) {
    V3 a = v3(x), b = v3(x + 3), c = v3(x + 6), e = v3(x + 9);
    switch (kind) {
        case 0: *d = d_PP(a, b); dPP_grad_hess(a, b, g, H); break;
        case 1: *d = d_PE(a, b, c); dPE_grad_hess(a, b, c, g, H); break;
        case 2: *d = d_PT(a, b, c, e); dPT_grad_hess(a, b, c, e, g, H); break;
        case 3: *d = d_EE(a, b, c, e); dEE_grad_hess(a, b, c, e, g, H); break;
        default: *d = ee_cross_norm2(a, b, c, e); eecn2_grad_hess(a, b, c, e, g, H); break;
    }
}
void ora_make_pd(int n, double* A) { make_pd(n, A); }

// ---------------------------------------------------------------------------
// Discrete-shell elasticity of the Hinge path (oracle/shell.hpp)
// ---------------------------------------------------------------------------

// rest data of every face: inverse of the rest first fundamental form, its
// determinant, vol = area * thickness, lambda = E nu / (1 - nu^2),
// mu = E / (2 (1 + nu)) (DISCRETE_SHELL.h:132-170, 328-342); 7 doubles per face
void ora_membrane_rest(int F, const int* faces, const double* X0, double thickness, double E, double nu,
                       double* mem) {
    const double lam = E * nu / (1.0 - nu * nu), mu = E / (2.0 * (1.0 + nu));
    for (int f = 0; f < F; ++f) {
        const V3 x1 = v3(X0 + 3 * faces[3 * f]), x2 = v3(X0 + 3 * faces[3 * f + 1]), x3 = v3(X0 + 3 * faces[3 * f + 2]);
        const V3 e01 = x2 - x1, e02 = x3 - x1;
        const double a00 = sq(e01), a01 = dot(e01, e02), a11 = sq(e02);
        const double det = a00 * a11 - a01 * a01;
        double* m = mem + 7 * f;
        m[0] = a11 / det;
        m[1] = -a01 / det;
        m[2] = a00 / det;
        m[3] = m[0] * m[2] - m[1] * m[1];
        m[4] = std::sqrt(sq(cross(e01, e02))) / 2 * thickness;
        m[5] = lam;
        m[6] = mu;
    }
}

static MemFace mem_at(const double* m) { return MemFace{m[0], m[1], m[2], m[3], m[4], m[5], m[6]}; }

// membrane energy of every face (summed in face order); gradient added into
// g (3V, may be null); element Hessians H (F x 81, may be null), projected
// to PSD when project (MEMBRANE.h:125-322); faces whose three vertices are
// all fixed (dbc, may be null) are skipped, as in the reference
double ora_membrane(int F, const int* faces, const double* X, const double* mem, double w, double* g, double* H,
                    int project, const unsigned char* dbc) {
    double E = 0;
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        if (dbc && dbc[t[0]] && dbc[t[1]] && dbc[t[2]]) {  // all-DBC faces are skipped (MEMBRANE.h:25)
            if (H)
                for (int i = 0; i < 81; ++i) H[81L * f + i] = 0.0;
            continue;
        }
        double ge[9];
        E += membrane_face(v3(X + 3 * t[0]), v3(X + 3 * t[1]), v3(X + 3 * t[2]), mem_at(mem + 7 * f), w,
                           g ? ge : nullptr, H ? H + 81L * f : nullptr);
        if (g)
            for (int a = 0; a < 3; ++a)
                for (int d = 0; d < 3; ++d) g[3 * t[a] + d] += ge[3 * a + d];
        if (H && project) make_pd(9, H + 81L * f);
    }
    return E;
}

// hinge stencils (x0, x1, x2, x3) of the surface edges in their order and
// (thetabar, ebar, hbar) at X0 (DISCRETE_SHELL.h:172-212): for edge (a, b),
// x0 follows b in the face holding the directed edge a->b, x1 = a, x2 = b,
// x3 follows a in the face holding b->a; boundary edges have no hinge.
int ora_shell_hinges(int V, int F, const int* faces, const double* X0, int nE, const int* edges, int* hinges,
                     double* info) {
    (void)V;
    std::map<std::pair<int, int>, int> e2t;
    for (int f = 0; f < F; ++f)
        for (int k = 0; k < 3; ++k) e2t[{faces[3 * f + k], faces[3 * f + (k + 1) % 3]}] = f;
    int n = 0;
    for (int e = 0; e < nE; ++e) {
        const int a = edges[2 * e], b = edges[2 * e + 1];
        auto it = e2t.find({a, b});
        if (it == e2t.end()) continue;
        const int* t = faces + 3 * it->second;
        int v0 = -1;
        for (int j = 0; j < 3; ++j)
            if (t[j] == b) v0 = t[(j + 1) % 3];
        auto jt = e2t.find({b, a});
        if (jt == e2t.end()) continue;
        const int* o = faces + 3 * jt->second;
        int v3i = 0;
        for (int j = 0; j < 3; ++j)
            if (o[j] == a) v3i = o[(j + 1) % 3];
        int* hh = hinges + 4 * n;
        hh[0] = v0; hh[1] = a; hh[2] = b; hh[3] = v3i;
        const V3 X0_ = v3(X0 + 3 * v0), X1 = v3(X0 + 3 * a), X2 = v3(X0 + 3 * b), X3 = v3(X0 + 3 * v3i);
        double* in = info + 3 * n;
        in[0] = dihedral_angle(X0_, X1, X2, X3);
        in[1] = std::sqrt(sq(X1 - X2));
        const V3 n1 = cross(X1 - X0_, X2 - X0_), n2 = cross(X2 - X3, X1 - X3);
        in[2] = (std::sqrt(sq(n1)) + std::sqrt(sq(n2))) / (in[1] * 6);
        ++n;
    }
    return n;
}

// bending energy of every hinge (hinge order); gradient into g (may be null);
// element Hessians H (Hn x 144, may be null), projected when project
double ora_bending(int Hn, const int* hinges, const double* info, double k, const double* X, double w, double* g,
                   double* H, int project, const unsigned char* dbc) {
    double E = 0;
    for (int i = 0; i < Hn; ++i) {
        const int* hh = hinges + 4 * i;
        if (dbc && dbc[hh[0]] && dbc[hh[1]] && dbc[hh[2]] && dbc[hh[3]]) {  // BENDING.h:56-60
            if (H)
                for (int q = 0; q < 144; ++q) H[144L * i + q] = 0.0;
            continue;
        }
        const double* in = info + 3 * i;
        double ge[12];
        E += bending_hinge(v3(X + 3 * hh[0]), v3(X + 3 * hh[1]), v3(X + 3 * hh[2]), v3(X + 3 * hh[3]), in[0], in[1],
                           in[2], k, w, g ? ge : nullptr, H ? H + 144L * i : nullptr);
        if (g)
            for (int a = 0; a < 4; ++a)
                for (int d = 0; d < 3; ++d) g[3 * hh[a] + d] += ge[3 * a + d];
        if (H && project) make_pd(12, H + 144L * i);
    }
    return E;
}

double ora_dihedral(const double* x, double* g, double* H) {
    const V3 a = v3(x), b = v3(x + 3), c = v3(x + 6), d = v3(x + 9);
    dihedral_derivs(a, b, c, d, g, H);
    return dihedral_angle(a, b, c, d);
}

// Normal-flow predictor shift (Update_Normal_Flow_Neumann,
// FEM/Shell/DISCRETE_SHELL.h:359-395): b_v += cross(X2-X1, X3-X1) over the
// surface triangles in order, then normalised; the shift `step` along b_v is
// returned as a velocity over h. Vertices on no triangle get zero.
void ora_normal_flow(int V, int nT, const int* tris, const double* X, double step, double h, double* vel) {
    std::vector<double> b(3 * (size_t)V, 0.0);
    std::vector<int> deg(V, 0);
    for (int f = 0; f < nT; ++f) {
        const int a = tris[3 * f], c1 = tris[3 * f + 1], c2 = tris[3 * f + 2];
        const double e1[3] = {X[3 * c1] - X[3 * a], X[3 * c1 + 1] - X[3 * a + 1], X[3 * c1 + 2] - X[3 * a + 2]};
        const double e2[3] = {X[3 * c2] - X[3 * a], X[3 * c2 + 1] - X[3 * a + 1], X[3 * c2 + 2] - X[3 * a + 2]};
        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        for (int k = 0; k < 3; ++k) {
            const int v = tris[3 * f + k];
            deg[v]++;
            for (int d = 0; d < 3; ++d) b[3 * v + d] += n[d];
        }
    }
    for (int v = 0; v < V; ++v) {
        const double sq = b[3 * v] * b[3 * v] + b[3 * v + 1] * b[3 * v + 1] + b[3 * v + 2] * b[3 * v + 2];
        const double w = (deg[v] > 0 && sq > 0) ? step / std::sqrt(sq) : 0.0;
        for (int d = 0; d < 3; ++d) vel[3 * v + d] = w * b[3 * v + d] / h;
    }
}

// ---------------------------------------------------------------------------
// Intersection check: Check_Edge_Tri_Intersect (FEM/IPC.h:2444-2517) with
// segTriIntersect (FEM/IPC.h:2390-2442). The reference decides the plane side
// with orient3d under USE_PREDICATES and the crossing point with an LU solve;
// this restatement decides both with exact orientation signs: the segment
// must cross the plane strictly, and the line through it must pass no
// triangle edge on the outside (no two strictly opposite edge orientations).
// Every triangle is tested against every edge whose AABB overlaps its own
// (the reference's spatial hash only prunes pairs that cannot intersect),
// after the reference's exclusions: shared vertex, all five vertices DBC.
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

// exact sign of det[a-d; b-d; c-d]: each difference is split exactly into two
// doubles (two-difference), the determinant's six signed triple products of
// differences expand into 48 triple products of doubles, each of which is
// split exactly into four doubles (fused multiply-add products), and the 192
// terms are summed into a nonoverlapping expansion whose largest component
// carries the sign (Shewchuk's grow-expansion, Discrete Comput. Geom. 18, 1997)
void xsum(double a, double b, double& x, double& y) {
    x = a + b;
    double bv = x - a, av = x - bv;
    y = (a - av) + (b - bv);
}

void xgrow(std::vector<double>& e, double b) {
    double q = b;
    size_t m = 0;
    for (size_t i = 0; i < e.size(); ++i) {
        double hh;
        xsum(q, e[i], q, hh);
        if (hh != 0.0) e[m++] = hh;
    }
    e.resize(m);
    if (q != 0.0) e.push_back(q);
}

int exact_orient3d(const double* a, const double* b, const double* c, const double* d) {
    double D[3][3][2];  // D[row][axis] = (hi, lo) of (p - d)
    const double* P[3] = {a, b, c};
    for (int r = 0; r < 3; ++r)
        for (int k = 0; k < 3; ++k) {
            double x = P[r][k] - d[k];
            double bv = P[r][k] - x, av = x + bv;
            D[r][k][0] = x;
            D[r][k][1] = (P[r][k] - av) + (bv - d[k]);
        }
    static const int perm[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
    static const double sgn[6] = {1, 1, 1, -1, -1, -1};
    std::vector<double> e;
    e.reserve(200);
    for (int p = 0; p < 6; ++p)
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const double u = D[0][perm[p][0]][i], v = D[1][perm[p][1]][j], w = D[2][perm[p][2]][k];
                    const double x = u * v, y = std::fma(u, v, -x);
                    const double x1 = x * w, y1 = std::fma(x, w, -x1);
                    const double x2 = y * w, y2 = std::fma(y, w, -x2);
                    xgrow(e, sgn[p] * y2);
                    xgrow(e, sgn[p] * x2);
                    xgrow(e, sgn[p] * y1);
                    xgrow(e, sgn[p] * x1);
                }
    if (e.empty()) return 0;
    return e.back() > 0 ? 1 : -1;
}

bool seg_tri_exact(const double* e0, const double* e1, const double* t0, const double* t1, const double* t2) {
    int o0 = exact_orient3d(t0, t1, t2, e0), o1 = exact_orient3d(t0, t1, t2, e1);
    if (o0 == 0 || o1 == 0 || o0 == o1) return false;
    int s[3] = {exact_orient3d(e0, e1, t0, t1), exact_orient3d(e0, e1, t1, t2), exact_orient3d(e0, e1, t2, t0)};
    bool pos = false, neg = false;
    for (int k = 0; k < 3; ++k) {
        pos |= s[k] > 0;
        neg |= s[k] < 0;
    }
    return !(pos && neg);
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Triangle shells in flow mode (Advance_One_Step_IE_Flow,
// FEM/Shell/DISCRETE_SHELL.h:1113).
// ---------------------------------------------------------------------------

// Initialize_Discrete_Shell (FEM/Shell/DISCRETE_SHELL.h:238-333): faces whose
// first fundamental form is singular are dropped (keep[f] = 0); lumped mass
// area * thickness * rho / 3 per corner; element volume area * thickness.
// Returns the number of faces kept.
int ora_shell_init(int V, int F, const int* faces, const double* X, double rho, double thickness,
                   unsigned char* keep, double* mass, double* vol) {
    for (int v = 0; v < V; ++v) mass[v] = 0.0;
    int kept = 0;
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        double e1[3], e2[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = X[3 * t[1] + d] - X[3 * t[0] + d];
            e2[d] = X[3 * t[2] + d] - X[3 * t[0] + d];
        }
        const double a = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
        const double b = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
        const double c = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
        keep[f] = (a * c - b * b) != 0.0;
        vol[f] = 0.0;
        if (!keep[f]) continue;
        ++kept;
        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) / 2;
        const double mp = area * thickness * rho / 3;
        for (int k = 0; k < 3; ++k) mass[t[k]] += mp;
        vol[f] = area * thickness;
    }
    return kept;
}

// Find_Surface_Primitives (Utils/MESHIO.h:728-766): every face is a surface
// triangle (in order); an edge is kept in its first orientation unless its
// reverse is already in the set; edges in set order (lexicographic); nodes
// every referenced vertex, ascending. Returns 0, or -1 if a capacity is short.
int ora_shell_surface(int V, int F, const int* faces, int capEdge, int* edges, int* nEdge, int* nodes, int* nNode) {
    std::set<std::pair<int, int>> es;
    std::vector<char> used(V, 0);
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        const int p[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
        for (auto& e : p)
            if (!es.count({e[1], e[0]})) es.insert({e[0], e[1]});
        used[t[0]] = used[t[1]] = used[t[2]] = 1;
    }
    if ((int)es.size() > capEdge) return -1;
    int k = 0;
    for (auto& e : es) {
        edges[2 * k] = e.first;
        edges[2 * k + 1] = e.second;
        ++k;
    }
    *nEdge = k;
    int m = 0;
    for (int v = 0; v < V; ++v)
        if (used[v]) nodes[m++] = v;
    *nNode = m;
    return 0;
}

// Lx of the flow energy (FEM/Shell/INC_POTENTIAL.h:53-66): per face, vertex i
// gains vol/6 (x_{i+1} + x_{i+2} - 2 x_i)
static void flow_Lx(int V, int F, const int* faces, const double* vol, const double* X, std::vector<double>& Lx) {
    Lx.assign(3 * (size_t)V, 0.0);
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d)
                Lx[3 * t[i] + d] += vol[f] / 6 * (X[3 * t[(i + 1) % 3] + d] + X[3 * t[(i + 2) % 3] + d] - 2 * X[3 * t[i] + d]);
    }
}

// flow energy -h/2 x^T L x (INC_POTENTIAL.h:53-73)
double ora_flow_energy(int V, int F, const int* faces, const double* vol, const double* X, double h) {
    std::vector<double> Lx;
    flow_Lx(V, F, faces, vol, X, Lx);
    double e = 0;
    for (int v = 0; v < V; ++v)
        for (int d = 0; d < 3; ++d) e += -h * 0.5 * X[3 * v + d] * Lx[3 * v + d];
    return e;
}

// flow gradient -h L x (INC_POTENTIAL.h:191-211), added to g
void ora_flow_gradient(int V, int F, const int* faces, const double* vol, const double* X, double h, double* g) {
    std::vector<double> Lx;
    flow_Lx(V, F, faces, vol, X, Lx);
    for (size_t k = 0; k < Lx.size(); ++k) g[k] += -h * Lx[k];
}

// flow Hessian triplets (INC_POTENTIAL.h:323-339): 27 per face (rows, cols, vals)
void ora_flow_hessian(int F, const int* faces, const double* vol, double h, int* rows, int* cols, double* vals) {
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        for (int i = 0; i < 3; ++i)
            for (int d = 0; d < 3; ++d) {
                const long b = (long)f * 27 + i * 9 + d * 3;
                rows[b] = rows[b + 1] = rows[b + 2] = 3 * t[i] + d;
                cols[b] = 3 * t[(i + 1) % 3] + d;
                cols[b + 1] = 3 * t[(i + 2) % 3] + d;
                cols[b + 2] = 3 * t[i] + d;
                vals[b] = -h * vol[f] / 6;
                vals[b + 1] = -h * vol[f] / 6;
                vals[b + 2] = 2 * h * vol[f] / 6;
            }
    }
}

int ora_orient3d(const double* a, const double* b, const double* c, const double* d) {
    return exact_orient3d(a, b, c, d);
}

// Writes up to cap (triangle, edge) pairs, sorted; returns their number.
long ora_edge_tri_intersections(int nT, const int* tris, int nE, const int* edges, const double* X,
                                const unsigned char* dbc, long cap, int* pairs) {
    std::vector<double> emin(3 * (size_t)nE), emax(3 * (size_t)nE);
    for (int e = 0; e < nE; ++e)
        for (int k = 0; k < 3; ++k) {
            emin[3 * e + k] = std::min(X[3 * edges[2 * e] + k], X[3 * edges[2 * e + 1] + k]);
            emax[3 * e + k] = std::max(X[3 * edges[2 * e] + k], X[3 * edges[2 * e + 1] + k]);
        }
    std::vector<std::vector<int>> hit(nT);
#pragma omp parallel for schedule(dynamic, 16)
    for (int f = 0; f < nT; ++f) {
        const int* t = tris + 3 * f;
        double tmin[3], tmax[3];
        for (int k = 0; k < 3; ++k) {
            tmin[k] = std::min(std::min(X[3 * t[0] + k], X[3 * t[1] + k]), X[3 * t[2] + k]);
            tmax[k] = std::max(std::max(X[3 * t[0] + k], X[3 * t[1] + k]), X[3 * t[2] + k]);
        }
        for (int e = 0; e < nE; ++e) {
            const int a = edges[2 * e], b = edges[2 * e + 1];
            if (a == t[0] || a == t[1] || a == t[2] || b == t[0] || b == t[1] || b == t[2]) continue;
            if (dbc[a] && dbc[b] && dbc[t[0]] && dbc[t[1]] && dbc[t[2]]) continue;
            bool sep = false;
            for (int k = 0; k < 3; ++k) sep |= emax[3 * e + k] < tmin[k] || emin[3 * e + k] > tmax[k];
            if (sep) continue;
            if (seg_tri_exact(X + 3 * a, X + 3 * b, X + 3 * t[0], X + 3 * t[1], X + 3 * t[2])) hit[f].push_back(e);
        }
    }
    long n = 0;
    for (int f = 0; f < nT; ++f)
        for (int e : hit[f]) {
            if (n < cap) {
                pairs[2 * n] = f;
                pairs[2 * n + 1] = e;
            }
            ++n;
        }
    return n;
}

}  // extern "C"
