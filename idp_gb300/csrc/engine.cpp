// Host side of the engine: context, instance upload, static structures
// (surface primitives in the reference's order, BSR pattern, chunk tables)
// and the batched Newton driver that restates
// Advance_One_Step_IE_Discrete_Shell (FEM/Shell/IMPLICIT_EULER.h:151-891) and
// Line_Search (IMPLICIT_EULER.h:9-149) for tet meshes with offset IPC, and its
// flow-mode variant for triangle shells (Advance_One_Step_IE_Flow).
//
// Every instance of a context runs its own Newton iteration; the kernels of
// one Newton iteration serve all instances that are still iterating, and an
// instance that converges drops out of the launches. Per-instance sums are
// taken in a fixed order, so an instance's trajectory does not depend on the
// other instances of the batch.
#include <algorithm>
#include <array>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <numeric>
#include <set>
#include <thread>
#include <vector>
#include "engine.hpp"

using namespace idp;

thread_local long long idp::g_launch_count = 0;

int DBuf::ensure(size_t n) {
    if (n <= bytes && p) return 0;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    size_t want = n < 256 ? 256 : n + n / 4;
    if (cudaMalloc(&p, want) != cudaSuccess) {
        p = nullptr;
        return 1;
    }
    bytes = want;
    return 0;
}
void DBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

struct idp_ctx {
    idp_params P;
    cudaStream_t s = nullptr;
    std::vector<HostInstance> inst;
    std::vector<InstState> st;
    Arena A;
    Work W;
    std::vector<DBuf> owned;  // arena storage (reused in order by the next commit after idp_reset)
    size_t owned_next = 0;
    bool committed = false;
    ContactSet cs;
    long prevC = 0;
    DBuf inst_buf;            // per-instance device scalars
    DBuf vel;                 // velocities (3V)
    DBuf snap;                // saved X and v (6V)
    std::vector<double> snap_kappa;
    bool has_snap = false;
    DBuf stage;               // 3V doubles in the caller's vertex order (transfers across the interface)
    DBuf bacc;                // body-force accelerations M^-1 b (3V), when some instance has one
    bool has_bacc = false;
    bool stepping = false;    // a step is in flight (begun, instances still iterating)
    // side stream: the CCD voxel size of an iteration's positions, computed
    // while the gradient and Hessian of the same positions are
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_x = nullptr, ev_vox = nullptr;
    std::chrono::steady_clock::time_point t_begin;  // the step's begin (latency origin)
};

namespace {

template <class T>
int upload(idp_ctx* c, T*& dst, const std::vector<T>& src) {
    if (c->owned_next == c->owned.size()) c->owned.emplace_back();
    DBuf& b = c->owned[c->owned_next++];
    if (b.ensure(sizeof(T) * (src.size() + 1))) return IDP_ERR_CUDA;
    dst = b.as<T>();
    if (!src.empty() && cudaMemcpy(dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return IDP_ERR_CUDA;
    return IDP_OK;
}

// Surface of a tet mesh in the reference's order: Find_Surface_TriMesh
// (Utils/MESHIO.h:485-544) keeps faces whose opposite-orientation twin is
// absent, ordered lexicographically by their oriented vertex triple;
// Find_Surface_Primitives_And_Compute_Area (MESHIO.h:768-834) takes every edge
// in the orientation of the first triangle that contains it, ordered
// lexicographically, and the surface nodes ascending.
void extract_surface(int V, const std::vector<int>& tets, std::vector<int>& tris, std::vector<int>& edges,
                     std::vector<int>& nodes) {
    long T = (long)tets.size() / 4;
    struct Face {
        int k[3];
        int s[3];
    };
    std::vector<Face> faces;
    faces.reserve(4 * T);
    for (long t = 0; t < T; ++t) {
        const int* e = &tets[4 * t];
        int f[4][3] = {{e[0], e[2], e[1]}, {e[0], e[3], e[2]}, {e[0], e[1], e[3]}, {e[1], e[2], e[3]}};
        for (auto& q : f) {
            Face F;
            for (int d = 0; d < 3; ++d) F.k[d] = F.s[d] = q[d];
            std::sort(F.s, F.s + 3);
            faces.push_back(F);
        }
    }
    // parity of an oriented triple relative to its sorted order
    auto parity = [](const int* k) {
        int inv = (k[0] > k[1]) + (k[0] > k[2]) + (k[1] > k[2]);
        return inv & 1;
    };
    std::vector<long> order(faces.size());
    if (V <= (1 << 21)) {
        // the sorted triple packed in 63 bits, ties by face index
        std::vector<std::pair<uint64_t, long>> key(faces.size());
        for (size_t i = 0; i < faces.size(); ++i)
            key[i] = {((uint64_t)faces[i].s[0] << 42) | ((uint64_t)faces[i].s[1] << 21) | (uint64_t)faces[i].s[2],
                      (long)i};
        std::sort(key.begin(), key.end());
        for (size_t i = 0; i < faces.size(); ++i) order[i] = key[i].second;
    } else {
        std::iota(order.begin(), order.end(), 0);
        std::sort(order.begin(), order.end(), [&](long a, long b) {
            const Face &A = faces[a], &B = faces[b];
            for (int d = 0; d < 3; ++d)
                if (A.s[d] != B.s[d]) return A.s[d] < B.s[d];
            return a < b;
        });
    }
    std::vector<std::array<int, 3>> bnd;
    for (size_t i = 0; i < order.size();) {
        size_t j = i;
        while (j < order.size() && std::equal(faces[order[j]].s, faces[order[j]].s + 3, faces[order[i]].s)) ++j;
        // a face is interior iff some face of the group has the opposite parity
        for (size_t a = i; a < j; ++a) {
            int pa = parity(faces[order[a]].k);
            bool twin = false;
            for (size_t b = i; b < j; ++b)
                if (b != a && parity(faces[order[b]].k) != pa) twin = true;
            if (!twin) {
                const int* k = faces[order[a]].k;
                bnd.push_back({k[0], k[1], k[2]});
            }
        }
        i = j;
    }
    std::sort(bnd.begin(), bnd.end());
    bnd.erase(std::unique(bnd.begin(), bnd.end()), bnd.end());
    tris.clear();
    for (auto& t : bnd) tris.insert(tris.end(), t.begin(), t.end());
    // edges: orientation of the first triangle (in order) containing them
    std::map<std::pair<int, int>, std::pair<int, int>> first;  // unordered key -> oriented
    for (auto& t : bnd) {
        int pr[3][2] = {{t[0], t[1]}, {t[1], t[2]}, {t[2], t[0]}};
        for (auto& p : pr) {
            auto key = std::make_pair(std::min(p[0], p[1]), std::max(p[0], p[1]));
            if (!first.count(key)) first[key] = {p[0], p[1]};
        }
    }
    std::vector<std::pair<int, int>> ev;
    for (auto& kv : first) ev.push_back(kv.second);
    std::sort(ev.begin(), ev.end());
    edges.clear();
    for (auto& e : ev) { edges.push_back(e.first); edges.push_back(e.second); }
    std::vector<char> is(V, 0);
    for (int v : tris) is[v] = 1;
    nodes.clear();
    for (int v = 0; v < V; ++v)
        if (is[v]) nodes.push_back(v);
}

void build_chunks(const std::vector<int>& off, std::vector<Chunk>& ch, std::vector<int>& coff) {
    ch.clear();
    coff.assign(off.size(), 0);
    for (size_t i = 0; i + 1 < off.size(); ++i) {
        coff[i] = (int)ch.size();
        for (int b = off[i]; b < off[i + 1]; b += kChunk) ch.push_back({(int)i, b, std::min(b + kChunk, off[i + 1])});
    }
    coff.back() = (int)ch.size();
    if (ch.empty()) ch.push_back({0, 0, 0});
}

// per-instance device scalar layout inside ctx->inst_buf
enum { S_ETET, S_EINERT, S_EBAR, S_MIND, S_NORM2, S_TOL, S_EDBC, S_DDBC, S_NUMD };
enum { SI_BAD, SI_BADB, SI_KFLAG, SI_CCDF, SI_ISECT, S_NUMI };

double* dsc(idp_ctx* c, int k) { return c->inst_buf.as<double>() + (long)k * c->A.nI; }
int* isc(idp_ctx* c, int k) { return reinterpret_cast<int*>(c->inst_buf.as<double>() + (long)S_NUMD * c->A.nI) + (long)k * c->A.nI; }

int set_mask(idp_ctx* c, const std::vector<unsigned char>& m) {
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.active, m.data(), m.size(), cudaMemcpyHostToDevice, c->s));
    return IDP_OK;
}

template <class T>
int fetch(idp_ctx* c, const T* d, std::vector<T>& h) {
    h.resize(c->A.nI);
    IDP_CUDA_TRY(cudaMemcpyAsync(h.data(), d, sizeof(T) * c->A.nI, cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

// every per-instance scalar (energies, norms, flags) in one copy and one
// synchronisation
struct InstScalars {
    std::vector<double> buf;
    int nI = 0;
    double d(int k, int i) const { return buf[(size_t)k * nI + i]; }
    int flag(int k, int i) const {
        return reinterpret_cast<const int*>(buf.data() + (size_t)S_NUMD * nI)[(size_t)k * nI + i];
    }
};

int fetch_scalars(idp_ctx* c, InstScalars& out) {
    const int nI = c->A.nI;
    out.nI = nI;
    out.buf.resize((size_t)(S_NUMD + S_NUMI) * nI);
    IDP_CUDA_TRY(cudaMemcpyAsync(out.buf.data(), c->inst_buf.p, sizeof(double) * S_NUMD * nI + sizeof(int) * S_NUMI * nI,
                                 cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

// Spatial order of an instance's vertices: Morton codes of the rest
// positions quantized to 10 bits per axis over the instance's bounding box,
// ties in the caller's order. perm[k] = caller index of device vertex k.
std::vector<int> morton_order(const HostInstance& h) {
    const int V = h.V;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int v = 0; v < V; ++v)
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], h.X0[3 * v + d]);
            hi[d] = std::max(hi[d], h.X0[3 * v + d]);
        }
    const double ext = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
    const double sc = ext > 0 ? 1023.0 / ext : 0.0;
    auto spread = [](uint64_t x) {
        uint64_t r = 0;
        for (int b = 0; b < 10; ++b) r |= ((x >> b) & 1ull) << (3 * b);
        return r;
    };
    std::vector<std::pair<uint64_t, int>> key(V);
    for (int v = 0; v < V; ++v) {
        uint64_t q[3];
        for (int d = 0; d < 3; ++d) {
            double t = (h.X0[3 * v + d] - lo[d]) * sc;
            q[d] = (uint64_t)std::min(1023.0, std::max(0.0, std::floor(t)));
        }
        key[v] = {spread(q[0]) | (spread(q[1]) << 1) | (spread(q[2]) << 2), v};
    }
    std::sort(key.begin(), key.end());
    std::vector<int> perm(V);
    for (int k = 0; k < V; ++k) perm[k] = key[k].second;
    return perm;
}

// copy of an instance with its vertices in device order `perm`: per-vertex
// arrays gathered, vertex ids in element, surface and DBC lists renamed
// (the lists keep their order)
HostInstance to_device_order(const HostInstance& h, const std::vector<int>& perm) {
    HostInstance d = h;
    const int V = h.V;
    std::vector<int> ip(V);
    for (int k = 0; k < V; ++k) ip[perm[k]] = k;
    auto g3 = [&](const std::vector<double>& a, std::vector<double>& o) {
        if (a.size() != 3 * (size_t)V) return;
        for (int k = 0; k < V; ++k)
            for (int j = 0; j < 3; ++j) o[3 * k + j] = a[3 * (size_t)perm[k] + j];
    };
    g3(h.X, d.X);
    g3(h.X0, d.X0);
    g3(h.v, d.v);
    g3(h.xtilde, d.xtilde);
    g3(h.bacc, d.bacc);
    g3(h.dbc_tgt, d.dbc_tgt);
    for (int k = 0; k < V; ++k) {
        d.mass[k] = h.mass[perm[k]];
        d.dbc[k] = h.dbc[perm[k]];
    }
    for (auto* a : {&d.tets, &d.faces, &d.hinges, &d.tris, &d.edges, &d.nodes, &d.dbc_list})
        for (int& v : *a) v = ip[v];
    d.perm = perm;
    return d;
}

// 3-vectors of instance i between the caller and the device: in device
// order at dst (+ the instance's offset) from the caller's host array src
int upload3(idp_ctx* c, int i, const double* src, double* dst) {
    const long o = 3L * c->A.v_off[i], n = 3L * c->inst[i].V;
    if (c->inst[i].perm.empty()) {
        IDP_CUDA_TRY(cudaMemcpyAsync(dst + o, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
        return IDP_OK;
    }
    IDP_CUDA_TRY(cudaMemcpyAsync(c->stage.as<double>() + o, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    return perm_to_device(c->A, c->A.v_off[i], c->inst[i].V, c->stage.as<double>(), dst, c->s);
}

// ... and back: the caller's host array dst from device-order src
int download3(idp_ctx* c, int i, const double* src, double* dst) {
    const long o = 3L * c->A.v_off[i], n = 3L * c->inst[i].V;
    if (c->inst[i].perm.empty()) {
        IDP_CUDA_TRY(cudaMemcpyAsync(dst, src + o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
        return IDP_OK;
    }
    int rc = perm_to_caller(c->A, c->A.v_off[i], c->inst[i].V, src, c->stage.as<double>(), c->s);
    if (rc) return rc;
    IDP_CUDA_TRY(cudaMemcpyAsync(dst, c->stage.as<double>() + o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    return IDP_OK;
}

// some instance has its moving-DBC penalty on (the device copy A.dstiff
// mirrors InstState::dbc_stiff)
bool dbc_penalty_on(idp_ctx* c) {
    for (const InstState& S : c->st)
        if (S.dbc_stiff > 0) return true;
    return false;
}

int upload_dbc_stiff(idp_ctx* c) {
    std::vector<double> k(c->A.nI);
    for (int i = 0; i < c->A.nI; ++i) k[i] = c->st[i].dbc_stiff;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.dstiff, k.data(), sizeof(double) * k.size(), cudaMemcpyHostToDevice, c->s));
    return IDP_OK;
}

// the rows projected to the identity for instance i: its fixed DBC vertices
// while the penalty pulls the moving ones, every DBC vertex otherwise
// (INC_POTENTIAL.h:387-394)
int set_projection(idp_ctx* c, int i, bool penalty) {
    const long o = c->A.v_off[i], n = c->inst[i].V;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.dbc + o, (penalty ? c->A.dfix : c->A.dbc_excl) + o, n, cudaMemcpyDeviceToDevice,
                                 c->s));
    return IDP_OK;
}

// incremental potential of the masked instances at X (INC_POTENTIAL.h:15-152):
// E = h^2 sum vol*Psi + inertia [+ barrier over a freshly built constraint
// set]. bad[i] = 1 when a tet is inverted, 2 when a constraint distance is
// not positive (the reference exits there).
int eval_energy(idp_ctx* c, const double* X, bool with_barrier, std::vector<double>& E, std::vector<int>& bad) {
    Arena& A = c->A;
    const int nI = A.nI;
    double h2 = c->P.h * c->P.h;
    IDP_CUDA_TRY(cudaMemsetAsync(isc(c, SI_BAD), 0, sizeof(int) * nI * 2, c->s));
    IDP_CUDA_TRY(cudaMemsetAsync(dsc(c, S_EBAR), 0, sizeof(double) * nI, c->s));
    c->W.timer.start(PhaseTimer::TET, c->s);
    int rc = tet_energy(A, c->W, X, h2, dsc(c, S_ETET), isc(c, SI_BAD), c->s);
    if (!rc) rc = flow_energy(A, c->W, X, dsc(c, S_ETET), c->s);
    if (!rc) rc = shell_energy(A, c->W, X, h2, dsc(c, S_ETET), c->s);
    c->W.timer.stop(c->s);
    if (rc) return rc;
    rc = vec_inertia(A, c->W, X, dsc(c, S_EINERT), nullptr, c->s);
    if (rc) return rc;
    if (with_barrier) {
        rc = barrier_energy(A, c->W, X, c->cs, dsc(c, S_EBAR), isc(c, SI_BADB), c->s);
        if (rc) return rc;
    }
    const bool dpen = dbc_penalty_on(c);
    if (dpen && (rc = dbc_sums(A, c->W, X, dsc(c, S_EDBC), dsc(c, S_DDBC), c->s))) return rc;
    // one copy of the whole per-instance scalar block, one synchronisation
    std::vector<double> hb((size_t)(S_NUMD + S_NUMI) * nI);
    IDP_CUDA_TRY(cudaMemcpyAsync(hb.data(), c->inst_buf.p, sizeof(double) * S_NUMD * nI + sizeof(int) * S_NUMI * nI,
                                 cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    const double* et = hb.data() + (size_t)S_ETET * nI;
    const double* ei = hb.data() + (size_t)S_EINERT * nI;
    const double* eb = hb.data() + (size_t)S_EBAR * nI;
    const double* ed = hb.data() + (size_t)S_EDBC * nI;
    const int* hi = reinterpret_cast<const int*>(hb.data() + (size_t)S_NUMD * nI);
    const int* b1 = hi + (size_t)SI_BAD * nI;
    const int* b2 = hi + (size_t)SI_BADB * nI;
    E.resize(nI);
    bad.resize(nI);
    for (int i = 0; i < nI; ++i) {
        E[i] = et[i] + ei[i] + eb[i];
        // Compute_DBC_Energy (FEM/Shell/DIRICHLET.h:26-45)
        if (dpen && c->st[i].dbc_stiff > 0) E[i] += 0.5 * c->st[i].dbc_stiff * ed[i];
        bad[i] = b1[i] ? 1 : (b2[i] ? 2 : 0);
    }
    return IDP_OK;
}

// gradient of the masked instances at X into A.g (INC_POTENTIAL.h:154-275),
// DBC rows zeroed (IMPLICIT_EULER.h:476-480)
int eval_gradient(idp_ctx* c, const double* X) {
    Arena& A = c->A;
    double h2 = c->P.h * c->P.h;
    c->W.timer.start(PhaseTimer::TET, c->s);
    int rc = tet_gradient(A, c->W, X, h2, nullptr, c->s);
    c->W.timer.stop(c->s);
    if (rc) return rc;
    rc = grad_gather_tet(A, c->W, X, A.g, c->s);
    if (!rc) rc = flow_gradient(A, X, A.g, c->s);
    if (!rc) rc = shell_gradient(A, c->W, X, h2, A.g, c->s);
    if (rc) return rc;
    c->W.timer.start(PhaseTimer::BARRIER, c->s);
    rc = barrier_gradient(A, c->W, X, c->cs, A.g, c->s);
    c->W.timer.stop(c->s);
    if (rc) return rc;
    // moving-DBC penalty (IMPLICIT_EULER.h:467-474), then the projected rows
    if (dbc_penalty_on(c) && (rc = dbc_gradient(A, X, A.g, c->s))) return rc;
    return vec_zero_dbc(A, A.g, c->s);
}

int eval_hessian(idp_ctx* c, const double* X, bool force_fp64 = false) {
    Arena& A = c->A;
    bool fp64 = force_fp64 || c->P.mode == IDP_MODE_FP64;
    c->W.timer.start(PhaseTimer::TET, c->s);
    int rc = tet_hessian(A, c->W, X, c->P.h * c->P.h, fp64, c->s);
    if (!rc) rc = shell_hessian(A, c->W, X, c->P.h * c->P.h, fp64, c->s);
    c->W.timer.stop(c->s);
    if (rc) return rc;
    c->W.timer.start(PhaseTimer::BARRIER, c->s);
    rc = barrier_hessian(A, c->W, X, c->cs, fp64, c->s);
    c->W.timer.stop(c->s);
    if (rc) return rc;
    c->W.timer.start(PhaseTimer::ASSEMBLY, c->s);
    rc = assemble(A, c->W, c->cs, fp64, c->s);
    if (!rc) rc = build_contact_clusters(A, c->W, c->cs, fp64, c->s);
    c->W.timer.stop(c->s);
    return rc;
}

// copy the current constraint set to the "previous" slot with its distances
int save_prev_set(idp_ctx* c, const double* X) {
    Arena& A = c->A;
    Work& W = c->W;
    long C = c->cs.C;
    long Ca = C > 0 ? C : 1;
    if (W[W_PREV_CONS].ensure(sizeof(int4) * Ca) || W[W_PREV_INST].ensure(sizeof(int) * Ca) ||
        W[W_PREV_DIST2].ensure(sizeof(double) * Ca))
        return IDP_ERR_CUDA;
    if (C > 0) {
        IDP_CUDA_TRY(cudaMemcpyAsync(W[W_PREV_CONS].p, W[W_CONS].p, sizeof(int4) * C, cudaMemcpyDeviceToDevice, c->s));
        IDP_CUDA_TRY(cudaMemcpyAsync(W[W_PREV_INST].p, W[W_CONS_INST].p, sizeof(int) * C, cudaMemcpyDeviceToDevice, c->s));
        int rc = constraint_min_dist2(A, W, X, W[W_PREV_CONS].as<int4>(), W[W_PREV_INST].as<int>(), C,
                                      W[W_PREV_DIST2].as<double>(), nullptr, c->s);
        if (rc) return rc;
    }
    c->prevC = C;
    return IDP_OK;
}

}  // namespace

// ============================================================== C ABI
extern "C" {

void idp_default_params(idp_params* p) {
    p->h = 0.1;
    p->newton_tol = 1e-3;
    p->max_newton = 2000;
    p->mode = IDP_MODE_MIXED;
    p->pcg_rel_tol = 1e-6;
    p->pcg_max_iters = 2000;
    p->thickness = 0.0;
    p->device = 0;
    p->pcg_grid_min_vertices = 0;
    p->pcg_grid_cta_vertices = 0;
    p->contact_block_vertices = 0;
    p->verify_iterates = 0;
    p->caller_vertex_order = 0;
    p->pcg_local_degree = 0;
    p->surface_device_min_tets = 0;
}

const char* idp_status_str(int s) {
    switch (s) {
        case IDP_OK: return "ok";
        case IDP_ERR_INVALID_ARG: return "invalid argument";
        case IDP_ERR_CUDA: return "CUDA error";
        case IDP_ERR_CAPACITY: return "capacity exceeded";
        case IDP_ERR_INVERTED: return "inverted tet (det F <= 0)";
        case IDP_ERR_NOT_CONVERGED: return "Newton did not converge within max_newton";
        case IDP_ERR_ZERO_STEP: return "CCD returned a zero step";
        case IDP_ERR_NONPOSITIVE_DIST: return "non-positive constraint distance";
        case IDP_ERR_STATE: return "call out of order";
        case IDP_WARN_ITER_CAP: return "ACCD iteration cap reached (step still conservative)";
        case IDP_ERR_INTERSECTION: return "accepted iterate has an edge-triangle intersection";
        default: return "unknown status";
    }
}

idp_ctx* idp_create(const idp_params* p, int* status) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        if (status) *status = IDP_ERR_CUDA;
        return nullptr;
    }
    idp_ctx* c = new idp_ctx();
    if (p) c->P = *p;
    else idp_default_params(&c->P);
    c->W.grid_min_v = c->P.pcg_grid_min_vertices > 0 ? c->P.pcg_grid_min_vertices : 16384;
    c->W.grid_vper = c->P.pcg_grid_cta_vertices > 0 ? c->P.pcg_grid_cta_vertices : 112;
    if (c->P.pcg_local_degree < 0 || c->P.pcg_local_degree > 8 || (c->P.pcg_local_degree & 1)) {
        delete c;
        if (status) *status = IDP_ERR_INVALID_ARG;
        return nullptr;
    }
    c->W.local_deg = c->P.pcg_local_degree;
    c->W.cl_cap = c->P.contact_block_vertices > 0 ? std::max(2, std::min(c->P.contact_block_vertices, kClusterCap))
                                                  : kClusterCap;
    int prio_lo = 0, prio_hi = 0;
    if (cudaSetDevice(c->P.device) != cudaSuccess || cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->s2, cudaStreamNonBlocking, prio_hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_x, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_vox, cudaEventDisableTiming) != cudaSuccess) {
        if (c->s) cudaStreamDestroy(c->s);
        if (c->s2) cudaStreamDestroy(c->s2);
        if (c->ev_x) cudaEventDestroy(c->ev_x);
        delete c;
        if (status) *status = IDP_ERR_CUDA;
        return nullptr;
    }
    if (status) *status = IDP_OK;
    return c;
}

void idp_destroy(idp_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->P.device);
    cudaStreamSynchronize(c->s);
    cudaStreamSynchronize(c->s2);
    for (auto& b : c->owned) b.release();
    c->W.release();
    c->inst_buf.release();
    c->vel.release();
    c->bacc.release();
    c->snap.release();
    cudaEventDestroy(c->ev_x);
    cudaEventDestroy(c->ev_vox);
    cudaStreamDestroy(c->s2);
    cudaStreamDestroy(c->s);
    delete c;
}

int idp_reset(idp_ctx* c) {
    if (!c) return IDP_ERR_INVALID_ARG;
    cudaSetDevice(c->P.device);
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    c->inst.clear();
    c->st.clear();
    c->A = Arena();
    c->owned_next = 0;
    c->committed = false;
    c->cs = ContactSet();
    c->prevC = 0;
    c->has_snap = false;
    c->has_bacc = false;
    c->stepping = false;
    c->snap_kappa.clear();
    c->W.stats = idp_stats{};
    c->W.dense_ready[0] = c->W.dense_ready[1] = false;
    return IDP_OK;
}

int idp_device_bytes(idp_ctx* c, size_t* bytes) {
    if (!c || !bytes) return IDP_ERR_INVALID_ARG;
    size_t n = c->inst_buf.bytes + c->vel.bytes + c->snap.bytes + c->bacc.bytes;
    for (const DBuf& b : c->owned) n += b.bytes;
    for (const DBuf& b : c->W.b) n += b.bytes;
    *bytes = n;
    return IDP_OK;
}

int idp_add_instance(idp_ctx* c, int V, const double* X, const double* X0, int T, const int32_t* tets,
                     const double* mass, const double* lam, const double* mu, int nDBC, const int32_t* dbc_idx,
                     double dHat2, double kappa, double kappa_max) {
    if (!c) return -IDP_ERR_INVALID_ARG;
    if (c->committed) return -IDP_ERR_STATE;
    if (V <= 0 || T <= 0 || !X || !tets || !mass || !lam || !mu || !(dHat2 > 0)) return -IDP_ERR_INVALID_ARG;
    HostInstance h;
    h.V = V;
    h.T = T;
    h.X.assign(X, X + 3 * (long)V);
    h.X0.assign(X0 ? X0 : X, (X0 ? X0 : X) + 3 * (long)V);
    h.tets.assign(tets, tets + 4 * (long)T);
    for (int v : h.tets)
        if (v < 0 || v >= V) return -IDP_ERR_INVALID_ARG;
    h.mass.assign(mass, mass + V);
    h.lam.assign(lam, lam + T);
    h.mu.assign(mu, mu + T);
    h.dbc.assign(V, 0);
    for (int k = 0; k < nDBC; ++k) {
        if (dbc_idx[k] < 0 || dbc_idx[k] >= V) return -IDP_ERR_INVALID_ARG;
        h.dbc[dbc_idx[k]] = 1;
    }
    if (nDBC > 0) h.dbc_list.assign(dbc_idx, dbc_idx + nDBC);
    h.v.assign(3 * (long)V, 0.0);
    h.dHat2 = dHat2;
    h.kappa = kappa;
    h.kappa_max = kappa_max;
    const long dev_min = c->P.surface_device_min_tets == 0 ? 65536 : c->P.surface_device_min_tets;
    if (dev_min > 0 && T >= dev_min && V <= (1 << 21)) {
        cudaSetDevice(c->P.device);
        const int rc = idp::extract_surface_device(V, h.tets, h.tris, h.edges, h.nodes, c->s);
        if (rc) return -rc;
    } else {
        extract_surface(V, h.tets, h.tris, h.edges, h.nodes);
    }
    double s = 0;
    for (size_t e = 0; e + 1 < h.edges.size(); e += 2) {
        const double* a = &h.X0[3 * h.edges[e]];
        const double* b = &h.X0[3 * h.edges[e + 1]];
        s += std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    }
    h.rest_mean_edge = h.edges.empty() ? 1.0 : s / (h.edges.size() / 2);
    c->inst.push_back(std::move(h));
    return (int)c->inst.size() - 1;
}

// Triangle shell common to flow mode and elastic shells, at its rest
// positions X: Initialize_Discrete_Shell's face filter, lumped mass and
// element volumes (FEM/Shell/DISCRETE_SHELL.h:238-333) and
// Find_Surface_Primitives (Utils/MESHIO.h:728-766) for the contact surface.
// Returns 0 or -IDP_*.
static int build_shell(HostInstance& h, int V, const double* X, int F, const int32_t* faces, double density,
                       double thickness, int nDBC, const int32_t* dbc_idx, double dHat2, double kappa,
                       double kappa_max) {
    if (V <= 0 || F <= 0 || !X || !faces || !(density > 0) || !(thickness > 0) || !(dHat2 > 0))
        return -IDP_ERR_INVALID_ARG;
    h.shell = true;
    h.V = V;
    h.T = 0;
    h.X.assign(X, X + 3 * (long)V);
    h.X0 = h.X;
    h.mass.assign(V, 0.0);
    for (int f = 0; f < F; ++f) {
        const int* t = faces + 3 * f;
        for (int k = 0; k < 3; ++k)
            if (t[k] < 0 || t[k] >= V) return -IDP_ERR_INVALID_ARG;
        double e1[3], e2[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = X[3 * t[1] + d] - X[3 * t[0] + d];
            e2[d] = X[3 * t[2] + d] - X[3 * t[0] + d];
        }
        const double a = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
        const double b = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
        const double cc = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
        if (a * cc - b * b == 0.0) continue;  // singular first fundamental form
        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double area = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) / 2;
        const double mp = area * thickness * density / 3;
        for (int k = 0; k < 3; ++k) {
            h.faces.push_back(t[k]);
            h.mass[t[k]] += mp;
        }
        h.fvol.push_back(area * thickness);
    }
    if (h.faces.empty()) return -IDP_ERR_INVALID_ARG;
    std::vector<char> used(V, 0);
    for (int v : h.faces) used[v] = 1;
    for (int v = 0; v < V; ++v)
        if (!used[v]) return -IDP_ERR_INVALID_ARG;  // every vertex needs a face (mass, diagonal block)
    h.dbc.assign(V, 0);
    for (int k = 0; k < nDBC; ++k) {
        if (!dbc_idx || dbc_idx[k] < 0 || dbc_idx[k] >= V) return -IDP_ERR_INVALID_ARG;
        h.dbc[dbc_idx[k]] = 1;
    }
    if (nDBC > 0) h.dbc_list.assign(dbc_idx, dbc_idx + nDBC);
    h.v.assign(3 * (long)V, 0.0);
    h.dHat2 = dHat2;
    h.kappa = kappa;
    h.kappa_max = kappa_max;
    // surface primitives: every face, edges in set order with the first
    // orientation unless the reverse is present, nodes ascending
    std::set<std::pair<int, int>> es;
    for (size_t f = 0; f < h.faces.size(); f += 3) {
        const int t[3] = {h.faces[f], h.faces[f + 1], h.faces[f + 2]};
        for (int k = 0; k < 3; ++k) {
            const int a = t[k], b = t[(k + 1) % 3];
            if (!es.count({b, a})) es.insert({a, b});
        }
    }
    h.tris = h.faces;
    for (auto& e : es) {
        h.edges.push_back(e.first);
        h.edges.push_back(e.second);
    }
    for (int v = 0; v < V; ++v) h.nodes.push_back(v);
    double sl = 0;
    for (size_t e = 0; e + 1 < h.edges.size(); e += 2) {
        const double* a = &h.X0[3 * h.edges[e]];
        const double* b = &h.X0[3 * h.edges[e + 1]];
        sl += std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    }
    h.rest_mean_edge = h.edges.empty() ? 1.0 : sl / (h.edges.size() / 2);
    return 0;
}

// Triangle shell in flow mode (Advance_One_Step_IE_Flow).
int idp_add_shell_instance(idp_ctx* c, int V, const double* X, int F, const int32_t* faces, double density,
                           double thickness, int nDBC, const int32_t* dbc_idx, double dHat2, double kappa,
                           double kappa_max) {
    if (!c) return -IDP_ERR_INVALID_ARG;
    if (c->committed) return -IDP_ERR_STATE;
    HostInstance h;
    int r = build_shell(h, V, X, F, faces, density, thickness, nDBC, dbc_idx, dHat2, kappa, kappa_max);
    if (r) return r;
    c->inst.push_back(std::move(h));
    return (int)c->inst.size() - 1;
}

// Dihedral angle of the hinge (x0, x1, x2, x3) with hinge edge x1-x2
// (Math/DIHEDRAL_ANGLE.h:10-24).
static double dihedral_host(const double* x0, const double* x1, const double* x2, const double* x3) {
    double a[3], b[3], c3[3], d[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = x1[k] - x0[k];
        b[k] = x2[k] - x0[k];
        c3[k] = x2[k] - x3[k];
        d[k] = x1[k] - x3[k];
    }
    const double n1[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
    const double n2[3] = {c3[1] * d[2] - c3[2] * d[1], c3[2] * d[0] - c3[0] * d[2], c3[0] * d[1] - c3[1] * d[0]};
    const double n11 = n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2];
    const double n22 = n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2];
    double cth = (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) / std::sqrt(n11 * n22);
    cth = std::max(-1.0, std::min(1.0, cth));
    double t = std::acos(cth);
    const double m[3] = {n2[1] * n1[2] - n2[2] * n1[1], n2[2] * n1[0] - n2[0] * n1[2], n2[0] * n1[1] - n2[1] * n1[0]};
    if (m[0] * (x1[0] - x2[0]) + m[1] * (x1[1] - x2[1]) + m[2] * (x1[2] - x2[2]) < 0) t = -t;
    return t;
}

// Elastic triangle shell of the Hinge path: neo-Hookean membrane per face and
// hinge bending per interior edge, with the rest data of
// Compute_Discrete_Shell_Inv_Basis and the stiffness of
// Initialize_Discrete_Shell (DISCRETE_SHELL.h:132-216,218-357).
int idp_add_elastic_shell_instance(idp_ctx* c, int V, const double* X, const double* X0, int F,
                                   const int32_t* faces, const double* mass, double density, double E, double nu,
                                   double thickness, double bending_mult, int nDBC, const int32_t* dbc_idx,
                                   double dHat2, double kappa, double kappa_max) {
    if (!c) return -IDP_ERR_INVALID_ARG;
    if (c->committed) return -IDP_ERR_STATE;
    if (!(E > 0) || !(nu > -1.0 && nu < 0.5) || !(bending_mult >= 0)) return -IDP_ERR_INVALID_ARG;
    if (!X0) X0 = X;
    HostInstance h;
    int r = build_shell(h, V, X0, F, faces, density, thickness, nDBC, dbc_idx, dHat2, kappa, kappa_max);
    if (r) return r;
    if (!X) return -IDP_ERR_INVALID_ARG;
    if (mass) {
        for (int v = 0; v < V; ++v)
            if (!(mass[v] > 0)) return -IDP_ERR_INVALID_ARG;
        h.mass.assign(mass, mass + V);
    }
    h.X.assign(X, X + 3 * (long)V);
    h.elastic = true;
    h.fvol.clear();  // no flow energy
    const double lam = E * nu / (1.0 - nu * nu), mu = E / (2.0 * (1.0 + nu));
    const size_t nf = h.faces.size() / 3;
    for (size_t f = 0; f < nf; ++f) {
        const double* x1 = &h.X0[3 * h.faces[3 * f]];
        const double* x2 = &h.X0[3 * h.faces[3 * f + 1]];
        const double* x3 = &h.X0[3 * h.faces[3 * f + 2]];
        double e1[3], e2[3];
        for (int d = 0; d < 3; ++d) {
            e1[d] = x2[d] - x1[d];
            e2[d] = x3[d] - x1[d];
        }
        const double a00 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
        const double a01 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
        const double a11 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
        const double det = a00 * a11 - a01 * a01;
        const double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double i00 = a11 / det, i01 = -a01 / det, i11 = a00 / det;
        const double vals[7] = {i00, i01, i11, i00 * i11 - i01 * i01,
                                std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) / 2 * thickness, lam, mu};
        h.mem.insert(h.mem.end(), vals, vals + 7);
    }
    // hinges of the surface edges in their order: x0 follows x2 in the face
    // holding the directed edge x1->x2, x3 follows x1 in the face holding
    // x2->x1 (DISCRETE_SHELL.h:172-212); boundary edges have none
    std::map<std::pair<int, int>, int> e2t;
    for (size_t f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) e2t[{h.faces[3 * f + k], h.faces[3 * f + (k + 1) % 3]}] = (int)f;
    const double kb = bending_mult * E * thickness * thickness * thickness / (24.0 * (1.0 - nu * nu));
    for (size_t e = 0; e + 1 < h.edges.size(); e += 2) {
        const int a = h.edges[e], b = h.edges[e + 1];
        auto it = e2t.find({a, b});
        if (it == e2t.end()) continue;
        auto jt = e2t.find({b, a});
        if (jt == e2t.end()) continue;
        const int* t = &h.faces[3 * it->second];
        const int* o = &h.faces[3 * jt->second];
        int v0 = -1, v3 = -1;
        for (int j = 0; j < 3; ++j) {
            if (t[j] == b) v0 = t[(j + 1) % 3];
            if (o[j] == a) v3 = o[(j + 1) % 3];
        }
        const double* P0 = &h.X0[3 * v0];
        const double* P1 = &h.X0[3 * a];
        const double* P2 = &h.X0[3 * b];
        const double* P3 = &h.X0[3 * v3];
        const double thb = dihedral_host(P0, P1, P2, P3);
        double d12[3], a1[3], b1[3], c1[3], dd[3];
        for (int d = 0; d < 3; ++d) {
            d12[d] = P1[d] - P2[d];
            a1[d] = P1[d] - P0[d];
            b1[d] = P2[d] - P0[d];
            c1[d] = P2[d] - P3[d];
            dd[d] = P1[d] - P3[d];
        }
        const double ebar = std::sqrt(d12[0] * d12[0] + d12[1] * d12[1] + d12[2] * d12[2]);
        const double n1[3] = {a1[1] * b1[2] - a1[2] * b1[1], a1[2] * b1[0] - a1[0] * b1[2], a1[0] * b1[1] - a1[1] * b1[0]};
        const double n2[3] = {c1[1] * dd[2] - c1[2] * dd[1], c1[2] * dd[0] - c1[0] * dd[2], c1[0] * dd[1] - c1[1] * dd[0]};
        const double hbar = (std::sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]) +
                             std::sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2])) / (ebar * 6);
        const int st[4] = {v0, a, b, v3};
        h.hinges.insert(h.hinges.end(), st, st + 4);
        h.hk.push_back(thb);
        h.hk.push_back(kb * ebar / hbar);
    }
    c->inst.push_back(std::move(h));
    return (int)c->inst.size() - 1;
}

int idp_set_velocity(idp_ctx* c, int i, const double* v) {
    if (!c || i < 0 || i >= (int)c->inst.size() || !v) return IDP_ERR_INVALID_ARG;
    HostInstance& h = c->inst[i];
    h.v.assign(v, v + 3 * (long)h.V);
    h.vel_set = true;
    if (c->committed) {
        int rc = upload3(c, i, v, c->vel.as<double>());
        if (rc) return rc;
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    }
    return IDP_OK;
}

int idp_set_body_force(idp_ctx* c, int i, const double* b) {
    if (!c || i < 0 || i >= (int)c->inst.size()) return IDP_ERR_INVALID_ARG;
    HostInstance& h = c->inst[i];
    if (!b) {
        h.bacc.clear();
    } else {
        // a = M^-1 b with the lumped (diagonal) mass
        std::vector<double> acc(3 * (size_t)h.V);
        for (int v = 0; v < h.V; ++v) {
            if (!(h.mass[v] > 0)) return IDP_ERR_INVALID_ARG;
            for (int d = 0; d < 3; ++d) acc[3 * v + d] = b[3 * v + d] / h.mass[v];
        }
        h.bacc.swap(acc);
    }
    if (c->committed) {
        cudaSetDevice(c->P.device);
        const long n = 3L * c->A.V, o = 3L * c->A.v_off[i];
        if (!c->has_bacc) {
            if (!b) return IDP_OK;
            if (c->bacc.ensure(sizeof(double) * (n + 3))) return IDP_ERR_CUDA;
            IDP_CUDA_TRY(cudaMemsetAsync(c->bacc.p, 0, sizeof(double) * n, c->s));
            c->has_bacc = true;
        }
        if (b) {
            int rc = upload3(c, i, h.bacc.data(), c->bacc.as<double>());
            if (rc) return rc;
        } else
            IDP_CUDA_TRY(cudaMemsetAsync(c->bacc.as<double>() + o, 0, sizeof(double) * 3 * h.V, c->s));
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    }
    return IDP_OK;
}

int idp_set_normal_flow(idp_ctx* c, int i, double step) {
    if (!c || i < -1 || i >= (int)c->inst.size() || !std::isfinite(step)) return IDP_ERR_INVALID_ARG;
    if (!c->committed) return IDP_ERR_STATE;
    cudaSetDevice(c->P.device);
    if (c->A.nI == 0) return IDP_OK;
    int rc = normal_flow_velocity(c->A, i, step, c->P.h, c->vel.as<double>(), c->s);
    if (rc) return rc;
    for (int k = 0; k < (int)c->inst.size(); ++k)
        if (i < 0 || k == i) c->inst[k].vel_set = true;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

int idp_set_positions(idp_ctx* c, int i, const double* X) {
    if (!c || i < 0 || i >= (int)c->inst.size() || !X) return IDP_ERR_INVALID_ARG;
    HostInstance& h = c->inst[i];
    h.X.assign(X, X + 3 * (long)h.V);
    if (c->committed) {
        int rc = upload3(c, i, X, c->A.X);
        if (rc) return rc;
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    }
    return IDP_OK;
}

int idp_set_dbc_targets(idp_ctx* c, int i, const double* targets) {
    if (!c || i < 0 || i >= (int)c->inst.size()) return IDP_ERR_INVALID_ARG;
    if (c->stepping) return IDP_ERR_STATE;
    HostInstance& h = c->inst[i];
    if (h.dbc_list.empty()) return targets ? IDP_ERR_INVALID_ARG : IDP_OK;
    if (!targets) {
        h.dbc_tgt.clear();
    } else {
        // one row per DBC vertex: a vertex listed twice has no single target
        std::vector<double> t(3 * (size_t)h.V, 0.0);
        std::vector<char> seen(h.V, 0);
        for (size_t k = 0; k < h.dbc_list.size(); ++k) {
            const int v = h.dbc_list[k];
            if (seen[v]) return IDP_ERR_INVALID_ARG;
            seen[v] = 1;
            for (int d = 0; d < 3; ++d) {
                if (!std::isfinite(targets[3 * k + d])) return IDP_ERR_INVALID_ARG;
                t[3 * v + d] = targets[3 * k + d];
            }
        }
        h.dbc_tgt.swap(t);
    }
    if (c->committed) {
        if (!c->A.dtgt) return IDP_ERR_STATE;
        cudaSetDevice(c->P.device);
        if (!h.dbc_tgt.empty()) {
            int rc = upload3(c, i, h.dbc_tgt.data(), c->A.dtgt);
            if (rc) return rc;
        }
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    }
    return IDP_OK;
}

int idp_commit(idp_ctx* c) {
    if (!c) return IDP_ERR_INVALID_ARG;
    if (c->committed) return IDP_ERR_STATE;
    if (c->inst.empty()) return IDP_ERR_INVALID_ARG;
    cudaSetDevice(c->P.device);
    Arena& A = c->A;
    const int nI = (int)c->inst.size();
    A.nI = nI;
    A.v_off.assign(nI + 1, 0);
    A.t_off.assign(nI + 1, 0);
    A.f_off.assign(nI + 1, 0);
    A.fm_off.assign(nI + 1, 0);
    A.hn_off.assign(nI + 1, 0);
    A.sn_off.assign(nI + 1, 0);
    A.se_off.assign(nI + 1, 0);
    A.st_off.assign(nI + 1, 0);
    // device order of each instance's vertices (the caller's order is kept
    // on the host; every transfer across the interface maps between them)
    std::vector<HostInstance> dview(nI);
    std::vector<const HostInstance*> hv(nI);
    for (int i = 0; i < nI; ++i) {
        if (c->P.caller_vertex_order || c->inst[i].perm.size() != (size_t)c->inst[i].V) c->inst[i].perm.clear();
        if (!c->P.caller_vertex_order && c->inst[i].V > 1) {
            // an instance added from a committed copy keeps its order
            dview[i] = to_device_order(c->inst[i], c->inst[i].perm.empty() ? morton_order(c->inst[i])
                                                                           : c->inst[i].perm);
            c->inst[i].perm = dview[i].perm;
            hv[i] = &dview[i];
        } else {
            hv[i] = &c->inst[i];
        }
    }
    for (int i = 0; i < nI; ++i) {
        const HostInstance& h = *hv[i];
        A.v_off[i + 1] = A.v_off[i] + h.V;
        A.t_off[i + 1] = A.t_off[i] + h.T;
        A.f_off[i + 1] = A.f_off[i] + (int)h.fvol.size();
        A.fm_off[i + 1] = A.fm_off[i] + (int)(h.mem.size() / 7);
        A.hn_off[i + 1] = A.hn_off[i] + (int)(h.hinges.size() / 4);
        A.sn_off[i + 1] = A.sn_off[i] + (int)h.nodes.size();
        A.se_off[i + 1] = A.se_off[i] + (int)h.edges.size() / 2;
        A.st_off[i + 1] = A.st_off[i] + (int)h.tris.size() / 3;
    }
    A.V = A.v_off[nI];
    A.T = A.t_off[nI];
    A.Sn = A.sn_off[nI];
    A.Se = A.se_off[nI];
    A.St = A.st_off[nI];
    A.F = A.f_off[nI];
    A.Fm = A.fm_off[nI];
    A.Hn = A.hn_off[nI];
    A.h = c->P.h;
    std::vector<double> X, X0, mass, vol, lam, mu, IB, vel, dHat2, kappa, thick, cell;
    std::vector<unsigned char> dbc;
    std::vector<int> vinst, snode, sedge, stri, sn_inst, se_inst, st_inst, v2s(A.V, -1), face;
    std::vector<double> fvol, mem, hk;
    std::vector<int> mface, finst, hinst;
    std::vector<int4> tet, hinge;
    std::vector<int> vsrc(A.V);
    for (int i = 0; i < nI; ++i) {
        const HostInstance& h = *hv[i];
        int vo = A.v_off[i];
        for (int k = 0; k < h.V; ++k) vsrc[vo + k] = vo + (h.perm.empty() ? k : h.perm[k]);
        X.insert(X.end(), h.X.begin(), h.X.end());
        X0.insert(X0.end(), h.X0.begin(), h.X0.end());
        mass.insert(mass.end(), h.mass.begin(), h.mass.end());
        lam.insert(lam.end(), h.lam.begin(), h.lam.end());
        mu.insert(mu.end(), h.mu.begin(), h.mu.end());
        vel.insert(vel.end(), h.v.begin(), h.v.end());
        dbc.insert(dbc.end(), h.dbc.begin(), h.dbc.end());
        vinst.insert(vinst.end(), h.V, i);
        for (int t = 0; t < h.T; ++t) {
            const int* e = &h.tets[4 * t];
            tet.push_back(make_int4(e[0] + vo, e[1] + vo, e[2] + vo, e[3] + vo));
            // rest basis and volume (FEM/DEFORMATION_GRADIENT.h:38-76)
            double B[9];
            for (int m = 0; m < 3; ++m)
                for (int d = 0; d < 3; ++d) B[d * 3 + m] = h.X0[3 * e[m + 1] + d] - h.X0[3 * e[0] + d];
            double C0 = B[4] * B[8] - B[5] * B[7], C1 = B[5] * B[6] - B[3] * B[8], C2 = B[3] * B[7] - B[4] * B[6];
            double J = B[0] * C0 + B[1] * C1 + B[2] * C2;
            if (!(J > 0)) return IDP_ERR_INVERTED;
            double Cf[9] = {C0, C1, C2, B[2] * B[7] - B[1] * B[8], B[0] * B[8] - B[2] * B[6], B[1] * B[6] - B[0] * B[7],
                            B[1] * B[5] - B[2] * B[4], B[2] * B[3] - B[0] * B[5], B[0] * B[4] - B[1] * B[3]};
            vol.push_back(J / 6.0);
            for (int r = 0; r < 3; ++r)
                for (int q = 0; q < 3; ++q) IB.push_back(Cf[q * 3 + r] / J);
        }
        if (h.flow()) {
            for (int v : h.faces) face.push_back(v + vo);
            fvol.insert(fvol.end(), h.fvol.begin(), h.fvol.end());
        }
        if (h.elastic) {
            for (int v : h.faces) mface.push_back(v + vo);
            mem.insert(mem.end(), h.mem.begin(), h.mem.end());
            finst.insert(finst.end(), h.mem.size() / 7, i);
            for (size_t k = 0; k < h.hinges.size(); k += 4)
                hinge.push_back(make_int4(h.hinges[k] + vo, h.hinges[k + 1] + vo, h.hinges[k + 2] + vo,
                                          h.hinges[k + 3] + vo));
            hk.insert(hk.end(), h.hk.begin(), h.hk.end());
            hinst.insert(hinst.end(), h.hinges.size() / 4, i);
        }
        for (size_t k = 0; k < h.nodes.size(); ++k) {
            v2s[h.nodes[k] + vo] = (int)snode.size();
            snode.push_back(h.nodes[k] + vo);
            sn_inst.push_back(i);
        }
        for (size_t k = 0; k < h.edges.size(); ++k) sedge.push_back(h.edges[k] + vo);
        se_inst.insert(se_inst.end(), h.edges.size() / 2, i);
        for (size_t k = 0; k < h.tris.size(); ++k) stri.push_back(h.tris[k] + vo);
        st_inst.insert(st_inst.end(), h.tris.size() / 3, i);
        dHat2.push_back(h.dHat2);
        kappa.push_back(h.kappa);
        thick.push_back(c->P.thickness);
        cell.push_back(h.rest_mean_edge);
        c->st.emplace_back();
        c->st.back().kappa = h.kappa;
        c->st.back().kappa_max = h.kappa_max;
    }
    int rc = IDP_OK;
    std::vector<double> zeros(3 * A.V, 0.0);
    std::vector<int4> tetv(tet);
    rc |= upload(c, A.X, X);
    rc |= upload(c, A.X0, X0);
    rc |= upload(c, A.Xn, X);
    rc |= upload(c, A.Xtilde, X);
    rc |= upload(c, A.Xprev, X);
    rc |= upload(c, A.g, zeros);
    rc |= upload(c, A.dir, zeros);
    rc |= upload(c, A.mass, mass);
    rc |= upload(c, A.dbc, dbc);
    rc |= upload(c, A.dbc_excl, dbc);
    {
        // moving-DBC targets (positions until set) and the per-instance
        // penalty stiffness, kept when some instance has DBC vertices
        bool any_dbc = false;
        std::vector<double> tgt;
        for (int i = 0; i < nI; ++i) any_dbc |= !hv[i]->dbc_list.empty();
        if (any_dbc) {
            tgt = X;
            for (int i = 0; i < nI; ++i)
                if (!hv[i]->dbc_tgt.empty())
                    std::copy(hv[i]->dbc_tgt.begin(), hv[i]->dbc_tgt.end(), tgt.begin() + 3L * A.v_off[i]);
            std::vector<unsigned char> fz(A.V, 0);
            rc |= upload(c, A.dtgt, tgt);
            rc |= upload(c, A.dfix, fz);
        } else {
            A.dtgt = nullptr;
            A.dfix = nullptr;
        }
        std::vector<double> zs(nI, 0.0);
        rc |= upload(c, A.dstiff, zs);
    }
    rc |= upload(c, A.vinst, vinst);
    rc |= upload(c, A.vsrc, vsrc);
    rc |= upload(c, A.tet, tetv);
    rc |= upload(c, A.IB, IB);
    rc |= upload(c, A.vol, vol);
    rc |= upload(c, A.lam, lam);
    rc |= upload(c, A.mu, mu);
    rc |= upload(c, A.snode, snode);
    {
        std::vector<int2> se2(A.Se);
        for (long e = 0; e < A.Se; ++e) se2[e] = make_int2(sedge[2 * e], sedge[2 * e + 1]);
        rc |= upload(c, A.sedge, se2);
    }
    rc |= upload(c, A.stri, stri);
    rc |= upload(c, A.sn_inst, sn_inst);
    rc |= upload(c, A.se_inst, se_inst);
    rc |= upload(c, A.st_inst, st_inst);
    rc |= upload(c, A.v2s, v2s);
    rc |= upload(c, A.dHat2, dHat2);
    rc |= upload(c, A.kappa, kappa);
    rc |= upload(c, A.thickness, thick);
    rc |= upload(c, A.cell, cell);
    std::vector<unsigned char> act(nI, 1);
    rc |= upload(c, A.active, act);
    std::vector<double> alpha(nI, 1.0);
    rc |= upload(c, A.alpha, alpha);
    rc |= upload(c, A.d_v_off, A.v_off);
    // chunk tables
    std::vector<Chunk> tch, vch;
    std::vector<int> tco, vco;
    build_chunks(A.t_off, tch, tco);
    build_chunks(A.v_off, vch, vco);
    A.n_tet_chunks = (int)tch.size();
    A.n_vert_chunks = (int)vch.size();
    rc |= upload(c, A.tet_chunks, tch);
    rc |= upload(c, A.vert_chunks, vch);
    rc |= upload(c, A.tet_chunk_off, tco);
    rc |= upload(c, A.vert_chunk_off, vco);
    // shell faces (flow mode): faces, volumes, chunks, vertex -> face lists
    {
        std::vector<Chunk> fch;
        std::vector<int> fco;
        build_chunks(A.f_off, fch, fco);
        A.n_face_chunks = (int)fch.size();
        rc |= upload(c, A.face, face);
        rc |= upload(c, A.fvol, fvol);
        rc |= upload(c, A.face_chunks, fch);
        rc |= upload(c, A.face_chunk_off, fco);
        std::vector<int> vfp(A.V + 1, 0), vf(face.size());
        for (int v : face) vfp[v + 1]++;
        for (long v = 0; v < A.V; ++v) vfp[v + 1] += vfp[v];
        std::vector<int> fill(vfp.begin(), vfp.end() - 1);
        for (size_t k = 0; k < face.size(); ++k) vf[fill[face[k]]++] = (int)k;  // face * 3 + corner
        rc |= upload(c, A.vert_face_ptr, vfp);
        rc |= upload(c, A.vert_face, vf);
    }
    // elastic shells: membrane faces, hinges, chunks, vertex -> element
    // gradient slots (faces ascending, then hinges ascending)
    {
        std::vector<Chunk> mch, hch;
        std::vector<int> mco, hco;
        build_chunks(A.fm_off, mch, mco);
        build_chunks(A.hn_off, hch, hco);
        A.n_mface_chunks = (int)mch.size();
        A.n_hinge_chunks = (int)hch.size();
        rc |= upload(c, A.mface, mface);
        rc |= upload(c, A.mem, mem);
        rc |= upload(c, A.finst, finst);
        rc |= upload(c, A.mface_chunks, mch);
        rc |= upload(c, A.mface_chunk_off, mco);
        rc |= upload(c, A.hinge, hinge);
        rc |= upload(c, A.hk, hk);
        rc |= upload(c, A.hinst, hinst);
        rc |= upload(c, A.hinge_chunks, hch);
        rc |= upload(c, A.hinge_chunk_off, hco);
        std::vector<int> vsp(A.V + 1, 0);
        for (int v : mface) vsp[v + 1]++;
        for (const int4& q : hinge) {
            vsp[q.x + 1]++; vsp[q.y + 1]++; vsp[q.z + 1]++; vsp[q.w + 1]++;
        }
        for (long v = 0; v < A.V; ++v) vsp[v + 1] += vsp[v];
        std::vector<int> vs(vsp[A.V]), fill(vsp.begin(), vsp.end() - 1);
        for (size_t k = 0; k < mface.size(); ++k) vs[fill[mface[k]]++] = (int)k;  // face * 3 + corner
        for (size_t k = 0; k < hinge.size(); ++k) {
            const int v[4] = {hinge[k].x, hinge[k].y, hinge[k].z, hinge[k].w};
            for (int a = 0; a < 4; ++a) vs[fill[v[a]]++] = (int)(mface.size() + 4 * k + a);
        }
        rc |= upload(c, A.vshell_ptr, vsp);
        rc |= upload(c, A.vshell, vs);
    }
    // BSR pattern of the tet stencil + contributor lists (fixed order)
    {
        // Row by row: the (column, contributor code) entries of a row, in
        // element order (tets ascending with the row's corner against every
        // corner, then flow faces, membrane faces and hinges likewise), are
        // stably sorted by column, so each block lists its contributors in
        // the order a global stable sort of all (row, column) keys gives.
        // Rows are independent: threads take contiguous row ranges.
        const long V = A.V;
        std::vector<long> roff(V + 1, 0);
        for (long t = 0; t < A.T; ++t) {
            roff[tet[t].x + 1] += 4; roff[tet[t].y + 1] += 4; roff[tet[t].z + 1] += 4; roff[tet[t].w + 1] += 4;
        }
        for (long f = 0; f < A.F; ++f)
            for (int a = 0; a < 3; ++a) roff[face[3 * f + a] + 1] += 3;
        for (long f = 0; f < A.Fm; ++f)
            for (int a = 0; a < 3; ++a) roff[mface[3 * f + a] + 1] += 3;
        for (long q = 0; q < A.Hn; ++q) {
            roff[hinge[q].x + 1] += 4; roff[hinge[q].y + 1] += 4; roff[hinge[q].z + 1] += 4; roff[hinge[q].w + 1] += 4;
        }
        for (long v = 0; v < V; ++v) roff[v + 1] += roff[v];
        std::vector<std::pair<int, int>> ent(roff[V]);  // (column, code)
        {
            std::vector<long> fill(roff.begin(), roff.end() - 1);
            for (long t = 0; t < A.T; ++t) {
                const int v[4] = {tet[t].x, tet[t].y, tet[t].z, tet[t].w};
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; b < 4; ++b) {
                        const int lo = std::min(a, b), hi = std::max(a, b);
                        const int k = lo * 4 - lo * (lo - 1) / 2 + (hi - lo);
                        ent[fill[v[a]]++] = {v[b], (int)((t * 10 + k) * 2 + (a > b ? 1 : 0))};
                    }
            }
            // shell faces in flow mode: -(2 f + diagonal) - 1 (INC_POTENTIAL.h:323-339)
            for (long f = 0; f < A.F; ++f)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        ent[fill[face[3 * f + a]]++] = {face[3 * f + b], -(int)(2 * f + (a == b ? 1 : 0)) - 1};
            // elastic-shell element blocks, stored after the tets' 10 per tet:
            // 6 per membrane face, 10 per hinge (upper blocks, a <= b)
            for (long f = 0; f < A.Fm; ++f)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) {
                        const int lo = std::min(a, b), hi = std::max(a, b);
                        const long k = 10 * A.T + 6 * f + lo * 3 - lo * (lo - 1) / 2 + (hi - lo);
                        ent[fill[mface[3 * f + a]]++] = {mface[3 * f + b], (int)(k * 2 + (a > b ? 1 : 0))};
                    }
            for (long q = 0; q < A.Hn; ++q) {
                const int v[4] = {hinge[q].x, hinge[q].y, hinge[q].z, hinge[q].w};
                for (int a = 0; a < 4; ++a)
                    for (int b = 0; b < 4; ++b) {
                        const int lo = std::min(a, b), hi = std::max(a, b);
                        const long k = 10 * A.T + 6 * A.Fm + 10 * q + lo * 4 - lo * (lo - 1) / 2 + (hi - lo);
                        ent[fill[v[a]]++] = {v[b], (int)(k * 2 + (a > b ? 1 : 0))};
                    }
            }
        }
        std::vector<int> nblk(V, 0);
        auto sort_rows = [&](long r0, long r1) {
            for (long r = r0; r < r1; ++r) {
                auto b0 = ent.begin() + roff[r], b1 = ent.begin() + roff[r + 1];
                std::stable_sort(b0, b1, [](const std::pair<int, int>& x, const std::pair<int, int>& y) {
                    return x.first < y.first;
                });
                int n = 0;
                for (auto it = b0; it != b1; ++it)
                    if (it == b0 || it->first != (it - 1)->first) ++n;
                nblk[r] = n;
            }
        };
        {
            const long nth = std::max<long>(1, std::min<long>(std::thread::hardware_concurrency(), V / 4096 + 1));
            std::vector<std::thread> th;
            for (long k = 1; k < nth; ++k) th.emplace_back(sort_rows, V * k / nth, V * (k + 1) / nth);
            sort_rows(0, V / nth);
            for (auto& x : th) x.join();
        }
        std::vector<int> rowptr(V + 1, 0), colidx, brow, src_ptr, src(roff[V]), diag(V, -1);
        for (long v = 0; v < V; ++v) rowptr[v + 1] = nblk[v];
        for (long v = 0; v < V; ++v) rowptr[v + 1] += rowptr[v];
        colidx.resize(rowptr[V]);
        brow.resize(rowptr[V]);
        src_ptr.resize(rowptr[V]);
        for (long r = 0; r < V; ++r) {
            int bk = rowptr[r] - 1;
            for (long e = roff[r]; e < roff[r + 1]; ++e) {
                if (e == roff[r] || ent[e].first != ent[e - 1].first) {
                    ++bk;
                    colidx[bk] = ent[e].first;
                    brow[bk] = (int)r;
                    src_ptr[bk] = (int)e;
                    if (ent[e].first == r) diag[r] = bk;
                }
                src[e] = ent[e].second;
            }
        }
        src_ptr.push_back((int)src.size());
        A.B = (long)colidx.size();
        // vertices without tets still need a diagonal block
        for (long v = 0; v < A.V; ++v)
            if (diag[v] < 0) return IDP_ERR_INVALID_ARG;
        rc |= upload(c, A.rowptr, rowptr);
        A.rowptr_h = rowptr;
        rc |= upload(c, A.colidx, colidx);
        rc |= upload(c, A.brow, brow);
        rc |= upload(c, A.src_ptr, src_ptr);
        rc |= upload(c, A.src, src);
        rc |= upload(c, A.diagblk, diag);
        // vertex -> (tet, corner) lists in tet order
        std::vector<int> vcp(A.V + 1, 0), vc(4 * A.T);
        for (long t = 0; t < A.T; ++t) {
            vcp[tet[t].x + 1]++; vcp[tet[t].y + 1]++; vcp[tet[t].z + 1]++; vcp[tet[t].w + 1]++;
        }
        for (long v = 0; v < A.V; ++v) vcp[v + 1] += vcp[v];
        std::vector<int> fill(vcp.begin(), vcp.end() - 1);
        for (long t = 0; t < A.T; ++t) {
            int v[4] = {tet[t].x, tet[t].y, tet[t].z, tet[t].w};
            for (int a = 0; a < 4; ++a) vc[fill[v[a]]++] = (int)(4 * t + a);
        }
        rc |= upload(c, A.vert_corner_ptr, vcp);
        rc |= upload(c, A.vert_corner, vc);
        // vertex -> incident surface triangles, ascending (normal-flow sums)
        std::vector<int> vtp(A.V + 1, 0), vt(stri.size());
        for (size_t k = 0; k < stri.size(); ++k) vtp[stri[k] + 1]++;
        for (long v = 0; v < A.V; ++v) vtp[v + 1] += vtp[v];
        std::vector<int> vfill(vtp.begin(), vtp.end() - 1);
        for (size_t f = 0; f < stri.size() / 3; ++f)
            for (int a = 0; a < 3; ++a) vt[vfill[stri[3 * f + a]]++] = (int)f;
        rc |= upload(c, A.vtri_ptr, vtp);
        rc |= upload(c, A.vtri, vt);
        // tiles (2048 items each) of the fixed-order estimate of each
        // instance's sum |dir| that decides whether the CCD span cap can apply
        // (toff[2i] = toff[2i+1]: no edge-length tiles, the voxel size is
        // summed in the reference's order by the instance's CTA)
        std::vector<SpanTile> tiles;
        std::vector<int> toff(2 * nI + 1, 0);
        for (int i = 0; i < nI; ++i) {
            const int start = 3 * A.sn_off[i], m = 3 * (A.sn_off[i + 1] - A.sn_off[i]);
            toff[2 * i] = toff[2 * i + 1] = (int)tiles.size();
            for (int k = 0; k * 2048 < m; ++k) tiles.push_back({i, 1, start, m, k});
        }
        toff[2 * nI] = (int)tiles.size();
        A.n_span_tiles = (int)tiles.size();
        rc |= upload(c, A.span_tiles, tiles);
        rc |= upload(c, A.span_tile_off, toff);
        rc |= upload(c, A.d_se_off, A.se_off);
        rc |= upload(c, A.d_sn_off, A.sn_off);
    }
    // algorithmic bytes of one FP32 PCG iteration per instance: BSR values
    // and column ids once, and ~7 vector reads/writes plus the 3x3
    // preconditioner block per vertex (FP64 mode doubles the value bytes)
    {
        std::vector<int> rp(A.V + 1);
        cudaMemcpy(rp.data(), A.rowptr, sizeof(int) * (A.V + 1), cudaMemcpyDeviceToHost);
        c->W.pcg_bytes_per_iter.assign(nI, 0.0);
        for (int i = 0; i < nI; ++i) {
            double Bi = rp[A.v_off[i + 1]] - rp[A.v_off[i]];
            double Vi = A.v_off[i + 1] - A.v_off[i];
            c->W.pcg_bytes_per_iter[i] = Bi * (36 + 4) + Vi * (12 * 7 + 36 + 4);
        }
    }
    if (c->inst_buf.ensure(sizeof(double) * (S_NUMD + S_NUMI) * (nI + 1))) rc = IDP_ERR_CUDA;
    else {
        c->W.tol_inst = dsc(c, S_TOL);
        std::vector<double> tl(nI, c->P.pcg_rel_tol);
        rc |= cudaMemcpy(c->W.tol_inst, tl.data(), sizeof(double) * nI, cudaMemcpyHostToDevice) != cudaSuccess;
    }
    if (c->vel.ensure(sizeof(double) * 3 * (A.V + 1))) rc = IDP_ERR_CUDA;
    else if (cudaMemcpy(c->vel.p, vel.data(), sizeof(double) * 3 * A.V, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = IDP_ERR_CUDA;
    if (rc) return IDP_ERR_CUDA;
    // body-force accelerations (only when some instance has one)
    c->has_bacc = false;
    for (const HostInstance& h : c->inst) c->has_bacc |= !h.bacc.empty();
    if (c->stage.ensure(sizeof(double) * 3 * (A.V + 1))) return IDP_ERR_CUDA;
    if (c->has_bacc) {
        std::vector<double> acc(3 * (size_t)A.V, 0.0);
        for (int i = 0; i < nI; ++i)
            if (!hv[i]->bacc.empty())
                std::copy(hv[i]->bacc.begin(), hv[i]->bacc.end(), acc.begin() + 3L * A.v_off[i]);
        if (c->bacc.ensure(sizeof(double) * 3 * (A.V + 1)) ||
            cudaMemcpy(c->bacc.p, acc.data(), sizeof(double) * 3 * A.V, cudaMemcpyHostToDevice) != cudaSuccess)
            return IDP_ERR_CUDA;
    }
    c->committed = true;
    return IDP_OK;
}

}  // extern "C"

namespace idp {

// milliseconds since t0 (host clock)
static double since_ms(const std::chrono::steady_clock::time_point& t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// collect the phase timers of one call into the step's running stats
static void collect_stats(idp_ctx* c, long long launches0) {
    Work& W = c->W;
    double ms[PhaseTimer::NPHASE], hms[PhaseTimer::NPHASE];
    W.timer.collect(ms, hms);
    if (std::getenv("IDP_PROFILE")) {
        const char* nm[] = {"pcg", "tet", "contact", "ccd", "total", "barrier", "assembly", "linesearch"};
        for (int k = 0; k < PhaseTimer::NPHASE; ++k)
            std::fprintf(stderr, "idp phase %-10s device %10.3f ms  host %10.3f ms\n", nm[k], ms[k], hms[k]);
        std::fprintf(stderr,
                     "idp accd pairs %lld, iterations %lld, longest %lld, pairs over 1000 iterations %lld; "
                     "contact blocks %d (max %d vertices); pcg iterations %lld; fp64 fallbacks %d\n",
                     W.accd_pairs, W.accd_total, W.accd_maxit, W.accd_long, W.cl.n, W.cl.max_n,
                     (long long)W.stats.pcg_iters, W.stats.fp64_fallbacks);
        W.accd_maxit = W.accd_long = W.accd_total = W.accd_pairs = 0;
        if (W.grid_prof[4]) {
            const double n = (double)W.grid_prof[4];
            std::fprintf(stderr, "idp grid pcg per iteration (CTA 0): spmv %.2f us, reduction A %.2f us, update %.2f us, reduction B %.2f us (%llu iterations)\n",
                         W.grid_prof[0] / n / 1e3, W.grid_prof[1] / n / 1e3, W.grid_prof[2] / n / 1e3, W.grid_prof[3] / n / 1e3,
                         W.grid_prof[4]);
            for (auto& v : W.grid_prof) v = 0;
        }
    }
    W.stats.barrier_ms += ms[PhaseTimer::BARRIER];
    W.stats.assembly_ms += ms[PhaseTimer::ASSEMBLY];
    W.stats.pcg_ms += ms[PhaseTimer::PCG];
    W.stats.tet_ms += ms[PhaseTimer::TET];
    W.stats.contact_ms += ms[PhaseTimer::CONTACT];
    W.stats.ccd_ms += ms[PhaseTimer::CCD];
    W.stats.total_ms += ms[PhaseTimer::TOTAL];
    W.stats.kernel_launches += g_launch_count - launches0;
}

// Dirichlet conditions at the start of a step of the instances in `which`
// (IMPLICIT_EULER.h:305-401): a DBC vertex whose target is its position is
// fixed; when some have to move, the CCD step of their displacement (every
// other vertex still) decides: alpha = 1 moves them onto their targets,
// alpha < 1 leaves them where they are and turns the penalty
// stiff/2 sum m |t - x|^2 on with stiff = 1e6, projecting only the fixed
// vertices. The active mask is `which` on return.
int dbc_stage(idp_ctx* c, const std::vector<unsigned char>& which) {
    Arena& A = c->A;
    Work& W = c->W;
    const int nI = A.nI;
    cudaStream_t s = c->s;
    int rc;
    std::vector<unsigned char> tm(nI, 0);
    bool anyt = false;
    for (int i = 0; i < nI; ++i) {
        if (!which[i] || c->inst[i].dbc_list.empty()) continue;
        if ((rc = set_projection(c, i, false))) return rc;  // every DBC vertex, unless the penalty turns on
        if (!c->inst[i].dbc_tgt.empty()) {
            tm[i] = 1;
            anyt = true;
        }
    }
    if (anyt) {
        if ((rc = set_mask(c, tm))) return rc;
        IDP_CUDA_TRY(cudaMemsetAsync(isc(c, SI_KFLAG), 0, sizeof(int) * nI, s));
        if ((rc = dbc_classify(A, A.X, A.dir, isc(c, SI_KFLAG), s))) return rc;
        std::vector<int> mv;
        if ((rc = fetch(c, isc(c, SI_KFLAG), mv))) return rc;
        std::vector<unsigned char> mm(nI, 0);
        bool anym = false;
        for (int i = 0; i < nI; ++i)
            if (tm[i] && mv[i]) {
                mm[i] = 1;
                anym = true;
            }
        if (anym) {
            if ((rc = set_mask(c, mm))) return rc;
            std::vector<double> alpha(nI, 1.0);
            std::vector<int> fl;
            IDP_CUDA_TRY(cudaMemcpyAsync(A.alpha, alpha.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
            W.timer.start(PhaseTimer::CCD, s);
            rc = ccd_stepsize(A, W, A.X, A.dir, A.alpha, isc(c, SI_CCDF), s);
            W.timer.stop(s);
            if (rc) return rc;
            IDP_CUDA_TRY(cudaMemcpyAsync(alpha.data(), A.alpha, sizeof(double) * nI, cudaMemcpyDeviceToHost, s));
            if ((rc = fetch(c, isc(c, SI_CCDF), fl))) return rc;
            std::vector<unsigned char> snap(nI, 0), pen(nI, 0);
            bool anys = false, anyp = false;
            for (int i = 0; i < nI; ++i) {
                if (!mm[i]) continue;
                if (fl[i] & 2) {  // no feasible step for the DBC (the reference exits)
                    c->st[i].status = IDP_ERR_ZERO_STEP;
                    c->st[i].active = false;
                } else if (alpha[i] == 1.0) {
                    snap[i] = 1;
                    anys = true;
                } else {
                    pen[i] = 1;
                    anyp = true;
                    c->st[i].dbc_stiff = 1e6;
                }
            }
            if (anys) {
                if ((rc = set_mask(c, snap))) return rc;
                if ((rc = dbc_snap(A, A.X, s))) return rc;
            }
            if (anyp) {
                if ((rc = upload_dbc_stiff(c))) return rc;
                if ((rc = set_mask(c, pen))) return rc;
                if ((rc = dbc_sums(A, W, A.X, dsc(c, S_EDBC), dsc(c, S_DDBC), s))) return rc;
                std::vector<double> d2;
                if ((rc = fetch(c, dsc(c, S_DDBC), d2))) return rc;
                for (int i = 0; i < nI; ++i)
                    if (pen[i]) {
                        c->st[i].dbc_pen0 = d2[i];
                        if ((rc = set_projection(c, i, true))) return rc;
                    }
            }
        }
    }
    return set_mask(c, which);
}

// Start one implicit-Euler step of the instances in `which` (the others keep
// their state): x^n = x, predictor x_tilde = x + h v (+ h^2 M^-1 b with a body
// force; IMPLICIT_EULER.h:195-216; a flow-mode shell's velocity is zeroed
// first unless a predictor was set for this step, :207-209), and the initial
// constraint set and energy (:418-434). The step's stats start here.
int step_begin(idp_ctx* c, const std::vector<unsigned char>& which) {
    if (!c) return IDP_ERR_INVALID_ARG;
    if (!c->committed) return IDP_ERR_STATE;
    cudaSetDevice(c->P.device);
    Arena& A = c->A;
    Work& W = c->W;
    const int nI = A.nI;
    const double h = c->P.h;
    cudaStream_t s = c->s;
    int rc;
    W.timer.reset();
    W.stats = idp_stats{};
    const long long launches0 = g_launch_count;
    W.timer.start(PhaseTimer::TOTAL, s);
    c->t_begin = std::chrono::steady_clock::now();
    if ((rc = set_mask(c, which))) return rc;
    for (int i = 0; i < nI; ++i) {
        if (!which[i]) continue;
        HostInstance& hi0 = c->inst[i];
        if (hi0.flow() && !hi0.vel_set)
            IDP_CUDA_TRY(cudaMemsetAsync(c->vel.as<double>() + 3L * A.v_off[i], 0, sizeof(double) * 3 * hi0.V, s));
        hi0.vel_set = false;
    }
    if ((rc = vec_copy_masked(A, A.active, A.X, A.Xn, s))) return rc;
    if ((rc = vec_xtilde(A, A.X, c->vel.as<double>(), h, A.Xtilde, s, c->has_bacc ? c->bacc.as<double>() : nullptr)))
        return rc;
    std::vector<InstState>& st = c->st;
    for (int i = 0; i < nI; ++i) {
        if (!which[i]) continue;
        InstState& S = st[i];
        double k = S.kappa, km = S.kappa_max;
        S = InstState();
        S.kappa = k;
        S.kappa_max = km;
        S.active = true;
        S.finalized = false;
        S.min_alpha = 1.0;
    }
    if ((rc = upload_dbc_stiff(c))) return rc;
    std::vector<double> kap(nI);
    for (int i = 0; i < nI; ++i) kap[i] = st[i].kappa;
    IDP_CUDA_TRY(cudaMemcpyAsync(A.kappa, kap.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
    if (A.dtgt && (rc = dbc_stage(c, which))) return rc;
    W.timer.start(PhaseTimer::CONTACT, s);
    rc = build_constraint_set(A, W, A.X, c->cs, s);
    W.timer.stop(s);
    if (rc) return rc;
    std::vector<double> E;
    std::vector<int> bad;
    if ((rc = eval_energy(c, A.X, true, E, bad))) return rc;
    for (int i = 0; i < nI; ++i) {
        if (!which[i]) continue;
        st[i].Eprev = E[i];
        st[i].ncons = c->cs.off[i + 1] - c->cs.off[i];
        if (bad[i] == 1) { st[i].status = IDP_ERR_INVERTED; st[i].active = false; }
        if (bad[i] == 2) { st[i].status = IDP_ERR_NONPOSITIVE_DIST; st[i].active = false; }
    }
    W.timer.stop(s);
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    collect_stats(c, launches0);
    c->stepping = true;
    return IDP_OK;
}

// Rebuild the constraint set and the previous-iterate set at the current
// positions of every iterating instance. After instances were resumed into a
// re-packed arena this restores what the end of their last Newton iteration
// had left: both sets are functions of the positions alone.
int step_prepare_resumed(idp_ctx* c) {
    Arena& A = c->A;
    const int nI = A.nI;
    std::vector<unsigned char> m(nI, 0);
    std::vector<double> kap(nI);
    for (int i = 0; i < nI; ++i) {
        m[i] = c->st[i].active ? 1 : 0;
        kap[i] = c->st[i].kappa;
    }
    int rc;
    IDP_CUDA_TRY(cudaMemcpyAsync(A.kappa, kap.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, c->s));
    if ((rc = set_mask(c, m))) return rc;
    if ((rc = build_constraint_set(A, c->W, A.X, c->cs, c->s))) return rc;
    if ((rc = save_prev_set(c, A.X))) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    c->stepping = true;
    return IDP_OK;
}

// At most max_iters Newton iterations (IMPLICIT_EULER.h:436-876) of every
// instance still iterating. Instances that stop have their velocity
// v = (x - x^n) / h (:882-888) written at the end of the call.
int step_iterate(idp_ctx* c, int max_iters, idp_result* results, int* n_active) {
    if (!c) return IDP_ERR_INVALID_ARG;
    if (!c->committed || !c->stepping) return IDP_ERR_STATE;
    cudaSetDevice(c->P.device);
    Arena& A = c->A;
    Work& W = c->W;
    const int nI = A.nI;
    const double h = c->P.h;
    const bool fp64 = c->P.mode == IDP_MODE_FP64;
    cudaStream_t s = c->s;
    int rc;
    W.timer.reset();
    const long long launches0 = g_launch_count;
    W.timer.start(PhaseTimer::TOTAL, s);
    auto build_cs = [&](const double* Xp) {
        W.timer.start(PhaseTimer::CONTACT, s);
        int r = build_constraint_set(A, W, Xp, c->cs, s);
        W.timer.stop(s);
        return r;
    };
    std::vector<unsigned char> mask(nI, 0);
    std::vector<InstState>& st = c->st;
    std::vector<double> kap(nI);
    for (int i = 0; i < nI; ++i) kap[i] = st[i].kappa;
    std::vector<int> nDBC(nI, 0), nvert(nI);
    for (int i = 0; i < nI; ++i) {
        for (unsigned char d : c->inst[i].dbc) nDBC[i] += d;
        nvert[i] = c->inst[i].V;
    }
    std::vector<double> E;
    std::vector<int> bad;
    std::vector<double> hv;
    std::vector<int> hi;
    for (int round = 0; round < max_iters; ++round) {
        bool any = false;
        for (int i = 0; i < nI; ++i) {
            mask[i] = st[i].active ? 1 : 0;
            any |= st[i].active;
        }
        if (!any) break;
        if ((rc = set_mask(c, mask))) return rc;
        // CCD voxel size at this iterate on the side stream (the CCD of the
        // line search starts from these positions); joined before the PCG
        IDP_CUDA_TRY(cudaEventRecord(c->ev_x, s));
        IDP_CUDA_TRY(cudaStreamWaitEvent(c->s2, c->ev_x, 0));
        if ((rc = ccd_voxel_size(A, W, A.X, c->s2))) return rc;
        IDP_CUDA_TRY(cudaEventRecord(c->ev_vox, c->s2));
        // ---- gradient, Hessian, direction
        if ((rc = eval_gradient(c, A.X))) return rc;
        // inexact Newton: PCG tolerance per instance follows |g| / |g_0|
        // (tight near convergence, where the step-length test is decided)
        if ((rc = vec_dir_norm2(A, W, A.g, dsc(c, S_NORM2), s))) return rc;
        if ((rc = fetch(c, dsc(c, S_NORM2), hv))) return rc;
        std::vector<double> tol(nI, c->P.pcg_rel_tol);
        {
            for (int i = 0; i < nI; ++i) {
                if (!mask[i]) continue;
                double gn = std::sqrt(hv[i]);
                if (st[i].iters == 0 || !(st[i].g0 > 0)) st[i].g0 = gn;
                double eta = st[i].g0 > 0 ? gn / st[i].g0 : 1.0;
                tol[i] = std::max(c->P.pcg_rel_tol, std::min(1e-2, eta));
                // a flow-mode shell may stop after this one step: solve it fully
                if (c->inst[i].flow()) tol[i] = c->P.pcg_rel_tol;
            }
            IDP_CUDA_TRY(cudaMemcpyAsync(W.tol_inst, tol.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
        }
        if ((rc = vec_neg(3 * A.V, A.g, A.g, s))) return rc;  // rhs = -g
        std::vector<unsigned char> newton(nI, 0), gd(nI, 0);
        bool any_newton = false, any_gd = false;
        for (int i = 0; i < nI; ++i) {
            if (!mask[i]) continue;
            if (st[i].use_gd) { gd[i] = 1; any_gd = true; }
            else { newton[i] = 1; any_newton = true; }
        }
        if (any_newton) {
            if ((rc = set_mask(c, newton))) return rc;
            if ((rc = eval_hessian(c, A.X))) return rc;
            std::vector<int> its;
            std::vector<double> rel;
            IDP_CUDA_TRY(cudaStreamWaitEvent(s, c->ev_vox, 0));  // the side stream is idle during the PCG
            if ((rc = pcg_solve(A, W, c->cs, fp64, A.g, A.dir, c->P.pcg_rel_tol, c->P.pcg_max_iters, its, rel, s,
                                 tol.data())))
                return rc;
            for (int i = 0; i < nI; ++i)
                if (newton[i]) st[i].pcg_iters += its[i];
            if (!fp64) {
                // FP64 fallback: instances whose refined mixed direction still
                // misses its tolerance by 10x (stiff contact the FP32 operator
                // cannot resolve) are re-solved with an FP64 Hessian
                std::vector<unsigned char> fb(nI, 0);
                bool any_fb = false;
                for (int i = 0; i < nI; ++i)
                    if (newton[i] && rel[i] > std::max(1e-2, 10.0 * tol[i])) {
                        fb[i] = 1;
                        any_fb = true;
                    }
                if (any_fb) {
                    if ((rc = set_mask(c, fb))) return rc;
                    if ((rc = eval_hessian(c, A.X, true))) return rc;
                    if ((rc = pcg_solve(A, W, c->cs, true, A.g, A.dir, c->P.pcg_rel_tol, c->P.pcg_max_iters, its, rel, s,
                                         tol.data())))
                        return rc;
                    for (int i = 0; i < nI; ++i)
                        if (fb[i]) {
                            st[i].pcg_iters += its[i];
                            W.stats.fp64_fallbacks += 1;
                        }
                }
            }
        }
        if (any_gd) {  // gradient descent direction (IMPLICIT_EULER.h:507-510)
            if ((rc = set_mask(c, gd))) return rc;
            if ((rc = vec_copy_masked(A, A.active, A.g, A.dir, s))) return rc;
        }
        if ((rc = set_mask(c, mask))) return rc;
        // ---- Line_Search (IMPLICIT_EULER.h:9-149)
        IDP_CUDA_TRY(cudaStreamWaitEvent(s, c->ev_vox, 0));
        W.timer.start(PhaseTimer::LINESEARCH, s);
        IDP_CUDA_TRY(cudaMemcpyAsync(A.Xprev, A.X, sizeof(double) * 3 * A.V, cudaMemcpyDeviceToDevice, s));
        std::vector<double> alpha(nI, 1.0);
        // inversion-feasible alpha (halve while any det F <= 0)
        std::vector<unsigned char> srch = mask;
        for (int trial = 0; trial < 80; ++trial) {
            bool anys = false;
            for (int i = 0; i < nI; ++i) anys |= srch[i] != 0;
            if (!anys) break;
            if ((rc = set_mask(c, srch))) return rc;
            IDP_CUDA_TRY(cudaMemcpyAsync(A.alpha, alpha.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
            if ((rc = vec_axpy_trial(A, A.Xprev, A.dir, A.X, s))) return rc;
            IDP_CUDA_TRY(cudaMemsetAsync(isc(c, SI_BAD), 0, sizeof(int) * nI, s));
            if ((rc = tet_energy(A, W, A.X, h * h, dsc(c, S_ETET), isc(c, SI_BAD), s))) return rc;
            if ((rc = fetch(c, isc(c, SI_BAD), hi))) return rc;
            for (int i = 0; i < nI; ++i) {
                if (!srch[i]) continue;
                if (hi[i]) alpha[i] /= 2.0;
                else srch[i] = 0;
            }
        }
        // CCD filter (IMPLICIT_EULER.h:96-100)
        if ((rc = set_mask(c, mask))) return rc;
        IDP_CUDA_TRY(cudaMemcpyAsync(A.alpha, alpha.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
        W.timer.start(PhaseTimer::CCD, s);
        rc = ccd_stepsize(A, W, A.Xprev, A.dir, A.alpha, isc(c, SI_CCDF), s, ccd_voxel_sizes(A, W));
        W.timer.stop(s);
        if (rc) return rc;
        hi.resize(nI);
        IDP_CUDA_TRY(cudaMemcpyAsync(alpha.data(), A.alpha, sizeof(double) * nI, cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaMemcpyAsync(hi.data(), isc(c, SI_CCDF), sizeof(int) * nI, cudaMemcpyDeviceToHost, s));
        IDP_CUDA_TRY(cudaStreamSynchronize(s));
        std::vector<double> feasible = alpha;
        for (int i = 0; i < nI; ++i) {
            if (!mask[i]) continue;
            if (hi[i] & 2) st[i].status = IDP_ERR_ZERO_STEP;
            if ((hi[i] & 1) && st[i].status == IDP_OK) st[i].status = IDP_WARN_ITER_CAP;
        }
        // backtracking until E <= Eprev
        srch = mask;
        std::vector<double> Eacc(nI, 0.0);
        std::vector<int> acc_trial(nI, -1);
        int last_trial = -1;
        for (int trial = 0; trial < 200; ++trial) {
            bool anys = false;
            for (int i = 0; i < nI; ++i) anys |= srch[i] != 0;
            if (!anys) break;
            if ((rc = set_mask(c, srch))) return rc;
            IDP_CUDA_TRY(cudaMemcpyAsync(A.alpha, alpha.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
            if ((rc = vec_axpy_trial(A, A.Xprev, A.dir, A.X, s))) return rc;
            // one pass over every searching instance: validity (det F > 0)
            // and elastic energy, inertia, constraint set, minimum distance
            // and barrier energy; one readback decides. An instance that
            // turns out inverted, or fails the distance safeguard, ignores
            // the values computed past that point.
            IDP_CUDA_TRY(cudaMemsetAsync(isc(c, SI_BAD), 0, sizeof(int) * nI * 2, s));
            IDP_CUDA_TRY(cudaMemsetAsync(dsc(c, S_EBAR), 0, sizeof(double) * nI, s));
            W.timer.start(PhaseTimer::TET, s);
            if ((rc = tet_energy(A, W, A.X, h * h, dsc(c, S_ETET), isc(c, SI_BAD), s))) return rc;
            if ((rc = flow_energy(A, W, A.X, dsc(c, S_ETET), s))) return rc;
            if ((rc = shell_energy(A, W, A.X, h * h, dsc(c, S_ETET), s))) return rc;
            W.timer.stop(s);
            if ((rc = vec_inertia(A, W, A.X, dsc(c, S_EINERT), nullptr, s))) return rc;
            for (int i = 0; i < nI; ++i) st[i].ls_trials += srch[i];
            if ((rc = build_cs(A.X))) return rc;
            last_trial = trial;
            if ((rc = vec_fill(dsc(c, S_MIND), nI, 1e300, s))) return rc;
            if ((rc = constraint_min_dist2(A, W, A.X, W[W_CONS].as<int4>(), W[W_CONS_INST].as<int>(), c->cs.C, nullptr,
                                           dsc(c, S_MIND), s)))
                return rc;
            if ((rc = barrier_energy(A, W, A.X, c->cs, dsc(c, S_EBAR), isc(c, SI_BADB), s))) return rc;
            const bool dpen = dbc_penalty_on(c);
            if (dpen && (rc = dbc_sums(A, W, A.X, dsc(c, S_EDBC), dsc(c, S_DDBC), s))) return rc;
            InstScalars sc;
            if ((rc = fetch_scalars(c, sc))) return rc;
            const double t2 = c->P.thickness * c->P.thickness;
            for (int i = 0; i < nI; ++i) {
                if (!srch[i]) continue;
                if (sc.flag(SI_BAD, i)) {  // inverted: halve (IMPLICIT_EULER.h:106-113)
                    alpha[i] /= 2.0;
                    continue;
                }
                if (c->cs.off[i + 1] > c->cs.off[i] && sc.d(S_MIND, i) - t2 <= 0) {
                    alpha[i] /= 2;  // safe guard backtrack (IMPLICIT_EULER.h:120-129)
                    continue;
                }
                double Ei = sc.d(S_ETET, i) + sc.d(S_EINERT, i) + sc.d(S_EBAR, i);
                if (dpen && st[i].dbc_stiff > 0) Ei += 0.5 * st[i].dbc_stiff * sc.d(S_EDBC, i);
                bool ok = sc.flag(SI_BADB, i) == 0 && std::isfinite(Ei) && !(Ei > st[i].Eprev);
                alpha[i] /= 2.0;
                if (ok) {
                    srch[i] = 0;
                    Eacc[i] = Ei;
                    acc_trial[i] = trial;
                }
            }
        }
        for (int i = 0; i < nI; ++i)
            if (srch[i]) st[i].status = IDP_ERR_ZERO_STEP;  // line search exhausted
        W.timer.stop(s);
        // X holds every instance's accepted trial; rebuild their constraint
        // set unless the last trial's build already covered all of them
        if ((rc = set_mask(c, mask))) return rc;
        bool fresh = last_trial >= 0;
        for (int i = 0; i < nI; ++i)
            if (mask[i] && acc_trial[i] != last_trial) fresh = false;
        if (!fresh && (rc = build_cs(A.X))) return rc;
        // exact intersection check of every accepted iterate (optional)
        if (c->P.verify_iterates) {
            const int2* pairs = nullptr;
            long npairs = 0;
            unsigned int* cnt = reinterpret_cast<unsigned int*>(isc(c, SI_ISECT));
            if ((rc = edge_tri_intersections(A, W, A.X, cnt, &pairs, &npairs, s))) return rc;
            if ((rc = fetch(c, isc(c, SI_ISECT), hi))) return rc;
            for (int i = 0; i < nI; ++i) {
                if (!mask[i]) continue;
                W.stats.verify_checks += 1;
                if (hi[i] != 0) {
                    W.stats.verify_failures += 1;
                    st[i].status = IDP_ERR_INTERSECTION;
                }
            }
        }
        for (int i = 0; i < nI; ++i)
            if (mask[i]) {
                st[i].Eprev = Eacc[i];
                st[i].alpha = alpha[i] * 2;
                st[i].min_alpha = std::min(st[i].min_alpha, alpha[i] * 2);
                st[i].feasible_alpha = feasible[i];
            }
        // ---- kappa adaptation (IMPLICIT_EULER.h:566-595) and the direction
        // norm of the stopping test, read back together
        bool have_prev = false;
        for (int i = 0; i < nI; ++i) have_prev |= mask[i] && st[i].have_prev;
        IDP_CUDA_TRY(cudaMemsetAsync(isc(c, SI_KFLAG), 0, sizeof(int) * nI, s));
        if (have_prev && c->prevC > 0)
            if ((rc = kappa_check(A, W, A.X, W[W_PREV_CONS].as<int4>(), W[W_PREV_INST].as<int>(),
                                  W[W_PREV_DIST2].as<double>(), c->prevC, isc(c, SI_KFLAG), s)))
                return rc;
        if ((rc = vec_dir_norm2(A, W, A.dir, dsc(c, S_NORM2), s))) return rc;
        if (dbc_penalty_on(c) && (rc = dbc_sums(A, W, A.X, dsc(c, S_EDBC), dsc(c, S_DDBC), s))) return rc;
        InstScalars ksc;
        if ((rc = fetch_scalars(c, ksc))) return rc;
        if (have_prev && c->prevC > 0) {
            std::vector<unsigned char> km(nI, 0);
            bool anyk = false;
            for (int i = 0; i < nI; ++i)
                if (mask[i] && st[i].have_prev && ksc.flag(SI_KFLAG, i) && st[i].kappa < st[i].kappa_max) {
                    st[i].kappa *= 2;
                    km[i] = 1;
                    anyk = true;
                }
            if (anyk) {
                for (int i = 0; i < nI; ++i) kap[i] = st[i].kappa;
                IDP_CUDA_TRY(cudaMemcpyAsync(A.kappa, kap.data(), sizeof(double) * nI, cudaMemcpyHostToDevice, s));
                if ((rc = set_mask(c, km))) return rc;
                if ((rc = eval_energy(c, A.X, true, E, bad))) return rc;
                for (int i = 0; i < nI; ++i)
                    if (km[i]) st[i].Eprev = E[i];
                if ((rc = set_mask(c, mask))) return rc;
            }
        }
        if ((rc = save_prev_set(c, A.X))) return rc;
        for (int i = 0; i < nI; ++i)
            if (mask[i]) st[i].have_prev = true;
        // ---- stopping criterion (IMPLICIT_EULER.h:647-676, 759, 855)
        std::vector<unsigned char> dbc_new(nI, 0);
        bool any_dbc_new = false;
        for (int i = 0; i < nI; ++i) {
            if (!mask[i]) continue;
            InstState& S = st[i];
            double L2 = std::sqrt(ksc.d(S_NORM2, i) / (nvert[i] - nDBC[i])) / h;
            S.ncons = c->cs.off[i + 1] - c->cs.off[i];
            S.iters += 1;
            S.last_res = L2;
            if (S.nres < 3) S.res[S.nres++] = L2;
            else { S.res[0] = S.res[1]; S.res[1] = S.res[2]; S.res[2] = L2; }
            double L2m = *std::max_element(S.res, S.res + S.nres);
            if (S.use_gd) L2m = c->P.newton_tol * 10;
            // switch to gradient descent after a vanishing step (IMPLICIT_EULER.h:682-699)
            S.use_gd = (S.alpha < 1e-8 && S.feasible_alpha > 1e-8);
            if (S.dbc_stiff > 0) {
                // moving DBC (IMPLICIT_EULER.h:701-757): until the DBC vertices
                // have covered 99 % of their way, keep iterating and double the
                // penalty whenever the solve has settled; then drop it and
                // project every DBC vertex where it is
                const double progress = 1 - std::sqrt(ksc.d(S_DDBC, i) / S.dbc_pen0);
                if (progress < 0.99) {
                    if (L2m < c->P.newton_tol * 10 && S.dbc_stiff < 1e8) {
                        S.dbc_stiff *= 2;
                        dbc_new[i] = 1;
                        any_dbc_new = true;
                    }
                    L2m = c->P.newton_tol * 10;
                } else {
                    S.dbc_stiff = 0;
                    dbc_new[i] = 1;
                    any_dbc_new = true;
                    if ((rc = set_projection(c, i, false))) return rc;
                }
            }
            if (S.status == IDP_ERR_ZERO_STEP || S.status == IDP_ERR_NONPOSITIVE_DIST ||
                S.status == IDP_ERR_INTERSECTION)
                S.active = false;
            else if (S.nres == 3 && L2m <= c->P.newton_tol) S.active = false;
            else if (S.iters >= c->P.max_newton) {
                S.active = false;
                S.status = IDP_ERR_NOT_CONVERGED;
            } else if (c->inst[i].flow() && c->cs.off[i + 1] == c->cs.off[i]) {
                S.active = false;  // flow mode without contacts: one Newton step (IMPLICIT_EULER.h:850-854)
            }
            if (!S.active) S.latency_ms = since_ms(c->t_begin);
        }
        if (any_dbc_new) {  // the energy with the new penalty (IMPLICIT_EULER.h:726-755)
            if ((rc = upload_dbc_stiff(c))) return rc;
            if ((rc = set_mask(c, dbc_new))) return rc;
            if ((rc = eval_energy(c, A.X, true, E, bad))) return rc;
            for (int i = 0; i < nI; ++i)
                if (dbc_new[i]) st[i].Eprev = E[i];
        }
    }
    // instances that stopped (in this call, or already at the step's begin):
    // velocity v = (x - x^n) / h (IMPLICIT_EULER.h:882-888)
    std::vector<unsigned char> fin(nI, 0);
    bool any_fin = false;
    int left = 0;
    for (int i = 0; i < nI; ++i) {
        if (st[i].active) {
            ++left;
            continue;
        }
        if (!st[i].finalized) {
            fin[i] = 1;
            any_fin = true;
            st[i].finalized = true;
            if (!(st[i].latency_ms > 0)) st[i].latency_ms = since_ms(c->t_begin);
        }
    }
    if (any_fin) {
        if ((rc = set_mask(c, fin))) return rc;
        if ((rc = vec_velocity(A, A.X, A.Xn, h, c->vel.as<double>(), s))) return rc;
        bool drop = false;
        for (int i = 0; i < nI; ++i)
            if (fin[i] && st[i].dbc_stiff > 0) {  // a step cut short by the iteration cap
                st[i].dbc_stiff = 0;
                drop = true;
                if ((rc = set_projection(c, i, false))) return rc;
            }
        if (drop && (rc = upload_dbc_stiff(c))) return rc;
    }
    W.timer.stop(s);
    IDP_CUDA_TRY(cudaStreamSynchronize(s));
    collect_stats(c, launches0);
    if (left == 0) c->stepping = false;
    if (n_active) *n_active = left;
    int worst = IDP_OK;
    for (int i = 0; i < nI; ++i) {
        if (results) {
            idp_result& r = results[i];
            r.status = st[i].status;
            r.newton_iters = st[i].iters;
            r.pcg_iters = st[i].pcg_iters;
            r.ls_trials = st[i].ls_trials;
            r.num_constraints = st[i].ncons;
            r.energy = st[i].Eprev;
            r.kappa = st[i].kappa;
            r.residual = st[i].last_res;
            r.min_alpha = st[i].min_alpha;
            r.latency_ms = st[i].active ? since_ms(c->t_begin) : st[i].latency_ms;
        }
        if (!st[i].active && st[i].status != IDP_OK && st[i].status != IDP_WARN_ITER_CAP && worst == IDP_OK)
            worst = st[i].status;
    }
    return worst;
}

int add_prebuilt(idp_ctx* c, const HostInstance& h) {
    if (!c) return -IDP_ERR_INVALID_ARG;
    if (c->committed) return -IDP_ERR_STATE;
    c->inst.push_back(h);
    return (int)c->inst.size() - 1;
}

const HostInstance* instance_host(idp_ctx* c, int i) {
    if (!c || i < 0 || i >= (int)c->inst.size()) return nullptr;
    return &c->inst[i];
}

int snapshot_instance(idp_ctx* c, int i, InstSnapshot& out) {
    if (!c || !c->committed || i < 0 || i >= c->A.nI) return IDP_ERR_INVALID_ARG;
    if (c->st[i].dbc_stiff > 0) return IDP_ERR_STATE;  // the penalty's projection is not carried over
    const long o = 3L * c->A.v_off[i], n = 3L * c->inst[i].V;
    out.st = c->st[i];
    out.X.resize(n);
    out.Xn.resize(n);
    out.Xt.resize(n);
    IDP_CUDA_TRY(cudaMemcpyAsync(out.X.data(), c->A.X + o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(out.Xn.data(), c->A.Xn + o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(out.Xt.data(), c->A.Xtilde + o, sizeof(double) * n, cudaMemcpyDeviceToHost, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

bool instance_active(idp_ctx* c, int i) {
    return c && i >= 0 && i < (int)c->st.size() && c->st[i].active;
}

int resume_instance(idp_ctx* c, int i, const InstSnapshot& in) {
    if (!c || !c->committed || i < 0 || i >= c->A.nI) return IDP_ERR_INVALID_ARG;
    const long o = 3L * c->A.v_off[i], n = 3L * c->inst[i].V;
    if ((long)in.X.size() != n || (long)in.Xn.size() != n || (long)in.Xt.size() != n) return IDP_ERR_INVALID_ARG;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.X + o, in.X.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.Xn + o, in.Xn.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.Xtilde + o, in.Xt.data(), sizeof(double) * n, cudaMemcpyHostToDevice, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    c->st[i] = in.st;
    return IDP_OK;
}

}  // namespace idp

extern "C" {

int idp_step_begin(idp_ctx* c) {
    if (!c) return IDP_ERR_INVALID_ARG;
    return idp::step_begin(c, std::vector<unsigned char>(c->A.nI, 1));
}

int idp_step_iterate(idp_ctx* c, int max_iters, idp_result* results, int* n_active) {
    if (max_iters < 0) return IDP_ERR_INVALID_ARG;
    return idp::step_iterate(c, max_iters, results, n_active);
}

int idp_advance(idp_ctx* c, idp_result* results) {
    int rc = idp_step_begin(c);
    if (rc) return rc;
    // the stats of idp_advance cover its begin and every Newton iteration
    return idp::step_iterate(c, INT_MAX, results, nullptr);
}

int idp_save_state(idp_ctx* c) {
    if (!c || !c->committed) return IDP_ERR_STATE;
    long n = 3L * c->A.V;
    if (c->snap.ensure(sizeof(double) * 2 * (n + 1))) return IDP_ERR_CUDA;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->snap.as<double>(), c->A.X, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(c->snap.as<double>() + n, c->vel.as<double>(), sizeof(double) * n,
                                 cudaMemcpyDeviceToDevice, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    c->snap_kappa.clear();
    for (auto& S : c->st) c->snap_kappa.push_back(S.kappa);
    c->has_snap = true;
    return IDP_OK;
}

int idp_restore_state(idp_ctx* c) {
    if (!c || !c->committed || !c->has_snap) return IDP_ERR_STATE;
    long n = 3L * c->A.V;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.X, c->snap.as<double>(), sizeof(double) * n, cudaMemcpyDeviceToDevice, c->s));
    IDP_CUDA_TRY(cudaMemcpyAsync(c->vel.as<double>(), c->snap.as<double>() + n, sizeof(double) * n,
                                 cudaMemcpyDeviceToDevice, c->s));
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    for (size_t i = 0; i < c->st.size(); ++i) c->st[i].kappa = c->snap_kappa[i];
    return IDP_OK;
}

int idp_get_stats(idp_ctx* c, idp_stats* out) {
    if (!c || !out) return IDP_ERR_INVALID_ARG;
    *out = c->W.stats;
    return IDP_OK;
}

int idp_get_state(idp_ctx* c, int i, double* X, double* v, double* kappa3) {
    if (!c || i < 0 || i >= (int)c->inst.size()) return IDP_ERR_INVALID_ARG;
    if (!c->committed) {
        const HostInstance& h = c->inst[i];
        if (X) std::memcpy(X, h.X.data(), sizeof(double) * 3 * h.V);
        if (v) std::memcpy(v, h.v.data(), sizeof(double) * 3 * h.V);
        if (kappa3) { kappa3[0] = h.kappa; kappa3[1] = h.kappa_max; kappa3[2] = 0; }
        return IDP_OK;
    }
    int rc;
    if (X) {
        if ((rc = download3(c, i, c->A.X, X))) return rc;
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));  // the staging buffer is reused below
    }
    if (v && (rc = download3(c, i, c->vel.as<double>(), v))) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    if (kappa3) {
        kappa3[0] = c->st[i].kappa;
        kappa3[1] = c->st[i].kappa_max;
        kappa3[2] = 0;
    }
    return IDP_OK;
}

int idp_set_kappa(idp_ctx* c, int i, const double* kappa3) {
    if (!c || i < 0 || i >= (int)c->inst.size() || !kappa3) return IDP_ERR_INVALID_ARG;
    if (!(kappa3[0] > 0) || !(kappa3[1] >= kappa3[0])) return IDP_ERR_INVALID_ARG;
    c->inst[i].kappa = kappa3[0];
    c->inst[i].kappa_max = kappa3[1];
    if (c->committed) {
        c->st[i].kappa = kappa3[0];
        c->st[i].kappa_max = kappa3[1];
    }
    return IDP_OK;
}

int idp_instance_info(idp_ctx* c, int i, int* V, int* T, int* nn, int* ne, int* nt) {
    if (!c) return IDP_ERR_INVALID_ARG;
    if (i < 0) {
        if (V) *V = (int)c->inst.size();
        return IDP_OK;
    }
    if (i >= (int)c->inst.size()) return IDP_ERR_INVALID_ARG;
    const HostInstance& h = c->inst[i];
    if (V) *V = h.V;
    if (T) *T = h.T;
    if (nn) *nn = (int)h.nodes.size();
    if (ne) *ne = (int)h.edges.size() / 2;
    if (nt) *nt = (int)h.tris.size() / 3;
    return IDP_OK;
}

int idp_get_surface(idp_ctx* c, int i, int32_t* nodes, int32_t* edges, int32_t* tris) {
    if (!c || i < 0 || i >= (int)c->inst.size()) return IDP_ERR_INVALID_ARG;
    const HostInstance& h = c->inst[i];
    if (nodes) std::copy(h.nodes.begin(), h.nodes.end(), nodes);
    if (edges) std::copy(h.edges.begin(), h.edges.end(), edges);
    if (tris) std::copy(h.tris.begin(), h.tris.end(), tris);
    return IDP_OK;
}

// ---- sub-steps on one instance at caller positions (scratch: A.Xprev)
static int prep_one(idp_ctx* c, int i, const double* X) {
    if (!c || !c->committed) return IDP_ERR_STATE;
    if (i < 0 || i >= c->A.nI || !X) return IDP_ERR_INVALID_ARG;
    cudaSetDevice(c->P.device);
    std::vector<unsigned char> m(c->A.nI, 0);
    m[i] = 1;
    int rc = set_mask(c, m);
    if (rc) return rc;
    if ((rc = upload3(c, i, X, c->A.Xprev))) return rc;
    // x_tilde from the instance's current positions and velocity
    rc = vec_xtilde(c->A, c->A.X, c->vel.as<double>(), c->P.h, c->A.Xtilde, c->s,
                    c->has_bacc ? c->bacc.as<double>() : nullptr);
    if (rc) return rc;
    std::vector<double> kap(c->A.nI);
    for (int k = 0; k < c->A.nI; ++k) kap[k] = c->st[k].kappa;
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.kappa, kap.data(), sizeof(double) * c->A.nI, cudaMemcpyHostToDevice, c->s));
    return IDP_OK;
}

int idp_eval_energy(idp_ctx* c, int i, const double* X, double* Ee, double* Ei, double* Eb) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if ((rc = build_constraint_set(c->A, c->W, c->A.Xprev, c->cs, c->s))) return rc;
    std::vector<double> E;
    std::vector<int> bad;
    if ((rc = eval_energy(c, c->A.Xprev, true, E, bad))) return rc;
    std::vector<double> et, ei, eb;
    fetch(c, dsc(c, S_ETET), et);
    fetch(c, dsc(c, S_EINERT), ei);
    fetch(c, dsc(c, S_EBAR), eb);
    if (Ee) *Ee = et[i];
    if (Ei) *Ei = ei[i];
    if (Eb) *Eb = eb[i];
    if (bad[i] == 1) return IDP_ERR_INVERTED;
    if (bad[i] == 2) return IDP_ERR_NONPOSITIVE_DIST;
    return IDP_OK;
}

int idp_eval_gradient(idp_ctx* c, int i, const double* X, double* g) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if ((rc = build_constraint_set(c->A, c->W, c->A.Xprev, c->cs, c->s))) return rc;
    if ((rc = eval_gradient(c, c->A.Xprev))) return rc;
    if ((rc = download3(c, i, c->A.g, g))) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

int idp_constraint_set(idp_ctx* c, int i, const double* X, int cap, int32_t* cons, int* count) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if ((rc = build_constraint_set(c->A, c->W, c->A.Xprev, c->cs, c->s))) return rc;
    int n = c->cs.off[i + 1] - c->cs.off[i];
    if (count) *count = n;
    if (n > cap) return IDP_ERR_CAPACITY;
    if (n > 0 && cons) {
        IDP_CUDA_TRY(cudaMemcpyAsync(cons, c->W[W_CONS].as<int4>() + c->cs.off[i], sizeof(int4) * n,
                                     cudaMemcpyDeviceToHost, c->s));
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
        // device ids are arena-global; return instance-local ids, keeping the
        // sign tags (-v-1), the -1 markers and the -count multiplicity slot
        // (and the caller's vertex numbering)
        int vo = c->A.v_off[i];
        const std::vector<int>& pm = c->inst[i].perm;
        auto loc = [&pm](int k) { return pm.empty() ? k : pm[k]; };
        auto pos = [vo, &loc](int v) { return loc(v - vo); };
        auto tag = [vo, &loc](int v) { return -loc((-v - 1) - vo) - 1; };
        for (int k = 0; k < n; ++k) {
            int* q = cons + 4 * k;
            if (q[0] >= 0) {  // edge-edge family: every negative entry is a tagged vertex
                for (int j = 0; j < 4; ++j) q[j] = q[j] >= 0 ? pos(q[j]) : tag(q[j]);
            } else {
                q[0] = tag(q[0]);
                q[1] = pos(q[1]);
                if (q[3] >= 0) { q[2] = pos(q[2]); q[3] = pos(q[3]); }
                else if (q[2] >= 0) q[2] = pos(q[2]);
            }
        }
    }
    return IDP_OK;
}

int idp_check_intersection(idp_ctx* c, int i, const double* X, int cap, int32_t* pairs, int* count) {
    if (!c || !c->committed) return IDP_ERR_STATE;
    if (i < 0 || i >= c->A.nI || cap < 0) return IDP_ERR_INVALID_ARG;
    int rc;
    const double* Xp = c->A.X;
    if (X) {
        if ((rc = prep_one(c, i, X))) return rc;
        Xp = c->A.Xprev;
    } else {
        cudaSetDevice(c->P.device);
        std::vector<unsigned char> m(c->A.nI, 0);
        m[i] = 1;
        if ((rc = set_mask(c, m))) return rc;
    }
    const int2* dp = nullptr;
    long n = 0;
    if ((rc = edge_tri_intersections(c->A, c->W, Xp, reinterpret_cast<unsigned int*>(isc(c, SI_ISECT)), &dp, &n,
                                     c->s)))
        return rc;
    if (count) *count = (int)n;
    if (n > cap) return IDP_ERR_CAPACITY;
    if (n > 0 && pairs) {
        std::vector<int32_t> h(2 * n);
        IDP_CUDA_TRY(cudaMemcpyAsync(h.data(), dp, sizeof(int2) * n, cudaMemcpyDeviceToHost, c->s));
        IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
        const int t0 = c->A.st_off[i], e0 = c->A.se_off[i];
        std::vector<std::pair<int, int>> v(n);
        for (long k = 0; k < n; ++k) v[k] = {h[2 * k] - t0, h[2 * k + 1] - e0};
        std::sort(v.begin(), v.end());
        for (long k = 0; k < n; ++k) {
            pairs[2 * k] = v[k].first;
            pairs[2 * k + 1] = v[k].second;
        }
    }
    return IDP_OK;
}

int idp_check_intersection_all(idp_ctx* c, int32_t* counts) {
    if (!c || !c->committed) return IDP_ERR_STATE;
    if (!counts) return IDP_ERR_INVALID_ARG;
    cudaSetDevice(c->P.device);
    int rc;
    std::vector<unsigned char> m(c->A.nI, 1);
    if ((rc = set_mask(c, m))) return rc;
    const int2* dp = nullptr;
    long n = 0;
    if ((rc = edge_tri_intersections(c->A, c->W, c->A.X, reinterpret_cast<unsigned int*>(isc(c, SI_ISECT)), &dp, &n,
                                     c->s)))
        return rc;
    std::vector<int> h;
    if ((rc = fetch(c, isc(c, SI_ISECT), h))) return rc;
    std::copy(h.begin(), h.end(), counts);
    return IDP_OK;
}

int idp_ccd_stepsize(idp_ctx* c, int i, const double* X, const double* dir, double* alpha) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if (!dir || !alpha) return IDP_ERR_INVALID_ARG;
    if ((rc = upload3(c, i, dir, c->A.dir))) return rc;
    std::vector<double> a(c->A.nI, *alpha);
    IDP_CUDA_TRY(cudaMemcpyAsync(c->A.alpha, a.data(), sizeof(double) * c->A.nI, cudaMemcpyHostToDevice, c->s));
    if ((rc = ccd_stepsize(c->A, c->W, c->A.Xprev, c->A.dir, c->A.alpha, isc(c, SI_CCDF), c->s))) return rc;
    std::vector<int> fl;
    fetch(c, c->A.alpha, a);
    fetch(c, isc(c, SI_CCDF), fl);
    *alpha = a[i];
    if (fl[i] & 2) return IDP_ERR_ZERO_STEP;
    if (fl[i] & 1) return IDP_WARN_ITER_CAP;
    return IDP_OK;
}

int idp_hessian_apply(idp_ctx* c, int i, const double* X, const double* x, double* y) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if ((rc = build_constraint_set(c->A, c->W, c->A.Xprev, c->cs, c->s))) return rc;
    if ((rc = eval_hessian(c, c->A.Xprev))) return rc;
    IDP_CUDA_TRY(cudaMemsetAsync(c->A.dir, 0, sizeof(double) * 3 * c->A.V, c->s));
    if ((rc = upload3(c, i, x, c->A.dir))) return rc;
    if ((rc = hessian_apply(c->A, c->W, c->P.mode == IDP_MODE_FP64, c->A.dir, c->A.g, c->s))) return rc;
    if ((rc = download3(c, i, c->A.g, y))) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    return IDP_OK;
}

int idp_newton_direction(idp_ctx* c, int i, const double* X, double* p, int* iters, double* relres) {
    int rc = prep_one(c, i, X);
    if (rc) return rc;
    if ((rc = build_constraint_set(c->A, c->W, c->A.Xprev, c->cs, c->s))) return rc;
    if ((rc = eval_gradient(c, c->A.Xprev))) return rc;
    if ((rc = vec_neg(3 * c->A.V, c->A.g, c->A.g, c->s))) return rc;
    if ((rc = eval_hessian(c, c->A.Xprev))) return rc;
    std::vector<int> its;
    std::vector<double> rel;
    if ((rc = pcg_solve(c->A, c->W, c->cs, c->P.mode == IDP_MODE_FP64, c->A.g, c->A.dir, c->P.pcg_rel_tol,
                        c->P.pcg_max_iters, its, rel, c->s)))
        return rc;
    if ((rc = download3(c, i, c->A.dir, p))) return rc;
    IDP_CUDA_TRY(cudaStreamSynchronize(c->s));
    if (iters) *iters = its[i];
    if (relres) *relres = rel[i];
    return IDP_OK;
}

}  // extern "C"
