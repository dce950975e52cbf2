// Device arena and per-module launchers of the GB300 injective-deformation
// engine. One arena holds every instance (mesh) of a context: vertices, tets
// and surface primitives of all instances are concatenated with per-instance
// offsets, so one launch serves the whole batch.
#pragma once
#include <vector>
#include <string>
#include <chrono>
#include "common.cuh"
#include "../../include/idp_gb300.h"

namespace idp {

// growable device buffer (grown only between solves, never under capture)
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    int ensure(size_t n);
    void release();
    template <class T>
    T* as() const { return reinterpret_cast<T*>(p); }
};

// per-instance host description, filled by idp_add_instance
struct HostInstance {
    int V = 0, T = 0;
    std::vector<double> X, X0, mass, lam, mu, v, xtilde;
    std::vector<int> tets;      // 4T, local ids
    std::vector<unsigned char> dbc;
    std::vector<int> dbc_list;      // DBC vertices in the order given (the reference's DBC rows)
    std::vector<double> dbc_tgt;    // 3V target positions of the DBC vertices (empty: all fixed)
    bool has_xtilde = false;
    double dHat2 = 0, kappa = 0, kappa_max = 0;
    // surface in reference order (local ids)
    std::vector<int> tris, edges, nodes;
    double rest_mean_edge = 0;
    // triangle shell advanced in flow mode (no tets): faces double as the
    // elements of the flow energy, fvol = area * thickness per face
    bool shell = false;
    std::vector<int> faces;
    std::vector<double> fvol;
    bool vel_set = false;  // predictor velocity given since the last advance
    std::vector<double> bacc;  // body-force acceleration M^-1 b (3V; empty = none)
    // elastic shell (the Hinge path's membrane + hinge bending) instead of
    // flow mode: per face (IB^-1 00, 01, 11, det IB^-1, vol, lam, mu); per
    // hinge its stencil (x0, x1, x2, x3) and (thetabar, k ebar / hbar)
    bool elastic = false;
    std::vector<double> mem;
    std::vector<int> hinges;
    std::vector<double> hk;
    bool flow() const { return shell && !elastic; }
    // device order: internal local index -> caller's local index (set at
    // commit; empty = the caller's order)
    std::vector<int> perm;
};

// per-instance Newton state kept on the host
struct InstState {
    bool active = false;       // still iterating
    bool searching = false;    // inside line search, trial not accepted yet
    bool use_gd = false;
    double Eprev = 0, alpha = 1, feasible_alpha = 1;
    double res[3] = {0, 0, 0};
    int nres = 0;
    int iters = 0, pcg_iters = 0, ls_trials = 0, status = 0;
    double last_res = 0;
    double kappa = 0, kappa_max = 0;
    double min_alpha = 1;
    double g0 = 0;             // gradient norm at the first Newton iteration
    bool have_prev = false;    // a previous iterate's constraint set exists (kappa test)
    bool finalized = true;     // stopped and its velocity written
    double dbc_stiff = 0;      // penalty stiffness of moving DBC (0: off, IMPLICIT_EULER.h:384-401)
    double dbc_pen0 = 0;       // sum |target - x^n|^2 over the DBC rows at the step's start
    double latency_ms = 0;     // host time from the step's begin until it stopped
    int ncons = 0;             // constraint-set size at its latest iterate
};

// one 2048-item tile of the fixed-order estimate of an instance's sum |dir|
// (the CCD span-cap test)
struct SpanTile {
    int inst;
    int kind;   // 1: |dir| components (the only kind built)
    int start;  // segment start in its array
    int m;      // segment length
    int k;      // tile index inside the segment
};

struct Arena {
    int nI = 0;
    long V = 0, T = 0, Sn = 0, Se = 0, St = 0;
    std::vector<int> v_off, t_off, sn_off, se_off, st_off;  // host, size nI+1

    // ---- device, per vertex (3V doubles unless noted)
    double *X = nullptr, *X0 = nullptr, *Xn = nullptr, *Xtilde = nullptr, *Xprev = nullptr, *mass = nullptr;
    double *g = nullptr, *dir = nullptr;          // gradient, Newton direction (3V)
    unsigned char* dbc = nullptr;                 // V: rows projected to the identity (Project_DBC)
    unsigned char* dbc_excl = nullptr;            // V: every DBC vertex (exclusions, skipped elements)
    double* dtgt = nullptr;                       // 3V DBC targets, when some instance has them
    unsigned char* dfix = nullptr;                // V: DBC vertex already at its target (step start)
    double* dstiff = nullptr;                     // nI: moving-DBC penalty stiffness (0: off)
    int* vinst = nullptr;                         // V
    int* vsrc = nullptr;                          // V: caller-order arena index of each device vertex
    // ---- per tet
    int4* tet = nullptr;
    double *IB = nullptr, *vol = nullptr, *lam = nullptr, *mu = nullptr;
    // ---- surface primitives (global vertex ids)
    int* snode = nullptr;
    int2* sedge = nullptr;
    int* stri = nullptr;                          // 3 St
    int *sn_inst = nullptr, *se_inst = nullptr, *st_inst = nullptr;
    // ---- per instance
    double *dHat2 = nullptr, *kappa = nullptr, *thickness = nullptr, *cell = nullptr;
    unsigned char* active = nullptr;              // nI: instance participates in this launch
    double* alpha = nullptr;                      // nI: current step per instance
    int* d_v_off = nullptr;
    // ---- chunk tables
    Chunk* tet_chunks = nullptr;
    int n_tet_chunks = 0;
    Chunk* vert_chunks = nullptr;
    int n_vert_chunks = 0;
    Chunk* node_chunks = nullptr;
    int n_node_chunks = 0;
    Chunk* edge_chunks = nullptr;
    int n_edge_chunks = 0;
    // ---- BSR pattern of the tet stencil (3x3 blocks)
    long B = 0;
    int *rowptr = nullptr, *colidx = nullptr, *diagblk = nullptr;
    std::vector<int> rowptr_h;                    // host copy of rowptr
    int *src_ptr = nullptr, *src = nullptr;       // per BSR block: contributing (tet*10+k)*2+transposed
    int* d_se_off = nullptr;                      // device copies of se_off / sn_off
    int* d_sn_off = nullptr;
    SpanTile* span_tiles = nullptr;               // CCD span-sum tiles, instance by instance
    int* span_tile_off = nullptr;                 // 2 nI + 1: first edge tile, first |dir| tile per instance
    int n_span_tiles = 0;
    int* vtri_ptr = nullptr;                      // per vertex: incident surface triangles, ascending
    int* vtri = nullptr;
    int* vert_corner_ptr = nullptr;               // per vertex: list of tet*4+corner
    int* vert_corner = nullptr;
    int* brow = nullptr;                          // row (vertex) of every BSR block
    int *tet_chunk_off = nullptr, *vert_chunk_off = nullptr;  // nI+1 chunk ranges
    int* v2s = nullptr;                           // vertex -> surface node (or -1)
    // ---- triangle shells in flow mode (faces are elements; global vertex ids)
    long F = 0;
    std::vector<int> f_off;                       // host, nI+1
    int* face = nullptr;                          // 3F
    double* fvol = nullptr;                       // F: area * thickness
    Chunk* face_chunks = nullptr;
    int n_face_chunks = 0;
    int* face_chunk_off = nullptr;                // nI+1
    int* vert_face_ptr = nullptr;                 // per vertex: list of face*3+corner, ascending
    int* vert_face = nullptr;
    double h = 0.1;                               // time step (flow Hessian coefficient)
    // ---- elastic shells: membrane faces and hinges (global vertex ids)
    long Fm = 0, Hn = 0;
    std::vector<int> fm_off, hn_off;              // host, nI+1
    int* mface = nullptr;                         // 3 Fm
    double* mem = nullptr;                        // 7 Fm: IB^-1 (00, 01, 11), det IB^-1, vol, lam, mu
    int* finst = nullptr;                         // Fm: instance of each face
    Chunk* mface_chunks = nullptr;
    int n_mface_chunks = 0;
    int* mface_chunk_off = nullptr;               // nI+1
    int4* hinge = nullptr;                        // Hn: (x0, x1, x2, x3)
    double* hk = nullptr;                         // 2 Hn: thetabar, k ebar / hbar
    int* hinst = nullptr;                         // Hn
    Chunk* hinge_chunks = nullptr;
    int n_hinge_chunks = 0;
    int* hinge_chunk_off = nullptr;               // nI+1
    int* vshell_ptr = nullptr;                    // per vertex: element gradient slots (3 doubles each)
    int* vshell = nullptr;
};

// In-flight state of one instance in the middle of a step, enough to resume
// its Newton loop in another arena (the request server re-packs a worker's
// arena when new jobs join): positions, step-start positions, predictor and
// the host-side Newton state. The constraint sets are rebuilt from X.
struct InstSnapshot {
    InstState st;
    std::vector<double> X, Xn, Xt;
};

// CUDA-event timing of the engine's phases on the context stream; elapsed
// times are collected once, when the caller asks for them
struct PhaseTimer {
    enum { PCG, TET, CONTACT, CCD, TOTAL, BARRIER, ASSEMBLY, LINESEARCH, NPHASE };
    struct Rec {
        int phase;
        cudaEvent_t a, b;
        double host_ms;
        std::chrono::steady_clock::time_point t0;
    };
    std::vector<cudaEvent_t> pool;
    std::vector<Rec> recs;
    std::vector<int> open;      // stack of open records
    size_t used = 0;
    bool enabled = true;
    cudaEvent_t take() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
    void start(int ph, cudaStream_t s) {
        if (!enabled) return;
        Rec r;
        r.phase = ph;
        r.a = take();
        r.b = nullptr;
        r.host_ms = 0;
        cudaEventRecord(r.a, s);
        r.t0 = std::chrono::steady_clock::now();
        open.push_back((int)recs.size());
        recs.push_back(r);
    }
    void stop(cudaStream_t s) {
        if (!enabled || open.empty()) return;
        Rec& r = recs[open.back()];
        open.pop_back();
        r.b = take();
        cudaEventRecord(r.b, s);
        r.host_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - r.t0).count();
    }
    void reset() {
        recs.clear();
        open.clear();
        used = 0;
    }
    // device (event) and host (enqueue-to-return) milliseconds per phase
    void collect(double* ms, double* host) {
        for (int k = 0; k < NPHASE; ++k) ms[k] = host[k] = 0;
        for (auto& r : recs) {
            if (!r.b) continue;
            float t = 0;
            cudaEventSynchronize(r.b);
            cudaEventElapsedTime(&t, r.a, r.b);
            ms[r.phase] += t;
            host[r.phase] += r.host_ms;
        }
    }
    void release() {
        for (auto e : pool) cudaEventDestroy(e);
        pool.clear();
        reset();
    }
};

// all scratch/work buffers reused across calls, indexed by slot
enum WorkSlot {
    W_SCRATCH, W_SCRATCH2, W_TET_GRAD, W_TET_HESS, W_CHUNK_SUM, W_INST_SUM, W_FLAGS,
    // grids (two slots: 0 and 1), 6 buffers each
    W_GRID0, W_GRID0_END = W_GRID0 + 6, W_GRID1 = W_GRID0_END, W_GRID1_END = W_GRID1 + 6,
    W_BOX_A, W_BOX_B, W_GRIDP, W_BBOX,
    W_CAND, W_CAND_CNT,
    W_CONS, W_CONS_INST, W_CONS_KEY_HI, W_CONS_KEY_LO, W_CONS_PERM, W_CONS_PERM2, W_CONS_TMP, W_CONS_TMP_INST,
    W_CONS_HEAD, W_CONS_OFF, W_CONS_CNT, W_DIST2,
    W_PREV_CONS, W_PREV_INST, W_PREV_DIST2,
    W_BH, W_BG, W_GENT_KEY, W_GENT_VAL, W_GENT_KEY2, W_GENT_VAL2, W_GENT_HEAD,
    W_TAIL_ROWPTR, W_TAIL_COL, W_TAIL_VAL, W_TAIL_KEYS,
    W_BSR_VAL, W_DIAG_INV, W_PCG_VEC, W_PCG_GRID, W_SPAN, W_CBASE, W_DENSE0, W_DENSE1, W_PCG_VEC64, W_CCD_TMP, W_CCD_ALPHA, W_MISC, W_MISC2,
    W_CL_INT, W_CL_DENSE, W_CL_HOSTCONS, W_PSD, W_SHELL_GRAD, W_CCD_VOX, W_SHELL_PSD,
    W_NUM
};
struct Work {
    DBuf b[W_NUM];
    idp_stats stats{};
    PhaseTimer timer;
    std::vector<double> pcg_bytes_per_iter;  // per instance
    double* tol_inst = nullptr;              // per-instance PCG tolerance (device)
    long grid_min_v = 16384;                 // grid-wide PCG above this many vertices
    long grid_vper = 112;                    // vertices per CTA in the grid-wide PCG
    int local_deg = 0;                       // degree of the grid PCG's CTA-local polynomial preconditioner
    int cl_cap = kClusterCap;                // vertices per dense contact block
    long long accd_maxit = 0;                // diagnostics (IDP_PROFILE)
    long long accd_long = 0, accd_total = 0, accd_pairs = 0;
    // contact-cluster preconditioner (rebuilt with every Hessian)
    struct Clusters {
        int n = 0;                 // clusters of >= 2 vertices
        long nvert = 0;            // vertices in clusters
        long dense = 0;            // total dense entries
        int* vcl = nullptr;        // V: cluster id or -1
        int* vloc = nullptr;       // V: index inside its cluster
        int* off = nullptr;        // n+1: vertex offsets
        int* vert = nullptr;       // nvert: vertex ids
        long long* doff = nullptr; // n+1: dense offsets
        int* ioff = nullptr;       // nI+1: clusters of each instance (clusters sorted by instance)
        int* ok = nullptr;         // n: factorisation succeeded
        int max_n = 0;
    } cl;
    long cand_cap_pt = 0, cand_cap_ee = 0;   // candidate list capacities (grown on overflow)
    long isect_cap = 0;                      // intersecting-pair list capacity
    long ccd_cap_pt = 0, ccd_cap_ee = 0;
    // dense cell tables of the two broad phases (0: constraint set, 1: CCD):
    // capacities from the last synchronised build, reused without a round trip
    bool dense_ready[2] = {false, false};
    unsigned long long dense_cells_cap[2] = {0, 0};
    long dense_ent_cap[2] = {0, 0};
    unsigned long long grid_prof[5] = {0, 0, 0, 0, 0};  // grid PCG phase ns (IDP_PROFILE)
    bool grid_prof_init = false;
    uint32_t* hpin = nullptr;                // 64 words of pinned host memory for batched readbacks
    uint32_t* pinned() {
        if (!hpin && cudaMallocHost(reinterpret_cast<void**>(&hpin), 64 * sizeof(uint32_t)) != cudaSuccess)
            hpin = nullptr;
        return hpin;
    }
    double* hpin_d = nullptr;               // pinned host doubles (per-instance readbacks)
    long hpin_d_n = 0;
    double* pinned_doubles(long n) {
        if (n > hpin_d_n) {
            if (hpin_d) cudaFreeHost(hpin_d);
            hpin_d = nullptr;
            hpin_d_n = 0;
            if (cudaMallocHost(reinterpret_cast<void**>(&hpin_d), sizeof(double) * (n + 8)) != cudaSuccess) return nullptr;
            hpin_d_n = n;
        }
        return hpin_d;
    }
    DBuf& operator[](int i) { return b[i]; }
    void release() {
        for (auto& x : b) x.release();
        timer.release();
        if (hpin) cudaFreeHost(hpin);
        hpin = nullptr;
        if (hpin_d) cudaFreeHost(hpin_d);
        hpin_d = nullptr;
        hpin_d_n = 0;
    }
};

struct Params {
    idp_params p;
};

// ---------------------------------------------------------------- stepping (engine.cpp)
// idp_advance = step_begin(all) + step_iterate(until none is left); the
// request server drives the parts itself.
int step_begin(idp_ctx* c, const std::vector<unsigned char>& which);
int step_iterate(idp_ctx* c, int max_iters, idp_result* results, int* n_active);
int step_prepare_resumed(idp_ctx* c);
// an instance taken from another context's committed copy (surface,
// device order and rest data already built), before idp_commit
int add_prebuilt(idp_ctx* c, const HostInstance& h);
const HostInstance* instance_host(idp_ctx* c, int i);
int snapshot_instance(idp_ctx* c, int i, InstSnapshot& out);
int resume_instance(idp_ctx* c, int i, const InstSnapshot& in);
bool instance_active(idp_ctx* c, int i);  // still iterating in the step in flight

// ---------------------------------------------------------------- launchers
// shell.cu: flow energy of triangle shells (INC_POTENTIAL.h:53-73, 191-211)
int flow_energy(Arena& A, Work& W, const double* X, double* inst_E, cudaStream_t s);  // accumulates
int flow_gradient(Arena& A, const double* X, double* g, cudaStream_t s);              // accumulates

// shell_elastic.cu: membrane + hinge bending of elastic shells
int shell_energy(Arena& A, Work& W, const double* X, double w_h2, double* inst_E, cudaStream_t s);  // accumulates
int shell_gradient(Arena& A, Work& W, const double* X, double w_h2, double* g, cudaStream_t s);     // accumulates
int shell_hessian(Arena& A, Work& W, const double* X, double w_h2, bool fp64, cudaStream_t s);

// tet.cu
int tet_energy(Arena& A, Work& W, const double* X, double w_h2, double* inst_E, int* inst_bad, cudaStream_t s);
int tet_detcheck(Arena& A, Work& W, const double* X, int* inst_bad, cudaStream_t s);
int tet_gradient(Arena& A, Work& W, const double* X, double w_h2, double* g, cudaStream_t s);
int tet_hessian(Arena& A, Work& W, const double* X, double w_h2, bool fp64, cudaStream_t s);

// contact.cu
struct ContactSet {
    long C = 0;                        // total constraints
    std::vector<int> off;              // host per-instance offsets (nI+1)
    int* d_off = nullptr;              // device offsets
};
int build_constraint_set(Arena& A, Work& W, const double* X, ContactSet& cs, cudaStream_t s);
int constraint_min_dist2(Arena& A, Work& W, const double* X, const int4* cons, const int* cinst, long C,
                         double* dist2, double* inst_min, cudaStream_t s);
// Edge-triangle intersections of the surfaces of the active instances at X
// (Check_Edge_Tri_Intersect, FEM/IPC.h:2444-2517, exact predicates):
// inst_count[nI] (device) receives each instance's number of intersecting
// pairs; *pairs (device, valid until the next broad phase) the *npairs pairs
// (arena triangle index, arena edge index) in no particular order.
// Synchronises the stream.
int edge_tri_intersections(Arena& A, Work& W, const double* X, unsigned int* inst_count, const int2** pairs,
                           long* npairs, cudaStream_t s);

// barrier.cu
int barrier_energy(Arena& A, Work& W, const double* X, const ContactSet& cs, double* inst_E, int* inst_bad,
                   cudaStream_t s);
int barrier_gradient(Arena& A, Work& W, const double* X, const ContactSet& cs, double* g, cudaStream_t s);
int barrier_hessian(Arena& A, Work& W, const double* X, const ContactSet& cs, bool fp64, cudaStream_t s);

// ccd.cu
// voxel size of the CCD hash at X for every instance (the mean surface edge
// length in the reference's summation order), into W_CCD_VOX; ccd_stepsize
// takes it instead of computing it when given
int ccd_voxel_size(Arena& A, Work& W, const double* X, cudaStream_t s);
const double* ccd_voxel_sizes(Arena& A, Work& W);
int ccd_stepsize(Arena& A, Work& W, const double* X, const double* dir, double* alpha /*device nI*/, int* flags,
                 cudaStream_t s, const double* voxel_pre = nullptr);

// solver.cu
int assemble(Arena& A, Work& W, const ContactSet& cs, bool fp64, cudaStream_t s);
int normal_flow_velocity(Arena& A, int sel, double step, double h, double* vel, cudaStream_t s);
int pcg_solve(Arena& A, Work& W, const ContactSet& cs, bool fp64, const double* rhs, double* sol,
              double rel_tol, int max_iters, std::vector<int>& iters_out, std::vector<double>& relres_out,
              cudaStream_t s, const double* tol_host = nullptr);

// vector helpers (solver.cu)
int vec_inertia(Arena& A, Work& W, const double* X, double* inst_E, double* g /*nullable*/, cudaStream_t s);
int vec_axpy_trial(Arena& A, const double* Xprev, const double* dir, double* Xout, cudaStream_t s);
int vec_zero_dbc(Arena& A, double* g, cudaStream_t s);
// vecops.cu: between the caller's vertex order (in) and the device order
// (out) for the instance's range [v0, v0 + n) of 3-vectors
int perm_to_device(Arena& A, long v0, long n, const double* in, double* out, cudaStream_t s);
int perm_to_caller(Arena& A, long v0, long n, const double* in, double* out, cudaStream_t s);
// surface.cu: surface of a tet mesh in the reference's order, on the device
int extract_surface_device(int V, const std::vector<int>& tets, std::vector<int>& tris, std::vector<int>& edges,
                           std::vector<int>& nodes, cudaStream_t s);
// dirichlet.cu: moving Dirichlet conditions (the augmented Lagrangian)
int dbc_classify(Arena& A, const double* X, double* dir, int* moving, cudaStream_t s);
int dbc_snap(Arena& A, double* X, cudaStream_t s);
int dbc_sums(Arena& A, Work& W, const double* X, double* inst_w, double* inst_d, cudaStream_t s);
int dbc_gradient(Arena& A, const double* X, double* g, cudaStream_t s);
int chunk_reduce(Arena& A, Work& W, const Chunk* chunks, int nchunks, const double* chunk_vals, double* inst_out,
                 cudaStream_t s);
int chunk_reduce_off(Arena& A, const int* coff, const double* part, double* out, bool accumulate, cudaStream_t s);
int grad_gather_tet(Arena& A, Work& W, const double* X, double* g, cudaStream_t s);
int hessian_apply(Arena& A, Work& W, bool fp64, const double* x, double* y, cudaStream_t s);
// contact-cluster blocks of the preconditioner from the current constraint set
int build_contact_clusters(Arena& A, Work& W, const ContactSet& cs, bool fp64, cudaStream_t s);
// vecops.cu
int vec_neg(long n, const double* a, double* out, cudaStream_t s);
int vec_fill(double* a, long n, double v, cudaStream_t s);
int vec_copy_masked(Arena& A, const unsigned char* mask, const double* src, double* dst, cudaStream_t s);
int vec_dir_norm2(Arena& A, Work& W, const double* dir, double* inst_out, cudaStream_t s);
int vec_velocity(Arena& A, const double* X, const double* Xn, double h, double* v, cudaStream_t s);
// x_tilde = x + h v, or x + (h v + h^2 acc) with a body force (acc = M^-1 b)
int vec_xtilde(Arena& A, const double* X, const double* v, double h, double* Xt, cudaStream_t s,
               const double* acc = nullptr);
int kappa_check(Arena& A, Work& W, const double* X, const int4* cons, const int* cinst, const double* d2prev, long C,
                int* inst_flag, cudaStream_t s);

}  // namespace idp
