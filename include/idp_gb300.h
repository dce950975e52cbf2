/*
 * idp_gb300 — C ABI of the GB300 injective-deformation Newton step.
 *
 * Replaces the pybind11 entry points FEM.DiscreteShell.Advance_One_Step_IE_Hinge
 * (Library/FEM/Shell/DISCRETE_SHELL.h:1110, body
 * Library/FEM/Shell/IMPLICIT_EULER.h:151-891) for tet meshes and
 * Advance_One_Step_IE_Flow (DISCRETE_SHELL.h:1113) for triangle shells in flow
 * mode, both with offset IPC self-contact; exposes the sub-steps the reference
 * computes inside them so a caller (or a test) can check each one; and adds
 * an exact intersection check, context reuse and a request server for many
 * independent solves.
 *
 * Conventions: positions are double[3*V] (x0,y0,z0,x1,...), tets int32[4*T]
 * with instance-local vertex ids. The caller owns every host buffer; the
 * library owns device state between calls and copies explicitly. No call
 * exits the process: every failure is an IDP_* status.
 */
#ifndef IDP_GB300_H
#define IDP_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (the reference prints and calls exit(-1) where these return) */
#define IDP_OK 0
#define IDP_ERR_INVALID_ARG 1
#define IDP_ERR_CUDA 2
#define IDP_ERR_CAPACITY 3
#define IDP_ERR_INVERTED 4          /* input has a tet with det F <= 0            */
#define IDP_ERR_NOT_CONVERGED 5     /* Newton stopped at max_newton               */
#define IDP_ERR_ZERO_STEP 6         /* CCD step 0 (IPC.h:2014-2031 exits)         */
#define IDP_ERR_NONPOSITIVE_DIST 7  /* barrier at d <= 0 (IPC.h:925-928 exits)    */
#define IDP_ERR_STATE 8             /* call out of order (e.g. advance before commit) */
#define IDP_WARN_ITER_CAP 9         /* an ACCD loop hit its cap; step still safe  */
#define IDP_ERR_INTERSECTION 10     /* an accepted iterate failed the exact
                                       edge-triangle intersection check (only
                                       with idp_params.verify_iterates)          */

#define IDP_MODE_FP64 0   /* plain FP64 path: FP64 Hessians, BSR and PCG          */
#define IDP_MODE_MIXED 1  /* FP32 Hessians/BSR/PCG + FP64 residual refinement   */

typedef struct idp_ctx idp_ctx;

typedef struct idp_params {
    double h;             /* time step (IMPLICIT_EULER.h:164 `h`)                   */
    double newton_tol;    /* PNTol, stop when max of last 3 ||p||/sqrt(N-nDBC)/h <= tol
                             (IMPLICIT_EULER.h:647-676,759,855)                       */
    int max_newton;       /* Newton iteration cap                                   */
    int mode;             /* IDP_MODE_FP64 or IDP_MODE_MIXED                        */
    double pcg_rel_tol;   /* relative residual of each Newton direction            */
    int pcg_max_iters;    /* PCG iteration cap per refinement sweep                 */
    double thickness;     /* IPC offset (`thickness` argument, IPC.h:53,757)        */
    int device;           /* CUDA device ordinal                                    */
    int pcg_grid_min_vertices; /* instances above this many vertices solve with the
                             grid-wide PCG (all SMs), the others with one thread-block
                             cluster each; 0 = default (16384)                        */
    int pcg_grid_cta_vertices; /* vertices per CTA in the grid-wide PCG; 0 = default (112) */
    int contact_block_vertices; /* largest group of contact-coupled vertices the
                             preconditioner inverts as one dense block (2..192);
                             0 = default (192)                                        */
    int verify_iterates;  /* nonzero: after every accepted Newton step, check each
                             instance's surface for edge-triangle intersections with
                             exact predicates (Check_Edge_Tri_Intersect,
                             FEM/IPC.h:2444-2517, which the reference keeps as a
                             diagnostic); an instance that fails stops with
                             IDP_ERR_INTERSECTION. Positive tet volumes are already
                             enforced by the line search. 0 = off (default)          */
    int caller_vertex_order; /* 0 (default): each instance's vertices are stored on
                             the device in a spatial (Morton) order of its rest
                             positions, which keeps the PCG's per-CTA row blocks
                             compact; every array crossing this interface stays in
                             the caller's order. Nonzero: stored in the caller's
                             order.                                                  */
    int pcg_local_degree; /* grid-wide PCG (pcg_grid_min_vertices) preconditioner:
                             0 (default) = 3x3 block Jacobi; an even degree d =
                             block Jacobi over each CTA's subdomain rows, every block
                             inverted by d terms of a Neumann series in D^-1 A_loc
                             (symmetric positive definite for even d). Instances
                             solved with contact blocks keep 3x3 block Jacobi.      */
    int surface_device_min_tets; /* tet meshes with at least this many tets (and
                             fewer than 2^21 vertices) extract their surface in
                             idp_add_instance on the device (same lists, same
                             order as the host extraction); 0 = default (65536),
                             negative = always on the host                          */
} idp_params;

typedef struct idp_result {
    int status;           /* IDP_* of this instance                                 */
    int newton_iters;     /* return value of Advance_One_Step_IE_Discrete_Shell     */
    int pcg_iters;        /* total PCG iterations over the step                     */
    int ls_trials;        /* line-search energy evaluations                         */
    int num_constraints;  /* |constraint set| at the end (IMPLICIT_EULER.h:860)     */
    double energy;        /* final incremental potential                            */
    double kappa;         /* barrier stiffness after adaptation (kappaVec[0])       */
    double residual;      /* last Newton residual                                   */
    double min_alpha;     /* smallest accepted line-search step                     */
    double latency_ms;    /* host time from the start of idp_advance until this
                             instance stopped iterating                             */
} idp_result;

/* Device-time accounting of the last idp_advance (CUDA events on the
 * context's stream; no counterpart in the reference, whose TIMER_FLAG scopes,
 * Utils/PROFILER.h:66-105,175-201, time the same phases on the host). */
typedef struct idp_stats {
    double pcg_ms;          /* PCG kernels                                        */
    double pcg_bytes;       /* algorithmic bytes of those PCG iterations          */
    long long pcg_iters;    /* PCG iterations, summed over instances              */
    int pcg_launches;       /* PCG kernel launches                                */
    double tet_ms;          /* elastic energy / gradient / Hessian kernels        */
    double contact_ms;      /* constraint-set builds                              */
    double ccd_ms;          /* CCD step-size evaluations                          */
    double total_ms;        /* the whole idp_advance                              */
    long long kernel_launches; /* kernels this library launched in idp_advance    */
    double barrier_ms;      /* barrier gradient / Hessian kernels                 */
    double assembly_ms;     /* BSR assembly and contact-block factorisation       */
    int fp64_fallbacks;     /* mixed-mode directions re-solved in FP64            */
    long long verify_checks;   /* iterates checked for intersections (verify_iterates) */
    long long verify_failures; /* of those, iterates with an intersecting pair      */
} idp_stats;

/* Defaults: h=0.1, newton_tol=1e-3, max_newton=2000, mode=MIXED,
   pcg_rel_tol=1e-6, pcg_max_iters=2000, thickness=0, device=0. */
void idp_default_params(idp_params* p);

/* Context: one CUDA stream and one device arena. */
idp_ctx* idp_create(const idp_params* p, int* status);
void idp_destroy(idp_ctx* ctx);
const char* idp_status_str(int status);

/* Add one mesh instance. Stands for the state the Python driver hands the
 * reference (FEMDiscreteShellBase.add_object_3D / initialize_added_objects /
 * initialize_OIPC, Python/Drivers/FEMDiscreteShellBase.py:184-242):
 *   X     current positions (X argument, mutated by the step)
 *   X0    rest positions (nodeAttr x0; used for Dm^-1, volumes, mollifier)
 *   mass  lumped mass per vertex (diagonal of M)
 *   lam, mu per-tet Lame parameters (tetElasticityAttr)
 *   dbc_idx fixed Dirichlet vertices (DBC storage with zero displacement)
 *   dHat2, kappa, kappa_max as returned by Initialize_OIPC
 *     (FEM/Shell/DISCRETE_SHELL.h:555-577).
 * Returns the instance id (>= 0) or -IDP_* on error. Before idp_commit only. */
int idp_add_instance(idp_ctx* ctx, int V, const double* X, const double* X0, int T, const int32_t* tets,
                     const double* mass, const double* lam, const double* mu, int nDBC, const int32_t* dbc_idx,
                     double dHat2, double kappa, double kappa_max);

/* Add a triangle shell advanced in flow mode (the Laplacian flow energy of
 * Advance_One_Step_IE_Flow, FEM/Shell/DISCRETE_SHELL.h:1113, with
 * INC_POTENTIAL.h:53-73,191-211,323-339) with offset-IPC self-contact.
 * faces int32[3F]; faces with a singular first fundamental form are dropped,
 * mass and element volumes follow Initialize_Discrete_Shell
 * (DISCRETE_SHELL.h:238-333: area * thickness * density / 3 per corner,
 * area * thickness per face); the contact surface is Find_Surface_Primitives
 * (Utils/MESHIO.h:728-766). In idp_advance the instance's velocity is zeroed
 * before the predictor unless idp_set_velocity or idp_set_normal_flow gave
 * one for this step, and without contacts it stops after one Newton step
 * (IMPLICIT_EULER.h:207-209, 850-854). Returns the instance index or -IDP_*. */
int idp_add_shell_instance(idp_ctx* ctx, int V, const double* X, int F, const int32_t* faces, double density,
                           double thickness, int nDBC, const int32_t* dbc_idx, double dHat2, double kappa,
                           double kappa_max);

/* Add an elastic triangle shell of the Hinge path (Advance_One_Step_IE_Hinge
 * with shell elements, FEM/Shell/DISCRETE_SHELL.h:1110): neo-Hookean
 * membrane on the first fundamental form of every face
 * (FEM/Shell/MEMBRANE.h:7-322) and hinge bending on the dihedral angle of
 * every interior edge (FEM/Shell/BENDING.h, KL = false;
 * Math/DIHEDRAL_ANGLE.h), with offset-IPC self-contact on all faces.
 * X: current positions, X0: rest positions (NULL = X); faces int32[3F]
 * (faces with a singular rest first fundamental form are dropped). mass:
 * lumped vertex masses (V, the nodeAttr m of Initialize_Discrete_Shell), or
 * NULL for area * thickness * density / 3 per corner; membrane lambda = E nu / (1 -
 * nu^2), mu = E / (2 (1 + nu)), vol = area * thickness; hinge stiffness
 * k = bending_mult * E thickness^3 / (24 (1 - nu^2)) with the rest angle,
 * |rest edge| and (|n1| + |n2|) / (6 |edge|) of Compute_Discrete_Shell_Inv_Basis
 * (DISCRETE_SHELL.h:132-357). Elements whose vertices are all fixed are
 * skipped. Before idp_commit; returns the instance index or -IDP_*. */
int idp_add_elastic_shell_instance(idp_ctx* ctx, int V, const double* X, const double* X0, int F,
                                   const int32_t* faces, const double* mass, double density, double E, double nu,
                                   double thickness, double bending_mult, int nDBC, const int32_t* dbc_idx,
                                   double dHat2, double kappa, double kappa_max);

/* Velocity v (3V); x_tilde = x + h v (IMPLICIT_EULER.h:195-216; a body force
 * adds h^2 M^-1 b, idp_set_body_force). MeshIO.Load_Velocity_X0
 * (Utils/MESHIO.h:986-1004) sets v = (target - x)/h. */
int idp_set_velocity(idp_ctx* ctx, int inst, const double* v);
/* Body force b (3V) of one instance, the `b` argument of
 * Advance_One_Step_IE_Hinge: the predictor becomes
 * x_tilde = x + (h v + h^2 M^-1 b) (IMPLICIT_EULER.h:195-216; M is the lumped
 * mass, so M^-1 b = b / m per vertex). Kept for every following step until
 * changed; b = NULL removes it. Before or after idp_commit. */
int idp_set_body_force(idp_ctx* ctx, int inst, const double* b);
/* Current positions (3V), e.g. a warm start between frames. */
int idp_set_positions(idp_ctx* ctx, int inst, const double* X);
/* Targets of the instance's DBC vertices: 3 doubles per vertex of the dbc_idx
 * list given when the instance was added, in that order (the reference's DBC
 * rows (index, x, y, z), VECTOR_STORAGE<T, dim + 1>; FEM.Load_Dirichlet,
 * BOUNDARY_CONDITION.h:175-197, refreshes them per frame). At the start of
 * each following step (IMPLICIT_EULER.h:305-401) a DBC vertex whose target is
 * its position is fixed; the others move onto their targets when the CCD step
 * of that displacement is 1, and otherwise are pulled there inside the Newton
 * loop by the penalty stiff/2 sum m |t - x|^2 (FEM/Shell/DIRICHLET.h), stiff
 * starting at 1e6 and doubling (up to 1e8) whenever the solve settles, until
 * the DBC vertices have covered 99 % of their way (:701-757); the step does
 * not stop before that. NULL clears the targets (every DBC vertex fixed).
 * Before or after idp_commit, not while a step is in flight; a dbc_idx list
 * that names a vertex twice has no targets (-> IDP_ERR_INVALID_ARG). */
int idp_set_dbc_targets(idp_ctx* ctx, int inst, const double* targets);

/* Normal-flow predictor for one instance (inst >= 0) or all (inst = -1),
 * computed on the device from the current positions: every surface vertex
 * gets x_tilde = x + step * n, n its normalised sum of incident surface
 * triangle normals cross(X2-X1, X3-X1); interior vertices get x_tilde = x.
 * Stored as the velocity v = (step / |n_sum|) * n_sum / h (zero inside).
 * Replaces Update_Normal_Flow_Neumann (FEM/Shell/DISCRETE_SHELL.h:359-395),
 * whose body force b = magnitude * m * n shifts x_tilde by h^2 * magnitude * n,
 * i.e. step = h^2 * magnitude. After idp_commit only. */
int idp_set_normal_flow(idp_ctx* ctx, int inst, double step);

/* Upload every instance to the device and build the static structures
 * (surface primitives, BSR pattern). */
int idp_commit(idp_ctx* ctx);

/* One implicit-Euler step of every instance: Newton to convergence with
 * PSD-projected Hessians, CCD-filtered backtracking line search and
 * adaptive kappa. Replaces Advance_One_Step_IE_Hinge
 * (FEM/Shell/DISCRETE_SHELL.h:1110 -> IMPLICIT_EULER.h:151-891).
 * results: array of idp_result, one per instance (may be NULL). */
int idp_advance(idp_ctx* ctx, idp_result* results);

/* The same step in bounded parts, for callers that interleave other work
 * between Newton iterations (the request server admits new meshes there):
 * idp_step_begin does what idp_advance does first (x^n = x, the predictor
 * x_tilde, the initial constraint set and energy, IMPLICIT_EULER.h:195-216,
 * 418-434); idp_step_iterate then runs at most max_iters Newton iterations
 * of the instances still iterating (IMPLICIT_EULER.h:436-876). An instance
 * that stops has its velocity and result final at the end of the call;
 * *n_active (may be NULL) receives how many are still iterating, and results
 * (may be NULL) one idp_result per instance. idp_advance = idp_step_begin,
 * then idp_step_iterate until none is left; the parts give the same results
 * bit for bit. idp_get_stats covers the step since its begin. The reference
 * runs the whole loop in one call. */
int idp_step_begin(idp_ctx* ctx);
int idp_step_iterate(idp_ctx* ctx, int max_iters, idp_result* results, int* n_active);

/* Device-side checkpoint of every instance's positions, velocity and kappa
 * (the reference restarts from OBJ files instead,
 * Python/Drivers/FEMDiscreteShellBase.py:244-253). Restore copies it back
 * device to device. */
int idp_save_state(idp_ctx* ctx);
int idp_restore_state(idp_ctx* ctx);

/* Stats of the last idp_advance (zeros before the first). */
int idp_get_stats(idp_ctx* ctx, idp_stats* out);

/* Read back positions X (3V), velocity v (3V) and kappa[3] of one instance. */
int idp_get_state(idp_ctx* ctx, int inst, double* X, double* v, double* kappa3);

/* Set kappa[0..1] = (kappa, kappa_max) of one instance, the in/out kappaVec
 * argument of Advance_One_Step_IE_Hinge (FEM/Shell/IMPLICIT_EULER.h:151-187,
 * doubled in place at :566-595); kappa[2] is ignored. */
int idp_set_kappa(idp_ctx* ctx, int inst, const double* kappa3);

/* Number of instances, and vertex/tet/surface counts of one instance. */
int idp_instance_info(idp_ctx* ctx, int inst, int* V, int* T, int* n_nodes, int* n_edges, int* n_tris);

/* Surface primitives of an instance, in the reference's order
 * (Find_Surface_TriMesh, Utils/MESHIO.h:485-544, and
 * Find_Surface_Primitives_And_Compute_Area, MESHIO.h:768-834). */
int idp_get_surface(idp_ctx* ctx, int inst, int32_t* nodes, int32_t* edges, int32_t* tris);

/* ---- sub-steps at caller-given positions (all for one instance) ---- */

/* Incremental potential parts at X: h^2 * sum vol*Psi (NEOHOOKEAN.h:78-93),
 * 0.5 (x-xt)^T M (x-xt) (INC_POTENTIAL.h:132-144) and the barrier sum over the
 * constraint set built at X (IPC.h:742-941). Returns IDP_ERR_INVERTED if a
 * tet has det F <= 0 (INC_POTENTIAL.h:98-108). */
int idp_eval_energy(idp_ctx* ctx, int inst, const double* X, double* E_elastic, double* E_inertia,
                    double* E_barrier);

/* Gradient (3V) of the incremental potential at X (INC_POTENTIAL.h:154-275),
 * with DBC rows zeroed (IMPLICIT_EULER.h:476-480). */
int idp_eval_gradient(idp_ctx* ctx, int inst, const double* X, double* g);

/* Constraint set at X (Compute_Constraint_Set, FEM/IPC.h:143-661): sign-tagged
 * int4 records sorted lexicographically. *count receives the size; at most cap
 * records are written (IDP_ERR_CAPACITY if cap is too small). */
int idp_constraint_set(idp_ctx* ctx, int inst, const double* X, int cap, int32_t* cons, int* count);

/* Largest intersection-free step alpha <= *alpha along dir from X
 * (Compute_Intersection_Free_StepSize, FEM/IPC.h:1879-2244). */
int idp_ccd_stepsize(idp_ctx* ctx, int inst, const double* X, const double* dir, double* alpha);

/* Assembled system matrix at X (tets + barrier + mass, PSD-projected;
 * Compute_IncPotential_Hessian, INC_POTENTIAL.h:277-395) times a vector:
 * y = H x (3V). Uses the precision of the context's mode. */
int idp_hessian_apply(idp_ctx* ctx, int inst, const double* X, const double* x, double* y);

/* Clear the context's instances so a new set can be added and committed,
 * keeping its device buffers (grow-only): the next commit and solve reuse them
 * instead of allocating. No counterpart in the reference, whose simulator
 * object is built once per scene. */
int idp_reset(idp_ctx* ctx);

/* Device memory the context holds (arena and work buffers), in bytes. */
int idp_device_bytes(idp_ctx* ctx, size_t* bytes);

/* Edge-triangle intersections of instance inst's surface at X (V x 3; NULL =
 * the instance's current state): Check_Edge_Tri_Intersect (FEM/IPC.h:2444-2517)
 * with segTriIntersect (FEM/IPC.h:2390-2442) decided by exact orientation
 * predicates. Pairs are (triangle, edge) indices into the idp_get_surface
 * lists, sorted; *count receives their number, at most cap are written
 * (IDP_ERR_CAPACITY if cap is too small). 0 pairs = intersection-free. */
int idp_check_intersection(idp_ctx* ctx, int inst, const double* X, int cap, int32_t* pairs, int* count);

/* The same check on every instance at its current state; counts[i] receives
 * instance i's number of intersecting pairs (no counterpart in the reference,
 * which checks one mesh per call). */
int idp_check_intersection_all(idp_ctx* ctx, int32_t* counts);

/* ---------------------------------------------------------------------------
 * Request server: continuous batching of independent solves on one GPU.
 * No counterpart in the reference, which advances one scene per Python call
 * (Python/Drivers/FEMDiscreteShellBase.py:333-361).
 *
 * Jobs (one mesh and its predictor each) are queued in arrival order. A pool
 * of worker threads, each driving its own context and CUDA stream, solves
 * the jobs it holds a few Newton iterations at a time. Between those chunks a
 * worker writes the result of every job that finished (at once, not when the
 * slowest job it holds finishes) and, once half of its max_batch slots are
 * free (or it holds none), admits jobs from the head of the queue into its
 * running arena (max_batch jobs at most): the jobs still iterating
 * are carried over to a rebuilt arena with the new ones and their Newton
 * loops continue where they were. Workers run on the device at the same
 * time. Admission keeps the sum over workers of max(device bytes the worker's
 * context holds, footprints of its unfinished jobs) within the budget; idle
 * workers give their contexts back when the head job needs that memory.
 * A job's result does not depend on the jobs it ran with (per-instance
 * reductions are fixed-order, and a carried-over instance resumes with its
 * exact state).
 * ------------------------------------------------------------------------- */
typedef struct idp_server idp_server;

typedef struct idp_job_desc {
    int V;                  /* mesh, as idp_add_instance                                */
    const double* X;
    const double* X0;       /* rest shape (NULL = X)                                    */
    int T;
    const int32_t* tets;
    const double* mass;
    const double* lam;      /* T values                                                 */
    const double* mu;       /* T values                                                 */
    int nDBC;
    const int32_t* dbc_idx;
    double dHat2, kappa, kappa_max;
    const double* v;        /* initial velocity (3V; NULL = zero): x_tilde = x + h v    */
    double normal_flow;     /* nonzero: predictor of idp_set_normal_flow(step) instead  */
    double* X_out;          /* 3V host buffer written when the job completes (or NULL)  */
    double* v_out;          /* 3V host buffer written when the job completes (or NULL)  */
} idp_job_desc;

typedef struct idp_job_info {
    int status;             /* IDP_* of the job                                         */
    idp_result result;      /* as idp_advance reports it                                */
    double submit_ms;       /* server clock: ms since idp_server_create                 */
    double admit_ms;        /* when a worker took it                                    */
    double done_ms;         /* when its result was written                              */
    int cohort;             /* id of the cohort it ran in                               */
    int cohort_size;        /* jobs in that cohort                                      */
    double footprint;       /* admission estimate, bytes                                */
} idp_job_info;

typedef struct idp_server_stats {
    long long submitted, completed, cohorts; /* cohorts: admission events           */
    double peak_resident;   /* largest sum of the footprints of admitted, unfinished jobs */
    int peak_concurrency;   /* most workers with unfinished jobs at once                */
    double device_bytes;    /* device memory the worker contexts hold now               */
    double peak_device;     /* largest sum over workers of max(bytes the context holds,
                               footprints of its unfinished jobs): what admission keeps
                               within the budget                                        */
} idp_server_stats;

/* Admission estimate of one job's device memory (arena, matrix, solver and
 * broad-phase buffers), bytes. */
double idp_job_footprint(int V, int T);

/* p: solver parameters of every job (NULL = defaults); hbm_budget: bytes the
 * admitted jobs' footprints may sum to; workers: concurrent cohorts (>= 1);
 * max_batch: jobs per cohort (>= 1). */
idp_server* idp_server_create(const idp_params* p, double hbm_budget, int workers, int max_batch, int* status);

/* Scheduler only, no device work: a job of V vertices "needs" 2 + V/1000
 * Newton iterations, an iteration of a worker takes ms_per_kvertex / 10 per
 * thousand vertices of its unfinished jobs, a worker's context "holds" the
 * largest sum of footprints its arena had (grow-only, as real contexts), and
 * every job completes with IDP_OK and its input positions. For testing
 * admission and scheduling without a GPU. */
idp_server* idp_server_create_simulated(double hbm_budget, int workers, int max_batch, double ms_per_kvertex,
                                        int* status);

/* Queue a job (inputs are copied; X_out / v_out must stay valid until the job
 * completes). Returns the job id (>= 0) or -IDP_ERR_* (a footprint above the
 * whole budget is IDP_ERR_CAPACITY). Thread-safe. */
int idp_server_submit(idp_server* s, const idp_job_desc* job);

/* Block until the job completes; info (may be NULL) receives its record. */
int idp_server_wait(idp_server* s, int job, idp_job_info* info);

/* Block until every submitted job has completed. */
int idp_server_drain(idp_server* s);

int idp_server_get_stats(idp_server* s, idp_server_stats* out);

/* Finishes the queued jobs, stops the workers and frees their contexts. */
void idp_server_destroy(idp_server* s);

/* Solve H p = -g at X with the context's PCG (mixed or FP64); returns PCG
 * iterations in *iters and the final relative residual in *relres. */
int idp_newton_direction(idp_ctx* ctx, int inst, const double* X, double* p, int* iters, double* relres);

/* Elastic energy weight * sum_t vol_t * Psi(F_t) of one tet mesh held in the
 * caller's DEVICE memory, without allocating anything: for callers that may
 * not call cudaMalloc while they run (a host application that reserved the
 * whole GPU budget up front and lends the library only its own buffers, or a
 * frame loop that cannot take the device-wide synchronisation of
 * cudaMalloc/cudaFree). No counterpart in the reference; it gives the same
 * number as idp_eval_energy's elastic term (same per-tet arithmetic and
 * reduction order) for a context-free caller.
 *   tets (4T int32), X (3V), IB (9T, row-major inverse rest basis), vol (T),
 *   lam (T), mu (T): device pointers. energy (1 double) and inverted (1 int32,
 *   set to 1 when some det F <= 0) are device pointers written by the call.
 *   stream: a cudaStream_t (NULL = legacy default stream); the call is
 *   asynchronous on it.
 * At most 16,777,216 tets per call (IDP_ERR_CAPACITY beyond). Scratch is a
 * fixed 128 KB device array inside the library shared by every call on a GPU:
 * calls that overlap on the GPU (other streams, other threads) race on it, so
 * order them. The first call on each device looks up that array's device
 * address (again after the device's context is re-created, e.g. by
 * cudaDeviceReset). */
int idp_tet_energy_noalloc(int T, const int32_t* tets, const double* X, const double* IB, const double* vol,
                           const double* lam, const double* mu, double weight, double* energy, int32_t* inverted,
                           void* stream);

#ifdef __cplusplus
}
#endif
#endif /* IDP_GB300_H */
