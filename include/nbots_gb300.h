/*
 * nbots_gb300: thin C ABI over the sm_103a CUDA kernels of nbots' 2D
 * linear-elastic FEM hot path.
 *
 * Two layers share this header:
 *   - device-pointer kernels (nbg_*): every array argument is a device
 *     pointer, `stream` is a cudaStream_t (NULL = legacy default stream),
 *     and scratch memory comes either from the caller (ws, ws_bytes) or,
 *     when ws is NULL, from cudaMalloc inside the call;
 *   - host-buffer conveniences (nbg_host_*, nbg_fem_*) used by the C
 *     drop-in of nbots' own entry points (include/nbots_dropin.h).
 *
 * Status codes: 0 success; positive values keep nbots' meanings (1 = CG did
 * not reach the tolerance, cg_precond_jacobi.c:86-89; 1 = distorted
 * element, static_elasticity2D.c:62-66); negative values are errors that
 * nbots has no code for.  No entry point exits the process or traps the GPU.
 */
#ifndef NBOTS_GB300_H
#define NBOTS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBG_OK 0
#define NBG_NOT_CONVERGED 1
#define NBG_DISTORTED 1
#define NBG_ERR_CUDA (-1)
#define NBG_ERR_TIMEOUT (-2)     /* a device-side wait ran out its limit */
#define NBG_ERR_ARG (-3)
#define NBG_ERR_NOMEM (-4)
#define NBG_ERR_PATTERN (-5)     /* an element pair is missing from the CSR pattern */
#define NBG_ERR_BREAKDOWN (-6)   /* CG met a zero or non-finite curvature */

/* ------------------------------------------------------------------ misc */
const char *nbg_version(void);
int nbg_device_count(void);
/* Last CUDA error text seen by the library in this thread. */
const char *nbg_last_error(void);

int nbg_dev_alloc(void **ptr, size_t bytes);
int nbg_dev_free(void *ptr);
int nbg_h2d(void *dst, const void *src, size_t bytes, void *stream);
int nbg_d2h(void *dst, const void *src, size_t bytes, void *stream);
int nbg_d2d(void *dst, const void *src, size_t bytes, void *stream);
int nbg_memset(void *dst, int value, size_t bytes, void *stream);
int nbg_stream_sync(void *stream);
/* 1 when kernels on the current device read and write ordinary (pageable)
 * host memory coherently through the host's page tables, as a Grace CPU's
 * memory over NVLink-C2C; else 0. */
int nbg_host_memory_access(void);
/* Device-side bounded wait: one thread polls *flag (device memory) until it
 * equals `expect`; after limit_ns nanoseconds it stores NBG_ERR_TIMEOUT in
 * *status (device memory) and returns, leaving the context usable. */
int nbg_wait_flag(const int *flag, int expect, uint64_t limit_ns, int *status, void *stream);

/* -------------------------------------------------------------- assembly */
/* Element stiffness and load of every element in nbots' operation order
 * (replaces the per-element work of pipeline_assemble_system,
 * pde_bot/finite_element/solid_mechanics/pipeline.c:83-230).
 * nen = 3 (T3) or 4 (Q4).  Ke: N_elem x (2nen)^2 row-major; Fe: N_elem x 2nen.
 * E: one modulus per element.  enabled may be NULL (all enabled).
 * distorted: one device uint32, set to the smallest distorted element id
 * (detJ < 0, utils.c:44-47) or left untouched; initialise it to UINT32_MAX. */
int nbg_element_stiffness_f64(uint32_t nen, uint32_t N_elem, const double *nod,
                              const uint32_t *conn, const double *E, double nu,
                              double thickness, double density, int self_weight,
                              double gx, double gy, const uint8_t *enabled,
                              double *Ke, double *Fe, uint32_t *distorted,
                              void *stream);

/* The same with damage[N_gp N_elem] (device, may be NULL): the constitutive
 * matrix of each Gauss point is scaled by (1 - damage) first
 * (DMG_pipeline_assemble_system, static_damage2D.c:474-569). */
int nbg_element_stiffness_damage_f64(uint32_t nen, uint32_t N_elem, const double *nod,
                                     const uint32_t *conn, const double *E, double nu,
                                     double thickness, double density, int self_weight,
                                     double gx, double gy, const uint8_t *enabled,
                                     const double *damage, double *Ke, double *Fe,
                                     uint32_t *distorted, void *stream);

/* Row-gather assembly into the CSR of nb_sparse_create(graph, NULL, 2)
 * (sparse.c:20-60) in ascending element order, so K and F equal nbots'
 * serial scatter (pipeline.c:60-69, 232-264) bit for bit; no float atomics.
 * inc_ptr/inc_elem/inc_local: node -> (element, local node) incidence sorted
 * by element id.  matched: one device uint64 counter, incremented by the
 * number of (node block, shared element) pairs found; it ends at
 * N_elem * nen^2 exactly when every element node pair is in the pattern
 * (nbots exits on a missing pair, sparse.c:213-218). */
int nbg_gather_assemble_f64(uint32_t nen, uint32_t N_nod, uint32_t N_elem,
                            const uint32_t *inc_ptr, const uint32_t *inc_elem,
                            const uint8_t *inc_local, const uint32_t *row_ptr,
                            const uint32_t *col_idx, const double *Ke, const double *Fe,
                            double *K, double *F, unsigned long long *matched, void *stream);

/* Sequential load increments F[idx[k]] += inc[k], in k order per index
 * (the Neumann loops of set_bconditions.c:63-190), grouped by index:
 * group g adds inc[group_ptr[g] .. group_ptr[g+1]) to F[idx_of_group[g]]
 * in that order. */
int nbg_apply_increments_f64(uint32_t n_groups, const uint32_t *idx_of_group,
                             const uint32_t *group_ptr, const double *inc,
                             double *F, void *stream);

/* Dirichlet elimination in nbots' event order (nb_sparse_set_Dirichlet_condition,
 * sparse.c:416-430, called per masked dof in set_bconditions.c:192-260).
 * Events are (dof, value) in application order; ev_ptr (N+1) lists, per
 * dof, the event numbers that touch it in ascending order (ev_of). */
int nbg_dirichlet_f64(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                      double *K, double *F, const uint32_t *ev_ptr, const uint32_t *ev_of,
                      const double *ev_val, int *status, void *stream);

/* Strain at Gauss points (pipeline.c:266-319) and stress from strain with
 * one modulus per element (static_elasticity2D.c:99-127). */
int nbg_strain_f64(uint32_t nen, uint32_t N_elem, const double *nod, const uint32_t *conn,
                   const double *u, double *strain, void *stream);
int nbg_stress_f64(uint32_t nen, uint32_t N_elem, const double *E, double nu,
                   const uint8_t *enabled, const double *strain, double *stress,
                   void *stream);
/* Principal stresses (pipeline_compute_main_stress, pipeline.c:321-340):
 * main_stress[2 N_gp N_elem] from stress[3 N_gp N_elem]; bit-exact. */
int nbg_main_stress_f64(uint32_t nen, uint32_t N_elem, const double *stress,
                        double *main_stress, void *stream);

/* ---------------------------------------------------------------- damage */
/* Strain, tension damage and damage threshold at every Gauss point
 * (DMG_pipeline_compute_strain with tension_damage and get_clfd,
 * static_damage2D.c:134-182, 571-647) for one plane-stress material
 * (E, nu, traction limit ft, fracture energy gf):
 * r[id] = max(r_prev[id], tau), damage[id] = 1 - (r0/r) exp(A (1 - r/r0)).
 * All arrays on the device; distorted as for nbg_element_stiffness_f64. */
int nbg_strain_damage_f64(uint32_t nen, uint32_t N_elem, const double *nod,
                          const uint32_t *conn, const double *u, double E, double nu,
                          double ft, double gf, const double *r_prev, double *r,
                          double *damage, double *strain, uint32_t *distorted, void *stream);
/* res = F - K u with nbots' row sums (static_damage2D.c:343-351) and
 * *norm2 = sum of res^2 (one device double, fixed summation tree).
 * ws: nbg_residual_workspace_bytes(N) device bytes. */
size_t nbg_residual_workspace_bytes(uint32_t N);
int nbg_residual_f64(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                     const double *K, const double *F, const double *u, double *res,
                     double *norm2, void *ws, void *stream);
/* x += dx (device arrays). */
int nbg_add_to_f64(uint32_t N, double *x, const double *dx, void *stream);

typedef struct {
    uint32_t niter;   /* sweeps performed */
    int status;       /* 0, 1 = not converged, NBG_ERR_TIMEOUT, < 0 error */
    double error;     /* sqrt(sum (b - A x)^2) at the last check */
} nbg_gs_result_t;

/* Levels of the forward substitution with the lower part of a CSR matrix
 * (host arrays): every row of level L depends only on rows of levels < L.
 * lev_rows[N] lists the rows level by level, ascending within a level;
 * lev_ptr[N+1] delimits the levels; *n_levels is set. */
int nbg_host_lower_levels(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                          uint32_t *lev_ptr, uint32_t *lev_rows, uint32_t *n_levels);
/* nb_sparse_solve_Gauss_Seidel (gauss_seidel.c:14-58) on the device, x as
 * the initial guess: each sweep forms c = b - (strict upper part) x and
 * error = |b - A x|^2, stops when error <= tol^2, else solves the lower part
 * by level-scheduled forward substitution (triangular.c:14-32).  One block
 * runs the whole solve; it stops with NBG_ERR_TIMEOUT after time_limit_s
 * seconds (0: no limit).  ws: nbg_gauss_seidel_workspace_bytes(N). */
size_t nbg_gauss_seidel_workspace_bytes(uint32_t N);
int nbg_gauss_seidel_f64(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                         const double *K, const double *b, double *x, const uint32_t *lev_ptr,
                         const uint32_t *lev_rows, uint32_t n_levels, uint32_t max_iter,
                         double tol, double time_limit_s, nbg_gs_result_t *result, void *ws,
                         void *stream);

/* ------------------------------------------------------------------ SpMV */
/* y = A x with nbots' per-row left-to-right sum and no FMA
 * (nb_sparse_multiply_vector, sparse.c:405-414): bit-exact. */
int nbg_spmv_csr_f64(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                     const double *val, const double *x, double *y, void *stream);

/* --------------------------------------------------------------------- CG */
#define NBG_CG_JACOBI 1u     /* Jacobi preconditioner (else plain CG) */
#define NBG_CG_RELATIVE 2u   /* stop on ||g|| <= tol ||b|| (else absolute, nbots) */
/* nbg_cg_bsr_f64 only: nbots' stop rule (cg_precond_jacobi.c:45, 80-89), the
 * lagged ||g|| of the previous iteration, reported as tol_reached (else the
 * current ||g||, confirmed on the true residual b - A x) */
#define NBG_CG_NBOTS_STOP 4u

typedef struct {
    uint32_t niter;       /* iterations performed */
    int status;           /* 0, 1 = not converged, < 0 error */
    double tol_reached;   /* nbots' lagged sqrt(dot_gg) */
    double bnorm;         /* ||b||_2 */
} nbg_cg_result_t;

/* Persistent FP64 CG in one cooperative launch, nbots' iteration
 * (cg_precond_jacobi.c:13-90 with NBG_CG_JACOBI, conjugate_gradient.c:13-77
 * without): g = Ax - b, lagged convergence test, division by the diagonal.
 * x holds x0 on entry.  Reductions are fixed-order (run-to-run identical). */
size_t nbg_cg_workspace_bytes(uint32_t N);
int nbg_cg_f64(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
               const double *val, const double *b, double *x, uint32_t max_iter,
               double tol, unsigned flags, nbg_cg_result_t *result, void *ws,
               size_t ws_bytes, void *stream);

/* nbg_cg_f64 without any device allocation, for callers that cannot
 * allocate device memory while they solve (a host application that keeps
 * the GPU's memory in its own pool and forbids libraries to call cudaMalloc,
 * or a loop that cannot take the device-wide synchronisation of
 * cudaMalloc / cudaFree).  No counterpart in nbots.  The scratch lives in a
 * 16 MiB file-scope device array that every GPU loading this library holds
 * until exit, so N is limited to 345,408 dofs (larger N: NBG_ERR_ARG, with
 * the reason in nbg_last_error).  Every call looks up the array's device
 * address on the current device (cudaGetSymbolAddress, no allocation), so a
 * cudaDeviceReset between calls is safe; the first call on a device loads
 * the library's kernels there: make it before any stream capture.  All calls
 * share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
int nbg_cg_f64_noalloc(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                       const double *val, const double *b, double *x, uint32_t max_iter,
                       double tol, unsigned flags, nbg_cg_result_t *result, void *stream);

/* ------------------------------------------------- 2x2-block SELL layout */
/* Device arrays of the node-block layout of a CSR from nb_sparse_create(.., 2)
 * (two rows per node with the same (2w, 2w+1) column pairs, sparse.c:36-52):
 * entry (slice s, k, lane r) sits at (slice_off[s] + k) * 32 + r; b64 holds
 * 4 doubles (a00 a01 a10 a11) per entry, b32 the same rounded to float but
 * column by column (a00 a10 a01 a11), and
 * the remainders (double - float) as biased 23-bit counts q + 2^22 of units
 * of 2^-46 float (|q| < 2^22): their low 16 bits in blo, their high 7 bits
 * in bxt, so that b32 + blo + bxt carries about 47 significant bits in 7
 * bytes; dinv = 1 / diagonal per scalar row.  Any array may be NULL when a
 * caller does not need it. */
typedef struct {
    uint32_t N;            /* scalar rows (= 2 Nn) */
    uint32_t Nn;           /* node rows */
    uint32_t n_slices;     /* ceil(Nn / 32) */
    uint64_t n_entries;    /* 32 * slice_off[n_slices] */
    const uint32_t *slice_off;
    const uint32_t *bcol;
    const double *b64;
    const float *b32;
    const uint16_t *blo;   /* low 16 bits of the 4 remainder counts per entry */
    const uint8_t *bxt;    /* their high 7 bits, one byte each */
    const double *dinv64;
    const float *dinv32;
    /* Optional node order (device, NULL = identity): slice row i holds node
     * perm[i], iperm[perm[i]] = i, and bcol, dinv and every vector inside the
     * solvers are in that order.  Sorting the nodes of each window of a few
     * hundred by row length (SELL-C-sigma) cuts the padding of unstructured
     * meshes.  The entry points below take and return vectors in the
     * original node order whatever the order. */
    const uint32_t *perm;
    const uint32_t *iperm;
} nbg_bsr_t;

/* Device: a SELL-C-sigma node order of a node-blocked CSR (row_ptr on the
 * device): within each window of `sigma` (<= 1024) consecutive nodes, nodes
 * by descending row length, ties by index; perm / iperm as in nbg_bsr_t and
 * the slice offsets of that order (n_slices + 1 entries). */
int nbg_bsr_plan_sigma_dev(uint32_t N_nod, const uint32_t *row_ptr, uint32_t sigma,
                           uint32_t *perm, uint32_t *iperm, uint32_t *slice_off, void *stream);

/* Host: check the block structure of a CSR and write the slice offsets
 * (n_slices + 1 entries).  NBG_ERR_PATTERN if it is not node-blocked. */
int nbg_bsr_plan(uint32_t N, const uint32_t *row_ptr, const uint32_t *col_idx,
                 uint32_t *slice_off);
/* Device: fill bcol/b64/b32/dinv from the CSR (device pointers). */
int nbg_bsr_fill(const nbg_bsr_t *A, const uint32_t *row_ptr, const uint32_t *col_idx,
                 const double *val, void *stream);
int nbg_spmv_bsr_f64(const nbg_bsr_t *A, const double *x, double *y, void *stream);
int nbg_spmv_bsr_f32(const nbg_bsr_t *A, const float *x, float *y, void *stream);

/* Fast persistent FP64 CG on the 2x2-block SELL layout (Jacobi with
 * NBG_CG_JACOBI, else plain): FMA arithmetic, reciprocal diagonal.  Default
 * stop: the current ||g|| meets the target and the true residual b - A x,
 * recomputed in FP64 at that point, meets it too (else that residual
 * replaces the recurrence's and the iteration goes on); tol_reached is then
 * the true residual norm.  A target below the FP64 floor of the system (the
 * true residual stops falling between two such checks, or the recurrence
 * does not meet the target again within twice the iterations its rate so
 * far needs)
 * ends the solve with status 1 and that floor in tol_reached.  With NBG_CG_NBOTS_STOP: nbots' iteration and stop
 * test (the lagged ||g||, one iteration past the first ||g|| <= tol),
 * iterates within rounding of nbots' own.  NBG_CG_RELATIVE selects
 * ||g|| <= tol ||b||.  x holds x0 on entry. */
size_t nbg_cg_bsr_workspace_bytes(uint32_t N);
int nbg_cg_bsr_f64(const nbg_bsr_t *A, const double *b, double *x, uint32_t max_iter,
                   double tol, unsigned flags, nbg_cg_result_t *result, void *ws,
                   size_t ws_bytes, void *stream);

/* Mixed-precision Jacobi-PCG with reliable updates.  The Krylov iteration
 * runs entirely on the FP32 pipes: matrix b32 + blo + bxt (about 47 bits),
 * residual, search direction, A p and the correction as FP32 pairs
 * (float-float), products and sums by error-free transformations (TwoProd /
 * TwoSum), dot products as float-float sums across threads and blocks, step
 * lengths as float-float quotients.  Whenever the recursive residual has
 * dropped by `delta` since the last update (and at the
 * end) the correction is added to the FP64 solution x and the residual is
 * recomputed in FP64 as r = b - A x on b64.  Convergence is judged on that
 * FP64 residual. */
typedef struct {
    uint32_t niter;        /* FP32 iterations */
    uint32_t n_updates;    /* FP64 residual recomputations */
    int status;            /* 0 converged, 1 not converged, < 0 error */
    double relres;         /* final FP64 ||b - A x|| / ||b|| */
    double bnorm;
} nbg_mixed_result_t;

/* The mixed solver's SpMV operator on its own: w = A p with A = b32 + blo and
 * p = ph + pl (FP32 pairs), products and sums error-free, result as
 * wh + wl (FP32 pairs); the first share of the matrix stream is loaded with
 * an L2 evict_last policy, as inside the solver. */
int nbg_spmv_bsr_mixed(const nbg_bsr_t *A, const float *ph, const float *pl, float *wh,
                       float *wl, void *stream);

/* Workspace: nbg_cg_mixed_workspace_bytes(N) at least.  With
 * nbg_cg_mixed_layout_workspace_bytes(A) (more: a 16-bit local column per
 * layout entry and per-block ghost lists) the solver takes its ghost-node
 * form when the system is small enough for each block's rows and ghosts to
 * live in shared memory: every block keeps the search direction p of its
 * own rows and of the rows its rows couple to (its ghosts) on chip, updates
 * the ghosts itself from their owners' published residual, and so needs
 * two grid barriers per iteration instead of three; the iterates are the
 * same bit for bit.  ws NULL allocates the larger size. */
size_t nbg_cg_mixed_workspace_bytes(uint32_t N);
size_t nbg_cg_mixed_layout_workspace_bytes(const nbg_bsr_t *A);
/* The form the calling thread's last nbg_cg_mixed launch took. */
#define NBG_MIXED_GLOBAL_ROWS 0   /* own rows and p in global memory */
#define NBG_MIXED_RESIDENT_ROWS 1 /* own rows in shared memory, p gathered from global */
#define NBG_MIXED_GHOST 2         /* own rows and ghosts in shared memory */
int nbg_cg_mixed_last_form(void);
int nbg_cg_mixed(const nbg_bsr_t *A, const double *b, double *x, uint32_t max_iter,
                 double tol, double delta, unsigned flags, nbg_mixed_result_t *result,
                 void *ws, size_t ws_bytes, void *stream);

/* Batched mixed-precision CG: n_sys independent systems stored as one
 * block-diagonal layout A, system i owning slices [slice_ptr[i],
 * slice_ptr[i+1]) (its node rows start on a multiple of 32), solved side by
 * side by one cooperative launch in which each system has its own group of
 * blocks, barrier, reductions and stopping test.  A launch (x = 0, the
 * solve, then the optional SIMP compliance sensitivities with a = b = x) is
 * one CUDA graph replayed on `stream`.  Blocks are shared out in
 * proportion to slices^gamma (nbg_mixed_batch_plan, gamma 1 at creation);
 * nbg_mixed_batch_tune times one launch per candidate gamma and keeps the
 * fastest.  Every system needs a co-resident block: n_sys is at most the
 * launch's resident block count.  No counterpart in nbots. */
typedef struct nbg_mixed_batch nbg_mixed_batch_t;
int nbg_mixed_batch_create(nbg_mixed_batch_t **out, const nbg_bsr_t *A, const double *b,
                           double *x, uint32_t n_sys, const uint32_t *slice_ptr,
                           uint32_t max_iter, double tol, double delta, unsigned flags,
                           void *stream);
void nbg_mixed_batch_destroy(nbg_mixed_batch_t *m);
int nbg_mixed_batch_plan(nbg_mixed_batch_t *m, double gamma);
/* Total blocks of the launch; blocks[i] per system and the gamma in use. */
uint32_t nbg_mixed_batch_blocks(const nbg_mixed_batch_t *m, uint32_t *blocks, double *gamma);
int nbg_mixed_batch_set_sensitivity(nbg_mixed_batch_t *m, uint32_t nen, uint32_t N_elem,
                                    const double *nod, const uint32_t *conn, double nu,
                                    double thickness, const double *rho, double penal,
                                    double E0, double Emin, double *dJ);
/* Asynchronous: one graph launch on the batch's stream. */
int nbg_mixed_batch_launch(nbg_mixed_batch_t *m);
/* Waits for the stream; per-system results and b.u (the compliance F^T u
 * when b is the load vector).  Returns the first error status, else 1 if
 * some system did not converge, else 0. */
int nbg_mixed_batch_results(nbg_mixed_batch_t *m, nbg_mixed_result_t *res, double *J);
int nbg_mixed_batch_tune(nbg_mixed_batch_t *m, uint32_t n_cand, const double *gammas,
                         double *ms);

/* ------------------------------------------------- host-buffer solver */
/* A CSR system in host memory (nb_sparse_create layout) solved on the GPU.
 * Device buffers persist in the context between calls; with
 * NBG_PATTERN_SAME a call re-sends only the values. */
#define NBG_METHOD_NBOTS 0   /* nbots' iteration in FP64 (nbg_cg_f64) */
#define NBG_METHOD_FP64 1    /* fast FP64 on the block layout (nbg_cg_bsr_f64) */
#define NBG_METHOD_MIXED 2   /* mixed precision, FP64 reliable updates (nbg_cg_mixed) */
#define NBG_METHOD_NBOTS_FAST 3  /* nbots' iteration and stop test on the block layout
                                  * (nbg_cg_bsr_f64 with NBG_CG_NBOTS_STOP) */
#define NBG_PATTERN_SAME 1u  /* same pattern as the previous call: send values only */
#define NBG_CSR_ONLY 2u      /* skip the block layout (only NBG_METHOD_NBOTS will run) */

typedef struct {
    uint32_t niter;
    uint32_t n_updates;    /* mixed precision: FP64 residual recomputations */
    int status;
    double relres;         /* final ||r|| / ||b|| the solver judged */
    double tol_reached;    /* final ||r|| */
} nbg_solve_info_t;

typedef struct nbg_solver nbg_solver_t;
int nbg_solver_create(nbg_solver_t **out, void *stream);
void nbg_solver_destroy(nbg_solver_t *s);
/* val NULL: the pattern only; the device values are left for the caller to
 * write (nbg_solver_device_csr, then nbg_solver_values_changed). */
int nbg_solver_set_matrix(nbg_solver_t *s, uint32_t N, const uint32_t *row_ptr,
                          const uint32_t *col_idx, const double *val, unsigned flags);
/* x holds x0 on entry and the solution on return (host memory). */
int nbg_solver_solve(nbg_solver_t *s, const double *b, double *x, uint32_t max_iter,
                     double tol, unsigned flags, int method, nbg_solve_info_t *info);

/* y = A x with nbots' row sums (nbg_spmv_csr_f64, bit-exact) on the
 * solver's matrix; in and out in host memory. */
int nbg_solver_multiply(nbg_solver_t *s, const double *in, double *out);
/* Device pointers of the solver's CSR (valid until the next set_matrix with a
 * new pattern or destroy); any output may be NULL.  A caller that writes
 * new values into *val on the device calls nbg_solver_values_changed so the
 * block layout follows. */
int nbg_solver_device_csr(nbg_solver_t *s, const uint32_t **row_ptr, const uint32_t **col_idx,
                          double **val);
int nbg_solver_values_changed(nbg_solver_t *s);
/* The solver's block layout (current with its values), or NBG_ERR_PATTERN
 * when the pattern is not node-blocked (two rows per node with the same
 * column pairs) or NBG_CSR_ONLY was set. */
int nbg_solver_block_layout(nbg_solver_t *s, nbg_bsr_t *out);
/* Device bytes the solver holds (matrix, block layout, vectors, workspace). */
size_t nbg_solver_device_bytes(const nbg_solver_t *s);

/* Page-locked host memory (for asynchronous copies). */
int nbg_host_alloc(void **ptr, size_t bytes);
int nbg_host_free(void *ptr);

/* ============================================================ host layer */
/* Mesh arrays on the host, nbots' layout (mshquad_struct.h:6-26,
 * msh3trg_struct.h:6-23): coordinates nod[2 i], connectivity conn[e nen + k]
 * counter-clockwise, edges edg[2 i]. */
typedef struct {
    uint32_t nen, N_nod, N_elem, N_edg;
    const double *nod;
    const uint32_t *conn;
    const uint32_t *edg;
} nbg_mesh_t;

/* One nbots bc atom (bc_atom.h:7-12, pushed by nb_bcond_push / _function):
 * kind 0 Dirichlet / 1 Neumann; where 0 input vertex / 1 input segment.
 * A function-valued atom carries its values where nbots evaluates them:
 * one row per segment node, or one row for a vertex (Neumann vertex loads
 * are read at (0,0), set_bconditions.c:156-171). */
typedef struct {
    uint32_t kind, where, id;
    uint8_t mask[2];
    double val[2];
    uint32_t n_nv;
    const double *node_vals;
} nbg_bc_t;

typedef struct {
    const uint32_t *vtx;        /* input vertex -> node */
    uint32_t N_sgm;
    const uint32_t *sgm_ptr;    /* N_sgm + 1 offsets into sgm_nodes */
    const uint32_t *sgm_nodes;  /* node sequence of each input segment */
    uint32_t N_bc;
    const nbg_bc_t *bc;         /* push order */
} nbg_bcs_t;

/* CSR pattern of nb_sparse_create(nodal graph, NULL, 2) (load_graph.c:230-328,
 * sparse.c:20-60).  row_ptr has 2 N_nod + 1 entries; with col_idx NULL only
 * row_ptr is filled (its last entry is nnz). */
int nbg_host_pattern(const nbg_mesh_t *m, uint32_t *row_ptr, uint32_t *col_idx);

/* The same three structures built on the device from device copies of the
 * connectivity and edges (pattern.cu): row_ptr[2 N_nod + 1], the incidence
 * (inc_ptr[N_nod + 1], inc_elem and inc_local [nen N_elem]) and, when
 * slice_off is not NULL, the block plan slice_off[ceil(N_nod / 32) + 1].
 * col_idx is allocated here (nbg_dev_alloc-compatible; free it with
 * nbg_dev_free) and *nnz set.  Word for word equal to nbg_host_pattern,
 * nbg_host_incidence and nbg_bsr_plan.  A node index out of range returns
 * NBG_ERR_ARG before anything is written. */
int nbg_pattern_dev(uint32_t nen, uint32_t N_nod, uint32_t N_elem, uint32_t N_edg,
                    const uint32_t *conn, const uint32_t *edg, uint32_t *row_ptr,
                    uint32_t **col_idx, uint64_t *nnz, uint32_t *inc_ptr, uint32_t *inc_elem,
                    uint8_t *inc_local, uint32_t *slice_off, void *stream);

/* Node -> (element, local node) incidence in ascending element order. */
int nbg_host_incidence(const nbg_mesh_t *m, uint32_t *inc_ptr, uint32_t *inc_elem,
                       uint8_t *inc_local);

/* Device-resident FEM system of one mesh: pattern, K, F, u, strain. */
typedef struct nbg_fem nbg_fem_t;

int nbg_fem_create(nbg_fem_t **out, const nbg_mesh_t *m, void *stream);
void nbg_fem_destroy(nbg_fem_t *f);
uint32_t nbg_fem_n_dof(const nbg_fem_t *f);
uint64_t nbg_fem_nnz(const nbg_fem_t *f);
/* pipeline_assemble_system with one modulus per element (host arrays;
 * enabled may be NULL).  Returns 0, NBG_DISTORTED, or an error. */
int nbg_fem_assemble(nbg_fem_t *f, const double *E, double nu, double thickness,
                     double density, int self_weight, const double gravity[2],
                     const uint8_t *enabled);
/* nb_fem_set_bconditions(mesh, K, F, bcond, factor) */
int nbg_fem_apply_bcs(nbg_fem_t *f, const nbg_bcs_t *b, double factor);
/* Jacobi-PCG on the assembled system, x0 = 0 (static_elasticity2D.c:83-97). */
int nbg_fem_solve(nbg_fem_t *f, uint32_t max_iter, double tol, unsigned flags,
                  nbg_cg_result_t *res);
/* The block layout of K (refilled from the current K values). */
int nbg_fem_block_layout(nbg_fem_t *f, nbg_bsr_t *out);
/* Node order of the block layout, fixed at the first nbg_fem_block_layout.
 * SIGMA sorts each window of `sigma` nodes (0: 512, at most 1024) by row
 * length.  AUTO is the mesh order: on the 4M-dof T3 L-shape the sigma order
 * cuts the padding from 44 % to 4 % and the FP64 CG's time per iteration by
 * 7-8 %, but the mixed solver's time per iteration rises by 6-8 % at every
 * sigma from 64 to 512 (its gathers lose locality), so it is taken only on
 * request. */
#define NBG_ORDER_AUTO 0
#define NBG_ORDER_MESH 1
#define NBG_ORDER_SIGMA 2
int nbg_fem_set_block_order(nbg_fem_t *f, int order, uint32_t sigma);
/* Fast FP64 CG and mixed-precision CG on the assembled system, x0 = 0. */
int nbg_fem_solve_fast(nbg_fem_t *f, uint32_t max_iter, double tol, unsigned flags,
                       nbg_cg_result_t *res);
int nbg_fem_solve_mixed(nbg_fem_t *f, uint32_t max_iter, double tol, double delta,
                        unsigned flags, nbg_mixed_result_t *res);
int nbg_fem_strain(nbg_fem_t *f);
int nbg_fem_stress(nbg_fem_t *f);
/* Principal stresses from the current stress (NBG_FEM_MAIN_STRESS). */
int nbg_fem_main_stress(nbg_fem_t *f);

/* ---------------------------------------------------- quasi-static damage */
typedef struct {
    uint32_t iterations;    /* residual evaluations, all load steps */
    uint32_t cg_solves;     /* conjugate-gradient solves */
    uint32_t cg_iterations; /* their iterations, summed */
    uint32_t gs_fallbacks;  /* solves handed to Gauss-Seidel */
    uint32_t gs_failures;   /* Gauss-Seidel runs that did not converge */
    double residual;        /* residual norm at the end of the last step */
} nbg_damage_info_t;

/* nb_fem_compute_2D_Non_Linear_Solid_Mechanics with the conjugate-gradient
 * solver (static_damage2D.c:239-470) for one plane-stress material with
 * traction limit ft and fracture energy gf: n_steps load steps with factor
 * (n+1)/n_steps, each iterating assembly with damage, boundary conditions,
 * residual F - K u, Jacobi-PCG (x0 = the step's last increment, max N
 * iterations, absolute tolerance 1e-8; Gauss-Seidel with 60 N sweeps when it
 * fails), u += du, strain and damage, until the residual is below rtol
 * (after the first iteration), max_iter iterations, or max_iter_noenh
 * iterations without a new best residual.  Appends nbots' log lines to
 * `logfile` (NULL: no log).  Displacements end in NBG_FEM_U, damage in
 * NBG_FEM_DAMAGE, strain in NBG_FEM_STRAIN.  Returns 0, NBG_DISTORTED, or an
 * error; Gauss-Seidel stops with NBG_ERR_TIMEOUT after 600 s.  method: the
 * inner solver, NBG_METHOD_NBOTS (nbots' arithmetic and iteration on the
 * CSR), NBG_METHOD_NBOTS_FAST (nbots' iteration and stop test on the block
 * layout, refilled after every assembly; the drop-in's choice) or
 * NBG_METHOD_FP64 (the fast FP64 CG on the block layout, stopping on the
 * current residual norm, confirmed on the true residual). */
int nbg_fem_damage(nbg_fem_t *f, const nbg_bcs_t *bcs, double E, double nu, double thickness,
                   double density, int self_weight, const double gravity[2], double ft,
                   double gf, uint32_t n_steps, uint32_t max_iter, uint32_t max_iter_noenh,
                   double rtol, int method, const char *logfile, nbg_damage_info_t *info);

/* ------------------------------------------------------------------ SIMP */
/* SIMP element sensitivities (no counterpart in nbots): with
 * E_e = Emin + rho_e^p (E0 - Emin), out[e] = -p rho_e^(p-1) (E0 - Emin)
 * a_e^T Ke0_e b_e, Ke0_e the element stiffness for E = 1 (device arrays). */
int nbg_simp_sensitivity_f64(uint32_t nen, uint32_t N_elem, const double *nod,
                             const uint32_t *conn, double nu, double thickness,
                             const double *rho, double penal, double E0, double Emin,
                             const double *a, const double *b, double *out, void *stream);
/* The SIMP moduli E[e] = Emin + rho[e]^p (E0 - Emin) (device arrays). */
int nbg_simp_modulus_f64(uint32_t N_elem, const double *rho, double penal, double E0,
                         double Emin, double *E, void *stream);

#define NBG_SIMP_COMPLIANCE 0   /* J = F^T u (self-adjoint) */
#define NBG_SIMP_DOF 1          /* J = u[dof], one adjoint solve K lambda = e_dof */

typedef struct {
    double J;
    uint32_t fwd_iters, adj_iters;
    int status;
} nbg_simp_info_t;

/* Objective and its gradient for densities rho (host arrays): assemble with
 * E(rho), apply the boundary conditions (homogeneous Dirichlet values),
 * solve K u = F (and K lambda = e_dof) with `method` (NBG_METHOD_FP64 or
 * NBG_METHOD_MIXED) to relative tolerance tol, write dJ/drho to dJ.  Returns
 * 0, 1 when a solve stopped short of tol (at the solver's iteration limit
 * or FP64 floor; J and dJ are still computed from it), or an error. */
int nbg_fem_simp(nbg_fem_t *f, const nbg_bcs_t *bcs, const double *rho, double nu,
                 double thickness, double penal, double E0, double Emin, int objective,
                 uint32_t dof, double tol, int method, double *dJ, nbg_simp_info_t *info);

#define NBG_FEM_ROW_PTR 0   /* uint32[N+1] */
#define NBG_FEM_COL_IDX 1   /* uint32[nnz] */
#define NBG_FEM_K 2         /* double[nnz] */
#define NBG_FEM_F 3         /* double[N] */
#define NBG_FEM_U 4         /* double[N] */
#define NBG_FEM_STRAIN 5    /* double[3 N_gp N_elem] */
#define NBG_FEM_STRESS 6    /* double[3 N_gp N_elem] */
#define NBG_FEM_E 7         /* double[N_elem] */
#define NBG_FEM_NOD 8       /* double[2 N_nod] */
#define NBG_FEM_CONN 9      /* uint32[nen N_elem] */
#define NBG_FEM_MAIN_STRESS 10  /* double[2 N_gp N_elem] */
#define NBG_FEM_DAMAGE 11   /* double[N_gp N_elem], after nbg_fem_damage */
/* Device pointer of one array, and a copy of it to host memory. */
void *nbg_fem_device_ptr(nbg_fem_t *f, int what);
size_t nbg_fem_bytes(const nbg_fem_t *f, int what);
int nbg_fem_download(nbg_fem_t *f, int what, void *host);
int nbg_fem_upload(nbg_fem_t *f, int what, const void *host);

/* ----------------------------------------------------------------- batch */
/* Independent FEM problems (meshes of uneven size, each with its own
 * boundary conditions, densities and loads) merged into one block-diagonal
 * system and solved side by side by nbg_mixed_batch_* with the SIMP
 * compliance sensitivities, one CUDA graph per launch.  Instance k's nodes
 * start at node_off[k], a multiple of 32; the padding nodes before the next
 * instance are fixed by Dirichlet conditions (identity rows, zero load).
 * Each instance's K and F equal, bit for bit, those nbg_fem_* builds for it
 * alone.  The mesh and bc arrays are copied at creation.  All meshes share
 * one element type.  No counterpart in nbots. */
typedef struct nbg_batch nbg_batch_t;
int nbg_batch_create(nbg_batch_t **out, uint32_t n_inst, const nbg_mesh_t *meshes,
                     const nbg_bcs_t *bcs, void *stream);
void nbg_batch_destroy(nbg_batch_t *b);
uint32_t nbg_batch_size(const nbg_batch_t *b);
/* n_inst + 1 offsets each (node_off in nodes, elem_off in elements);
 * either may be NULL. */
int nbg_batch_offsets(const nbg_batch_t *b, uint32_t *node_off, uint32_t *elem_off);
nbg_fem_t *nbg_batch_fem(nbg_batch_t *b);
nbg_mixed_batch_t *nbg_batch_solver(nbg_batch_t *b);
/* E = Emin + rho^p (E0 - Emin) per merged element (host array), assembly,
 * every instance's boundary conditions (factor 1), block layout. */
int nbg_batch_assemble_simp(nbg_batch_t *b, const double *rho, double nu, double thickness,
                            double penal, double E0, double Emin);
/* (Re)creates the batched solver on the assembled system: mixed CG per
 * instance, NBG_CG_RELATIVE in flags for ||r|| <= tol ||F_k||. */
int nbg_batch_setup(nbg_batch_t *b, uint32_t max_iter, double tol, double delta,
                    unsigned flags);
/* One graph launch (asynchronous): u = 0, solve, sensitivities. */
int nbg_batch_launch(nbg_batch_t *b);
/* Waits; per-instance results and compliance F_k^T u_k. */
int nbg_batch_results(nbg_batch_t *b, nbg_mixed_result_t *res, double *J);
/* dJ/drho of each instance's compliance, per merged element (host array). */
int nbg_batch_sensitivities(nbg_batch_t *b, double *dJ);

#ifdef __cplusplus
}
#endif
#endif
