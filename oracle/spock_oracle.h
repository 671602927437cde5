/*
 * FP64 CPU oracle for the SPOCK solve -- TEST INFRASTRUCTURE ONLY.
 *
 * This is the checker: a plain-C restatement of the reference solver's algorithm
 * (ruairimoran/spock.cu, src/cache.cuh, src/operator.cuh, src/costs.cuh, src/constraints.cuh,
 * src/dynamics.cuh, src/risks.cuh, src/projections.cuh, src/definitions.cu) and of its offline
 * factory (api/python/spock/problem.py, build.py).  Only tests/, the smoke entry point and the
 * benchmark's CPU-baseline leg may load it; the product library never calls into it.
 *
 * Parity pins: the fixtures under tests/golden/ written by the reference's own Python factory (operator
 * and adjoint fixtures, M-inner product, offline cache tensors, step size) and the literal
 * known answers of the reference's CUDA tests (SOC projections, AVaR index pattern, box clamp).
 */
#ifndef SPOCK_ORACLE_H
#define SPOCK_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrProblem OrProblem;

/* Load `data.json` + `*_d.bt` / `*_u.bt` from a data folder (path ends with '/').
 * Returns NULL on error; or_last_error() explains. */
OrProblem *or_load(const char *path);
void or_free(OrProblem *p);
const char *or_last_error(void);

/* Sizes: [numNodes, numNonleaf, numStages, nx, nu, numEvents, yDim, nullDim,
 *         sizePrim, sizeDual, preconditioned]  */
void or_sizes(const OrProblem *p, long *out11);
double or_step_size(const OrProblem *p);
void or_scaling(const OrProblem *p, double *out_nx_plus_nu);

/* Linear operator L (prim -> dual) and its adjoint (dual -> prim), operator.cuh:40-82. */
void or_op(const OrProblem *p, const double *prim, double *dual);
void or_adj(const OrProblem *p, const double *dual, double *prim);

/* Pieces of the CP step. x0 is the (already scaled) initial state. */
void or_project_dynamics(const OrProblem *p, const double *x0, double *x, double *u);
void or_project_kernel(const OrProblem *p, double *y, double *t, double *s);
void or_project_dual(const OrProblem *p, double *dual);           /* projection onto C */
void or_cp_step(const OrProblem *p, const double *x0s, const double *z, double *cand);
double or_dot_m(const OrProblem *p, const double *x, const double *y);

/* Elementwise primitives (definitions.cu kernels). */
void or_project_soc_columns(double *data, long dim, long ncones);
void or_project_box(double *v, const double *lb, const double *ub, long n);

/* Solver options (CacheBuilder defaults, cache.cuh:1154-1163). */
typedef struct {
    double tol_abs, tol_rel, max_time_secs;
    long max_outer, max_inner, anderson;
} OrOptions;

typedef struct {
    int status;          /* -1 notRun, 0 converged, 1 outOfIter, 2 outOfTime */
    long iters;          /* outer iterations (solveIter) */
    long calls_T;        /* CP operator evaluations */
    long k0, k1, k2, k2bt, k3;
    double tol, err;
    double seconds;
} OrStats;

/* runSpock / runCp (cache.cuh:967-1132).  x0 unscaled (as the user passes it); z has size
 * sizePrim+sizeDual and holds the warm start if warm != 0 (else it is zeroed); on return z
 * is the solution iterate (scaled variables, exactly like Cache::solution()). */
int or_run_spock(const OrProblem *p, const OrOptions *o, const double *x0, double *z, int warm, OrStats *st);
int or_run_cp(const OrProblem *p, const OrOptions *o, const double *x0, double *z, int warm, OrStats *st);

/* Unscaled states (nx*numNodes) and inputs (nu*numNonleaf) of an iterate (cache.cuh:386-412). */
void or_states_inputs(const OrProblem *p, const double *z, double *states, double *inputs);

/* Solve `count` instances (x0s: count*nx) over `threads` POSIX threads; writes statuses,
 * iteration counts and the first-stage input of each instance (count*nu).  Returns wall s. */
double or_solve_many(const OrProblem *p, const OrOptions *o, long count, const double *x0s,
                     int threads, int *status, long *iters, double *u0, double *zs_or_null);
/* Same; with warm != 0 each instance starts from its iterate in zs (count*sZ, required) -- the
 * previousSolution warm start of cache.cuh:611-632 -- and zs receives the solutions.  calls, if
 * not NULL, receives each instance's number of T evaluations. */
double or_solve_many_warm(const OrProblem *p, const OrOptions *o, long count, const double *x0s,
                          int threads, int *status, long *iters, double *u0, double *zs, int warm,
                          long *calls);

/* Offline dynamics cache (problem.py:192-213) from per-node [A B] (nx x (nx+nu) x n):
 * writes P (nx*nx*n), K (nu*nx*nnl), lowChol (nu*nu*nnl), ABKTr (nx*nx*n), APB (nx*nu*n). */
void or_offline_dynamics(const OrProblem *p, const double *AB, double *P, double *K,
                         double *lowChol, double *ABKTr, double *APB);
/* AVaR nullspace projector for node i (problem.py:215-231); out nullDim x nullDim. */
void or_offline_kernel(const OrProblem *p, double alpha, long node, double *nntr);
/* Largest eigenvalue of L*L by power iteration (problem.py:402-417 computes it with ARPACK). */
double or_norm_L_sq(const OrProblem *p, long iters);

/* FP32 emulation (process-wide; 0 = plain FP64, the default).  Explains how single-precision
 * arithmetic changes the iteration's path, without a GPU:
 *   OR_EMU_DATA   problem data rounded to float when a problem is loaded (set before or_load);
 *   OR_EMU_ACC    every small matrix-vector product accumulated with float FMAs;
 *   OR_EMU_VEC    every vector of the CP step and of the SuperMann loop stored as float;
 *   OR_EMU_GRAM   Anderson by normal equations: float-accumulated Gram matrix, ridge 1e-7 x its
 *                 largest diagonal entry, FP64 Cholesky (instead of Householder QR);
 *   OR_EMU_FWD64  the forward rollout of the dynamics projection accumulated in double;
 *   OR_EMU_FWDC   the forward rollout accumulated in float with compensation (the Dot2
 *                 algorithm: error-free products by FMA, TwoSum additions);
 *   OR_EMU_FWDCX  the same for the children's states [A B][x; u] only (u = Kx + d plain);
 *   OR_EMU_FWDK   the forward rollout with Kahan's compensated summation of the rounded float
 *                 products (half the operations of Dot2; the products' own errors remain);
 *   OR_EMU_ACCX_OPS   L and L* accumulate exactly although OR_EMU_ACC is set;
 *   OR_EMU_ACCX_BACK  the dynamics projection's backward sweep accumulates exactly although
 *                     OR_EMU_ACC is set. */
enum { OR_EMU_DATA = 1, OR_EMU_ACC = 2, OR_EMU_VEC = 4, OR_EMU_GRAM = 8, OR_EMU_FWD64 = 16, OR_EMU_FWDC = 32,
       OR_EMU_FWDCX = 64, OR_EMU_FWDK = 128, OR_EMU_ACCX_OPS = 256, OR_EMU_ACCX_BACK = 512 };
void or_set_emulation(int mode);

#ifdef __cplusplus
}
#endif
#endif
