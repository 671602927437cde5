/*
 * spock_gb300 -- C ABI of the GB300-native SPOCK solver (risk-averse optimal control on
 * scenario trees, SuperMann-accelerated Chambolle-Pock).
 *
 * Every entry point takes plain pointers and sizes and returns 0 on success or a nonzero
 * SPOCK_E_* code; spock_last_error() then returns the message (thread-local).  The C++
 * wrapper include/spock_gb300.hpp rebuilds the reference's class interface on top of this.
 *
 * Each declaration names the reference interface it replaces (ruairimoran/spock.cu).
 */
#ifndef SPOCK_GB300_H
#define SPOCK_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define SPOCK_OK 0
#define SPOCK_E_INVALID 1  /* invalid argument / malformed data folder (std::invalid_argument) */
#define SPOCK_E_CUDA 2     /* CUDA runtime failure */
#define SPOCK_E_UNKNOWN 3

/* Exit statuses of a solve (src/cache.cuh:68-73), plus 3 = stopped on a non-finite residual. */
#define SPOCK_NOT_RUN (-1)
#define SPOCK_CONVERGED 0
#define SPOCK_OUT_OF_ITER 1
#define SPOCK_OUT_OF_TIME 2
#define SPOCK_DIVERGED 3

#define SPOCK_ALGO_SPOCK 0 /* Cache::runSpock (src/cache.cuh:1008-1132) */
#define SPOCK_ALGO_CP 1    /* Cache::runCp    (src/cache.cuh:967-1002) */

typedef struct spock_problem_s *spock_problem; /* ScenarioTree<T> + ProblemData<T> */
typedef struct spock_solver_s *spock_solver;   /* Cache<T> (one or a batch of instances) */

/* Solver options: the CacheBuilder setters (src/cache.cuh:1154-1210). */
typedef struct {
    double tol_abs;        /* toleranceAbsolute (default 1e-3) */
    double tol_rel;        /* toleranceRelative (default 0) */
    double max_time_secs;  /* maxTimeSecs (0 = none) */
    long max_iters;        /* maxIters, outer iterations (0 = unlimited) */
    long max_inner;        /* maxItersInner (default 8) */
    long anderson;         /* andersonBuffer (default 3, at most 8) */
    int precision;         /* 64 (double, the reference's T=double) or 32 (float) */
    long batch;            /* number of instances solved together (>= 1) */
    int device;            /* CUDA device ordinal */
} spock_options;

/* Fills the CacheBuilder defaults (src/cache.cuh:1154-1163): tol_abs 1e-3, tol_rel 0,
 * max_inner 8, anderson 3; precision 64, batch 1, device 0. */
void spock_options_default(spock_options *opts);

/* Message of the last failing call on this thread (the reference's static `err` stream,
 * include/gpu.cuh:24-25, without its accumulation). */
const char *spock_last_error(void);

/* Load a data folder written by the offline factory: ScenarioTree<T>(path)
 * (src/tree.cuh:102-179) + ProblemData<T>(tree) (src/problem.cuh:126-153).  Host-side only;
 * device copies are made per solver. */
int spock_problem_load(const char *path, spock_problem *out);
void spock_problem_free(spock_problem p);
/* sizes[10] = numEvents, numNodes, numNonleafNodes, numStages, numStates, numInputs,
 * sizePrimal, sizeDual, preconditioned, nullDim  (tree.cuh:207-229, cache.cuh:367-369) */
int spock_problem_sizes(spock_problem p, long *sizes10);
/* stepSize (problem.cuh:521) and the preconditioning scaling (nx+nu, ones if none). */
int spock_problem_step(spock_problem p, double *step, double *scaling_or_null);

/* The offline cache of the dynamics projection -- P, K, the lower Cholesky factors, (A+BK)' and
 * (A+BK)'PB per node, which the reference computes in numpy when it generates a problem
 * (api/python/spock/problem.py:192-213) -- recomputed on GPU `device` in FP64 from the problem's
 * [A B] and tree.  Outputs (NULL skips one) use the layouts of the dynamics_P, _K, _lowCholesky,
 * _ABKTr and _APB .bt files: nx*nx*numNodes, nu*nx*numNonleaf, nu*nu*numNonleaf, nx*nx*numNodes,
 * nx*nu*numNodes doubles.  With replace != 0 the problem's cache is replaced by this one, so
 * solvers created afterwards use it. */
int spock_offline_dynamics(spock_problem p, int device, int replace, double *P, double *K, double *lowChol,
                           double *ABKTr, double *APB);

/* Complete a data folder whose problem data is written but whose offline cache is not: the
 * GPU half of the reference's Problem constructor (api/python/spock/problem.py:192-231, 402-417),
 * all in FP64 on GPU `device`.  It reads the folder (cache files may be absent, stepSize may be
 * 0), computes the dynamics cache, the AVaR nullspace projectors I - S'(SS')^-1 S and the step
 * size 0.99 / ||L|| (power iteration with the library's L and L*: at most `iters` steps, stopped
 * once the estimate is steady to 1e-14), and writes dynamics_P, _K, _lowCholesky, _ABKTr, _APB,
 * risk_NNtr (with the folder's _d or _f suffix) and data.json's stepSize.  *step (may be NULL)
 * receives the step size. */
int spock_offline_complete(const char *path, int device, int iters, double *step);

/* CacheBuilder<T>(tree, data)...build() (src/cache.cuh:1215-1244). */
int spock_solver_create(spock_problem p, const spock_options *opts, spock_solver *out);
void spock_solver_free(spock_solver s);

/* Cache::runSpock / runCp (src/cache.cuh:967-1132) for every instance of the batch.
 * x0: count*nx host doubles (unscaled, as the user passes them); instance b uses row
 * b % count.  warm: NULL for a cold start (the reference's reset() + run), else count*(sizePrimal
 * + sizeDual) previous iterates (the `previousSolution` argument).  statuses/iters: batch
 * entries each, may be NULL.  Blocks until every instance has stopped. */
int spock_solve(spock_solver s, int algo, const double *x0, long count, const double *warm, int *statuses, long *iters);
/* Same, with x0 already on the device as nx x batch values of the solver precision laid out
 * element-major (x0[c * batch + b]); results stay on the device until read. */
int spock_solve_device(spock_solver s, int algo, const void *x0_device, int *statuses, long *iters);

/* Mixed batches (instances of different trees and dimensions, one solver per problem): cold-start
 * solves of `count` distinct solvers at once; returns when all have stopped.  SPOCK solves on one
 * device run as one launch sequence: each round is a single CUDA graph holding every running
 * solver's round, so the GPU runs the solvers' kernels side by side (finished solvers leave the
 * graph); CP solves, or solvers on several devices, run one host thread each.  x0s[i] holds
 * x0counts[i] rows for solver i (as spock_solve); statuses[i] / iters[i] (batch entries each) may be
 * NULL, as may statuses / iters.  No reference counterpart. */
int spock_solve_group(long count, spock_solver *solvers, int algo, const double *const *x0s, const long *x0counts,
                      int *const *statuses, long *const *iters);

/* Re-solve every instance warm-started from the solver's current iterate -- the solution of
 * the previous solve, still on the device -- with new initial states: the reference's
 * previousSolution warm start (cache.cuh:611-632) for a control loop that re-solves as the state
 * moves, without sending iterates through the host.  x0 as in spock_solve (host, unscaled) or
 * spock_solve_device (device, solver precision).  After spock_reset the iterate is zero. */
int spock_resolve(spock_solver s, int algo, const double *x0, long count, int *statuses, long *iters);
int spock_resolve_device(spock_solver s, int algo, const void *x0_device, int *statuses, long *iters);

/* Replace dst's iterate by src's, converted on the device to dst's precision: two solvers of the
 * same problem and batch on the same GPU.  With src an FP32 solver and dst an FP64 one, a
 * following spock_resolve(dst, ...) with the same initial states is the FP64 polish of the FP32
 * solution (it continues from it under dst's tolerances).  No reference counterpart. */
int spock_copy_iterate(spock_solver dst, spock_solver src);
/* Replace the solver's iterate by a device array of sizePrimal + sizeDual rows x batch columns,
 * element-major (z[k * batch + b]), FP32 (bits = 32) or FP64 (64), converted on the device; a
 * following spock_resolve starts every instance from it (a warm start predicted on the GPU). */
int spock_set_iterate_device(spock_solver s, const void *z_device, int bits);

/* Results.  Cache::solution() (cache.cuh:378): the raw iterate of one instance, sizePrimal +
 * sizeDual doubles.  Cache::states()/inputs() (cache.cuh:386-412): unscaled, nx*numNodes and
 * nu*numNonleafNodes doubles.  first_inputs: the unscaled u_0 of every instance (batch*nu). */
int spock_get_iterate(spock_solver s, long instance, double *out);
int spock_get_iterates(spock_solver s, double *out_batch_by_size);
int spock_get_states_inputs(spock_solver s, long instance, double *states, double *inputs);
int spock_get_first_inputs(spock_solver s, double *out);
/* status(), solveIter(), solveTime() (cache.cuh:357-361) of one instance. */
int spock_status(spock_solver s, long instance, int *status, long *iters, double *seconds);
/* K0/K1/K2/backtracks/K3 counts, T evaluations and iterations of instance 0 (the debug
 * counters of cache.cuh:1101-1130). */
int spock_counters(spock_solver s, long *out7);
/* The same seven counters for every instance of the batch: batch x 7 values. */
int spock_counters_all(spock_solver s, long *out_batch_by_7);
/* reset() (cache.cuh:436-479): zero the iterate. */
int spock_reset(spock_solver s);

/* Operator-level entry points (the reference tests reach these through friend access,
 * tests/cuda/testOperator.cu, testCache.cu): single instance, host buffers. */
int spock_op(spock_solver s, const double *prim, double *dual);            /* LinearOperator::op  (operator.cuh:40-60) */
int spock_adj(spock_solver s, const double *dual, double *prim);           /* LinearOperator::adj (operator.cuh:62-82) */
int spock_cp_step(spock_solver s, const double *x0, const double *z, double *cand); /* Cache::iter (cache.cuh:795-801) */
int spock_apply_m(spock_solver s, const double *z, double *mz);            /* M of Cache::dotM (cache.cuh:721-734) */
/* Cache::getDual (cache.cuh:371-376): the dual candidate prox_{g*}(z_d + gamma L(2 prim - z_p))
 * for a given primal candidate `prim` (sizePrimal values) at the solver's current iterate z
 * (instance 0; for a batch, every instance gets `prim`); `dual` receives sizeDual values. */
int spock_get_dual(spock_solver s, const double *prim, double *dual);
/* The reductions a SuperMann round makes on the device, for a residual r and M r (sizeIterate
 * values each, instance 0): out3 = {r'Mr (the square of normM, cache.cuh:721-742), max|Mr| (the
 * error check's maximum, cache.cuh:909-961), r'r}, as the controller receives them (FP64 sums of
 * the kernels' partials).  A check of their accuracy for FP32 solvers; no reference counterpart. */
int spock_reduce_check(spock_solver s, const double *r, const double *mr, double *out3);

/* Measurement hooks for the benchmark: CUDA-event time of one launch of a named kernel
 * ("lstar", "lop", "mlstar", "mlop", "dyn", "reduce", "update", "teval", "round"), its
 * algorithmic bytes, and the device time of `rounds` replays of the captured SuperMann round. */
int spock_kernel_time(spock_solver s, const char *which, int reps, double *ms, long *bytes);
int spock_round_time(spock_solver s, int rounds, double *ms);
/* Rounds (one T evaluation + one M application per instance each), kernel launches and instance
 * compactions (running instances moved to the leading slots) of the last solve; NULL skips one. */
int spock_run_stats(spock_solver s, long *rounds, long *launches, long *compactions);
/* Tile shapes the built-in autotuner chose (it times 1, 2, 4 and 8 instance tiles per CTA once,
 * before the first solve): out5 = {L* tiles per CTA, L* double-buffered, L tiles per CTA, L
 * double-buffered, dynamics-sweep tiles per CTA (0 when the small-batch kernels run)}.  No
 * reference counterpart. */
int spock_tuning(spock_solver s, int *out5);
/* The step size gamma = 0.99 / ||L|| that Problem.__get_step_size computes with ARPACK
 * (api/python/spock/problem.py:402-417), here from `iters` steps of the power iteration on
 * lambda_max(L* L) run on the GPU with the solver's own L and L* kernels; outputs may be NULL. */
int spock_step_size(spock_solver s, int iters, double *norm_sq, double *step);

/* Override the autotuner: in3 = {L* tiles per CTA, L tiles per CTA, dynamics-sweep tiles per CTA},
 * each 1, 2, 4 or 8 (double-buffered where two tiles fit in shared memory).  No effect on the
 * small-batch kernels.  No reference counterpart. */
int spock_set_tuning(spock_solver s, const int *in3);

/* FP64 finish of an FP32 batched solver (batch >= 32): once a SPOCK solve has run `rounds`
 * rounds and at most 32 of its instances are still running, those instances move with their
 * whole SuperMann state (iterate, Anderson memory, controller state, tolerance) into an FP64
 * solver of the same problem, made on first use with batch 32, which continues the same
 * iteration in FP64 until they stop; their final iterates, statuses and counters come back.
 * rounds = 0 (the default) turns it off.  No effect on FP64 solvers or batches below 32; where
 * the problem has no FP64 batched kernels (node data beyond their shared memory) the solve
 * continues in FP32 and the finish turns itself off.  No reference counterpart: the reference
 * iterates in one precision (cache.cuh:1008-1132). */
int spock_set_fp64_finish(spock_solver s, long rounds);

/* Dynamics projection that allocates no device memory.  No counterpart in the reference: it
 * is for callers that cannot allocate while they solve, such as a control loop re-solving
 * under a hard deadline (a cudaMalloc's latency or failure is not acceptable there) or a host
 * whose framework owns the device memory pool.  It projects one instance (u, x) onto the
 * dynamics exactly like the projection inside spock_cp_step, in place, with the sweep's
 * workspaces in a static 8 MiB device buffer built into the library.
 *   s: a solver created with batch 1;  x0: the initial state in the solver's (preconditioned)
 *   coordinates, nx device values;  prim_ux: device array [u (nu x numNonleaf) | x (nx x
 *   numNodes)] in the solver precision, the head of a primal vector, overwritten with the
 *   projection;  stream: a cudaStream_t (NULL for the default stream); returns when done (it
 *   synchronises the stream, unless the stream is capturing).  The caller's current device is
 *   the same after the call as before it.
 * Problems whose workspaces (nx*numNodes + nu*numNonleaf values) exceed 8 MiB are rejected
 * with SPOCK_E_INVALID.  The first call on a device looks up the buffer's device address (with
 * the CUDA runtime's lazy module loading, that is also when the 8 MiB are placed on the
 * device), so make that first call before any stream capture.  All calls share the one buffer: calls that
 * overlap on the GPU (other threads, other streams) race with each other. */
int spock_project_dynamics_noalloc(spock_solver s, const void *x0, void *prim_ux, void *stream);

/* ---- Tensor-core GEMM and the learned warm start's reconstruction (no reference counterpart).
 * spock_gemm_bf16: D = alpha A B' (+ rowAdd[m]) (+ colAdd[n]) on the tcgen05 tensor cores, A
 * (M x K) and B (N x K) BF16 device arrays, row-major with K contiguous, K a multiple of 64,
 * FP32 accumulation; D (FP32 row-major M x N, leading dimension ldd) gets the sum and Dact its
 * GELU (tanh form) when gelu is nonzero; either may be NULL.  Synchronous on `device`.
 * spock_warm_start_pca: sets a solver's iterate to mean + basis coef' (basis: sizeIterate x
 * k, coef: batch x k, BF16 row-major, k a multiple of 64; mean: sizeIterate FP32 values, all
 * device arrays) with the same GEMM writing the solver's element-major iterate directly; then
 * re-solve with spock_resolve. */
int spock_gemm_bf16(const void *A, const void *B, long M, long N, int K, float alpha, const float *rowAdd,
                    const float *colAdd, int gelu, float *D, float *Dact, long ldd, int device);
int spock_warm_start_pca(spock_solver s, const void *basis, const void *coef, int k, const float *mean);

/* ---- Learned warm start (no reference counterpart).  A three-layer MLP x0 -> coefficients of a
 * solution basis, trained and evaluated by the library's own kernels: dims4 = {inputs, hidden,
 * hidden, outputs}; GELU (tanh form) after the two hidden layers; BF16 weight copies read by every
 * product, FP32 master weights updated by Adam, FP32 accumulation.  Tensors are column-major
 * float device arrays with one sample per column.  Parameters pack W1 (d1 x d0), b1, W2 (d2 x d1),
 * b2, W3 (d3 x d2), b3. */
typedef struct spock_mlp_s *spock_mlp;
int spock_mlp_create(const int *dims4, int device, spock_mlp *out);
void spock_mlp_free(spock_mlp m);
long spock_mlp_param_count(spock_mlp m);
int spock_mlp_set_params(spock_mlp m, const float *params);              /* host -> master + BF16 */
int spock_mlp_get_params(spock_mlp m, float *params, float *grads);       /* host copies; NULL skips */
int spock_mlp_forward(spock_mlp m, const void *x_device, int cols, void *y_device);
/* forward, mean-squared-error gradient against t_device (d3 x cols), and an Adam step (lr > 0;
 * lr = 0 only computes the gradients); *loss = mean squared error before the step. */
int spock_mlp_train_step(spock_mlp m, const void *x_device, const void *t_device, int cols, float lr, float *loss);

#ifdef __cplusplus
}
#endif
#endif
