// C ABI (include/spock_gb300.h) over the engine.  Exceptions never cross the boundary:
// they become SPOCK_E_* codes with the message kept for spock_last_error().
#include "../../include/spock_gb300.h"

#include <cmath>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "capi_internal.hpp"
#include "engine.cuh"
#include "offline.hpp"
#include "problem.hpp"

struct spock_problem_s {
    spock::HostProblem hp;
};

struct spock_solver_s {
    std::unique_ptr<spock::EngineBase> eng;
    std::vector<int> status;
    std::vector<long> iters;
    double seconds = 0;
};

namespace {
thread_local std::string g_error;

template <typename F>
int guard(F &&f) {
    try {
        f();
        return SPOCK_OK;
    } catch (const std::invalid_argument &e) {
        g_error = e.what();
        return SPOCK_E_INVALID;
    } catch (const std::runtime_error &e) {
        g_error = e.what();
        return SPOCK_E_CUDA;
    } catch (const std::exception &e) {
        g_error = e.what();
        return SPOCK_E_UNKNOWN;
    } catch (...) {
        g_error = "unknown error";
        return SPOCK_E_UNKNOWN;
    }
}

void need(const void *p, const char *what) {
    if (!p) throw std::invalid_argument(std::string("[spock] null argument: ") + what);
}

spock_solver_s *solver(spock_solver s) {
    need(s, "solver");
    return s;
}

// Take over a freshly computed dynamics cache, with Pe = P e per node for affine dynamics
// (dynamics.cuh:236).
void adoptCache(spock::HostProblem &hp, const spock::OfflineCache &c) {
    hp.P = c.P;
    hp.K = c.K;
    hp.lowChol = c.lowChol;
    hp.ABKTr = c.ABKTr;
    hp.APB = c.APB;
    if (hp.affine) {
        const long n = hp.numNodes, nx = hp.nx;
        hp.Pe.assign((size_t)(nx * n), 0.);
        for (long j = 0; j < n; j++)
            for (long col = 0; col < nx; col++)
                for (long r = 0; r < nx; r++) hp.Pe[j * nx + r] += hp.P[j * nx * nx + col * nx + r] * hp.e[j * nx + col];
    }
}
}  // namespace

extern "C" {

void spock_options_default(spock_options *o) {
    if (!o) return;
    o->tol_abs = 1e-3;
    o->tol_rel = 0.;
    o->max_time_secs = 0.;
    o->max_iters = 0;
    o->max_inner = 8;
    o->anderson = 3;
    o->precision = 64;
    o->batch = 1;
    o->device = 0;
}

const char *spock_last_error(void) { return g_error.c_str(); }

int spock_problem_load(const char *path, spock_problem *out) {
    return guard([&] {
        need(path, "path");
        need(out, "out");
        auto p = std::make_unique<spock_problem_s>();
        p->hp = spock::HostProblem::load(path);
        *out = p.release();
    });
}

void spock_problem_free(spock_problem p) { delete p; }

int spock_problem_sizes(spock_problem p, long *s) {
    return guard([&] {
        need(p, "problem");
        need(s, "sizes");
        const auto &h = p->hp;
        long v[10] = {h.numEvents, h.numNodes, h.numNonleaf, h.numStages, h.nx, h.nu, h.sizePrim, h.sizeDual,
                      h.preconditioned ? 1L : 0L, h.nullDim};
        std::memcpy(s, v, sizeof v);
    });
}

int spock_problem_step(spock_problem p, double *step, double *scaling) {
    return guard([&] {
        need(p, "problem");
        if (step) *step = p->hp.stepSize;
        if (scaling) std::memcpy(scaling, p->hp.scaling.data(), sizeof(double) * p->hp.scaling.size());
    });
}

int spock_solver_create(spock_problem p, const spock_options *o, spock_solver *out) {
    return guard([&] {
        need(p, "problem");
        need(out, "out");
        spock_options def;
        spock_options_default(&def);
        if (!o) o = &def;
        if (o->tol_abs < 0 || o->tol_rel < 0 || o->max_time_secs < 0 || o->max_iters < 0 || o->max_inner < 1)
            throw std::invalid_argument("[CacheBuilder] negative tolerance/time/iterations");
        spock::Options opt;
        opt.tolAbs = o->tol_abs;
        opt.tolRel = o->tol_rel;
        opt.maxTimeSecs = o->max_time_secs;
        opt.maxOuter = o->max_iters;
        opt.maxInner = o->max_inner;
        opt.anderson = o->anderson;
        auto s = std::make_unique<spock_solver_s>();
        s->eng.reset(spock::makeEngine(p->hp, opt, o->batch, o->precision, o->device));
        s->status.assign(o->batch, SPOCK_NOT_RUN);
        s->iters.assign(o->batch, 0);
        *out = s.release();
    });
}

void spock_solver_free(spock_solver s) { delete s; }

static void finishSolve(spock_solver_s *s, int *statuses, long *iters) {
    s->eng->getStatus(s->status.data(), s->iters.data());
    s->seconds = s->eng->lastSeconds();
    const long B = s->eng->batch();
    for (long b = 0; b < B; b++) {
        if (statuses) statuses[b] = s->status[b];
        if (iters) iters[b] = s->iters[b];
    }
}

int spock_solve(spock_solver sv, int algo, const double *x0, long count, const double *warm, int *statuses, long *iters) {
    return guard([&] {
        auto *s = solver(sv);
        need(x0, "x0");
        if (algo != SPOCK_ALGO_SPOCK && algo != SPOCK_ALGO_CP) throw std::invalid_argument("[Cache] unknown algorithm");
        s->eng->setInitialStates(x0, count);
        if (warm) s->eng->setIterate(warm, count);
        s->eng->run(algo == SPOCK_ALGO_SPOCK ? spock::kSpock : spock::kCp, warm != nullptr);
        finishSolve(s, statuses, iters);
    });
}

int spock_solve_device(spock_solver sv, int algo, const void *x0, int *statuses, long *iters) {
    return guard([&] {
        auto *s = solver(sv);
        need(x0, "x0");
        s->eng->setInitialStatesDevice(x0, s->eng->batch());
        s->eng->run(algo == SPOCK_ALGO_SPOCK ? spock::kSpock : spock::kCp, false);
        finishSolve(s, statuses, iters);
    });
}

int spock_offline_dynamics(spock_problem pp, int device, int replace, double *P, double *K, double *lowChol,
                           double *ABKTr, double *APB) {
    return guard([&] {
        need(pp, "problem");
        spock::HostProblem &hp = pp->hp;
        spock::OfflineCache c = spock::offlineDynamicsGpu(hp, device);
        auto put = [](const std::vector<double> &v, double *out) {
            if (out) std::memcpy(out, v.data(), sizeof(double) * v.size());
        };
        put(c.P, P);
        put(c.K, K);
        put(c.lowChol, lowChol);
        put(c.ABKTr, ABKTr);
        put(c.APB, APB);
        if (replace) adoptCache(hp, c);
    });
}

int spock_offline_complete(const char *path, int device, int iters, double *step) {
    return guard([&] {
        need(path, "path");
        if (iters < 1) throw std::invalid_argument("[offlineComplete] iters must be positive");
        spock::HostProblem hp = spock::HostProblem::load(path, true);
        adoptCache(hp, spock::offlineDynamicsGpu(hp, device));
        hp.NNtr = spock::offlineNullspaceGpu(hp, device);
        // ||L||^2 does not depend on the step size; the engine wants a positive one to start
        if (!(hp.stepSize > 0)) hp.stepSize = 1.;
        spock::Options opt;
        std::unique_ptr<spock::EngineBase> eng(spock::makeEngine(hp, opt, 1, 64, device));
        const double lam = eng->normLsq(iters, 1e-14);
        eng.reset();
        if (!(lam > 0)) throw std::invalid_argument("[offlineComplete] ||L|| is zero");
        hp.stepSize = 0.99 / std::sqrt(lam);
        spock::writeOfflineCache(hp);
        if (step) *step = hp.stepSize;
    });
}

// Active instances of each solver of a group: out[e] = number of statuses -1 of solver e.
__global__ void k_group_active(const int *const *status, const long *batch, int count, int *out) {
    const int e = blockIdx.x;
    if (e >= count) return;
    int c = 0;
    for (long b = threadIdx.x; b < batch[e]; b += blockDim.x) c += status[e][b] == -1;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    __shared__ int part[32];
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += part[w];
        out[e] = s;
    }
}

#define GCK(x)                                                                                     \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess) throw std::runtime_error(std::string("[solveGroup] ") + cudaGetErrorString(e_)); \
    } while (0)

// SPOCK solves of several solvers (different problems, one device) as one launch sequence: every
// round is a single CUDA graph holding each still-running solver's captured round as a child
// graph, so the solvers' node kernels run side by side; every 10 rounds one kernel counts each
// solver's running instances, and the graph is rebuilt without the finished solvers whenever a
// quarter of the remaining ones (at least one) has finished.
static void solveGroupGraph(const std::vector<spock_solver_s *> &sv, int device) {
    const int n = (int)sv.size();
    GCK(cudaSetDevice(device));
    for (auto *s : sv) s->eng->groupBegin(false);
    cudaStream_t st = nullptr;
    const int **dStatus = nullptr;
    long *dBatch = nullptr;
    int *dActive = nullptr, *hActive = nullptr;
    cudaGraphExec_t exec = nullptr;
    auto cleanup = [&] {
        if (exec) cudaGraphExecDestroy(exec);
        if (st) cudaStreamSynchronize(st);
        cudaFree(dStatus);
        cudaFree(dBatch);
        cudaFree(dActive);
        if (hActive) cudaFreeHost(hActive);
        if (st) cudaStreamDestroy(st);
    };
    try {
        GCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        std::vector<const int *> hs((size_t)n);
        std::vector<long> hb((size_t)n);
        for (int e = 0; e < n; e++) {
            hs[(size_t)e] = sv[(size_t)e]->eng->statusDevice();
            hb[(size_t)e] = sv[(size_t)e]->eng->batch();
        }
        GCK(cudaMalloc(&dStatus, sizeof(int *) * n));
        GCK(cudaMalloc(&dBatch, sizeof(long) * n));
        GCK(cudaMalloc(&dActive, sizeof(int) * n));
        GCK(cudaMallocHost(&hActive, sizeof(int) * n));
        GCK(cudaMemcpy(dStatus, hs.data(), sizeof(int *) * n, cudaMemcpyHostToDevice));
        GCK(cudaMemcpy(dBatch, hb.data(), sizeof(long) * n, cudaMemcpyHostToDevice));
        std::vector<char> alive((size_t)n, 1);
        std::vector<long> rounds((size_t)n, 0);
        int nAlive = n, aliveAtBuild = 0;
        auto build = [&] {
            if (exec) GCK(cudaGraphExecDestroy(exec));
            exec = nullptr;
            cudaGraph_t g;
            GCK(cudaGraphCreate(&g, 0));
            for (int e = 0; e < n; e++)
                if (alive[(size_t)e]) {
                    cudaGraphNode_t node;
                    GCK(cudaGraphAddChildGraphNode(&node, g, nullptr, 0, sv[(size_t)e]->eng->roundGraph()));
                }
            const cudaError_t ie = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            GCK(ie);
            aliveAtBuild = nAlive;
        };
        build();
        long r = 0;
        while (nAlive > 0) {
            GCK(cudaGraphLaunch(exec, st));
            r++;
            for (int e = 0; e < n; e++)
                if (alive[(size_t)e]) rounds[(size_t)e] = r;
            if (r % 10) continue;
            k_group_active<<<n, 128, 0, st>>>(dStatus, dBatch, n, dActive);
            GCK(cudaGetLastError());
            GCK(cudaMemcpyAsync(hActive, dActive, sizeof(int) * n, cudaMemcpyDeviceToHost, st));
            GCK(cudaStreamSynchronize(st));
            for (int e = 0; e < n; e++)
                if (alive[(size_t)e] && hActive[e] == 0) {
                    alive[(size_t)e] = 0;
                    nAlive--;
                }
            if (nAlive > 0 && aliveAtBuild - nAlive >= std::max(1, aliveAtBuild / 4)) build();
        }
        GCK(cudaStreamSynchronize(st));
        for (int e = 0; e < n; e++) sv[(size_t)e]->eng->groupEnd(rounds[(size_t)e]);
    } catch (...) {
        cleanup();
        throw;
    }
    cleanup();
}

int spock_solve_group(long count, spock_solver *solvers, int algo, const double *const *x0s, const long *x0counts,
                      int *const *statuses, long *const *iters) {
    return guard([&] {
        if (count < 1 || !solvers || !x0s || !x0counts) throw std::invalid_argument("[solveGroup] bad arguments");
        if (algo != SPOCK_ALGO_SPOCK && algo != SPOCK_ALGO_CP) throw std::invalid_argument("[Cache] unknown algorithm");
        for (long i = 0; i < count; i++) {
            solver(solvers[i]);
            need(x0s[i], "x0");
            for (long j = 0; j < i; j++)
                if (solvers[j] == solvers[i]) throw std::invalid_argument("[solveGroup] a solver appears twice");
        }
        bool oneDevice = true;
        for (long i = 1; i < count; i++) oneDevice = oneDevice && solver(solvers[i])->eng->device() == solver(solvers[0])->eng->device();
        if (algo == SPOCK_ALGO_SPOCK && oneDevice) {
            std::vector<spock_solver_s *> sv;
            for (long i = 0; i < count; i++) {
                auto *s = solver(solvers[i]);
                GCK(cudaSetDevice(s->eng->device()));
                s->eng->setInitialStates(x0s[i], x0counts[i]);
                sv.push_back(s);
            }
            solveGroupGraph(sv, sv[0]->eng->device());
            for (long i = 0; i < count; i++) finishSolve(sv[(size_t)i], statuses ? statuses[i] : nullptr, iters ? iters[i] : nullptr);
            return;
        }
        std::vector<std::string> errors((size_t)count);
        std::vector<std::thread> threads;
        threads.reserve((size_t)count);
        for (long i = 0; i < count; i++)
            threads.emplace_back([&, i] {
                try {
                    auto *s = solver(solvers[i]);
                    if (cudaSetDevice(s->eng->device()) != cudaSuccess) throw std::runtime_error("cudaSetDevice failed");
                    s->eng->setInitialStates(x0s[i], x0counts[i]);
                    s->eng->run(algo == SPOCK_ALGO_SPOCK ? spock::kSpock : spock::kCp, false);
                    finishSolve(s, statuses ? statuses[i] : nullptr, iters ? iters[i] : nullptr);
                } catch (const std::exception &e) {
                    errors[(size_t)i] = e.what();
                }
            });
        for (auto &t : threads) t.join();
        for (long i = 0; i < count; i++)
            if (!errors[(size_t)i].empty())
                throw std::invalid_argument("[solveGroup] solver " + std::to_string(i) + ": " + errors[(size_t)i]);
    });
}

int spock_resolve(spock_solver sv, int algo, const double *x0, long count, int *statuses, long *iters) {
    return guard([&] {
        auto *s = solver(sv);
        need(x0, "x0");
        if (algo != SPOCK_ALGO_SPOCK && algo != SPOCK_ALGO_CP) throw std::invalid_argument("[Cache] unknown algorithm");
        s->eng->setInitialStates(x0, count);
        s->eng->run(algo == SPOCK_ALGO_SPOCK ? spock::kSpock : spock::kCp, true);
        finishSolve(s, statuses, iters);
    });
}

int spock_resolve_device(spock_solver sv, int algo, const void *x0, int *statuses, long *iters) {
    return guard([&] {
        auto *s = solver(sv);
        need(x0, "x0");
        if (algo != SPOCK_ALGO_SPOCK && algo != SPOCK_ALGO_CP) throw std::invalid_argument("[Cache] unknown algorithm");
        s->eng->setInitialStatesDevice(x0, s->eng->batch());
        s->eng->run(algo == SPOCK_ALGO_SPOCK ? spock::kSpock : spock::kCp, true);
        finishSolve(s, statuses, iters);
    });
}

int spock_set_iterate_device(spock_solver sv, const void *z_device, int bits) {
    return guard([&] {
        auto *s = solver(sv);
        need(z_device, "z");
        if (bits != 32 && bits != 64) throw std::invalid_argument("[setIterate] bits must be 32 or 64");
        s->eng->setIterateFromDevice(z_device, bits, s->eng->problem().sizeIterate(), s->eng->batch(),
                                     s->eng->device());
    });
}

int spock_copy_iterate(spock_solver dst, spock_solver src) {
    return guard([&] {
        auto *d = solver(dst);
        auto *s = solver(src);
        // the source's stream has finished: every solve and setter synchronizes before returning
        d->eng->setIterateFromDevice(s->eng->iterateDevice(), s->eng->precisionBits(),
                                     s->eng->problem().sizeIterate(), s->eng->batch(), s->eng->device());
    });
}

int spock_get_iterate(spock_solver sv, long instance, double *out) {
    return guard([&] {
        auto *s = solver(sv);
        need(out, "out");
        s->eng->getIterate(instance, out);
    });
}

int spock_get_iterates(spock_solver sv, double *out) {
    return guard([&] {
        auto *s = solver(sv);
        need(out, "out");
        s->eng->getIterates(out);
    });
}

int spock_get_states_inputs(spock_solver sv, long instance, double *states, double *inputs) {
    return guard([&] {
        auto *s = solver(sv);
        const auto &h = s->eng->problem();
        std::vector<double> z(h.sizeIterate());
        s->eng->getIterate(instance, z.data());
        if (states)
            for (long j = 0; j < h.numNodes; j++)
                for (long k = 0; k < h.nx; k++) states[j * h.nx + k] = z[h.sizeU + j * h.nx + k] / h.scaling[k];
        if (inputs)
            for (long i = 0; i < h.numNonleaf; i++)
                for (long k = 0; k < h.nu; k++) inputs[i * h.nu + k] = z[i * h.nu + k] / h.scaling[h.nx + k];
    });
}

int spock_get_first_inputs(spock_solver sv, double *out) {
    return guard([&] {
        auto *s = solver(sv);
        need(out, "out");
        s->eng->getFirstInputs(out);
    });
}

int spock_status(spock_solver sv, long instance, int *status, long *iters, double *seconds) {
    return guard([&] {
        auto *s = solver(sv);
        if (instance < 0 || instance >= s->eng->batch()) throw std::invalid_argument("[Cache] instance out of range");
        if (status) *status = s->status[instance];
        if (iters) *iters = s->iters[instance];
        if (seconds) *seconds = s->seconds;
    });
}

int spock_counters(spock_solver sv, long *out7) {
    return guard([&] {
        auto *s = solver(sv);
        need(out7, "out");
        s->eng->getCounters(out7);
    });
}

int spock_counters_all(spock_solver sv, long *out) {
    return guard([&] {
        auto *s = solver(sv);
        need(out, "out");
        s->eng->getCountersAll(out);
    });
}

int spock_reset(spock_solver sv) {
    return guard([&] {
        auto *s = solver(sv);
        s->eng->zeroIterate();
        std::fill(s->status.begin(), s->status.end(), SPOCK_NOT_RUN);
    });
}

int spock_op(spock_solver sv, const double *prim, double *dual) {
    return guard([&] {
        auto *s = solver(sv);
        need(prim, "prim");
        need(dual, "dual");
        s->eng->op(prim, dual);
    });
}

int spock_adj(spock_solver sv, const double *dual, double *prim) {
    return guard([&] {
        auto *s = solver(sv);
        need(prim, "prim");
        need(dual, "dual");
        s->eng->adj(dual, prim);
    });
}

int spock_cp_step(spock_solver sv, const double *x0, const double *z, double *cand) {
    return guard([&] {
        auto *s = solver(sv);
        need(x0, "x0");
        need(z, "z");
        need(cand, "cand");
        s->eng->cpStep(x0, z, cand);
    });
}

int spock_reduce_check(spock_solver sv, const double *r, const double *mr, double *out3) {
    return guard([&] {
        auto *s = solver(sv);
        need(r, "r");
        need(mr, "mr");
        need(out3, "out3");
        s->eng->reduceCheck(r, mr, out3);
    });
}

int spock_get_dual(spock_solver sv, const double *prim, double *dual) {
    return guard([&] {
        auto *s = solver(sv);
        need(prim, "prim");
        need(dual, "dual");
        s->eng->dualOf(prim, dual);
    });
}

int spock_apply_m(spock_solver sv, const double *z, double *mz) {
    return guard([&] {
        auto *s = solver(sv);
        need(z, "z");
        need(mz, "mz");
        s->eng->applyM(z, mz);
    });
}

int spock_kernel_time(spock_solver sv, const char *which, int reps, double *ms, long *bytes) {
    return guard([&] {
        auto *s = solver(sv);
        need(which, "which");
        if (ms) *ms = s->eng->kernelMs(which, reps < 1 ? 1 : reps);
        if (bytes) *bytes = s->eng->bytesPerRoundAlgorithmic(which);
    });
}

int spock_round_time(spock_solver sv, int rounds, double *ms) {
    return guard([&] {
        auto *s = solver(sv);
        float f = 0;
        s->eng->timedRounds(rounds < 1 ? 1 : rounds, &f);
        if (ms) *ms = f;
    });
}

int spock_run_stats(spock_solver sv, long *rounds, long *launches, long *compactions) {
    return guard([&] {
        auto *s = solver(sv);
        if (rounds) *rounds = s->eng->lastRounds();
        if (launches) *launches = s->eng->lastLaunches();
        if (compactions) *compactions = s->eng->lastCompactions();
    });
}

int spock_tuning(spock_solver sv, int *out5) {
    return guard([&] {
        if (!out5) throw std::invalid_argument("[spock_tuning] null output");
        solver(sv)->eng->tuning(out5);
    });
}

int spock_step_size(spock_solver sv, int iters, double *norm_sq, double *step) {
    return guard([&] {
        if (iters < 1) throw std::invalid_argument("[stepSize] iters must be positive");
        const double lam = solver(sv)->eng->normLsq(iters);
        if (norm_sq) *norm_sq = lam;
        if (step) *step = 0.99 / std::sqrt(lam);
    });
}

int spock_set_fp64_finish(spock_solver sv, long rounds) {
    return guard([&] { solver(sv)->eng->setFinishDouble(rounds); });
}

int spock_set_tuning(spock_solver sv, const int *in3) {
    return guard([&] {
        need(in3, "tiles");
        solver(sv)->eng->setTuning(in3[0], in3[1], in3[2]);
    });
}

}  // extern "C"

namespace spock {
EngineBase *engineOf(spock_solver s) { return solver(s)->eng.get(); }
int guardedCall(const std::function<void()> &f) { return guard(f); }
}  // namespace spock
