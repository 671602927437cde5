// spock_gb300.hpp -- header-only C++ interface over the C ABI (spock_gb300.h) with the class
// names and call shapes of the reference library, so a program written against it
// (examples/*/main.cu: ScenarioTree -> ProblemData -> CacheBuilder -> Cache::runSpock) builds
// against this one by changing the include.
//
//   reference (ruairimoran/spock.cu)                this header
//   ScenarioTree<T>(path)      src/tree.cuh:102      ScenarioTree<T>(path)
//   ProblemData<T>(tree)       src/problem.cuh:126   ProblemData<T>(tree)
//   CacheBuilder<T>(tree, d)   src/cache.cuh:1154    CacheBuilder<T>(tree, d), same setters, + batch()
//   Cache<T>::runSpock/runCp   src/cache.cuh:967-1132 same, + runSpockBatch()
//   toString(int)              src/cache.cuh:75-88   toString(int)
//
// T = double runs the FP64 iteration, T = float the FP32 one.  Errors throw
// std::invalid_argument with the library's message, as the reference does (include/gpu.cuh:24).
// Differences: solution()/solutionPrim()/solutionDual() return std::vector<T> copies of the
// iterate instead of references to device tensors; the tree and the problem data are one
// device-independent host object that the tree owns.
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "spock_gb300.h"

namespace spock_gb300 {

inline void check(int rc) {
    if (rc != SPOCK_OK) throw std::invalid_argument(spock_last_error());
}

enum CacheStatus { notRun = SPOCK_NOT_RUN, converged = SPOCK_CONVERGED, outOfIter = SPOCK_OUT_OF_ITER,
                   outOfTime = SPOCK_OUT_OF_TIME };

inline const char *toString(int status) {
    switch (status) {
        case notRun: return "Cache has not been run!";
        case converged: return "Converged!";
        case outOfIter: return "Out of iterations!";
        case outOfTime: return "Out of time!";
        case SPOCK_DIVERGED: return "Stopped on a non-finite residual!";
        default: return "Unknown status.";
    }
}

template <typename T>
class ScenarioTree {
   public:
    explicit ScenarioTree(std::string path = "./data/") : path_(std::move(path)) {
        if (!path_.empty() && path_.back() != '/') path_ += '/';
        spock_problem p = nullptr;
        check(spock_problem_load(path_.c_str(), &p));
        h_.reset(p);
        check(spock_problem_sizes(p, sizes_));
    }
    std::string path() const { return path_; }
    std::string fpFileExt() const { return sizeof(T) == 8 ? "_d.bt" : "_f.bt"; }
    size_t numEvents() const { return (size_t)sizes_[0]; }
    size_t numNodes() const { return (size_t)sizes_[1]; }
    size_t numNonleafNodes() const { return (size_t)sizes_[2]; }
    size_t numLeafNodes() const { return numNodes() - numNonleafNodes(); }
    size_t numStages() const { return (size_t)sizes_[3]; }
    size_t numStates() const { return (size_t)sizes_[4]; }
    size_t numInputs() const { return (size_t)sizes_[5]; }
    size_t numStatesAndInputs() const { return numStates() + numInputs(); }
    spock_problem handle() const { return h_.get(); }
    long sizePrimal() const { return sizes_[6]; }
    long sizeDual() const { return sizes_[7]; }

   private:
    struct Free {
        void operator()(spock_problem p) const { spock_problem_free(p); }
    };
    std::string path_;
    std::unique_ptr<std::remove_pointer_t<spock_problem>, Free> h_;
    long sizes_[10] = {};
};

template <typename T>
class ProblemData {
   public:
    explicit ProblemData(ScenarioTree<T> &tree) : tree_(tree) {
        double step = 0;
        check(spock_problem_step(tree.handle(), &step, nullptr));
        step_ = (T)step;
    }
    ScenarioTree<T> &tree() const { return tree_; }
    T stepSize() const { return step_; }
    T stepSizeRecip() const { return T(1) / step_; }

   private:
    ScenarioTree<T> &tree_;  // must outlive this object, as in the reference (problem.cuh:24)
    T step_ = 0;
};

template <typename T>
class Cache {
   public:
    Cache(ScenarioTree<T> &tree, const spock_options &o) : tree_(tree), batch_(o.batch) {
        spock_solver s = nullptr;
        check(spock_solver_create(tree.handle(), &o, &s));
        h_.reset(s);
        status_.assign((size_t)batch_, notRun);
        iters_.assign((size_t)batch_, 0);
    }

    // Cache::runSpock (cache.cuh:1008-1132); `previousSolution` warm-starts from a full iterate.
    int runSpock(std::vector<T> &initState, std::vector<T> *previousSolution = nullptr) {
        return run(SPOCK_ALGO_SPOCK, initState, previousSolution, 1);
    }
    // Cache::runCp (cache.cuh:967-1002).
    int runCp(std::vector<T> &initState, std::vector<T> *previousSolution = nullptr) {
        return run(SPOCK_ALGO_CP, initState, previousSolution, 1);
    }
    // Every instance of the batch: initStates holds `count` rows of numStates values (instance b
    // uses row b % count); warm, if given, one full iterate per row.  Returns the statuses.
    std::vector<int> runSpockBatch(const std::vector<T> &initStates, const std::vector<T> *warm = nullptr) {
        const long count = (long)(initStates.size() / tree_.numStates());
        std::vector<T> x0(initStates);
        run(SPOCK_ALGO_SPOCK, x0, warm, count);
        return status_;
    }

    // Re-solve warm-started from the current iterate (the previous solution, kept on the device)
    // with new initial states: the control-loop form of runSpock(x0, &previousSolution).
    std::vector<int> resolveBatch(const std::vector<T> &initStates) {
        const long count = (long)(initStates.size() / tree_.numStates());
        if (count < 1 || initStates.size() != tree_.numStates() * (size_t)count)
            throw std::invalid_argument("[initialiseState] wrong number of states");
        std::vector<double> x(initStates.begin(), initStates.end());
        check(spock_resolve(h_.get(), SPOCK_ALGO_SPOCK, x.data(), count, status_.data(), iters_.data()));
        return status_;
    }

    int status(long instance = 0) const { return status_[(size_t)instance]; }
    size_t solveIter(long instance = 0) const { return (size_t)iters_[(size_t)instance]; }
    T solveTime() const {
        double secs = 0;
        check(spock_status(h_.get(), 0, nullptr, nullptr, &secs));
        return (T)secs;
    }
    size_t sizePrimal() const { return (size_t)tree_.sizePrimal(); }
    size_t sizeDual() const { return (size_t)tree_.sizeDual(); }
    size_t sizeIterate() const { return sizePrimal() + sizeDual(); }
    long batch() const { return batch_; }

    std::vector<T> solution(long instance = 0) const {
        std::vector<double> z(sizeIterate());
        check(spock_get_iterate(h_.get(), instance, z.data()));
        return std::vector<T>(z.begin(), z.end());
    }
    std::vector<T> solutionPrim(long instance = 0) const {
        std::vector<T> z = solution(instance);
        z.resize(sizePrimal());
        return z;
    }
    std::vector<T> solutionDual(long instance = 0) const {
        std::vector<T> z = solution(instance);
        return std::vector<T>(z.begin() + (long)sizePrimal(), z.end());
    }
    // Cache::getDual (cache.cuh:371-376): the dual candidate for a given primal candidate at the
    // current iterate (a copy instead of a device tensor).
    std::vector<T> getDual(const std::vector<T> &primal) const {
        if ((long)primal.size() != (long)sizePrimal()) throw std::invalid_argument("[getDual] primal has the wrong size");
        std::vector<double> p(primal.begin(), primal.end()), d(sizeDual());
        check(spock_get_dual(h_.get(), p.data(), d.data()));
        return std::vector<T>(d.begin(), d.end());
    }
    // Cache::states()/inputs() (cache.cuh:386-412), unscaled.
    std::vector<T> states(long instance = 0) const {
        std::vector<double> xs(tree_.numStates() * tree_.numNodes());
        check(spock_get_states_inputs(h_.get(), instance, xs.data(), nullptr));
        return std::vector<T>(xs.begin(), xs.end());
    }
    std::vector<T> inputs(long instance = 0) const {
        std::vector<double> us(tree_.numInputs() * tree_.numNonleafNodes());
        check(spock_get_states_inputs(h_.get(), instance, nullptr, us.data()));
        return std::vector<T>(us.begin(), us.end());
    }
    void reset() {
        check(spock_reset(h_.get()));
        status_.assign((size_t)batch_, notRun);
    }
    // FP32 batched solvers: the last <= 32 running instances finish in FP64 after `rounds`
    // rounds (spock_set_fp64_finish); 0 turns it off.  No reference counterpart.
    void fp64Finish(size_t rounds) { check(spock_set_fp64_finish(h_.get(), (long)rounds)); }

   private:
    template <typename V>
    int run(int algo, V &x0, const std::vector<T> *warm, long count) {
        if (x0.size() != tree_.numStates() * (size_t)count)
            throw std::invalid_argument("[initialiseState] Error initialising state: problem setup for " +
                                        std::to_string(tree_.numStates()) + " states but given " +
                                        std::to_string(x0.size() / (size_t)count));
        std::vector<double> x(x0.begin(), x0.end()), w;
        if (warm) {
            if (warm->size() != sizeIterate() * (size_t)count)
                throw std::invalid_argument("[initialisePrev] previous solution has the wrong size");
            w.assign(warm->begin(), warm->end());
        }
        check(spock_solve(h_.get(), algo, x.data(), count, warm ? w.data() : nullptr, status_.data(), iters_.data()));
        return status_[0];
    }
    struct Free {
        void operator()(spock_solver s) const { spock_solver_free(s); }
    };
    ScenarioTree<T> &tree_;
    long batch_;
    std::unique_ptr<std::remove_pointer_t<spock_solver>, Free> h_;
    std::vector<int> status_;
    std::vector<long> iters_;
};

// CacheBuilder (cache.cuh:1154-1244): the same setters, plus batch() and device().
template <typename T>
class CacheBuilder {
   public:
    CacheBuilder(ScenarioTree<T> &tree, ProblemData<T> &data) : tree_(tree) {
        (void)data;
        spock_options_default(&o_);
        o_.precision = sizeof(T) == 8 ? 64 : 32;
    }
    CacheBuilder &toleranceAbsolute(T tol) { o_.tol_abs = (double)tol; return *this; }
    CacheBuilder &toleranceRelative(T tol) { o_.tol_rel = (double)tol; return *this; }
    CacheBuilder &tol(T tol) { o_.tol_abs = o_.tol_rel = (double)tol; return *this; }
    CacheBuilder &maxTimeSecs(T secs) { o_.max_time_secs = (double)secs; return *this; }
    CacheBuilder &maxIters(size_t iters) { o_.max_iters = (long)iters; return *this; }
    CacheBuilder &maxItersInner(size_t iters) { o_.max_inner = (long)iters; return *this; }
    CacheBuilder &andersonBuffer(size_t m) { o_.anderson = (long)m; return *this; }
    // The reference's debug mode caps the iterations at 1000 when none are set (cache.cuh:1204-1208)
    // and records error histories; only the cap is kept here.
    CacheBuilder &enableDebug(bool enable = true) {
        if (enable && o_.max_iters == 0) o_.max_iters = 1000;
        return *this;
    }
    CacheBuilder &batch(size_t instances) { o_.batch = (long)instances; return *this; }
    CacheBuilder &device(int ordinal) { o_.device = ordinal; return *this; }
    Cache<T> build() { return Cache<T>(tree_, o_); }
    std::unique_ptr<Cache<T>> make_unique() { return std::make_unique<Cache<T>>(tree_, o_); }

   private:
    ScenarioTree<T> &tree_;
    spock_options o_;
};

}  // namespace spock_gb300
