// Problem generator in C++: scenario trees, problem data and the data folder, without Python.
//
// The reference generates problems with its Python API (api/python/spock/tree.py,
// build.py, problem.py) and its C++ solver reads the folder that API writes.  This header
// builds the same folder from C++: the trees of tree.py (stopped Markov chains, tree.py:350-479;
// i.i.d. processes, tree.py:492-588), the dynamics, costs, constraints and AVaR risk of build.py,
// the diagonal preconditioning of problem.py:159-190, the cost data (square roots and the
// translations of the quadratic-plus-linear costs, build.py:184-216, 495-535) and the files of
// problem.py:437-687.  The offline cache (the dynamics projection cache, the AVaR nullspace
// projectors and the step size, problem.py:192-231, 402-417) is computed on the GPU in FP64 by
// the library (spock_offline_complete), so generateProblem() needs libspock_gb300 at link time
// and a GPU; writeProblemData() is host code only and writes the folder without that cache.
//
// Every matrix is dense and column-major.  Header-only, C++17, no CUDA.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "spock_gb300.h"

namespace spock {
namespace factory {

// ---------------------------------------------------------------------------------- matrices

struct Matrix {
    long rows = 0, cols = 0;
    std::vector<double> a;  // column-major

    Matrix() = default;
    Matrix(long r, long c, double v = 0.) : rows(r), cols(c), a((size_t)(r * c), v) {}
    static Matrix identity(long n) {
        Matrix m(n, n);
        for (long i = 0; i < n; i++) m(i, i) = 1.;
        return m;
    }
    static Matrix diagonal(const std::vector<double> &d) {
        Matrix m((long)d.size(), (long)d.size());
        for (size_t i = 0; i < d.size(); i++) m((long)i, (long)i) = d[i];
        return m;
    }
    double &operator()(long r, long c) { return a[(size_t)(c * rows + r)]; }
    double operator()(long r, long c) const { return a[(size_t)(c * rows + r)]; }
    bool empty() const { return a.empty(); }
};

namespace detail {

[[noreturn]] inline void fail(const std::string &m) { throw std::invalid_argument(m); }

// numpy.allclose(a, b) for scalars: |a - b| <= 1e-8 + 1e-5 |b|
inline bool close(double a, double b) { return std::fabs(a - b) <= 1e-8 + 1e-5 * std::fabs(b); }

// x = M^-1 y by Gaussian elimination with partial pivoting (M square).
inline std::vector<double> solve(const Matrix &M, std::vector<double> y) {
    const long n = M.rows;
    if (M.cols != n || (long)y.size() != n) fail("[solve] dimension mismatch");
    Matrix A = M;
    for (long k = 0; k < n; k++) {
        long p = k;
        for (long r = k + 1; r < n; r++)
            if (std::fabs(A(r, k)) > std::fabs(A(p, k))) p = r;
        if (A(p, k) == 0.) fail("[solve] singular matrix");
        if (p != k) {
            for (long c = 0; c < n; c++) std::swap(A(k, c), A(p, c));
            std::swap(y[(size_t)k], y[(size_t)p]);
        }
        for (long r = k + 1; r < n; r++) {
            const double f = A(r, k) / A(k, k);
            if (f == 0.) continue;
            for (long c = k; c < n; c++) A(r, c) -= f * A(k, c);
            y[(size_t)r] -= f * y[(size_t)k];
        }
    }
    for (long r = n - 1; r >= 0; r--) {
        double s = y[(size_t)r];
        for (long c = r + 1; c < n; c++) s -= A(r, c) * y[(size_t)c];
        y[(size_t)r] = s / A(r, r);
    }
    return y;
}

// Principal square root of a symmetric positive semidefinite matrix: the square roots of the
// diagonal when M is diagonal (as the reference factory's shortcut), else V sqrt(max(L, 0)) V'
// from a cyclic Jacobi eigendecomposition.
inline Matrix sqrtm(const Matrix &M) {
    const long n = M.rows;
    if (M.cols != n) fail("[sqrtm] matrix is not square");
    bool diag = true;
    double scale = 0.;
    for (long c = 0; c < n; c++)
        for (long r = 0; r < n; r++) {
            scale = std::max(scale, std::fabs(M(r, c)));
            if (r != c && M(r, c) != 0.) diag = false;
        }
    Matrix out(n, n);
    if (diag) {
        for (long i = 0; i < n; i++) out(i, i) = std::sqrt(std::max(M(i, i), 0.));
        return out;
    }
    for (long c = 0; c < n; c++)
        for (long r = 0; r < c; r++)
            if (std::fabs(M(r, c) - M(c, r)) > 1e-12 * scale) fail("[sqrtm] cost matrix is not symmetric");
    Matrix A = M, V = Matrix::identity(n);
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.;
        for (long c = 0; c < n; c++)
            for (long r = 0; r < c; r++) off += A(r, c) * A(r, c);
        if (std::sqrt(off) <= 1e-17 * scale * n) break;
        for (long p = 0; p < n - 1; p++)
            for (long q = p + 1; q < n; q++) {
                const double apq = A(p, q);
                if (apq == 0.) continue;
                // rotation that zeroes A(p, q): t = tan(theta), theta from cot(2 theta)
                const double th = (A(q, q) - A(p, p)) / (2. * apq);
                const double t = (th >= 0 ? 1. : -1.) / (std::fabs(th) + std::sqrt(th * th + 1.));
                const double cs = 1. / std::sqrt(t * t + 1.), sn = t * cs;
                for (long k = 0; k < n; k++) {  // A <- A J
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = cs * akp - sn * akq;
                    A(k, q) = sn * akp + cs * akq;
                }
                for (long k = 0; k < n; k++) {  // A <- J' A
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = cs * apk - sn * aqk;
                    A(q, k) = sn * apk + cs * aqk;
                }
                for (long k = 0; k < n; k++) {  // V <- V J
                    const double vkp = V(k, p), vkq = V(k, q);
                    V(k, p) = cs * vkp - sn * vkq;
                    V(k, q) = sn * vkp + cs * vkq;
                }
            }
    }
    for (long c = 0; c < n; c++)
        for (long r = 0; r < n; r++) {
            double s = 0.;
            for (long k = 0; k < n; k++) s += V(r, k) * std::sqrt(std::max(A(k, k), 0.)) * V(c, k);
            out(r, c) = s;
        }
    return out;
}

inline double dot(const std::vector<double> &x, const std::vector<double> &y) {
    double s = 0.;
    for (size_t i = 0; i < x.size(); i++) s += x[i] * y[i];
    return s;
}

}  // namespace detail

// ---------------------------------------------------------------------------------- .bt files

// `.bt`: three little-endian uint64 (rows, cols, mats), then the column-major payload as FP64
// ('d'), FP32 ('f') or uint64 ('u') (the GPUtils format, modelFactory.jl:26-60).
inline void writeTensor(const std::string &file, char dtype, const std::vector<double> &v, uint64_t rows,
                        uint64_t cols = 1, uint64_t mats = 1) {
    if ((size_t)(rows * cols * mats) != v.size()) detail::fail("[writeTensor] " + file + ": size does not match dims");
    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    if (!f) detail::fail("[writeTensor] cannot write " + file);
    const uint64_t h[3] = {rows, cols, mats};
    f.write(reinterpret_cast<const char *>(h), sizeof h);
    if (dtype == 'd') {
        f.write(reinterpret_cast<const char *>(v.data()), (std::streamsize)(v.size() * 8));
    } else if (dtype == 'f') {
        std::vector<float> w(v.begin(), v.end());
        f.write(reinterpret_cast<const char *>(w.data()), (std::streamsize)(w.size() * 4));
    } else {
        detail::fail("[writeTensor] dtype must be 'd' or 'f'");
    }
    if (!f) detail::fail("[writeTensor] cannot write " + file);
}

// Index tensor: -1 is written as the largest uint64 (the root's ancestor and event).
inline void writeIndex(const std::string &file, const std::vector<long> &v) {
    std::ofstream f(file, std::ios::binary | std::ios::trunc);
    if (!f) detail::fail("[writeIndex] cannot write " + file);
    const uint64_t h[3] = {(uint64_t)v.size(), 1, 1};
    f.write(reinterpret_cast<const char *>(h), sizeof h);
    for (long x : v) {
        const uint64_t u = x < 0 ? std::numeric_limits<uint64_t>::max() : (uint64_t)x;
        f.write(reinterpret_cast<const char *>(&u), 8);
    }
    if (!f) detail::fail("[writeIndex] cannot write " + file);
}

// Read a `_d` or `_f` tensor as doubles; dims receives rows, cols, mats.
inline std::vector<double> readTensor(const std::string &file, uint64_t dims[3]) {
    std::ifstream f(file, std::ios::binary);
    if (!f) detail::fail("[readTensor] cannot open " + file);
    f.read(reinterpret_cast<char *>(dims), 24);
    if (!f) detail::fail("[readTensor] truncated header in " + file);
    const size_t n = (size_t)(dims[0] * dims[1] * dims[2]);
    std::vector<double> v(n);
    const char kind = file.size() >= 4 ? file[file.size() - 4] : '?';
    if (kind == 'd') {
        f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)(n * 8));
    } else if (kind == 'f') {
        std::vector<float> w(n);
        f.read(reinterpret_cast<char *>(w.data()), (std::streamsize)(n * 4));
        std::copy(w.begin(), w.end(), v.begin());
    } else {
        detail::fail("[readTensor] " + file + " is neither _d.bt nor _f.bt");
    }
    if (!f) detail::fail("[readTensor] truncated payload in " + file);
    return v;
}

// ---------------------------------------------------------------------------------- trees

// Nodes numbered stage by stage with the children of a node contiguous (tree.py:7-265).
struct ScenarioTree {
    std::vector<long> stages, ancestors, events;  // the root's ancestor and event are -1
    std::vector<double> probability;
    // derived by finish()
    long numNodes = 0, numStages = 0, numNonleaf = 0, numEvents = 0;
    std::vector<long> childFrom, numChildren, stageFrom, stageTo;
    std::vector<double> condProb;

    void finish() {
        numNodes = (long)ancestors.size();
        numStages = stages.back() + 1;
        numNonleaf = 0;
        for (long s : stages) numNonleaf += s < numStages - 1;
        childFrom.assign((size_t)numNonleaf, -1);
        numChildren.assign((size_t)numNonleaf, 0);
        for (long j = 1; j < numNodes; j++) {
            const long i = ancestors[(size_t)j];
            if (childFrom[(size_t)i] < 0) childFrom[(size_t)i] = j;
            numChildren[(size_t)i]++;
        }
        numEvents = *std::max_element(numChildren.begin(), numChildren.end());
        condProb.assign((size_t)numNodes, -1.);
        for (long j = 1; j < numNodes; j++) condProb[(size_t)j] = probability[(size_t)j] / probability[(size_t)ancestors[(size_t)j]];
        stageFrom.assign((size_t)numStages, -1);
        stageTo.assign((size_t)numStages, -1);
        for (long j = 0; j < numNodes; j++) {
            const long s = stages[(size_t)j];
            if (stageFrom[(size_t)s] < 0) stageFrom[(size_t)s] = j;
            stageTo[(size_t)s] = j;
        }
    }
};

namespace detail {

// Stage-by-stage branching (tree.py:396-437 and 522-559): every node of stages 1 .. stopping-1
// branches into cover(value), after the stopping stage every node has one child that repeats
// its value.  Fills ancestors, values and stages.
template <typename Cover>
void branchingTree(const std::vector<long> &first, Cover cover, long horizon, long stopping, ScenarioTree &t) {
    t.ancestors.assign(1, -1);
    t.events.assign(1, -1);
    t.stages.assign(1, 0);
    for (long v : first) {
        t.ancestors.push_back(0);
        t.events.push_back(v);
        t.stages.push_back(1);
    }
    long cursor = 1, width = (long)first.size();
    for (long stage = 1; stage < stopping; stage++) {
        long added = 0;
        for (long i = 0; i < width; i++) {
            const long node = cursor + i;
            for (long w : cover(t.events[(size_t)node])) {
                t.ancestors.push_back(node);
                t.events.push_back(w);
                added++;
            }
        }
        cursor += width;
        width = added;
        t.stages.insert(t.stages.end(), (size_t)added, stage + 1);
    }
    for (long stage = stopping; stage < horizon; stage++) {
        const long n0 = (long)t.events.size();
        for (long i = 0; i < width; i++) {
            t.ancestors.push_back(cursor + i);
            t.events.push_back(t.events[(size_t)(n0 - width + i)]);
        }
        cursor += width;
        t.stages.insert(t.stages.end(), (size_t)width, stage + 1);
    }
}

}  // namespace detail

// Tree of a Markov chain stopped at `stopping` (tree.py:350-479): transition matrix P (rows sum
// to 1), initial distribution v.
class MarkovChain {
   public:
    MarkovChain(const Matrix &P, std::vector<double> v, long horizon, long stopping = -1)
        : P_(P), v_(std::move(v)), N_(horizon), tau_(stopping < 0 ? horizon : stopping) {
        if (N_ < 1 || tau_ < 1) detail::fail("horizon and stopping stage must be at least 1");
        if (tau_ > N_) detail::fail("stopping time greater than number of stages");
        if (P_.rows != P_.cols || P_.rows != (long)v_.size()) detail::fail("[MarkovChain] dimension mismatch");
        auto check = [](const std::vector<double> &p) {
            double s = 0.;
            for (double x : p) {
                s += x;
                if (x < -1e-16) detail::fail("invalid probability vector");
            }
            if (std::fabs(s - 1.) >= 1e-10) detail::fail("invalid probability vector");
        };
        for (long r = 0; r < P_.rows; r++) {
            std::vector<double> row((size_t)P_.cols);
            for (long c = 0; c < P_.cols; c++) row[(size_t)c] = P_(r, c);
            check(row);
        }
        check(v_);
    }
    ScenarioTree build() const {
        ScenarioTree t;
        std::vector<long> first;
        for (size_t k = 0; k < v_.size(); k++)
            if (v_[k] != 0.) first.push_back((long)k);
        detail::branchingTree(
            first,
            [&](long w) {
                std::vector<long> c;
                for (long k = 0; k < P_.cols; k++)
                    if (P_(w, k) != 0.) c.push_back(k);
                return c;
            },
            N_, tau_, t);
        t.probability.assign(t.ancestors.size(), 0.);
        t.probability[0] = 1.;
        for (size_t i = 1; i < t.ancestors.size(); i++) {
            const long a = t.ancestors[i];
            if (t.stages[i] == 1) t.probability[i] = v_[(size_t)t.events[i]];
            else if (t.stages[i] <= tau_) t.probability[i] = t.probability[(size_t)a] * P_(t.events[(size_t)a], t.events[i]);
            else t.probability[i] = t.probability[(size_t)a];
        }
        t.finish();
        return t;
    }

   private:
    Matrix P_;
    std::vector<double> v_;
    long N_, tau_;
};

// n-ary tree of an i.i.d. process with distribution d (tree.py:492-588).
class IidProcess {
   public:
    IidProcess(std::vector<double> d, long horizon, long stopping = -1)
        : d_(std::move(d)), N_(horizon), tau_(stopping < 0 ? horizon : stopping) {
        if (N_ < 1 || tau_ < 1) detail::fail("horizon and stopping stage must be at least 1");
        if (tau_ > N_) detail::fail("stopping time greater than number of stages");
        double s = 0.;
        for (double x : d_) {
            s += x;
            if (x <= 1e-16) detail::fail("invalid distribution");
        }
        if (std::fabs(s - 1.) >= 1e-10) detail::fail("invalid distribution");
    }
    ScenarioTree build() const {
        ScenarioTree t;
        std::vector<long> cover;
        for (size_t k = 0; k < d_.size(); k++) cover.push_back((long)k);
        detail::branchingTree(cover, [&](long) { return cover; }, N_, tau_, t);
        t.probability.assign(t.ancestors.size(), 0.);
        t.probability[0] = 1.;
        for (size_t i = 1; i < t.ancestors.size(); i++) {
            const long a = t.ancestors[i];
            t.probability[i] = t.stages[i] <= tau_ ? t.probability[(size_t)a] * d_[(size_t)t.events[i]] : t.probability[(size_t)a];
        }
        t.finish();
        return t;
    }

   private:
    std::vector<double> d_;
    long N_, tau_;
};

// ---------------------------------------------------------------------------------- building blocks

// x+ = A x + B u (+ c) (build.py:13-75).
struct Dynamics {
    Matrix A, B;
    std::vector<double> c;  // empty for linear dynamics
    static Dynamics linear(Matrix A, Matrix B) { return {std::move(A), std::move(B), {}}; }
    static Dynamics affine(Matrix A, Matrix B, std::vector<double> c) { return {std::move(A), std::move(B), std::move(c)}; }
    bool isAffine() const { return !c.empty(); }
};

// "quadratic" (x'Qx + u'Ru), "quadraticPlusLinear" (+ q'x + r'u) or "linear" (q'x + r'u);
// leaf costs carry Q and q only (build.py:184-668).
struct Cost {
    std::string kind;
    Matrix Q, R;  // empty when absent
    std::vector<double> q, r;
    bool leaf = false;

    static Cost quadratic(Matrix Q, Matrix R) { return {"quadratic", std::move(Q), std::move(R), {}, {}, false}; }
    static Cost quadraticLeaf(Matrix Q) { return {"quadratic", std::move(Q), {}, {}, {}, true}; }
    static Cost quadraticPlusLinear(Matrix Q, std::vector<double> q, Matrix R, std::vector<double> r) {
        return {"quadraticPlusLinear", std::move(Q), std::move(R), std::move(q), std::move(r), false};
    }
    static Cost quadraticPlusLinearLeaf(Matrix Q, std::vector<double> q) {
        return {"quadraticPlusLinear", std::move(Q), {}, std::move(q), {}, true};
    }
    static Cost linear(std::vector<double> q, std::vector<double> r) { return {"linear", {}, {}, std::move(q), std::move(r), false}; }
    static Cost linearLeaf(std::vector<double> q) { return {"linear", {}, {}, std::move(q), {}, true}; }
};

// "no", "rectangle" (lb <= z <= ub), "polyhedron" (glb <= G z <= gub), "polyhedronWithIdentity"
// (both, build.py:1025-1096) and "rectangleInputBall" (box on x, ||u||_2 <= radius; nonleaf only,
// not in the reference).
struct Constraint {
    std::string kind = "no";
    std::vector<double> lb, ub;    // rectangle part
    Matrix G;                      // polyhedron part
    std::vector<double> glb, gub;
    long nx = 0;                   // rectangleInputBall: states bounded by lb/ub
    double radius = 0.;

    static Constraint none() { return {}; }
    static Constraint rectangle(std::vector<double> lb, std::vector<double> ub) {
        if (lb.size() != ub.size()) detail::fail("Rectangle constraint bounds invalid");
        for (size_t i = 0; i < lb.size(); i++)
            if (lb[i] > ub[i]) detail::fail("Rectangle constraint bounds invalid");
        Constraint c;
        c.kind = "rectangle";
        c.lb = std::move(lb);
        c.ub = std::move(ub);
        return c;
    }
    static Constraint polyhedron(Matrix G, std::vector<double> glb, std::vector<double> gub) {
        if ((long)glb.size() != G.rows || (long)gub.size() != G.rows) detail::fail("Polyhedron constraint bounds invalid");
        Constraint c;
        c.kind = "polyhedron";
        c.G = std::move(G);
        c.glb = std::move(glb);
        c.gub = std::move(gub);
        return c;
    }
    static Constraint polyhedronWithIdentity(const Constraint &rect, const Constraint &poly) {
        if (rect.kind != "rectangle" || poly.kind != "polyhedron")
            detail::fail("PolyhedronWithIdentity takes a Rectangle and a Polyhedron");
        if (poly.G.cols != (long)rect.lb.size()) detail::fail("PolyhedronWithIdentity: Gamma and the rectangle differ in dimension");
        Constraint c = poly;
        c.kind = "polyhedronWithIdentity";
        c.lb = rect.lb;
        c.ub = rect.ub;
        return c;
    }
    static Constraint rectangleInputBall(const std::vector<double> &xlb, const std::vector<double> &xub, long numInputs,
                                         double radius) {
        if (xlb.size() != xub.size() || !(radius > 0)) detail::fail("RectangleInputBall constraint invalid");
        for (size_t i = 0; i < xlb.size(); i++)
            if (xlb[i] > xub[i]) detail::fail("RectangleInputBall constraint invalid");
        Constraint c;
        c.kind = "rectangleInputBall";
        const double inf = std::numeric_limits<double>::infinity();
        c.lb = xlb;
        c.ub = xub;
        c.lb.insert(c.lb.end(), (size_t)numInputs, -inf);
        c.ub.insert(c.ub.end(), (size_t)numInputs, inf);
        c.nx = (long)xlb.size();
        c.radius = radius;
        return c;
    }
};

// AVaR_alpha: E = [alpha I; -I; 1'], b = [p; 0; 1] (build.py:1160-1193).
struct AVaR {
    double alpha = 1.;
    explicit AVaR(double a) : alpha(a) {
        if (!(a >= 0. && a <= 1.)) detail::fail("AVaR alpha must be in [0, 1]");
    }
};

// ---------------------------------------------------------------------------------- the factory

// Fluent interface of problem.Factory (problem.py:702-879).
class ProblemFactory {
   public:
    ProblemFactory(ScenarioTree tree, long numStates, long numInputs)
        : t_(std::move(tree)), nx_(numStates), nu_(numInputs), risk_(1.) {}

    ProblemFactory &withDynamics(const Dynamics &d) { return withDynamicsEvents(std::vector<Dynamics>((size_t)eventCount(), d)); }
    ProblemFactory &withDynamicsEvents(std::vector<Dynamics> ds) {
        dyn_ = std::move(ds);
        return *this;
    }
    ProblemFactory &withCostNonleaf(const Cost &c) { return withCostNonleafEvents(std::vector<Cost>((size_t)eventCount(), c)); }
    ProblemFactory &withCostNonleafEvents(std::vector<Cost> cs) {
        for (const Cost &c : cs)
            if (c.leaf) detail::fail("Cannot use leaf cost for nonleaf nodes!");
        cost_ = std::move(cs);
        return *this;
    }
    ProblemFactory &withCostLeaf(const Cost &c) {
        if (!c.leaf) detail::fail("Cannot use nonleaf cost for leaf nodes!");
        leaf_ = c;
        hasLeaf_ = true;
        return *this;
    }
    ProblemFactory &withConstraintNonleaf(const Constraint &c) {
        nlCon_ = c;
        return *this;
    }
    ProblemFactory &withConstraintLeaf(const Constraint &c) {
        if (c.kind == "rectangleInputBall") detail::fail("an input ball constrains nonleaf nodes only");
        lCon_ = c;
        return *this;
    }
    ProblemFactory &withRisk(const AVaR &r) {
        risk_ = r;
        hasRisk_ = true;
        return *this;
    }
    ProblemFactory &withPreconditioning(bool enable = true) {
        precondition_ = enable;
        return *this;
    }
    // Multiply every cost term by factor > 0 (not in the reference factory): the minimiser is
    // unchanged, the optimal value scales with it.
    ProblemFactory &withCostScaling(double factor) {
        if (!(factor > 0)) detail::fail("cost scaling factor must be positive");
        costScale_ = factor;
        return *this;
    }

    // The folder without the offline cache (stepSize 0): the part of the reference's Problem
    // constructor that is not its offline cache.  dtype 'd' writes FP64 tensors, 'f' FP32.
    void writeProblemData(const std::string &path, char dtype = 'd') const {
        if (dtype != 'd' && dtype != 'f') detail::fail("[generateProblem] dtype must be 'd' or 'f'");
        Data d = assemble();
        write(d, path, dtype);
    }

    // The complete folder: writeProblemData, then the offline cache and the step size on GPU
    // `device` in FP64 (spock_offline_complete).  Returns the step size.
    double generateProblem(const std::string &path, char dtype = 'd', int device = 0, int iters = 20000) const {
        writeProblemData(path, dtype);
        double step = 0.;
        const int rc = spock_offline_complete(path.c_str(), device, iters, &step);
        if (rc == SPOCK_E_INVALID) throw std::invalid_argument(spock_last_error());
        if (rc != SPOCK_OK) throw std::runtime_error(spock_last_error());
        return step;
    }

   private:
    // Per-node problem data after preconditioning, in (node-major) column-major blocks.
    struct Data {
        long n = 0, nnl = 0, nx = 0, nu = 0, yd = 0, nd = 0;
        bool affine = false, preconditioned = false;
        std::string costKind, leafKind;
        std::vector<double> sx, su;
        std::vector<Matrix> A, B, Q, R, sQ, sR;
        std::vector<std::vector<double>> c, q, r, trans;
        Matrix lQ, lsQ;
        std::vector<double> lq, ltrans, b;
    };

    long eventCount() const {
        long m = 0;
        for (size_t i = 1; i < t_.events.size(); i++) m = std::max(m, t_.events[i]);
        return m + 1;
    }

    Data assemble() const {
        const long n = t_.numNodes, nnl = t_.numNonleaf, nx = nx_, nu = nu_;
        if (dyn_.empty()) detail::fail("[generateProblem] no dynamics");
        if (cost_.empty() || !hasLeaf_) detail::fail("[generateProblem] no nonleaf or leaf cost");
        if (!hasRisk_) detail::fail("[generateProblem] no risk");
        if ((long)dyn_.size() < eventCount() || (long)cost_.size() < eventCount())
            detail::fail("[generateProblem] fewer dynamics or costs than events");
        Data d;
        d.n = n;
        d.nnl = nnl;
        d.nx = nx;
        d.nu = nu;
        d.affine = dyn_[0].isAffine();
        d.costKind = cost_[0].kind;
        d.leafKind = leaf_.kind;
        d.A.assign((size_t)n, Matrix(nx, nx));
        d.B.assign((size_t)n, Matrix(nx, nu));
        d.c.assign((size_t)n, std::vector<double>((size_t)nx, 0.));
        d.Q.assign((size_t)n, Matrix(nx, nx));
        d.R.assign((size_t)n, Matrix(nu, nu));
        d.q.assign((size_t)n, std::vector<double>((size_t)nx, 0.));
        d.r.assign((size_t)n, std::vector<double>((size_t)nu, 0.));
        const double cs = costScale_;
        auto scaled = [cs](Matrix M) {
            for (double &v : M.a) v *= cs;
            return M;
        };
        auto scaledV = [cs](std::vector<double> v) {
            for (double &x : v) x *= cs;
            return v;
        };
        for (long i = 1; i < n; i++) {  // node 0 carries zeros (problem.py:744-757)
            const long e = t_.events[(size_t)i];
            const Dynamics &dy = dyn_[(size_t)e];
            if (dy.A.rows != nx || dy.A.cols != nx || dy.B.rows != nx || dy.B.cols != nu)
                detail::fail("[generateProblem] dynamics dimensions do not match the state and input sizes");
            d.A[(size_t)i] = dy.A;
            d.B[(size_t)i] = dy.B;
            if (dy.isAffine()) d.c[(size_t)i] = dy.c;
            const Cost &ce = cost_[(size_t)e];
            if (!ce.Q.empty()) d.Q[(size_t)i] = scaled(ce.Q);
            if (!ce.R.empty()) d.R[(size_t)i] = scaled(ce.R);
            if (!ce.q.empty()) d.q[(size_t)i] = scaledV(ce.q);
            if (!ce.r.empty()) d.r[(size_t)i] = scaledV(ce.r);
        }
        d.lQ = leaf_.Q.empty() ? Matrix(nx, nx) : scaled(leaf_.Q);
        d.lq = leaf_.q.empty() ? std::vector<double>((size_t)nx, 0.) : scaledV(leaf_.q);
        // preconditioning (problem.py:159-190)
        d.sx.assign((size_t)nx, 1.);
        d.su.assign((size_t)nu, 1.);
        if (precondition_) {
            for (long k = 0; k < nx; k++) {
                double m = 1.;
                for (long i = 1; i < n; i++) {
                    if (d.costKind != "linear") m = std::max(m, std::sqrt(d.Q[(size_t)i](k, k)));
                    if (d.costKind != "quadratic") m = std::max(m, std::fabs(d.q[(size_t)i][(size_t)k]));
                }
                if (d.leafKind != "linear") m = std::max(m, std::sqrt(d.lQ(k, k)));
                if (d.leafKind != "quadratic") m = std::max(m, std::fabs(d.lq[(size_t)k]));
                d.sx[(size_t)k] = m;
            }
            for (long k = 0; k < nu; k++) {
                double m = 1.;
                for (long i = 1; i < n; i++) {
                    if (d.costKind != "linear") m = std::max(m, std::sqrt(d.R[(size_t)i](k, k)));
                    if (d.costKind != "quadratic") m = std::max(m, std::fabs(d.r[(size_t)i][(size_t)k]));
                }
                d.su[(size_t)k] = m;
            }
            const double mul = std::sqrt((double)*std::max_element(t_.numChildren.begin(), t_.numChildren.end()));
            bool ones = true;
            for (double &v : d.sx) ones = detail::close(v *= mul, 1.) && ones;
            for (double &v : d.su) ones = detail::close(v *= mul, 1.) && ones;
            d.preconditioned = !ones;
        }
        if (!d.preconditioned) {
            std::fill(d.sx.begin(), d.sx.end(), 1.);
            std::fill(d.su.begin(), d.su.end(), 1.);
        } else {
            const auto &sx = d.sx, &su = d.su;
            for (long i = 1; i < n; i++) {
                Matrix &A = d.A[(size_t)i], &B = d.B[(size_t)i], &Q = d.Q[(size_t)i], &R = d.R[(size_t)i];
                for (long c = 0; c < nx; c++)
                    for (long r = 0; r < nx; r++) {
                        A(r, c) = sx[(size_t)r] * A(r, c) / sx[(size_t)c];
                        Q(r, c) = Q(r, c) / sx[(size_t)r] / sx[(size_t)c];
                    }
                for (long c = 0; c < nu; c++) {
                    for (long r = 0; r < nx; r++) B(r, c) = sx[(size_t)r] * B(r, c) / su[(size_t)c];
                    for (long r = 0; r < nu; r++) R(r, c) = R(r, c) / su[(size_t)r] / su[(size_t)c];
                }
                for (long k = 0; k < nx; k++) {
                    d.c[(size_t)i][(size_t)k] *= sx[(size_t)k];
                    d.q[(size_t)i][(size_t)k] /= sx[(size_t)k];
                }
                for (long k = 0; k < nu; k++) d.r[(size_t)i][(size_t)k] /= su[(size_t)k];
            }
            for (long c = 0; c < nx; c++)
                for (long r = 0; r < nx; r++) d.lQ(r, c) = d.lQ(r, c) / sx[(size_t)r] / sx[(size_t)c];
            for (long k = 0; k < nx; k++) d.lq[(size_t)k] /= sx[(size_t)k];
        }
        // cost data (build.py:184-216, 495-535): square roots per event, translations
        if (d.costKind != "linear") {
            d.sQ.assign((size_t)n, Matrix(nx, nx));
            d.sR.assign((size_t)n, Matrix(nu, nu));
            d.trans.assign((size_t)n, std::vector<double>((size_t)(nx + nu + 2), 0.));
            std::vector<long> seen((size_t)eventCount(), -1);
            for (long i = 1; i < n; i++) {
                const long e = t_.events[(size_t)i];
                if (seen[(size_t)e] < 0) {
                    seen[(size_t)e] = i;
                    d.sQ[(size_t)i] = detail::sqrtm(d.Q[(size_t)i]);
                    d.sR[(size_t)i] = detail::sqrtm(d.R[(size_t)i]);
                } else {
                    d.sQ[(size_t)i] = d.sQ[(size_t)seen[(size_t)e]];
                    d.sR[(size_t)i] = d.sR[(size_t)seen[(size_t)e]];
                }
                auto &tr = d.trans[(size_t)i];
                if (d.costKind == "quadratic") {
                    tr[(size_t)(nx + nu)] = -.5;
                    tr[(size_t)(nx + nu + 1)] = .5;
                } else {
                    const auto a = detail::solve(d.sQ[(size_t)i], d.q[(size_t)i]);
                    const auto bb = detail::solve(d.sR[(size_t)i], d.r[(size_t)i]);
                    const double nq = -.125 * detail::dot(d.q[(size_t)i], detail::solve(d.Q[(size_t)i], d.q[(size_t)i])) -
                                      .125 * detail::dot(d.r[(size_t)i], detail::solve(d.R[(size_t)i], d.r[(size_t)i]));
                    for (long k = 0; k < nx; k++) tr[(size_t)k] = .5 * a[(size_t)k];
                    for (long k = 0; k < nu; k++) tr[(size_t)(nx + k)] = .5 * bb[(size_t)k];
                    tr[(size_t)(nx + nu)] = -.5 + nq;
                    tr[(size_t)(nx + nu + 1)] = .5 + nq;
                }
            }
        }
        if (d.leafKind != "linear") {
            d.lsQ = detail::sqrtm(d.lQ);
            d.ltrans.assign((size_t)(nx + 2), 0.);
            if (d.leafKind == "quadratic") {
                d.ltrans[(size_t)nx] = -.5;
                d.ltrans[(size_t)nx + 1] = .5;
            } else {
                const auto a = detail::solve(d.lsQ, d.lq);
                const double nq = -.125 * detail::dot(d.lq, detail::solve(d.lQ, d.lq));
                for (long k = 0; k < nx; k++) d.ltrans[(size_t)k] = .5 * a[(size_t)k];
                d.ltrans[(size_t)nx] = -.5 + nq;
                d.ltrans[(size_t)nx + 1] = .5 + nq;
            }
        }
        // risk (build.py:1184-1193): b = [conditional probabilities of the children; 0; 1]
        const long E = t_.numEvents;
        d.yd = 2 * E + 1;
        d.nd = 4 * E + 1;
        d.b.assign((size_t)(d.yd * nnl), 0.);
        for (long i = 0; i < nnl; i++) {
            const long c0 = t_.childFrom[(size_t)i], m = t_.numChildren[(size_t)i];
            for (long j = 0; j < m; j++) d.b[(size_t)(i * d.yd + j)] = t_.condProb[(size_t)(c0 + j)];
            d.b[(size_t)(i * d.yd + 2 * m)] = 1.;
        }
        return d;
    }

    static void writeConstraint(const std::string &dir, const std::string &part, char dt, const Constraint &con,
                                const std::vector<double> &scale) {
        const std::string ext = "_" + std::string(1, dt) + ".bt";
        auto times = [&](const std::vector<double> &v) {
            if (v.size() != scale.size()) detail::fail("[" + part + "] bounds do not match the dimension they bound");
            std::vector<double> o(v.size());
            for (size_t k = 0; k < v.size(); k++) o[k] = v[k] * scale[k];
            return o;
        };
        auto gamma = [&]() {  // Gamma / scale per column
            if (con.G.cols != (long)scale.size()) detail::fail("[" + part + "Gamma] wrong number of columns");
            Matrix G = con.G;
            for (long c = 0; c < G.cols; c++)
                for (long r = 0; r < G.rows; r++) G(r, c) /= scale[(size_t)c];
            return G;
        };
        if (con.kind == "no") return;
        if (con.kind == "rectangle" || con.kind == "rectangleInputBall") {
            const auto lo = times(con.lb), hi = times(con.ub);
            writeTensor(dir + part + "ILB" + ext, dt, lo, lo.size());
            writeTensor(dir + part + "IUB" + ext, dt, hi, hi.size());
            if (con.kind == "rectangleInputBall") {
                const size_t nxb = (size_t)con.nx;
                for (size_t k = nxb; k < scale.size(); k++)
                    if (!detail::close(scale[k], scale[nxb]))
                        detail::fail("an input ball needs the same preconditioning scale on every input "
                                     "(or withPreconditioning(false))");
                writeTensor(dir + part + "Radius" + ext, dt, {con.radius * scale[nxb]}, 1);
            }
        } else if (con.kind == "polyhedron" || con.kind == "polyhedronWithIdentity") {
            const Matrix G = gamma();
            writeTensor(dir + part + "Gamma" + ext, dt, G.a, (uint64_t)G.rows, (uint64_t)G.cols);
            writeTensor(dir + part + "GLB" + ext, dt, con.glb, con.glb.size());
            writeTensor(dir + part + "GUB" + ext, dt, con.gub, con.gub.size());
            if (con.kind == "polyhedronWithIdentity") {
                const auto lo = times(con.lb), hi = times(con.ub);
                writeTensor(dir + part + "ILB" + ext, dt, lo, lo.size());
                writeTensor(dir + part + "IUB" + ext, dt, hi, hi.size());
            }
        } else {
            detail::fail("constraint kind " + con.kind + " not supported by this factory");
        }
    }

    void write(const Data &d, const std::string &path, char dt) const {
        std::filesystem::create_directories(path);
        std::string dir = path;
        if (dir.empty() || dir.back() != '/') dir += '/';
        const std::string ext = "_" + std::string(1, dt) + ".bt";
        const long n = d.n, nnl = d.nnl, nx = d.nx, nu = d.nu;
        // tree (tree.py:240-265)
        writeIndex(dir + "stages_u.bt", t_.stages);
        writeIndex(dir + "ancestors_u.bt", t_.ancestors);
        writeIndex(dir + "events_u.bt", t_.events);
        writeIndex(dir + "childrenFrom_u.bt", t_.childFrom);
        std::vector<long> childTo(t_.childFrom.size());
        for (size_t i = 0; i < childTo.size(); i++) childTo[i] = t_.childFrom[i] + t_.numChildren[i] - 1;
        writeIndex(dir + "childrenTo_u.bt", childTo);
        writeIndex(dir + "numChildren_u.bt", t_.numChildren);
        writeIndex(dir + "stageFrom_u.bt", t_.stageFrom);
        writeIndex(dir + "stageTo_u.bt", t_.stageTo);
        writeTensor(dir + "probabilities" + ext, dt, t_.probability, (uint64_t)n);
        writeTensor(dir + "conditionalProbabilities" + ext, dt, t_.condProb, (uint64_t)n);
        // per-node stacks: matrix i of a tensor is node i
        auto stack = [n](const std::vector<Matrix> &ms, long rows, long cols, bool transpose) {
            std::vector<double> v;
            v.reserve((size_t)(rows * cols * n));
            for (const Matrix &m : ms)
                for (long c = 0; c < cols; c++)
                    for (long r = 0; r < rows; r++) v.push_back(transpose ? m(c, r) : m(r, c));
            return v;
        };
        auto stackV = [](const std::vector<std::vector<double>> &vs) {
            std::vector<double> v;
            for (const auto &x : vs) v.insert(v.end(), x.begin(), x.end());
            return v;
        };
        writeTensor(dir + "dynamics_BTr" + ext, dt, stack(d.B, nu, nx, true), nu, nx, n);
        std::vector<double> AB;
        AB.reserve((size_t)(nx * (nx + nu) * n));
        for (long i = 0; i < n; i++) {
            AB.insert(AB.end(), d.A[(size_t)i].a.begin(), d.A[(size_t)i].a.end());
            AB.insert(AB.end(), d.B[(size_t)i].a.begin(), d.B[(size_t)i].a.end());
        }
        writeTensor(dir + "dynamics_AB" + ext, dt, AB, nx, nx + nu, n);
        if (d.affine) writeTensor(dir + "dynamics_c" + ext, dt, stackV(d.c), nx, 1, n);
        writeTensor(dir + "risk_b" + ext, dt, d.b, d.yd, 1, nnl);
        if (d.preconditioned) {
            std::vector<double> s = d.sx;
            s.insert(s.end(), d.su.begin(), d.su.end());
            writeTensor(dir + "scaling" + ext, dt, s, s.size());
        }
        if (d.costKind == "linear") {
            std::vector<double> g;
            for (long i = 0; i < n; i++) {
                g.insert(g.end(), d.q[(size_t)i].begin(), d.q[(size_t)i].end());
                g.insert(g.end(), d.r[(size_t)i].begin(), d.r[(size_t)i].end());
            }
            writeTensor(dir + "nonleafCost_gradient" + ext, dt, g, 1, nx + nu, n);
        } else {
            writeTensor(dir + "nonleafCost_sqrtQ" + ext, dt, stack(d.sQ, nx, nx, false), nx, nx, n);
            writeTensor(dir + "nonleafCost_sqrtR" + ext, dt, stack(d.sR, nu, nu, false), nu, nu, n);
            writeTensor(dir + "nonleafCost_translation" + ext, dt, stackV(d.trans), nx + nu + 2, 1, n);
            if (d.costKind == "quadraticPlusLinear") {
                writeTensor(dir + "nonleafCost_q" + ext, dt, stackV(d.q), nx, 1, n);
                writeTensor(dir + "nonleafCost_r" + ext, dt, stackV(d.r), nu, 1, n);
            }
        }
        if (d.leafKind == "linear") {
            writeTensor(dir + "leafCost_gradient" + ext, dt, d.lq, 1, nx, 1);
        } else {
            writeTensor(dir + "leafCost_sqrtQ" + ext, dt, d.lsQ.a, nx, nx, 1);
            writeTensor(dir + "leafCost_translation" + ext, dt, d.ltrans, nx + 2);
            if (d.leafKind == "quadraticPlusLinear") writeTensor(dir + "leafCost_q" + ext, dt, d.lq, nx);
        }
        std::vector<double> sxu = d.sx;
        sxu.insert(sxu.end(), d.su.begin(), d.su.end());
        writeConstraint(dir, "nonleafConstraint", dt, nlCon_, sxu);
        writeConstraint(dir, "leafConstraint", dt, lCon_, d.sx);
        // data.json (jinja2.py:1-33), stepSize 0 until the offline cache is computed
        const std::string js = dir + "data.json";
        std::FILE *f = std::fopen(js.c_str(), "w");
        if (!f) detail::fail("[generateProblem] cannot write " + js);
        std::fprintf(f,
                     "{\n \"numEvents\": %ld,\n \"numNonleafNodes\": %ld,\n \"numNodes\": %ld,\n \"numStages\": %ld,\n"
                     " \"numStates\": %ld,\n \"numInputs\": %ld,\n \"dynamics\": {\n  \"type\": \"%s\"\n },\n"
                     " \"cost\": {\n  \"nonleaf\": \"%s\",\n  \"leaf\": \"%s\"\n },\n"
                     " \"constraint\": {\n  \"nonleaf\": \"%s\",\n  \"leaf\": \"%s\"\n },\n"
                     " \"risk\": {\n  \"type\": \"avar\",\n  \"alpha\": %.17g\n },\n"
                     " \"rowsS2\": %ld,\n \"rowsNNtr\": %ld,\n \"stepSize\": 0.0,\n \"preconditioned\": %s\n}",
                     t_.numEvents, nnl, n, t_.numStages, nx, nu, d.affine ? "affine" : "linear", d.costKind.c_str(),
                     d.leafKind.c_str(), nlCon_.kind.c_str(), lCon_.kind.c_str(), risk_.alpha, t_.numEvents, d.nd,
                     d.preconditioned ? "true" : "false");
        const bool ok = std::ferror(f) == 0;
        if (std::fclose(f) != 0 || !ok) detail::fail("[generateProblem] cannot write " + js);
    }

    ScenarioTree t_;
    long nx_, nu_;
    std::vector<Dynamics> dyn_;
    std::vector<Cost> cost_;
    Cost leaf_;
    bool hasLeaf_ = false;
    Constraint nlCon_, lCon_;
    AVaR risk_;
    bool hasRisk_ = false;
    bool precondition_ = true;
    double costScale_ = 1.;
};

}  // namespace factory
}  // namespace spock
