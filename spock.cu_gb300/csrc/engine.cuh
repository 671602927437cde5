// SPOCK solve engine for GB300 (sm_103a): device data, per-iteration kernels, SuperMann
// controller and the host loop that drives them.
//
// Memory layout.  Every iterate-sized vector of a batch of B instances is one array
// [element][instance]: entry k of instance b lives at k*B + b.  Element order is the
// reference's iterate layout (cache.cuh:481-497, 529-581):
//   prim = [u (nu x nonleaf) | x (nx x nodes) | y ((2E+1) x nonleaf) | t (nodes) | s (nodes)]
//   dual = [I ((2E+1) x nonleaf) | II (nonleaf) | III (nonleaf constraint) |
//           IV (nonleaf cost, every node incl. root) | V (leaf constraint) | VI (leaf cost)]
// so with B = 1 it is exactly the reference's vector, and with B > 1 a warp reads 32
// instances of one element in one coalesced transaction.  Per-node problem matrices are
// shared by all instances (uniform batch) and read as warp-wide broadcasts.
#pragma once

#include <cuda_runtime.h>

#include <chrono>
#include <string>
#include <vector>

#include "problem.hpp"

namespace spock {

struct Dims {
    int n, nnl, nl, ns, nx, nu, nxu, ne, yD, nd;
    int costNl, costL, conNl, conL, affine;
    int dIII, dIV, dV, dVI;
    int gNl, gL;  // rows of the nonleaf / leaf polyhedral constraint matrices Gamma
    long oX, oY, oT, oS, sPrim;              // primal offsets
    long oI, oII, oIII, oIV, oV, oVI, sDual;  // dual offsets, absolute (dual starts at sPrim)
    long sZ;
    int B;   // instances
    int TB;  // instances per CTA in the node kernels
    int gmat;  // kernels that read their node matrices in place (kGmat* bits of kernels_batch.cuh)
};

template <typename T>
struct DevProblem {
    const int *anc, *chFrom, *numCh;
    const T *BTr, *AB, *K, *ABKTr, *APB, *chol, *e, *Pe;
    const T *sqrtQ, *sqrtR, *q, *r, *trans;
    const T *lSqrtQ, *lq, *lTrans;
    const T *nlLo, *nlHi, *lLo, *lHi;
    const T *NNtr, *b;
    const T *grad, *lGrad;  // linear costs: gradient per node ((nx + nu) x n) and of the leaves (nx)
    T step;
    T radius;               // input ball of kConRectangleInputBall
};

// out = base + cL * Op(v), v = a1*in1 (+ a2*in2), base = b1*base1 (+ b2*base2).
template <typename T>
struct OpArgs {
    const T *in1, *in2;
    T a1, a2;
    const T *base1, *base2;
    T b1, b2;
    T cL;
    T *out;
    T *outBase;     // when set, base is stored here too
    T *outR;        // mode 0: the residual Z - out of every entry finalized by this kernel
    const T *x0s;   // scaled initial states, nx x B
    const int *live;  // per tile of 32 instances: nonzero while one of them runs (null: all)
};

struct Options {
    double tolAbs = 1e-3, tolRel = 0., maxTimeSecs = 0.;
    long maxOuter = 0, maxInner = 8, anderson = 3;
};

enum Algo { kSpock = 0, kCp = 1 };

// Per-instance SuperMann / CP state, structure of arrays on the device.
struct DevState {
    int *phase, *iOut, *iIn, *status, *errInit, *action, *head, *useAnd, *iters;
    int *k0, *k1, *k2, *k2bt, *k3, *calls;
    double *tau, *zeta, *w, *wSafe, *tol, *err, *coef, *G, *gamma;
    int *timeUp, *active;
    int *tileLive;  // per tile of 32 instances: nonzero while one of them is running
};

class EngineBase {
public:
    virtual ~EngineBase() = default;
    virtual void setInitialStates(const double *x0, long count) = 0;   // host, unscaled, count*nx
    virtual void setInitialStatesDevice(const void *x0, long count) = 0;  // device, unscaled, T
    virtual void setIterate(const double *z, long count) = 0;           // host warm start, count*sZ
    virtual void zeroIterate() = 0;
    virtual int run(Algo algo, bool warm) = 0;  // returns number of rounds
    // A SPOCK solve driven from outside, for a group of solvers whose rounds run as one CUDA graph:
    // groupBegin sets the solve up (synchronously); roundGraph is the solver's captured round
    // (owned by the solver); statusDevice its per-instance status (-1 while running); groupEnd
    // records the rounds it took.
    // FP32 solvers: after `rounds` rounds (0: never), once at most 32 instances are running, they
    // finish in FP64 (the same iteration continued by an FP64 solver of the same problem).
    virtual void setFinishDouble(long rounds) = 0;
    virtual void groupBegin(bool warm) = 0;
    virtual cudaGraph_t roundGraph() = 0;
    virtual const int *statusDevice() const = 0;
    virtual void groupEnd(long rounds) = 0;
    virtual void getIterate(long inst, double *out) = 0;
    virtual void getIterates(double *out) = 0;  // all, instance-major count*sZ
    virtual void getFirstInputs(double *out) = 0;  // unscaled u_0, B*nu
    virtual void getStatus(int *status, long *iters) = 0;
    virtual void getCounters(long *out7) = 0;  // instance 0: k0,k1,k2,k2bt,k3,calls,iters
    virtual void getCountersAll(long *out) = 0;  // every instance: B x 7, same order
    virtual void op(const double *prim, double *dual) = 0;
    virtual void adj(const double *dual, double *prim) = 0;
    virtual void cpStep(const double *x0, const double *z, double *cand) = 0;
    virtual void applyM(const double *z, double *mz) = 0;
    virtual void dualOf(const double *prim, double *dual) = 0;
    // The round's reductions (k_reduce) for residual r and M r (instance 0, empty Anderson memory):
    // out3 = {r'Mr, max|Mr|, r'r} summed over the partials in FP64.
    virtual void reduceCheck(const double *r, const double *mr, double *out3) = 0;
    // Learned warm start: iterate = mean + basis coef' on the device (FP32 accumulation), where basis
    // is sZ x k and coef batch x k, BF16 row-major, k a multiple of 64 (tcgen05 GEMM).
    virtual void warmStartPca(const void *basis, const void *coef, int k, const float *mean) = 0;
    virtual int precisionBits() const = 0;
    // The current iterate on the device (sZ x batch, element-major, in the solver precision), and
    // its replacement by another solver's iterate of the same problem size and batch, converted
    // to this solver's precision on the device (an FP32 solve handing over to an FP64 polish).
    virtual const void *iterateDevice() const = 0;
    virtual void setIterateFromDevice(const void *src, int srcBits, long sZ, long batch, int srcDevice) = 0;
    virtual double lastSeconds() const = 0;
    virtual double kernelMs(const char *which, int reps) = 0;  // CUDA-event timing of one kernel
    virtual void timedRounds(int rounds, float *ms) = 0;
    virtual long bytesPerRoundAlgorithmic(const char *which) const = 0;
    virtual int launchesPerRound() const = 0;
    // Tile shapes in use: L* instance tiles per CTA, L* double-buffered, the same for L, and the
    // dynamics sweep's tiles per CTA (0: the small-batch kernels).  Runs the autotuner if needed.
    virtual void tuning(int *out5) = 0;
    // Override the tuner: tiles per CTA of L*, L and the dynamics sweep (1, 2, 4 or 8), double
    // buffering where more than one tile fits twice in shared memory.
    virtual void setTuning(int lstar, int lop, int dyn) = 0;
    // ||L||^2 = lambda_max(L* L) by at most `iters` steps of the power iteration on the device,
    // with the solver's own L and L* kernels (instance 0); the step size is 0.99 / sqrt of it.
    // With rtol > 0 it stops once the estimate changed by at most rtol (relative) in each of
    // 20 consecutive steps.
    virtual double normLsq(int iters, double rtol = 0.) = 0;
    long lastRounds() const { return lastRounds_; }
    long lastCompactions() const { return lastCompactions_; }
    int device() const { return device_; }
    // Dynamics projection of a single-instance solver on caller-owned device memory: primUX is
    // the head [u | x] of a primal vector (solver precision), x0 the scaled initial state, and
    // the sweep's two workspaces live in `scratch` (scratchBytes long); runs on `stream`.
    virtual void projectDynamicsOn(const void *x0, void *primUX, void *scratch, size_t scratchBytes,
                                   cudaStream_t stream) = 0;
    long lastLaunches() const { return lastLaunches_; }
    const HostProblem &problem() const { return hp_; }
    long batch() const { return B_; }

protected:
    HostProblem hp_;
    long B_ = 1;
    long lastRounds_ = 0, lastLaunches_ = 0, lastCompactions_ = 0;
    int device_ = 0;
};

EngineBase *makeEngine(const HostProblem &hp, const Options &opt, long batch, int precisionBits, int device);

}  // namespace spock
