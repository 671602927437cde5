// SPOCK engine: SuperMann/CP control on the device and the host loop (see engine.cuh).
//
// A SuperMann solve (src/cache.cuh:1008-1132) is run as a sequence of identical "rounds".
// In every round each instance evaluates T at its current point Z (one CP step), forms the
// residual r = Z - T(Z) and M r (one L + L* pair), and a per-instance controller decides
// the next point from the reference's rules:
//   phase A (outer iteration start): error check every 25 outer iterations, w = ||r||_M,
//            Anderson direction, then K0 (blind) or the start of the line search;
//   phase B (line search step tau): K1 (educated), K2 (safeguard), backtrack, or K3 (restore).
// Both phases need exactly one T evaluation and one M application per round, so a batch of
// instances in different phases still runs one fixed sequence of launches, which is captured
// once as a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "engine.cuh"
#include "kernels.cuh"
#include "umma_gemm.hpp"
#include "kernels_batch.cuh"

namespace spock {

#define CK(x)                                                                                      \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + \
                                     __FILE__ + ":" + std::to_string(__LINE__));                   \
    } while (0)

constexpr int kMaxAnderson = 8;
constexpr int kNV0 = 5;  // r.Mr, max|Mr|, Mr.d, c.c, c.r ; then c.R_s (8 slots) and R_s.r (8 slots)

enum Action { kActNone = 0, kActFinish = 1, kActAK0 = 2, kActALs = 3, kActBK1 = 4, kActBK2 = 5, kActBK3 = 6, kActBBt = 7,
              kActCp = 8 };

// ------------------------------------------------------------------------------------------ reductions
template <typename T>
struct RedArgs {
    const T *R, *MR, *D, *RPREV, *ANDR;
    const int *phase, *status;
    double *part;
    int m, nv, chunks, algo;
    long rowsPerChunk;
};

// Rows a thread sums in the solver precision before adding the block's sum into its running
// sum.  Blocked summation (Higham, "Accuracy and Stability of Numerical Algorithms", 2nd ed.,
// section 4.2) bounds the error by about (kRedBlock - 1) u times the sum of magnitudes when the
// running sum is kept exactly enough.  In FP32 solvers the running sum is a float pair (hi, lo)
// updated by Knuth's TwoSum, which carries about twice the float precision (GB300's FP64 rate is
// ~1/64 of its FP32 rate, too slow for FP64 arithmetic per row or per block); in FP64 solvers it
// is a double.  The pairs are widened to FP64 once per thread, before the lanes are combined.
constexpr int kRedBlock = 32;

__device__ __forceinline__ void runningAdd(float &hi, float &lo, float x) {
    const float s = __fadd_rn(hi, x), z = __fsub_rn(s, hi);
    lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, z)), __fsub_rn(x, z)));
    hi = s;
}
__device__ __forceinline__ void runningAdd(double &hi, double &, double x) { hi += x; }

// Per-instance partial reductions over one chunk of rows: r.Mr, max|Mr|, Mr.d (line search),
// and in phase A the Anderson quantities c.c, c.r, c.R_s and R_s.r with c = r - r_prev.
// Threads are TB instances x `lanes` row lanes; the lanes' FP64 sums are combined by a tree in
// shared memory (log2(lanes) steps).
// M = the Anderson memory (A.m), a template parameter so that only the 5 + 2M accumulators in
// use occupy registers; the partials keep slots kNV0 + s and kNV0 + kMaxAnderson + s for the
// Anderson products whatever M is.
template <typename T, int M>
__global__ void __launch_bounds__(kRedThreads) k_reduce(const Dims Dm, const RedArgs<T> A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    double *sred = reinterpret_cast<double *>(smraw);  // [nv][lanes][TB]
    constexpr int NV = kNV0 + 2 * M;                  // accumulator k goes to partials slot slotOf(k)
    auto slotOf = [](int k) { return k < kNV0 + M ? k : k - M + kMaxAnderson; };
    const int B = Dm.B;
    const int TB = B >= 32 ? 32 : B;
    const int lb = threadIdx.x % TB, lane = threadIdx.x / TB, lanes = kRedThreads / TB;
    const bool laneOk = lane < lanes;
    const int b = blockIdx.x * TB + lb;
    const bool act = laneOk && b < B;
    const int chunk = blockIdx.y;
    const long k0 = (long)chunk * A.rowsPerChunk;
    const long k1 = k0 + A.rowsPerChunk < Dm.sZ ? k0 + A.rowsPerChunk : Dm.sZ;
    // accumulators indexed only by compile-time constants so they stay in registers
    T hi[NV], lo[NV];
#pragma unroll
    for (int v = 0; v < NV; v++) hi[v] = lo[v] = 0;
    T amax = 0;
    const int ph = act ? A.phase[b] : 1;
    const bool running = act && A.status[b] == -1;
    const bool wantA = running && A.algo == kSpock && ph == 0;
    const bool wantB = running && A.algo == kSpock && ph == 1;
    const size_t slot = (size_t)Dm.sZ * B;
    if (running) {
        for (long kb = k0 + lane; kb < k1; kb += (long)kRedBlock * lanes) {
            const long ke = kb + (long)kRedBlock * lanes < k1 ? kb + (long)kRedBlock * lanes : k1;
            T blk[NV];
#pragma unroll
            for (int v = 0; v < NV; v++) blk[v] = 0;
            // kU rows per step: every load of the step is issued (predicated on the phase, no
            // branch) before any of its products, so kU x (3 + M) loads per thread are in flight
            constexpr int kU = 4;
            for (long k = kb; k < ke; k += (long)kU * lanes) {
                T r[kU], mr[kU], rp[kU], dd[kU], an[M][kU];
#pragma unroll
                for (int q = 0; q < kU; q++) {
                    const long kk = k + (long)q * lanes;
                    const bool ok = kk < ke;
                    const size_t o = ix(ok ? kk : k, B, b);
                    r[q] = ok ? A.R[o] : T(0);
                    mr[q] = ok ? A.MR[o] : T(0);
                    dd[q] = ok && wantB ? A.D[o] : T(0);
                    rp[q] = ok && wantA ? A.RPREV[o] : T(0);
#pragma unroll
                    for (int s = 0; s < M; s++) an[s][q] = ok && wantA ? A.ANDR[s * slot + o] : T(0);
                }
#pragma unroll
                for (int q = 0; q < kU; q++) {
                    blk[0] += r[q] * mr[q];
                    amax = fmax(amax, fabs(mr[q]));
                    blk[2] += mr[q] * dd[q];
                    const T c = wantA ? r[q] - rp[q] : T(0);
                    blk[3] += c * c;
                    blk[4] += c * r[q];
#pragma unroll
                    for (int s = 0; s < M; s++) {
                        blk[kNV0 + s] += c * an[s][q];
                        blk[kNV0 + M + s] += an[s][q] * r[q];
                    }
                }
            }
            runningAdd(hi[0], lo[0], blk[0]);
            if (wantB) runningAdd(hi[2], lo[2], blk[2]);
            if (wantA) {
#pragma unroll
                for (int v = 3; v < NV; v++) runningAdd(hi[v], lo[v], blk[v]);
            }
        }
    }
    hi[1] = amax;
    lo[1] = 0;
    if (laneOk) {
#pragma unroll
        for (int v = 0; v < NV; v++) sred[(slotOf(v) * lanes + lane) * TB + lb] = (double)hi[v] + (double)lo[v];
        for (int v = kNV0 + M; v < kNV0 + kMaxAnderson; v++) sred[(v * lanes + lane) * TB + lb] = 0;
        for (int v = kNV0 + kMaxAnderson + M; v < A.nv; v++) sred[(v * lanes + lane) * TB + lb] = 0;
    }
    __syncthreads();
    int half = 1;
    while (2 * half < lanes) half *= 2;
    for (; half >= 1; half /= 2) {  // lane l takes lane l + half (when it exists)
        if (laneOk && lane < half && lane + half < lanes)
            for (int v = 0; v < A.nv; v++) {
                double *x = sred + (v * lanes + lane) * TB + lb;
                const double y = x[half * TB];
                *x = (v == 1) ? fmax(*x, y) : *x + y;
            }
        __syncthreads();
    }
    if (act && lane == 0)
        for (int v = 0; v < A.nv; v++)
            A.part[((size_t)b * A.nv + v) * A.chunks + chunk] = sred[(v * lanes) * TB + lb];  // [instance][value][chunk]
}

// ------------------------------------------------------------------------------------------ controller
struct CtlArgs {
    DevState S;
    const double *part;
    int chunks, nv, m, algo;
    double gamma, tolAbs, tolRel;
    long maxOuter, maxInner;
    double ridge;
};

// Solve the m x m SPD system G g = h (FP64 Cholesky with a small ridge); false on breakdown.
__device__ bool solveGram(const double *G, const double *h, int m, double ridge, double *g) {
    double L[kMaxAnderson * kMaxAnderson];
    double dmax = 0;
    for (int i = 0; i < m; i++) dmax = fmax(dmax, G[i * m + i]);
    if (!(dmax > 0)) return false;
    for (int j = 0; j < m; j++) {
        double s = G[j * m + j] + ridge * dmax;
        for (int k = 0; k < j; k++) s -= L[j * m + k] * L[j * m + k];
        if (!(s > 0)) return false;
        const double d = sqrt(s);
        L[j * m + j] = d;
        for (int i = j + 1; i < m; i++) {
            double a = G[i * m + j];
            for (int k = 0; k < j; k++) a -= L[i * m + k] * L[j * m + k];
            L[i * m + j] = a / d;
        }
    }
    double y[kMaxAnderson];
    for (int i = 0; i < m; i++) {
        double a = h[i];
        for (int k = 0; k < i; k++) a -= L[i * m + k] * y[k];
        y[i] = a / L[i * m + i];
    }
    for (int i = m - 1; i >= 0; i--) {
        double a = y[i];
        for (int k = i + 1; k < m; k++) a -= L[k * m + i] * g[k];
        g[i] = a / L[i * m + i];
    }
    for (int i = 0; i < m; i++)
        if (!isfinite(g[i])) return false;
    return true;
}

// The SuperMann / CP decision of instance b from its reduced values v (see k_control).
__device__ void controlInstance(const CtlArgs &A, const int b, const double *v) {
    const DevState &S = A.S;
    const double c0 = .99, c1 = .99, c2 = .99, beta = .5, sigma = .1, lambda = 1.;
    const int m = A.m;
    // error check (cache.cuh:909-961): r/gamma - [L* r_d; L r_p] = (M r)/gamma
    auto errorCheck = [&](int idx) {
        if (idx % 25 != 0) return;
        const double e = v[1] / A.gamma;
        if (S.errInit[b]) {
            S.tol[b] = fmax(A.tolAbs, A.tolRel * e);
            S.errInit[b] = 0;
        } else {
            S.err[b] = e;
            int st = -1;
            if (e <= S.tol[b]) st = 0;
            if (A.maxOuter && idx >= A.maxOuter) st = 1;
            if (*S.timeUp && idx % 1000 == 0) st = 2;
            if (!isfinite(e)) st = 3;
            if (st != -1) {
                S.status[b] = st;
                S.iters[b] = idx;
            }
        }
    };
    S.calls[b] += 1;
    if (A.algo == kCp) {
        errorCheck(S.iOut[b]);
        S.iOut[b] += 1;
        S.action[b] = kActCp;
        return;
    }
    if (S.phase[b] == 0) {
        const int iOut = S.iOut[b];
        errorCheck(iOut);
        if (S.status[b] != -1) {
            S.action[b] = kActFinish;
            return;
        }
        const double w = sqrt(fmax(v[0], 0.));
        S.w[b] = w;
        // Anderson (cache.cuh:860-904) on a ring of m physical slots: the new column
        // c = r - r_prev replaces the oldest slot h; G is the Gram matrix of the slots.
        const int h = S.head[b];
        double *G = S.G + (size_t)b * kMaxAnderson * kMaxAnderson;
        double rhs[kMaxAnderson];
        for (int s = 0; s < m; s++) {
            if (s == h) continue;
            G[h * m + s] = G[s * m + h] = v[kNV0 + s];
            rhs[s] = v[kNV0 + kMaxAnderson + s];
        }
        G[h * m + h] = v[3];
        rhs[h] = v[4];
        double *gam = S.gamma + (size_t)b * kMaxAnderson;
        int use = 0;
        if (iOut >= m) use = solveGram(G, rhs, m, A.ridge, gam) ? 1 : 0;
        if (!use)
            for (int s = 0; s < m; s++) gam[s] = 0;
        S.useAnd[b] = use;
        S.head[b] = (h + 1) % m;
        if (w <= c0 * S.zeta[b]) {  // K0: blind update
            S.zeta[b] = w;
            S.k0[b] += 1;
            S.iOut[b] = iOut + 1;
            S.action[b] = kActAK0;
        } else {  // line search starts at tau = 1
            S.tau[b] = 1.;
            S.iIn[b] = 0;
            S.phase[b] = 1;
            S.action[b] = kActALs;
        }
        return;
    }
    // phase B: line search step
    const double w = S.w[b], tau = S.tau[b];
    const double wT = sqrt(fmax(v[0], 0.));
    const int iOut = S.iOut[b];
    if (w <= S.wSafe[b] && wT <= c1 * w) {  // K1: educated update
        S.wSafe[b] = wT + pow(c2, (double)iOut);
        S.k1[b] += 1;
        S.phase[b] = 0;
        S.iOut[b] = iOut + 1;
        S.action[b] = kActBK1;
        return;
    }
    const double rho = wT * wT - tau * v[2];  // r'M(tau d) = tau (M r)'d
    if (rho >= sigma * wT * w) {               // K2: safeguard
        S.coef[b] = lambda * rho / (wT * wT);
        S.k2[b] += 1;
        S.phase[b] = 0;
        S.iOut[b] = iOut + 1;
        S.action[b] = kActBK2;
        return;
    }
    S.tau[b] = tau * beta;
    S.k2bt[b] += 1;
    if (S.iIn[b] >= A.maxInner - 1) {  // K3: restore the backed-up T(z)
        S.k3[b] += 1;
        S.phase[b] = 0;
        S.iOut[b] = iOut + 1;
        S.action[b] = kActBK3;
        return;
    }
    S.iIn[b] += 1;
    S.action[b] = kActBBt;
}

// One warp per instance: the lanes reduce the chunk partials of the 21 values (sums, and a
// maximum for max|Mr|) with shuffles, then lane 0 takes the instance's decision.
__global__ void k_control(const int B, const CtlArgs A) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int b = blockIdx.x * (blockDim.x >> 5) + warp;
    if (b >= B) return;  // the whole warp
    if (A.S.status[b] != -1) {
        if (lane == 0) A.S.action[b] = kActNone;
        return;
    }
    double v[kNV0 + 2 * kMaxAnderson];
#pragma unroll
    for (int k = 0; k < kNV0 + 2 * kMaxAnderson; k++) {
        double s = 0;
        if (k < A.nv)
            for (int c = lane; c < A.chunks; c += 32) {
                const double x = A.part[((size_t)b * A.nv + k) * A.chunks + c];
                s = (k == 1) ? fmax(s, x) : s + x;
            }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double y = __shfl_xor_sync(0xffffffffu, s, o);
            s = (k == 1) ? fmax(s, y) : s + y;
        }
        v[k] = s;
    }
    if (lane == 0) controlInstance(A, b, v);
}

// ------------------------------------------------------------------------------------------ vector update
template <typename T>
struct UpdArgs {
    T *Z, *CAND, *R, *PREV, *RPREV, *BACKUP, *D, *ANDR, *ANDZ;
    const int *action, *head, *useAnd;
    const double *gamma, *tau, *coef;
    int m;
};

// M = the Anderson memory (A.m) as a template parameter: the coefficients and the loop over the
// memory's columns are sized at compile time.  Four CTAs of 256 threads per SM (at most 64
// registers a thread) keep enough loads in flight for HBM.
template <typename T, int M>
__global__ void __launch_bounds__(256, 4) k_update(const Dims Dm, const UpdArgs<T> A) {
    // thread = instance b (x) and a stride of rows (y): consecutive lanes touch consecutive
    // instances of a row (coalesced), the action is read once, and the row loop is unrolled over
    // non-aliasing pointers so several rows' loads are in flight per thread
    const int B = Dm.B;
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const size_t slot = (size_t)Dm.sZ * B;
    const int act = A.action[b];
    if (act == kActNone || act == kActBK1) return;
    T *__restrict__ Z = A.Z;
    const T *__restrict__ CAND = A.CAND;
    const T *__restrict__ R = A.R;
    const long step = gridDim.y, k0 = blockIdx.y, n = Dm.sZ;
    if (act == kActAK0 || act == kActALs) {
        T *__restrict__ PREV = A.PREV;
        T *__restrict__ RPREV = A.RPREV;
        T *__restrict__ BACKUP = A.BACKUP;
        T *__restrict__ D = A.D;
        T *__restrict__ ANDR = A.ANDR;
        T *__restrict__ ANDZ = A.ANDZ;
        const int h = (A.head[b] + M - 1) % M;  // slot written this round (head already advanced)
        T g[M];
        const bool useAnd = A.useAnd[b];
#pragma unroll
        for (int s2 = 0; s2 < M; s2++)
            g[s2] = (useAnd && s2 != h) ? T(A.gamma[(size_t)b * kMaxAnderson + s2]) : T(0);
        const T gh = useAnd ? T(A.gamma[(size_t)b * kMaxAnderson + h]) : T(0);
#pragma unroll 2
        for (long k = k0; k < n; k += step) {
            const size_t o = (size_t)k * B + b;
            const T z = Z[o], r = R[o], c = CAND[o];
            const T dr = r - RPREV[o];
            const T dzr = (z - PREV[o]) - dr;
            T d = -r - gh * dzr;
#pragma unroll
            for (int s2 = 0; s2 < M; s2++)
                if (s2 != h) d -= g[s2] * ANDZ[s2 * slot + o];
            ANDR[h * slot + o] = dr;
            ANDZ[h * slot + o] = dzr;
            D[o] = d;
            PREV[o] = z;
            RPREV[o] = r;
            BACKUP[o] = c;
            Z[o] = z + d;
        }
        return;
    }
    const T cf = act == kActBK2 ? T(A.coef[b]) : T(0), tau = act == kActBBt ? T(A.tau[b]) : T(0);
    const T *__restrict__ PREVc = A.PREV;
    const T *__restrict__ BACKUPc = A.BACKUP;
    const T *__restrict__ Dc = A.D;
#pragma unroll 4
    for (long k = k0; k < n; k += step) {
        const size_t o = (size_t)k * B + b;
        switch (act) {
            case kActFinish:
            case kActCp: Z[o] = CAND[o]; break;
            case kActBK2: Z[o] = PREVc[o] - cf * R[o]; break;
            case kActBK3: Z[o] = BACKUPc[o]; break;
            case kActBBt: Z[o] = PREVc[o] + tau * Dc[o]; break;
            default: break;
        }
    }
}

// Batches below one tile: one thread per element (consecutive elements, consecutive threads).
template <typename T>
__global__ void __launch_bounds__(256) k_update_flat(const Dims Dm, const UpdArgs<T> A) {
    const int B = Dm.B;
    const size_t total = (size_t)Dm.sZ * B;
    const size_t slot = (size_t)Dm.sZ * B;
    for (size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < total; o += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(o % B);
        const int act = A.action[b];
        switch (act) {
            case kActAK0:
            case kActALs: {
                const T z = A.Z[o], r = A.R[o], c = A.CAND[o];
                const T dr = r - A.RPREV[o];
                const T dzr = (z - A.PREV[o]) - dr;
                const int m = A.m;
                const int h = (A.head[b] + m - 1) % m;  // slot written this round (head already advanced)
                T d = -r;
                if (A.useAnd[b]) {
                    const double *g = A.gamma + (size_t)b * kMaxAnderson;
                    for (int s = 0; s < m; s++) d -= T(g[s]) * (s == h ? dzr : A.ANDZ[s * slot + o]);
                }
                A.ANDR[h * slot + o] = dr;
                A.ANDZ[h * slot + o] = dzr;
                A.D[o] = d;
                A.PREV[o] = z;
                A.RPREV[o] = r;
                A.BACKUP[o] = c;
                A.Z[o] = z + d;
                break;
            }
            case kActFinish:
            case kActCp:
                A.Z[o] = A.CAND[o];
                break;
            case kActBK2:
                A.Z[o] = A.PREV[o] - T(A.coef[b]) * A.R[o];
                break;
            case kActBK3:
                A.Z[o] = A.BACKUP[o];
                break;
            case kActBBt:
                A.Z[o] = A.PREV[o] + T(A.tau[b]) * A.D[o];
                break;
            default:
                break;
        }
    }
}

// ------------------------------------------------------------------------------------------ small kernels
template <typename T>
__global__ void k_fill(T *p, size_t n, T v) {
    for (size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x) p[o] = v;
}

template <typename D, typename S>
__global__ void k_convert(D *dst, const S *src, size_t n) {
    for (size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x)
        dst[o] = (D)src[o];
}

template <typename T>
__global__ void k_copy(T *dst, const T *src, size_t n) {
    for (size_t o = (size_t)blockIdx.x * blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x) dst[o] = src[o];
}

template <typename T>
__global__ void k_scale_x0(T *x0s, const T *x0, const T *scal, int nx, int B) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nx * B) return;
    const int c = o / B;
    x0s[o] = x0[o] * scal[c];
}

__global__ void k_init_state(DevState S, int B, int warm) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    S.phase[b] = 0; S.iOut[b] = 0; S.iIn[b] = 0; S.status[b] = -1; S.errInit[b] = 1; S.action[b] = kActNone;
    S.head[b] = 0; S.useAnd[b] = 0; S.iters[b] = 0;
    S.k0[b] = S.k1[b] = S.k2[b] = S.k2bt[b] = S.k3[b] = S.calls[b] = 0;
    S.tau[b] = 0; S.zeta[b] = INFINITY; S.w[b] = INFINITY; S.wSafe[b] = INFINITY; S.tol[b] = 0; S.err[b] = INFINITY;
    S.coef[b] = 0;
    for (int k = 0; k < kMaxAnderson * kMaxAnderson; k++) S.G[(size_t)b * kMaxAnderson * kMaxAnderson + k] = 0;
    for (int k = 0; k < kMaxAnderson; k++) S.gamma[(size_t)b * kMaxAnderson + k] = 0;
    if (b == 0) { *S.timeUp = 0; }
}

// Instance compaction.  dst[k * B + s] = src[k * B + from[s]] for rows k of an element-major
// buffer: slot s receives the column of slot from[s].
template <typename T>
__global__ void k_gather_cols(T *__restrict__ dst, const T *__restrict__ src, const int *__restrict__ from, long rows,
                              int B) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const int f = from[s];
    for (long k = blockIdx.y; k < rows; k += gridDim.y) dst[(size_t)k * B + s] = src[(size_t)k * B + f];
}

// The controller state of slot s from slot from[s]: nInt int fields and nDbl double fields laid out
// [field][instance], then the m x m Gram matrices and the Anderson coefficients per instance.
__global__ void k_gather_state(int *__restrict__ id, const int *__restrict__ is, double *__restrict__ dd,
                               const double *__restrict__ ds, const int *__restrict__ from, int B, int nInt, int nDbl,
                               int perG, int perGamma) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const int f = from[s];
    for (int q = 0; q < nInt; q++) id[(size_t)q * B + s] = is[(size_t)q * B + f];
    for (int q = 0; q < nDbl; q++) dd[(size_t)q * B + s] = ds[(size_t)q * B + f];
    const size_t g0 = (size_t)nDbl * B, a0 = g0 + (size_t)perG * B;
    for (int q = 0; q < perG; q++) dd[g0 + (size_t)s * perG + q] = ds[g0 + (size_t)f * perG + q];
    for (int q = 0; q < perGamma; q++) dd[a0 + (size_t)s * perGamma + q] = ds[a0 + (size_t)f * perGamma + q];
}

// FP64 finish: columns of an element-major buffer between two solvers of different batch and
// precision, dst[k * Bd + dIdx[s]] = src[k * Bs + sIdx[s]] for s < count <= 32 (one warp lane per
// instance, warps over the rows).
template <typename TD, typename TS>
__global__ void k_move_cols(TD *__restrict__ dst, long Bd, const TS *__restrict__ src, long Bs, const int *__restrict__ dIdx,
                            const int *__restrict__ sIdx, int count, long rows) {
    const int s = threadIdx.x & 31;
    if (s >= count) return;
    const size_t d = (size_t)dIdx[s], f = (size_t)sIdx[s];
    const long w = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), nw = (long)gridDim.x * (blockDim.x >> 5);
    for (long k = w; k < rows; k += nw) dst[(size_t)k * Bd + d] = (TD)src[(size_t)k * Bs + f];
}

// The controller state of instance sIdx[s] of one solver into slot dIdx[s] of another (layouts as
// in k_gather_state, batches Bs and Bd); s < count.
__global__ void k_move_state(int *__restrict__ id, long Bd, const int *__restrict__ is, long Bs, double *__restrict__ dd,
                             const double *__restrict__ ds, const int *__restrict__ dIdx, const int *__restrict__ sIdx,
                             int count, int nInt, int nDbl, int perG, int perGamma) {
    const int s = threadIdx.x;
    if (s >= count) return;
    const size_t d = (size_t)dIdx[s], f = (size_t)sIdx[s];
    for (int q = 0; q < nInt; q++) id[(size_t)q * Bd + d] = is[(size_t)q * Bs + f];
    for (int q = 0; q < nDbl; q++) dd[(size_t)q * Bd + d] = ds[(size_t)q * Bs + f];
    const size_t gd = (size_t)nDbl * Bd, gs = (size_t)nDbl * Bs;
    for (int q = 0; q < perG; q++) dd[gd + d * perG + q] = ds[gs + f * perG + q];
    const size_t ad = gd + (size_t)perG * Bd, as = gs + (size_t)perG * Bs;
    for (int q = 0; q < perGamma; q++) dd[ad + d * perGamma + q] = ds[as + f * perGamma + q];
}

// Slots from `from` on hold no instance: mark them stopped so that they change nothing.
__global__ void k_stop_from(int *status, int from, int B) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= from && b < B) status[b] = 0;
}

// Measurement helper: put every instance in phase A with an Anderson update pending.
__global__ void k_force_phaseA(DevState S, int B, int m) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    S.status[b] = -1;
    S.phase[b] = 0;
    S.action[b] = kActALs;
    S.useAnd[b] = 1;
    S.head[b] = 1 % m;
}

// Convergence mask of the node kernels: tile t (instances 32t .. 32t+31) stays live while one
// of its instances is running; the batched kernels skip the others.
__global__ void k_tile_flags(const int *status, int B, int *tileLive) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned any = __ballot_sync(0xffffffffu, b < B && status[b] == -1);
    if ((threadIdx.x & 31) == 0 && b < B) tileLive[b >> 5] = any != 0;
}

// sum of squares of x[0 .. n) into *out (FP64)
template <typename T>
__global__ void k_sumsq(const T *x, size_t n, double *out) {
    double s = 0;
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x)
        s += (double)x[o] * (double)x[o];
    for (int q = 16; q > 0; q >>= 1) s += __shfl_xor_sync(0xffffffffu, s, q);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}

template <typename T>
__global__ void k_scale(T *x, size_t n, double f) {
    for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < n; o += (size_t)gridDim.x * blockDim.x)
        x[o] = (T)((double)x[o] * f);
}

__global__ void k_count_active(const int *status, int B, int *out) {
    __shared__ int cnt;
    if (threadIdx.x == 0) cnt = 0;
    __syncthreads();
    int c = 0;
    for (int b = threadIdx.x; b < B; b += blockDim.x) c += status[b] == -1;
    atomicAdd(&cnt, c);
    __syncthreads();
    if (threadIdx.x == 0) *out = cnt;
}

// ------------------------------------------------------------------------------------------ engine
template <typename T>
class Engine final : public EngineBase {
    template <typename U>
    friend class Engine;  // the FP64 finish moves state between an FP32 solver and its FP64 twin

public:
    Engine(const HostProblem &hp, const Options &opt, long batch, int device) {
        hp_ = hp;
        B_ = batch;
        device_ = device;
        opt_ = opt;
        if (batch < 1) throw std::invalid_argument("[Cache] batch must be >= 1");
        if (opt.anderson < 1 || opt.anderson > kMaxAnderson)
            throw std::invalid_argument("[Cache] Anderson buffer must be in [1, " + std::to_string(kMaxAnderson) + "]");
        CK(cudaSetDevice(device));
        CK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
        buildDims();
        upload();
        allocate();
        chooseKernels();
        raiseSharedLimits();
    }

    ~Engine() override {
        if (graph_) cudaGraphExecDestroy(graph_);
        for (auto &kv : graphsLive_) cudaGraphExecDestroy(kv.second);
        if (graphTemplate_) cudaGraphDestroy(graphTemplate_);
        for (void *p : allocs_) cudaFree(p);
        if (hostActive_) cudaFreeHost(hostActive_);
        if (stream_) cudaStreamDestroy(stream_);
    }

    int precisionBits() const override { return sizeof(T) * 8; }
    double lastSeconds() const override { return lastSeconds_; }

    void setInitialStates(const double *x0, long count) override {
        checkCount(count);
        std::vector<T> h((size_t)D_.nx * B_);
        for (long b = 0; b < B_; b++)
            for (int c = 0; c < D_.nx; c++) h[(size_t)c * B_ + b] = (T)(x0[(b % count) * D_.nx + c] * hp_.scaling[c]);
        CK(cudaMemcpyAsync(x0s_, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
    }

    void setInitialStatesDevice(const void *x0, long count) override {
        checkCount(count);
        if (count != B_) throw std::invalid_argument("[Cache] device initial states must cover the whole batch");
        // x0 is [nx][B] (element-major) in T precision; scale on the device
        k_scale_x0<T><<<(D_.nx * (int)B_ + 255) / 256, 256, 0, stream_>>>(x0s_, (const T *)x0, scal_, D_.nx, (int)B_);
        CK(cudaGetLastError());
    }

    void setIterate(const double *z, long count) override {
        checkCount(count);
        std::vector<T> h((size_t)D_.sZ * B_);
        for (long b = 0; b < B_; b++) {
            const double *zb = z + (size_t)(b % count) * D_.sZ;
            for (long k = 0; k < D_.sZ; k++) h[(size_t)k * B_ + b] = (T)zb[k];
        }
        CK(cudaMemcpyAsync(Z_, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
        CK(cudaStreamSynchronize(stream_));
    }

    const void *iterateDevice() const override { return Z_; }

    void setIterateFromDevice(const void *src, int srcBits, long sZ, long batch, int srcDevice) override {
        if (sZ != D_.sZ || batch != B_)
            throw std::invalid_argument("[copyIterate] solvers differ in problem size or batch");
        if (srcDevice != device_) throw std::invalid_argument("[copyIterate] solvers are on different devices");
        const size_t n = (size_t)D_.sZ * B_;
        const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
        if (srcBits == 64) k_convert<T, double><<<grid, 256, 0, stream_>>>(Z_, (const double *)src, n);
        else k_convert<T, float><<<grid, 256, 0, stream_>>>(Z_, (const float *)src, n);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream_));
    }

    void zeroIterate() override {
        fill(Z_, (size_t)D_.sZ * B_, T(0));
    }

    // The start of a solve: cold or warm buffers (cache.cuh:611-632), controller state, every tile live.
    void beginSolve(Algo algo, bool warm) {
        const size_t nz = (size_t)D_.sZ * B_;
        if (!warm) fill(Z_, nz, T(0));
        if (algo == kSpock) {
            if (warm) {  // cache.cuh:624-628: prev := z (the residual memory starts at zero)
                copy(PREV_, Z_, nz);
                fill(RPREV_, nz, T(0));
            } else {     // cache.cuh:629-631: prev := ones, residual_prev := ones
                fill(PREV_, nz, T(1));
                fill(RPREV_, nz, T(1));
            }
            fill(ANDR_, nz * opt_.anderson, T(0));
            fill(ANDZ_, nz * opt_.anderson, T(0));
        }
        k_init_state<<<((int)B_ + 127) / 128, 128, 0, stream_>>>(S_, (int)B_, warm ? 1 : 0);
        CK(cudaGetLastError());
        allLive();
        capacity_ = B_;
        compactions_ = 0;
    }

    void groupBegin(bool warm) override {
        beginSolve(kSpock, warm);
        ensureGraph();
        CK(cudaStreamSynchronize(stream_));
        groupT0_ = std::chrono::steady_clock::now();
    }
    cudaGraph_t roundGraph() override {
        ensureGraph();
        return graphTemplate_;
    }
    const int *statusDevice() const override { return S_.status; }
    void groupEnd(long rounds) override {
        lastRounds_ = rounds;
        lastCompactions_ = 0;
        lastLaunches_ = (long)launchesPerRound() * rounds + 7;
        lastSeconds_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - groupT0_).count();
    }

    void setFinishDouble(long rounds) override {
        if (rounds < 0) throw std::invalid_argument("[fp64Finish] rounds must be >= 0");
        finishAfter_ = rounds;
    }

    int run(Algo algo, bool warm) override {
        const auto t0 = std::chrono::steady_clock::now();
        beginSolve(algo, warm);
        int rounds = 0, polls = 0;
        long launches = (algo == kSpock ? 5 : 2) + 2;  // buffer fills + state init + tile flags
        const int poll = B_ > 1 ? 10 : 25;
        if (algo == kSpock) {
            cudaGraphExec_t round = graphFor(B_);
            for (;;) {
                CK(cudaGraphLaunch(round, stream_));
                rounds++;
                launches += launchesPerRound();
                if (rounds % poll == 0) {
                    polls++;
                    const int act = activeCount(t0);
                    if (act == 0) break;
                    if (maybeCompact(act)) round = graphFor(levelFor(capacity_));
                    if (finishAfter_ > 0 && rounds >= finishAfter_ && act <= kTileB && sizeof(T) == 4 && batched_) {
                        long r2 = 0, l2 = 0;
                        if (finishInDouble(t0, r2, l2)) {
                            rounds += (int)r2;
                            launches += l2;
                            break;
                        }
                    }
                }
            }
            restoreOrder();
        } else {
            for (;;) {
                teval();
                const bool check = rounds % 25 == 0;
                if (check) applyMres();
                reduceLaunch(kCp, check);
                controlLaunch(kCp);
                updateLaunch();
                tileFlagsLaunch();
                rounds++;
                launches += (D_.ns - 1) * 2 + 2 + (check ? 3 : 2) + 2;
                if (rounds % poll == 0) {
                    polls++;
                    if (activeCount(t0) == 0) break;
                }
            }
        }
        lastRounds_ = rounds;
        lastCompactions_ = compactions_;
        lastLaunches_ = launches + polls;
        CK(cudaStreamSynchronize(stream_));
        lastSeconds_ = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        return rounds;
    }

    void getIterate(long inst, double *out) override {
        if (inst < 0 || inst >= B_) throw std::invalid_argument("[Cache] instance out of range");
        std::vector<T> h((size_t)D_.sZ * B_);
        CK(cudaMemcpyAsync(h.data(), Z_, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (long k = 0; k < D_.sZ; k++) out[k] = (double)h[(size_t)k * B_ + inst];
    }

    void getIterates(double *out) override {
        std::vector<T> h((size_t)D_.sZ * B_);
        CK(cudaMemcpyAsync(h.data(), Z_, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (long b = 0; b < B_; b++)
            for (long k = 0; k < D_.sZ; k++) out[(size_t)b * D_.sZ + k] = (double)h[(size_t)k * B_ + b];
    }

    void getFirstInputs(double *out) override {
        std::vector<T> h((size_t)D_.nu * B_);
        CK(cudaMemcpyAsync(h.data(), Z_, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (long b = 0; b < B_; b++)
            for (int c = 0; c < D_.nu; c++) out[(size_t)b * D_.nu + c] = (double)h[(size_t)c * B_ + b] / hp_.scaling[D_.nx + c];
    }

    void getStatus(int *status, long *iters) override {
        std::vector<int> st(B_), it(B_);
        CK(cudaMemcpyAsync(st.data(), S_.status, B_ * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        CK(cudaMemcpyAsync(it.data(), S_.iters, B_ * sizeof(int), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (long b = 0; b < B_; b++) {
            if (status) status[b] = st[b];
            if (iters) iters[b] = it[b];
        }
    }

    void getCounters(long *out) override {
        int *ptrs[7] = {S_.k0, S_.k1, S_.k2, S_.k2bt, S_.k3, S_.calls, S_.iters};
        for (int k = 0; k < 7; k++) {
            int v = 0;
            CK(cudaMemcpyAsync(&v, ptrs[k], sizeof(int), cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            out[k] = v;
        }
    }

    void getCountersAll(long *out) override {
        int *ptrs[7] = {S_.k0, S_.k1, S_.k2, S_.k2bt, S_.k3, S_.calls, S_.iters};
        std::vector<int> h((size_t)B_);
        for (int k = 0; k < 7; k++) {
            CK(cudaMemcpyAsync(h.data(), ptrs[k], sizeof(int) * (size_t)B_, cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            for (long b = 0; b < B_; b++) out[(size_t)b * 7 + k] = h[(size_t)b];
        }
    }

    void op(const double *prim, double *dual) override {
        allLive();
        uploadSlice(W1_, prim, 0, D_.sPrim);
        OpArgs<T> A = blankArgs();
        A.in1 = W1_; A.a1 = 1; A.cL = 1; A.out = W2_;
        launchLop<2>(A);
        downloadSlice(W2_, dual, D_.sPrim, D_.sDual);
    }

    void adj(const double *dual, double *prim) override {
        allLive();
        uploadSlice(W1_, dual, D_.sPrim, D_.sDual);
        OpArgs<T> A = blankArgs();
        A.in1 = W1_; A.a1 = 1; A.cL = 1; A.out = W2_;
        launchLstar<2>(A);
        downloadSlice(W2_, prim, 0, D_.sPrim);
    }

    void cpStep(const double *x0, const double *z, double *cand) override {
        allLive();
        setInitialStates(x0, 1);
        uploadSlice(Z_, z, 0, D_.sZ);
        teval();
        downloadSlice(CAND_, cand, 0, D_.sZ);
    }

    // Cache::getDual (cache.cuh:371-376): the dual half of T at the current iterate with the given
    // primal candidate, prox_{g*}(z_d + gamma L(2 prim - z_p)) (T form of L with CAND = prim).
    void dualOf(const double *prim, double *dual) override {
        allLive();
        uploadSlice(CAND_, prim, 0, D_.sPrim);
        launchLop<0>(tevalLopArgs());
        downloadSlice(CAND_, dual, D_.sPrim, D_.sDual);
    }

    void warmStartPca(const void *basis, const void *coef, int k, const float *mean) override {
        if (!basis || !coef || !mean) throw std::invalid_argument("[warmStart] null device pointer");
        if (!gemmErr_) gemmErr_ = dalloc<int>(1);
        CK(cudaMemsetAsync(gemmErr_, 0, sizeof(int), stream_));
        GemmEpilogue E;
        E.rowAdd = mean;
        // element-major sZ x B = row-major with ldd = B, in the solver's precision
        if (sizeof(T) == 4) E.D = reinterpret_cast<float *>(Z_);
        else E.D64 = reinterpret_cast<double *>(Z_);
        E.ldd = B_;
        E.err = gemmErr_;
        gemmBf16(basis, coef, D_.sZ, B_, k, E, stream_);
        int err = 0;
        CK(cudaMemcpyAsync(&err, gemmErr_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        if (err) throw std::runtime_error("[warmStart] the tensor-core pipeline gave up (code " + std::to_string(err) + ")");
    }

    void reduceCheck(const double *r, const double *mr, double *out3) override {
        allLive();
        uploadSlice(R_, r, 0, D_.sZ);
        uploadSlice(MR_, mr, 0, D_.sZ);
        const size_t nz = (size_t)D_.sZ * B_;
        fill(RPREV_, nz, T(0));
        fill(ANDR_, nz * opt_.anderson, T(0));
        k_force_phaseA<<<((int)B_ + 127) / 128, 128, 0, stream_>>>(S_, (int)B_, (int)opt_.anderson);
        CK(cudaGetLastError());
        reduceLaunch(kSpock, true);
        std::vector<double> h((size_t)chunks_ * nv_);
        CK(cudaMemcpyAsync(h.data(), part_, h.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));  // instance 0
        CK(cudaStreamSynchronize(stream_));
        double s0 = 0, mx = 0, s3 = 0;
        for (int c = 0; c < chunks_; c++) {
            s0 += h[(size_t)0 * chunks_ + c];
            mx = std::max(mx, h[(size_t)1 * chunks_ + c]);
            s3 += h[(size_t)3 * chunks_ + c];
        }
        out3[0] = s0; out3[1] = mx; out3[2] = s3;  // c = r - r_prev = r: c'c = r'r
    }

    void applyM(const double *z, double *mz) override {
        allLive();
        // M z through the residual kernels, which read the residual buffer
        uploadSlice(R_, z, 0, D_.sZ);
        applyMres();
        downloadSlice(MR_, mz, 0, D_.sZ);
    }

    double normLsq(int iters, double rtol) override {  // problem.py:402-417 computes the same with ARPACK
        allLive();
        const size_t np = (size_t)D_.sPrim * B_;
        fill(W1_, (size_t)D_.sZ * B_, T(0));
        fill(W1_, np, T(1));
        double *dsum = nullptr;
        CK(cudaMalloc(&dsum, sizeof(double)));
        double lam = 0, nrm2 = 0;
        auto norm2 = [&]() {
            CK(cudaMemsetAsync(dsum, 0, sizeof(double), stream_));
            k_sumsq<T><<<(int)std::min<size_t>((np + 255) / 256, 152 * 8), 256, 0, stream_>>>(W1_, np, dsum);
            CK(cudaGetLastError());
            double h = 0;
            CK(cudaMemcpyAsync(&h, dsum, sizeof(double), cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            return h;
        };
        nrm2 = norm2();
        k_scale<T><<<(int)std::min<size_t>((np + 255) / 256, 152 * 8), 256, 0, stream_>>>(W1_, np, 1. / std::sqrt(nrm2));
        int steady = 0;
        for (int it = 0; it < iters; it++) {
            OpArgs<T> A = blankArgs();
            A.in1 = W1_; A.a1 = 1; A.cL = 1; A.out = W2_;  // W2 dual = L p
            launchLop<2>(A);
            OpArgs<T> A2 = blankArgs();
            A2.in1 = W2_; A2.a1 = 1; A2.cL = 1; A2.out = W1_;  // W1 prim = L* L p
            launchLstar<2>(A2);
            nrm2 = norm2();
            const double prev = lam;
            lam = std::sqrt(nrm2);  // ||L* L p|| with ||p|| = 1
            if (!(lam > 0)) break;
            steady = std::fabs(lam - prev) <= rtol * lam ? steady + 1 : 0;
            if (rtol > 0 && steady >= 20) break;
            k_scale<T><<<(int)std::min<size_t>((np + 255) / 256, 152 * 8), 256, 0, stream_>>>(W1_, np, 1. / lam);
            CK(cudaGetLastError());
        }
        cudaFree(dsum);
        return lam;  // every instance holds the same vector, and the norm runs over all of them
    }

    void setTuning(int lstar, int lop, int dyn) override {
        for (int v : {lstar, lop, dyn})
            if (v != 1 && v != 2 && v != 4 && v != 8) throw std::invalid_argument("[tuning] tiles per CTA must be 1, 2, 4 or 8");
        if (!batched_) return;
        tuned_ = true;
        tpcLstar_ = lstar;
        lstarDbl_ = lstar > 1 && canDblLstar();
        tpcLop_ = lop;
        lopDbl_ = lop > 1 && canDblLop();
        tpcDyn_ = dyn;
        backDbl_ = dyn > 1 && canDblBack();
        fwdDbl_ = dyn > 1 && canDblFwd();
        dropGraphs();  // the captured rounds have the old launch shapes
    }

    void tuning(int *out5) override {
        autotune();
        out5[0] = tpcLstar_; out5[1] = lstarDbl_; out5[2] = tpcLop_; out5[3] = lopDbl_; out5[4] = batched_ ? tpcDyn_ : 0;
    }

    double kernelMs(const char *which, int reps) override {
        autotune();
        allLive();  // time the kernels over the whole batch
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        std::string w(which);
        if (w == "reduce" || w == "update") {  // time the bookkeeping with every instance in phase A
            k_force_phaseA<<<((int)B_ + 127) / 128, 128, 0, stream_>>>(S_, (int)B_, (int)opt_.anderson);
            CK(cudaGetLastError());
        }
        auto once = [&]() {
            if (w == "lop") launchLop<0>(tevalLopArgs());
            else if (w == "lstar") launchLstar<0>(tevalLstarArgs());
            else if (w == "mlop") launchLop<1>(mLopArgs());
            else if (w == "mlstar") launchLstar<1>(mLstarArgs());
            else if (w == "reduce") reduceLaunch(kSpock, true);
            else if (w == "update") updateLaunch();
            else if (w == "dyn") dynamics();
            else if (w == "teval") teval();
            else if (w == "round") roundSpock();
            else throw std::invalid_argument("unknown kernel " + w);
        };
        once();
        CK(cudaEventRecord(e0, stream_));
        for (int r = 0; r < reps; r++) once();
        CK(cudaEventRecord(e1, stream_));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return ms / reps;
    }

    void timedRounds(int rounds, float *ms) override {
        ensureGraph();
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        CK(cudaEventRecord(e0, stream_));
        for (int r = 0; r < rounds; r++) CK(cudaGraphLaunch(graph_, stream_));
        CK(cudaEventRecord(e1, stream_));
        CK(cudaEventSynchronize(e1));
        CK(cudaEventElapsedTime(ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }

    // Algorithmic bytes per launch: distinct matrix bytes once + vector elements read and
    // written once, for all B instances.
    long bytesPerRoundAlgorithmic(const char *which) const override {
        const std::string w(which);
        const long s = sizeof(T), B = B_;
        const long n = D_.n, nnl = D_.nnl, nl = D_.nl, nx = D_.nx, nu = D_.nu;
        const long matL = s * (n * (nx * nx + nu * nu) + nx * nx);          // sqrtQ, sqrtR, leaf sqrtQ
        const long matK = s * nnl * (long)D_.nd * D_.nd;                     // NNtr
        const long sXU = nx * n + nu * nnl;  // x and u: their residual rows are written by the dynamics sweep
        // T form of L: reads p and pbar, reads d, writes the candidate d and its residual
        if (w == "lop") return matL + s * B * (2 * D_.sPrim + 3 * D_.sDual);
        // T form of L*: reads d, reads p, writes the candidate p and the residual of y, t, s
        if (w == "lstar") return matL + matK + s * B * (D_.sDual + 2 * D_.sPrim + (D_.sPrim - sXU));
        if (w == "mlop") return matL + s * B * (D_.sPrim + 2 * D_.sDual);    // reads r_p, r_d; writes (Mr)_d
        if (w == "mlstar") return matL + s * B * (D_.sDual + 2 * D_.sPrim);  // reads r_d, r_p; writes (Mr)_p
        if (w == "update") return s * B * D_.sZ * (5 + 7 + (opt_.anderson - 1));
        if (w == "reduce") return s * B * D_.sZ * (3 + opt_.anderson);
        if (w == "dyn") {
            const long mats = s * (n * (nu * nx + nx * nu + nx * nx + nx * (nx + nu)) + nnl * (nu * nx + nu * nu));
            return mats + s * B * (4 * (nx * n + nu * nnl));
        }
        (void)nl;
        return 0;
    }

    void projectDynamicsOn(const void *x0, void *primUX, void *scratch, size_t scratchBytes,
                           cudaStream_t stream) override {
        if (B_ != 1) throw std::invalid_argument("[projectDynamics] needs a solver built with batch 1");
        const size_t need = ((size_t)D_.nx * D_.n + (size_t)D_.nu * D_.nnl) * sizeof(T);
        if (need > scratchBytes)
            throw std::invalid_argument("[projectDynamics] problem needs " + std::to_string(need) +
                                        " bytes of workspace, more than the " + std::to_string(scratchBytes) +
                                        "-byte static buffer");
        T *Q = static_cast<T *>(scratch), *DD = Q + (size_t)D_.nx * D_.n;
        T *cand = static_cast<T *>(primUX);
        const int N = D_.ns - 1;
        for (int st = N - 1; st >= 0; st--) {
            k_dyn_back<T><<<nodeGrid(stageCount_[st]), kNodeThreads, smBack(), stream>>>(P_, D_, cand, Q, DD, stageFrom_[st], st);
            CK(cudaGetLastError());
        }
        for (int st = 0; st < N; st++) {
            k_dyn_fwd<T><<<nodeGrid(stageCount_[st]), kNodeThreads, smFwd(), stream>>>(P_, D_, cand, DD, (const T *)x0,
                                                                                       stageFrom_[st], nullptr, nullptr);
            CK(cudaGetLastError());
        }
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CK(cudaStreamIsCapturing(stream, &cs));
        if (cs == cudaStreamCaptureStatusNone) CK(cudaStreamSynchronize(stream));  // a capturing stream cannot wait
    }

    int launchesPerRound() const override { return 2 * (D_.ns - 1) + 2 + 2 + 4; }

private:
    Options opt_;
    Dims D_{};
    DevProblem<T> P_{};
    PadMats<T> M_{};
    bool batched_ = false;  // kernels_batch.cuh for >= 32 instances, kernels.cuh otherwise
    bool lstarDbl_ = false, lopDbl_ = false;  // L*, L double-buffer their instance tiles
    int tpcLstar_ = 1, tpcLop_ = 1;           // instance tiles per L* / L CTA (autotune())
    int tpcDyn_ = 1;                          // instance tiles per dynamics-sweep CTA
    bool backDbl_ = false, fwdDbl_ = false;
    bool tuned_ = false;
    static constexpr int kTilesPerCta = 8;
    DevState S_{};
    cudaStream_t stream_ = nullptr;
    cudaGraphExec_t graph_ = nullptr;
    cudaGraph_t graphTemplate_ = nullptr;
    std::map<long, cudaGraphExec_t> graphsLive_;  // rounds over fewer slots (after compactions)
    long gridB_ = 0;                               // slots the launches cover while capturing (0: all)
    std::chrono::steady_clock::time_point groupT0_;
    std::vector<void *> allocs_;
    T *Z_ = nullptr, *CAND_ = nullptr, *R_ = nullptr, *MR_ = nullptr, *PREV_ = nullptr, *RPREV_ = nullptr;
    T *BACKUP_ = nullptr, *DIR_ = nullptr, *ANDR_ = nullptr, *ANDZ_ = nullptr, *Q_ = nullptr, *DD_ = nullptr;
    T *x0s_ = nullptr, *W1_ = nullptr, *W2_ = nullptr, *scal_ = nullptr;
    // instance compaction: slot s holds instance slotInst_[s]; state blocks and their copies
    int *ib_ = nullptr, *ibTmp_ = nullptr, *from_ = nullptr;
    double *db_ = nullptr, *dbTmp_ = nullptr;
    std::vector<int> slotInst_;
    long capacity_ = 0;  // slots in live tiles after the last compaction
    int compactions_ = 0;
    double *part_ = nullptr;
    int *gemmErr_ = nullptr;  // error flag of the tensor-core GEMM (warmStartPca)
    long finishAfter_ = 0;    // FP64 finish: rounds after which the last tile moves to FP64 (0: never)
    std::unique_ptr<Engine<double>> twin_;
    int *twinIdx_ = nullptr;  // slot lists of a move: twin slots, then this solver's slots
    int *hostActive_ = nullptr, *devActive_ = nullptr;
    int chunks_ = 1, nv_ = 0;
    long rowsPerChunk_ = 1;
    double lastSeconds_ = 0;
    std::vector<int> stageFrom_, stageCount_;

    void checkCount(long count) const {
        if (count < 1 || count > B_) throw std::invalid_argument("[Cache] instance count out of range");
    }

    template <typename U>
    U *dalloc(size_t n) {
        void *p = nullptr;
        CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(U)));
        allocs_.push_back(p);
        return (U *)p;
    }

    template <typename U>
    const U *upvec(const std::vector<double> &v) {
        if (v.empty()) return nullptr;
        std::vector<U> h(v.begin(), v.end());
        U *d = dalloc<U>(h.size());
        CK(cudaMemcpy(d, h.data(), h.size() * sizeof(U), cudaMemcpyHostToDevice));
        return d;
    }

    const int *upidx(const std::vector<long> &v) {
        std::vector<int> h(v.begin(), v.end());
        int *d = dalloc<int>(h.size());
        CK(cudaMemcpy(d, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
        return d;
    }

    void buildDims() {
        const HostProblem &p = hp_;
        Dims &D = D_;
        D.n = (int)p.numNodes; D.nnl = (int)p.numNonleaf; D.nl = (int)p.numLeaf; D.ns = (int)p.numStages;
        D.nx = (int)p.nx; D.nu = (int)p.nu; D.nxu = D.nx + D.nu; D.ne = (int)p.numEvents;
        D.yD = (int)p.yDim; D.nd = (int)p.nullDim;
        D.costNl = p.costNonleaf; D.costL = p.costLeaf; D.conNl = p.conNonleaf; D.conL = p.conLeaf;
        D.affine = p.affine ? 1 : 0;
        D.dIII = (int)p.dimIII; D.dIV = (int)p.dimIV; D.dV = (int)p.dimV; D.dVI = (int)p.dimVI;
        D.gNl = (int)p.nlGammaRows; D.gL = (int)p.lGammaRows;
        D.oX = p.sizeU; D.oY = D.oX + p.sizeX; D.oT = D.oY + p.sizeY; D.oS = D.oT + p.sizeT; D.sPrim = p.sizePrim;
        D.oI = p.sizePrim; D.oII = D.oI + p.sizeI; D.oIII = D.oII + p.sizeII; D.oIV = D.oIII + p.sizeIII;
        D.oV = D.oIV + p.sizeIV; D.oVI = D.oV + p.sizeV; D.sDual = p.sizeDual; D.sZ = p.sizeIterate();
        D.B = (int)B_;
        D.TB = B_ >= 32 ? 32 : (int)B_;
        for (long s = 0; s < p.numStages; s++) {
            stageFrom_.push_back((int)p.stageFrom[s]);
            stageCount_.push_back((int)(p.stageTo[s] - p.stageFrom[s] + 1));
        }
        if (D.nd > 64 || D.nx > 4096) throw std::invalid_argument("[Cache] problem dimensions exceed kernel limits");
    }

    void upload() {
        const HostProblem &p = hp_;
        P_.anc = upidx(p.ancestors);
        P_.chFrom = upidx(p.childFrom);
        P_.numCh = upidx(p.numChildren);
        P_.BTr = upvec<T>(p.BTr); P_.AB = upvec<T>(p.AB); P_.K = upvec<T>(p.K); P_.ABKTr = upvec<T>(p.ABKTr);
        P_.APB = upvec<T>(p.APB); P_.chol = upvec<T>(p.lowChol); P_.e = upvec<T>(p.e); P_.Pe = upvec<T>(p.Pe);
        P_.sqrtQ = upvec<T>(p.sqrtQ); P_.sqrtR = upvec<T>(p.sqrtR); P_.q = upvec<T>(p.q); P_.r = upvec<T>(p.r);
        P_.trans = upvec<T>(p.translation);
        P_.lSqrtQ = upvec<T>(p.leafSqrtQ); P_.lq = upvec<T>(p.leafQ); P_.lTrans = upvec<T>(p.leafTranslation);
        P_.nlLo = upvec<T>(p.nlLower); P_.nlHi = upvec<T>(p.nlUpper); P_.lLo = upvec<T>(p.lLower); P_.lHi = upvec<T>(p.lUpper);
        P_.NNtr = upvec<T>(p.NNtr); P_.b = upvec<T>(p.b);
        P_.grad = upvec<T>(p.gradient); P_.lGrad = upvec<T>(p.leafGradient);
        P_.radius = (T)p.nlRadius;
        P_.step = (T)p.stepSize;
        scal_ = const_cast<T *>(upvec<T>(p.scaling));
    }

    // Column-major matrices re-laid with the leading dimension padded to a multiple of 16 rows
    // (zero pad), optionally transposed, for the warp-uniform vector loads of kernels_batch.cuh.
    const T *padUpload(const std::vector<double> &src, int rows, int cols, long mats, bool transpose = false) {
        if (src.empty()) return nullptr;
        const int ld = pad16(rows);
        std::vector<T> h((size_t)ld * cols * mats, T(0));
        for (long m = 0; m < mats; m++)
            for (int c = 0; c < cols; c++)
                for (int r = 0; r < rows; r++) {
                    const size_t s = transpose ? (size_t)m * rows * cols + (size_t)r * cols + c
                                               : (size_t)m * rows * cols + (size_t)c * rows + r;
                    h[(size_t)m * ld * cols + (size_t)c * ld + r] = (T)src[s];
                }
        T *d = dalloc<T>(h.size());
        CK(cudaMemcpy(d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
        return d;
    }

    // Shared memory of the batched kernels (rows staged x 32 instances).
    size_t lx() const { return (size_t)pad16(D_.nx); }
    size_t lu() const { return (size_t)pad16(D_.nu); }
    // L* and L stage the node's matrices once and one (or, double-buffered, two) instance
    // tiles of input and base rows.
    // rows of the constraint blocks: identity part and Gamma part (nonleaf, leaf)
    int idNl() const {
        return (D_.conNl == kConRectangle || D_.conNl == kConPolyhedronWithIdentity || D_.conNl == kConRectangleInputBall)
                   ? D_.nxu
                   : 0;
    }
    int idL() const { return (D_.conL == kConRectangle || D_.conL == kConPolyhedronWithIdentity) ? D_.nx : 0; }
    int gNl() const { return (D_.conNl == kConPolyhedron || D_.conNl == kConPolyhedronWithIdentity) ? D_.gNl : 0; }
    int gL() const { return (D_.conL == kConPolyhedron || D_.conL == kConPolyhedronWithIdentity) ? D_.gL : 0; }
    bool needsBatched() const {
        return D_.costNl == kCostLinear || D_.costL == kCostLinear || gNl() > 0 || gL() > 0 ||
               D_.conNl == kConPolyhedronWithIdentity || D_.conL == kConPolyhedronWithIdentity ||
               D_.conNl == kConRectangleInputBall;
    }
    // Shared memory of the batched kernels; `gm`: node matrices read in place, not staged.
    size_t bLstar(bool dbl = false) const { return bLstar(dbl, (D_.gmat & kGmatLstar) != 0); }
    size_t bLstar(bool dbl, bool gm) const {
        const size_t in = (size_t)std::max(D_.ne * D_.dIV + idNl() + gNl() + D_.yD + 2 + 2 * D_.ne, D_.dVI + idL() + gL());
        const size_t base = (size_t)std::max(D_.nxu + D_.yD + 2 * D_.ne + 2, D_.nx);
        const size_t mats = gm ? 0 :
                            std::max((size_t)D_.ne * (lx() * D_.nx + lu() * D_.nu + lx() + lu()), lx() * D_.nx + lx()) +
                            std::max((size_t)pad16(D_.nxu) * gNl(), (size_t)pad16(D_.nx) * gL());
        const size_t gv = (gNl() || gL() || D_.costNl == kCostLinear || D_.costL == kCostLinear) ? (size_t)D_.nxu : 0;
        return (mats + ((dbl ? 2 : 1) * (in + base) + (size_t)D_.nd + gv) * kTileB) * sizeof(T) + (in + base) * sizeof(int);
    }
    size_t bLop(bool dbl = false) const { return bLop(dbl, (D_.gmat & kGmatLop) != 0); }
    size_t bLop(bool dbl, bool gm) const {
        const size_t in = (size_t)std::max(2 * D_.nxu + D_.yD + 2, D_.nxu + D_.nx + 2);
        const size_t base = (size_t)std::max(D_.yD + 1 + idNl() + gNl() + D_.dIV, D_.dIV + idL() + gL() + D_.dVI);
        const size_t mats = gm ? 0 :
                            2 * lx() * D_.nx + lu() * D_.nu +
                            std::max((size_t)pad16(gNl()) * D_.nxu, (size_t)pad16(gL()) * D_.nx);
        return (mats + ((size_t)std::max({D_.dIV, D_.dVI, D_.nu}) + kTileWarps + (dbl ? 2 : 1) * (2 * in + base)) * kTileB) *
                   sizeof(T) +
               (in + base) * sizeof(int);
    }
    size_t smLstarB() const { return bLstar(lstarDbl_); }
    size_t smLopB() const { return bLop(lopDbl_); }
    bool canDblLstar() const { return bLstar(true) <= 220 * 1024; }
    bool canDblLop() const { return bLop(true) <= 220 * 1024; }
    size_t bBack(bool dbl = false) const { return bBack(dbl, (D_.gmat & kGmatBack) != 0); }
    size_t bBack(bool dbl, bool gm) const {
        const size_t mats = gm ? 0 : (size_t)D_.ne * (lu() * D_.nx + lx() * D_.nu + lx() * D_.nx) + lx() * D_.nu + lu() * D_.nu;
        const size_t dOwn = sizeof(T) == 4 && D_.nx < D_.nu ? D_.nu : 0;  // d's own rows (k_dyn_back_b)
        return (mats + ((dbl ? 2 : 1) * (size_t)(D_.ne * D_.nx + D_.nu + D_.nx) + D_.nu + dOwn) * kTileB) * sizeof(T);
    }
    size_t bFwd(bool dbl = false) const { return bFwd(dbl, (D_.gmat & kGmatFwd) != 0); }
    size_t bFwd(bool dbl, bool gm) const {
        const size_t mats = gm ? 0 : lu() * D_.nx + (size_t)D_.ne * lx() * D_.nxu;
        return (mats + (dbl ? 2 : 1) * (size_t)(D_.nxu + 2 * D_.nu + D_.ne * D_.nx + D_.nx) * kTileB) * sizeof(T);
    }
    bool canDblBack() const { return bBack(true) <= 220 * 1024; }
    bool canDblFwd() const { return bFwd(true) <= 220 * 1024; }

    void chooseKernels() {
        const int maxRows = kRT * kTileWarps * kMaxTasks;
        // node matrices too large for shared memory are read in place by the kernels concerned
        const size_t cap = 220 * 1024;
        D_.gmat = (bLstar(false, false) > cap ? kGmatLstar : 0) | (bLop(false, false) > cap ? kGmatLop : 0) |
                  (bBack(false, false) > cap ? kGmatBack : 0) |
                  (bFwd(false, false) > cap ? kGmatFwd : 0);
        // linear costs and polyhedral constraints exist only in the batched kernels, which also run
        // batches below one tile (the lanes past the batch stay idle)
        const bool fits = pad16(D_.nx) <= maxRows && pad16(D_.nu) <= maxRows && pad16(D_.nxu) <= maxRows &&
                          pad16(std::max(gNl(), gL())) <= maxRows && D_.nd <= 64 &&
                          std::max({bLstar(), bLop(), bBack(), bFwd()}) <= 220 * 1024;
        if (needsBatched() && !fits)
            throw std::invalid_argument("[Cache] problem too large for the kernels that support its costs and constraints");
        batched_ = fits && (B_ >= kTileB || needsBatched());
        if (!batched_) return;
        const HostProblem &p = hp_;
        const int nx = D_.nx, nu = D_.nu;
        M_.sqrtQ = padUpload(p.sqrtQ, nx, nx, p.numNodes);
        M_.sqrtR = padUpload(p.sqrtR, nu, nu, p.numNodes);
        M_.q = padUpload(p.q, nx, 1, p.numNodes);
        M_.r = padUpload(p.r, nu, 1, p.numNodes);
        M_.lSqrtQ = padUpload(p.leafSqrtQ, nx, nx, 1);
        M_.lq = padUpload(p.leafQ, nx, 1, 1);
        M_.BTr = padUpload(p.BTr, nu, nx, p.numNodes);
        M_.APB = padUpload(p.APB, nx, nu, p.numNodes);
        M_.ABKTr = padUpload(p.ABKTr, nx, nx, p.numNodes);
        M_.Kt = padUpload(p.K, nx, nu, p.numNonleaf, true);  // K' from K (nu x nx)
        M_.K = padUpload(p.K, nu, nx, p.numNonleaf);
        M_.chol = padUpload(p.lowChol, nu, nu, p.numNonleaf);
        if (sizeof(T) == 4) {  // (I + sum B'PB)^-1 as a float pair hi + lo
            std::vector<double> inv = choleskyInverses(p.lowChol, nu, p.numNonleaf), lo(inv.size());
            for (size_t k = 0; k < inv.size(); k++) lo[k] = inv[k] - (double)(float)inv[k];
            M_.cholInv = padUpload(inv, nu, nu, p.numNonleaf);
            M_.cholInvLo = padUpload(lo, nu, nu, p.numNonleaf);
        }
        M_.AB = padUpload(p.AB, nx, nx + nu, p.numNodes);
        if (gNl()) {
            M_.nlG = padUpload(p.nlGamma, gNl(), D_.nxu, 1);
            M_.nlGT = padUpload(p.nlGamma, D_.nxu, gNl(), 1, true);
        }
        if (gL()) {
            M_.lG = padUpload(p.lGamma, gL(), nx, 1);
            M_.lGT = padUpload(p.lGamma, nx, gL(), 1, true);
        }
    }

    // (L L')^-1 of every lower Cholesky factor L (nu x nu, column-major), in FP64.
    static std::vector<double> choleskyInverses(const std::vector<double> &chol, int nu, long mats) {
        std::vector<double> out((size_t)nu * nu * mats), Li((size_t)nu * nu);
        for (long m = 0; m < mats; m++) {
            const double *L = chol.data() + (size_t)m * nu * nu;  // L(r, c) at c * nu + r
            std::fill(Li.begin(), Li.end(), 0.);
            for (int c = 0; c < nu; c++) {  // column c of L^-1 by forward substitution
                for (int r = c; r < nu; r++) {
                    double v = r == c ? 1. : 0.;
                    for (int k = c; k < r; k++) v -= L[(size_t)k * nu + r] * Li[(size_t)c * nu + k];
                    Li[(size_t)c * nu + r] = v / L[(size_t)r * nu + r];
                }
            }
            double *O = out.data() + (size_t)m * nu * nu;
            for (int c = 0; c < nu; c++)
                for (int r = 0; r < nu; r++) {  // (L^-T L^-1)(r, c) = sum_k Li(k, r) Li(k, c)
                    double v = 0;
                    for (int k = std::max(r, c); k < nu; k++) v += Li[(size_t)r * nu + k] * Li[(size_t)c * nu + k];
                    O[(size_t)c * nu + r] = v;
                }
        }
        return out;
    }

    void allocate() {
        const size_t nz = (size_t)D_.sZ * B_;
        Z_ = dalloc<T>(nz); CAND_ = dalloc<T>(nz); R_ = dalloc<T>(nz); MR_ = dalloc<T>(nz);
        PREV_ = dalloc<T>(nz); RPREV_ = dalloc<T>(nz); BACKUP_ = dalloc<T>(nz); DIR_ = dalloc<T>(nz);
        ANDR_ = dalloc<T>(nz * opt_.anderson); ANDZ_ = dalloc<T>(nz * opt_.anderson);
        Q_ = dalloc<T>((size_t)D_.nx * D_.n * B_); DD_ = dalloc<T>((size_t)D_.nu * D_.nnl * B_);
        x0s_ = dalloc<T>((size_t)D_.nx * B_);
        W1_ = dalloc<T>(nz); W2_ = dalloc<T>(nz);
        fill(Z_, nz, T(0)); fill(CAND_, nz, T(0)); fill(R_, nz, T(0)); fill(MR_, nz, T(0));
        fill(DIR_, nz, T(0)); fill(W1_, nz, T(0)); fill(W2_, nz, T(0)); fill(x0s_, (size_t)D_.nx * B_, T(0));
        nv_ = kNV0 + 2 * kMaxAnderson;
        const int tiles = (int)((B_ + 31) / 32);
        const int target = 1216;  // ~8 CTAs per SM
        chunks_ = std::max(1, std::min<int>(target / tiles, (int)((D_.sZ + 255) / 256)));
        rowsPerChunk_ = (D_.sZ + chunks_ - 1) / chunks_;
        part_ = dalloc<double>((size_t)chunks_ * nv_ * B_);
        const size_t Bi = (size_t)B_;
        int *ib = dalloc<int>(Bi * 16);
        ib_ = ib;
        S_.phase = ib; S_.iOut = ib + Bi; S_.iIn = ib + 2 * Bi; S_.status = ib + 3 * Bi; S_.errInit = ib + 4 * Bi;
        S_.action = ib + 5 * Bi; S_.head = ib + 6 * Bi; S_.useAnd = ib + 7 * Bi; S_.iters = ib + 8 * Bi;
        S_.k0 = ib + 9 * Bi; S_.k1 = ib + 10 * Bi; S_.k2 = ib + 11 * Bi; S_.k2bt = ib + 12 * Bi; S_.k3 = ib + 13 * Bi;
        S_.calls = ib + 14 * Bi;
        double *db = dalloc<double>(Bi * (8 + 2 * kMaxAnderson * kMaxAnderson));
        db_ = db;
        if (B_ >= 2 * kTileB) {  // compaction workspaces
            ibTmp_ = dalloc<int>(Bi * 16);
            dbTmp_ = dalloc<double>(Bi * (8 + 2 * kMaxAnderson * kMaxAnderson));
            from_ = dalloc<int>(Bi);
        }
        slotInst_.resize(Bi);
        for (size_t q = 0; q < Bi; q++) slotInst_[q] = (int)q;
        S_.tau = db; S_.zeta = db + Bi; S_.w = db + 2 * Bi; S_.wSafe = db + 3 * Bi; S_.tol = db + 4 * Bi;
        S_.err = db + 5 * Bi; S_.coef = db + 6 * Bi; S_.G = db + 8 * Bi;
        S_.gamma = S_.G + Bi * kMaxAnderson * kMaxAnderson;
        int *misc = dalloc<int>(4);
        S_.timeUp = misc; S_.active = misc + 1;
        devActive_ = misc + 2;
        S_.tileLive = dalloc<int>((size_t)tiles);
        allLive();
        CK(cudaMemset(misc, 0, 4 * sizeof(int)));
        CK(cudaMemset(ib, 0, Bi * 16 * sizeof(int)));
        CK(cudaMemset(db, 0, Bi * (8 + 2 * kMaxAnderson * kMaxAnderson) * sizeof(double)));
        CK(cudaMallocHost((void **)&hostActive_, sizeof(int)));
        k_init_state<<<((int)B_ + 127) / 128, 128, 0, stream_>>>(S_, (int)B_, 0);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(stream_));
    }

    // Opt in to more than 48 KB of dynamic shared memory where a problem needs it.
    template <typename K>
    void optIn(K kernel, size_t bytes) {
        if (bytes <= 40 * 1024) return;  // the default limit also covers static shared memory
        if (bytes > 227 * 1024) throw std::invalid_argument("[Cache] problem too large for the shared-memory tiles");
        CK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    }

    // The same through a launcher translation unit's cudaFuncSetAttribute.
    void optInBytes(cudaError_t (*setter)(int), size_t bytes) {
        if (bytes <= 40 * 1024) return;
        if (bytes > 227 * 1024) throw std::invalid_argument("[Cache] problem too large for the shared-memory tiles");
        CK(setter((int)bytes));
    }

    void raiseSharedLimits() {
        if (batched_) {
            // the limit covers the largest shape the tuner may pick
            const bool gS = D_.gmat & kGmatLstar, gL = D_.gmat & kGmatLop;
            optInBytes(gS ? optInLstarB<T, 0, true> : optInLstarB<T, 0, false>, bLstar(canDblLstar()));
            optInBytes(gS ? optInLstarB<T, 1, true> : optInLstarB<T, 1, false>, bLstar(canDblLstar()));
            optInBytes(gS ? optInLstarB<T, 2, true> : optInLstarB<T, 2, false>, bLstar(canDblLstar()));
            optInBytes(gL ? optInLopB<T, 0, true> : optInLopB<T, 0, false>, bLop(canDblLop()));
            optInBytes(gL ? optInLopB<T, 1, true> : optInLopB<T, 1, false>, bLop(canDblLop()));
            optInBytes(gL ? optInLopB<T, 2, true> : optInLopB<T, 2, false>, bLop(canDblLop()));
            if (D_.gmat & kGmatBack) optIn(k_dyn_back_b<T, true>, bBack(canDblBack()));
            else optIn(k_dyn_back_b<T, false>, bBack(canDblBack()));
            if (D_.gmat & kGmatFwd) optIn(k_dyn_fwd_b<T, true>, bFwd(canDblFwd()));
            else optIn(k_dyn_fwd_b<T, false>, bFwd(canDblFwd()));
            return;
        }
        optIn(k_dyn_back<T>, smBack());
        optIn(k_dyn_fwd<T>, smFwd());
        optIn(k_lstar<T, 0>, smLstar());
        optIn(k_lstar<T, 1>, smLstar());
        optIn(k_lstar<T, 2>, smLstar());
        optIn(k_lop<T, 0>, smLop());
        optIn(k_lop<T, 1>, smLop());
        optIn(k_lop<T, 2>, smLop());
    }

    size_t smBack() const { return (size_t)(D_.ne * D_.nx + 2 * D_.nu) * D_.TB * sizeof(T); }
    size_t smFwd() const { return (size_t)(D_.nx + D_.nu) * D_.TB * sizeof(T); }
    size_t smLstar() const { return (size_t)D_.nd * D_.TB * sizeof(T); }
    size_t smLop() const { return (size_t)std::max(D_.dIV, D_.dVI) * D_.TB * sizeof(T); }

    void fill(T *p, size_t n, T v) {
        k_fill<T><<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream_>>>(p, n, v);
        CK(cudaGetLastError());
    }

    // Every tile live: before a solve's first round and before any launch outside a solve.
    void allLive() {
        const size_t tiles = (size_t)((B_ + 31) / 32);
        k_fill<int><<<(int)((tiles + 255) / 256), 256, 0, stream_>>>(S_.tileLive, tiles, 1);
        CK(cudaGetLastError());
    }

    void tileFlagsLaunch() {
        k_tile_flags<<<(int)((B_ + 255) / 256), 256, 0, stream_>>>(S_.status, (int)B_, S_.tileLive);
        CK(cudaGetLastError());
    }

    void copy(T *dst, const T *src, size_t n) {
        k_copy<T><<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, stream_>>>(dst, src, n);
        CK(cudaGetLastError());
    }

    // host slice [off, off+len) of instance 0 <-> device element-major buffer (B must be 1 for
    // exact placement; for B > 1 the slice is replicated into every instance)
    void uploadSlice(T *dst, const double *src, long off, long len) {
        std::vector<T> h((size_t)len * B_);
        for (long k = 0; k < len; k++)
            for (long b = 0; b < B_; b++) h[(size_t)k * B_ + b] = (T)src[k];
        CK(cudaMemcpyAsync(dst + (size_t)off * B_, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, stream_));
        CK(cudaStreamSynchronize(stream_));
    }

    void downloadSlice(const T *src, double *dst, long off, long len) {
        std::vector<T> h((size_t)len * B_);
        CK(cudaMemcpyAsync(h.data(), src + (size_t)off * B_, h.size() * sizeof(T), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        for (long k = 0; k < len; k++) dst[k] = (double)h[(size_t)k * B_];
    }

    OpArgs<T> blankArgs() const {
        OpArgs<T> A{};
        A.a1 = 1; A.a2 = 0; A.b1 = 1; A.b2 = 0; A.cL = 1;
        A.x0s = x0s_;
        A.live = S_.tileLive;
        return A;
    }

    // T evaluation: CAND = T(Z), and the residual R = Z - CAND of every entry as it is finalized
    OpArgs<T> tevalLstarArgs() const {  // p - gamma L* d, then prox (cache.cuh:748-764)
        OpArgs<T> A = blankArgs();
        A.in1 = Z_; A.base1 = Z_; A.cL = -P_.step; A.out = CAND_; A.outR = R_;
        return A;
    }
    OpArgs<T> tevalLopArgs() const {  // d + gamma L(2 pbar - p), then dual prox (cache.cuh:770-789)
        OpArgs<T> A = blankArgs();
        A.in1 = CAND_; A.a1 = 2; A.in2 = Z_; A.a2 = -1; A.base1 = Z_; A.cL = P_.step; A.out = CAND_; A.outR = R_;
        return A;
    }
    OpArgs<T> mLstarArgs() const {  // M r = r - gamma [L* r_d; L r_p], reading the residual R
        OpArgs<T> A = blankArgs();
        A.in1 = R_; A.base1 = R_; A.cL = -P_.step; A.out = MR_;
        return A;
    }
    OpArgs<T> mLopArgs() const {  // r_d - gamma L r_p
        OpArgs<T> A = mLstarArgs();
        return A;
    }

    dim3 nodeGrid(int nodes) const { return dim3((unsigned)((B_ + D_.TB - 1) / D_.TB), (unsigned)nodes); }

    dim3 tileGrid(int nodes) const { return dim3((unsigned)((B_ + kTileB - 1) / kTileB), (unsigned)nodes); }

    // L and L*: every node x groups of `tpc` instance tiles; the dynamics sweep: every node of a stage.
    dim3 opGridNodes(int tpc, int nodes) const {
        const long tiles = (gB() + kTileB - 1) / kTileB;
        return dim3((unsigned)((tiles + tpc - 1) / tpc), (unsigned)nodes);
    }
    dim3 opGrid(int tpc) const { return opGridNodes(tpc, D_.n); }

    // Autotuner of the tile shapes of L, L* and the dynamics sweep: instance tiles per CTA in
    // {1, 2, 4, 8}, double-buffered when more than one and the shared memory allows.  Each
    // candidate is timed (best of two trials of 5 launches of the T-form kernel, or of 5 whole
    // sweeps, with CUDA events on the solver stream); a larger shape replaces a smaller one only
    // when it is at least 5% faster.  Runs once, before the round is captured; it
    // writes only CAND, R and the sweep's workspaces, which every round rewrites first.
    void autotune() {
        if (!batched_ || tuned_) return;
        tuned_ = true;
        allLive();
        const int tiles = (int)((B_ + kTileB - 1) / kTileB);
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0));
        CK(cudaEventCreate(&e1));
        auto timeIt = [&](auto launch) {  // best of two trials of 5 launches after a warm-up
            launch();
            float best = 1e30f;
            for (int trial = 0; trial < 2; trial++) {
                CK(cudaEventRecord(e0, stream_));
                for (int r = 0; r < 5; r++) launch();
                CK(cudaEventRecord(e1, stream_));
                CK(cudaEventSynchronize(e1));
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, e0, e1));
                best = std::min(best, ms);
            }
            return best;
        };
        float bestS = 1e30f, bestL = 1e30f;
        int tS = 1, tL = 1;
        for (int tpc = 1; tpc <= kTilesPerCta && tpc <= tiles; tpc *= 2) {
            tpcLstar_ = tpcLop_ = tpc;
            lstarDbl_ = tpc > 1 && canDblLstar();
            lopDbl_ = tpc > 1 && canDblLop();
            const float ms = timeIt([&] { launchLstar<0>(tevalLstarArgs()); });
            if (ms < 0.95f * bestS) { bestS = ms; tS = tpc; }
            const float ml = timeIt([&] { launchLop<0>(tevalLopArgs()); });
            if (ml < 0.95f * bestL) { bestL = ml; tL = tpc; }
        }
        tpcLstar_ = tS;
        lstarDbl_ = tS > 1 && canDblLstar();
        tpcLop_ = tL;
        lopDbl_ = tL > 1 && canDblLop();
        float bestD = 1e30f;
        int tD = 1;
        for (int tpc = 1; tpc <= kTilesPerCta && tpc <= tiles; tpc *= 2) {  // the whole sweep, both directions
            tpcDyn_ = tpc;
            backDbl_ = tpc > 1 && canDblBack();
            fwdDbl_ = tpc > 1 && canDblFwd();
            const float md = timeIt([&] { dynamics(); });
            if (md < 0.95f * bestD) { bestD = md; tD = tpc; }
        }
        tpcDyn_ = tD;
        backDbl_ = tD > 1 && canDblBack();
        fwdDbl_ = tD > 1 && canDblFwd();
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }

    template <int MODE>
    void launchLstar(const OpArgs<T> &A) {
        if (batched_) {
            if (D_.gmat & kGmatLstar)
                launchLstarB<T, MODE, true>(opGrid(tpcLstar_), smLstarB(), stream_, P_, D_, A, M_, tpcLstar_, (int)lstarDbl_);
            else
                launchLstarB<T, MODE, false>(opGrid(tpcLstar_), smLstarB(), stream_, P_, D_, A, M_, tpcLstar_, (int)lstarDbl_);
            CK(cudaGetLastError());
            return;
        }
        k_lstar<T, MODE><<<nodeGrid(D_.n), kNodeThreads, smLstar(), stream_>>>(P_, D_, A);
        CK(cudaGetLastError());
    }

    template <int MODE>
    void launchLop(const OpArgs<T> &A) {
        if (batched_) {
            if (D_.gmat & kGmatLop)
                launchLopB<T, MODE, true>(opGrid(tpcLop_), smLopB(), stream_, P_, D_, A, M_, tpcLop_, (int)lopDbl_);
            else
                launchLopB<T, MODE, false>(opGrid(tpcLop_), smLopB(), stream_, P_, D_, A, M_, tpcLop_, (int)lopDbl_);
            CK(cudaGetLastError());
            return;
        }
        k_lop<T, MODE><<<nodeGrid(D_.n), kNodeThreads, smLop(), stream_>>>(P_, D_, A);
        CK(cudaGetLastError());
    }

    void dynamics() {
        const int N = D_.ns - 1;
        if (batched_) {
            const size_t smB = bBack(backDbl_), smF = bFwd(fwdDbl_);
            auto back = D_.gmat & kGmatBack ? k_dyn_back_b<T, true> : k_dyn_back_b<T, false>;
            auto fwd = D_.gmat & kGmatFwd ? k_dyn_fwd_b<T, true> : k_dyn_fwd_b<T, false>;
            for (int st = N - 1; st >= 0; st--) {
                back<<<opGridNodes(tpcDyn_, stageCount_[st]), kTileB * kTileWarps, smB, stream_>>>(
                    P_, D_, M_, CAND_, Q_, DD_, stageFrom_[st], st, tpcDyn_, (int)backDbl_, S_.tileLive);
                CK(cudaGetLastError());
            }
            for (int st = 0; st < N; st++) {
                fwd<<<opGridNodes(tpcDyn_, stageCount_[st]), kTileB * kTileWarps, smF, stream_>>>(
                    P_, D_, M_, CAND_, DD_, x0s_, stageFrom_[st], Z_, R_, tpcDyn_, (int)fwdDbl_, S_.tileLive);
                CK(cudaGetLastError());
            }
            return;
        }
        const size_t smB = smBack(), smF = smFwd();
        for (int st = N - 1; st >= 0; st--) {
            k_dyn_back<T><<<nodeGrid(stageCount_[st]), kNodeThreads, smB, stream_>>>(P_, D_, CAND_, Q_, DD_, stageFrom_[st], st);
            CK(cudaGetLastError());
        }
        for (int st = 0; st < N; st++) {
            k_dyn_fwd<T><<<nodeGrid(stageCount_[st]), kNodeThreads, smF, stream_>>>(P_, D_, CAND_, DD_, x0s_, stageFrom_[st],
                                                                                    Z_, R_);
            CK(cudaGetLastError());
        }
    }

    void teval() {
        launchLstar<0>(tevalLstarArgs());
        dynamics();
        launchLop<0>(tevalLopArgs());
    }

    void applyMres() {
        launchLstar<1>(mLstarArgs());
        launchLop<1>(mLopArgs());
    }

    void reduceLaunch(Algo algo, bool withData) {
        RedArgs<T> A{};
        A.R = R_; A.MR = MR_; A.D = DIR_; A.RPREV = RPREV_; A.ANDR = ANDR_;
        A.phase = S_.phase; A.status = S_.status; A.part = part_;
        A.m = (int)opt_.anderson; A.nv = nv_; A.chunks = chunks_; A.algo = algo; A.rowsPerChunk = rowsPerChunk_;
        if (!withData) {  // CP rounds between error checks: no reduction needed
            CK(cudaMemsetAsync(part_, 0, sizeof(double) * (size_t)chunks_ * nv_ * B_, stream_));
            return;
        }
        const int TB = B_ >= 32 ? 32 : (int)B_;
        const int lanes = kRedThreads / TB;
        const size_t sm = (size_t)nv_ * lanes * TB * sizeof(double);
        dim3 grid((unsigned)((gB() + TB - 1) / TB), (unsigned)chunks_);
        withAnderson([&](auto mc) { k_reduce<T, decltype(mc)::value><<<grid, kRedThreads, sm, stream_>>>(D_, A); });
        CK(cudaGetLastError());
    }

    void controlLaunch(Algo algo) {
        CtlArgs A{};
        A.S = S_; A.part = part_; A.chunks = chunks_; A.nv = nv_; A.m = (int)opt_.anderson; A.algo = algo;
        A.gamma = hp_.stepSize;
        const double ts = hp_.preconditioned ? hp_.minScaling() : 1.;  // cache.cuh:302-306
        A.tolAbs = opt_.tolAbs * ts;
        A.tolRel = opt_.tolRel * ts;
        A.maxOuter = opt_.maxOuter;
        A.maxInner = opt_.maxInner;
        A.ridge = sizeof(T) == 8 ? 1e-13 : 1e-7;
        k_control<<<((int)gB() + 3) / 4, 128, 0, stream_>>>((int)B_, A);  // 4 instances (warps) per block
        CK(cudaGetLastError());
    }

    void updateLaunch() {
        UpdArgs<T> A{};
        A.Z = Z_; A.CAND = CAND_; A.R = R_; A.PREV = PREV_; A.RPREV = RPREV_; A.BACKUP = BACKUP_; A.D = DIR_;
        A.ANDR = ANDR_; A.ANDZ = ANDZ_; A.action = S_.action; A.head = S_.head; A.useAnd = S_.useAnd;
        A.gamma = S_.gamma; A.tau = S_.tau; A.coef = S_.coef; A.m = (int)opt_.anderson;
        if (B_ < 32) {
            const size_t total = (size_t)D_.sZ * B_;
            const int grid = (int)std::min<size_t>((total + 255) / 256, 152 * 8);
            k_update_flat<T><<<grid, 256, 0, stream_>>>(D_, A);
            CK(cudaGetLastError());
            return;
        }
        // Blocks as wide as the slots the round covers, at most 256 (k_update takes its instance
        // from blockIdx.x * blockDim.x + threadIdx.x and its rows from blockIdx.y): after a
        // compaction to one tile, 256-wide blocks would leave 7 of 8 threads without an instance.
        // As many threads as about 8 blocks of 256 per SM.
        const long live = gB();
        const int tx = live >= 256 ? 256 : (int)((live + 31) / 32 * 32);
        const long bx = (live + tx - 1) / tx;
        const long blocks = 152L * 8 * 256 / tx;
        const long by = std::max<long>(1, std::min<long>((blocks + bx - 1) / bx, D_.sZ));
        withAnderson([&](auto mc) {
            k_update<T, decltype(mc)::value><<<dim3((unsigned)bx, (unsigned)by), tx, 0, stream_>>>(D_, A);
        });
        CK(cudaGetLastError());
    }

    // f(std::integral_constant<int, m>) for the solver's Anderson memory m (1 .. kMaxAnderson).
    template <typename F>
    void withAnderson(F f) const {
        switch (opt_.anderson) {
            case 1: f(std::integral_constant<int, 1>{}); break;
            case 2: f(std::integral_constant<int, 2>{}); break;
            case 3: f(std::integral_constant<int, 3>{}); break;
            case 4: f(std::integral_constant<int, 4>{}); break;
            case 5: f(std::integral_constant<int, 5>{}); break;
            case 6: f(std::integral_constant<int, 6>{}); break;
            case 7: f(std::integral_constant<int, 7>{}); break;
            default: f(std::integral_constant<int, 8>{}); break;
        }
    }

    void roundSpock() {
        teval();
        applyMres();
        reduceLaunch(kSpock, true);
        controlLaunch(kSpock);
        updateLaunch();
        tileFlagsLaunch();
    }

    // Instance compaction.  The node kernels skip tiles of 32 instances that have all stopped, but
    // a batch's slowest instances are spread over every tile.  When the running instances would
    // fill at most 3/4 of the slots still in live tiles (and free two tiles or more), they are moved
    // to the leading slots -- every buffer that carries state from round to round, the initial
    // states and the controller state -- so only ceil(active / 32) tiles stay live.  The captured
    // round reads the same buffers, which keep their addresses, and from then on the rounds run
    // with grids over the leading slots only (graphFor: one captured round per power-of-two count
    // of tiles), so stopped tiles cost no CTAs.  restoreOrder() puts every instance back in its
    // own slot when the solve ends.
    bool maybeCompact(int active) {
        if (!from_ || !batched_) return false;
        const long need = ((long)active + kTileB - 1) / kTileB * kTileB;
        if (4 * (long)active > 3 * capacity_ || capacity_ - need < 2 * kTileB) return false;
        std::vector<int> st((size_t)B_);
        CK(cudaMemcpyAsync(st.data(), S_.status, sizeof(int) * (size_t)B_, cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        std::vector<int> from;
        from.reserve((size_t)B_);
        for (long q = 0; q < B_; q++)
            if (st[(size_t)q] == -1) from.push_back((int)q);
        for (long q = 0; q < B_; q++)
            if (st[(size_t)q] != -1) from.push_back((int)q);
        permute(from);
        capacity_ = need;
        compactions_++;
        return true;
    }

    void restoreOrder() {
        bool ident = true;
        for (long q = 0; q < B_; q++) ident = ident && slotInst_[(size_t)q] == (int)q;
        if (ident) return;
        std::vector<int> from((size_t)B_);
        for (long q = 0; q < B_; q++) from[(size_t)slotInst_[(size_t)q]] = (int)q;  // instance q sits in slot ...
        permute(from);
    }

    // Slot s takes the instance in slot from[s], in every persistent buffer.
    void permute(const std::vector<int> &from) {
        CK(cudaMemcpyAsync(from_, from.data(), sizeof(int) * (size_t)B_, cudaMemcpyHostToDevice, stream_));
        auto gatherRows = [&](T *buf, long rows) {
            const dim3 grid((unsigned)((B_ + 255) / 256), (unsigned)std::min<long>(rows, 8192));
            k_gather_cols<T><<<grid, 256, 0, stream_>>>(W1_, buf, from_, rows, (int)B_);
            CK(cudaGetLastError());
            CK(cudaMemcpyAsync(buf, W1_, sizeof(T) * (size_t)rows * B_, cudaMemcpyDeviceToDevice, stream_));
        };
        const long nzr = D_.sZ;
        for (T *buf : {Z_, PREV_, RPREV_, BACKUP_, DIR_}) gatherRows(buf, nzr);
        for (long q = 0; q < opt_.anderson; q++) {
            gatherRows(ANDR_ + (size_t)q * nzr * B_, nzr);
            gatherRows(ANDZ_ + (size_t)q * nzr * B_, nzr);
        }
        gatherRows(x0s_, D_.nx);
        const int perG = kMaxAnderson * kMaxAnderson, perGamma = kMaxAnderson;
        k_gather_state<<<(int)((B_ + 255) / 256), 256, 0, stream_>>>(ibTmp_, ib_, dbTmp_, db_, from_, (int)B_, 16, 8, perG,
                                                                    perGamma);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(ib_, ibTmp_, sizeof(int) * (size_t)B_ * 16, cudaMemcpyDeviceToDevice, stream_));
        CK(cudaMemcpyAsync(db_, dbTmp_, sizeof(double) * (size_t)B_ * (8 + perG + perGamma), cudaMemcpyDeviceToDevice,
                           stream_));
        std::vector<int> inst((size_t)B_);
        for (long q = 0; q < B_; q++) inst[(size_t)q] = slotInst_[(size_t)from[(size_t)q]];
        slotInst_ = inst;
        tileFlagsLaunch();
        CK(cudaStreamSynchronize(stream_));
    }

    // Instances the round's grids cover: the whole batch, or (after an instance compaction) the
    // leading slots that can still hold running instances, rounded up to a power of two of tiles.
    long gB() const { return gridB_ > 0 ? gridB_ : B_; }
    long levelFor(long capacity) const {
        long tiles = 1;
        while (tiles * kTileB < capacity) tiles *= 2;
        return std::min<long>(B_, tiles * kTileB);
    }
    // The round for grids over the first `gridB` slots (captured once per level).
    cudaGraphExec_t graphFor(long gridB) {
        ensureGraph();
        if (gridB >= B_) return graph_;
        auto it = graphsLive_.find(gridB);
        if (it != graphsLive_.end()) return it->second;
        cudaGraph_t g;
        gridB_ = gridB;
        CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        roundSpock();
        CK(cudaStreamEndCapture(stream_, &g));
        gridB_ = 0;
        cudaGraphExec_t e;
        CK(cudaGraphInstantiate(&e, g, 0));
        CK(cudaGraphDestroy(g));
        graphsLive_[gridB] = e;
        return e;
    }
    void dropGraphs() {
        if (graph_) CK(cudaGraphExecDestroy(graph_));
        graph_ = nullptr;
        for (auto &kv : graphsLive_) CK(cudaGraphExecDestroy(kv.second));
        graphsLive_.clear();
    }

    // The round captured once as a CUDA graph; the template stays, so that a group of solvers
    // can run their rounds as one graph (spock_solve_group).
    void ensureGraph() {
        if (graph_) return;
        autotune();
        if (graphTemplate_) {
            CK(cudaGraphDestroy(graphTemplate_));
            graphTemplate_ = nullptr;
        }
        CK(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        roundSpock();
        CK(cudaStreamEndCapture(stream_, &graphTemplate_));
        CK(cudaGraphInstantiate(&graph_, graphTemplate_, 0));
    }

    // FP64 finish.  The instances still running (at most one tile of 32) move with their whole
    // SuperMann state -- iterate, previous iterate and residual, backup, direction, Anderson
    // memory, initial state and controller state -- into an FP64 solver of the same problem
    // (batch 32, made on first use), which continues the same iteration in FP64 until they
    // stop; their final iterates and controller state (status, counters) come back converted.
    // Only the arithmetic of the remaining iterations changes: an FP32 instance that stalls near
    // the tolerance on float rounding finishes in the FP64 number of iterations.
    // Returns false, and turns the finish off, when this problem has no FP64 batched kernels (its
    // node data exceed their shared memory): the solve then continues in FP32.
    bool finishInDouble(std::chrono::steady_clock::time_point t0, long &rounds, long &launches) {
        if constexpr (sizeof(T) == 4) {
            std::vector<int> st((size_t)B_);
            CK(cudaMemcpyAsync(st.data(), S_.status, sizeof(int) * (size_t)B_, cudaMemcpyDeviceToHost, stream_));
            CK(cudaStreamSynchronize(stream_));
            std::vector<int> idx;  // [0, count): twin slots; [kTileB, kTileB + count): this solver's slots
            for (long q = 0; q < B_ && (long)idx.size() < kTileB; q++)
                if (st[(size_t)q] == -1) idx.push_back((int)q);
            const int count = (int)idx.size();
            if (count == 0) return false;
            if (!twin_) {  // made, tuned and captured before any state moves in
                try {
                    twin_.reset(new Engine<double>(hp_, opt_, kTileB, device_));
                } catch (const std::invalid_argument &) {
                    finishAfter_ = 0;
                    return false;
                }
                twinIdx_ = dalloc<int>(2 * kTileB);
                twin_->ensureGraph();
                CK(cudaStreamSynchronize(twin_->stream_));
            }
            Engine<double> &tw = *twin_;
            std::vector<int> both(2 * kTileB, 0);
            for (int s = 0; s < count; s++) {
                both[(size_t)s] = s;
                both[(size_t)(kTileB + s)] = idx[(size_t)s];
            }
            CK(cudaMemcpyAsync(twinIdx_, both.data(), sizeof(int) * both.size(), cudaMemcpyHostToDevice, stream_));
            const int *dTw = twinIdx_, *dMe = twinIdx_ + kTileB;
            const long nzr = D_.sZ;
            auto toTwin = [&](double *dst, const T *src, long rows) {
                const int grid = (int)std::min<long>((rows + 7) / 8, 152 * 8);
                k_move_cols<double, T><<<grid, 256, 0, stream_>>>(dst, tw.B_, src, B_, dTw, dMe, count, rows);
                CK(cudaGetLastError());
            };
            toTwin(tw.Z_, Z_, nzr);
            toTwin(tw.PREV_, PREV_, nzr);
            toTwin(tw.RPREV_, RPREV_, nzr);
            toTwin(tw.BACKUP_, BACKUP_, nzr);
            toTwin(tw.DIR_, DIR_, nzr);
            for (long q = 0; q < opt_.anderson; q++) {
                toTwin(tw.ANDR_ + (size_t)q * nzr * tw.B_, ANDR_ + (size_t)q * nzr * B_, nzr);
                toTwin(tw.ANDZ_ + (size_t)q * nzr * tw.B_, ANDZ_ + (size_t)q * nzr * B_, nzr);
            }
            toTwin(tw.x0s_, x0s_, D_.nx);
            const int perG = kMaxAnderson * kMaxAnderson, perGamma = kMaxAnderson;
            k_move_state<<<1, kTileB, 0, stream_>>>(tw.ib_, tw.B_, ib_, B_, tw.db_, db_, dTw, dMe, count, 16, 8, perG,
                                                   perGamma);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(stream_));
            k_stop_from<<<1, kTileB, 0, tw.stream_>>>(tw.S_.status, count, (int)tw.B_);
            CK(cudaGetLastError());
            CK(cudaMemsetAsync(tw.S_.timeUp, 0, sizeof(int), tw.stream_));
            tw.continueSolve(t0, rounds, launches);
            // back: the final iterates and the controller state
            const int grid = (int)std::min<long>((nzr + 7) / 8, 152 * 8);
            k_move_cols<T, double><<<grid, 256, 0, stream_>>>(Z_, B_, tw.Z_, tw.B_, dMe, dTw, count, nzr);
            CK(cudaGetLastError());
            k_move_state<<<1, kTileB, 0, stream_>>>(ib_, B_, tw.ib_, tw.B_, db_, tw.db_, dMe, dTw, count, 16, 8, perG,
                                                   perGamma);
            CK(cudaGetLastError());
            CK(cudaStreamSynchronize(stream_));
            launches += 2 * (7 + 2 * opt_.anderson) + 4;
            return true;
        }
        return false;
    }

    // Run rounds on the state already in place (no re-initialisation) until every instance stops.
    void continueSolve(std::chrono::steady_clock::time_point t0, long &rounds, long &launches) {
        allLive();
        capacity_ = B_;
        cudaGraphExec_t round = graphFor(B_);
        for (;;) {
            CK(cudaGraphLaunch(round, stream_));
            rounds++;
            launches += launchesPerRound();
            if (rounds % 10 == 0 && activeCount(t0) == 0) break;
        }
        CK(cudaStreamSynchronize(stream_));
    }

    int activeCount(std::chrono::steady_clock::time_point t0) {
        if (opt_.maxTimeSecs > 0) {
            const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            if (el >= opt_.maxTimeSecs) {
                const int one = 1;
                CK(cudaMemcpyAsync(S_.timeUp, &one, sizeof(int), cudaMemcpyHostToDevice, stream_));
            }
        }
        k_count_active<<<1, 256, 0, stream_>>>(S_.status, (int)B_, devActive_);
        CK(cudaGetLastError());
        CK(cudaMemcpyAsync(hostActive_, devActive_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
        CK(cudaStreamSynchronize(stream_));
        return *hostActive_;
    }
};

EngineBase *makeEngine(const HostProblem &hp, const Options &opt, long batch, int precisionBits, int device) {
    if (precisionBits == 64) return new Engine<double>(hp, opt, batch, device);
    if (precisionBits == 32) return new Engine<float>(hp, opt, batch, device);
    throw std::invalid_argument("[Cache] precision must be 32 or 64");
}

}  // namespace spock
