// Per-iteration kernels of the SPOCK solve (sm_103a).  See engine.cuh for the memory layout.
//
// One Chambolle-Pock step T (src/cache.cuh:748-801) is 2N+2 launches:
//   k_lstar<0>  : p - gamma L*(d), root s prox, AVaR kernel projection  (cache.cuh:748-764, 650-676)
//   k_dyn_back  : one launch per stage N-1..0, backward Riccati-like sweep (dynamics.cuh:85-139)
//   k_dyn_fwd   : one launch per stage 0..N-1, forward rollout             (dynamics.cuh:143-173)
//   k_lop<0>    : d + gamma L(2 pbar - p), translate, project, Moreau      (cache.cuh:770-789, 678-698)
// The M operator M r = r - gamma [L* r_d; L r_p] (cache.cuh:721-742) reuses the same two
// operator kernels in mode 1, and modes 2 are the bare L / L* used by the tests.
// Every kernel works on one tree node per CTA row (blockIdx.y) and TB instances per CTA
// (blockIdx.x); threads split into TB instance lanes x RG row groups.
#pragma once

#include "engine.cuh"

namespace spock {

constexpr int kNodeThreads = 128;
constexpr int kRedThreads = 256;

__device__ __forceinline__ size_t ix(long k, int B, int b) { return (size_t)k * (size_t)B + (size_t)b; }

// ------------------------------------------------------------------------------------------
// L* (adjoint) with optional primal prox (MODE 0), residual/M form (MODE 1) or bare (MODE 2).
// ------------------------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void __launch_bounds__(kNodeThreads) k_lstar(const DevProblem<T> P, const Dims D, const OpArgs<T> A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sv = reinterpret_cast<T *>(smraw);
    const int TB = D.TB, B = D.B;
    const int lb = threadIdx.x % TB, rg = threadIdx.x / TB, RG = kNodeThreads / TB;
    const bool laneOk = rg < RG;
    const int b = blockIdx.x * TB + lb;
    const bool act = laneOk && b < B;
    const int i = blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu;

    auto IN = [&](long k) -> T {
        T v = A.a1 * A.in1[ix(k, B, b)];
        if (A.in2) v += A.a2 * A.in2[ix(k, B, b)];
        return v;
    };
    auto BASE = [&](long k) -> T {
        T v = 0;
        if (A.base1) v = A.b1 * A.base1[ix(k, B, b)];
        if (A.base2) v += A.b2 * A.base2[ix(k, B, b)];
        return v;
    };
    auto EMIT = [&](long k, T lv) {
        const T bs = BASE(k);
        if (A.outBase) A.outBase[ix(k, B, b)] = bs;
        A.out[ix(k, B, b)] = bs + A.cL * lv;
    };

    if (i < D.nnl) {
        const int c0 = P.chFrom[i], nc = P.numCh[i];
        if (act) {
            for (int r = rg; r < nxu; r += RG) {
                T acc = 0;
                if (D.conNl == kConRectangle) acc = IN(D.oIII + (long)i * nxu + r);
                for (int j = c0; j < c0 + nc; j++) {
                    const long ivo = D.oIV + (long)j * D.dIV;
                    if (r < nx) {
                        const T *M = P.sqrtQ + (size_t)j * nx * nx + r;
                        for (int c = 0; c < nx; c++) acc += M[(size_t)c * nx] * IN(ivo + c);
                        if (D.costNl == kCostQuadraticPlusLinear)
                            acc -= T(0.5) * P.q[(size_t)j * nx + r] * (IN(ivo + nxu) + IN(ivo + nxu + 1));
                    } else {
                        const int rr = r - nx;
                        const T *M = P.sqrtR + (size_t)j * nu * nu + rr;
                        for (int c = 0; c < nu; c++) acc += M[(size_t)c * nu] * IN(ivo + nx + c);
                        if (D.costNl == kCostQuadraticPlusLinear)
                            acc -= T(0.5) * P.r[(size_t)j * nu + rr] * (IN(ivo + nxu) + IN(ivo + nxu + 1));
                    }
                }
                EMIT(r < nx ? D.oX + (long)i * nx + r : (long)i * nu + (r - nx), acc);
            }
        }
        // y_i and the (t, s) of the children: gathered as one vector of the AVaR kernel
        // projection (padded to 4E+1, cache.cuh:655-663)
        auto entry = [&](int k, long &outk) -> T {
            outk = -1;
            if (k < D.yD) {
                outk = D.oY + (long)i * D.yD + k;
                return IN(D.oI + (long)i * D.yD + k) - P.b[(size_t)i * D.yD + k] * IN(D.oII + i);
            }
            if (k < D.yD + D.ne) {
                const int jj = k - D.yD;
                if (jj >= nc) return T(0);
                const int j = c0 + jj;
                outk = D.oT + j;
                const long ivo = D.oIV + (long)j * D.dIV;
                return T(0.5) * (IN(ivo + nxu) + IN(ivo + nxu + 1));
            }
            const int jj = k - D.yD - D.ne;
            if (jj >= nc) return T(0);
            const int j = c0 + jj;
            outk = D.oS + j;
            if (j < D.nnl) return IN(D.oII + j);
            const long vio = D.oVI + (long)(j - D.nnl) * D.dVI;
            return T(0.5) * (IN(vio + nx) + IN(vio + nx + 1));
        };
        if (MODE == 0) {
            if (laneOk)
                for (int k = rg; k < D.nd; k += RG) {
                    long outk = -1;
                    T lv = act ? entry(k, outk) : T(0);
                    sv[k * TB + lb] = (act && outk >= 0) ? BASE(outk) + A.cL * lv : T(0);
                }
            __syncthreads();
            if (act) {
                const T *N = P.NNtr + (size_t)i * D.nd * D.nd;
                for (int k = rg; k < D.nd; k += RG) {
                    long outk = -1;
                    (void)entry(k, outk);
                    if (outk < 0) continue;
                    T acc = 0;
                    for (int c = 0; c < D.nd; c++) acc += N[(size_t)c * D.nd + k] * sv[c * TB + lb];
                    A.out[ix(outk, B, b)] = acc;
                    if (A.outR) A.outR[ix(outk, B, b)] = BASE(outk) - acc;
                }
            }
        } else if (act) {
            for (int k = rg; k < D.nd; k += RG) {
                long outk = -1;
                T lv = entry(k, outk);
                if (outk >= 0) EMIT(outk, lv);
            }
        }
    } else if (act) {
        const int l = i - D.nnl;
        const long vio = D.oVI + (long)l * D.dVI;
        for (int r = rg; r < nx; r += RG) {
            T acc = (D.conL == kConRectangle) ? IN(D.oV + (long)l * nx + r) : T(0);
            const T *M = P.lSqrtQ + r;
            for (int c = 0; c < nx; c++) acc += M[(size_t)c * nx] * IN(vio + c);
            if (D.costL == kCostQuadraticPlusLinear) acc -= T(0.5) * P.lq[r] * (IN(vio + nx) + IN(vio + nx + 1));
            EMIT(D.oX + (long)i * nx + r, acc);
        }
    }
    if (i == 0 && act && rg == 0) {
        EMIT(D.oT, T(0));  // t_0 carries no cost term
        const T lv = IN(D.oII);
        if (MODE == 0) {
            const T s0 = BASE(D.oS) + A.cL * lv - P.step;  // prox of s_0 (cache.cuh:638-642)
            A.out[ix(D.oS, B, b)] = s0;
            if (A.outR) {
                A.outR[ix(D.oS, B, b)] = BASE(D.oS) - s0;
                A.outR[ix(D.oT, B, b)] = T(0);
            }
        } else EMIT(D.oS, lv);
    }
}

// ------------------------------------------------------------------------------------------
// Dynamics projection, backward sweep for one stage (dynamics.cuh:85-139).
// Reads pbar x, u from CAND; writes d (DD) and, above stage 0, q (Q).
// ------------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kNodeThreads) k_dyn_back(const DevProblem<T> P, const Dims D, const T *__restrict__ cand,
                                                          T *__restrict__ Q, T *__restrict__ DD, int stageFrom, int stage) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = reinterpret_cast<T *>(smraw);
    const int TB = D.TB, B = D.B;
    const int lb = threadIdx.x % TB, rg = threadIdx.x / TB, RG = kNodeThreads / TB;
    const bool laneOk = rg < RG;
    const int b = blockIdx.x * TB + lb;
    const bool act = laneOk && b < B;
    const int i = stageFrom + blockIdx.y;
    const int nx = D.nx, nu = D.nu;
    const int c0 = P.chFrom[i], nc = P.numCh[i];
    T *sq = sm;                       // [nc][nx][TB]
    T *sd = sq + D.ne * nx * TB;      // [nu][TB]
    T *su = sd + nu * TB;             // [nu][TB]
    if (act) {
        for (int t = rg; t < nc * nx; t += RG) {
            const int jj = t / nx, c = t % nx, j = c0 + jj;
            T v = (j >= D.nnl) ? -cand[ix(D.oX + (long)j * nx + c, B, b)] : Q[ix((long)j * nx + c, B, b)];
            if (D.affine) v += P.Pe[(size_t)j * nx + c];
            sq[t * TB + lb] = v;
        }
        for (int c = rg; c < nu; c += RG) su[c * TB + lb] = cand[ix((long)i * nu + c, B, b)];
    }
    __syncthreads();
    if (act)
        for (int r = rg; r < nu; r += RG) {
            T acc = su[r * TB + lb];
            for (int jj = 0; jj < nc; jj++) {
                const T *M = P.BTr + (size_t)(c0 + jj) * nu * nx + r;
                const T *qv = sq + jj * nx * TB + lb;
                for (int c = 0; c < nx; c++) acc -= M[(size_t)c * nu] * qv[c * TB];
            }
            sd[r * TB + lb] = acc;
        }
    __syncthreads();
    if (act && rg == 0) {  // (I + sum B'PB) d = rhs with the cached lower Cholesky factor
        const T *L = P.chol + (size_t)i * nu * nu;
        T *v = sd + lb;
        for (int r = 0; r < nu; r++) {
            T acc = v[r * TB];
            for (int k = 0; k < r; k++) acc -= L[(size_t)k * nu + r] * v[k * TB];
            v[r * TB] = acc / L[(size_t)r * nu + r];
        }
        for (int r = nu - 1; r >= 0; r--) {
            T acc = v[r * TB];
            for (int k = r + 1; k < nu; k++) acc -= L[(size_t)r * nu + k] * v[k * TB];
            v[r * TB] = acc / L[(size_t)r * nu + r];
        }
    }
    __syncthreads();
    if (!act) return;
    for (int r = rg; r < nu; r += RG) DD[ix((long)i * nu + r, B, b)] = sd[r * TB + lb];
    if (stage == 0) return;
    for (int r = rg; r < nx; r += RG) {
        T acc = -cand[ix(D.oX + (long)i * nx + r, B, b)];
        for (int jj = 0; jj < nc; jj++) {
            const int j = c0 + jj;
            const T *M1 = P.APB + (size_t)j * nx * nu + r;
            for (int c = 0; c < nu; c++) acc += M1[(size_t)c * nx] * sd[c * TB + lb];
            const T *M2 = P.ABKTr + (size_t)j * nx * nx + r;
            const T *qv = sq + jj * nx * TB + lb;
            for (int c = 0; c < nx; c++) acc += M2[(size_t)c * nx] * qv[c * TB];
        }
        const T *Kt = P.K + (size_t)i * nu * nx + (size_t)r * nu;  // column r of K = row r of K'
        for (int c = 0; c < nu; c++) acc += Kt[c] * (sd[c * TB + lb] - su[c * TB + lb]);
        Q[ix((long)i * nx + r, B, b)] = acc;
    }
}

// Row r of a column-major matrix (column stride ld) times [v1 (n1 values); v2 (n2 values)]
// (vector entries `vs` apart), plus d.  FP64: plain accumulation starting from d.  FP32: Dot2
// (Ogita, Rump and Oishi, SIAM J. Sci. Comput. 26, 2005), with every product's exact error from
// an FMA and every sum's from Knuth's TwoSum, for the reasons given at k_dyn_fwd_b.
__device__ __forceinline__ double rolloutDot(const double *M, int ld, const double *v1, int vs, int n1, const double *v2,
                                             int n2, double d) {
    double acc = d;
    for (int c = 0; c < n1; c++) acc += M[(size_t)c * ld] * v1[c * vs];
    for (int c = 0; c < n2; c++) acc += M[(size_t)(n1 + c) * ld] * v2[c * vs];
    return acc;
}
__device__ __forceinline__ void twoSumAcc(float &s, float &cmp, float m, float v) {
    const float h = __fmul_rn(m, v), pe = __fmaf_rn(m, v, -h);
    const float t = __fadd_rn(s, h), z = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, z)), __fsub_rn(h, z));
    cmp = __fadd_rn(cmp, __fadd_rn(e, pe));
    s = t;
}
__device__ __forceinline__ float rolloutDot(const float *M, int ld, const float *v1, int vs, int n1, const float *v2, int n2,
                                            float d) {
    float s = 0.f, cmp = 0.f;
    for (int c = 0; c < n1; c++) twoSumAcc(s, cmp, M[(size_t)c * ld], v1[c * vs]);
    for (int c = 0; c < n2; c++) twoSumAcc(s, cmp, M[(size_t)(n1 + c) * ld], v2[c * vs]);
    const float h = __fadd_rn(s, d), z = __fsub_rn(h, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(h, z)), __fsub_rn(d, z));
    return __fadd_rn(h, __fadd_rn(e, cmp));
}

// ------------------------------------------------------------------------------------------
// Dynamics projection, forward rollout for one stage (dynamics.cuh:143-173), compensated in
// FP32 (rolloutDot).
// ------------------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kNodeThreads) k_dyn_fwd(const DevProblem<T> P, const Dims D, T *__restrict__ cand,
                                                         const T *__restrict__ DD, const T *__restrict__ x0s, int stageFrom,
                                                         const T *__restrict__ Z, T *__restrict__ R) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sx = reinterpret_cast<T *>(smraw);  // [nx][TB]
    const int TB = D.TB, B = D.B;
    const int lb = threadIdx.x % TB, rg = threadIdx.x / TB, RG = kNodeThreads / TB;
    const bool laneOk = rg < RG;
    const int b = blockIdx.x * TB + lb;
    const bool act = laneOk && b < B;
    const int i = stageFrom + blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu;
    T *su = sx + nx * TB;  // [nu][TB]
    if (act)
        for (int c = rg; c < nx; c += RG) {
            T v;
            if (i == 0) {
                v = x0s[ix(c, B, b)];
                cand[ix(D.oX + c, B, b)] = v;
                if (R) R[ix(D.oX + c, B, b)] = Z[ix(D.oX + c, B, b)] - v;
            } else {
                v = cand[ix(D.oX + (long)i * nx + c, B, b)];
            }
            sx[c * TB + lb] = v;
        }
    __syncthreads();
    if (act)
        for (int r = rg; r < nu; r += RG) {
            const T acc = rolloutDot(P.K + (size_t)i * nu * nx + r, nu, sx + lb, TB, nx, nullptr, 0,
                                     DD[ix((long)i * nu + r, B, b)]);
            su[r * TB + lb] = acc;
            cand[ix((long)i * nu + r, B, b)] = acc;
            if (R) R[ix((long)i * nu + r, B, b)] = Z[ix((long)i * nu + r, B, b)] - acc;
        }
    __syncthreads();
    if (!act) return;
    const int c0 = P.chFrom[i], nc = P.numCh[i];
    for (int t = rg; t < nc * nx; t += RG) {
        const int jj = t / nx, r = t % nx, j = c0 + jj;
        const T *M = P.AB + (size_t)j * nx * nxu + r;
        const T acc = rolloutDot(M, nx, sx + lb, TB, nx, su + lb, nu, D.affine ? P.e[(size_t)j * nx + r] : T(0));
        cand[ix(D.oX + (long)j * nx + r, B, b)] = acc;
        if (R) R[ix(D.oX + (long)j * nx + r, B, b)] = Z[ix(D.oX + (long)j * nx + r, B, b)] - acc;
    }
}

// Box clamp with the exact arithmetic of k_projectRectangle (definitions.cu:38-48).
template <typename T>
__device__ __forceinline__ T boxProject(T v, T lo, T hi) {
    const int lower = v <= lo, upper = v >= hi;
    const T lbi = isinf(lo) ? T(0) : lower * lo;
    const T ubi = isinf(hi) ? T(0) : upper * hi;
    return v * (1 - lower) * (1 - upper) + lbi + ubi;
}

// ------------------------------------------------------------------------------------------
// L with optional dual prox (MODE 0), residual/M form (MODE 1) or bare (MODE 2).
// ------------------------------------------------------------------------------------------
template <typename T, int MODE>
__global__ void __launch_bounds__(kNodeThreads) k_lop(const DevProblem<T> P, const Dims D, const OpArgs<T> A) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sw = reinterpret_cast<T *>(smraw);  // [block][TB]
    __shared__ T sScale[32], sNrm[32];
    __shared__ int sCase[32];
    const int TB = D.TB, B = D.B;
    const int lb = threadIdx.x % TB, rg = threadIdx.x / TB, RG = kNodeThreads / TB;
    const bool laneOk = rg < RG;
    const int b = blockIdx.x * TB + lb;
    const bool act = laneOk && b < B;
    const int j = blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu;
    const T g = P.step, gi = T(1) / P.step;

    auto INP = [&](long k) -> T {
        T v = A.a1 * A.in1[ix(k, B, b)];
        if (A.in2) v += A.a2 * A.in2[ix(k, B, b)];
        return v;
    };
    auto BASE = [&](long k) -> T {
        T v = 0;
        if (A.base1) v = A.b1 * A.base1[ix(k, B, b)];
        if (A.base2) v += A.b2 * A.base2[ix(k, B, b)];
        return v;
    };
    auto EMIT = [&](long k, T lv) {
        const T bs = BASE(k);
        if (A.outBase) A.outBase[ix(k, B, b)] = bs;
        A.out[ix(k, B, b)] = bs + A.cL * lv;
    };
    // MODE 0: v = (d + gamma L.)/gamma (+ translation); cand = gamma (v - proj_C(v))  (cache.cuh:782-789)
    auto FIN = [&](long k, T val) {
        A.out[ix(k, B, b)] = val;
        if (A.outR) A.outR[ix(k, B, b)] = BASE(k) - val;
    };

    if (j < D.nnl) {
        if (act) {
            const int nm = 2 * P.numCh[j];
            for (int k = rg; k < D.yD; k += RG) {
                const long o = D.oI + (long)j * D.yD + k;
                const T lv = INP(D.oY + (long)j * D.yD + k);
                if (MODE == 0) {
                    const T v = (BASE(o) + A.cL * lv) * gi;
                    const T pr = (k < nm && v < T(0)) ? T(0) * v : v;  // AVaR dual cone (risks.cuh:99-106)
                    FIN(o, (v - pr) * g);
                } else EMIT(o, lv);
            }
            if (rg == 0) {
                T lv = INP(D.oS + j);
                for (int k = 0; k < D.yD; k++) lv -= P.b[(size_t)j * D.yD + k] * INP(D.oY + (long)j * D.yD + k);
                const long o = D.oII + j;
                if (MODE == 0) {
                    const T v = (BASE(o) + A.cL * lv) * gi;
                    FIN(o, (v - (v > T(0) ? v : T(0))) * g);  // nonnegative orthant
                } else EMIT(o, lv);
            }
            if (D.conNl == kConRectangle)
                for (int k = rg; k < nxu; k += RG) {
                    const long o = D.oIII + (long)j * nxu + k;
                    const T lv = k < nx ? INP(D.oX + (long)j * nx + k) : INP((long)j * nu + (k - nx));
                    if (MODE == 0) {
                        const T v = (BASE(o) + A.cL * lv) * gi;
                        const T pr = boxProject(v, P.nlLo[(size_t)j * nxu + k], P.nlHi[(size_t)j * nxu + k]);
                        FIN(o, (v - pr) * g);
                    } else EMIT(o, lv);
                }
        }
    }
    // IV: cost epigraph of node j, reading the ancestor's (x, u) (costs.cuh:126-161, 379-417)
    {
        const int dIV = D.dIV;
        const long ivo = D.oIV + (long)j * dIV;
        const int a = j > 0 ? P.anc[j] : 0;
        auto lvIV = [&](int c) -> T {
            if (j == 0) return T(0);
            if (c < nx) {
                const T *M = P.sqrtQ + (size_t)j * nx * nx + c;
                T acc = 0;
                for (int cc = 0; cc < nx; cc++) acc += M[(size_t)cc * nx] * INP(D.oX + (long)a * nx + cc);
                return acc;
            }
            if (c < nxu) {
                const int rr = c - nx;
                const T *M = P.sqrtR + (size_t)j * nu * nu + rr;
                T acc = 0;
                for (int cc = 0; cc < nu; cc++) acc += M[(size_t)cc * nu] * INP((long)a * nu + cc);
                return acc;
            }
            T h = T(0.5) * INP(D.oT + j);
            if (D.costNl == kCostQuadraticPlusLinear) {
                T lin = 0;
                for (int cc = 0; cc < nx; cc++) lin += P.q[(size_t)j * nx + cc] * INP(D.oX + (long)a * nx + cc);
                for (int cc = 0; cc < nu; cc++) lin += P.r[(size_t)j * nu + cc] * INP((long)a * nu + cc);
                h -= T(0.5) * lin;
            }
            return h;
        };
        if (MODE == 0) {
            if (act)
                for (int c = rg; c < dIV; c += RG)
                    sw[c * TB + lb] = (BASE(ivo + c) + A.cL * lvIV(c)) * gi + P.trans[(size_t)j * dIV + c];
            __syncthreads();
            if (act && rg == 0) {
                T ss = 0;
                for (int c = 0; c < dIV - 1; c++) ss += sw[c * TB + lb] * sw[c * TB + lb];
                const T nrm = sqrt(ss), tt = sw[(dIV - 1) * TB + lb];
                const int i1 = nrm <= tt, i2 = (nrm <= -tt) && !i1, i3 = !i1 && !i2;
                sScale[lb] = (nrm + tt) / (T(2) * nrm + T(1 - i3));
                sNrm[lb] = nrm;
                sCase[lb] = i1 ? 1 : (i2 ? 2 : 3);
            }
            __syncthreads();
            if (act)
                for (int c = rg; c < dIV; c += RG) {
                    const T v = sw[c * TB + lb];
                    const int cs = sCase[lb];
                    const T pr = cs == 1 ? v : (cs == 2 ? T(0) : (c < dIV - 1 ? sScale[lb] * v : sScale[lb] * sNrm[lb]));
                    FIN(ivo + c, (v - pr) * g);
                }
        } else if (act) {
            for (int c = rg; c < dIV; c += RG) EMIT(ivo + c, lvIV(c));
        }
    }
    if (j >= D.nnl) {
        const int l = j - D.nnl;
        if (D.conL == kConRectangle && act)
            for (int k = rg; k < nx; k += RG) {
                const long o = D.oV + (long)l * nx + k;
                const T lv = INP(D.oX + (long)j * nx + k);
                if (MODE == 0) {
                    const T v = (BASE(o) + A.cL * lv) * gi;
                    const T pr = boxProject(v, P.lLo[(size_t)l * nx + k], P.lHi[(size_t)l * nx + k]);
                    FIN(o, (v - pr) * g);
                } else EMIT(o, lv);
            }
        const int dVI = D.dVI;
        const long vio = D.oVI + (long)l * dVI;
        auto lvVI = [&](int c) -> T {
            if (c < nx) {
                const T *M = P.lSqrtQ + c;
                T acc = 0;
                for (int cc = 0; cc < nx; cc++) acc += M[(size_t)cc * nx] * INP(D.oX + (long)j * nx + cc);
                return acc;
            }
            T h = T(0.5) * INP(D.oS + j);
            if (D.costL == kCostQuadraticPlusLinear) {
                T lin = 0;
                for (int cc = 0; cc < nx; cc++) lin += P.lq[cc] * INP(D.oX + (long)j * nx + cc);
                h -= T(0.5) * lin;
            }
            return h;
        };
        if (MODE == 0) {
            __syncthreads();
            if (act)
                for (int c = rg; c < dVI; c += RG) sw[c * TB + lb] = (BASE(vio + c) + A.cL * lvVI(c)) * gi + P.lTrans[c];
            __syncthreads();
            if (act && rg == 0) {
                T ss = 0;
                for (int c = 0; c < dVI - 1; c++) ss += sw[c * TB + lb] * sw[c * TB + lb];
                const T nrm = sqrt(ss), tt = sw[(dVI - 1) * TB + lb];
                const int i1 = nrm <= tt, i2 = (nrm <= -tt) && !i1, i3 = !i1 && !i2;
                sScale[lb] = (nrm + tt) / (T(2) * nrm + T(1 - i3));
                sNrm[lb] = nrm;
                sCase[lb] = i1 ? 1 : (i2 ? 2 : 3);
            }
            __syncthreads();
            if (act)
                for (int c = rg; c < dVI; c += RG) {
                    const T v = sw[c * TB + lb];
                    const int cs = sCase[lb];
                    const T pr = cs == 1 ? v : (cs == 2 ? T(0) : (c < dVI - 1 ? sScale[lb] * v : sScale[lb] * sNrm[lb]));
                    FIN(vio + c, (v - pr) * g);
                }
        } else if (act) {
            for (int c = rg; c < dVI; c += RG) EMIT(vio + c, lvVI(c));
        }
    }
}

}  // namespace spock
