// Node kernels for batches of >= 32 instances (sm_103a, FP32 or FP64).
//
// Same mathematics as kernels.cuh (which serves small batches and the single-instance solve),
// mapped for throughput.  A CTA owns one tree node and a tile of 32 instances, one per lane:
//  1. gather: every input row and every base row the CTA needs (for a row k, the 32
//     instances k*B + b0 .. b0+31 are one 128-byte coalesced segment) is copied into shared
//     memory with cp.async, all issued before the first wait, so hundreds of loads are in
//     flight per SM;
//     The node's matrices, kept on the device with the leading dimension padded to a
//     multiple of 16 rows, are copied to shared memory in the same asynchronous batch;
//  2. compute: each warp accumulates blocks of 16 output rows in registers (16 FMAs per
//     shared-memory input read, matrix columns read as warp-uniform 16-byte loads);
//  3. write: outputs (and, in a T evaluation, the residual Z - T(Z)) go out as coalesced rows.
// Nothing in steps 2-3 reads global memory through a pointer that a store could alias.
#pragma once

#include "kernels.cuh"

namespace spock {

constexpr int kTileB = 32;     // instances per CTA (one per lane)
constexpr int kTileWarps = 8;  // warps per CTA
constexpr int kRT = 16;        // output rows per register block
constexpr int kMaxTasks = 2;   // register blocks per warp: rows <= 16 * 8 * 2 = 256
// Dims::gmat bits: the kernel reads its node matrices in place (global memory, through L1/L2)
// instead of staging them in shared memory, for problems whose matrices exceed it.
constexpr int kGmatLstar = 1, kGmatLop = 2, kGmatBack = 4, kGmatFwd = 8;

__host__ __device__ inline int pad16(int r) { return (r + 15) & ~15; }

// L and L* keep two CTAs on an SM in FP32 (their shared memory allows it, so registers are capped
// at 128); in FP64 the shared memory of one CTA already fills the SM.
template <typename T>
constexpr int kOpCtasPerSm = sizeof(T) == 4 ? 2 : 1;

// Register blocks of a matrix with `rows` rows, and the slot a warp takes in a matrix whose
// blocks are dealt out starting at warp `first` (so two matrices accumulated side by side,
// e.g. sqrt(Q) and sqrt(R), keep different warps busy).
__host__ __device__ inline int tasksOf(int rows) { return pad16(rows) / kRT; }
__device__ __forceinline__ int slotFrom(int warp, int first) {
    return (warp - first % kTileWarps + kTileWarps) % kTileWarps;
}

// Pre-padded per-node matrices (column-major, leading dimension pad16(rows)).
template <typename T>
struct PadMats {
    const T *sqrtQ, *sqrtR, *q, *r;  // nonleaf cost, per node
    const T *lSqrtQ, *lq;            // leaf cost
    const T *BTr, *APB, *ABKTr;      // per node (child j)
    const T *Kt, *K, *chol;          // per nonleaf node: K' (nx x nu), K (nu x nx), lower Cholesky (nu x nu)
    const T *cholInv, *cholInvLo;    // per nonleaf node: (I + sum B'PB)^-1 (nu x nu) from the factor in FP64,
                                     // as float hi + lo (FP32 solvers only)
    const T *AB;                     // per node: [A B] (nx x nxu)
    const T *nlG, *nlGT, *lG, *lGT;  // polyhedral constraints: Gamma and Gamma' (nonleaf, leaf)
};

__device__ __forceinline__ unsigned smemAddr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

template <typename T>
__device__ __forceinline__ void cpAsyncElem(T *dst, const T *src) {
    if (sizeof(T) == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smemAddr(dst)), "l"(src));
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smemAddr(dst)), "l"(src));
}

__device__ __forceinline__ void cpAsync16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smemAddr(dst)), "l"(src));
}

// Copy a padded matrix block (count elements, count * sizeof(T) a multiple of 16 bytes).
template <typename T>
__device__ __forceinline__ void stageMat(T *dst, const T *src, int count) {
    const int chunks = count * (int)sizeof(T) / 16;
    for (int c = threadIdx.x; c < chunks; c += blockDim.x)
        cpAsync16(reinterpret_cast<char *>(dst) + 16 * (size_t)c, reinterpret_cast<const char *>(src) + 16 * (size_t)c);
}

__device__ __forceinline__ void cpAsyncWaitAll() {
    asm volatile("cp.async.commit_group;\n" ::);
    asm volatile("cp.async.wait_group 0;\n" ::);
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;\n" ::); }
// Wait for every group but the most recent one (double buffering) or for all of them.
__device__ __forceinline__ void cpAsyncWaitPrev(bool dbl) {
    if (dbl) asm volatile("cp.async.wait_group 1;\n" ::);
    else asm volatile("cp.async.wait_group 0;\n" ::);
}

// 16 consecutive matrix entries (16-byte aligned, shared memory) as warp-uniform vector loads.
__device__ __forceinline__ void load16(const float *p, float v[kRT]) {
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const float4 a = q[i];
        v[4 * i] = a.x; v[4 * i + 1] = a.y; v[4 * i + 2] = a.z; v[4 * i + 3] = a.w;
    }
}

__device__ __forceinline__ void load16(const double *p, double v[kRT]) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const double2 a = q[i];
        v[2 * i] = a.x; v[2 * i + 1] = a.y;
    }
}

template <typename T>
__device__ __forceinline__ void zeroAcc(T acc[kMaxTasks][kRT]) {
#pragma unroll
    for (int q = 0; q < kMaxTasks; q++)
#pragma unroll
        for (int t = 0; t < kRT; t++) acc[q][t] = T(0);
}

// acc[t] += m[t] * v for the 16 rows of a register block.  FP32 uses the packed two-lane FMA
// (fma.rn.f32x2, one instruction for two rows): each lane is an IEEE fused multiply-add
// rounded to nearest, bit-identical to the scalar FMA it replaces, with half the issue slots.
__device__ __forceinline__ void axpy16(float acc[kRT], const float m[kRT], float v) {
    unsigned long long vv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(vv) : "f"(v));
#pragma unroll
    for (int t = 0; t < kRT; t += 2) {
        unsigned long long a, mm;
        asm("mov.b64 %0, {%1, %2};" : "=l"(a) : "f"(acc[t]), "f"(acc[t + 1]));
        asm("mov.b64 %0, {%1, %2};" : "=l"(mm) : "f"(m[t]), "f"(m[t + 1]));
        asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(a) : "l"(mm), "l"(vv));
        asm("mov.b64 {%0, %1}, %2;" : "=f"(acc[t]), "=f"(acc[t + 1]) : "l"(a));
    }
}
__device__ __forceinline__ void axpy16(double acc[kRT], const double m[kRT], double v) {
#pragma unroll
    for (int t = 0; t < kRT; t++) acc[t] = fma(m[t], v, acc[t]);
}

// acc[q][t] += sum_k M[(slot + 8q)*16 + t, k] * in(k), M padded column-major (ld = pad16(rows)).
template <typename T, typename In>
__device__ __forceinline__ void gemv(T acc[kMaxTasks][kRT], const T *M, int rows, int K, int slot, In in) {
    const int ld = pad16(rows);
    const int nTasks = ld / kRT;
#pragma unroll
    for (int q = 0; q < kMaxTasks; q++) {
        const int task = slot + q * kTileWarps;
        if (task >= nTasks) continue;
        const T *col = M + task * kRT;
        int k = 0;
        for (; k + 2 <= K; k += 2) {
            T m0[kRT], m1[kRT];
            load16(col + (size_t)k * ld, m0);
            load16(col + (size_t)(k + 1) * ld, m1);
            const T v0 = in(k), v1 = in(k + 1);
            axpy16(acc[q], m0, v0);
            axpy16(acc[q], m1, v1);
        }
        if (k < K) {
            T m0[kRT];
            load16(col + (size_t)k * ld, m0);
            axpy16(acc[q], m0, in(k));
        }
    }
}

// Compensated matrix-vector accumulation for the forward rollout of the dynamics projection.
// Algorithm Dot2 of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005): every product m*v is split into its rounded value h and its exact error
// fma(m, v, -h); h is added to the running sum by Knuth's TwoSum, whose exact error goes, with
// the product's, into a second accumulator.  acc + cmp is then the dot product as accurate as
// if it had been accumulated in twice the working precision.  In FP32 each step is ten packed
// two-lane instructions (rounded to nearest, never contracted: inline PTX); in FP64 it is the
// plain FMA and cmp stays zero.
__device__ __forceinline__ unsigned long long pack2(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void unpack2(unsigned long long r, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ void axpy16c(float acc[kRT], float cmp[kRT], const float m[kRT], float v) {
    const unsigned long long vv = pack2(v, v), nv = pack2(-v, -v);
#pragma unroll
    for (int t = 0; t < kRT; t += 2) {
        const unsigned long long a = pack2(acc[t], acc[t + 1]), mm = pack2(m[t], m[t + 1]);
        unsigned long long c = pack2(cmp[t], cmp[t + 1]);
        unsigned long long nh, pe, s, z, t1, t2, t3, e;
        asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(nh) : "l"(mm), "l"(nv));         // -h, h = fl(m v)
        asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(pe) : "l"(mm), "l"(vv), "l"(nh));  // m v - h exactly
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(s) : "l"(a), "l"(nh));           // s = fl(a + h)
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(z) : "l"(s), "l"(a));            // TwoSum(a, h)
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t1) : "l"(s), "l"(z));
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t2) : "l"(a), "l"(t1));          // a - (s - z)
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(t3) : "l"(nh), "l"(z));          // -(h - z)
        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(e) : "l"(t2), "l"(t3));          // a + h - s exactly
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(e) : "l"(e), "l"(pe));
        asm("add.rn.f32x2 %0, %1, %2;" : "=l"(c) : "l"(c), "l"(e));
        unpack2(s, acc[t], acc[t + 1]);
        unpack2(c, cmp[t], cmp[t + 1]);
    }
}
__device__ __forceinline__ void axpy16c(double acc[kRT], double *, const double m[kRT], double v) { axpy16(acc, m, v); }

// The compensated sum's value plus an addend d: TwoSum(s, d), then both errors (FP32), or
// s + d (FP64, where the compensation is not used).
__device__ __forceinline__ float finishc(float s, float c, float d) {
    const float h = __fadd_rn(s, d), z = __fsub_rn(h, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(h, z)), __fsub_rn(d, z));
    return __fadd_rn(h, __fadd_rn(e, c));
}
__device__ __forceinline__ double finishc(double s, double, double d) { return s + d; }

// gemv with Dot2 accumulation, one matrix column per step.
template <typename T, typename In>
__device__ __forceinline__ void gemvc(T acc[kMaxTasks][kRT], T cmp[kMaxTasks][kRT], const T *M, int rows, int K, int slot,
                                      In in) {
    const int ld = pad16(rows);
    const int nTasks = ld / kRT;
#pragma unroll
    for (int q = 0; q < kMaxTasks; q++) {
        const int task = slot + q * kTileWarps;
        if (task >= nTasks) continue;
        const T *col = M + task * kRT;
#pragma unroll 1
        for (int k = 0; k < K; k++) {
            T m0[kRT];
            load16(col + (size_t)k * ld, m0);
            axpy16c(acc[q], cmp[q], m0, in(k));
        }
    }
}

// One 16-row block `task` of a padded matrix: acc[t] += sum_k M[task*16 + t, k] * in(k).
template <typename T, typename In>
__device__ __forceinline__ void gemvTask(T acc[kRT], const T *M, int rows, int K, int task, In in) {
    const int ld = pad16(rows);
    const T *col = M + task * kRT;
    int k = 0;
    for (; k + 2 <= K; k += 2) {
        T m0[kRT], m1[kRT];
        load16(col + (size_t)k * ld, m0);
        load16(col + (size_t)(k + 1) * ld, m1);
        const T v0 = in(k), v1 = in(k + 1);
        axpy16(acc, m0, v0);
        axpy16(acc, m1, v1);
    }
    if (k < K) {
        T m0[kRT];
        load16(col + (size_t)k * ld, m0);
        axpy16(acc, m0, in(k));
    }
}

// The same with Dot2 accumulation (see gemvc).
template <typename T, typename In>
__device__ __forceinline__ void gemvcTask(T acc[kRT], T cmp[kRT], const T *M, int rows, int K, int task, In in) {
    const int ld = pad16(rows);
    const T *col = M + task * kRT;
#pragma unroll 1
    for (int k = 0; k < K; k++) {
        T m0[kRT];
        load16(col + (size_t)k * ld, m0);
        axpy16c(acc, cmp, m0, in(k));
    }
}

// Gather rows rowOf(0..n-1) of `src` for instances b0 .. b0+31 into sm[r*32 + lane].
template <typename T, typename RowOf>
__device__ __forceinline__ void gather(T *sm, int n, const T *src, int B, int b0, int lane, int warp, RowOf rowOf) {
    const int bs = (b0 + lane < B) ? b0 + lane : 0;
    for (int r = warp; r < n; r += kTileWarps) cpAsyncElem(sm + r * kTileB + lane, src + (size_t)rowOf(r) * B + bs);
}

// ------------------------------------------------------------------------------------------
// L* (MODE 0: with the primal prox of cache.cuh:748-764; 1: M form; 2: bare)
// input rows, nonleaf i: [IV_j, j in ch(i)][III_i][I_i][II_i][s-source of each child, 2 rows]
//             leaf i:    [VI_l][V_l]
// base rows,  nonleaf i: [x_i][u_i][y_i][t_ch][s_ch][t_0 s_0 at the root];  leaf: [x_i]
// ------------------------------------------------------------------------------------------
template <typename T, int MODE, bool GM>
__global__ void __launch_bounds__(kTileB *kTileWarps, kOpCtasPerSm<T>) k_lstar_b(const DevProblem<T> P, const Dims D, const OpArgs<T> A,
                                                                const PadMats<T> M, int tilesPerCta, int dbl) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = reinterpret_cast<T *>(smraw);
    const int B = D.B, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu, dIV = D.dIV, dVI = D.dVI, yD = D.yD;
    const bool nonleaf = i < D.nnl;
    const int c0 = nonleaf ? P.chFrom[i] : 0, nc = nonleaf ? P.numCh[i] : 0;
    const int l = i - D.nnl;
    // constraint rows: identity part (rectangle, polyhedron with identity) and Gamma part
    // (polyhedron, polyhedron with identity); linear costs have 2-row IV / VI blocks [g'xu | t]
    const int con = nonleaf ? D.conNl : D.conL;
    const int nId =
        (con == kConRectangle || con == kConPolyhedronWithIdentity || con == kConRectangleInputBall) ? (nonleaf ? nxu : nx) : 0;
    const int nG = (con == kConPolyhedron || con == kConPolyhedronWithIdentity) ? (nonleaf ? D.gNl : D.gL) : 0;
    const bool linNl = D.costNl == kCostLinear, linL = D.costL == kCostLinear;
    // input row map
    const int rIII = nc * dIV, rIIIg = rIII + (nonleaf ? nId : 0), rI = rIIIg + (nonleaf ? nG : 0);
    const int rII = rI + yD, rS = rII + 1, rRootT = rS + 2 * nc;
    const int nIn = nonleaf ? rRootT + (linNl && i == 0 ? 1 : 0) : dVI + nId + nG;
    auto rowIV = [&](int j, int q) -> long {  // row q of IV_j
        if (linNl) return q == 0 ? D.oIV + j : D.oIV + D.n + j;
        return D.oIV + (long)j * dIV + q;
    };
    auto rowIn = [&](int r) -> long {
        if (!nonleaf) {
            if (r < dVI) return linL ? (r == 0 ? D.oVI + l : D.oVI + D.nl + l) : D.oVI + (long)l * dVI + r;
            if (r < dVI + nId) return D.oV + (long)l * nx + (r - dVI);
            return D.oV + (con == kConPolyhedron ? 0 : (long)D.nl * nx) + (long)l * D.gL + (r - dVI - nId);
        }
        if (r < rIII) return rowIV(c0 + r / dIV, r % dIV);
        if (r < rIIIg) return D.oIII + (long)i * nxu + (r - rIII);
        if (r < rI) return D.oIII + (con == kConPolyhedron ? 0 : (long)D.nnl * nxu) + (long)i * D.gNl + (r - rIIIg);
        if (r < rII) return D.oI + (long)i * yD + (r - rI);
        if (r == rII) return D.oII + i;
        if (r == rRootT) return D.oIV + D.n;  // t_0 of a linear cost
        const int jj = (r - rS) >> 1, j = c0 + jj;
        if (j < D.nnl) return D.oII + j;
        if (linL) return D.oVI + D.nl + (j - D.nnl);  // both rows: s_l itself, 0.5 (s + s) = s
        return D.oVI + (long)(j - D.nnl) * dVI + nx + ((r - rS) & 1);
    };
    const int bY = nxu, bT = bY + yD, bS = bT + nc, bRoot = bS + nc;
    const int nBase = nonleaf ? bRoot + (i == 0 ? 2 : 0) : nx;
    auto rowBase = [&](int r) -> long {
        if (!nonleaf || r < nx) return D.oX + (long)i * nx + r;
        if (r < bY) return (long)i * nu + (r - nx);
        if (r < bT) return D.oY + (long)i * yD + (r - bY);
        if (r < bS) return D.oT + c0 + (r - bT);
        if (r < bRoot) return D.oS + c0 + (r - bS);
        return r == bRoot ? D.oT : D.oS;
    };
    const int inArr = A.in2 ? 2 : 1, baseArr = A.base2 ? 2 : (A.base1 ? 1 : 0);
    const int ldx = pad16(nx), ldu = pad16(nu);
    const int perChild = linNl ? 0 : ldx * nx + ldu * nu + ldx + ldu;
    const int dG = nonleaf ? nxu : nx;  // Gamma' has dG rows (padded) and nG columns
    const int matG = nG ? pad16(dG) * nG : 0;
    // matrices staged in shared memory, or (GM: too large for it) read in place
    constexpr bool gm = GM;
    const int matElems = gm ? 0 : (nonleaf ? nc * perChild : (linL ? 0 : ldx * nx + ldx)) + matG;
    const int bufElems = (nIn * inArr + nBase * baseArr) * kTileB;  // one tile's input and base rows
    T *sMat = sm, *sBuf = sMat + matElems;
    const T *sGT = gm ? (nonleaf ? M.nlGT : M.lGT) : sMat + matElems - matG;
    // child jj's [sqrtQ | sqrtR | q | r]: staged per child, or the per-node device arrays
    auto mSqrtQ = [&](int jj) -> const T * { return gm ? M.sqrtQ + (size_t)(c0 + jj) * ldx * nx : sMat + jj * perChild; };
    auto mSqrtR = [&](int jj) -> const T * {
        return gm ? M.sqrtR + (size_t)(c0 + jj) * ldu * nu : sMat + jj * perChild + ldx * nx;
    };
    auto mQv = [&](int jj) -> const T * { return gm ? M.q + (size_t)(c0 + jj) * ldx : sMat + jj * perChild + ldx * nx + ldu * nu; };
    auto mRv = [&](int jj) -> const T * {
        return gm ? M.r + (size_t)(c0 + jj) * ldu : sMat + jj * perChild + ldx * nx + ldu * nu + ldx;
    };
    const T *mLeafQ = gm ? M.lSqrtQ : sMat, *mLeafq = gm ? M.lq : sMat + ldx * nx;
    T *sAv = sBuf + (dbl ? 2 : 1) * bufElems;  // the 4E+1 vector of the kernel projection
    // per-row extra terms of x_i / u_i (Gamma' times the Gamma rows, linear-cost gradients), dG x 32
    const bool extra = nG > 0 || (nonleaf ? linNl : linL);
    T *sGv = sAv + D.nd * kTileB;
    if (nG && !gm) stageMat(const_cast<T *>(sGT), nonleaf ? M.nlGT : M.lGT, matG);
    if (gm) {
    } else if (nonleaf && !linNl) {
        const bool qplNl = D.costNl == kCostQuadraticPlusLinear;
        for (int jj = 0; jj < nc; jj++) {
            const int j = c0 + jj;
            T *m = sMat + jj * perChild;
            stageMat(m, M.sqrtQ + (size_t)j * ldx * nx, ldx * nx);
            stageMat(m + ldx * nx, M.sqrtR + (size_t)j * ldu * nu, ldu * nu);
            if (qplNl) {
                stageMat(m + ldx * nx + ldu * nu, M.q + (size_t)j * ldx, ldx);
                stageMat(m + ldx * nx + ldu * nu + ldx, M.r + (size_t)j * ldu, ldu);
            }
        }
    } else if (!nonleaf && !linL) {
        stageMat(sMat, M.lSqrtQ, ldx * nx);
        if (D.costL == kCostQuadraticPlusLinear) stageMat(sMat + ldx * nx, M.lq, ldx);
    }
    // This CTA's instance tiles [t0, t1): with double buffering the rows of tile t + 1 are in
    // flight while tile t is computed; the node's matrices are staged once for all of them.
    const int nTiles = (B + kTileB - 1) / kTileB;
    const int t0 = blockIdx.x * tilesPerCta, t1 = min(t0 + tilesPerCta, nTiles);
    auto live = [&](int t) { return !A.live || A.live[t] != 0; };
    {  // nothing to do when every instance of this CTA's tiles has stopped
        bool any = false;
        for (int t = t0; t < t1; t++) any = any || live(t);
        if (!any) return;
    }
    // The node's row maps, evaluated once per CTA into shared memory: every tile's gathers and
    // output writes then take their iterate rows from these tables.
    int *sRowIn = reinterpret_cast<int *>(sGv + (extra ? dG : 0) * kTileB), *sRowBase = sRowIn + nIn;
    for (int r = threadIdx.x; r < nIn; r += blockDim.x) sRowIn[r] = (int)rowIn(r);
    for (int r = threadIdx.x; r < nBase; r += blockDim.x) sRowBase[r] = (int)rowBase(r);
    __syncthreads();
    auto tabIn = [&](int r) -> long { return sRowIn[r]; };
    auto tabBase = [&](int r) -> long { return sRowBase[r]; };
    auto prefetch = [&](int t) {
        if (!live(t)) return;
        T *buf = sBuf + (dbl ? ((t - t0) & 1) * bufElems : 0);
        const int bb = t * kTileB;
        gather(buf, nIn, A.in1, B, bb, lane, warp, tabIn);
        if (A.in2) gather(buf + nIn * kTileB, nIn, A.in2, B, bb, lane, warp, tabIn);
        T *bs = buf + nIn * inArr * kTileB;
        if (A.base1) gather(bs, nBase, A.base1, B, bb, lane, warp, tabBase);
        if (A.base2) gather(bs + nBase * kTileB, nBase, A.base2, B, bb, lane, warp, tabBase);
    };
    if (t0 < t1) prefetch(t0);
    cpAsyncCommit();
    for (int tile = t0; tile < t1; tile++) {
        if (dbl && tile + 1 < t1) prefetch(tile + 1);
        cpAsyncCommit();
        cpAsyncWaitPrev(dbl);
        __syncthreads();
        const T *sIn = sBuf + (dbl ? ((tile - t0) & 1) * bufElems : 0), *sBase = sIn + nIn * inArr * kTileB;
        const int b0 = tile * kTileB, b = b0 + lane;
        const bool act = b < B;
        auto tileBody = [&]() {
        auto IN = [&](int r) -> T {
            T v = A.a1 * sIn[r * kTileB + lane];
            if (inArr == 2) v += A.a2 * sIn[(nIn + r) * kTileB + lane];
            return v;
        };
        auto BASE = [&](int r) -> T {
            if (!baseArr) return T(0);
            T v = A.b1 * sBase[r * kTileB + lane];
            if (baseArr == 2) v += A.b2 * sBase[(nBase + r) * kTileB + lane];
            return v;
        };
        auto EMIT = [&](int rb, T lv) {
            if (!act) return;
            const T bs = BASE(rb);
            const size_t o = (size_t)sRowBase[rb] * B + b;
            if (A.outBase) A.outBase[o] = bs;
            A.out[o] = bs + A.cL * lv;
        };
        auto FIN = [&](int rb, T val) {  // a final primal entry (mode 0) and its residual
            if (!act) return;
            const size_t o = (size_t)sRowBase[rb] * B + b;
            A.out[o] = val;
            if (A.outR) A.outR[o] = BASE(rb) - val;
        };
        if (extra) {  // Gamma' times the Gamma rows of III or V (constraints.cuh:272-285, 410-425), plus the
                      // linear-cost gradients times IV / VI (costs.cuh:274-292), into shared memory
            T accG[kMaxTasks][kRT];
            zeroAcc(accG);
            const int rg = nonleaf ? rIIIg : dVI + nId;
            if (nG) gemv(accG, sGT, dG, nG, warp, [&](int k) { return IN(rg + k); });
    #pragma unroll
            for (int q = 0; q < kMaxTasks; q++) {
                const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                for (int t = 0; t < kRT; t++) {
                    const int r = r0 + t;
                    if (r >= dG) continue;
                    T v = accG[q][t];
                    if (nonleaf && linNl)
                        for (int jj = 0; jj < nc; jj++) v += __ldg(P.grad + (size_t)(c0 + jj) * nxu + r) * IN(jj * dIV);
                    if (!nonleaf && linL) v += __ldg(P.lGrad + r) * IN(0);
                    sGv[r * kTileB + lane] = v;
                }
            }
            __syncthreads();
        }
        // constraint and linear-cost part of x_i / u_i (row r of [x; u])
        auto conPart = [&](int r, int rId) -> T {
            T v = nId ? IN(rId + r) : T(0);
            if (extra) v += sGv[r * kTileB + lane];
            return v;
        };
        T accX[kMaxTasks][kRT], accU[kMaxTasks][kRT];
        zeroAcc(accX);
        zeroAcc(accU);
        if (nonleaf) {
            const bool qpl = D.costNl == kCostQuadraticPlusLinear;
            const int sx = warp, su = slotFrom(warp, tasksOf(nx));  // x and u blocks on different warps
            for (int jj = 0; jj < nc && !linNl; jj++) {
                const int r0 = jj * dIV;
                gemv(accX, mSqrtQ(jj), nx, nx, sx, [&](int k) { return IN(r0 + k); });
                gemv(accU, mSqrtR(jj), nu, nu, su, [&](int k) { return IN(r0 + nx + k); });
                if (qpl) {
                    const T d23 = T(-0.5) * (IN(r0 + nxu) + IN(r0 + nxu + 1));
                    gemv(accX, mQv(jj), nx, 1, sx, [&](int) { return d23; });
                    gemv(accU, mRv(jj), nu, 1, su, [&](int) { return d23; });
                }
            }
    #pragma unroll
            for (int q = 0; q < kMaxTasks; q++) {
                const int rx0 = (sx + q * kTileWarps) * kRT, ru0 = (su + q * kTileWarps) * kRT;
    #pragma unroll
                for (int t = 0; t < kRT; t++) {
                    if (rx0 + t < nx) EMIT(rx0 + t, accX[q][t] + conPart(rx0 + t, rIII));
                    if (ru0 + t < nu) EMIT(nx + ru0 + t, accU[q][t] + conPart(nx + ru0 + t, rIII));
                }
            }
            // y_i, the children's t and s, and the AVaR kernel projection (cache.cuh:650-676): entry
            // k of the 4E+1 vector is formed by warp k % 8; in a T evaluation it goes to shared
            // memory and each warp then applies rows of N N' to it
            const T II = IN(rII);
            auto avarOut = [&](int k) -> int {  // base row of entry k, -1 for padding
                if (k < yD) return bY + k;
                if (k < yD + D.ne) return k - yD < nc ? bT + (k - yD) : -1;
                return k - yD - D.ne < nc ? bS + (k - yD - D.ne) : -1;
            };
            auto avarLin = [&](int k) -> T {  // the L* part of entry k
                if (k < yD) return IN(rI + k) - P.b[(size_t)i * yD + k] * II;
                if (k < yD + D.ne) {  // t_j: half the sum of the last two IV rows, or IV's t row (linear)
                    const int jj = k - yD;
                    return linNl ? IN(jj * dIV + 1) : T(0.5) * (IN(jj * dIV + nxu) + IN(jj * dIV + nxu + 1));
                }
                const int jj = k - yD - D.ne;
                return (c0 + jj < D.nnl) ? IN(rS + 2 * jj) : T(0.5) * (IN(rS + 2 * jj) + IN(rS + 2 * jj + 1));
            };
            if (MODE == 0) {
                for (int k = warp; k < D.nd; k += kTileWarps) {
                    const int ob = avarOut(k);
                    sAv[k * kTileB + lane] = ob >= 0 ? BASE(ob) + A.cL * avarLin(k) : T(0);
                }
                __syncthreads();
                const T *N = P.NNtr + (size_t)i * D.nd * D.nd;
                for (int k = warp; k < D.nd; k += kTileWarps) {
                    const int ob = avarOut(k);
                    if (ob < 0) continue;
                    T acc = 0;
                    for (int c = 0; c < D.nd; c++) acc += __ldg(N + (size_t)c * D.nd + k) * sAv[c * kTileB + lane];
                    FIN(ob, acc);
                }
            } else {
                for (int k = warp; k < D.nd; k += kTileWarps) {
                    const int ob = avarOut(k);
                    if (ob >= 0) EMIT(ob, avarLin(k));
                }
            }
            if (warp == 0) {
                if (i == 0) {  // t_0: no cost term (or IV's t row of a linear cost); s_0 gets the prox of the objective
                    const T t0 = linNl ? IN(rRootT) : T(0);
                    if (MODE == 0) {
                        FIN(bRoot, BASE(bRoot) + A.cL * t0);
                        FIN(bRoot + 1, BASE(bRoot + 1) + A.cL * II - P.step);
                    } else {
                        EMIT(bRoot, t0);
                        EMIT(bRoot + 1, II);
                    }
                }
            }
        } else {
            if (!linL) {
                gemv(accX, mLeafQ, nx, nx, warp, [&](int k) { return IN(k); });
                if (D.costL == kCostQuadraticPlusLinear) {
                    const T d23 = T(-0.5) * (IN(nx) + IN(nx + 1));
                    gemv(accX, mLeafq, nx, 1, warp, [&](int) { return d23; });
                }
            }
    #pragma unroll
            for (int q = 0; q < kMaxTasks; q++) {
                const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                for (int t = 0; t < kRT; t++) {
                    const int r = r0 + t;
                    if (r < nx) EMIT(r, accX[q][t] + conPart(r, dVI));
                }
            }
        }
        };
        if (live(tile)) tileBody();
        __syncthreads();  // every warp is done with this tile's rows before the buffer is refilled
        if (!dbl && tile + 1 < t1) prefetch(tile + 1);
    }
}

// ------------------------------------------------------------------------------------------
// L (MODE 0: with the dual prox of cache.cuh:770-789; 1: M form; 2: bare)
// input rows: [x_a][u_a][t_j] (a = ancestor of j; zero rows at the root), then nonleaf j:
//             [y_j][s_j][x_j][u_j], leaf j: [x_j][s_j]
// base rows:  nonleaf j: [I_j][II_j][III_j][IV_j];  leaf j: [IV_j][V_l][VI_l]
// ------------------------------------------------------------------------------------------
template <typename T, int MODE, bool GM>
__global__ void __launch_bounds__(kTileB *kTileWarps, kOpCtasPerSm<T>) k_lop_b(const DevProblem<T> P, const Dims D, const OpArgs<T> A,
                                                              const PadMats<T> M, int tilesPerCta, int dbl) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = reinterpret_cast<T *>(smraw);
    const int B = D.B, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int j = blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu, dIV = D.dIV, dVI = D.dVI, yD = D.yD;
    const bool nonleaf = j < D.nnl;
    const int l = j - D.nnl;
    const int a = j > 0 ? P.anc[j] : 0;
    // constraint rows of this node: an identity part (rectangle, polyhedron with identity) and a
    // Gamma part (polyhedron, polyhedron with identity); linear costs have a 2-row IV / VI
    const int con = nonleaf ? D.conNl : D.conL;
    const int nId =
        (con == kConRectangle || con == kConPolyhedronWithIdentity || con == kConRectangleInputBall) ? (nonleaf ? nxu : nx) : 0;
    const int nG = (con == kConPolyhedron || con == kConPolyhedronWithIdentity) ? (nonleaf ? D.gNl : D.gL) : 0;
    const bool linNl = D.costNl == kCostLinear, linL = D.costL == kCostLinear;
    const T g = P.step, gi = T(1) / P.step;
    const int rOwn = nxu + 1;
    const int nIn = nonleaf ? rOwn + yD + 1 + nxu : rOwn + nx + 1;
    auto rowIn = [&](int r) -> long {
        if (r < nx) return D.oX + (long)a * nx + r;
        if (r < nxu) return (long)a * nu + (r - nx);
        if (r == nxu) return D.oT + j;
        const int q = r - rOwn;
        if (nonleaf) {
            if (q < yD) return D.oY + (long)j * yD + q;
            if (q == yD) return D.oS + j;
            if (q < yD + 1 + nx) return D.oX + (long)j * nx + (q - yD - 1);
            return (long)j * nu + (q - yD - 1 - nx);
        }
        if (q < nx) return D.oX + (long)j * nx + q;
        return D.oS + j;
    };
    const int bIII = yD + 1, bIIIg = bIII + nId, bIVn = bIIIg + nG;
    const int bIV = nonleaf ? bIVn : 0, bV = dIV, bVg = bV + nId, bVI = bVg + nG;
    const int nBase = nonleaf ? bIVn + dIV : bVI + dVI;
    auto rowIV = [&](int q) -> long {  // row q of IV_j: per node (quadratic), or [g'xu | t] (linear)
        if (linNl) return q == 0 ? D.oIV + j : D.oIV + D.n + j;
        return D.oIV + (long)j * dIV + q;
    };
    auto rowBase = [&](int r) -> long {
        if (nonleaf) {
            if (r < yD) return D.oI + (long)j * yD + r;
            if (r == yD) return D.oII + j;
            if (r < bIIIg) return D.oIII + (long)j * nxu + (r - bIII);
            if (r < bIVn)
                return D.oIII + (con == kConPolyhedron ? 0 : (long)D.nnl * nxu) + (long)j * D.gNl + (r - bIIIg);
            return rowIV(r - bIVn);
        }
        if (r < bV) return rowIV(r);
        if (r < bVg) return D.oV + (long)l * nx + (r - bV);
        if (r < bVI) return D.oV + (con == kConPolyhedron ? 0 : (long)D.nl * nx) + (long)l * D.gL + (r - bVg);
        if (linL) return r == bVI ? D.oVI + l : D.oVI + D.nl + l;
        return D.oVI + (long)l * dVI + (r - bVI);
    };
    const int inArr = A.in2 ? 2 : 1, baseArr = A.base2 ? 2 : (A.base1 ? 1 : 0);
    const int dSoc = max(max(dIV, dVI), nu);  // sw holds an SOC block or the inputs of an input ball
    const int ldx = pad16(nx), ldu = pad16(nu);
    const int matIV = linNl ? 0 : ldx * nx + ldu * nu, matVI = (!nonleaf && !linL) ? ldx * nx : 0;
    const int matG = nG ? pad16(nG) * (nonleaf ? nxu : nx) : 0;  // Gamma, padded column-major
    constexpr bool gm = GM;  // matrices read in place instead of staged
    const int matElems = gm ? 0 : matIV + matVI + matG;
    const int bufElems = (nIn * inArr + nBase * baseArr) * kTileB;  // one tile's input and base rows
    T *sMatS = sm, *sw = sMatS + matElems, *sPart = sw + dSoc * kTileB, *sBuf = sPart + kTileWarps * kTileB;
    if (!gm) {
        if (j > 0 && !linNl) {
            stageMat(sMatS, M.sqrtQ + (size_t)j * ldx * nx, ldx * nx);
            stageMat(sMatS + ldx * nx, M.sqrtR + (size_t)j * ldu * nu, ldu * nu);
        }
        if (matVI) stageMat(sMatS + matIV, M.lSqrtQ, ldx * nx);
        if (nG) stageMat(sMatS + matIV + matVI, nonleaf ? M.nlG : M.lG, matG);
    }
    const T *sG = gm ? (nonleaf ? M.nlG : M.lG) : sMatS + matIV + matVI;
    const T *mSqrtQ = gm ? M.sqrtQ + (size_t)j * ldx * nx : sMatS, *mSqrtR = gm ? M.sqrtR + (size_t)j * ldu * nu : sMatS + ldx * nx;
    const T *mLeafQ = gm ? M.lSqrtQ : sMatS + matIV;
    // This CTA's instance tiles [t0, t1), double-buffered as in k_lstar_b.
    const int nTiles = (B + kTileB - 1) / kTileB;
    const int t0 = blockIdx.x * tilesPerCta, t1 = min(t0 + tilesPerCta, nTiles);
    auto live = [&](int t) { return !A.live || A.live[t] != 0; };
    {  // nothing to do when every instance of this CTA's tiles has stopped
        bool any = false;
        for (int t = t0; t < t1; t++) any = any || live(t);
        if (!any) return;
    }
    // The node's row maps, evaluated once per CTA into shared memory: every tile's gathers and
    // output writes then take their iterate rows from these tables.
    int *sRowIn = reinterpret_cast<int *>(sBuf + (dbl ? 2 : 1) * bufElems), *sRowBase = sRowIn + nIn;
    for (int r = threadIdx.x; r < nIn; r += blockDim.x) sRowIn[r] = (int)rowIn(r);
    for (int r = threadIdx.x; r < nBase; r += blockDim.x) sRowBase[r] = (int)rowBase(r);
    __syncthreads();
    auto tabIn = [&](int r) -> long { return sRowIn[r]; };
    auto tabBase = [&](int r) -> long { return sRowBase[r]; };
    auto prefetch = [&](int t) {
        if (!live(t)) return;
        T *buf = sBuf + (dbl ? ((t - t0) & 1) * bufElems : 0);
        const int bb = t * kTileB;
        gather(buf, nIn, A.in1, B, bb, lane, warp, tabIn);
        if (A.in2) gather(buf + nIn * kTileB, nIn, A.in2, B, bb, lane, warp, tabIn);
        T *bs = buf + nIn * inArr * kTileB;
        if (A.base1) gather(bs, nBase, A.base1, B, bb, lane, warp, tabBase);
        if (A.base2) gather(bs + nBase * kTileB, nBase, A.base2, B, bb, lane, warp, tabBase);
    };
    if (t0 < t1) prefetch(t0);
    cpAsyncCommit();
    for (int tile = t0; tile < t1; tile++) {
        if (dbl && tile + 1 < t1) prefetch(tile + 1);
        cpAsyncCommit();
        cpAsyncWaitPrev(dbl);
        __syncthreads();
        const T *sIn = sBuf + (dbl ? ((tile - t0) & 1) * bufElems : 0), *sBase = sIn + nIn * inArr * kTileB;
        const int b0 = tile * kTileB, b = b0 + lane;
        const bool act = b < B;
        auto tileBody = [&]() {
        auto INP = [&](int r) -> T {
            T v = A.a1 * sIn[r * kTileB + lane];
            if (inArr == 2) v += A.a2 * sIn[(nIn + r) * kTileB + lane];
            return v;
        };
        auto BASE = [&](int r) -> T {
            if (!baseArr) return T(0);
            T v = A.b1 * sBase[r * kTileB + lane];
            if (baseArr == 2) v += A.b2 * sBase[(nBase + r) * kTileB + lane];
            return v;
        };
        auto EMIT = [&](int rb, T lv) {
            if (!act) return;
            const T bs = BASE(rb);
            const size_t o = (size_t)sRowBase[rb] * B + b;
            if (A.outBase) A.outBase[o] = bs;
            A.out[o] = bs + A.cL * lv;
        };
        auto FIN = [&](int rb, T val) {  // a final dual entry (mode 0) and its residual
            if (!act) return;
            const size_t o = (size_t)sRowBase[rb] * B + b;
            A.out[o] = val;
            if (A.outR) A.outR[o] = BASE(rb) - val;
        };
        // (v - proj(v)) * gamma for an SOC block staged in sw (dim rows), called by every warp after
        // the barrier that publishes sw: the squared norm is summed over warps in shared memory
        auto socBlock = [&](int dim, int rb0) {
            T ss = 0;
            for (int c = warp; c < dim - 1; c += kTileWarps) ss += sw[c * kTileB + lane] * sw[c * kTileB + lane];
            sPart[warp * kTileB + lane] = ss;
            __syncthreads();
            ss = 0;
    #pragma unroll
            for (int w = 0; w < kTileWarps; w++) ss += sPart[w * kTileB + lane];
            const T nrm = sqrt(ss), tt = sw[(dim - 1) * kTileB + lane];
            const int i1 = nrm <= tt, i2 = (nrm <= -tt) && !i1, i3 = !i1 && !i2;
            const T sc = (nrm + tt) / (T(2) * nrm + T(1 - i3));
            for (int c = warp; c < dim; c += kTileWarps) {
                const T v = sw[c * kTileB + lane];
                const T pr = i1 ? v : (i2 ? T(0) : (c < dim - 1 ? sc * v : sc * nrm));
                FIN(rb0 + c, (v - pr) * g);
            }
        };
        if (nonleaf) {
            const int nm = 2 * P.numCh[j];
            const int ry = rOwn, rs = rOwn + yD, rx = rs + 1, ru = rx + nx;
            for (int k = warp; k < yD; k += kTileWarps) {
                const T lv = INP(ry + k);
                if (MODE == 0) {
                    const T v = (BASE(k) + A.cL * lv) * gi;
                    const T pr = (k < nm && v < T(0)) ? T(0) * v : v;  // AVaR dual cone (risks.cuh:99-106)
                    FIN(k, (v - pr) * g);
                } else EMIT(k, lv);
            }
            if (warp == kTileWarps - 1) {
                T lv = INP(rs);
                for (int k = 0; k < yD; k++) lv -= __ldg(P.b + (size_t)j * yD + k) * INP(ry + k);
                if (MODE == 0) {
                    const T v = (BASE(yD) + A.cL * lv) * gi;
                    FIN(yD, (v - (v > T(0) ? v : T(0))) * g);
                } else EMIT(yD, lv);
            }
            auto boxRow = [&](int rb, T lv) {  // III row: [x; u] or Gamma [x; u], box bounds (constraints.cuh:70-74)
                if (MODE == 0) {
                    const size_t bi = (size_t)(sRowBase[rb] - D.oIII);
                    const T v = (BASE(rb) + A.cL * lv) * gi;
                    FIN(rb, (v - boxProject(v, P.nlLo[bi], P.nlHi[bi])) * g);
                } else EMIT(rb, lv);
            };
            if (con == kConRectangleInputBall && MODE == 0) {
                // box on the x rows; u * min(1, r / ||u||) on the u rows, the norm summed over warps
                for (int k = warp; k < nx; k += kTileWarps) boxRow(bIII + k, INP(rx + k));
                T ss = 0;
                for (int k = warp; k < nu; k += kTileWarps) {
                    const T v = (BASE(bIII + nx + k) + A.cL * INP(ru + k)) * gi;
                    sw[k * kTileB + lane] = v;
                    ss += v * v;
                }
                sPart[warp * kTileB + lane] = ss;
                __syncthreads();
                ss = 0;
    #pragma unroll
                for (int w = 0; w < kTileWarps; w++) ss += sPart[w * kTileB + lane];
                const T nrm = sqrt(ss), f = nrm > P.radius ? P.radius / nrm : T(1);
                for (int k = warp; k < nu; k += kTileWarps) {
                    const T v = sw[k * kTileB + lane];
                    FIN(bIII + nx + k, (v - f * v) * g);
                }
                __syncthreads();  // sw and sPart are reused below
            } else {
                for (int k = warp; k < nId; k += kTileWarps) boxRow(bIII + k, k < nx ? INP(rx + k) : INP(ru + k - nx));
            }
            if (nG) {  // Gamma [x_j; u_j] (constraints.cuh:251-264, 386-401)
                T accG[kMaxTasks][kRT];
                zeroAcc(accG);
                gemv(accG, sG, nG, nxu, warp, [&](int k) { return INP(rx + k); });
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++)
                        if (r0 + t < nG) boxRow(bIIIg + r0 + t, accG[q][t]);
                }
            }
        }
        auto linEpi = [&](int rb, T lv0, T lv1) {  // linear-cost epigraph rows (costs.cuh:261-301)
            if (MODE == 0) {
                const T v0 = (BASE(rb) + A.cL * lv0) * gi, v1 = (BASE(rb + 1) + A.cL * lv1) * gi;
                FIN(rb, (v0 - (v0 < v1 ? v0 : v1)) * g);  // the first entry is clamped from above by the second
                FIN(rb + 1, T(0));
            } else {
                EMIT(rb, lv0);
                EMIT(rb + 1, lv1);
            }
        };
        if (linNl) {  // IV_j = [g_j'(x_a, u_a); t_j]; the root has no g term
            if (warp == 0) {
                T lin = 0;
                if (j > 0)
                    for (int k = 0; k < nxu; k++) lin += __ldg(P.grad + (size_t)j * nxu + k) * INP(k);
                linEpi(bIV, lin, INP(nxu));
            }
        } else {  // IV_j = [sqrtQ_j x_a; sqrtR_j u_a; h; h] (costs.cuh:126-161, 379-417); zero at the root
            T accX[kMaxTasks][kRT], accU[kMaxTasks][kRT];
            zeroAcc(accX);
            zeroAcc(accU);
            T h = 0;
            const int sx = warp, su = slotFrom(warp, tasksOf(nx));  // x and u blocks on different warps
            if (j > 0) {
                gemv(accX, mSqrtQ, nx, nx, sx, [&](int k) { return INP(k); });
                gemv(accU, mSqrtR, nu, nu, su, [&](int k) { return INP(nx + k); });
                h = T(0.5) * INP(nxu);
                if (D.costNl == kCostQuadraticPlusLinear) {
                    T lin = 0;
                    for (int k = 0; k < nx; k++) lin += __ldg(P.q + (size_t)j * nx + k) * INP(k);
                    for (int k = 0; k < nu; k++) lin += __ldg(P.r + (size_t)j * nu + k) * INP(nx + k);
                    h -= T(0.5) * lin;
                }
            }
            if (MODE == 0) {
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int rx0 = (sx + q * kTileWarps) * kRT, ru0 = (su + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++) {
                        const int r = rx0 + t, ru = ru0 + t;
                        if (r < nx) sw[r * kTileB + lane] = (BASE(bIV + r) + A.cL * accX[q][t]) * gi + P.trans[(size_t)j * dIV + r];
                        if (ru < nu)
                            sw[(nx + ru) * kTileB + lane] =
                                (BASE(bIV + nx + ru) + A.cL * accU[q][t]) * gi + P.trans[(size_t)j * dIV + nx + ru];
                    }
                }
                if (warp == 0)
                    for (int r = nxu; r < dIV; r++) sw[r * kTileB + lane] = (BASE(bIV + r) + A.cL * h) * gi + P.trans[(size_t)j * dIV + r];
                __syncthreads();
                socBlock(dIV, bIV);
            } else {
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int rx0 = (sx + q * kTileWarps) * kRT, ru0 = (su + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++) {
                        if (rx0 + t < nx) EMIT(bIV + rx0 + t, accX[q][t]);
                        if (ru0 + t < nu) EMIT(bIV + nx + ru0 + t, accU[q][t]);
                    }
                }
                if (warp == 0)
                    for (int r = nxu; r < dIV; r++) EMIT(bIV + r, h);
            }
        }
        if (!nonleaf) {  // V and VI of a leaf (constraints.cuh:168-170, costs.cuh:149-161/404-417)
            const int rx = rOwn, rs = rOwn + nx;
            auto boxRowL = [&](int rb, T lv) {
                if (MODE == 0) {
                    const size_t bi = (size_t)(sRowBase[rb] - D.oV);
                    const T v = (BASE(rb) + A.cL * lv) * gi;
                    FIN(rb, (v - boxProject(v, P.lLo[bi], P.lHi[bi])) * g);
                } else EMIT(rb, lv);
            };
            for (int k = warp; k < nId; k += kTileWarps) boxRowL(bV + k, INP(rx + k));
            if (nG) {
                T accG[kMaxTasks][kRT];
                zeroAcc(accG);
                gemv(accG, sG, nG, nx, warp, [&](int k) { return INP(rx + k); });
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++)
                        if (r0 + t < nG) boxRowL(bVg + r0 + t, accG[q][t]);
                }
            }
            if (linL) {  // VI_l = [g'x_l; s_l]
                if (warp == 0) {
                    T lin = 0;
                    for (int k = 0; k < nx; k++) lin += __ldg(P.lGrad + k) * INP(rx + k);
                    linEpi(bVI, lin, INP(rs));
                }
                return;  // nothing else in this tile; the caller's barrier follows
            }
            T accX[kMaxTasks][kRT];
            zeroAcc(accX);
            gemv(accX, mLeafQ, nx, nx, warp, [&](int k) { return INP(rx + k); });
            T h = T(0.5) * INP(rs);
            if (D.costL == kCostQuadraticPlusLinear) {
                T lin = 0;
                for (int k = 0; k < nx; k++) lin += __ldg(P.lq + k) * INP(rx + k);
                h -= T(0.5) * lin;
            }
            if (MODE == 0) {
                __syncthreads();  // sw is reused after the IV block
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++) {
                        const int r = r0 + t;
                        if (r < nx) sw[r * kTileB + lane] = (BASE(bVI + r) + A.cL * accX[q][t]) * gi + P.lTrans[r];
                    }
                }
                if (warp == 0)
                    for (int r = nx; r < dVI; r++) sw[r * kTileB + lane] = (BASE(bVI + r) + A.cL * h) * gi + P.lTrans[r];
                __syncthreads();
                socBlock(dVI, bVI);
            } else {
    #pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int r0 = (warp + q * kTileWarps) * kRT;
    #pragma unroll
                    for (int t = 0; t < kRT; t++) {
                        const int r = r0 + t;
                        if (r < nx) EMIT(bVI + r, accX[q][t]);
                    }
                }
                if (warp == 0)
                    for (int r = nx; r < dVI; r++) EMIT(bVI + r, h);
            }
        }
        };
        if (live(tile)) tileBody();
        __syncthreads();  // every warp is done with this tile's rows (and sw) before they are refilled
        if (!dbl && tile + 1 < t1) prefetch(tile + 1);
    }
}

// ------------------------------------------------------------------------------------------
// Dynamics projection, one stage of the backward sweep (dynamics.cuh:85-139).
// inputs per instance tile: q of the children (-x of leaves at the last stage, else Q), u_i, x_i.
// A CTA stages node i's matrices once and runs `tilesPerCta` instance tiles, double-buffered
// when `dbl` (the rows of tile t + 1 load while tile t is computed).
// Work split per tile, in three phases separated by barriers (U = 16-row blocks of u, X = of x):
//  1. warps 0..U-1 form rhs = u_i - sum_j B_j' q_j, while the x blocks (on the warps after them,
//     wrapping round) accumulate sum_j (A_j + B_j K_j)' P_j q_j, which does not depend on d;
//  2. d = (I + sum B'PB)^-1 rhs: FP32 multiplies by the inverse, precomputed in FP64 from the
//     cached Cholesky factor and kept as a float pair hi + lo (so the solve is a product on U
//     warps instead of a serial triangular solve on one); FP64 keeps the reference's triangular
//     solves;
//  3. the x blocks add sum_j A_j'P_j B_j d + K_i'(d - u_i) and write q_i - x_i.
// ------------------------------------------------------------------------------------------
template <typename T, bool GM>
__global__ void __launch_bounds__(kTileB *kTileWarps, 2) k_dyn_back_b(const DevProblem<T> P, const Dims D, const PadMats<T> M,
                                                                  const T *__restrict__ cand, T *__restrict__ Q,
                                                                  T *__restrict__ DD, int stageFrom, int stage,
                                                                  int tilesPerCta, int dbl, const int *live) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = reinterpret_cast<T *>(smraw);
    const int B = D.B, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = stageFrom + blockIdx.y;
    const int nx = D.nx, nu = D.nu;
    const int c0 = P.chFrom[i], nc = P.numCh[i];
    const bool leafChildren = c0 >= D.nnl;
    const int ldx = pad16(nx), ldu = pad16(nu);
    const int U = tasksOf(nu);
    const int perChild = ldu * nx + ldx * nu + ldx * nx;  // B', APB, (A+BK)'
    const int bufElems = (nc * nx + nu + nx) * kTileB;   // one tile's q, u and x rows
    constexpr bool kInverse = sizeof(T) == 4;            // FP32: d by the inverse (phase 2)
    constexpr bool gm = GM;  // matrices read in place instead of staged
    const int matElems = gm ? 0 : nc * perChild + ldx * nu + ldu * nu;
    // d: FP32 writes it next to rhs (into the tile's q rows, free after phase 1, when they are
    // large enough: nx >= nu; else into a buffer of its own); FP64 solves in place
    const bool dOwn = kInverse && nx < nu;
    T *sMat = sm, *sd = sm + matElems, *sdOwn = sd + nu * kTileB, *sBuf = sdOwn + (dOwn ? nu * kTileB : 0);
    T *sKtS = sMat + nc * perChild, *sLS = sKtS + ldx * nu;
    const T *gL = (kInverse ? M.cholInv : M.chol) + (size_t)i * ldu * nu;
    const T *sKt = gm ? M.Kt + (size_t)i * ldx * nu : sKtS, *sL = gm ? gL : sLS;
    const T *sLlo = kInverse ? M.cholInvLo + (size_t)i * ldu * nu : nullptr;  // small: read in place
    auto mBTr = [&](int jj) -> const T * { return gm ? M.BTr + (size_t)(c0 + jj) * ldu * nx : sMat + jj * perChild; };
    auto mAPB = [&](int jj) -> const T * {
        return gm ? M.APB + (size_t)(c0 + jj) * ldx * nu : sMat + jj * perChild + ldu * nx;
    };
    auto mABKTr = [&](int jj) -> const T * {
        return gm ? M.ABKTr + (size_t)(c0 + jj) * ldx * nx : sMat + jj * perChild + ldu * nx + ldx * nu;
    };
    if (!gm) {
        for (int jj = 0; jj < nc; jj++) {
            const int j = c0 + jj;
            T *m = sMat + jj * perChild;
            stageMat(m, M.BTr + (size_t)j * ldu * nx, ldu * nx);
            if (stage > 0) {
                stageMat(m + ldu * nx, M.APB + (size_t)j * ldx * nu, ldx * nu);
                stageMat(m + ldu * nx + ldx * nu, M.ABKTr + (size_t)j * ldx * nx, ldx * nx);
            }
        }
        if (stage > 0) stageMat(sKtS, M.Kt + (size_t)i * ldx * nu, ldx * nu);
        stageMat(sLS, gL, ldu * nu);
    }
    const int nTiles = (B + kTileB - 1) / kTileB;
    const int t0 = blockIdx.x * tilesPerCta, t1 = min(t0 + tilesPerCta, nTiles);
    auto isLive = [&](int t) { return !live || live[t] != 0; };
    {  // nothing to do when every instance of this CTA's tiles has stopped
        bool any = false;
        for (int t = t0; t < t1; t++) any = any || isLive(t);
        if (!any) return;
    }
    auto prefetch = [&](int t) {
        if (!isLive(t)) return;
        T *sq = sBuf + (dbl ? ((t - t0) & 1) * bufElems : 0), *su = sq + nc * nx * kTileB, *sx = su + nu * kTileB;
        const int bb = t * kTileB;
        if (leafChildren)
            gather(sq, nc * nx, cand, B, bb, lane, warp, [&](int r) { return D.oX + (long)c0 * nx + r; });
        else
            gather(sq, nc * nx, (const T *)Q, B, bb, lane, warp, [&](int r) { return (long)c0 * nx + r; });
        gather(su, nu, cand, B, bb, lane, warp, [&](int r) { return (long)i * nu + r; });
        if (stage > 0) gather(sx, nx, cand, B, bb, lane, warp, [&](int r) { return D.oX + (long)i * nx + r; });
    };
    if (t0 < t1) prefetch(t0);
    cpAsyncCommit();
    const int sxw = slotFrom(warp, U);  // the x blocks start on the warp after the u blocks
    for (int tile = t0; tile < t1; tile++) {
        if (dbl && tile + 1 < t1) prefetch(tile + 1);
        cpAsyncCommit();
        cpAsyncWaitPrev(dbl);
        __syncthreads();
        T *sq = sBuf + (dbl ? ((tile - t0) & 1) * bufElems : 0), *su = sq + nc * nx * kTileB, *sx = su + nu * kTileB;
        const int b = tile * kTileB + lane;
        const bool act = b < B;
        auto tileBody = [&]() {
        if (leafChildren || D.affine) {  // q of a leaf is -x; affine dynamics add P e (dynamics.cuh:96-99)
            for (int t = warp; t < nc * nx; t += kTileWarps) {
                T v = sq[t * kTileB + lane];
                if (leafChildren) v = -v;
                if (D.affine) v += P.Pe[(size_t)c0 * nx + t];
                sq[t * kTileB + lane] = v;
            }
            __syncthreads();
        }
        // phase 1
        for (int task = warp; task < U; task += kTileWarps) {
            T a[kRT];
#pragma unroll
            for (int t = 0; t < kRT; t++) a[t] = T(0);
            for (int jj = 0; jj < nc; jj++) {
                const T *qv = sq + jj * nx * kTileB + lane;
                gemvTask(a, mBTr(jj), nu, nx, task, [&](int k) { return qv[k * kTileB]; });
            }
#pragma unroll
            for (int t = 0; t < kRT; t++) {
                const int r = task * kRT + t;
                if (r < nu) sd[r * kTileB + lane] = su[r * kTileB + lane] - a[t];
            }
        }
        T acc[kMaxTasks][kRT];
        zeroAcc(acc);
        if (stage > 0)
            for (int jj = 0; jj < nc; jj++) {
                const T *qv = sq + jj * nx * kTileB + lane;
                gemv(acc, mABKTr(jj), nx, nx, sxw, [&](int k) { return qv[k * kTileB]; });
            }
        __syncthreads();
        // phase 2
        T *sd2 = dOwn ? sdOwn : sq;
        const T *dv = kInverse ? sd2 : sd;
        if (kInverse) {
            for (int task = warp; task < U; task += kTileWarps) {  // d = Rinv_hi rhs + Rinv_lo rhs
                T a[kRT], cm[kRT];
#pragma unroll
                for (int t = 0; t < kRT; t++) a[t] = cm[t] = T(0);
                gemvTask(a, sL, nu, nu, task, [&](int k) { return sd[k * kTileB + lane]; });
                gemvTask(cm, sLlo, nu, nu, task, [&](int k) { return sd[k * kTileB + lane]; });
#pragma unroll
                for (int t = 0; t < kRT; t++) {
                    const int r = task * kRT + t;
                    if (r < nu) sd2[r * kTileB + lane] = a[t] + cm[t];
                }
            }
        } else if (warp == 0) {  // (I + sum B'PB) d = rhs with the cached lower Cholesky factor
            const T *L = sL;  // padded: L(r, k) at k * ldu + r
            T *v = sd + lane;
            for (int r = 0; r < nu; r++) {
                T s = v[r * kTileB];
                for (int k = 0; k < r; k++) s -= L[k * ldu + r] * v[k * kTileB];
                v[r * kTileB] = s / L[r * ldu + r];
            }
            for (int r = nu - 1; r >= 0; r--) {
                T s = v[r * kTileB];
                for (int k = r + 1; k < nu; k++) s -= L[r * ldu + k] * v[k * kTileB];
                v[r * kTileB] = s / L[r * ldu + r];
            }
        }
        __syncthreads();
        if (act)
            for (int r = warp; r < nu; r += kTileWarps) DD[ix((long)i * nu + r, B, b)] = dv[r * kTileB + lane];
        // phase 3
        if (stage > 0) {
            for (int jj = 0; jj < nc; jj++)
                gemv(acc, mAPB(jj), nx, nu, sxw, [&](int k) { return dv[k * kTileB + lane]; });
            gemv(acc, sKt, nx, nu, sxw, [&](int k) { return dv[k * kTileB + lane] - su[k * kTileB + lane]; });
            if (act) {
#pragma unroll
                for (int q = 0; q < kMaxTasks; q++) {
                    const int r0 = (sxw + q * kTileWarps) * kRT;
#pragma unroll
                    for (int t = 0; t < kRT; t++) {
                        const int r = r0 + t;
                        if (r < nx) Q[ix((long)i * nx + r, B, b)] = acc[q][t] - sx[r * kTileB + lane];
                    }
                }
            }
        }
        };
        if (isLive(tile)) tileBody();
        __syncthreads();  // sd and this tile's rows are reused by the next tile
        if (!dbl && tile + 1 < t1) prefetch(tile + 1);
    }
}

// ------------------------------------------------------------------------------------------
// Dynamics projection, one stage of the forward rollout (dynamics.cuh:143-173), writing the
// candidate (x, u) and its residual Z - cand.  Tiles as in k_dyn_back_b.  Both products,
// u = K x + d and x+ = [A B][x; u] (+ e), are Dot2-compensated in FP32: the rollout is ten
// stages deep, and plain float accumulation there leaves errors (~1e-6 relative) that change
// from one T evaluation to the next and spoil the residual differences Anderson and the
// SuperMann tests compare.
// Work split per tile: the u blocks (U of them) go to warps 0..U-1; the children's x blocks
// (X per child) are dealt to the register slots after them.  Children whose blocks fit in that
// first deal accumulate A_j x while u is being formed, and add B_j u after the barrier; any
// further children (wide trees with large states) follow one at a time.
// ------------------------------------------------------------------------------------------
template <typename T, bool GM>
__global__ void __launch_bounds__(kTileB *kTileWarps, 2) k_dyn_fwd_b(const DevProblem<T> P, const Dims D, const PadMats<T> M,
                                                                 T *__restrict__ cand, const T *__restrict__ DD,
                                                                 const T *__restrict__ x0s, int stageFrom,
                                                                 const T *__restrict__ Z, T *__restrict__ R,
                                                                 int tilesPerCta, int dbl, const int *live) {
    extern __shared__ __align__(16) unsigned char smraw[];
    T *sm = reinterpret_cast<T *>(smraw);
    const int B = D.B, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int i = stageFrom + blockIdx.y;
    const int nx = D.nx, nu = D.nu, nxu = D.nxu;
    const int c0 = P.chFrom[i], nc = P.numCh[i];
    const int ldx = pad16(nx), ldu = pad16(nu);
    const int U = tasksOf(nu), X = tasksOf(nx);
    // children overlapped with u (their blocks take the slots U .. U + G X - 1 of 8 kMaxTasks)
    const int G = min(nc, max(0, (kTileWarps * kMaxTasks - U) / X));
    const int nZ = nu + nc * nx + (i == 0 ? nx : 0);      // Z of [u_i][x_children][x_0]
    const int bufElems = (nxu + nu + nZ) * kTileB;         // one tile's [x_i u_i], d_i and Z rows
    constexpr bool gm = GM;  // matrices read in place instead of staged
    T *sKS = sm, *sABS = sKS + ldu * nx, *sBuf = gm ? sm : sABS + nc * ldx * nxu;
    const T *sK = gm ? M.K + (size_t)i * ldu * nx : sKS, *sAB = gm ? M.AB + (size_t)c0 * ldx * nxu : sABS;
    if (!gm) {
        stageMat(sKS, M.K + (size_t)i * ldu * nx, ldu * nx);
        for (int jj = 0; jj < nc; jj++) stageMat(sABS + jj * ldx * nxu, M.AB + (size_t)(c0 + jj) * ldx * nxu, ldx * nxu);
    }
    const int nTiles = (B + kTileB - 1) / kTileB;
    const int t0 = blockIdx.x * tilesPerCta, t1 = min(t0 + tilesPerCta, nTiles);
    auto isLive = [&](int t) { return !live || live[t] != 0; };
    {  // nothing to do when every instance of this CTA's tiles has stopped
        bool any = false;
        for (int t = t0; t < t1; t++) any = any || isLive(t);
        if (!any) return;
    }
    auto prefetch = [&](int t) {
        if (!isLive(t)) return;
        T *sxu = sBuf + (dbl ? ((t - t0) & 1) * bufElems : 0), *sdd = sxu + nxu * kTileB, *sz = sdd + nu * kTileB;
        const int bb = t * kTileB;
        if (i == 0) gather(sxu, nx, x0s, B, bb, lane, warp, [&](int r) { return (long)r; });
        else gather(sxu, nx, (const T *)cand, B, bb, lane, warp, [&](int r) { return D.oX + (long)i * nx + r; });
        gather(sdd, nu, DD, B, bb, lane, warp, [&](int r) { return (long)i * nu + r; });
        if (R)
            gather(sz, nZ, Z, B, bb, lane, warp, [&](int r) -> long {
                if (r < nu) return (long)i * nu + r;
                if (r < nu + nc * nx) return D.oX + (long)c0 * nx + (r - nu);
                return D.oX + (r - nu - nc * nx);
            });
    };
    if (t0 < t1) prefetch(t0);
    cpAsyncCommit();
    for (int tile = t0; tile < t1; tile++) {
        if (dbl && tile + 1 < t1) prefetch(tile + 1);
        cpAsyncCommit();
        cpAsyncWaitPrev(dbl);
        __syncthreads();
        T *sxu = sBuf + (dbl ? ((tile - t0) & 1) * bufElems : 0), *sdd = sxu + nxu * kTileB, *sz = sdd + nu * kTileB;
        const int b = tile * kTileB + lane;
        const bool act = b < B;
        auto tileBody = [&]() {
        if (i == 0 && act)
            for (int r = warp; r < nx; r += kTileWarps) {
                const T x = sxu[r * kTileB + lane];
                cand[ix(D.oX + r, B, b)] = x;
                if (R) R[ix(D.oX + r, B, b)] = sz[(nu + nc * nx + r) * kTileB + lane] - x;
            }
        T acc[kMaxTasks][kRT], cmp[kMaxTasks][kRT];  // Dot2 sums (gemvc): the rollout is compensated
        zeroAcc(acc);
        zeroAcc(cmp);
        // register slot q of this warp holds block (warp + 8 q) of the deal: u blocks first, then
        // the overlapped children's x blocks
        auto childOf = [&](int q, int &jj, int &task) {
            const int ct = warp + q * kTileWarps - U;
            if (ct < 0 || ct >= G * X) return false;
            jj = ct / X;
            task = ct % X;
            return true;
        };
        // phase 1: u = K x + d on the u blocks' warps; A_j x of the overlapped children
#pragma unroll
        for (int q = 0; q < kMaxTasks; q++) {
            const int blk = warp + q * kTileWarps;
            if (blk < U) {
                gemvcTask(acc[q], cmp[q], sK, nu, nx, blk, [&](int k) { return sxu[k * kTileB + lane]; });
#pragma unroll
                for (int t = 0; t < kRT; t++) {
                    const int r = blk * kRT + t;
                    if (r < nu) {
                        const T u = finishc(acc[q][t], cmp[q][t], sdd[r * kTileB + lane]);
                        sxu[(nx + r) * kTileB + lane] = u;
                        if (act) {
                            cand[ix((long)i * nu + r, B, b)] = u;
                            if (R) R[ix((long)i * nu + r, B, b)] = sz[r * kTileB + lane] - u;
                        }
                    }
                }
                continue;
            }
            int jj, task;
            if (childOf(q, jj, task))
                gemvcTask(acc[q], cmp[q], sAB + jj * ldx * nxu, nx, nx, task, [&](int k) { return sxu[k * kTileB + lane]; });
        }
        __syncthreads();  // u is complete before the children read it
        // phase 2: + B_j u, then x_j = (sum) + e_j for the overlapped children
#pragma unroll
        for (int q = 0; q < kMaxTasks; q++) {
            int jj, task;
            if (!childOf(q, jj, task)) continue;
            gemvcTask(acc[q], cmp[q], sAB + jj * ldx * nxu + (size_t)nx * ldx, nx, nu, task,
                      [&](int k) { return sxu[(nx + k) * kTileB + lane]; });
            if (!act) continue;
            const int j = c0 + jj;
#pragma unroll
            for (int t = 0; t < kRT; t++) {
                const int r = task * kRT + t;
                if (r < nx) {
                    const T x = finishc(acc[q][t], cmp[q][t], D.affine ? P.e[(size_t)j * nx + r] : T(0));
                    cand[ix(D.oX + (long)j * nx + r, B, b)] = x;
                    if (R) R[ix(D.oX + (long)j * nx + r, B, b)] = sz[(nu + jj * nx + r) * kTileB + lane] - x;
                }
            }
        }
        // the remaining children, one at a time over all warps
        for (int jj = G; jj < nc; jj++) {
            const int j = c0 + jj;
            zeroAcc(acc);
            zeroAcc(cmp);
            const int slot = slotFrom(warp, jj * X);  // children's blocks on different warps
            gemvc(acc, cmp, sAB + jj * ldx * nxu, nx, nxu, slot, [&](int k) { return sxu[k * kTileB + lane]; });
            if (!act) continue;
#pragma unroll
            for (int q = 0; q < kMaxTasks; q++) {
                const int r0 = (slot + q * kTileWarps) * kRT;
#pragma unroll
                for (int t = 0; t < kRT; t++) {
                    const int r = r0 + t;
                    if (r < nx) {
                        const T x = finishc(acc[q][t], cmp[q][t], D.affine ? P.e[(size_t)j * nx + r] : T(0));
                        cand[ix(D.oX + (long)j * nx + r, B, b)] = x;
                        if (R) R[ix(D.oX + (long)j * nx + r, B, b)] = sz[(nu + jj * nx + r) * kTileB + lane] - x;
                    }
                }
            }
        }
        };
        if (isLive(tile)) tileBody();
        __syncthreads();  // this tile's rows are reused by the next tile
        if (!dbl && tile + 1 < t1) prefetch(tile + 1);
    }
}

}  // namespace spock

namespace spock {

// Host-side launchers of the two largest kernels.  Each (kernel, precision, mode) is compiled in
// a translation unit of its own (ops_batch.cu, built once per combination), so their device
// code compiles in parallel; the engine calls these instead of launching the kernels itself.
// GM: the variant that reads node matrices in place (problems whose matrices exceed shared memory).
template <typename T, int MODE, bool GM>
void launchLstarB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                  const PadMats<T> &M, int tilesPerCta, int dbl);
template <typename T, int MODE, bool GM>
void launchLopB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                const PadMats<T> &M, int tilesPerCta, int dbl);
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) of the same kernels.
template <typename T, int MODE, bool GM>
cudaError_t optInLstarB(int bytes);
template <typename T, int MODE, bool GM>
cudaError_t optInLopB(int bytes);

}  // namespace spock
