// Offline cache of the dynamics projection and the AVaR nullspace projectors, computed on the
// GPU in FP64.
//
// The reference builds it in numpy when it generates a problem (problem.py:192-213), from the
// leaves to the root: with P_j = I at the leaves, for every nonleaf node i and its children j
//   R_i   = I + sum_j B_j' P_j B_j            (nu x nu), lower Cholesky factor L_i
//   K_i   = -R_i^{-1} sum_j B_j' P_j A_j      (nu x nx)
//   Abk_j = A_j + B_j K_i,  ABKTr_j = Abk_j',  APB_j = Abk_j' P_j B_j
//   P_i   = I + K_i' K_i + sum_j Abk_j' P_j Abk_j.
// Here one launch per stage (children before parents) runs one CTA per nonleaf node of the
// stage; every product is a loop of FP64 dot products spread over the CTA's threads, with the
// node's intermediates in a global scratch area (any nx, nu).  All matrices are column-major
// per node, the layout of the .bt files the problem loader reads.
//
// The AVaR kernel projection reads, for every nonleaf node i with m children, the orthogonal
// projector onto ker S_i of the padded matrix S_i = [E_i' -I -I] (problem.py:215-231, 263-267,
// with E = [alpha I; -I; 1'] from build.py:1184-1193): row j of S_i (m x (4E+1)) holds alpha in
// column j, -1 in column m + j, 1 in column 2m, -1 in columns 2E+1+j and 3E+1+j.  The reference
// takes an SVD nullspace basis N and stores N N'; the same projector is I - S'(SS')^-1 S, which
// one CTA per node forms here with a Cholesky factor of the m x m Gram matrix.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <string>
#include <vector>

#include "offline.hpp"

namespace spock {

namespace {

#define OCK(x)                                                                                     \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + \
                                     __FILE__ + ":" + std::to_string(__LINE__));                   \
    } while (0)

struct OfflineArgs {
    const double *AB;     // nx x (nx + nu) per node: [A_j B_j]
    const long *chFrom, *numCh;
    double *P, *K, *L, *ABKTr, *APB;
    double *scratch;      // per CTA: R (nu^2), S (nu nx), BtP (nu nx), Abk (nx^2), T (nx^2), PB (nx nu)
    int nx, nu, stageFrom, ok;
    int *fail;            // set when a Cholesky pivot is not positive
};

// C (R x C, column-major) op= sum_k X(r, k) Y(k, c), X given by element functors.
template <typename FX, typename FY, typename FOut>
__device__ void matmul(int R, int C, int Kd, FX x, FY y, FOut out) {
    for (int e = threadIdx.x; e < R * C; e += blockDim.x) {
        const int r = e % R, c = e / R;
        double s = 0;
        for (int k = 0; k < Kd; k++) s += x(r, k) * y(k, c);
        out(r, c, s);
    }
}

__global__ void k_offline_stage(const OfflineArgs a) {
    const int i = a.stageFrom + blockIdx.x;
    const int nx = a.nx, nu = a.nu, nxu = nx + nu;
    const long c0 = a.chFrom[i], nc = a.numCh[i];
    const size_t per = (size_t)nu * nu + 2 * (size_t)nu * nx + 2 * (size_t)nx * nx + (size_t)nx * nu;
    double *R = a.scratch + blockIdx.x * per, *S = R + nu * nu, *BtP = S + nu * nx, *Abk = BtP + nu * nx;
    double *Tm = Abk + nx * nx, *PB = Tm + nx * nx;
    double *Pi = a.P + (size_t)i * nx * nx, *Ki = a.K + (size_t)i * nu * nx, *Li = a.L + (size_t)i * nu * nu;
    for (int e = threadIdx.x; e < nu * nu; e += blockDim.x) R[e] = (e % nu == e / nu) ? 1. : 0.;
    for (int e = threadIdx.x; e < nu * nx; e += blockDim.x) S[e] = 0.;
    __syncthreads();
    for (long j = c0; j < c0 + nc; j++) {
        const double *ABj = a.AB + (size_t)j * nx * nxu, *Pj = a.P + (size_t)j * nx * nx;
        auto A = [&](int r, int c) { return ABj[c * nx + r]; };
        auto Bm = [&](int r, int c) { return ABj[(nx + c) * nx + r]; };
        // BtP = B_j' P_j
        matmul(nu, nx, nx, [&](int r, int k) { return Bm(k, r); }, [&](int k, int c) { return Pj[c * nx + k]; },
               [&](int r, int c, double s) { BtP[c * nu + r] = s; });
        __syncthreads();
        matmul(nu, nu, nx, [&](int r, int k) { return BtP[k * nu + r]; }, Bm,
               [&](int r, int c, double s) { R[c * nu + r] += s; });
        matmul(nu, nx, nx, [&](int r, int k) { return BtP[k * nu + r]; }, A,
               [&](int r, int c, double s) { S[c * nu + r] += s; });
        __syncthreads();
    }
    // lower Cholesky factor of R (one thread; nu is small) into L_i
    if (threadIdx.x == 0) {
        for (int e = 0; e < nu * nu; e++) Li[e] = 0.;
        for (int c = 0; c < nu; c++) {
            double d = R[c * nu + c];
            for (int k = 0; k < c; k++) d -= Li[k * nu + c] * Li[k * nu + c];
            if (!(d > 0.)) {
                *a.fail = 1;
                d = 1.;
            }
            d = sqrt(d);
            Li[c * nu + c] = d;
            for (int r = c + 1; r < nu; r++) {
                double s = R[c * nu + r];
                for (int k = 0; k < c; k++) s -= Li[k * nu + r] * Li[k * nu + c];
                Li[c * nu + r] = s / d;
            }
        }
    }
    __syncthreads();
    // K_i = -R^{-1} S: one column per thread, forward then backward substitution with L_i
    for (int c = threadIdx.x; c < nx; c += blockDim.x) {
        double *k = Ki + (size_t)c * nu;
        for (int r = 0; r < nu; r++) {
            double s = -S[c * nu + r];
            for (int q = 0; q < r; q++) s -= Li[q * nu + r] * k[q];
            k[r] = s / Li[r * nu + r];
        }
        for (int r = nu - 1; r >= 0; r--) {
            double s = k[r];
            for (int q = r + 1; q < nu; q++) s -= Li[r * nu + q] * k[q];
            k[r] = s / Li[r * nu + r];
        }
    }
    __syncthreads();
    // P_i = I + K'K, then the children's terms
    matmul(nx, nx, nu, [&](int r, int q) { return Ki[r * nu + q]; }, [&](int q, int c) { return Ki[c * nu + q]; },
           [&](int r, int c, double s) { Pi[c * nx + r] = s + (r == c ? 1. : 0.); });
    __syncthreads();
    for (long j = c0; j < c0 + nc; j++) {
        const double *ABj = a.AB + (size_t)j * nx * nxu, *Pj = a.P + (size_t)j * nx * nx;
        auto Bm = [&](int r, int c) { return ABj[(nx + c) * nx + r]; };
        // Abk = A_j + B_j K_i
        matmul(nx, nx, nu, Bm, [&](int q, int c) { return Ki[c * nu + q]; },
               [&](int r, int c, double s) { Abk[c * nx + r] = ABj[c * nx + r] + s; });
        // PB = P_j B_j
        matmul(nx, nu, nx, [&](int r, int k) { return Pj[k * nx + r]; }, Bm,
               [&](int r, int c, double s) { PB[c * nx + r] = s; });
        __syncthreads();
        double *ABKTrj = a.ABKTr + (size_t)j * nx * nx, *APBj = a.APB + (size_t)j * nx * nu;
        for (int e = threadIdx.x; e < nx * nx; e += blockDim.x) {
            const int r = e % nx, c = e / nx;
            ABKTrj[c * nx + r] = Abk[r * nx + c];
        }
        // APB_j = Abk' (P_j B_j);  T = P_j Abk
        matmul(nx, nu, nx, [&](int r, int k) { return Abk[r * nx + k]; }, [&](int k, int c) { return PB[c * nx + k]; },
               [&](int r, int c, double s) { APBj[c * nx + r] = s; });
        matmul(nx, nx, nx, [&](int r, int k) { return Pj[k * nx + r]; }, [&](int k, int c) { return Abk[c * nx + k]; },
               [&](int r, int c, double s) { Tm[c * nx + r] = s; });
        __syncthreads();
        // P_i += Abk' T
        matmul(nx, nx, nx, [&](int r, int k) { return Abk[r * nx + k]; }, [&](int k, int c) { return Tm[c * nx + k]; },
               [&](int r, int c, double s) { Pi[c * nx + r] += s; });
        __syncthreads();
    }
}

// One CTA per nonleaf node; shared memory S (m x nd, row-major), the Gram factor (m x m) and
// W = (SS')^-1 S (m x nd), with m <= E.
__global__ void k_offline_nullspace(const long *numCh, int E, int nd, double alpha, double *NNtr, int *fail) {
    extern __shared__ double sh[];
    const int i = blockIdx.x, m = (int)numCh[i], yd = 2 * E + 1;
    double *S = sh, *G = S + (size_t)E * nd, *W = G + (size_t)E * E;
    for (int e = threadIdx.x; e < m * nd; e += blockDim.x) S[e] = 0.;
    __syncthreads();
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
        S[j * nd + j] = alpha;
        S[j * nd + m + j] = -1.;
        S[j * nd + 2 * m] = 1.;
        S[j * nd + yd + j] = -1.;
        S[j * nd + yd + E + j] = -1.;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < m * m; e += blockDim.x) {  // G = S S'
        const int r = e % m, c = e / m;
        double s = 0.;
        for (int k = 0; k < nd; k++) s += S[r * nd + k] * S[c * nd + k];
        G[c * m + r] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // lower Cholesky factor in place (column-major, lower triangle)
        for (int c = 0; c < m; c++) {
            double d = G[c * m + c];
            for (int k = 0; k < c; k++) d -= G[k * m + c] * G[k * m + c];
            if (!(d > 0.)) {
                *fail = 1;
                d = 1.;
            }
            d = sqrt(d);
            G[c * m + c] = d;
            for (int r = c + 1; r < m; r++) {
                double s = G[c * m + r];
                for (int k = 0; k < c; k++) s -= G[k * m + r] * G[k * m + c];
                G[c * m + r] = s / d;
            }
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < nd; c += blockDim.x) {  // W(:, c) = G^-1 S(:, c)
        for (int r = 0; r < m; r++) {
            double s = S[r * nd + c];
            for (int q = 0; q < r; q++) s -= G[q * m + r] * W[q * nd + c];
            W[r * nd + c] = s / G[r * m + r];
        }
        for (int r = m - 1; r >= 0; r--) {
            double s = W[r * nd + c];
            for (int q = r + 1; q < m; q++) s -= G[r * m + q] * W[q * nd + c];
            W[r * nd + c] = s / G[r * m + r];
        }
    }
    __syncthreads();
    double *out = NNtr + (size_t)i * nd * nd;
    for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {  // I - S' W, column-major
        const int r = e % nd, c = e / nd;
        double s = r == c ? 1. : 0.;
        for (int j = 0; j < m; j++) s -= S[j * nd + r] * W[j * nd + c];
        out[e] = s;
    }
}

template <typename V>
double *upload(const V &v) {
    double *d = nullptr;
    OCK(cudaMalloc(&d, sizeof(double) * (v.size() ? v.size() : 1)));
    if (!v.empty()) OCK(cudaMemcpy(d, v.data(), sizeof(double) * v.size(), cudaMemcpyHostToDevice));
    return d;
}

}  // namespace

OfflineCache offlineDynamicsGpu(const HostProblem &p, int device) {
    OCK(cudaSetDevice(device));
    const long n = p.numNodes, nnl = p.numNonleaf, nx = p.nx, nu = p.nu;
    std::vector<double> P0((size_t)nx * nx * n, 0.);
    for (long j = nnl; j < n; j++)
        for (long r = 0; r < nx; r++) P0[(size_t)j * nx * nx + r * nx + r] = 1.;  // leaves: P = I
    std::vector<long> chFrom(p.childFrom.begin(), p.childFrom.end()), numCh(p.numChildren.begin(), p.numChildren.end());
    long *dCh = nullptr, *dNum = nullptr;
    int *dFail = nullptr;
    OCK(cudaMalloc(&dCh, sizeof(long) * chFrom.size()));
    OCK(cudaMalloc(&dNum, sizeof(long) * numCh.size()));
    OCK(cudaMemcpy(dCh, chFrom.data(), sizeof(long) * chFrom.size(), cudaMemcpyHostToDevice));
    OCK(cudaMemcpy(dNum, numCh.data(), sizeof(long) * numCh.size(), cudaMemcpyHostToDevice));
    OCK(cudaMalloc(&dFail, sizeof(int)));
    OCK(cudaMemset(dFail, 0, sizeof(int)));
    OfflineArgs a{};
    a.AB = upload(p.AB);
    a.chFrom = dCh;
    a.numCh = dNum;
    a.P = upload(P0);
    a.K = upload(std::vector<double>((size_t)nu * nx * nnl, 0.));
    a.L = upload(std::vector<double>((size_t)nu * nu * nnl, 0.));
    a.ABKTr = upload(std::vector<double>((size_t)nx * nx * n, 0.));
    a.APB = upload(std::vector<double>((size_t)nx * nu * n, 0.));
    long maxStage = 0;
    for (long s = 0; s < p.numStages; s++) maxStage = std::max(maxStage, p.stageTo[s] - p.stageFrom[s] + 1);
    const size_t per = (size_t)nu * nu + 2 * (size_t)nu * nx + 2 * (size_t)nx * nx + (size_t)nx * nu;
    OCK(cudaMalloc(&a.scratch, sizeof(double) * per * (size_t)maxStage));
    a.nx = (int)nx;
    a.nu = (int)nu;
    a.fail = dFail;
    for (long s = p.numStages - 2; s >= 0; s--) {  // nonleaf stages, children first
        const long from = p.stageFrom[s], to = p.stageTo[s];
        if (from >= nnl) continue;
        a.stageFrom = (int)from;
        k_offline_stage<<<(unsigned)(std::min(to, nnl - 1) - from + 1), 256>>>(a);
        OCK(cudaGetLastError());
    }
    OCK(cudaDeviceSynchronize());
    int fail = 0;
    OCK(cudaMemcpy(&fail, dFail, sizeof(int), cudaMemcpyDeviceToHost));
    OfflineCache out;
    auto down = [&](const double *d, size_t count, std::vector<double> &h) {
        h.resize(count);
        OCK(cudaMemcpy(h.data(), d, sizeof(double) * count, cudaMemcpyDeviceToHost));
    };
    down(a.P, (size_t)nx * nx * n, out.P);
    down(a.K, (size_t)nu * nx * nnl, out.K);
    down(a.L, (size_t)nu * nu * nnl, out.lowChol);
    down(a.ABKTr, (size_t)nx * nx * n, out.ABKTr);
    down(a.APB, (size_t)nx * nu * n, out.APB);
    for (void *ptr : {(void *)a.AB, (void *)dCh, (void *)dNum, (void *)a.P, (void *)a.K, (void *)a.L, (void *)a.ABKTr,
                      (void *)a.APB, (void *)a.scratch, (void *)dFail})
        cudaFree(ptr);
    if (fail) throw std::invalid_argument("[offlineDynamics] I + sum B'PB is not positive definite");
    return out;
}

std::vector<double> offlineNullspaceGpu(const HostProblem &p, int device) {
    const int E = (int)p.numEvents, nd = (int)p.nullDim;
    const long nnl = p.numNonleaf;
    if (nd != 4 * E + 1) throw std::invalid_argument("[offlineNullspace] rowsNNtr must be 4 numEvents + 1");
    const size_t smem = sizeof(double) * (2 * (size_t)E * nd + (size_t)E * E);
    if (smem > 200 * 1024) throw std::invalid_argument("[offlineNullspace] too many events for one CTA");
    OCK(cudaSetDevice(device));
    OCK(cudaFuncSetAttribute(k_offline_nullspace, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    std::vector<long> numCh(p.numChildren.begin(), p.numChildren.end());
    long *dNum = nullptr;
    double *dOut = nullptr;
    int *dFail = nullptr;
    OCK(cudaMalloc(&dNum, sizeof(long) * numCh.size()));
    OCK(cudaMalloc(&dOut, sizeof(double) * (size_t)nd * nd * nnl));
    OCK(cudaMalloc(&dFail, sizeof(int)));
    OCK(cudaMemcpy(dNum, numCh.data(), sizeof(long) * numCh.size(), cudaMemcpyHostToDevice));
    OCK(cudaMemset(dFail, 0, sizeof(int)));
    k_offline_nullspace<<<(unsigned)nnl, 128, smem>>>(dNum, E, nd, p.alpha, dOut, dFail);
    OCK(cudaGetLastError());
    OCK(cudaDeviceSynchronize());
    std::vector<double> out((size_t)nd * nd * nnl);
    int fail = 0;
    OCK(cudaMemcpy(out.data(), dOut, sizeof(double) * out.size(), cudaMemcpyDeviceToHost));
    OCK(cudaMemcpy(&fail, dFail, sizeof(int), cudaMemcpyDeviceToHost));
    for (void *ptr : {(void *)dNum, (void *)dOut, (void *)dFail}) cudaFree(ptr);
    if (fail) throw std::invalid_argument("[offlineNullspace] S S' is not positive definite");
    return out;
}

}  // namespace spock
