// The `count` smallest singular values of a batch of matrices, with their first
// and second k-derivatives (arnoldi::sv / sv_1st_der / sv_2nd_der,
// include/singular_values_arnoldi.hpp:29-66, source/utilities/singular_values_arnoldi.cpp:19-246).
//
// The reference hands ARPACK the Hermitian operator M = [0 T^-H; T^-1 0] of order
// 2n (eigenvalues +-1/sigma_j) through one LU of T, asks for the 2 count eigenvalues
// of largest magnitude to relative residual acc, and returns sigma_j = |1 / theta|
// in ascending order.  The same eigenpairs come here from a block subspace
// iteration on T^-1 T^-H (M^2 restricted to the v half) with one Rayleigh-Ritz
// step per iteration, all matrices of the batch in lock step:
//   Q = qr(T^-1 R)                              R: p seeded columns, p <= 32
//   repeat  T^-H Q = QB RB,  RB = Z S W^H       S = diag(s_1 >= s_2 >= ...)
//           Ritz pairs of M: theta_j = s_j, x_j = (QB z_j; Q w_j) / sqrt2, and
//           M x_j - theta_j x_j = (0; T^-1 QB z_j - s_j Q w_j) / sqrt2
//           stop when |T^-1 QB z_j - s_j Q w_j| <= sqrt2 tol s_j for all j < count
//           (ARPACK's test |r| <= tol |theta|), else Q = qr(T^-1 QB)
//   sigma_j = 1 / s_j,  v_j = Q w_j.
// The Ritz values converge like (sigma_j / sigma_{p+1})^(4 it).  RB's singular
// pairs come from one-sided Jacobi on one warp (the columns of RB W are s_j z_j).
// sigma' = Re u^H T' v with u = T v / |T v| (the x^H W' x of
// singular_values_arnoldi.cpp:110-126) and sigma'' from the bordered 2n x 2n system
// of singular_values_arnoldi.cpp:183-244; both shared with the randomized path
// (rsvd.cu) through sv_der_from_vectors.
#include <algorithm>
#include <cmath>
#include <vector>

#include "hbem_device.cuh"
#include "smem_linalg.cuh"

namespace hbem {

constexpr int kArnThreads = 256;
constexpr int kArnMaxP = 32;

struct Sv2Work {
    cplx *B = nullptr, *ub = nullptr, *ud = nullptr, *rhs = nullptr, *tb = nullptr;
    int *piv2 = nullptr, *perm2 = nullptr, *info2 = nullptr, *mcol = nullptr;
};
cudaError_t sv_der_from_vectors(int n, int nvec, int per, int D, const cplx* T, long long mat_stride,
                                long long der_stride, double* out, cplx* uv, const Sv2Work& w, cudaStream_t st,
                                long long& nl);
size_t sv2_carve(int n, int nvec, int D, char* base, Sv2Work& w);
cudaError_t qr_global_batched(int n, int nmat, int s, cplx* X, long long xstride, cplx* Rf, cudaStream_t st);
cudaError_t copy_mats_batched(long long nn, int nmat, const cplx* src, long long sstride, cplx* dst,
                              long long dstride, cudaStream_t st);
cudaError_t lu_factor_batched(int n, int nmat, cplx* A, long long stride, int* piv, int* perm, int* info,
                              cudaStream_t st, long long* launches);
cudaError_t lu_solve_batched(int n, int nmat, int trans, const cplx* LU, long long stride, const int* perm, int s,
                             cplx* X, long long xstride, cudaStream_t st);
bool lu_solve_supported(int n);

// Start block entry (r, c): real and imaginary parts uniform in [-1/2, 1/2) from a
// SplitMix64 hash of (seed, r, c); the same block for every matrix of a batch.
static __device__ __forceinline__ cplx arn_start(unsigned long long seed, int r, int c) {
    unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (1ull + ((unsigned long long)c << 32 | (unsigned)r));
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    const double re = (double)(z >> 40) * (1.0 / 16777216.0) - 0.5;
    const double im = (double)(z & 0xffffffull) * (1.0 / 16777216.0) - 0.5;
    return mk(re, im);
}

struct ArnJob {
    int n, nmat, p, count, maxit;
    double tol;
    unsigned long long seed;
    const cplx* T;
    long long mat_stride;
    double* out;      // sigma_j of matrix m at out[os (m count + j)]
    int os;
    cplx* uv;         // optional [nmat count][2n]: v_j into the second half
    int* status;      // [nmat]: 0 converged, 5 zero pivot, 6 iteration limit
    int* iters;       // [nmat]
};

// Ritz step: Jacobi on the p x p factor Rs (in place: columns s_j z_j), W its right
// vectors; nrm[j] = s_j^2; ord[0..count) = columns by decreasing s_j.  With flag
// (a shared int) the Jacobi runs on the whole CTA (jacobi_cta), else on warp 0.
static __device__ void arn_ritz(cplx* Rs, cplx* W, int p, int count, double* nrm, int* ord, int* flag = nullptr) {
    if (flag) jacobi_cta(Rs, p, W, flag);
    if (threadIdx.x < 32) {
        if (!flag) jacobi_warp(Rs, p, W);
        const int lane = threadIdx.x;
        if (lane < p) {
            double a = 0.;
            for (int r = 0; r < p; ++r) a += norm2(Rs[lane * p + r]);
            nrm[lane] = a;
        }
        __syncwarp();
        if (lane == 0)
            for (int j = 0; j < count; ++j) {
                int best = -1;
                for (int c = 0; c < p; ++c) {
                    bool taken = false;
                    for (int i = 0; i < j; ++i) taken |= ord[i] == c;
                    if (!taken && (best < 0 || nrm[c] > nrm[best])) best = c;
                }
                ord[j] = best;
            }
    }
    __syncthreads();
}

// |Y Rs[:, o] - s_o^2 X W[:, o]|^2 <= 2 tol^2 s_o^4 for the count leading Ritz pairs
// (the residual of the unit Ritz vector scaled by s_o); Y = T^-1 QB, X = Q.
static __device__ bool arn_converged(const cplx* X, const cplx* Y, int n, int p, const cplx* Rs, const cplx* W,
                                     const double* nrm, const int* ord, int count, double tol, double* red) {
    bool conv = true;
    for (int j = 0; j < count; ++j) {
        const int o = ord[j];
        const double s2 = nrm[o];
        double part = 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            cplx a = mk(0.), b = mk(0.);
            for (int c = 0; c < p; ++c) {
                cfma(a, Y[r + (long long)c * n], Rs[c + o * p]);
                cfma(b, X[r + (long long)c * n], W[c + o * p]);
            }
            part += norm2(a - s2 * b);
        }
        const double tot = bsum(part, red + 32 * (j & 1));
        conv &= tot <= 2. * tol * tol * s2 * s2;
    }
    return conv;
}

// sigma_j = 1 / s_j and v_j = X W[:, ord j] of the finished iteration
static __device__ void arn_write(const ArnJob& J, int mat, const cplx* X, const cplx* W, const double* nrm,
                                 const int* ord) {
    const int n = J.n, p = J.p;
    for (int j = threadIdx.x; j < J.count; j += blockDim.x) {
        const double s2 = nrm[ord[j]];
        J.out[(long long)J.os * ((long long)mat * J.count + j)] = s2 > 0. ? 1. / sqrt(s2) : CUDART_INF;
    }
    if (J.uv)
        for (int j = 0; j < J.count; ++j) {
            const int o = ord[j];
            cplx* v = J.uv + 2LL * n * ((long long)mat * J.count + j) + n;
            for (int r = threadIdx.x; r < n; r += blockDim.x) {
                cplx b = mk(0.);
                for (int c = 0; c < p; ++c) cfma(b, X[r + (long long)c * n], W[c + o * p]);
                v[r] = b;
            }
        }
}

static __device__ void arn_fail(const ArnJob& J, int mat, int code) {
    for (int j = threadIdx.x; j < J.count; j += blockDim.x)
        J.out[(long long)J.os * ((long long)mat * J.count + j)] = CUDART_NAN;
    if (J.uv)
        for (long long e = threadIdx.x; e < 2LL * J.n * J.count; e += blockDim.x)
            J.uv[2LL * J.n * J.count * mat + e] = mk(0.);
    if (threadIdx.x == 0) {
        J.status[mat] = code;
        J.iters[mat] = 0;
    }
}

// ------------------------------------------------------------------ one CTA per matrix

size_t arn_smem_bytes(int n, int p) {
    return ((size_t)n * n + 2 * (size_t)n * p + 2 * (size_t)p * p + kArnMaxP + n) * sizeof(cplx) +
           (128 + kArnMaxP) * sizeof(double) + (2 * (size_t)n + kArnMaxP + 32) * sizeof(int);
}

__global__ void __launch_bounds__(kArnThreads) k_arn_small(ArnJob J) {
    extern __shared__ double smraw[];
    const int n = J.n, p = J.p, mat = blockIdx.x;
    cplx* A = reinterpret_cast<cplx*>(smraw);        // n x n: T, then its LU
    cplx* X = A + (long long)n * n;                  // n x p: Q
    cplx* Y = X + (long long)n * p;                  // n x p: QB, then T^-1 QB
    cplx* Rs = Y + (long long)n * p;                 // p x p
    cplx* W = Rs + p * p;                            // p x p
    cplx* coef = W + p * p;                          // kArnMaxP
    cplx* buf = coef + kArnMaxP;                     // n
    double* red = reinterpret_cast<double*>(buf + n);   // 128
    double* nrm = red + 128;                         // kArnMaxP
    int* piv = reinterpret_cast<int*>(nrm + kArnMaxP);  // n
    int* perm = piv + n;                             // n
    int* ord = perm + n;                             // kArnMaxP
    __shared__ int s_sing, s_rot;
    if (threadIdx.x == 0) s_sing = 0;
    const cplx* T0 = J.T + (long long)mat * J.mat_stride;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = T0[e];
    for (int e = threadIdx.x; e < n * p; e += blockDim.x) X[e] = arn_start(J.seed, e % n, e / n);
    __syncthreads();
    lu_smem(A, n, piv, &s_sing, buf);
    __syncthreads();
    if (s_sing) {
        arn_fail(J, mat, 5);
        return;
    }
    perm_from_piv(piv, n, perm);
    // U's diagonal replaced by its reciprocals: the solves multiply
    for (int k = threadIdx.x; k < n; k += blockDim.x) A[k + (long long)k * n] = cdiv(mk(1.), A[k + (long long)k * n]);
    __syncthreads();
    solve_lu_blk(A, perm, n, X, p, buf, nullptr, true);
    qr_cgs2(X, n, p, coef, red);
    int it = 1;
    bool conv = false;
    for (;; ++it) {
        for (int e = threadIdx.x; e < n * p; e += blockDim.x) Y[e] = X[e];
        __syncthreads();
        solve_lu_h_blk(A, perm, n, Y, p, buf, nullptr, true);
        qr_cgs2(Y, n, p, coef, red, Rs);
        __syncthreads();
        arn_ritz(Rs, W, p, J.count, nrm, ord, &s_rot);
        solve_lu_blk(A, perm, n, Y, p, buf, nullptr, true);
        __syncthreads();
        conv = arn_converged(X, Y, n, p, Rs, W, nrm, ord, J.count, J.tol, red);
        if (conv || it >= J.maxit) break;
        qr_cgs2(Y, n, p, coef, red);
        cplx* t = X;
        X = Y;
        Y = t;
    }
    arn_write(J, mat, X, W, nrm, ord);
    if (threadIdx.x == 0) {
        J.status[mat] = conv ? 0 : 6;
        J.iters[mat] = it;
    }
}

// ------------------------------------------------------------------ matrices of any order
//
// The same iteration with the LU and the n x p blocks in global memory: the solves
// by the batched LU solves, QR by one CTA per matrix, the Ritz step and the
// convergence test by the kernels below; the host stops when every matrix is done.

__global__ void k_arn_start(int n, int p, unsigned long long seed, cplx* X, long long xs) {
    const long long len = (long long)n * p;
    cplx* Xm = X + (long long)blockIdx.y * xs;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x)
        Xm[e] = arn_start(seed, (int)(e % n), (int)(e / n));
}

// done[m] = 1 for matrices whose LU met a zero pivot (status 5, sigma NaN)
__global__ void k_arn_init(ArnJob J, const int* info, int* done, int* ndone) {
    const int mat = blockIdx.x;
    const bool sing = info[mat] != 0;
    if (sing) arn_fail(J, mat, 5);
    if (threadIdx.x == 0) {
        done[mat] = sing ? 1 : 0;
        if (sing) atomicAdd(ndone, 1);
    }
}

// Ritz step of every unfinished matrix: Rf (p x p per matrix) -> Rs in place, Wg, nrm, ord
__global__ void __launch_bounds__(32) k_arn_ritz(int p, int count, cplx* Rf, cplx* Wg, double* nrmg, int* ordg,
                                                 const int* done) {
    __shared__ cplx Rs[kArnMaxP * kArnMaxP], W[kArnMaxP * kArnMaxP];
    __shared__ double nrm[kArnMaxP];
    __shared__ int ord[kArnMaxP];
    const int mat = blockIdx.x;
    if (done[mat]) return;
    cplx* R = Rf + (long long)mat * p * p;
    for (int e = threadIdx.x; e < p * p; e += blockDim.x) Rs[e] = R[e];
    __syncwarp();
    arn_ritz(Rs, W, p, count, nrm, ord);
    for (int e = threadIdx.x; e < p * p; e += blockDim.x) {
        R[e] = Rs[e];
        Wg[(long long)mat * p * p + e] = W[e];
    }
    for (int j = threadIdx.x; j < p; j += blockDim.x) {
        nrmg[(long long)mat * kArnMaxP + j] = nrm[j];
        ordg[(long long)mat * kArnMaxP + j] = ord[j];
    }
}

// Convergence test of every unfinished matrix after Y = T^-1 QB; converged matrices
// (or all at the last iteration) write sigma, v and their status.
__global__ void __launch_bounds__(kArnThreads) k_arn_check(ArnJob J, const cplx* X, const cplx* Y, long long xs,
                                                           const cplx* Rf, const cplx* Wg, const double* nrmg,
                                                           const int* ordg, int* done, int* ndone, int it, int last) {
    __shared__ cplx Rs[kArnMaxP * kArnMaxP], W[kArnMaxP * kArnMaxP];
    __shared__ double nrm[kArnMaxP], red[128];
    __shared__ int ord[kArnMaxP];
    const int mat = blockIdx.x, p = J.p;
    if (done[mat]) return;
    for (int e = threadIdx.x; e < p * p; e += blockDim.x) {
        Rs[e] = Rf[(long long)mat * p * p + e];
        W[e] = Wg[(long long)mat * p * p + e];
    }
    for (int j = threadIdx.x; j < p; j += blockDim.x) {
        nrm[j] = nrmg[(long long)mat * kArnMaxP + j];
        ord[j] = ordg[(long long)mat * kArnMaxP + j];
    }
    __syncthreads();
    const cplx* Xm = X + (long long)mat * xs;
    const bool conv = arn_converged(Xm, Y + (long long)mat * xs, J.n, p, Rs, W, nrm, ord, J.count, J.tol, red);
    if (!conv && !last) return;
    arn_write(J, mat, Xm, W, nrm, ord);
    if (threadIdx.x == 0) {
        J.status[mat] = conv ? 0 : 6;
        J.iters[mat] = it;
        done[mat] = 1;
        atomicAdd(ndone, 1);
    }
}

#define AR_CK(x)                                \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

// ------------------------------------------------------------------ orchestration

struct ArnWork {
    cplx *A = nullptr, *X = nullptr, *Y = nullptr, *Rf = nullptr, *Wg = nullptr, *uv = nullptr;
    double* nrm = nullptr;
    int *piv = nullptr, *perm = nullptr, *info = nullptr, *ord = nullptr, *done = nullptr, *ndone = nullptr;
    int *status = nullptr, *iters = nullptr;
    Sv2Work sv2;
};

int arnoldi_block(int n, int count) { return std::min(std::min(n, kArnMaxP), std::max(12, 2 * count)); }

bool arnoldi_small_fits(int n, int p) { return arn_smem_bytes(n, p) <= 220 * 1024; }

// The block must hold the count wanted vectors plus a margin of 4 for the
// convergence ratio sigma_count / sigma_(p+1), unless it spans the whole space.
bool arnoldi_supported(int n, int count, int D) {
    const int p = arnoldi_block(n, count);
    if (count < 1 || n < 2 || count > p || (p < n && count > p - 4)) return false;
    if (!arnoldi_small_fits(n, p) && !lu_solve_supported(n)) return false;
    if (D == 2 && !lu_solve_supported(2 * n)) return false;
    return true;
}

size_t arnoldi_carve(int n, int nmat, int count, int D, char* base, ArnWork& w) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* q = base ? base + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return q;
    };
    const int p = arnoldi_block(n, count);
    const size_t nm = (size_t)nmat, c = sizeof(cplx), ii = sizeof(int);
    w.status = (int*)take(nm * ii);
    w.iters = (int*)take(nm * ii);
    if (!arnoldi_small_fits(n, p)) {
        w.A = (cplx*)take(nm * n * n * c);
        w.X = (cplx*)take(nm * n * p * c);
        w.Y = (cplx*)take(nm * n * p * c);
        w.Rf = (cplx*)take(nm * p * p * c);
        w.Wg = (cplx*)take(nm * p * p * c);
        w.nrm = (double*)take(nm * kArnMaxP * sizeof(double));
        w.piv = (int*)take(nm * n * ii);
        w.perm = (int*)take(nm * n * ii);
        w.info = (int*)take(nm * ii);
        w.ord = (int*)take(nm * kArnMaxP * ii);
        w.done = (int*)take(nm * ii);
        w.ndone = (int*)take(ii);
    }
    if (D >= 1) w.uv = (cplx*)take(nm * count * 2 * n * c);
    Sv2Work v;
    const size_t b2 = sv2_carve(n, nmat * count, D, nullptr, v);
    char* p2 = take(std::max<size_t>(b2, 1));
    if (base) sv2_carve(n, nmat * count, D, p2, w.sv2);
    return off;
}

size_t arnoldi_work_bytes(int n, int nmat, int count, int D) {
    ArnWork w;
    return arnoldi_carve(n, nmat, count, D, nullptr, w);
}

// sigma_j (ascending), sigma_j' (D >= 1), sigma_j'' (D = 2) of the count smallest
// singular values of nmat matrices of order n: out[(D+1)(m count + j) + t];
// status_host[m], iters_host[m].  maxit >= 1; tol relative (ARPACK's tol).
cudaError_t arnoldi_batched(int n, int nmat, int count, int D, double tol, int maxit, unsigned long long seed,
                            const cplx* T, long long mat_stride, long long der_stride, double* out, void* work,
                            size_t work_bytes, int* status_host, int* iters_host, cudaStream_t st,
                            long long* launches) {
    if (!arnoldi_supported(n, count, D) || D < 0 || D > 2 || nmat < 1 || nmat > 65535 || maxit < 1 ||
        !(tol > 0.) || (long long)nmat * count > 65535)
        return cudaErrorInvalidValue;
    const int p = arnoldi_block(n, count), os = D + 1;
    ArnWork w;
    if (arnoldi_carve(n, nmat, count, D, nullptr, w) > work_bytes) return cudaErrorInvalidValue;
    arnoldi_carve(n, nmat, count, D, static_cast<char*>(work), w);
    ArnJob J{n, nmat, p, count, maxit, tol, seed, T, mat_stride, out, os, w.uv, w.status, w.iters};
    long long nl = 0;
    if (arnoldi_small_fits(n, p)) {
        const size_t smem = arn_smem_bytes(n, p);
        AR_CK(cudaFuncSetAttribute(k_arn_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_arn_small<<<nmat, kArnThreads, smem, st>>>(J);
        ++nl;
        AR_CK(cudaGetLastError());
    } else {
        const long long nn = (long long)n * n, ns = (long long)n * p;
        AR_CK(copy_mats_batched(nn, nmat, T, mat_stride, w.A, nn, st));
        AR_CK(lu_factor_batched(n, nmat, w.A, nn, w.piv, w.perm, w.info, st, &nl));
        AR_CK(cudaMemsetAsync(w.ndone, 0, sizeof(int), st));
        k_arn_init<<<nmat, 32, 0, st>>>(J, w.info, w.done, w.ndone);
        dim3 g((unsigned)std::min<long long>((ns + 255) / 256, 1024), (unsigned)nmat);
        k_arn_start<<<g, 256, 0, st>>>(n, p, seed, w.X, ns);
        nl += 3;
        AR_CK(cudaGetLastError());
        AR_CK(lu_solve_batched(n, nmat, 0, w.A, nn, w.perm, p, w.X, ns, st));
        AR_CK(qr_global_batched(n, nmat, p, w.X, ns, nullptr, st));
        nl += 2;
        cplx *X = w.X, *Y = w.Y;
        for (int it = 1;; ++it) {
            const int last = it >= maxit;
            AR_CK(cudaMemcpyAsync(Y, X, (size_t)nmat * ns * sizeof(cplx), cudaMemcpyDeviceToDevice, st));
            AR_CK(lu_solve_batched(n, nmat, 1, w.A, nn, w.perm, p, Y, ns, st));
            AR_CK(qr_global_batched(n, nmat, p, Y, ns, w.Rf, st));
            k_arn_ritz<<<nmat, 32, 0, st>>>(p, count, w.Rf, w.Wg, w.nrm, w.ord, w.done);
            AR_CK(lu_solve_batched(n, nmat, 0, w.A, nn, w.perm, p, Y, ns, st));
            k_arn_check<<<nmat, kArnThreads, 0, st>>>(J, X, Y, ns, w.Rf, w.Wg, w.nrm, w.ord, w.done, w.ndone, it,
                                                      last);
            nl += 5;
            AR_CK(cudaGetLastError());
            int nd = 0;
            AR_CK(cudaMemcpyAsync(&nd, w.ndone, sizeof(int), cudaMemcpyDeviceToHost, st));
            AR_CK(cudaStreamSynchronize(st));
            if (nd >= nmat || last) break;
            AR_CK(qr_global_batched(n, nmat, p, Y, ns, nullptr, st));
            ++nl;
            std::swap(X, Y);
        }
    }
    if (D >= 1)
        AR_CK(sv_der_from_vectors(n, nmat * count, count, D, T, mat_stride, der_stride, out, w.uv, w.sv2, st, nl));
    AR_CK(cudaMemcpyAsync(status_host, w.status, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    if (iters_host) AR_CK(cudaMemcpyAsync(iters_host, w.iters, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    AR_CK(cudaStreamSynchronize(st));
    if (launches) *launches += nl;
    return cudaSuccess;
}

}  // namespace hbem
