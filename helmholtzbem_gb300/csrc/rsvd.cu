// Randomized smallest singular value (randomized_svd::sv / sv_der,
// source/utilities/randsvd.cpp:99-169) for batches of matrices that fit in shared
// memory: one CTA per matrix, everything in FP64.
//
//   P T = L U (partial pivoting, in place in shared memory)
//   Q = qr(T^-1 R); q times: Q = qr(T^-1 qr(T^-H Q)); B = T^-H Q
//   sigma_min ~ 1 / sigma_max(B)          (one-sided Jacobi on the n x s matrix B)
// For sv_der the top singular pair of B gives the Ritz vectors of T's smallest
// triplet: u = B w / |B w|, v = Q w, and sigma' = Re u^H T' v.  (The reference
// recomputes the null vector of the 2n x 2n Wielandt matrix by a column-pivoted
// QR; the Ritz vectors are that null vector to the accuracy of the sketch.)
#include "hbem_device.cuh"

namespace hbem {

constexpr int kRsvdThreads = 256;
constexpr int kRsvdMaxS = 32;

__device__ __forceinline__ double bsum(double x, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    __syncthreads();
    if (lane == 0) red[warp] = x;
    __syncthreads();
    double s = 0.;
    for (int w = 0; w < nw; ++w) s += red[w];
    return s;
}

// LU with partial pivoting of the n x n column-major matrix A (shared memory).
// piv[k] = row exchanged with row k at step k.  Returns via *sing a zero-pivot flag.
__device__ void lu_smem(cplx* A, int n, int* piv, double* redv, int* redi, int* sing) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < n; ++k) {
        // pivot: largest |A[i,k]|, i >= k (ties: smallest i)
        double best = -1.;
        int bi = k;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
            double a = norm2(A[i + (long long)k * n]);
            if (a > best) { best = a; bi = i; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double ob = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) { redv[warp] = best; redi[warp] = bi; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double b = redv[0];
            int p = redi[0];
            for (int w = 1; w < nw; ++w)
                if (redv[w] > b || (redv[w] == b && redi[w] < p)) { b = redv[w]; p = redi[w]; }
            piv[k] = p;
            if (b == 0.) *sing = 1;
        }
        __syncthreads();
        const int p = piv[k];
        if (p != k)
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                cplx t = A[k + (long long)j * n];
                A[k + (long long)j * n] = A[p + (long long)j * n];
                A[p + (long long)j * n] = t;
            }
        __syncthreads();
        const cplx d = A[k + (long long)k * n];
        if (norm2(d) > 0.) {
            const cplx id = cdiv(mk(1.), d);
            for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) A[i + (long long)k * n] = A[i + (long long)k * n] * id;
        }
        __syncthreads();
        const int m = n - k - 1;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = k + 1 + e % m, j = k + 1 + e / m;
            A[i + (long long)j * n] -= A[i + (long long)k * n] * A[k + (long long)j * n];
        }
        __syncthreads();
    }
}

// X <- T^-1 X  (s columns, leading dimension n), with P T = L U in A
__device__ void solve_lu(const cplx* A, const int* piv, int n, cplx* X, int s) {
    for (int k = 0; k < n; ++k) {          // row exchanges in order
        const int p = piv[k];
        if (p != k)
            for (int c = threadIdx.x; c < s; c += blockDim.x) {
                cplx t = X[k + c * n];
                X[k + c * n] = X[p + c * n];
                X[p + c * n] = t;
            }
        __syncthreads();
    }
    for (int k = 0; k < n; ++k) {          // L y = P b (unit diagonal)
        for (int e = threadIdx.x; e < (n - k - 1) * s; e += blockDim.x) {
            const int i = k + 1 + e % (n - k - 1), c = e / (n - k - 1);
            X[i + c * n] -= A[i + (long long)k * n] * X[k + c * n];
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {     // U x = y
        for (int c = threadIdx.x; c < s; c += blockDim.x) X[k + c * n] = cdiv(X[k + c * n], A[k + (long long)k * n]);
        __syncthreads();
        for (int e = threadIdx.x; e < k * s; e += blockDim.x) {
            const int i = e % k, c = e / k;
            X[i + c * n] -= A[i + (long long)k * n] * X[k + c * n];
        }
        __syncthreads();
    }
}

// X <- T^-H X:  T^H = U^H L^H P  =>  x = P^T L^-H U^-H b
__device__ void solve_lu_h(const cplx* A, const int* piv, int n, cplx* X, int s) {
    for (int k = 0; k < n; ++k) {          // U^H y = b (lower triangular, diagonal conj(u_kk))
        for (int c = threadIdx.x; c < s; c += blockDim.x) X[k + c * n] = cdiv(X[k + c * n], conj(A[k + (long long)k * n]));
        __syncthreads();
        for (int e = threadIdx.x; e < (n - k - 1) * s; e += blockDim.x) {
            const int i = k + 1 + e % (n - k - 1), c = e / (n - k - 1);
            X[i + c * n] -= conj(A[k + (long long)i * n]) * X[k + c * n];
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {     // L^H z = y (unit upper triangular)
        for (int e = threadIdx.x; e < k * s; e += blockDim.x) {
            const int i = e % k, c = e / k;
            X[i + c * n] -= conj(A[k + (long long)i * n]) * X[k + c * n];
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {     // x = P^T z (exchanges in reverse order)
        const int p = piv[k];
        if (p != k)
            for (int c = threadIdx.x; c < s; c += blockDim.x) {
                cplx t = X[k + c * n];
                X[k + c * n] = X[p + c * n];
                X[p + c * n] = t;
            }
        __syncthreads();
    }
}

// Orthonormalise the s columns of X (n x s) in place: classical Gram-Schmidt,
// twice per column ("twice is enough").  coef: s entries of scratch.
__device__ void qr_cgs2(cplx* X, int n, int s, cplx* coef, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < s; ++j) {
        cplx* xj = X + j * n;
        for (int pass = 0; pass < 2; ++pass) {
            for (int i = warp; i < j; i += nw) {
                const cplx* qi = X + i * n;
                double cr = 0., ci = 0.;
                for (int r = lane; r < n; r += 32) {
                    cplx a = qi[r], b = xj[r];
                    cr = fma(a.re, b.re, fma(a.im, b.im, cr));
                    ci = fma(a.re, b.im, fma(-a.im, b.re, ci));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    cr += __shfl_xor_sync(0xffffffffu, cr, o);
                    ci += __shfl_xor_sync(0xffffffffu, ci, o);
                }
                if (lane == 0) coef[i] = mk(cr, ci);
            }
            __syncthreads();
            for (int r = threadIdx.x; r < n; r += blockDim.x) {
                cplx v = xj[r];
                for (int i = 0; i < j; ++i) v -= X[i * n + r] * coef[i];
                xj[r] = v;
            }
            __syncthreads();
        }
        double part = 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) part += norm2(xj[r]);
        const double nrm = sqrt(bsum(part, red));
        const double inv = nrm > 0. ? 1. / nrm : 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) xj[r] = inv * xj[r];
        __syncthreads();
    }
}

// One-sided Jacobi on the n x s matrix B (columns in place), W (s x s) accumulates
// the right rotations.  Serial over pairs (s is small), each pair on the whole CTA.
__device__ void jacobi_thin(cplx* B, int n, int s, cplx* W, double* red) {
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) W[e] = mk((e % s) == (e / s) ? 1. : 0.);
    __syncthreads();
    const double tol = 1e-15;
    for (int sweep = 0; sweep < 30; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < s - 1; ++p)
            for (int q = p + 1; q < s; ++q) {
                cplx* bp = B + p * n;
                cplx* bq = B + q * n;
                double al = 0., be = 0., gr = 0., gi = 0.;
                for (int r = threadIdx.x; r < n; r += blockDim.x) {
                    cplx x = bp[r], y = bq[r];
                    al += norm2(x);
                    be += norm2(y);
                    gr = fma(x.re, y.re, fma(x.im, y.im, gr));
                    gi = fma(x.re, y.im, fma(-x.im, y.re, gi));
                }
                al = bsum(al, red);
                be = bsum(be, red + 32);
                gr = bsum(gr, red + 64);
                gi = bsum(gi, red + 96);
                double g = hypot(gr, gi);
                if (g == 0. || g <= tol * sqrt(al * be)) continue;
                rotated = 1;
                double zeta = (be - al) / (2. * g);
                double t = (zeta >= 0. ? 1. : -1.) / (fabs(zeta) + sqrt(1. + zeta * zeta));
                double c = 1. / sqrt(1. + t * t), sn = c * t;
                cplx eph = mk(gr / g, -gi / g);
                for (int r = threadIdx.x; r < n; r += blockDim.x) {
                    cplx x = bp[r], y = eph * bq[r];
                    bp[r] = c * x - sn * y;
                    bq[r] = sn * x + c * y;
                }
                for (int r = threadIdx.x; r < s; r += blockDim.x) {
                    cplx x = W[p * s + r], y = eph * W[q * s + r];
                    W[p * s + r] = c * x - sn * y;
                    W[q * s + r] = sn * x + c * y;
                }
                __syncthreads();
            }
        if (!rotated) break;
    }
}

struct RsvdJob {
    int n, nmat, s, q, D;
    const cplx* T;            // matrix m at T + m*mat_stride, T' at + der_stride
    long long mat_stride, der_stride;
    const cplx* R;            // n x s sketch (shared by all matrices)
    double* out;              // [nmat][2]: sigma estimate, sigma'
    int* status;              // [nmat]: 0 ok, 5 singular pivot
};

__global__ void __launch_bounds__(kRsvdThreads) k_rsvd_small(RsvdJob J) {
    extern __shared__ double smraw[];
    const int n = J.n, s = J.s, mat = blockIdx.x;
    cplx* A = reinterpret_cast<cplx*>(smraw);       // n x n
    cplx* X = A + (long long)n * n;                 // n x s (Q)
    cplx* Y = X + (long long)n * s;                 // n x s (work)
    cplx* W = Y + (long long)n * s;                 // s x s
    cplx* coef = W + s * s;                         // s
    double* red = reinterpret_cast<double*>(coef + s);   // 128
    int* piv = reinterpret_cast<int*>(red + 128);   // n
    int* redi = piv + n;                            // 32
    __shared__ int s_sing;
    if (threadIdx.x == 0) s_sing = 0;
    const cplx* T0 = J.T + (long long)mat * J.mat_stride;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = T0[e];
    for (int e = threadIdx.x; e < n * s; e += blockDim.x) X[e] = J.R[e];
    __syncthreads();
    lu_smem(A, n, piv, red, redi, &s_sing);
    // Q = qr(T^-1 R)
    solve_lu(A, piv, n, X, s);
    qr_cgs2(X, n, s, coef, red);
    for (int it = 0; it < J.q; ++it) {
        solve_lu_h(A, piv, n, X, s);
        qr_cgs2(X, n, s, coef, red);
        solve_lu(A, piv, n, X, s);
        qr_cgs2(X, n, s, coef, red);
    }
    // B = T^-H Q (keep Q in X, B in Y)
    for (int e = threadIdx.x; e < n * s; e += blockDim.x) Y[e] = X[e];
    __syncthreads();
    solve_lu_h(A, piv, n, Y, s);
    jacobi_thin(Y, n, s, W, red);
    // largest column of B W
    double best = -1.;
    int bj = 0;
    for (int j = 0; j < s; ++j) {
        double part = 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) part += norm2(Y[j * n + r]);
        double nb = bsum(part, red);
        if (nb > best) { best = nb; bj = j; }
    }
    const double smax = sqrt(best);
    if (threadIdx.x == 0) {
        J.out[2LL * mat] = smax > 0. ? 1. / smax : 0.;
        J.out[2LL * mat + 1] = 0.;
        J.status[mat] = s_sing ? 5 : 0;
    }
    if (J.D == 0) return;
    // Ritz vectors: u = B w / |B w| (column bj of Y), v = Q w (w = column bj of W)
    __syncthreads();
    const double isn = smax > 0. ? 1. / smax : 0.;
    // sigma' = Re u^H T' v accumulated row by row
    double part_re = 0.;
    const cplx* T1 = T0 + J.der_stride;
    const cplx* w = W + bj * s;
    // v_r = sum_c X[r, c] w_c ; stash v in A (the LU factors are no longer needed)
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx v = mk(0.);
        for (int c = 0; c < s; ++c) v += X[c * n + r] * w[c];
        A[r] = v;
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx tv = mk(0.);
        for (int c = 0; c < n; ++c) tv += T1[r + (long long)c * n] * A[c];
        cplx ur = isn * Y[bj * n + r];
        part_re += ur.re * tv.re + ur.im * tv.im;   // Re(conj(u_r) tv_r)
    }
    const double d1 = bsum(part_re, red);
    if (threadIdx.x == 0) J.out[2LL * mat + 1] = d1;
}

size_t rsvd_smem_bytes(int n, int s) {
    return ((size_t)n * n + 2 * (size_t)n * s + (size_t)s * s + s) * sizeof(cplx) + 128 * sizeof(double) +
           ((size_t)n + 32) * sizeof(int);
}

cudaError_t launch_rsvd_small(int n, int nmat, int s, int q, int D, const cplx* T, long long mat_stride,
                              long long der_stride, const cplx* R, double* out, int* status, cudaStream_t st) {
    const size_t limit = 220 * 1024;
    size_t smem = rsvd_smem_bytes(n, s);
    if (smem > limit || s > kRsvdMaxS || s < 1 || s > n) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_rsvd_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    RsvdJob J{n, nmat, s, q, D, T, mat_stride, der_stride, R, out, status};
    k_rsvd_small<<<nmat, kRsvdThreads, smem, st>>>(J);
    return cudaGetLastError();
}

}  // namespace hbem
