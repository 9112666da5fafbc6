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
#include <algorithm>

#include "hbem_device.cuh"
#include "smem_linalg.cuh"

namespace hbem {

constexpr int kRsvdThreads = 256;
constexpr int kRsvdMaxS = 32;
constexpr int kRitzRefine = 2;     // inverse-iteration steps on the right Ritz vector

struct RsvdJob {
    int n, nmat, s, q, D;
    const cplx* T;            // matrix m at T + m*mat_stride, T' at + der_stride
    long long mat_stride, der_stride;
    const cplx* R;            // n x s sketch (shared by all matrices)
    double* out;              // [nmat][D + 1]: sigma estimate, sigma' (D >= 1), sigma'' slot (D = 2)
    int* status;              // [nmat]: 0 ok, 5 singular pivot
    cplx* uv;                 // optional [nmat][2n]: Ritz vectors u, v of sigma
};

__global__ void __launch_bounds__(kRsvdThreads) k_rsvd_small(RsvdJob J) {
    extern __shared__ double smraw[];
    const int n = J.n, s = J.s, mat = blockIdx.x, os = J.D + 1;
    cplx* A = reinterpret_cast<cplx*>(smraw);       // n x n
    cplx* X = A + (long long)n * n;                 // n x s (Q)
    cplx* Y = X + (long long)n * s;                 // n x s (work)
    cplx* W = Y + (long long)n * s;                 // s x s
    cplx* coef = W + s * s;                         // s
    double* red = reinterpret_cast<double*>(coef + s);   // 128
    int* piv = reinterpret_cast<int*>(red + 128);   // n
    int* redi = piv + n;                            // 32
    int* perm = redi + 32;                          // n
    cplx* vb = reinterpret_cast<cplx*>(piv + (2 * n + 32 + 3) / 4 * 4);   // n, 16-byte aligned
    __shared__ int s_sing;
    if (threadIdx.x == 0) s_sing = 0;
    const cplx* T0 = J.T + (long long)mat * J.mat_stride;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) A[e] = T0[e];
    for (int e = threadIdx.x; e < n * s; e += blockDim.x) X[e] = J.R[e];
    __syncthreads();
    lu_smem(A, n, piv, &s_sing, vb);
    // blocked solves: rows permuted once, U's diagonal replaced by its reciprocals
    perm_from_piv(piv, n, perm);
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const cplx d = A[k + (long long)k * n];
        A[k + (long long)k * n] = norm2(d) > 0. ? cdiv(mk(1.), d) : mk(0.);
    }
    __syncthreads();
    // Q = qr(T^-1 R)
    solve_lu_blk(A, perm, n, X, s, vb, nullptr, true);
    qr_cgs2(X, n, s, coef, red);
    for (int it = 0; it < J.q; ++it) {
        solve_lu_h_blk(A, perm, n, X, s, vb, nullptr, true);
        qr_cgs2(X, n, s, coef, red);
        solve_lu_blk(A, perm, n, X, s, vb, nullptr, true);
        qr_cgs2(X, n, s, coef, red);
    }
    // B = T^-H Q (keep Q in X, B in Y)
    for (int e = threadIdx.x; e < n * s; e += blockDim.x) Y[e] = X[e];
    __syncthreads();
    solve_lu_h_blk(A, perm, n, Y, s, vb, nullptr, true);
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
        J.out[(long long)os * mat] = smax > 0. ? 1. / smax : 0.;
        for (int t = 1; t < os; ++t) J.out[(long long)os * mat + t] = 0.;
        J.status[mat] = s_sing ? 5 : 0;
    }
    if (J.D == 0) return;
    // right Ritz vector v = Q w (w = column bj of W), then two steps of inverse
    // iteration v <- T^-1 T^-H v with the LU in shared memory; u, sigma' follow in
    // k_rsvd_vec
    __syncthreads();
    const cplx* w = W + bj * s;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx v = mk(0.);
        for (int c = 0; c < s; ++c) cfma(v, X[c * n + r], w[c]);
        vb[r] = v;
    }
    __syncthreads();
    for (int it = 0; it < kRitzRefine; ++it) {   // Y is free now: row-permutation scratch
        solve_lu_h_blk(A, perm, n, vb, 1, Y, nullptr, true);
        solve_lu_blk(A, perm, n, vb, 1, Y, nullptr, true);
    }
    for (int r = threadIdx.x; r < n; r += blockDim.x) J.uv[2LL * n * mat + n + r] = vb[r];
}

size_t rsvd_smem_bytes(int n, int s) {
    return ((size_t)n * n + 2 * (size_t)n * s + (size_t)s * s + s) * sizeof(cplx) + 128 * sizeof(double) +
           (((size_t)2 * n + 32 + 3) / 4 * 4) * sizeof(int) + (size_t)n * sizeof(cplx);
}

cudaError_t launch_rsvd_small(int n, int nmat, int s, int q, int D, const cplx* T, long long mat_stride,
                              long long der_stride, const cplx* R, double* out, int* status, cplx* uv,
                              cudaStream_t st) {
    const size_t limit = 220 * 1024;
    size_t smem = rsvd_smem_bytes(n, s);
    if (smem > limit || s > kRsvdMaxS || s < 1 || s > n) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_rsvd_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    RsvdJob J{n, nmat, s, q, D, T, mat_stride, der_stride, R, out, status, uv};
    k_rsvd_small<<<nmat, kRsvdThreads, smem, st>>>(J);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ matrices of any order
//
// The same algorithm with the LU, the n x s blocks and the Wielandt system in
// global memory (lu.cu): T^-1 / T^-H applications by the batched solves, the QR
// steps by one CTA per matrix, sigma from the s x s triangular factor of T^-H Q.

cudaError_t lu_factor_batched(int n, int nmat, cplx* A, long long stride, int* piv, int* perm, int* info,
                              cudaStream_t st, long long* launches);
cudaError_t lu_solve_batched(int n, int nmat, int trans, const cplx* LU, long long stride, const int* perm, int s,
                             cplx* X, long long xstride, cudaStream_t st);
bool lu_solve_supported(int n);

__global__ void k_copy_mats(int nn, const cplx* src, long long sstride, cplx* dst, long long dstride) {
    const cplx* a = src + (long long)blockIdx.y * sstride;
    cplx* b = dst + (long long)blockIdx.y * dstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nn; e += (long long)gridDim.x * blockDim.x)
        b[e] = a[e];
}

__global__ void __launch_bounds__(kRsvdThreads) k_qr_global(int n, int s, cplx* X, long long xstride, cplx* Rf) {
    __shared__ cplx coef[kRsvdMaxS];
    __shared__ double red[128];
    qr_cgs2(X + (long long)blockIdx.x * xstride, n, s, coef, red, Rf ? Rf + (long long)blockIdx.x * s * s : nullptr);
}

// sigma from the triangular factor Rf of B = T^-H Q = Q_B Rf: sigma_max(B) =
// sigma_max(Rf).  D >= 1: the right Ritz vector v = Q w (w the top right singular
// vector of Rf) into the v half of uv.
__global__ void __launch_bounds__(kRsvdThreads) k_rsvd_tail(int n, int s, int D, const cplx* Q, const cplx* QB,
                                                             long long xstride, const cplx* Rf, const cplx* T,
                                                             long long mat_stride, long long der_stride,
                                                             const int* info, double* out, int* status, cplx* uv,
                                                             const int* tc_err) {
    __shared__ cplx Rs[kRsvdMaxS * kRsvdMaxS], W[kRsvdMaxS * kRsvdMaxS], tw[kRsvdMaxS];
    const int mat = blockIdx.x, os = D + 1;
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) Rs[e] = Rf[(long long)mat * s * s + e];
    __syncthreads();
    if (threadIdx.x < 32) jacobi_warp(Rs, s, W);
    __syncthreads();
    double best = -1.;
    int bj = 0;
    for (int j = 0; j < s; ++j) {
        double nb = 0.;
        for (int r = 0; r < s; ++r) nb += norm2(Rs[j * s + r]);
        if (nb > best) { best = nb; bj = j; }
    }
    const double smax = sqrt(best), isn = smax > 0. ? 1. / smax : 0.;
    if (threadIdx.x == 0) {
        out[(long long)os * mat] = isn;
        for (int t = 1; t < os; ++t) out[(long long)os * mat + t] = 0.;
        status[mat] = info[mat] ? 5 : ((tc_err && *tc_err) ? 4 : 0);
    }
    if (D == 0) return;
    if (threadIdx.x < s) tw[threadIdx.x] = W[bj * s + threadIdx.x];   // w
    __syncthreads();
    const cplx* Qm = Q + (long long)mat * xstride;
    cplx* v = uv + 2LL * n * mat + n;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx b = mk(0.);
        for (int c = 0; c < s; ++c) cfma(b, Qm[r + (long long)c * n], tw[c]);
        v[r] = b;
    }
}

// After the inverse-iteration steps: v <- v / |v|, u = T v / |T v|, and
// sigma' = Re u^H T' v (the Wielandt form x^H W' x with x = (u; v)/sqrt2).
// Vector blockIdx.x belongs to matrix blockIdx.x / per.
__global__ void __launch_bounds__(kRsvdThreads) k_rsvd_vec(int n, int D, const cplx* T, long long mat_stride,
                                                            long long der_stride, double* out, cplx* uv, int per) {
    __shared__ double red[128];
    const int mat = blockIdx.x, os = D + 1;
    cplx* u = uv + 2LL * n * mat;
    cplx* v = u + n;
    double part = 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) part += norm2(v[r]);
    const double nv = sqrt(bsum(part, red));
    const double iv = nv > 0. ? 1. / nv : 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) v[r] = iv * v[r];
    __syncthreads();
    const cplx* Tm = T + (long long)(mat / per) * mat_stride;
    part = 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx a = mk(0.);
        for (int c = 0; c < n; ++c) cfma(a, Tm[r + (long long)c * n], v[c]);
        u[r] = a;
        part += norm2(a);
    }
    const double nu = sqrt(bsum(part, red + 32));
    const double iu = nu > 0. ? 1. / nu : 0.;
    const cplx* T1 = Tm + der_stride;
    part = 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx tv = mk(0.);
        for (int c = 0; c < n; ++c) cfma(tv, T1[r + (long long)c * n], v[c]);
        const cplx ur = iu * u[r];
        u[r] = ur;
        part += ur.re * tv.re + ur.im * tv.im;
    }
    const double d1 = bsum(part, red + 64);
    if (threadIdx.x == 0) out[(long long)os * mat + 1] = d1;
}

// ------------------------------------------------------------------ sigma'' (sv_der2)
//
// randsvd.cpp:171-216: with x the unit null vector of W - sigma I, W = [0 T; T^H 0],
// m = argmax |x_l|, u = x / x_m and B = W - sigma I with column m replaced by -u,
//   u' = -B^-1 (W' u), t = u'_m (= sigma'), u'_m = 0,
//   sigma'' = -[B^-1 (W'' u + 2 (W' u' - t u'))]_m.
// Here x = (u_R; v_R)/sqrt2 from the Ritz vectors of the sketch.

__global__ void __launch_bounds__(256) k_sv2_prep(int n, const cplx* uv, cplx* ub, int* mcol) {
    const int mat = blockIdx.x, n2 = 2 * n;
    const cplx* x = uv + (long long)n2 * mat;
    __shared__ double rv[8];
    __shared__ int ri[8];
    __shared__ int s_m;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double best = -1.;
    int bi = 0;
    for (int l = threadIdx.x; l < n2; l += blockDim.x) {
        const double a = norm2(x[l]);
        if (a > best) { best = a; bi = l; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    if (lane == 0) { rv[warp] = best; ri[warp] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = rv[0];
        int p = ri[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            if (rv[w] > b || (rv[w] == b && ri[w] < p)) { b = rv[w]; p = ri[w]; }
        s_m = p;
        mcol[mat] = p;
    }
    __syncthreads();
    const cplx xm = x[s_m];
    const cplx ixm = norm2(xm) > 0. ? cdiv(mk(1.), xm) : mk(0.);
    for (int l = threadIdx.x; l < n2; l += blockDim.x) ub[(long long)n2 * mat + l] = x[l] * ixm;
}

__global__ void k_build_bordered(int n, const cplx* T, long long mat_stride, int per, const double* out, int os,
                                 const cplx* ub, const int* mcol, cplx* B) {
    const int mat = blockIdx.y, n2 = 2 * n, m = mcol[mat];
    const double sig = out[(long long)os * mat];
    const cplx* Tm = T + (long long)(mat / per) * mat_stride;
    const cplx* u = ub + (long long)n2 * mat;
    cplx* Bm = B + (long long)n2 * n2 * mat;
    const long long tot = (long long)n2 * n2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e % n2), j = (int)(e / n2);
        cplx v = mk(0.);
        if (j == m) v = -u[i];
        else {
            if (i == j) v = mk(-sig);
            else if (i < n && j >= n) v = Tm[i + (long long)(j - n) * n];
            else if (i >= n && j < n) v = conj(Tm[j + (long long)(i - n) * n]);
        }
        Bm[e] = v;
    }
}

// y = alpha [A x2; A^H x1] (+ y if acc), A = matrix mat / per of the batch, x = [x1; x2]
__global__ void __launch_bounds__(256) k_wapply(int n, const cplx* A, long long mat_stride, int per, const cplx* x,
                                                cplx* y, double alpha, int acc) {
    const int mat = blockIdx.x, n2 = 2 * n;
    const cplx* Am = A + (long long)(mat / per) * mat_stride;
    const cplx* x1 = x + (long long)n2 * mat;
    const cplx* x2 = x1 + n;
    cplx* y1 = y + (long long)n2 * mat;
    cplx* y2 = y1 + n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        cplx sacc = mk(0.);
        for (int j = 0; j < n; ++j) cfma(sacc, Am[i + (long long)j * n], x2[j]);
        y1[i] = acc ? y1[i] + alpha * sacc : alpha * sacc;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < n; j += nw) {
        double sr = 0., si = 0.;
        const cplx* col = Am + (long long)j * n;
        for (int i = lane; i < n; i += 32) {
            const cplx a = conj(col[i]), b = x1[i];
            sr = fma(a.re, b.re, fma(-a.im, b.im, sr));
            si = fma(a.re, b.im, fma(a.im, b.re, si));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0) y2[j] = acc ? y2[j] + alpha * mk(sr, si) : alpha * mk(sr, si);
    }
}

__global__ void k_sv2_extract(int n, int nmat, cplx* ud, const int* mcol, cplx* tb) {
    const int mat = blockIdx.x * blockDim.x + threadIdx.x;
    if (mat >= nmat) return;
    cplx* u = ud + 2LL * n * mat;
    tb[mat] = u[mcol[mat]];
    u[mcol[mat]] = mk(0.);
}

__global__ void k_sv2_axpy(int n, cplx* rhs, const cplx* ud, const cplx* tb) {
    const int mat = blockIdx.x, n2 = 2 * n;
    const cplx t2 = 2. * tb[mat];
    for (int l = threadIdx.x; l < n2; l += blockDim.x) cfms(rhs[(long long)n2 * mat + l], t2, ud[(long long)n2 * mat + l]);
}

__global__ void k_sv2_out(int n, int nmat, const cplx* sol, const int* mcol, const int* info, double* out) {
    const int mat = blockIdx.x * blockDim.x + threadIdx.x;
    if (mat >= nmat) return;
    out[3LL * mat + 2] = info[mat] ? CUDART_NAN : -sol[2LL * n * mat + mcol[mat]].re;
}

#define RS_CK(x)                                \
    do {                                        \
        cudaError_t e_ = (x);                   \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

// ------------------------------------------------------------------ mixed precision
//
// Complex-FP32 LU; the subspace iterations solve with the FP32 factors alone (an
// O(eps_32 cond) perturbation of the sketch subspace changes the Ritz value only at
// second order), while the final T^-H Q and the Ritz-vector solves are refined in
// FP64: x <- x + LU32^-1 (b - op(T) x), residuals from the FP64 T.

cudaError_t lu_factor_batched_f32(int n, int nmat, cplxf* A, long long stride, int* piv, int* perm, int* info,
                                  cudaStream_t st, long long* launches, int* tc_err);
cudaError_t lu_solve_batched_f32(int n, int nmat, int trans, const cplxf* LU, long long stride, const int* perm,
                                 int s, cplxf* X, long long xstride, cudaStream_t st);
bool lu_solve_supported_f32(int n);

__global__ void k_to_f32(long long len, const cplx* src, long long sstride, cplxf* dst, long long dstride) {
    const cplx* a = src + (long long)blockIdx.y * sstride;
    cplxf* b = dst + (long long)blockIdx.y * dstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x)
        b[e] = mkf((float)a[e].re, (float)a[e].im);
}

// dst = src (overwrite) or dst += src
__global__ void k_acc_f64(long long len, const cplxf* src, long long sstride, cplx* dst, long long dstride,
                          int overwrite) {
    const cplxf* a = src + (long long)blockIdx.y * sstride;
    cplx* b = dst + (long long)blockIdx.y * dstride;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < len; e += (long long)gridDim.x * blockDim.x) {
        const cplx v = mk((double)a[e].re, (double)a[e].im);
        b[e] = overwrite ? v : b[e] + v;
    }
}

constexpr int kResChunk = 16;

// Rres = B - T X, one thread per row, grid (ceil(n / 256), nmat)
__global__ void __launch_bounds__(256) k_resid_n(int n, int s, const cplx* T, long long mat_stride, const cplx* X,
                                                  long long xs, const cplx* B, long long bs, cplx* Rr, long long rs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const cplx* Tm = T + (long long)blockIdx.y * mat_stride;
    const cplx* Xm = X + (long long)blockIdx.y * xs;
    const cplx* Bm = B + (long long)blockIdx.y * bs;
    cplx* Rm = Rr + (long long)blockIdx.y * rs;
    for (int cb = 0; cb < s; cb += kResChunk) {
        const int cs = min(kResChunk, s - cb);
        cplx acc[kResChunk];
#pragma unroll
        for (int c = 0; c < kResChunk; ++c) acc[c] = mk(0.);
        for (int r = 0; r < n; ++r) {
            const cplx t = Tm[i + (long long)r * n];
#pragma unroll
            for (int c = 0; c < kResChunk; ++c)
                if (c < cs) cfma(acc[c], t, Xm[r + (long long)(cb + c) * n]);
        }
#pragma unroll
        for (int c = 0; c < kResChunk; ++c)
            if (c < cs) Rm[i + (long long)(cb + c) * n] = Bm[i + (long long)(cb + c) * n] - acc[c];
    }
}

// Rres = B - T^H X, one warp per row, grid (ceil(n / 8), nmat), 256 threads
__global__ void __launch_bounds__(256) k_resid_h(int n, int s, const cplx* T, long long mat_stride, const cplx* X,
                                                  long long xs, const cplx* B, long long bs, cplx* Rr, long long rs) {
    const int lane = threadIdx.x & 31, i = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (i >= n) return;
    const cplx* col = T + (long long)blockIdx.y * mat_stride + (long long)i * n;
    const cplx* Xm = X + (long long)blockIdx.y * xs;
    const cplx* Bm = B + (long long)blockIdx.y * bs;
    cplx* Rm = Rr + (long long)blockIdx.y * rs;
    for (int cb = 0; cb < s; cb += kResChunk) {
        const int cs = min(kResChunk, s - cb);
        cplx acc[kResChunk];
#pragma unroll
        for (int c = 0; c < kResChunk; ++c) acc[c] = mk(0.);
        for (int r = lane; r < n; r += 32) {
            const cplx t = conj(col[r]);
#pragma unroll
            for (int c = 0; c < kResChunk; ++c)
                if (c < cs) cfma(acc[c], t, Xm[r + (long long)(cb + c) * n]);
        }
#pragma unroll
        for (int c = 0; c < kResChunk; ++c) {
            if (c >= cs) break;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                acc[c].re += __shfl_xor_sync(0xffffffffu, acc[c].re, o);
                acc[c].im += __shfl_xor_sync(0xffffffffu, acc[c].im, o);
            }
            if (lane == 0) Rm[i + (long long)(cb + c) * n] = Bm[i + (long long)(cb + c) * n] - acc[c];
        }
    }
}

struct MixedBufs {
    const cplxf* LU32;
    const int* perm;
    cplx* Bsave;
    cplx* Rres;
    cplxf* X32;
};

static dim3 grid_len(long long len, int nmat) {
    return dim3((unsigned)std::min<long long>(1024, (len + 255) / 256), (unsigned)nmat);
}

// X_m <- op(T_m)^-1 X_m for ncol columns (leading dimension n, matrix stride xs):
// iters = 1 is the plain FP32 solve, each further iteration one FP64 residual and
// one FP32 correction.
cudaError_t solve_mixed(int n, int nmat, int trans, const MixedBufs& mb, const cplx* T, long long mat_stride, cplx* X,
                        int ncol, long long xs, int iters, cudaStream_t st, long long& nl) {
    const long long len = (long long)n * ncol, nn = (long long)n * n;
    const dim3 g = grid_len(len, nmat);
    if (iters > 1) {
        k_copy_mats<<<g, 256, 0, st>>>((int)len, X, xs, mb.Bsave, len);
        ++nl;
    }
    k_to_f32<<<g, 256, 0, st>>>(len, X, xs, mb.X32, len);
    RS_CK(lu_solve_batched_f32(n, nmat, trans, mb.LU32, nn, mb.perm, ncol, mb.X32, len, st));
    k_acc_f64<<<g, 256, 0, st>>>(len, mb.X32, len, X, xs, 1);
    nl += 3;
    for (int it = 1; it < iters; ++it) {
        if (trans)
            k_resid_h<<<dim3((n + 7) / 8, nmat), 256, 0, st>>>(n, ncol, T, mat_stride, X, xs, mb.Bsave, len, mb.Rres, len);
        else
            k_resid_n<<<dim3((n + 255) / 256, nmat), 256, 0, st>>>(n, ncol, T, mat_stride, X, xs, mb.Bsave, len, mb.Rres,
                                                                  len);
        k_to_f32<<<g, 256, 0, st>>>(len, mb.Rres, len, mb.X32, len);
        RS_CK(lu_solve_batched_f32(n, nmat, trans, mb.LU32, nn, mb.perm, ncol, mb.X32, len, st));
        k_acc_f64<<<g, 256, 0, st>>>(len, mb.X32, len, X, xs, 0);
        nl += 4;
    }
    return cudaGetLastError();
}

// ------------------------------------------------------------------ orchestration

struct Sv2Work {
    cplx *B = nullptr, *ub = nullptr, *ud = nullptr, *rhs = nullptr, *tb = nullptr;
    int *piv2 = nullptr, *perm2 = nullptr, *info2 = nullptr, *mcol = nullptr;
};
cudaError_t sv_der_from_vectors(int n, int nvec, int per, int D, const cplx* T, long long mat_stride,
                                long long der_stride, double* out, cplx* uv, const Sv2Work& w, cudaStream_t st,
                                long long& nl);

struct RsvdWork {
    cplx *A = nullptr, *X = nullptr, *Y = nullptr, *Rf = nullptr, *uv = nullptr;
    int *piv = nullptr, *perm = nullptr, *info = nullptr;
    cplxf *A32 = nullptr, *X32 = nullptr;
    int* tc_err = nullptr;
    cplx *Bsave = nullptr, *Rres = nullptr;
    cplx *B = nullptr, *ub = nullptr, *ud = nullptr, *rhs = nullptr, *tb = nullptr;
    int *piv2 = nullptr, *perm2 = nullptr, *info2 = nullptr, *mcol = nullptr;
};

static Sv2Work sv2_work(const RsvdWork& w) {
    Sv2Work v;
    v.B = w.B; v.ub = w.ub; v.ud = w.ud; v.rhs = w.rhs; v.tb = w.tb;
    v.piv2 = w.piv2; v.perm2 = w.perm2; v.info2 = w.info2; v.mcol = w.mcol;
    return v;
}

// Carve the workspace (base == nullptr: only count).  Returns the bytes needed.
size_t rsvd_carve(int n, int nmat, int s, int D, bool small, bool mixed, char* base, RsvdWork& w) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return p;
    };
    const size_t nm = (size_t)nmat, nn = (size_t)n * n, c = sizeof(cplx), cf = sizeof(cplxf), ii = sizeof(int);
    if (!small) {
        if (mixed) {
            w.A32 = (cplxf*)take(nm * nn * cf);
            w.tc_err = (int*)take(sizeof(int));
            w.X32 = (cplxf*)take(nm * n * s * cf);
            w.Bsave = (cplx*)take(nm * n * s * c);
            w.Rres = (cplx*)take(nm * n * s * c);
        } else {
            w.A = (cplx*)take(nm * nn * c);
        }
        w.piv = (int*)take(nm * n * ii);
        w.perm = (int*)take(nm * n * ii);
        w.info = (int*)take(nm * ii);
        w.X = (cplx*)take(nm * n * s * c);
        w.Y = (cplx*)take(nm * n * s * c);
        w.Rf = (cplx*)take(nm * s * s * c);
    }
    if (D >= 1) w.uv = (cplx*)take(nm * 2 * n * c);
    if (D == 2) {
        w.B = (cplx*)take(nm * 4 * nn * c);
        w.piv2 = (int*)take(nm * 2 * n * ii);
        w.perm2 = (int*)take(nm * 2 * n * ii);
        w.info2 = (int*)take(nm * ii);
        w.ub = (cplx*)take(nm * 2 * n * c);
        w.ud = (cplx*)take(nm * 2 * n * c);
        w.rhs = (cplx*)take(nm * 2 * n * c);
        w.tb = (cplx*)take(nm * c);
        w.mcol = (int*)take(nm * ii);
    }
    return off;
}

bool rsvd_small_fits(int n, int s) { return rsvd_smem_bytes(n, s) <= 220 * 1024 && s <= kRsvdMaxS; }

bool rsvd_supported(int n, int s, int D) {
    if (s < 1 || s > kRsvdMaxS || s > n) return false;
    if (!rsvd_small_fits(n, s) && !lu_solve_supported(n)) return false;
    if (D == 2 && !lu_solve_supported(2 * n)) return false;
    return true;
}

// precision 0: FP64 throughout; 1: complex-FP32 LU with FP64 refinement (matrices
// that fit one CTA's shared memory always take the FP64 single-kernel path)
size_t rsvd_work_bytes(int n, int nmat, int s, int D, int precision) {
    RsvdWork w;
    return rsvd_carve(n, nmat, s, D, rsvd_small_fits(n, s), precision == 1, nullptr, w);
}

// sigma (D = 0), sigma' (D >= 1), sigma'' (D = 2) of nmat matrices of order n;
// out[(D+1) m + t], status[m] (0 ok, 5 zero pivot in the LU of T).
cudaError_t rsvd_batched(int n, int nmat, int s, int q, int D, int precision, int refine, const cplx* T,
                         long long mat_stride, long long der_stride, const cplx* R, double* out, int* status,
                         void* work, size_t work_bytes, cudaStream_t st, long long* launches) {
    if (!rsvd_supported(n, s, D) || D < 0 || D > 2 || nmat < 1 || nmat > 65535 || precision < 0 || precision > 1 ||
        refine < 1 || refine > 16)
        return cudaErrorInvalidValue;
    const bool small = rsvd_small_fits(n, s), mixed = precision == 1 && !small;
    RsvdWork w;
    if (rsvd_carve(n, nmat, s, D, small, mixed, nullptr, w) > work_bytes) return cudaErrorInvalidValue;
    rsvd_carve(n, nmat, s, D, small, mixed, static_cast<char*>(work), w);
    long long nl = 0;
    if (small) {
        RS_CK(launch_rsvd_small(n, nmat, s, q, D, T, mat_stride, der_stride, R, out, status, w.uv, st));
        ++nl;
    } else {
        const long long nn = (long long)n * n, ns = (long long)n * s;
        const MixedBufs mb{w.A32, w.perm, w.Bsave, w.Rres, w.X32};
        // op(T)^-1 on ncol columns: FP64 factors, or FP32 factors with `iters` refinement passes
        auto solve = [&](int trans, cplx* X, int ncol, long long xs, int iters) -> cudaError_t {
            if (!mixed) {
                ++nl;
                return lu_solve_batched(n, nmat, trans, w.A, nn, w.perm, ncol, X, xs, st);
            }
            return solve_mixed(n, nmat, trans, mb, T, mat_stride, X, ncol, xs, iters, st, nl);
        };
        if (mixed) {
            k_to_f32<<<grid_len(nn, nmat), 256, 0, st>>>(nn, T, mat_stride, w.A32, nn);
            RS_CK(cudaMemsetAsync(w.tc_err, 0, sizeof(int), st));
            RS_CK(lu_factor_batched_f32(n, nmat, w.A32, nn, w.piv, w.perm, w.info, st, &nl, w.tc_err));
        } else {
            k_copy_mats<<<grid_len(nn, nmat), 256, 0, st>>>((int)nn, T, mat_stride, w.A, nn);
            RS_CK(lu_factor_batched(n, nmat, w.A, nn, w.piv, w.perm, w.info, st, &nl));
        }
        k_copy_mats<<<grid_len(ns, nmat), 256, 0, st>>>((int)ns, R, 0, w.X, ns);
        nl += 2;
        RS_CK(solve(0, w.X, s, ns, 1));
        k_qr_global<<<nmat, kRsvdThreads, 0, st>>>(n, s, w.X, ns, nullptr);
        ++nl;
        for (int it = 0; it < q; ++it) {
            RS_CK(solve(1, w.X, s, ns, 1));
            k_qr_global<<<nmat, kRsvdThreads, 0, st>>>(n, s, w.X, ns, nullptr);
            RS_CK(solve(0, w.X, s, ns, 1));
            k_qr_global<<<nmat, kRsvdThreads, 0, st>>>(n, s, w.X, ns, nullptr);
            nl += 2;
        }
        RS_CK(cudaMemcpyAsync(w.Y, w.X, (size_t)nmat * ns * sizeof(cplx), cudaMemcpyDeviceToDevice, st));
        RS_CK(solve(1, w.Y, s, ns, refine));
        k_qr_global<<<nmat, kRsvdThreads, 0, st>>>(n, s, w.Y, ns, w.Rf);
        k_rsvd_tail<<<nmat, kRsvdThreads, 0, st>>>(n, s, D, w.X, w.Y, ns, w.Rf, T, mat_stride, der_stride, w.info,
                                                    out, status, w.uv, w.tc_err);
        nl += 2;
        RS_CK(cudaGetLastError());
        if (D >= 1)
            for (int it = 0; it < kRitzRefine; ++it) {
                RS_CK(solve(1, w.uv + n, 1, 2LL * n, refine));
                RS_CK(solve(0, w.uv + n, 1, 2LL * n, refine));
            }
    }
    if (D >= 1) RS_CK(sv_der_from_vectors(n, nmat, 1, D, T, mat_stride, der_stride, out, w.uv, sv2_work(w), st, nl));
    if (launches) *launches += nl;
    return cudaSuccess;
}

// sigma' (D >= 1) and sigma'' (D = 2) of nvec singular triplets whose right vectors
// v sit in the v halves of uv ([nvec][2n]) and whose sigma sits in out[(D+1) t];
// triplet t belongs to matrix t / per.  v is normalised, u = T v / |T v|, sigma' =
// Re u^H T' v; sigma'' by the bordered system above.
cudaError_t sv_der_from_vectors(int n, int nvec, int per, int D, const cplx* T, long long mat_stride,
                                long long der_stride, double* out, cplx* uv, const Sv2Work& w, cudaStream_t st,
                                long long& nl) {
    k_rsvd_vec<<<nvec, kRsvdThreads, 0, st>>>(n, D, T, mat_stride, der_stride, out, uv, per);
    ++nl;
    RS_CK(cudaGetLastError());
    if (D < 2) return cudaSuccess;
    const int n2 = 2 * n;
    const long long nn2 = (long long)n2 * n2;
    k_sv2_prep<<<nvec, 256, 0, st>>>(n, uv, w.ub, w.mcol);
    k_build_bordered<<<grid_len(nn2, nvec), 256, 0, st>>>(n, T, mat_stride, per, out, 3, w.ub, w.mcol, w.B);
    RS_CK(lu_factor_batched(n2, nvec, w.B, nn2, w.piv2, w.perm2, w.info2, st, &nl));
    k_wapply<<<nvec, 256, 0, st>>>(n, T + der_stride, mat_stride, per, w.ub, w.ud, -1., 0);
    RS_CK(lu_solve_batched(n2, nvec, 0, w.B, nn2, w.perm2, 1, w.ud, n2, st));
    k_sv2_extract<<<(nvec + 127) / 128, 128, 0, st>>>(n, nvec, w.ud, w.mcol, w.tb);
    k_wapply<<<nvec, 256, 0, st>>>(n, T + 2 * der_stride, mat_stride, per, w.ub, w.rhs, 1., 0);
    k_wapply<<<nvec, 256, 0, st>>>(n, T + der_stride, mat_stride, per, w.ud, w.rhs, 2., 1);
    k_sv2_axpy<<<nvec, 256, 0, st>>>(n, w.rhs, w.ud, w.tb);
    RS_CK(lu_solve_batched(n2, nvec, 0, w.B, nn2, w.perm2, 1, w.rhs, n2, st));
    k_sv2_out<<<(nvec + 127) / 128, 128, 0, st>>>(n, nvec, w.rhs, w.mcol, w.info2, out);
    nl += 10;
    return cudaGetLastError();
}

// Workspace of sv_der_from_vectors for nvec triplets (base == nullptr: only count).
size_t sv2_carve(int n, int nvec, int D, char* base, Sv2Work& w) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        char* p = base ? base + off : nullptr;
        off += (bytes + 255) / 256 * 256;
        return p;
    };
    if (D < 2) return 0;
    const size_t nv = (size_t)nvec, nn = (size_t)n * n, c = sizeof(cplx), ii = sizeof(int);
    w.B = (cplx*)take(nv * 4 * nn * c);
    w.piv2 = (int*)take(nv * 2 * n * ii);
    w.perm2 = (int*)take(nv * 2 * n * ii);
    w.info2 = (int*)take(nv * ii);
    w.ub = (cplx*)take(nv * 2 * n * c);
    w.ud = (cplx*)take(nv * 2 * n * c);
    w.rhs = (cplx*)take(nv * 2 * n * c);
    w.tb = (cplx*)take(nv * c);
    w.mcol = (int*)take(nv * ii);
    return off;
}

// Launchers shared with the block iteration of arnoldi.cu
cudaError_t qr_global_batched(int n, int nmat, int s, cplx* X, long long xstride, cplx* Rf, cudaStream_t st) {
    if (s < 1 || s > kRsvdMaxS) return cudaErrorInvalidValue;
    k_qr_global<<<nmat, kRsvdThreads, 0, st>>>(n, s, X, xstride, Rf);
    return cudaGetLastError();
}

cudaError_t copy_mats_batched(long long nn, int nmat, const cplx* src, long long sstride, cplx* dst,
                              long long dstride, cudaStream_t st) {
    k_copy_mats<<<grid_len(nn, nmat), 256, 0, st>>>((int)nn, src, sstride, dst, dstride);
    return cudaGetLastError();
}

}  // namespace hbem
