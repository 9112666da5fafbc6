// Mass projection of T(k) (gen_sol_op.cpp:45-48): T_proj = F^-1 T F^-T with
// F = blockdiag(L, L), L the Cholesky factor of the P1 mass matrix M.  M is
// cyclic tridiagonal, so L is lower bidiagonal plus a dense last row (the fill
// of the wrap-around coupling): every solve is an O(N) recurrence.
//   diag inverse  id[i] = 1/L[i][i]
//   sub           sb[i] = L[i+1][i]          (i < N-1; sb[N-2] is also the last row's)
//   last row      lr[i] = L[N-1][i]          (i < N-1)
#include "hbem_device.cuh"

namespace hbem {

struct CholView {
    int N;
    const double* id;
    const double* sb;
    const double* lr;
};

// forward substitution L z = t on a strided vector, in place
__device__ __forceinline__ void chol_solve_strided(const CholView& L, cplx* x, long long stride) {
    const int N = L.N;
    cplx acc = mk(0.);                        // sum_{i < N-1} lr[i] z[i]
    cplx zprev = mk(0.);
    for (int i = 0; i < N - 1; ++i) {
        cplx t = x[i * stride];
        if (i > 0) { t.re -= L.sb[i - 1] * zprev.re; t.im -= L.sb[i - 1] * zprev.im; }
        cplx z = L.id[i] * t;
        x[i * stride] = z;
        axpy(acc, L.lr[i], z);
        zprev = z;
    }
    cplx t = x[(long long)(N - 1) * stride] - acc;
    x[(long long)(N - 1) * stride] = L.id[N - 1] * t;
}

// Y = T F^-T: each thread owns one row r of one matrix and solves along its two column blocks.
__global__ void k_proj_rows(CholView L, cplx* T, long long mat_stride, int nmat) {
    const int n = 2 * L.N;
    long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long tot = (long long)nmat * n;
    if (gid >= tot) return;
    int r = (int)(gid % n);
    long long m = gid / n;
    cplx* A = T + m * mat_stride;
    chol_solve_strided(L, A + r, n);                          // columns 0..N-1
    chol_solve_strided(L, A + r + (long long)L.N * n, n);     // columns N..2N-1
}

// T_proj = F^-1 Y: each thread owns one column and solves along its two row blocks.
__global__ void k_proj_cols(CholView L, cplx* T, long long mat_stride, int nmat) {
    const int n = 2 * L.N;
    long long gid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long tot = (long long)nmat * n;
    if (gid >= tot) return;
    int c = (int)(gid % n);
    long long m = gid / n;
    cplx* A = T + m * mat_stride + (long long)c * n;
    chol_solve_strided(L, A, 1);
    chol_solve_strided(L, A + L.N, 1);
}

cudaError_t launch_projection(int N, const double* id, const double* sb, const double* lr, cplx* T, int nmat,
                              cudaStream_t st) {
    CholView L{N, id, sb, lr};
    long long n = 2LL * N;
    long long tot = nmat * n;
    unsigned g = (unsigned)((tot + 127) / 128);
    k_proj_rows<<<g, 128, 0, st>>>(L, T, n * n, nmat);
    k_proj_cols<<<g, 128, 0, st>>>(L, T, n * n, nmat);
    return cudaGetLastError();
}

// T, T' (and T'' when d = 2) at x_q = x_src + h_q (q < nq <= 2) from T, T', T'' at
// x_src (src: three n x n matrices one after another) by their Taylor polynomials,
//   T(x_q) = T + h T' + h^2/2 T'',  T'(x_q) = T' + h T'',  T''(x_q) = T'',
// into dst = [q][0 .. d].  The terms left out are h^3/6 T''', h^2/2 T''' and h T''':
// for |h| <= 1e-6 (T''' of the order of (sqrt(c) r)^2 T' for panel distances r) they
// are below 1e-11 of T' and T, and T'' (which only sets a Newton step's length) is
// good to ~1e-5.
__global__ void k_taylor_near(long long mat, const cplx* src, int nq, double h0, double h1, int d, cplx* dst) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= mat) return;
    const cplx t0 = src[e], t1 = src[mat + e], t2 = src[2 * mat + e];
    for (int q = 0; q < nq; ++q) {
        const double h = q ? h1 : h0;
        cplx* o = dst + (long long)q * (d + 1) * mat;
        o[e] = t0 + h * (t1 + (0.5 * h) * t2);
        o[mat + e] = t1 + h * t2;
        if (d == 2) o[2 * mat + e] = t2;
    }
}

cudaError_t launch_taylor_near(long long mat, const cplx* src, int nq, double h0, double h1, int d, cplx* dst,
                               cudaStream_t st) {
    if (nq < 1 || nq > 2 || d < 1 || d > 2) return cudaErrorInvalidValue;
    k_taylor_near<<<(unsigned)((mat + 255) / 256), 256, 0, st>>>(mat, src, nq, h0, h1, d, dst);
    return cudaGetLastError();
}

}  // namespace hbem
