// Dense linear algebra on one CTA, operands in shared (or global) memory: block
// sums, LU with partial pivoting and its two solve forms, classical Gram-Schmidt
// QR (twice), and one-sided Jacobi for thin matrices.  Used by the randomized SVD
// (rsvd.cu) and the dense singular-value kernels (dense.cu).
#pragma once
#include "hbem_device.cuh"

namespace hbem {

static __device__ __forceinline__ double bsum(double x, double* red) {
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
// Per step: warp 0 finds the pivot (largest |A[i,k]|^2, i >= k, ties to the smallest
// i), exchanges the two rows and scales column k into lbuf (n entries of scratch) and
// A; after one barrier all warps update the trailing matrix, a warp per column and
// its lanes over the rows; a second barrier ends the step.
static __device__ void lu_smem(cplx* A, int n, int* piv, int* sing, cplx* lbuf) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int k = 0; k < n; ++k) {
        if (warp == 0) {
            double best = -1.;
            int bi = k;
            for (int i = k + lane; i < n; i += 32) {
                const double a = norm2(A[i + (long long)k * n]);
                if (a > best) { best = a; bi = i; }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double ob = __shfl_xor_sync(0xffffffffu, best, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            const int p = bi;   // the same on every lane
            if (lane == 0) {
                piv[k] = p;
                if (best == 0.) *sing = 1;
            }
            if (p != k)
                for (int j = lane; j < n; j += 32) {
                    const cplx t = A[k + (long long)j * n];
                    A[k + (long long)j * n] = A[p + (long long)j * n];
                    A[p + (long long)j * n] = t;
                }
            __syncwarp();
            const cplx d = A[k + (long long)k * n];
            const bool nz = norm2(d) > 0.;
            const cplx id = nz ? cdiv(mk(1.), d) : mk(0.);
            for (int i = k + 1 + lane; i < n; i += 32) {
                cplx l = A[i + (long long)k * n];
                if (nz) l = l * id;
                A[i + (long long)k * n] = l;
                lbuf[i] = l;
            }
        }
        __syncthreads();
        for (int j = k + 1 + warp; j < n; j += nw) {
            const cplx u = A[k + (long long)j * n];
            for (int i = k + 1 + lane; i < n; i += 32) cfms(A[i + (long long)j * n], lbuf[i], u);
        }
        __syncthreads();
    }
}

// X <- T^-1 X  (s columns, leading dimension n), with P T = L U in A
static __device__ void solve_lu(const cplx* A, const int* piv, int n, cplx* X, int s) {
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
            cfms(X[i + c * n], A[i + (long long)k * n], X[k + c * n]);
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {     // U x = y
        for (int c = threadIdx.x; c < s; c += blockDim.x) X[k + c * n] = cdiv(X[k + c * n], A[k + (long long)k * n]);
        __syncthreads();
        for (int e = threadIdx.x; e < k * s; e += blockDim.x) {
            const int i = e % k, c = e / k;
            cfms(X[i + c * n], A[i + (long long)k * n], X[k + c * n]);
        }
        __syncthreads();
    }
}

// X <- T^-H X:  T^H = U^H L^H P  =>  x = P^T L^-H U^-H b
static __device__ void solve_lu_h(const cplx* A, const int* piv, int n, cplx* X, int s) {
    for (int k = 0; k < n; ++k) {          // U^H y = b (lower triangular, diagonal conj(u_kk))
        for (int c = threadIdx.x; c < s; c += blockDim.x) X[k + c * n] = cdiv(X[k + c * n], conj(A[k + (long long)k * n]));
        __syncthreads();
        for (int e = threadIdx.x; e < (n - k - 1) * s; e += blockDim.x) {
            const int i = k + 1 + e % (n - k - 1), c = e / (n - k - 1);
            cfms_c(X[i + c * n], A[k + (long long)i * n], X[k + c * n]);
        }
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {     // L^H z = y (unit upper triangular)
        for (int e = threadIdx.x; e < k * s; e += blockDim.x) {
            const int i = e % k, c = e / k;
            cfms_c(X[i + c * n], A[k + (long long)i * n], X[k + c * n]);
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
// twice per column ("twice is enough").  coef: s entries of scratch.  If Rf is
// given it receives the s x s upper-triangular factor (column-major), X = Q Rf.
static __device__ void qr_cgs2(cplx* X, int n, int s, cplx* coef, double* red, cplx* Rf = nullptr) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < s; ++j) {
        cplx* xj = X + (long long)j * n;
        if (Rf)
            for (int i = threadIdx.x; i < s; i += blockDim.x) Rf[i + j * s] = mk(0.);
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
            if (Rf)
                for (int i = threadIdx.x; i < j; i += blockDim.x) Rf[i + j * s] += coef[i];
            for (int r = threadIdx.x; r < n; r += blockDim.x) {
                cplx v = xj[r];
                for (int i = 0; i < j; ++i) cfms(v, X[(long long)i * n + r], coef[i]);
                xj[r] = v;
            }
            __syncthreads();
        }
        double part = 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) part += norm2(xj[r]);
        const double nrm = sqrt(bsum(part, red));
        if (Rf && threadIdx.x == 0) Rf[j + j * s] = mk(nrm);
        const double inv = nrm > 0. ? 1. / nrm : 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) xj[r] = inv * xj[r];
        __syncthreads();
    }
}

// One-sided Jacobi on the n x s matrix B (columns in place), W (s x s) accumulates
// the right rotations.  Serial over pairs (s is small), each pair on the whole CTA.
static __device__ void jacobi_thin(cplx* B, int n, int s, cplx* W, double* red) {
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) W[e] = mk((e % s) == (e / s) ? 1. : 0.);
    __syncthreads();
    // orthogonal at the rounding level of an n-term inner product (see jacobi_cta)
    const double tol = fmax(1e-15, 2.0 * n * 2.220446049250313e-16);
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


// The same one-sided Jacobi for a square s x s matrix (s <= 32) on one warp: lane r
// holds row r, reductions by shuffles, no block-wide barriers.
static __device__ void jacobi_warp(cplx* B, int s, cplx* W) {
    const int r = threadIdx.x & 31;
    for (int e = r; e < s * s; e += 32) W[e] = mk((e % s) == (e / s) ? 1. : 0.);
    __syncwarp();
    // orthogonal once |x^H y| <= 2 s eps |x||y|, the rounding level of the computed
    // inner product (a tighter test keeps rotating on noise up to the sweep cap)
    const double tol = 2.0 * s * 2.220446049250313e-16;
    for (int sweep = 0; sweep < 30; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < s - 1; ++p)
            for (int q = p + 1; q < s; ++q) {
                const cplx x = r < s ? B[p * s + r] : mk(0.), y = r < s ? B[q * s + r] : mk(0.);
                double al = norm2(x), be = norm2(y);
                double gr = fma(x.re, y.re, x.im * y.im), gi = fma(x.re, y.im, -x.im * y.re);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    al += __shfl_xor_sync(0xffffffffu, al, o);
                    be += __shfl_xor_sync(0xffffffffu, be, o);
                    gr += __shfl_xor_sync(0xffffffffu, gr, o);
                    gi += __shfl_xor_sync(0xffffffffu, gi, o);
                }
                const double g = hypot(gr, gi);
                if (g == 0. || g <= tol * sqrt(al * be)) continue;
                rotated = 1;
                const double zeta = (be - al) / (2. * g);
                const double t = (zeta >= 0. ? 1. : -1.) / (fabs(zeta) + sqrt(1. + zeta * zeta));
                const double c = 1. / sqrt(1. + t * t), sn = c * t;
                const cplx eph = mk(gr / g, -gi / g);
                if (r < s) {
                    const cplx ey = eph * y;
                    B[p * s + r] = c * x - sn * ey;
                    B[q * s + r] = sn * x + c * ey;
                    const cplx wx = W[p * s + r], wy = eph * W[q * s + r];
                    W[p * s + r] = c * wx - sn * wy;
                    W[q * s + r] = sn * wx + c * wy;
                }
                __syncwarp();
            }
        if (!rotated) break;
    }
}


// The same one-sided Jacobi for a square s x s matrix (s <= 32) on the whole CTA:
// the column pairs of a round-robin step go to different warps (lane r holds row
// r of both columns), one barrier per step instead of one pair after the other on a
// single warp.  The reductions are broadcast from lane 0, so every lane applies the
// same rotation.  flag: one shared int of scratch.
static __device__ void jacobi_cta(cplx* B, int s, cplx* W, int* flag) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int e = threadIdx.x; e < s * s; e += blockDim.x) W[e] = mk((e % s) == (e / s) ? 1. : 0.);
    const int sp = s + (s & 1), m = sp - 1, npairs = sp / 2;
    // a pair counts as orthogonal once |x^H y| <= 2 s eps |x||y|: the computed inner
    // product of two s-vectors carries rounding of that order, so a tighter test
    // (1e-15 for s = 12) would keep rotating on noise until the sweep cap
    const double tol = 2.0 * s * 2.220446049250313e-16;
    __syncthreads();
    for (int sweep = 0; sweep < 30; ++sweep) {
        if (threadIdx.x == 0) *flag = 0;
        __syncthreads();
        for (int r = 0; r < m; ++r) {
            for (int k = warp; k < npairs; k += nw) {
                // round-robin ("circle") schedule: column 0 fixed, the others rotate
                int p, q;
                if (k == 0) { p = 0; q = r + 1; }
                else { p = (r + k) % m + 1; q = (r - k + m) % m + 1; }
                if (p >= s || q >= s) continue;
                if (p > q) { const int t = p; p = q; q = t; }
                const cplx x = lane < s ? B[p * s + lane] : mk(0.), y = lane < s ? B[q * s + lane] : mk(0.);
                double al = norm2(x), be = norm2(y);
                double gr = fma(x.re, y.re, x.im * y.im), gi = fma(x.re, y.im, -x.im * y.re);
                // rows >= s hold zeros: for s <= 16 the lower half-warp has the sums
                for (int o = s <= 16 ? 8 : 16; o > 0; o >>= 1) {
                    al += __shfl_xor_sync(0xffffffffu, al, o);
                    be += __shfl_xor_sync(0xffffffffu, be, o);
                    gr += __shfl_xor_sync(0xffffffffu, gr, o);
                    gi += __shfl_xor_sync(0xffffffffu, gi, o);
                }
                al = __shfl_sync(0xffffffffu, al, 0);
                be = __shfl_sync(0xffffffffu, be, 0);
                gr = __shfl_sync(0xffffffffu, gr, 0);
                gi = __shfl_sync(0xffffffffu, gi, 0);
                // rotation from |g|^2 and one reciprocal square root: shorter dependent
                // chain than hypot and the divisions by |g|
                const double g2 = fma(gr, gr, gi * gi);
                if (g2 == 0. || g2 <= (tol * tol) * (al * be)) continue;
                if (lane == 0) *flag = 1;
                const double ig = rsqrt(g2);
                const double zeta = (be - al) * (0.5 * ig);
                const double t = (zeta >= 0. ? 1. : -1.) / (fabs(zeta) + sqrt(fma(zeta, zeta, 1.)));
                const double c = rsqrt(fma(t, t, 1.)), sn = c * t;
                const cplx eph = mk(gr * ig, -gi * ig);
                if (lane < s) {
                    const cplx ey = eph * y;
                    B[p * s + lane] = c * x - sn * ey;
                    B[q * s + lane] = sn * x + c * ey;
                    const cplx wx = W[p * s + lane], wy = eph * W[q * s + lane];
                    W[p * s + lane] = c * wx - sn * wy;
                    W[q * s + lane] = sn * wx + c * wy;
                }
            }
            __syncthreads();
        }
        if (*flag == 0) break;
        __syncthreads();
    }
}


// ---------------------------------------------------------------- blocked solves
//
// The same two solves with the row exchanges composed into one permutation
// (perm[i] = source row of row i of P T) and the triangular sweeps blocked by 32
// rows: one warp per right-hand side solves the 32 x 32 diagonal block with
// shuffles, then all threads update the remaining rows -- two barriers per block
// instead of two per row.  buf: n entries of scratch; A, X may be in shared or
// global memory.

static __device__ void perm_from_piv(const int* piv, int n, int* perm) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = i;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; ++k) {
            const int p = piv[k];
            if (p != k) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
        }
    __syncthreads();
}

static __device__ void permute_cols(cplx* X, int n, int s, const int* perm, cplx* buf, bool inverse,
                                    cplx* wide = nullptr) {
    if (wide) {   // all columns in one pass through an n x s scratch
        for (int e = threadIdx.x; e < n * s; e += blockDim.x) wide[e] = X[e];
        __syncthreads();
        for (int e = threadIdx.x; e < n * s; e += blockDim.x) {
            const int i = e % n, c = e / n;
            if (!inverse) X[e] = wide[perm[i] + (long long)c * n];
            else X[perm[i] + (long long)c * n] = wide[e];
        }
        __syncthreads();
        return;
    }
    for (int c = 0; c < s; ++c) {
        cplx* x = X + (long long)c * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = x[i];
        __syncthreads();
        if (!inverse)
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = buf[perm[i]];
        else
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[perm[i]] = buf[i];
        __syncthreads();
    }
}

// X <- T^-1 X.  wide (optional): n x s scratch for a one-pass row permutation;
// inv_diag: A's diagonal holds 1 / u_kk (multiplications instead of divisions).
static __device__ void solve_lu_blk(const cplx* A, const int* perm, int n, cplx* X, int s, cplx* buf,
                                    cplx* wide = nullptr, bool inv_diag = false) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    permute_cols(X, n, s, perm, buf, false, wide);
    for (int b0 = 0; b0 < n; b0 += 32) {                       // L y = P b, L unit lower
        const int bs = min(32, n - b0);
        for (int c = warp; c < s; c += nw) {
            cplx* x = X + (long long)c * n + b0;
            cplx v = lane < bs ? x[lane] : mk(0.);
            for (int k = 0; k < bs; ++k) {
                cplx vk;
                vk.re = __shfl_sync(0xffffffffu, v.re, k);
                vk.im = __shfl_sync(0xffffffffu, v.im, k);
                if (lane > k && lane < bs) cfms(v, A[(b0 + lane) + (long long)(b0 + k) * n], vk);
            }
            if (lane < bs) x[lane] = v;
        }
        __syncthreads();
        const int rest = n - b0 - bs;
        for (int e = threadIdx.x; e < rest * s; e += blockDim.x) {
            const int i = b0 + bs + e % rest, c = e / rest;
            const cplx* xb = X + (long long)c * n + b0;
            cplx acc = mk(0.);
            for (int k = 0; k < bs; ++k) cfma(acc, A[i + (long long)(b0 + k) * n], xb[k]);
            X[i + (long long)c * n] -= acc;
        }
        __syncthreads();
    }
    for (int b0 = ((n - 1) / 32) * 32; b0 >= 0; b0 -= 32) {    // U x = y
        const int bs = min(32, n - b0);
        for (int c = warp; c < s; c += nw) {
            cplx* x = X + (long long)c * n + b0;
            cplx v = lane < bs ? x[lane] : mk(0.);
            for (int k = bs - 1; k >= 0; --k) {
                if (lane == k) {
                    const cplx d = A[(b0 + k) + (long long)(b0 + k) * n];
                    v = inv_diag ? v * d : cdiv(v, d);
                }
                cplx vk;
                vk.re = __shfl_sync(0xffffffffu, v.re, k);
                vk.im = __shfl_sync(0xffffffffu, v.im, k);
                if (lane < k) cfms(v, A[(b0 + lane) + (long long)(b0 + k) * n], vk);
            }
            if (lane < bs) x[lane] = v;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < b0 * s; e += blockDim.x) {
            const int i = e % b0, c = e / b0;
            const cplx* xb = X + (long long)c * n + b0;
            cplx acc = mk(0.);
            for (int k = 0; k < bs; ++k) cfma(acc, A[i + (long long)(b0 + k) * n], xb[k]);
            X[i + (long long)c * n] -= acc;
        }
        __syncthreads();
    }
}

// X <- T^-H X:  T^H = U^H L^H P, x = P^T L^-H U^-H b (wide, inv_diag as in solve_lu_blk)
static __device__ void solve_lu_h_blk(const cplx* A, const int* perm, int n, cplx* X, int s, cplx* buf,
                                      cplx* wide = nullptr, bool inv_diag = false) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int b0 = 0; b0 < n; b0 += 32) {                       // U^H y = b (lower, diagonal conj(u_kk))
        const int bs = min(32, n - b0);
        for (int c = warp; c < s; c += nw) {
            cplx* x = X + (long long)c * n + b0;
            cplx v = lane < bs ? x[lane] : mk(0.);
            for (int k = 0; k < bs; ++k) {
                if (lane == k) {
                    const cplx d = conj(A[(b0 + k) + (long long)(b0 + k) * n]);
                    v = inv_diag ? v * d : cdiv(v, d);
                }
                cplx vk;
                vk.re = __shfl_sync(0xffffffffu, v.re, k);
                vk.im = __shfl_sync(0xffffffffu, v.im, k);
                if (lane > k && lane < bs) cfms_c(v, A[(b0 + k) + (long long)(b0 + lane) * n], vk);
            }
            if (lane < bs) x[lane] = v;
        }
        __syncthreads();
        const int rest = n - b0 - bs;
        for (int e = threadIdx.x; e < rest * s; e += blockDim.x) {
            const int i = b0 + bs + e % rest, c = e / rest;
            const cplx* xb = X + (long long)c * n + b0;
            const cplx* col = A + (long long)i * n + b0;        // U[b0.., i]
            cplx acc = mk(0.);
            for (int k = 0; k < bs; ++k) cfma_c(acc, col[k], xb[k]);
            X[i + (long long)c * n] -= acc;
        }
        __syncthreads();
    }
    for (int b0 = ((n - 1) / 32) * 32; b0 >= 0; b0 -= 32) {    // L^H z = y (unit upper)
        const int bs = min(32, n - b0);
        for (int c = warp; c < s; c += nw) {
            cplx* x = X + (long long)c * n + b0;
            cplx v = lane < bs ? x[lane] : mk(0.);
            for (int k = bs - 1; k >= 0; --k) {
                cplx vk;
                vk.re = __shfl_sync(0xffffffffu, v.re, k);
                vk.im = __shfl_sync(0xffffffffu, v.im, k);
                if (lane < k) cfms_c(v, A[(b0 + k) + (long long)(b0 + lane) * n], vk);
            }
            if (lane < bs) x[lane] = v;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < b0 * s; e += blockDim.x) {
            const int i = e % b0, c = e / b0;
            const cplx* xb = X + (long long)c * n + b0;
            const cplx* col = A + (long long)i * n + b0;        // L[b0.., i]
            cplx acc = mk(0.);
            for (int k = 0; k < bs; ++k) cfma_c(acc, col[k], xb[k]);
            X[i + (long long)c * n] -= acc;
        }
        __syncthreads();
    }
    permute_cols(X, n, s, perm, buf, true, wide);
}

}  // namespace hbem
