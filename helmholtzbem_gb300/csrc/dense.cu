// Batched dense singular values of small complex matrices and the first/second
// wavenumber derivatives of the smallest one.
//
// Replaces direct::sv / sv_1st_der / sv_2nd_der (source/utilities/singular_values.cpp:7-147),
// which diagonalise the Hermitian Wielandt matrix W = [[0, T], [T^H, 0]] (eigenvalues
// +-sigma_j).  Here: one-sided (Hestenes) Jacobi on T itself, one CTA per matrix,
// T in shared memory when it fits; then, for sigma = sigma_i with vectors (u, v):
//   sigma'  = Re u^H T' v
//   sigma'' = Re u^H T'' v + 1/2 sum_{j != i} |a_j + b_j|^2 / (sigma - sigma_j)
//                          + 1/2 sum_j      |a_j - b_j|^2 / (sigma + sigma_j)
// with a_j = u_j^H T' v, b_j = v_j^H T'^H u -- the second-order eigenvalue
// perturbation of W.  Partners numerically degenerate with sigma
// (|sigma_j - sigma| <= 1e-9 sigma) are left out of the first sum: a
// perturbation that keeps the degeneracy does not couple them.
#include <atomic>

#include <cooperative_groups.h>

#include "hbem_device.cuh"
#include "smem_linalg.cuh"

namespace hbem {

namespace cg = cooperative_groups;

constexpr int kSvdThreads = 512;
constexpr int kSvdMaxSweeps = 40;

__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

__device__ __forceinline__ void rr_pair(int r, int k, int m, int& p, int& q) {
    // round-robin ("circle") schedule over n' = m + 1 columns
    if (k == 0) { p = 0; q = r + 1; return; }
    p = (r + k) % m + 1;
    q = (r - k + m) % m + 1;
}

struct SvdJob {
    int n, nmat, D, which;
    const cplx* T;          // matrix m, derivative t at T + m*mat_stride + t*der_stride
    long long mat_stride, der_stride;
    cplx* gA;               // global scratch [nmat][n][n] (used when A does not fit in smem)
    cplx* gV;               // [nmat][n][n]
    double* out;            // [nmat][3]
    double* sig_all;        // optional [nmat][n]
    int* status;            // [nmat]
    int a_in_smem;
};

// single-precision complex (cplxf) for the first Jacobi stage of the mixed-precision kernel
typedef cplxf cpf;

__device__ __forceinline__ float warp_sumf(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// Stage 1 of the mixed-precision path: one-sided Jacobi of T in FP32 (A32 and V32
// both in shared memory), to the FP32 noise level.  Only V32 is used afterwards.
// Each column pair of a round-robin step is handled by a group of G lanes (G = 8 for
// n <= 128: the 64 groups of a 512-thread CTA take a whole step at once, with
// 3-level shuffle reductions), G = 32 for larger n.
//
// Warm start (Vw != null, n x n unitary to FP32 working precision, typically the V32
// of a nearby wavenumber): the sweeps start from A = T Vw, V = Vw instead of A = T,
// V = I.  The stopping rule is the same, so the result has the cold start's accuracy;
// when T Vw is nearly column-orthogonal far fewer sweeps are needed.  rowbuf: one row
// of n entries per warp (shared memory).
template <int G>
__device__ void jacobi_fp32_g(const cplx* T0, int n, cpf* A32, cpf* V32, int* s_rot, const cpf* Vw, cpf* rowbuf) {
    const int np = n + (n & 1), m = np - 1;
    const int gl = threadIdx.x % G, grp = threadIdx.x / G, ngrp = blockDim.x / G;
    const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        cplx t = T0[e];
        A32[e] = mkf((float)t.re, (float)t.im);
        V32[e] = Vw ? Vw[e] : mkf((e % n) == (e / n) ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    if (Vw) {
        // A <- A V row by row: each warp copies its row to rowbuf, then its lanes form
        // the row's entries (only the warp's own row of A is read or written)
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        cpf* rb = rowbuf + (long long)warp * n;
        for (int i = warp; i < n; i += nw) {
            for (int c = lane; c < n; c += 32) rb[c] = A32[i + (long long)c * n];
            __syncwarp();
            for (int j = lane; j < n; j += 32) {
                const cpf* vj = V32 + (long long)j * n;
                float ar = 0.f, ai = 0.f;
                for (int c = 0; c < n; ++c) {
                    const cpf a = rb[c], v = vj[c];
                    ar = fmaf(a.re, v.re, fmaf(-a.im, v.im, ar));
                    ai = fmaf(a.re, v.im, fmaf(a.im, v.re, ai));
                }
                A32[i + (long long)j * n] = mkf(ar, ai);
            }
            __syncwarp();
        }
        __syncthreads();
    }
    const float tol = 4e-6f;
    for (int sweep = 0; sweep < 30; ++sweep) {
        if (threadIdx.x == 0) *s_rot = 0;
        __syncthreads();
        for (int r = 0; r < m; ++r) {
            for (int k = grp; k < np / 2; k += ngrp) {
                int p, q;
                rr_pair(r, k, m, p, q);
                if (p >= n || q >= n) continue;
                if (p > q) { int t = p; p = q; q = t; }
                cpf* ap = A32 + p * n;
                cpf* aq = A32 + q * n;
                float al = 0.f, be = 0.f, gr = 0.f, gi = 0.f;
                for (int i = gl; i < n; i += G) {
                    cpf x = ap[i], y = aq[i];
                    al = fmaf(x.re, x.re, fmaf(x.im, x.im, al));
                    be = fmaf(y.re, y.re, fmaf(y.im, y.im, be));
                    gr = fmaf(x.re, y.re, fmaf(x.im, y.im, gr));
                    gi = fmaf(x.re, y.im, fmaf(-x.im, y.re, gi));
                }
#pragma unroll
                for (int o = G / 2; o > 0; o >>= 1) {
                    al += __shfl_xor_sync(gmask, al, o);
                    be += __shfl_xor_sync(gmask, be, o);
                    gr += __shfl_xor_sync(gmask, gr, o);
                    gi += __shfl_xor_sync(gmask, gi, o);
                }
                float g = hypotf(gr, gi);
                if (g == 0.f || g <= tol * sqrtf(al * be)) continue;
                if (gl == 0) *s_rot = 1;
                float zeta = (be - al) / (2.f * g);
                float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
                float c = 1.f / sqrtf(1.f + t * t), s = c * t;
                float er = gr / g, ei = -gi / g;
                cpf* vp = V32 + p * n;
                cpf* vq = V32 + q * n;
                for (int i = gl; i < n; i += G) {
                    cpf x = ap[i], y0 = aq[i];
                    cpf y = mkf(er * y0.re - ei * y0.im, er * y0.im + ei * y0.re);
                    ap[i] = mkf(c * x.re - s * y.re, c * x.im - s * y.im);
                    aq[i] = mkf(s * x.re + c * y.re, s * x.im + c * y.im);
                    cpf xv = vp[i], yv0 = vq[i];
                    cpf yv = mkf(er * yv0.re - ei * yv0.im, er * yv0.im + ei * yv0.re);
                    vp[i] = mkf(c * xv.re - s * yv.re, c * xv.im - s * yv.im);
                    vq[i] = mkf(s * xv.re + c * yv.re, s * xv.im + c * yv.im);
                }
            }
            __syncthreads();
        }
        if (*s_rot == 0) break;
        __syncthreads();
    }
}

__device__ void jacobi_fp32(const cplx* T0, int n, cpf* A32, cpf* V32, int* s_rot, const cpf* Vw = nullptr,
                            cpf* rowbuf = nullptr) {
    if (n <= 128) jacobi_fp32_g<8>(T0, n, A32, V32, s_rot, Vw, rowbuf);
    else jacobi_fp32_g<32>(T0, n, A32, V32, s_rot, Vw, rowbuf);
}

// Stage 2: V = orthonormalised columns of V32 in FP64 (classical Gram-Schmidt; one
// pass suffices because V32 is unitary to the FP32 level).  vcol, red: smem scratch.
__device__ void orthonormalise_fp64(const cpf* V32, int n, cplx* V, cplx* vcol, cplx* coef, double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < n; ++j) {
        for (int r = threadIdx.x; r < n; r += blockDim.x) vcol[r] = mk((double)V32[j * n + r].re, (double)V32[j * n + r].im);
        __syncthreads();
        for (int i = warp; i < j; i += nw) {       // coef_i = v_i^H vcol
            const cplx* vi = V + (long long)i * n;
            double cr = 0., ci = 0.;
            for (int r = lane; r < n; r += 32) {
                cplx a = vi[r], b = vcol[r];
                cr = fma(a.re, b.re, fma(a.im, b.im, cr));
                ci = fma(a.re, b.im, fma(-a.im, b.re, ci));
            }
            cr = warp_sum(cr);
            ci = warp_sum(ci);
            if (lane == 0) coef[i] = mk(cr, ci);
        }
        __syncthreads();
        double part = 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            cplx s = vcol[r];
            for (int i = 0; i < j; ++i) cfms(s, V[(long long)i * n + r], coef[i]);
            vcol[r] = s;
            part += norm2(s);
        }
        part = warp_sum(part);
        if (lane == 0) red[warp] = part;
        __syncthreads();
        double nrm2 = 0.;
        for (int w = 0; w < nw; ++w) nrm2 += red[w];
        const double inv = nrm2 > 0. ? 1. / sqrt(nrm2) : 0.;
        for (int r = threadIdx.x; r < n; r += blockDim.x) V[(long long)j * n + r] = inv * vcol[r];
        __syncthreads();
    }
}

// Stage 3: A = T V in FP64 (A in shared memory, overwriting the FP32 stage's space)
__device__ void product_fp64(const cplx* T0, const cplx* V, int n, cplx* A) {
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int r = e % n, c = e / n;
        const cplx* vc = V + (long long)c * n;
        cplx s = mk(0.);
        for (int k = 0; k < n; ++k) cfma(s, T0[r + (long long)k * n], vc[k]);
        A[e] = s;
    }
    __syncthreads();
}

template <bool MIXED>
__global__ void __launch_bounds__(kSvdThreads) k_svd_jacobi(SvdJob J) {
    extern __shared__ double smraw[];
    const int n = J.n, mat = blockIdx.x;
    const int np = n + (n & 1);           // padded to even
    const int m = np - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    cplx* sbase = reinterpret_cast<cplx*>(smraw);
    cplx* A = J.a_in_smem ? sbase : J.gA + (long long)mat * n * n;
    cplx* vec = J.a_in_smem ? sbase + (long long)n * n : sbase;   // 4n scratch vectors
    cplx* uy = vec;            // y = T' v_i, later T'' v_i
    cplx* uz = vec + n;        // z = T'^H u_i
    cplx* ui = vec + 2 * n;    // u_i
    cplx* vi = vec + 3 * n;    // v_i
    double* red = reinterpret_cast<double*>(vec + 4 * n);   // [64]
    __shared__ int s_rot;
    __shared__ int s_imin;
    cplx* V = J.gV + (long long)mat * n * n;
    const cplx* T0 = J.T + (long long)mat * J.mat_stride;
    if (MIXED) {
        // FP32 Jacobi for the bulk of the rotations, then an FP64 start from T V with
        // V orthonormalised in FP64; the FP64 sweeps below only polish (A must be in
        // shared memory: the FP32 stage uses the same space)
        cpf* A32 = reinterpret_cast<cpf*>(sbase);
        jacobi_fp32(T0, n, A32, A32 + (long long)n * n, &s_rot);
        orthonormalise_fp64(A32 + (long long)n * n, n, V, uy, uz, red);
        product_fp64(T0, V, n, A);
    } else {
        for (long long e = threadIdx.x; e < (long long)n * n; e += blockDim.x) {
            A[e] = T0[e];
            int r = (int)(e % n), c = (int)(e / n);
            V[e] = mk(r == c ? 1. : 0.);
        }
        __syncthreads();
    }
    int sweep = 0;
    const double tol = fmax(1e-15, sqrt((double)n) * kEps);   // rounding level of the Gram entries
    for (; sweep < kSvdMaxSweeps; ++sweep) {
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        for (int r = 0; r < m; ++r) {
            for (int k = warp; k < np / 2; k += nw) {
                int p, q;
                rr_pair(r, k, m, p, q);
                if (p >= n || q >= n) continue;   // padding column
                if (p > q) { int t = p; p = q; q = t; }
                cplx* ap = A + (long long)p * n;
                cplx* aq = A + (long long)q * n;
                double al = 0., be = 0., gr = 0., gi = 0.;
                for (int i = lane; i < n; i += 32) {
                    cplx x = ap[i], y = aq[i];
                    al = fma(x.re, x.re, fma(x.im, x.im, al));
                    be = fma(y.re, y.re, fma(y.im, y.im, be));
                    gr = fma(x.re, y.re, fma(x.im, y.im, gr));   // conj(x) y
                    gi = fma(x.re, y.im, fma(-x.im, y.re, gi));
                }
                al = warp_sum(al); be = warp_sum(be); gr = warp_sum(gr); gi = warp_sum(gi);
                double g = hypot(gr, gi);
                if (g == 0. || g <= tol * sqrt(al * be)) continue;
                if (lane == 0) s_rot = 1;
                double zeta = (be - al) / (2. * g);
                double t = (zeta >= 0. ? 1. : -1.) / (fabs(zeta) + sqrt(1. + zeta * zeta));
                double c = 1. / sqrt(1. + t * t), s = c * t;
                // e^{-i phi}, phi = arg(gamma)
                cplx eph = mk(gr / g, -gi / g);
                cplx* vp = V + (long long)p * n;
                cplx* vq = V + (long long)q * n;
                for (int i = lane; i < n; i += 32) {
                    cplx x = ap[i], y = eph * aq[i];
                    ap[i] = c * x - s * y;
                    aq[i] = s * x + c * y;
                    cplx xv = vp[i], yv = eph * vq[i];
                    vp[i] = c * xv - s * yv;
                    vq[i] = s * xv + c * yv;
                }
            }
            __syncthreads();
        }
        if (s_rot == 0) break;
        __syncthreads();
    }
    // column norms = singular values
    double* sig = red + 64;   // n doubles after the reduction scratch
    for (int j = warp; j < n; j += nw) {
        const cplx* aj = A + (long long)j * n;
        double s2 = 0.;
        for (int i = lane; i < n; i += 32) s2 = fma(aj[i].re, aj[i].re, fma(aj[i].im, aj[i].im, s2));
        s2 = warp_sum(s2);
        if (lane == 0) sig[j] = sqrt(s2);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        // index of the (which)-th smallest singular value (ties broken by column index)
        int chosen = 0;
        if (J.which == 0) {
            for (int j = 1; j < n; ++j)
                if (sig[j] < sig[chosen]) chosen = j;
        } else {
            for (int j = 0; j < n; ++j) {
                int rank = 0;
                for (int l = 0; l < n; ++l)
                    if (sig[l] < sig[j] || (sig[l] == sig[j] && l < j)) ++rank;
                if (rank == J.which) { chosen = j; break; }
            }
        }
        s_imin = chosen;
        J.status[mat] = (sweep >= kSvdMaxSweeps) ? 4 : 0;
    }
    __syncthreads();
    if (J.sig_all)
        for (int j = threadIdx.x; j < n; j += blockDim.x) J.sig_all[(long long)mat * n + j] = sig[j];
    const int im = s_imin;
    const double sg = sig[im];
    double* out = J.out + 3LL * mat;
    if (threadIdx.x == 0) { out[0] = sg; out[1] = 0.; out[2] = 0.; }
    if (J.D == 0) return;
    const double isg = sg > 0. ? 1. / sg : 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        ui[i] = isg * A[(long long)im * n + i];
        vi[i] = V[(long long)im * n + i];
    }
    __syncthreads();
    const cplx* T1 = T0 + J.der_stride;
    // y = T' v  (thread per row),  z = T'^H u (thread per column)
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx y = mk(0.);
        for (int c = 0; c < n; ++c) cfma(y, T1[r + (long long)c * n], vi[c]);
        uy[r] = y;
        cplx z = mk(0.);
        const cplx* col = T1 + (long long)r * n;
        for (int i = 0; i < n; ++i) cfma_c(z, col[i], ui[i]);
        uz[r] = z;
    }
    __syncthreads();
    // a_j = u_j^H y, b_j = v_j^H z;  accumulate sigma' and the sigma'' sums
    double part1 = 0., part2 = 0.;
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const cplx* aj = A + (long long)j * n;
        const cplx* vj = V + (long long)j * n;
        cplx a = mk(0.), b = mk(0.);
        for (int i = 0; i < n; ++i) {
            cfma_c(a, aj[i], uy[i]);
            cfma_c(b, vj[i], uz[i]);
        }
        double sj = sig[j];
        a = (sj > 0. ? 1. / sj : 0.) * a;
        if (j == im) part1 += a.re;
        cplx pl = a + b, mi = a - b;
        if (j != im && fabs(sj - sg) > 1e-9 * sg) part2 += 0.5 * norm2(pl) / (sg - sj);
        if (sg + sj > 0.) part2 += 0.5 * norm2(mi) / (sg + sj);
    }
    // block reductions
    part1 = warp_sum(part1);
    part2 = warp_sum(part2);
    if (lane == 0) { red[warp] = part1; red[32 + warp] = part2; }
    __syncthreads();
    double d1 = 0., d2s = 0.;
    if (threadIdx.x == 0) {
        for (int w = 0; w < nw; ++w) { d1 += red[w]; d2s += red[32 + w]; }
        out[1] = d1;
    }
    if (J.D < 2) return;
    __syncthreads();
    const cplx* T2 = T0 + 2 * J.der_stride;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx y = mk(0.);
        for (int c = 0; c < n; ++c) cfma(y, T2[r + (long long)c * n], vi[c]);
        uy[r] = y;
    }
    __syncthreads();
    double p3 = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        cplx t = conj(ui[i]) * uy[i];
        p3 += t.re;
    }
    p3 = warp_sum(p3);
    __syncthreads();
    if (lane == 0) red[warp] = p3;
    __syncthreads();
    if (threadIdx.x == 0) {
        double w2 = 0.;
        for (int w = 0; w < nw; ++w) w2 += red[w];
        out[2] = w2 + d2s;
    }
}

size_t svd_smem_bytes(int n, bool a_in_smem) {
    size_t v = (size_t)4 * n * sizeof(cplx) + (64 + (size_t)n) * sizeof(double);
    return a_in_smem ? v + (size_t)n * n * sizeof(cplx) : v;
}

// FP64 one-sided Jacobi from the identity (every n; A in shared memory when it fits)
cudaError_t launch_svd(int n, int nmat, int D, int which, const cplx* T, long long mat_stride, long long der_stride,
                       cplx* gA, cplx* gV, double* out, double* sig_all, int* status, cudaStream_t st) {
    const size_t limit = 220 * 1024;
    bool in_smem = svd_smem_bytes(n, true) <= limit;
    size_t smem = svd_smem_bytes(n, in_smem);
    cudaError_t e = cudaFuncSetAttribute(k_svd_jacobi<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    SvdJob J{n, nmat, D, which, T, mat_stride, der_stride, gA, gV, out, sig_all, status, in_smem ? 1 : 0};
    k_svd_jacobi<false><<<nmat, kSvdThreads, smem, st>>>(J);
    return cudaGetLastError();
}

// Mixed precision where A fits in shared memory: FP32 Jacobi, FP64 re-start from
// T V, FP64 polishing sweeps (same results to FP64 accuracy, far fewer FP64
// operations); the FP64-only kernel otherwise.
cudaError_t launch_svd_mixed(int n, int nmat, int D, int which, const cplx* T, long long mat_stride,
                             long long der_stride, cplx* gA, cplx* gV, double* out, double* sig_all, int* status,
                             cudaStream_t st) {
    const size_t limit = 220 * 1024;
    if (svd_smem_bytes(n, true) > limit)
        return launch_svd(n, nmat, D, which, T, mat_stride, der_stride, gA, gV, out, sig_all, status, st);
    cudaError_t e = cudaFuncSetAttribute(k_svd_jacobi<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    SvdJob J{n, nmat, D, which, T, mat_stride, der_stride, gA, gV, out, sig_all, status, 1};
    k_svd_jacobi<true><<<nmat, kSvdThreads, svd_smem_bytes(n, true), st>>>(J);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- FP32 Jacobi + FP64 refinement
//
// sigma_min, sigma', sigma'' of one matrix per CTA with O(n^3) work only in FP32
// (the Jacobi sweeps) and in one FP64 LU; everything else in FP64 is O(n^2 k):
//  1. FP32 one-sided Jacobi: all singular triplets to the FP32 noise level.
//  2. The near block: the right vectors of the k = min(n, 8) smallest FP32 singular
//     values.  FP64 LU of T in shared memory; one to four block inverse iterations
//     X <- qr(T^-1 T^-H X); Rayleigh-Ritz: T X = Q_Y R, SVD of the k x k factor R
//     gives FP64 Ritz triplets (sigma_j, u_j, v_j).
//  3. sigma = smallest Ritz value, sigma' = Re u^H T' v.
//  4. sigma'' = Re u^H T'' v + the minus terms of the target and its degenerate
//     partners D (relative gap <= 1e-9; their plus terms are left out as above) +
//     the rest of the second-order sum as a resolvent, 2 Re b_f^H (sigma - W)^-1 b_f,
//     b_f the Wielandt vector W' x projected off D.  (sigma - W)^-1 reduces to
//     y = (T T^H - sigma^2)^+ r on the complement of the left vectors of D, solved by
//     conjugate gradients preconditioned with (T T^H)^-1 = T^-H T^-1 from the same
//     LU: the preconditioned spectrum is 1 - sigma^2 / sigma_j^2.
// A CG that does not converge sets status 4 and a singular LU status 5; the host
// then recomputes the batch with the FP64-polished Jacobi kernel.

// Near-block width: 8 holds the target with a few degenerate pairs (the circle's
// sigma come in pairs) and needs as many inverse iterations as 12 near the minima
// the searches evaluate, at two thirds of the FP64 solve and Rayleigh-Ritz work
// (measured: 142.8 -> 138.0 ms per bench step; 139.7 ms with 10).  At least 8: the
// block's storage doubles as the Jacobi warm start's row buffer (16 warps x n).
constexpr int kFastKmax = 8;
constexpr int kFastInvIter = 4;
constexpr int kFastNeumannMax = 200;   // preconditioned CG iteration cap
// launches of at most this many matrices run the paired (two-CTA cluster) form
static std::atomic<int> g_svd_pair_max{16};
// per host thread: set while long-running launches of other streams keep the GPU full.
// A cluster needs two SMs of one GPC free at once, and the block scheduler fills SMs
// that free one at a time with the other streams' blocks, whatever their priority, so
// a cluster launch waits until those launches have drained; one-CTA launches do not.
thread_local int t_svd_pair_hold = 0;

struct SvdFastJob {
    int n, nmat, D;
    const cplx* T;
    long long mat_stride, der_stride;
    double* out;     // [nmat][3]
    int* status;     // [nmat]
    // optional pool of n x n FP32 right-singular-vector sets: matrix m starts its FP32
    // Jacobi from slot warm_slot[m] (>= 0) and stores its V32 in slot out_slot[m] (>= 0)
    cpf* vpool;
    const int* warm_slot;
    const int* out_slot;
    cplx* uv;        // optional [nmat][2n]: u, v of sigma_min
};

struct FastSmem {
    size_t r0, x, y, w, rf, vec, coef, red, sig32, piv, perm, redi, idx, sigb, ab, total;
};

__host__ __device__ inline FastSmem fast_layout(int n) {
    FastSmem L;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 15) / 16 * 16; return o; };
    const size_t c = sizeof(cplx), K = kFastKmax;
    L.r0 = take((size_t)n * n * c);          // FP32 A32 | V32, then the FP64 LU of T
    L.x = take((size_t)n * K * c);
    L.y = take((size_t)n * K * c);
    L.w = take(K * K * c);
    L.rf = take(K * K * c);
    L.vec = take(9 * (size_t)n * c);
    L.coef = take(K * c);
    L.red = take(128 * sizeof(double));
    L.sig32 = take((size_t)n * sizeof(float));
    L.piv = take((size_t)n * sizeof(int));
    L.perm = take((size_t)n * sizeof(int));
    L.redi = take(32 * sizeof(int));
    L.idx = take(K * sizeof(int));
    L.sigb = take(K * sizeof(double));
    L.ab = take(2 * K * c);
    L.total = off;
    return L;
}

size_t svd_fast_smem_bytes(int n) { return fast_layout(n).total; }

// y = A x for the global column-major n x n matrix A: four consecutive lanes per
// row, each over every fourth column (four times the loads in flight of a thread per
// row), summed by shuffles within the four
static __device__ void gemv_n(const cplx* A, int n, const cplx* x, cplx* y) {
    const int sub = threadIdx.x & 3;
    const unsigned gmask = 0xFu << (threadIdx.x & 28);
    for (int r = threadIdx.x >> 2; r < n; r += blockDim.x >> 2) {
        cplx a = mk(0.);
        for (int c = sub; c < n; c += 4) cfma(a, A[r + (long long)c * n], x[c]);
        a.re += __shfl_xor_sync(gmask, a.re, 1);
        a.im += __shfl_xor_sync(gmask, a.im, 1);
        a.re += __shfl_xor_sync(gmask, a.re, 2);
        a.im += __shfl_xor_sync(gmask, a.im, 2);
        if (sub == 0) y[r] = a;
    }
    __syncthreads();
}

// y = A^H x (warp per column)
static __device__ void gemv_h(const cplx* A, int n, const cplx* x, cplx* y) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int c = warp; c < n; c += nw) {
        const cplx* col = A + (long long)c * n;
        double sr = 0., si = 0.;
        for (int r = lane; r < n; r += 32) {
            const cplx a = conj(col[r]), b = x[r];
            sr = fma(a.re, b.re, fma(-a.im, b.im, sr));
            si = fma(a.re, b.im, fma(a.im, b.re, si));
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        if (lane == 0) y[c] = mk(sr, si);
    }
    __syncthreads();
}

// out[j] = B[:, j]^H x for the kb columns of B (n x kb, leading dimension n)
static __device__ void dots_h(const cplx* B, int n, int kb, const cplx* x, cplx* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = warp; j < kb; j += nw) {
        const cplx* b = B + (long long)j * n;
        double sr = 0., si = 0.;
        for (int r = lane; r < n; r += 32) {
            const cplx a = conj(b[r]), v = x[r];
            sr = fma(a.re, v.re, fma(-a.im, v.im, sr));
            si = fma(a.re, v.im, fma(a.im, v.re, si));
        }
        sr = warp_sum(sr);
        si = warp_sum(si);
        if (lane == 0) out[j] = mk(sr, si);
    }
    __syncthreads();
}

// x <- x - B c  (B n x kb)
static __device__ void sub_span(const cplx* B, int n, int kb, const cplx* c, cplx* x) {
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx v = x[r];
        for (int j = 0; j < kb; ++j) cfms(v, B[r + (long long)j * n], c[j]);
        x[r] = v;
    }
    __syncthreads();
}

static __device__ double dot_re(const cplx* a, const cplx* b, int n, double* red) {
    double part = 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) part += a[r].re * b[r].re + a[r].im * b[r].im;
    return bsum(part, red);
}

// Rows of B (n x kb) times the kb x kb matrix M, in place, row by row.
static __device__ void rows_times(cplx* B, int n, int kb, const cplx* M) {
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx row[kFastKmax], outr[kFastKmax];
#pragma unroll
        for (int j = 0; j < kFastKmax; ++j) row[j] = j < kb ? B[r + (long long)j * n] : mk(0.);
#pragma unroll
        for (int j = 0; j < kFastKmax; ++j) {
            cplx a = mk(0.);
#pragma unroll
            for (int l = 0; l < kFastKmax; ++l)
                if (l < kb) cfma(a, row[l], M[l + j * kb]);
            outr[j] = a;
        }
#pragma unroll
        for (int j = 0; j < kFastKmax; ++j)
            if (j < kb) B[r + (long long)j * n] = outr[j];
    }
    __syncthreads();
}

// PAIR: a cluster of two CTAs per matrix (blocks 2m, 2m + 1), for launches of a few
// matrices where the latency of one matrix matters.  CTA 0 runs stage 1 (FP32 Jacobi,
// near block) while CTA 1 factors T in FP64; CTA 0 then copies the factors out of CTA
// 1's shared memory and the two split the columns of the inverse iterations and of
// Y = T X between them, exchanging columns through distributed shared memory; CTA 1
// finishes alone.  Every column sees the single-CTA kernel's arithmetic in the same
// order, so both forms give bit-identical results.
template <bool PAIR>
__global__ void __launch_bounds__(kSvdThreads) k_svd_fast(SvdFastJob J) {
    extern __shared__ double smraw[];
    char* sb = reinterpret_cast<char*>(smraw);
    const int n = J.n, mat = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    int rank = 0;   // PAIR: 0 = the Jacobi CTA, 1 = the LU CTA
    if constexpr (PAIR) {
        rank = (int)cg::this_cluster().block_rank();
        cg::this_cluster().sync();   // both CTAs are running before either touches the other's memory
    }
    const FastSmem L = fast_layout(n);
    cplx* T64 = reinterpret_cast<cplx*>(sb + L.r0);
    cpf* A32 = reinterpret_cast<cpf*>(sb + L.r0);
    cpf* V32 = A32 + (long long)n * n;
    cplx* X = reinterpret_cast<cplx*>(sb + L.x);
    cplx* Y = reinterpret_cast<cplx*>(sb + L.y);
    cplx* W = reinterpret_cast<cplx*>(sb + L.w);
    cplx* Rf = reinterpret_cast<cplx*>(sb + L.rf);
    cplx* vec = reinterpret_cast<cplx*>(sb + L.vec);
    cplx* coef = reinterpret_cast<cplx*>(sb + L.coef);
    double* red = reinterpret_cast<double*>(sb + L.red);
    float* sig32 = reinterpret_cast<float*>(sb + L.sig32);
    int* piv = reinterpret_cast<int*>(sb + L.piv);
    int* perm = reinterpret_cast<int*>(sb + L.perm);
    int* idx = reinterpret_cast<int*>(sb + L.idx);
    double* sigb = reinterpret_cast<double*>(sb + L.sigb);
    cplx* ab = reinterpret_cast<cplx*>(sb + L.ab);   // a_j, b_j
    cplx *F = vec, *G = vec + n, *f1 = vec + 2 * n, *f2 = vec + 3 * n, *rr = vec + 4 * n, *acc = vec + 5 * n,
         *term = vec + 6 * n, *z2 = vec + 7 * n, *sbuf = vec + 8 * n;
    __shared__ int s_rot, s_kb, s_im, s_sing, s_conv, s_iters, s_next;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const cplx* T0 = J.T + (long long)mat * J.mat_stride;
    double* out = J.out + 3LL * mat;

    const long long nn = (long long)n * n;
    if (!PAIR || rank == 0) {
    // 1. FP32 Jacobi, from the pool's V set of a nearby wavenumber when given
    const int wslot = (J.vpool && J.warm_slot) ? J.warm_slot[mat] : -1;
    const int oslot = (J.vpool && J.out_slot) ? J.out_slot[mat] : -1;
    jacobi_fp32(T0, n, A32, V32, &s_rot, wslot >= 0 ? J.vpool + wslot * nn : nullptr, reinterpret_cast<cpf*>(X));
    if (oslot >= 0) {
        cpf* dst = J.vpool + oslot * nn;
        for (long long e = threadIdx.x; e < nn; e += blockDim.x) dst[e] = V32[e];
    }
    for (int j = warp; j < n; j += nw) {
        float s2 = 0.f;
        for (int i = lane; i < n; i += 32) s2 = fmaf(A32[j * n + i].re, A32[j * n + i].re,
                                                     fmaf(A32[j * n + i].im, A32[j * n + i].im, s2));
        s2 = warp_sumf(s2);
        if (lane == 0) sig32[j] = sqrtf(s2);
    }
    __syncthreads();
    // 2. near block: the kb smallest FP32 singular values (ascending, ties by index):
    // column j goes to position rank(j) when that is below kb; the column of rank kb
    // (the next singular value) bounds the inverse iterations' convergence below
    if (threadIdx.x == 0) s_next = -1;
    __syncthreads();
    {
        const int kbs = min(n, kFastKmax);
        // NaN (non-finite T) sorts as +inf, so the ranks stay a permutation of 0..n-1
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            const float sj = isnan(sig32[j]) ? INFINITY : sig32[j];
            int rank = 0;
            for (int i = 0; i < n; ++i) {
                const float si = isnan(sig32[i]) ? INFINITY : sig32[i];
                rank += (si < sj || (si == sj && i < j)) ? 1 : 0;
            }
            if (rank < kbs) idx[rank] = j;
            if (rank == kbs) s_next = j;   // exactly one column when n > kb
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int kb = min(n, kFastKmax);
        s_kb = kb;
        // Block inverse iterations: the start block's components outside the kb
        // smallest singular directions shrink by (sigma_1 / sigma_kb+1)^2 per iteration.
        // Four iterations at a ratio of 1/3 (a factor 3^-8) are the least reduction the
        // kernel accepts; with a margin of 100 (and the FP32 values' absolute error
        // 4 eps32 sigma_max added to the ratio) fewer iterations reach it when the
        // smallest singular value is well separated, as it is near a resonance.
        int iters = kFastInvIter;
        if (n > kb && s_next >= 0) {
            float smax = 0.f;
            for (int j = 0; j < n; ++j) smax = fmaxf(smax, sig32[j]);
            const float snext = sig32[s_next];
            const double err = 4.0 * 1.1920928955078125e-7 * (double)smax;
            const double lo = (double)snext - err;
            if (lo > 0.) {
                const double r = ((double)sig32[idx[0]] + err) / lo;
                if (r < 1.) {
                    const double need = log(100.0 * 6561.0) / (2.0 * log(1.0 / r));
                    iters = min(kFastInvIter, max(1, (int)ceil(need)));
                }
            }
        }
        s_iters = iters;
    }
    __syncthreads();
    {
        const int kb = s_kb;
        for (int e = threadIdx.x; e < n * kb; e += blockDim.x) {
            const cpf v = V32[idx[e / n] * n + e % n];
            X[e] = mk((double)v.re, (double)v.im);
        }
        __syncthreads();
        if constexpr (PAIR) {   // the start block and its two counts to CTA 1
            cg::cluster_group cl = cg::this_cluster();
            cplx* Xr = cl.map_shared_rank(X, 1);
            for (int e = threadIdx.x; e < n * kb; e += blockDim.x) Xr[e] = X[e];
            if (threadIdx.x == 0) {
                *cl.map_shared_rank(&s_kb, 1) = kb;
                *cl.map_shared_rank(&s_iters, 1) = s_iters;
            }
        }
    }
    }   // stage 1
    if (!PAIR || rank == 1) {
        // FP64 LU of T (in the single-CTA form over the FP32 work space)
        if (threadIdx.x == 0) s_sing = 0;
        for (int e = threadIdx.x; e < n * n; e += blockDim.x) T64[e] = T0[e];
        __syncthreads();
        lu_smem(T64, n, piv, &s_sing, sbuf);
        perm_from_piv(piv, n, perm);
        // U's diagonal replaced by its reciprocals: the solves below multiply
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            const cplx d = T64[k + (long long)k * n];
            T64[k + (long long)k * n] = norm2(d) > 0. ? cdiv(mk(1.), d) : mk(0.);
        }
        __syncthreads();
    }
    if constexpr (PAIR) {
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();   // CTA 1 holds the start block; CTA 0 is done with its FP32 work space
        if (rank == 0) {   // the factors and the permutation from CTA 1
            const cplx* Tr = cl.map_shared_rank(T64, 1);
            for (long long e = threadIdx.x; e < nn; e += blockDim.x) T64[e] = Tr[e];
            const int* pr = cl.map_shared_rank(perm, 1);
            for (int i = threadIdx.x; i < n; i += blockDim.x) perm[i] = pr[i];
            __syncthreads();
        }
    }
    const int kb = s_kb;
    qr_cgs2(X, n, kb, coef, red);
    // the columns this CTA iterates on: all of them, or its half in the paired form
    int col0 = 0, cnt = kb;
    if constexpr (PAIR) {
        const int h = (kb + 1) / 2;
        col0 = rank ? h : 0;
        cnt = rank ? kb - h : h;
    }
    cplx* Xc = X + (long long)col0 * n;
    const int inv_iters = s_iters;
    for (int it = 0; it < inv_iters; ++it) {   // Y is free until the Rayleigh-Ritz step
        solve_lu_h_blk(T64, perm, n, Xc, cnt, sbuf, Y, true);
        solve_lu_blk(T64, perm, n, Xc, cnt, sbuf, Y, true);
        if constexpr (PAIR) {   // each CTA's columns to the other, then both orthonormalise all
            cg::cluster_group cl = cg::this_cluster();
            cl.sync();   // the other CTA has finished reading its block (the last QR)
            cplx* Xr = cl.map_shared_rank(Xc, rank ^ 1);
            for (int e = threadIdx.x; e < n * cnt; e += blockDim.x) Xr[e] = Xc[e];
            cl.sync();
        }
        qr_cgs2(X, n, kb, coef, red);
    }
    // Rayleigh-Ritz: Y = T X = Q_Y Rf, Rf W = Q_R Sigma.  One thread per entry of Y:
    // consecutive threads take consecutive rows (coalesced reads of T's columns from
    // global memory), X's entries are shared-memory broadcasts.  Paired: CTA 0 writes
    // its columns straight into CTA 1's Y and leaves.
    {
        cplx* Yd = Y;
        if constexpr (PAIR) Yd = cg::this_cluster().map_shared_rank(Y, 1);
        for (int e = threadIdx.x; e < n * cnt; e += blockDim.x) {
            const int r = e % n, j = col0 + e / n;
            const cplx* xj = X + (long long)j * n;
            cplx a0 = mk(0.), a1 = mk(0.);
            int c = 0;
            for (; c + 1 < n; c += 2) {
                cfma(a0, T0[r + (long long)c * n], xj[c]);
                cfma(a1, T0[r + (long long)(c + 1) * n], xj[c + 1]);
            }
            if (c < n) cfma(a0, T0[r + (long long)c * n], xj[c]);
            Yd[r + (long long)j * n] = a0 + a1;
        }
    }
    if constexpr (PAIR) {
        cg::this_cluster().sync();
        if (rank == 0) return;
    }
    __syncthreads();
    qr_cgs2(Y, n, kb, coef, red, Rf);
    jacobi_cta(Rf, kb, W, &s_rot);
    if (threadIdx.x < kb) {
        double s2 = 0.;
        for (int r = 0; r < kb; ++r) s2 += norm2(Rf[threadIdx.x * kb + r]);
        sigb[threadIdx.x] = sqrt(s2);
    }
    __syncthreads();
    // Q_R = (Rf W) Sigma^-1 in place
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const double sj = sigb[e / kb];
        Rf[e] = (sj > 0. ? 1. / sj : 0.) * Rf[e];
    }
    __syncthreads();
    rows_times(X, n, kb, W);     // V_b = X W
    rows_times(Y, n, kb, Rf);    // U_b = Q_Y Q_R
    if (threadIdx.x == 0) {
        int im = 0;
        for (int j = 1; j < kb; ++j)
            if (sigb[j] < sigb[im]) im = j;
        s_im = im;
        s_conv = 1;
    }
    __syncthreads();
    const int im = s_im;
    const double sg = sigb[im];
    const cplx* u = Y + (long long)im * n;
    const cplx* v = X + (long long)im * n;
    if (threadIdx.x == 0) {
        out[0] = sg;
        out[1] = 0.;
        out[2] = 0.;
    }
    if (J.uv)
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            J.uv[2LL * n * mat + r] = u[r];
            J.uv[2LL * n * mat + n + r] = v[r];
        }
    if (J.D == 0) {
        if (threadIdx.x == 0) J.status[mat] = s_sing ? 5 : 0;
        return;
    }
    // 3. sigma'
    const cplx* T1 = T0 + J.der_stride;
    gemv_n(T1, n, v, F);
    const double d1 = dot_re(u, F, n, red);
    if (threadIdx.x == 0) out[1] = d1;
    if (J.D == 1) {
        if (threadIdx.x == 0) J.status[mat] = s_sing ? 5 : 0;
        return;
    }
    // 4. sigma''
    const cplx* T2 = T0 + 2 * J.der_stride;
    gemv_n(T2, n, v, acc);
    const double c0 = dot_re(u, acc, n, red + 32);
    gemv_h(T1, n, u, G);
    cplx* a_j = ab;
    cplx* b_j = ab + kFastKmax;
    dots_h(Y, n, kb, F, a_j);
    dots_h(X, n, kb, G, b_j);
    // D: the target and its numerically degenerate partners (relative gap <= 1e-9);
    // their minus terms explicitly, every other triplet through the resolvent
    if (threadIdx.x == 0) {
        int nd = 0;
        for (int j = 0; j < kb; ++j)
            if (j == im || fabs(sigb[j] - sg) <= 1e-9 * sg) idx[nd++] = j;
        s_kb = nd;
    }
    __syncthreads();
    const int nd = s_kb;
    double near_sum = 0.;
    for (int l = 0; l < nd; ++l) {
        const int j = idx[l];
        const double sj = sigb[j];
        const cplx mi = a_j[j] - b_j[j];
        if (sg + sj > 0.) near_sum += 0.5 * norm2(mi) / (sg + sj);
    }
    // gather the D columns of U_b, V_b to the front (Y, X columns 0..nd-1)
    for (int e = threadIdx.x; e < n; e += blockDim.x) {
        cplx uu[kFastKmax], vv[kFastKmax];
        for (int l = 0; l < nd; ++l) {
            uu[l] = Y[e + (long long)idx[l] * n];
            vv[l] = X[e + (long long)idx[l] * n];
        }
        for (int l = 0; l < nd; ++l) {
            Y[e + (long long)l * n] = uu[l];
            X[e + (long long)l * n] = vv[l];
        }
    }
    __syncthreads();
    // b_f = (P_U T' v; P_V T'^H u) / sqrt2 with P_U, P_V projecting off D
    const double is2 = 0.70710678118654752440;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        f1[r] = is2 * F[r];
        f2[r] = is2 * G[r];
    }
    __syncthreads();
    dots_h(Y, n, nd, f1, coef);
    sub_span(Y, n, nd, coef, f1);
    dots_h(X, n, nd, f2, coef);
    sub_span(X, n, nd, coef, f2);
    // y = (T T^H - sigma^2)^+ (sigma f1 + T f2) on the complement of U_D: preconditioned
    // CG with M = (T T^H)^-1 = T^-H T^-1 (eigenvalues of M A: 1 - sigma^2 / sigma_j^2)
    gemv_n(T0, n, f2, rr);
    for (int r = threadIdx.x; r < n; r += blockDim.x) rr[r] = sg * f1[r] + rr[r];   // residual (y = 0)
    __syncthreads();
    dots_h(Y, n, nd, rr, coef);
    sub_span(Y, n, nd, coef, rr);
    cplx* yv = acc;
    cplx* pv = term;
    cplx* zv = z2;      // preconditioned residual, later reused
    cplx* ap = G;       // A p (T'^H u no longer needed)
    cplx* tmp = F;      // T^H p (T' v no longer needed)
    const double s2 = sg * sg;
    for (int r = threadIdx.x; r < n; r += blockDim.x) { yv[r] = mk(0.); zv[r] = rr[r]; }
    __syncthreads();
    solve_lu_blk(T64, perm, n, zv, 1, sbuf, nullptr, true);                 // z = T^-H T^-1 res
    solve_lu_h_blk(T64, perm, n, zv, 1, sbuf, nullptr, true);
    dots_h(Y, n, nd, zv, coef);
    sub_span(Y, n, nd, coef, zv);
    for (int r = threadIdx.x; r < n; r += blockDim.x) pv[r] = zv[r];
    __syncthreads();
    double rz = dot_re(rr, zv, n, red);
    const double rz0 = rz;
    int it = 0;
    for (; it < kFastNeumannMax && rz > 1e-32 * rz0 && rz > 0.; ++it) {
        gemv_h(T0, n, pv, tmp);                    // A p = T T^H p - sigma^2 p
        gemv_n(T0, n, tmp, ap);
        for (int r = threadIdx.x; r < n; r += blockDim.x) ap[r] = ap[r] - s2 * pv[r];
        __syncthreads();
        dots_h(Y, n, nd, ap, coef);
        sub_span(Y, n, nd, coef, ap);
        const double pap = dot_re(pv, ap, n, red + 32);
        if (!(pap > 0.)) break;
        const double alpha = rz / pap;
        for (int r = threadIdx.x; r < n; r += blockDim.x) {
            yv[r] += alpha * pv[r];
            rr[r] -= alpha * ap[r];
            zv[r] = rr[r];
        }
        __syncthreads();
        solve_lu_blk(T64, perm, n, zv, 1, sbuf, nullptr, true);
        solve_lu_h_blk(T64, perm, n, zv, 1, sbuf, nullptr, true);
        dots_h(Y, n, nd, zv, coef);
        sub_span(Y, n, nd, coef, zv);
        const double rz1 = dot_re(rr, zv, n, red + 64);
        const double beta = rz1 / rz;
        rz = rz1;
        for (int r = threadIdx.x; r < n; r += blockDim.x) pv[r] = zv[r] + beta * pv[r];
        __syncthreads();
    }
    if (threadIdx.x == 0 && rz > 1e-24 * rz0) s_conv = 0;
    for (int r = threadIdx.x; r < n; r += blockDim.x) yv[r] = -yv[r];   // z1
    __syncthreads();
    gemv_h(T0, n, yv, z2);
    const double isg = sg > 0. ? 1. / sg : 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) z2[r] = isg * (f2[r] + z2[r]);
    __syncthreads();
    const double far = dot_re(f1, yv, n, red) + dot_re(f2, z2, n, red + 32);
    if (threadIdx.x == 0) {
        out[2] = c0 + near_sum + 2. * far;
        J.status[mat] = s_sing ? 5 : (s_conv ? 0 : 4);
    }
}

// sigma' = Re u^H T' v for nmat derivative matrices T'_m (column-major n x n at
// T1 + m * mat_stride) with the singular vectors (u, v) = uv + 2 n idx[m] of the same
// wavenumber from an earlier dense-sigma launch: one CTA per matrix, a thread per row.
__global__ void __launch_bounds__(128) k_sigma1_uv(int n, const cplx* T1, long long mat_stride, const cplx* uv,
                                                   const int* idx, double* d1) {
    __shared__ double red[32];
    const int m = blockIdx.x;
    const cplx* A = T1 + (long long)m * mat_stride;
    const cplx* u = uv + 2LL * n * idx[m];
    const cplx* v = u + n;
    double part = 0.;
    for (int r = threadIdx.x; r < n; r += blockDim.x) {
        cplx w = mk(0.);
        for (int c = 0; c < n; ++c) cfma(w, A[r + (long long)c * n], v[c]);
        part += u[r].re * w.re + u[r].im * w.im;
    }
    const double tot = bsum(part, red);
    if (threadIdx.x == 0) d1[m] = tot;
}

cudaError_t launch_sigma1_uv(int n, int nmat, const cplx* T1, long long mat_stride, const cplx* uv, const int* idx,
                             double* d1, cudaStream_t st) {
    k_sigma1_uv<<<nmat, 128, 0, st>>>(n, T1, mat_stride, uv, idx, d1);
    return cudaGetLastError();
}

cudaError_t launch_svd_fast(int n, int nmat, int D, const cplx* T, long long mat_stride, long long der_stride,
                            double* out, int* status, cudaStream_t st, cplxf* vpool, const int* warm_slot,
                            const int* out_slot, cplx* uv) {
    const size_t limit = 220 * 1024, smem = svd_fast_smem_bytes(n);
    if (smem > limit || n < 2) return cudaErrorInvalidValue;
    SvdFastJob J{n, nmat, D, T, mat_stride, der_stride, out, status, vpool, warm_slot, out_slot, uv};
    if (t_svd_pair_hold || nmat > g_svd_pair_max.load(std::memory_order_relaxed)) {
        cudaError_t e = cudaFuncSetAttribute(k_svd_fast<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
        if (e != cudaSuccess) return e;
        k_svd_fast<false><<<nmat, kSvdThreads, smem, st>>>(J);
        return cudaGetLastError();
    }
    cudaError_t e = cudaFuncSetAttribute(k_svd_fast<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * nmat);
    cfg.blockDim = dim3(kSvdThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_svd_fast<true>, J);
}

void svd_set_pair_max(int m) { g_svd_pair_max = m < 0 ? 0 : m; }
int svd_get_pair_max() { return g_svd_pair_max.load(); }
void svd_pair_hold(int on) { t_svd_pair_hold = on ? 1 : 0; }

// ---------------------------------------------------------------- allocation-free variant
//
// Working memory of hbem_sv_dense_batch_noalloc: the right singular vectors V of
// every matrix in the batch (nmat * n * n complex128).  It is a fixed array in
// this library's device image, so every GPU that loads the library holds these
// 8 MiB until the process exits.
constexpr size_t kNoAllocScratchElems = size_t(1) << 19;   // complex128 elements: 8 MiB
static __device__ __align__(256) cplx g_noalloc_scratch[kNoAllocScratchElems];

int set_error(int code, const char* msg);

}  // namespace hbem

#include <mutex>

#include "../../include/hbem.h"

namespace {
std::mutex g_noalloc_mu;
constexpr int kMaxDevices = 64;
void* g_noalloc_ptr[kMaxDevices] = {nullptr};   // device address of the scratch, per device

// p points into device (or managed) memory that device dev can use directly
bool on_device(const void* p, int dev) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();   // the failed query's error is not the caller's
        return false;
    }
    if (a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeDevice && a.device == dev;
}
}  // namespace

// See include/hbem.h.  The matrix must fit in shared memory (n <= 116) because the
// allocation-free path has no global scratch for A; V lives in the fixed array.
extern "C" int hbem_sv_dense_batch_noalloc(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                                           long long der_stride, double* out_dev, int* status_dev, void* stream) {
    using namespace hbem;
    if (n < 2 || nmat < 1 || d > 2 || !T_dev || !out_dev || !status_dev)
        return set_error(HBEM_ERR_INVALID, "sv_dense_batch_noalloc: bad argument");
    if (svd_smem_bytes(n, true) > 220 * 1024)
        return set_error(HBEM_ERR_INVALID, "sv_dense_batch_noalloc: matrix order above 116 (the matrix must fit in shared memory)");
    if ((size_t)nmat * (size_t)n * (size_t)n > kNoAllocScratchElems)
        return set_error(HBEM_ERR_INVALID,
                         "sv_dense_batch_noalloc: nmat * n * n exceeds the fixed scratch of 524288 complex elements (8 MiB)");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(HBEM_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return set_error(HBEM_ERR_INVALID, "sv_dense_batch_noalloc: device ordinal out of range");
    // the kernel reads T and writes out / status on the current device: pointers to
    // host memory or to another device are refused here (no allocation involved)
    const void* ptrs[3] = {T_dev, out_dev, status_dev};
    for (const void* q : ptrs) {
        if (!on_device(q, dev))
            return set_error(HBEM_ERR_INVALID,
                             "sv_dense_batch_noalloc: T_dev, out_dev and status_dev must be memory of the current device");
    }
    void* scratch = nullptr;
    {
        // first call on a device: resolve the device address of the fixed array with
        // that device current (the host-side name is only a stand-in, not a device
        // address).  A cached address that no longer maps this device's memory (the
        // device was reset since) is resolved again.
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (g_noalloc_ptr[dev] && !on_device(g_noalloc_ptr[dev], dev)) g_noalloc_ptr[dev] = nullptr;
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess) return set_error(HBEM_ERR_CUDA, cudaGetErrorString(e));
            g_noalloc_ptr[dev] = p;
        }
        scratch = g_noalloc_ptr[dev];
    }
    e = launch_svd(n, nmat, (int)d, 0, static_cast<const cplx*>(T_dev), mat_stride, der_stride, nullptr,
                   static_cast<cplx*>(scratch), out_dev, nullptr, status_dev, static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return set_error(HBEM_ERR_CUDA, cudaGetErrorString(e));
    return HBEM_OK;
}
