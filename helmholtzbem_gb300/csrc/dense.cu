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
#include "hbem_device.cuh"

namespace hbem {

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
__device__ void jacobi_fp32(const cplx* T0, int n, cpf* A32, cpf* V32, int* s_rot) {
    const int np = n + (n & 1), m = np - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        cplx t = T0[e];
        A32[e] = mkf((float)t.re, (float)t.im);
        V32[e] = mkf((e % n) == (e / n) ? 1.f : 0.f, 0.f);
    }
    __syncthreads();
    const float tol = 4e-6f;
    for (int sweep = 0; sweep < 30; ++sweep) {
        if (threadIdx.x == 0) *s_rot = 0;
        __syncthreads();
        for (int r = 0; r < m; ++r) {
            for (int k = warp; k < np / 2; k += nw) {
                int p, q;
                rr_pair(r, k, m, p, q);
                if (p >= n || q >= n) continue;
                if (p > q) { int t = p; p = q; q = t; }
                cpf* ap = A32 + p * n;
                cpf* aq = A32 + q * n;
                float al = 0.f, be = 0.f, gr = 0.f, gi = 0.f;
                for (int i = lane; i < n; i += 32) {
                    cpf x = ap[i], y = aq[i];
                    al = fmaf(x.re, x.re, fmaf(x.im, x.im, al));
                    be = fmaf(y.re, y.re, fmaf(y.im, y.im, be));
                    gr = fmaf(x.re, y.re, fmaf(x.im, y.im, gr));
                    gi = fmaf(x.re, y.im, fmaf(-x.im, y.re, gi));
                }
                al = warp_sumf(al); be = warp_sumf(be); gr = warp_sumf(gr); gi = warp_sumf(gi);
                float g = hypotf(gr, gi);
                if (g == 0.f || g <= tol * sqrtf(al * be)) continue;
                if (lane == 0) *s_rot = 1;
                float zeta = (be - al) / (2.f * g);
                float t = (zeta >= 0.f ? 1.f : -1.f) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
                float c = 1.f / sqrtf(1.f + t * t), s = c * t;
                float er = gr / g, ei = -gi / g;
                cpf* vp = V32 + p * n;
                cpf* vq = V32 + q * n;
                for (int i = lane; i < n; i += 32) {
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
            for (int i = 0; i < j; ++i) s -= V[(long long)i * n + r] * coef[i];
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
        for (int k = 0; k < n; ++k) s += T0[r + (long long)k * n] * vc[k];
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
        for (int c = 0; c < n; ++c) y += T1[r + (long long)c * n] * vi[c];
        uy[r] = y;
        cplx z = mk(0.);
        const cplx* col = T1 + (long long)r * n;
        for (int i = 0; i < n; ++i) z += conj(col[i]) * ui[i];
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
            a += conj(aj[i]) * uy[i];
            b += conj(vj[i]) * uz[i];
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
        for (int c = 0; c < n; ++c) y += T2[r + (long long)c * n] * vi[c];
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
    void* scratch = nullptr;
    {
        // first call on a device: resolve the device address of the fixed array with
        // that device current (the host-side name is only a stand-in, not a device address)
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
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
