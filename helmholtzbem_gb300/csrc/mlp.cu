// The learned resonance proposal's network: a multilayer perceptron
//   n_in -> width (GELU) -> ... -> width (GELU) -> n_out
// trained and evaluated on the GPU in BF16 with FP32 accumulation (weights kept in
// FP32 for the optimiser, BF16 copies for the products).
//
// Every product is one kernel: C (FP32, M x N, row-major) = A (BF16, M x K, row-major)
// x B (BF16, N x K, row-major)^T on the 5th-generation tensor cores (tcgen05.mma
// kind::f16 with BF16 operands, FP32 accumulator in tensor memory), 128 x 128 tiles,
// K in chunks of 64 staged in 128-byte-swizzled K-major shared memory.  Forward
// Y = X W^T; backward dX = dY W (B operand W^T), dW = dY^T X (operands transposed
// into K-major copies first).  Bias, GELU, the loss and Adam are elementwise kernels.
// Shapes are padded on the host: rows and columns to multiples of 128, K to 64.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "../../include/hbem.h"

namespace hbem {

int set_error(int code, const char* msg);
void count_launches(long long n);

namespace {

constexpr int kGM = 128, kGN = 128, kGK = 64;
constexpr int kGThreads = 256;
constexpr uint32_t kGTileBytes = 128u * 128u;       // 128 rows x 128 bytes (64 BF16)
constexpr size_t kGSmemBytes = 2 * (size_t)kGTileBytes + 1024;
constexpr uint32_t kGTmemCols = 128;
constexpr long long kGSpinCap = 1LL << 24;

// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28
constexpr uint32_t kGIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kGN >> 3) << 17) |
                             ((uint32_t)(kGM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor for a 128-byte-swizzled K-major operand: start
// address >> 4, leading byte offset 1 (unused), stride byte offset 1024 >> 4 between
// 8-row groups, version 1, swizzle mode 128 B
__device__ __forceinline__ uint64_t sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

// byte offset of 16-byte chunk c (0..7) of row r in a 128-row swizzled tile
__device__ __forceinline__ uint32_t chunk_off(int r, int c) {
    return (uint32_t)(r >> 3) * 1024u + (uint32_t)(r & 7) * 128u + ((uint32_t)(c ^ (r & 7)) << 4);
}

struct GemmJob {
    int M, N, K;                 // multiples of 128, 128, 64
    const __nv_bfloat16* A;      // M x K, leading dimension lda (multiple of 8)
    const __nv_bfloat16* B;      // N x K, leading dimension ldb
    float* C;                    // M x N, leading dimension ldc
    long long lda, ldb, ldc;
    int* err;
};

__global__ void __launch_bounds__(kGThreads) k_gemm_bf16_tc(GemmJob J) {
    extern __shared__ uint8_t g_smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(g_smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* As = base;
    uint8_t* Bs = base + kGTileBytes;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r0 = blockIdx.x * kGM, c0 = blockIdx.y * kGN;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(kGTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t taddr = tmem_slot, mbar_addr = smem_addr(&mbar);
    const int nk = J.K / kGK;
    for (int kc = 0; kc < nk; ++kc) {
        // stage A and B chunks: 128 rows x 8 16-byte chunks each, 4 + 4 per thread
        uint4 va[4], vb[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * kGThreads, r = e >> 3, c = e & 7;
            va[q] = *reinterpret_cast<const uint4*>(J.A + (long long)(r0 + r) * J.lda + kc * kGK + 8 * c);
            vb[q] = *reinterpret_cast<const uint4*>(J.B + (long long)(c0 + r) * J.ldb + kc * kGK + 8 * c);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * kGThreads, r = e >> 3, c = e & 7;
            *reinterpret_cast<uint4*>(As + chunk_off(r, c)) = va[q];
            *reinterpret_cast<uint4*>(Bs + chunk_off(r, c)) = vb[q];
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            for (int kk = 0; kk < kGK / 16; ++kk) {
                const uint64_t ad = sw128(smem_addr(As) + (uint32_t)kk * 32u);
                const uint64_t bd = sw128(smem_addr(Bs) + (uint32_t)kk * 32u);
                const uint32_t acc = (kc > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
                    "l"(ad), "l"(bd), "r"(kGIdesc), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_addr)
                         : "memory");
        }
        // the staged chunk is read by the MMAs: wait (bounded) before the next overwrite
        uint32_t done = 0;
        for (long long it = 0; it < kGSpinCap && !done; ++it)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(mbar_addr), "r"((uint32_t)(kc & 1))
                : "memory");
        if (!done) s_fail = 1;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        __syncthreads();
        if (s_fail) break;
    }
    if (!s_fail) {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (rows), columns 64 (w / 4) .. + 63
        const int wq = warp & 3, half = warp >> 2;
        const int row = r0 + wq * 32 + lane;
        const uint32_t lane_base = taddr + ((uint32_t)(wq * 32) << 16);
        for (int j0 = half * 64; j0 < half * 64 + 64; j0 += 16) {
            uint32_t v[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(lane_base + (uint32_t)j0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float* out = J.C + (long long)row * J.ldc + c0 + j0;
#pragma unroll
            for (int jj = 0; jj < 16; jj += 4)
                *reinterpret_cast<float4*>(out + jj) = make_float4(__uint_as_float(v[jj]), __uint_as_float(v[jj + 1]),
                                                                   __uint_as_float(v[jj + 2]),
                                                                   __uint_as_float(v[jj + 3]));
        }
    } else if (tid == 0) {
        atomicExch(J.err, 1);
        uint32_t done = 0;
        for (long long it = 0; it < kGSpinCap && !done; ++it)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(mbar_addr), "r"(0u)
                : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kGTmemCols));
    }
}

// FP32 FMA reference of the same product (one thread per output), for tests
__global__ void k_gemm_bf16_simt(GemmJob J) {
    const int i = blockIdx.y, j = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= J.M || j >= J.N) return;
    float acc = 0.f;
    for (int k = 0; k < J.K; ++k)
        acc = fmaf(__bfloat162float(J.A[(long long)i * J.lda + k]), __bfloat162float(J.B[(long long)j * J.ldb + k]), acc);
    J.C[(long long)i * J.ldc + j] = acc;
}

// ------------------------------------------------------------------ elementwise kernels

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// Z = C + bias (pre-activation, kept for the backward pass); H = act(Z) in BF16
// (rows x cols of the padded layout, cols_used real columns, the rest zero)
__global__ void k_bias_act(int rows, int cols, int cols_used, int rows_used, const float* C, const float* bias,
                           int act, float* Z, __nv_bfloat16* H) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)rows * cols) return;
    const int r = (int)(e / cols), c = (int)(e % cols);
    float z = 0.f;
    if (c < cols_used && r < rows_used) z = C[e] + bias[c];
    if (Z) Z[e] = z;
    if (H) H[e] = __float2bfloat16(act ? gelu(z) : z);
}

// loss = sum of squared errors over the used rows / columns; G = 2 (Y - T) / count
__global__ void k_mse(int rows, int cols, int rows_used, int cols_used, const float* Y, const float* T, float inv_count,
                      float* G, float* loss) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    float d = 0.f;
    if (e < (long long)rows * cols) {
        const int r = (int)(e / cols), c = (int)(e % cols);
        if (r < rows_used && c < cols_used) d = Y[e] - T[(long long)r * cols_used + c];
        G[e] = 2.f * d * inv_count;
    }
    float s = d * d;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(loss, s * inv_count);
}

// dZ = dH * act'(Z), in place on the FP32 gradient; BF16 copy for the products
__global__ void k_act_bwd(long long n, const float* Z, int act, float* G, __nv_bfloat16* Gb) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n) return;
    float g = G[e];
    if (act) g *= gelu_grad(Z[e]);
    G[e] = g;
    Gb[e] = __float2bfloat16(g);
}

// out (cols x rows) = in (rows x cols)^T, BF16
__global__ void k_transpose_bf16(int rows, int cols, const __nv_bfloat16* in, __nv_bfloat16* out) {
    __shared__ __nv_bfloat16 t[32][33];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int r = by + j, c = bx + threadIdx.x;
        if (r < rows && c < cols) t[j][threadIdx.x] = in[(long long)r * cols + c];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int c = bx + j, r = by + threadIdx.x;
        if (r < rows && c < cols) out[(long long)c * rows + r] = t[threadIdx.x][j];
    }
}

__global__ void k_to_bf16(long long n, const float* in, __nv_bfloat16* out) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e < n) out[e] = __float2bfloat16(in[e]);
}

// column sums of G (rows x cols) -> out (cols): the bias gradient
__global__ void k_colsum(int rows, int cols, const float* G, float* out) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.f;
    for (int r = 0; r < rows; ++r) s += G[(long long)r * cols + c];
    out[c] = s;
}

// Adam on the FP32 master copy (bias-corrected step), BF16 copy refreshed
__global__ void k_adam(long long n, float* p, const float* g, float* m, float* v, float lr, float b1, float b2,
                       float eps, float c1, float c2, __nv_bfloat16* pb) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float gi = g[e];
    const float mi = b1 * m[e] + (1.f - b1) * gi, vi = b2 * v[e] + (1.f - b2) * gi * gi;
    m[e] = mi;
    v[e] = vi;
    const float q = p[e] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[e] = q;
    if (pb) pb[e] = __float2bfloat16(q);
}

// ------------------------------------------------------------------ host side

int round_up(int x, int m) { return (x + m - 1) / m * m; }

#define ML_CK(x)                                                                                       \
    do {                                                                                               \
        cudaError_t e_ = (x);                                                                          \
        if (e_ != cudaSuccess) return set_error(HBEM_ERR_CUDA, (std::string(#x) + ": " + cudaGetErrorString(e_)).c_str()); \
    } while (0)

template <class T>
struct DVec {
    T* p = nullptr;
    size_t n = 0;
    cudaError_t ensure(size_t count) {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

bool g_mlp_tensor_cores = true;

}  // namespace

cudaError_t gemm_bf16(int M, int N, int K, const __nv_bfloat16* A, long long lda, const __nv_bfloat16* B,
                      long long ldb, float* C, long long ldc, int* err, bool tc, cudaStream_t st) {
    if (M % kGM || N % kGN || K % kGK || lda % 8 || ldb % 8 || ldc % 4 || M <= 0 || N <= 0 || K <= 0)
        return cudaErrorInvalidValue;
    GemmJob J{M, N, K, A, B, C, lda, ldb, ldc, err};
    if (tc) {
        static bool attr = false;
        if (!attr) {
            cudaError_t e = cudaFuncSetAttribute(k_gemm_bf16_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kGSmemBytes);
            if (e != cudaSuccess) return e;
            attr = true;
        }
        k_gemm_bf16_tc<<<dim3(M / kGM, N / kGN), kGThreads, kGSmemBytes, st>>>(J);
    } else {
        k_gemm_bf16_simt<<<dim3((N + 127) / 128, M), 128, 0, st>>>(J);
    }
    return cudaGetLastError();
}

void mlp_set_tensor_cores(int on) { g_mlp_tensor_cores = on != 0; }
int mlp_get_tensor_cores() { return g_mlp_tensor_cores ? 1 : 0; }

}  // namespace hbem

using namespace hbem;

// A layer: W (out x in, row-major, padded to out_p x in_p), b (out)
struct hbem_mlp_s {
    int n_in = 0, width = 0, depth = 0, n_out = 0, nlayers = 0, device = 0;
    std::vector<int> din, dout, din_p, dout_p;           // per layer, real and padded
    std::vector<DVec<float>> W, b, gW, gb, mW, vW, mb, vb;
    std::vector<DVec<__nv_bfloat16>> Wb, WTb;             // BF16 copies: W and W^T (in_p x out_p)
    std::vector<DVec<float>> Z;                           // pre-activations (batch_p x out_p)
    std::vector<DVec<__nv_bfloat16>> H;                   // activations, layer inputs (batch_p x in_p)
    DVec<float> C, G, Y, T, loss;
    DVec<__nv_bfloat16> Gb, GTb, HTb, X;
    DVec<int> err;
    long long step = 0;
    ~hbem_mlp_s() {
        for (auto* v : {&W, &b, &gW, &gb, &mW, &vW, &mb, &vb, &Z})
            for (auto& d : *v) d.release();
        for (auto* v : {&Wb, &WTb, &H})
            for (auto& d : *v) d.release();
        C.release(); G.release(); Y.release(); T.release(); loss.release();
        Gb.release(); GTb.release(); HTb.release(); X.release(); err.release();
    }
};

namespace {

long long nblk(long long n, int t = 256) { return (n + t - 1) / t; }

int refresh_bf16(hbem_mlp m, int l) {
    const long long n = (long long)m->dout_p[l] * m->din_p[l];
    k_to_bf16<<<(unsigned)nblk(n), 256>>>(n, m->W[l].p, m->Wb[l].p);
    k_transpose_bf16<<<dim3((m->din_p[l] + 31) / 32, (m->dout_p[l] + 31) / 32), dim3(32, 8)>>>(
        m->dout_p[l], m->din_p[l], m->Wb[l].p, m->WTb[l].p);
    count_launches(2);
    ML_CK(cudaGetLastError());
    return HBEM_OK;
}

// forward over a padded batch already in m->H[0]; output FP32 in m->Y (batch_p x out_p)
int forward(hbem_mlp m, int batch, int batch_p) {
    for (int l = 0; l < m->nlayers; ++l) {
        const bool last = l == m->nlayers - 1;
        ML_CK(m->Z[l].ensure((size_t)batch_p * m->dout_p[l]));
        ML_CK(gemm_bf16(batch_p, m->dout_p[l], m->din_p[l], m->H[l].p, m->din_p[l], m->Wb[l].p, m->din_p[l], m->C.p,
                        m->dout_p[l], m->err.p, g_mlp_tensor_cores, 0));
        const long long n = (long long)batch_p * m->dout_p[l];
        if (!last) {
            ML_CK(m->H[l + 1].ensure((size_t)batch_p * m->din_p[l + 1]));
            k_bias_act<<<(unsigned)nblk(n), 256>>>(batch_p, m->dout_p[l], m->dout[l], batch, m->C.p, m->b[l].p, 1,
                                                   m->Z[l].p, m->H[l + 1].p);
        } else {
            k_bias_act<<<(unsigned)nblk(n), 256>>>(batch_p, m->dout_p[l], m->dout[l], batch, m->C.p, m->b[l].p, 0,
                                                   m->Y.p, nullptr);
        }
        count_launches(2);
        ML_CK(cudaGetLastError());
    }
    return HBEM_OK;
}

int load_batch(hbem_mlp m, const float* X_host, int batch, int batch_p) {
    const int w0 = std::max(m->din_p[0], 1);
    std::vector<__nv_bfloat16> xb((size_t)batch_p * w0, __float2bfloat16(0.f));
    for (int r = 0; r < batch; ++r)
        for (int c = 0; c < m->n_in; ++c) xb[(size_t)r * w0 + c] = __float2bfloat16(X_host[(size_t)r * m->n_in + c]);
    ML_CK(m->H[0].ensure(xb.size()));
    ML_CK(cudaMemcpy(m->H[0].p, xb.data(), xb.size() * sizeof(__nv_bfloat16), cudaMemcpyHostToDevice));
    const int wmax = *std::max_element(m->dout_p.begin(), m->dout_p.end());
    ML_CK(m->C.ensure((size_t)batch_p * wmax));
    ML_CK(m->Y.ensure((size_t)batch_p * m->dout_p.back()));
    return HBEM_OK;
}

// forward + loss + backward: gradients in gW, gb; returns the loss
int backward(hbem_mlp m, const float* T_host, int batch, int batch_p, float* loss_host) {
    const int L = m->nlayers;
    const int wmax = std::max(*std::max_element(m->dout_p.begin(), m->dout_p.end()),
                              *std::max_element(m->din_p.begin(), m->din_p.end()));
    ML_CK(m->T.ensure((size_t)batch * m->n_out));
    ML_CK(cudaMemcpy(m->T.p, T_host, (size_t)batch * m->n_out * sizeof(float), cudaMemcpyHostToDevice));
    ML_CK(m->G.ensure((size_t)batch_p * wmax));
    ML_CK(m->Gb.ensure((size_t)batch_p * wmax));
    ML_CK(m->GTb.ensure((size_t)batch_p * wmax));
    ML_CK(m->HTb.ensure((size_t)batch_p * wmax));
    ML_CK(m->loss.ensure(1));
    ML_CK(cudaMemset(m->loss.p, 0, sizeof(float)));
    const long long no = (long long)batch_p * m->dout_p[L - 1];
    k_mse<<<(unsigned)nblk(no), 256>>>(batch_p, m->dout_p[L - 1], batch, m->n_out, m->Y.p, m->T.p,
                                       1.f / (float)((long long)batch * m->n_out), m->G.p, m->loss.p);
    k_to_bf16<<<(unsigned)nblk(no), 256>>>(no, m->G.p, m->Gb.p);
    count_launches(2);
    for (int l = L - 1; l >= 0; --l) {
        const int op = m->dout_p[l], ip = m->din_p[l];
        // dW = dZ^T H: A = dZ^T (op x batch_p), B = H^T (ip x batch_p)
        k_transpose_bf16<<<dim3((op + 31) / 32, (batch_p + 31) / 32), dim3(32, 8)>>>(batch_p, op, m->Gb.p, m->GTb.p);
        k_transpose_bf16<<<dim3((ip + 31) / 32, (batch_p + 31) / 32), dim3(32, 8)>>>(batch_p, ip, m->H[l].p, m->HTb.p);
        ML_CK(gemm_bf16(op, ip, batch_p, m->GTb.p, batch_p, m->HTb.p, batch_p, m->gW[l].p, ip, m->err.p,
                        g_mlp_tensor_cores, 0));
        k_colsum<<<(unsigned)nblk(op), 256>>>(batch_p, op, m->G.p, m->gb[l].p);
        count_launches(4);
        if (l == 0) break;
        // dH = dZ W: A = dZ (batch_p x op), B = W^T (ip x op)
        ML_CK(gemm_bf16(batch_p, ip, op, m->Gb.p, op, m->WTb[l].p, op, m->C.p, ip, m->err.p, g_mlp_tensor_cores, 0));
        // dZ_(l-1) = dH * GELU'(Z_(l-1)) (the padded columns stay zero: Z there is zero, dH too)
        const long long n = (long long)batch_p * ip;
        ML_CK(cudaMemcpy(m->G.p, m->C.p, n * sizeof(float), cudaMemcpyDeviceToDevice));
        k_act_bwd<<<(unsigned)nblk(n), 256>>>(n, m->Z[l - 1].p, 1, m->G.p, m->Gb.p);
        count_launches(2);
        ML_CK(cudaGetLastError());
    }
    ML_CK(cudaMemcpy(loss_host, m->loss.p, sizeof(float), cudaMemcpyDeviceToHost));
    int e = 0;
    ML_CK(cudaMemcpy(&e, m->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return set_error(HBEM_ERR_NOCONV, "mlp: a tensor-core completion wait timed out");
    return HBEM_OK;
}

}  // namespace

extern "C" {

int hbem_mlp_create(int n_in, int width, int depth, int n_out, unsigned long long seed, hbem_mlp* out) {
    if (n_in < 1 || width < 1 || depth < 1 || n_out < 1 || !out || n_in > 4096 || width > 8192 || depth > 64 ||
        n_out > 8192)
        return set_error(HBEM_ERR_INVALID, "mlp_create: bad argument");
    hbem_mlp m = new hbem_mlp_s;
    m->n_in = n_in;
    m->width = width;
    m->depth = depth;
    m->n_out = n_out;
    m->nlayers = depth + 1;
    cudaGetDevice(&m->device);
    for (int l = 0; l < m->nlayers; ++l) {
        const int i = l == 0 ? n_in : width, o = l == depth ? n_out : width;
        m->din.push_back(i);
        m->dout.push_back(o);
        m->din_p.push_back(round_up(i, 128));    // a layer's input is the previous output (padded to 128)
        m->dout_p.push_back(round_up(o, 128));
    }
    const int L = m->nlayers;
    m->W.resize(L); m->b.resize(L); m->gW.resize(L); m->gb.resize(L);
    m->mW.resize(L); m->vW.resize(L); m->mb.resize(L); m->vb.resize(L);
    m->Wb.resize(L); m->WTb.resize(L); m->Z.resize(L); m->H.resize(L + 1);
    std::mt19937_64 gen(seed);
    for (int l = 0; l < L; ++l) {
        const size_t nw = (size_t)m->dout_p[l] * m->din_p[l];
        // He-style initialisation, zero padding
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)m->din[l]));
        std::vector<float> w(nw, 0.f), z(nw, 0.f), bz(m->dout_p[l], 0.f);
        for (int r = 0; r < m->dout[l]; ++r)
            for (int c = 0; c < m->din[l]; ++c) w[(size_t)r * m->din_p[l] + c] = nd(gen);
        for (auto* d : {&m->W[l], &m->gW[l], &m->mW[l], &m->vW[l]})
            if (d->ensure(nw) != cudaSuccess) { delete m; return set_error(HBEM_ERR_NOMEM, "mlp_create: cudaMalloc"); }
        for (auto* d : {&m->b[l], &m->gb[l], &m->mb[l], &m->vb[l]})
            if (d->ensure(m->dout_p[l]) != cudaSuccess) { delete m; return set_error(HBEM_ERR_NOMEM, "mlp_create: cudaMalloc"); }
        if (m->Wb[l].ensure(nw) != cudaSuccess || m->WTb[l].ensure(nw) != cudaSuccess) {
            delete m;
            return set_error(HBEM_ERR_NOMEM, "mlp_create: cudaMalloc");
        }
        cudaMemcpy(m->W[l].p, w.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
        for (auto* d : {&m->gW[l], &m->mW[l], &m->vW[l]}) cudaMemcpy(d->p, z.data(), nw * sizeof(float), cudaMemcpyHostToDevice);
        for (auto* d : {&m->b[l], &m->gb[l], &m->mb[l], &m->vb[l]})
            cudaMemcpy(d->p, bz.data(), bz.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (int r = refresh_bf16(m, l)) { delete m; return r; }
    }
    if (m->err.ensure(1) != cudaSuccess) { delete m; return set_error(HBEM_ERR_NOMEM, "mlp_create: cudaMalloc"); }
    cudaMemset(m->err.p, 0, sizeof(int));
    if (cudaDeviceSynchronize() != cudaSuccess) { delete m; return set_error(HBEM_ERR_CUDA, "mlp_create: CUDA error"); }
    *out = m;
    return HBEM_OK;
}

int hbem_mlp_destroy(hbem_mlp m) {
    delete m;
    return HBEM_OK;
}

int hbem_mlp_num_params(hbem_mlp m, long long* count) {
    if (!m || !count) return set_error(HBEM_ERR_INVALID, "mlp: bad argument");
    long long c = 0;
    for (int l = 0; l < m->nlayers; ++l) c += (long long)m->dout[l] * m->din[l] + m->dout[l];
    *count = c;
    return HBEM_OK;
}

// parameters (or gradients) as one vector: per layer W (out x in, row-major) then b
static int params_io(hbem_mlp m, float* host, int which, bool to_host) {
    if (!m || !host) return set_error(HBEM_ERR_INVALID, "mlp: bad argument");
    size_t off = 0;
    for (int l = 0; l < m->nlayers; ++l) {
        DVec<float>& W = which ? m->gW[l] : m->W[l];
        DVec<float>& b = which ? m->gb[l] : m->b[l];
        const int o = m->dout[l], i = m->din[l], ip = m->din_p[l];
        std::vector<float> w((size_t)m->dout_p[l] * ip);
        if (to_host || !which) ML_CK(cudaMemcpy(w.data(), W.p, w.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int r = 0; r < o; ++r)
            for (int c = 0; c < i; ++c) {
                float& dst = w[(size_t)r * ip + c];
                if (to_host) host[off + (size_t)r * i + c] = dst;
                else dst = host[off + (size_t)r * i + c];
            }
        off += (size_t)o * i;
        std::vector<float> bv(m->dout_p[l]);
        ML_CK(cudaMemcpy(bv.data(), b.p, bv.size() * sizeof(float), cudaMemcpyDeviceToHost));
        for (int r = 0; r < o; ++r) {
            if (to_host) host[off + r] = bv[r];
            else bv[r] = host[off + r];
        }
        off += o;
        if (!to_host) {
            ML_CK(cudaMemcpy(W.p, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
            ML_CK(cudaMemcpy(b.p, bv.data(), bv.size() * sizeof(float), cudaMemcpyHostToDevice));
            if (int r = refresh_bf16(m, l)) return r;
        }
    }
    return HBEM_OK;
}

int hbem_mlp_get_params(hbem_mlp m, float* host) { return params_io(m, host, 0, true); }
int hbem_mlp_set_params(hbem_mlp m, const float* host) { return params_io(m, const_cast<float*>(host), 0, false); }

int hbem_mlp_forward(hbem_mlp m, const float* X_host, int batch, float* Y_host) {
    if (!m || !X_host || !Y_host || batch < 1) return set_error(HBEM_ERR_INVALID, "mlp_forward: bad argument");
    ML_CK(cudaSetDevice(m->device));
    const int bp = round_up(batch, 128);
    if (int r = load_batch(m, X_host, batch, bp)) return r;
    if (int r = forward(m, batch, bp)) return r;
    const int op = m->dout_p.back();
    std::vector<float> y((size_t)bp * op);
    ML_CK(cudaMemcpy(y.data(), m->Y.p, y.size() * sizeof(float), cudaMemcpyDeviceToHost));
    int e = 0;
    ML_CK(cudaMemcpy(&e, m->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) return set_error(HBEM_ERR_NOCONV, "mlp: a tensor-core completion wait timed out");
    for (int r = 0; r < batch; ++r)
        for (int c = 0; c < m->n_out; ++c) Y_host[(size_t)r * m->n_out + c] = y[(size_t)r * op + c];
    return HBEM_OK;
}

int hbem_mlp_gradients(hbem_mlp m, const float* X_host, const float* T_host, int batch, float* loss_host,
                       float* grads_host) {
    if (!m || !X_host || !T_host || !loss_host || batch < 1) return set_error(HBEM_ERR_INVALID, "mlp: bad argument");
    ML_CK(cudaSetDevice(m->device));
    const int bp = round_up(batch, 128);
    if (int r = load_batch(m, X_host, batch, bp)) return r;
    if (int r = forward(m, batch, bp)) return r;
    if (int r = backward(m, T_host, batch, bp, loss_host)) return r;
    if (grads_host) return params_io(m, grads_host, 1, true);
    return HBEM_OK;
}

int hbem_mlp_train_step(hbem_mlp m, const float* X_host, const float* T_host, int batch, float lr, float* loss_host) {
    if (int r = hbem_mlp_gradients(m, X_host, T_host, batch, loss_host, nullptr)) return r;
    ++m->step;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
    for (int l = 0; l < m->nlayers; ++l) {
        const long long nw = (long long)m->dout_p[l] * m->din_p[l];
        k_adam<<<(unsigned)nblk(nw), 256>>>(nw, m->W[l].p, m->gW[l].p, m->mW[l].p, m->vW[l].p, lr, b1, b2, eps, c1, c2,
                                           m->Wb[l].p);
        k_adam<<<(unsigned)nblk(m->dout_p[l]), 256>>>(m->dout_p[l], m->b[l].p, m->gb[l].p, m->mb[l].p, m->vb[l].p, lr,
                                                     b1, b2, eps, c1, c2, nullptr);
        k_transpose_bf16<<<dim3((m->din_p[l] + 31) / 32, (m->dout_p[l] + 31) / 32), dim3(32, 8)>>>(
            m->dout_p[l], m->din_p[l], m->Wb[l].p, m->WTb[l].p);
        count_launches(3);
    }
    ML_CK(cudaGetLastError());
    return HBEM_OK;
}

int hbem_bf16_gemm_device(int M, int N, int K, const void* A, long long lda, const void* B, long long ldb, void* C,
                          long long ldc, int tensor_cores) {
    if (!A || !B || !C) return set_error(HBEM_ERR_INVALID, "bf16_gemm: bad argument");
    static thread_local DVec<int> err;
    ML_CK(err.ensure(1));
    ML_CK(cudaMemset(err.p, 0, sizeof(int)));
    cudaError_t e = gemm_bf16(M, N, K, static_cast<const __nv_bfloat16*>(A), lda, static_cast<const __nv_bfloat16*>(B),
                              ldb, static_cast<float*>(C), ldc, err.p, tensor_cores != 0, 0);
    if (e == cudaErrorInvalidValue)
        return set_error(HBEM_ERR_INVALID, "bf16_gemm: M, N must be multiples of 128, K of 64, lda, ldb of 8");
    ML_CK(e);
    count_launches(1);
    int h = 0;
    ML_CK(cudaMemcpy(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return set_error(HBEM_ERR_NOCONV, "bf16_gemm: a tensor-core completion wait timed out");
    return HBEM_OK;
}

}  // extern "C"
