// Batched complex64 update C -= A B on the 5th-generation tensor cores (tcgen05,
// kind::tf32) with 3xTF32 split products and FP32 accumulation in tensor memory.
// It is the trailing update of the complex-FP32 LU (csrc/lu.cu); K is taken in
// chunks of 32 complex columns (the LU's blocks are 128 wide).
//
// Complex product as one real GEMM of a 128 x 64 complex tile:
//   A' = [A_r | A_i]               (128 x 64 real, K-major)
//   B' = [[B_r,  B_i],             (K x N = 64 x 128 real; stored N x K, K-major)
//         [-B_i, B_r]]
//   C' = A' B' = [Re(A B) | Im(A B)]  (128 x 128 FP32 in TMEM)
// Each operand is split x = hi + lo with hi = tf32(x), lo = tf32(x - hi), and
// C' = A_hi B_hi + A_hi B_lo + A_lo B_hi (three MMA groups of 8 K-steps).
//
// Shared-memory operands: 128-byte-swizzled K-major canonical layout, 8-row atoms of
// 1024 bytes, each 32-element K block (128 bytes per row) a separate 16 KB region;
// the MMA for K-step kk starts at block kk / 4, byte offset 32 (kk % 4).
// One elected thread issues the MMAs and commits them to an mbarrier; all threads
// wait on it with an iteration cap (a timeout sets an error flag and the CTA still
// releases its tensor memory); eight warps read the accumulator back with tcgen05.ld
// (warp w: TMEM lanes 32 (w % 4) .. + 31, column half w / 4) and update C in global
// memory.  Each thread issues its operand and C loads in batches before using them.
#include <cstdint>

#include "hbem_device.cuh"

namespace hbem {

constexpr int kTcM = 128;                    // complex rows per tile = MMA M
constexpr int kTcNc = 64;                    // complex columns per tile
constexpr int kTcN = 2 * kTcNc;              // MMA N (real): [re | im]
constexpr int kTcKc = 32;                    // complex K per chunk
constexpr int kTcK = 2 * kTcKc;              // real K: [re | im]
constexpr int kTcThreads = 256;
constexpr uint32_t kTcKBlockBytes = 128u * 128u;           // 128 rows x 128 bytes
constexpr uint32_t kTcOperandBytes = 2u * kTcKBlockBytes;  // two K blocks
constexpr uint32_t kTcTmemCols = 256;        // allocation (the accumulator uses 128)
constexpr size_t kTcSmemBytes = 4 * (size_t)kTcOperandBytes + 1024;
constexpr long long kTcSpinCap = 1LL << 24;

// instruction descriptor, kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32 (bits 7-9,
// 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28
constexpr uint32_t kTcIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                              ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t tf32_bits(float x) {
    uint32_t r;
    asm volatile("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// byte offset of (row r, real K index k) in a 128-row operand
__device__ __forceinline__ uint32_t sw128_offset(int r, int k) {
    const int kb = k >> 5, kk = k & 31, chunk = kk >> 2, within = kk & 3, atom = r >> 3, rr = r & 7;
    return (uint32_t)kb * kTcKBlockBytes + (uint32_t)atom * 1024u + (uint32_t)rr * 128u +
           ((uint32_t)(chunk ^ rr) << 4) + ((uint32_t)within << 2);
}

// shared-memory matrix descriptor: start address >> 4 (bits 0-13), leading byte
// offset (16-29; unused for swizzled K-major, 1), stride byte offset >> 4 (32-45:
// 1024 bytes between 8-row groups), version 1 (46-47), swizzle 128 B (61-63 = 2)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

__device__ __forceinline__ void store_split(uint8_t* hi, uint8_t* lo, uint32_t off, float x) {
    const uint32_t h = tf32_bits(x);
    const uint32_t l = tf32_bits(x - __uint_as_float(h));
    *reinterpret_cast<uint32_t*>(hi + off) = h;
    *reinterpret_cast<uint32_t*>(lo + off) = l;
}

struct TcJob {
    int m, n, k;                 // C is m x n, K = k <= 32
    const cplxf* A;              // m x k, column-major, leading dimension lda
    const cplxf* B;              // k x n
    cplxf* C;                    // m x n
    long long lda, ldb, ldc;
    long long sa, sb, sc;        // batch strides (elements)
    int* err;                    // set to 1 if a tensor-core wait timed out
};

__global__ void __launch_bounds__(kTcThreads) k_cgemm_tc(TcJob J) {
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* Ahi = base;
    uint8_t* Alo = base + kTcOperandBytes;
    uint8_t* Bhi = base + 2 * kTcOperandBytes;
    uint8_t* Blo = base + 3 * kTcOperandBytes;
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    __shared__ int s_last;   // last chunk whose MMAs were committed (-1: none)
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int r0 = blockIdx.x * kTcM, c0 = blockIdx.y * kTcNc;
    const cplxf* A = J.A + (long long)blockIdx.z * J.sa;
    const cplxf* B = J.B + (long long)blockIdx.z * J.sb;
    cplxf* C = J.C + (long long)blockIdx.z * J.sc;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTcTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        s_fail = 0;
        s_last = -1;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&mbar)), "r"(1));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // The K dimension in chunks of 32 complex columns: each chunk's A' and B' are split
    // into TF32 hi / lo parts in shared memory and multiplied into the same TMEM
    // accumulator.  The global loads of chunk c + 1 are issued into registers before
    // the wait for chunk c's MMAs, whose operands they then overwrite.
    constexpr int perA = kTcM * kTcKc / kTcThreads;    // 16 complex per thread
    constexpr int perB = kTcKc * kTcNc / kTcThreads;   // 8 complex per thread
    cplxf a[perA], b[perB];
    auto load_chunk = [&](int kc) {
#pragma unroll
        for (int q = 0; q < perA; ++q) {
            const int e = tid + q * kTcThreads, r = e % kTcM, k = kc + e / kTcM;
            a[q] = (r0 + r < J.m && k < J.k) ? A[(r0 + r) + (long long)k * J.lda] : mkf(0.f);
        }
#pragma unroll
        for (int q = 0; q < perB; ++q) {
            const int e = tid + q * kTcThreads, k = kc + e % kTcKc, j = e / kTcKc;
            b[q] = (k < J.k && c0 + j < J.n) ? B[k + (long long)(c0 + j) * J.ldb] : mkf(0.f);
        }
    };
    const int nchunk = (J.k + kTcKc - 1) / kTcKc;
    const uint32_t mbar_addr = smem_u32(&mbar);
    load_chunk(0);
    for (int c = 0; c < nchunk; ++c) {
        if (c > 0) {
            // the MMAs of chunk c - 1 (commit number c - 1: phase parity (c - 1) & 1)
            // must be done before their operands are overwritten; bounded wait
            uint32_t done = 0;
            for (long long it = 0; it < kTcSpinCap && !done && !s_fail; ++it)
                asm volatile(
                    "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                    : "=r"(done)
                    : "r"(mbar_addr), "r"((uint32_t)((c - 1) & 1))
                    : "memory");
            if (!done) s_fail = 1;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            __syncthreads();
            if (s_fail) break;
        }
        // A' = [A_r | A_i]: row r, K index k (re) and 32 + k (im)
#pragma unroll
        for (int q = 0; q < perA; ++q) {
            const int e = tid + q * kTcThreads, r = e % kTcM, k = e / kTcM;
            store_split(Ahi, Alo, sw128_offset(r, k), a[q].re);
            store_split(Ahi, Alo, sw128_offset(r, kTcKc + k), a[q].im);
        }
        // B' rows (N index): j -> (B_r ; -B_i), 64 + j -> (B_i ; B_r)
#pragma unroll
        for (int q = 0; q < perB; ++q) {
            const int e = tid + q * kTcThreads, k = e % kTcKc, j = e / kTcKc;
            store_split(Bhi, Blo, sw128_offset(j, k), b[q].re);
            store_split(Bhi, Blo, sw128_offset(j, kTcKc + k), -b[q].im);
            store_split(Bhi, Blo, sw128_offset(kTcNc + j, k), b[q].im);
            store_split(Bhi, Blo, sw128_offset(kTcNc + j, kTcKc + k), b[q].re);
        }
        // generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t taddr = tmem_slot;
            const uint8_t* as[3] = {Alo, Ahi, Ahi};
            const uint8_t* bs[3] = {Bhi, Blo, Bhi};
            for (int g = 0; g < 3; ++g)
                for (int kk = 0; kk < kTcK / 8; ++kk) {
                    const uint32_t koff = (uint32_t)(kk >> 2) * kTcKBlockBytes + (uint32_t)(kk & 3) * 32u;
                    const uint64_t ad = sw128_desc(smem_u32(as[g]) + koff);
                    const uint64_t bd = sw128_desc(smem_u32(bs[g]) + koff);
                    const uint32_t acc = (c == 0 && g == 0 && kk == 0) ? 0u : 1u;
                    asm volatile(
                        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
                        "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc));
                }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_addr)
                         : "memory");
            s_last = c;
        }
        if (c + 1 < nchunk) load_chunk((c + 1) * kTcKc);
    }
    const uint32_t taddr = tmem_slot;
    // wait for the last chunk's MMAs (commit number nchunk - 1), bounded
    if (!s_fail) {
        uint32_t done = 0;
        for (long long it = 0; it < kTcSpinCap && !done; ++it)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(mbar_addr), "r"((uint32_t)((nchunk - 1) & 1))
                : "memory");
        if (!done) s_fail = 1;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    if (!s_fail) {
        // epilogue: warp w reads TMEM lanes (rows) 32 (w % 4) .. + 31, column half w / 4
        const int wq = warp & 3, half = warp >> 2;
        const int row = r0 + wq * 32 + lane;
        const uint32_t lane_base = taddr + ((uint32_t)(wq * 32) << 16);
        for (int j0 = half * (kTcNc / 2); j0 < (half + 1) * (kTcNc / 2); j0 += 16) {
            uint32_t re[16], im[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(re[0]), "=r"(re[1]), "=r"(re[2]), "=r"(re[3]), "=r"(re[4]), "=r"(re[5]), "=r"(re[6]),
                  "=r"(re[7]), "=r"(re[8]), "=r"(re[9]), "=r"(re[10]), "=r"(re[11]), "=r"(re[12]), "=r"(re[13]),
                  "=r"(re[14]), "=r"(re[15])
                : "r"(lane_base + (uint32_t)j0));
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(im[0]), "=r"(im[1]), "=r"(im[2]), "=r"(im[3]), "=r"(im[4]), "=r"(im[5]), "=r"(im[6]),
                  "=r"(im[7]), "=r"(im[8]), "=r"(im[9]), "=r"(im[10]), "=r"(im[11]), "=r"(im[12]), "=r"(im[13]),
                  "=r"(im[14]), "=r"(im[15])
                : "r"(lane_base + (uint32_t)(kTcNc + j0)));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < J.m) {
                cplxf c[16];
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) {
                    const int col = c0 + j0 + jj;
                    c[jj] = col < J.n ? C[row + (long long)col * J.ldc] : mkf(0.f);
                }
#pragma unroll
                for (int jj = 0; jj < 16; ++jj) {
                    const int col = c0 + j0 + jj;
                    if (col < J.n)
                        C[row + (long long)col * J.ldc] =
                            mkf(c[jj].re - __uint_as_float(re[jj]), c[jj].im - __uint_as_float(im[jj]));
                }
            }
        }
    } else if (tid == 0) {
        atomicExch(J.err, 1);
        // give the last committed MMAs another bounded chance to finish before the
        // memory is released
        uint32_t done = 0;
        for (long long it = 0; it < kTcSpinCap && !done && s_last >= 0; ++it)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(done)
                : "r"(mbar_addr), "r"((uint32_t)(s_last & 1))
                : "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTcTmemCols));
    }
}

// Plain FP32 reference of the same update (one thread per output entry), for tests
// and for shapes the tensor-core kernel does not take.
__global__ void k_cgemm_simt(TcJob J) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y;
    if (i >= J.m || j >= J.n) return;
    const cplxf* A = J.A + (long long)blockIdx.z * J.sa;
    const cplxf* B = J.B + (long long)blockIdx.z * J.sb;
    cplxf* C = J.C + (long long)blockIdx.z * J.sc;
    cplxf acc = mkf(0.f);
    for (int k = 0; k < J.k; ++k) cfma(acc, A[i + (long long)k * J.lda], B[k + (long long)j * J.ldb]);
    cplxf* cp = C + i + (long long)j * J.ldc;
    *cp = *cp - acc;
}

size_t cgemm_tc_smem_bytes() { return kTcSmemBytes; }

cudaError_t launch_cgemm_f32(int m, int n, int k, const cplxf* A, long long lda, long long sa, const cplxf* B,
                             long long ldb, long long sb, cplxf* C, long long ldc, long long sc, int nmat,
                             int use_tc, int* err, cudaStream_t st) {
    if (m < 0 || n < 0 || k < 0 || nmat < 1 || nmat > 65535) return cudaErrorInvalidValue;
    if (m == 0 || n == 0 || k == 0) return cudaSuccess;
    TcJob J{m, n, k, A, B, C, lda, ldb, ldc, sa, sb, sc, err};
    if (use_tc) {
        if (!err) return cudaErrorInvalidValue;
        static bool attr = false;
        if (!attr) {
            cudaError_t e = cudaFuncSetAttribute(k_cgemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)kTcSmemBytes);
            if (e != cudaSuccess) return e;
            attr = true;
        }
        const dim3 grid((m + kTcM - 1) / kTcM, (n + kTcNc - 1) / kTcNc, nmat);
        if (grid.y > 65535) return cudaErrorInvalidValue;
        k_cgemm_tc<<<grid, kTcThreads, kTcSmemBytes, st>>>(J);
    } else {
        if (n > 65535) return cudaErrorInvalidValue;
        k_cgemm_simt<<<dim3((m + 127) / 128, n, nmat), 128, 0, st>>>(J);
    }
    return cudaGetLastError();
}

}  // namespace hbem
