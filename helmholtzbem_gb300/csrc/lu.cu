// Batched LU with partial pivoting of complex128 matrices in global memory, and
// the two triangular-solve forms randomized_svd needs (T x = b and T^H x = b).
// It replaces Eigen::PartialPivLU at source/utilities/randsvd.cpp:104 (the LU of
// T(k)) and :205 (the bordered Wielandt system of sv_der2).
//
// Right-looking blocked factorisation, panel width 32, three launches per panel:
//   k_lu_panel      one CTA per matrix: unblocked LU of the n-k0 x 32 panel
//   k_lu_swap_trsm  row exchanges on every column block outside the panel and
//                   U12 = L11^-1 A12 on the blocks right of it
//   k_lu_gemm       A22 -= L21 U12, 64 x 64 tiles, all matrices in one grid
// Matrices are column-major with leading dimension n (Eigen's layout); matrix m
// starts at A + m * stride.  piv[m*n + k] = row exchanged with row k at step k
// (LAPACK's ipiv, 0-based); perm[m*n + i] = source row of row i of P A.
#include <cooperative_groups.h>

#include <algorithm>
#include <type_traits>

#include "hbem_device.cuh"

namespace cg = cooperative_groups;

namespace hbem {

constexpr int kLuNB = 32;
constexpr int kLuPanelThreads = 512;
constexpr int kLuTile = 64;
constexpr int kLuSolveThreads = 512;
constexpr int kLuSolveChunk = 16;      // right-hand sides held in registers at a time

// Unblocked LU of the panel rows [k0, n) x columns [k0, k0 + nb).  STAGED: the
// panel is copied to shared memory (column-major, leading dimension n - k0), factored
// there and written back; otherwise it is factored in place in global memory (L2).
template <class E, bool STAGED>
__global__ void __launch_bounds__(kLuPanelThreads) k_lu_panel(int n, int k0, int nb, E* A, long long stride,
                                                              int* piv, int* info) {
    extern __shared__ double panel_sm[];
    E* P = reinterpret_cast<E*>(panel_sm);
    E* M = A + (long long)blockIdx.x * stride;
    int* pv = piv + (long long)blockIdx.x * n;
    const int m = n - k0;
    __shared__ double rv[32];
    __shared__ int ri[32];
    __shared__ E prow[kLuNB];
    __shared__ int s_p;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // element (row i, panel column cc)
    auto at = [&](int i, int cc) -> E& {
        return STAGED ? P[(i - k0) + cc * m] : M[i + (long long)(k0 + cc) * n];
    };
    if (STAGED) {
        for (int e = threadIdx.x; e < m * nb; e += blockDim.x) P[e] = M[(k0 + e % m) + (long long)(k0 + e / m) * n];
        __syncthreads();
    }
    for (int j = 0; j < nb; ++j) {
        const int c = k0 + j;
        double best = -1.;
        int bi = c;
        for (int i = c + threadIdx.x; i < n; i += blockDim.x) {
            const double a = norm2(at(i, j));
            if (a > best) { best = a; bi = i; }
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
            for (int w = 1; w < nw; ++w)
                if (rv[w] > b || (rv[w] == b && ri[w] < p)) { b = rv[w]; p = ri[w]; }
            s_p = p;
            pv[c] = p;
            if (b == 0. && info[blockIdx.x] == 0) info[blockIdx.x] = c + 1;
        }
        __syncthreads();
        const int p = s_p;
        if (threadIdx.x < nb) {
            E& xa = at(c, threadIdx.x);
            E& ya = at(p, threadIdx.x);
            const E x = xa, y = ya;
            if (p != c) { xa = y; ya = x; }
            prow[threadIdx.x] = (p != c) ? y : x;
        }
        __syncthreads();
        const E d = prow[j];
        const bool nz = norm2(d) > 0;
        const E id = nz ? cdiv(Elem<E>::one(), d) : Elem<E>::zero();
        for (int i = c + 1 + threadIdx.x; i < n; i += blockDim.x) {
            E l = at(i, j);
            if (nz) { l = l * id; at(i, j) = l; }
            for (int cc = j + 1; cc < nb; ++cc) cfms(at(i, cc), l, prow[cc]);
        }
        __syncthreads();
    }
    if (STAGED)
        for (int e = threadIdx.x; e < m * nb; e += blockDim.x) M[(k0 + e % m) + (long long)(k0 + e / m) * n] = P[e];
}

// Panels too tall for one CTA's shared memory: a cluster of CS CTAs per matrix (grid
// nmat * CS), CTA r holding panel rows [k0 + r R, k0 + (r + 1) R) in its shared memory
// (column-major, leading dimension R).  Per column: every CTA posts its pivot
// candidate, all read all candidates through distributed shared memory (cluster
// barrier 1), every CTA copies the pivot row, the owner of the pivot row copies the
// row it will receive (barrier 2), the two owners write the exchanged rows, and each
// CTA applies the rank-1 update to its own rows.
template <class E>
__global__ void __launch_bounds__(kLuPanelThreads) k_lu_panel_cluster(int n, int k0, int nb, int R, E* A,
                                                                      long long stride, int* piv, int* info) {
    cg::cluster_group cl = cg::this_cluster();
    const int ncta = (int)cl.num_blocks(), rank = (int)cl.block_rank();
    const int mat = blockIdx.x / ncta;
    extern __shared__ double panel_sm[];
    E* P = reinterpret_cast<E*>(panel_sm);
    __shared__ double cand_v;
    __shared__ int cand_i;
    __shared__ double rv[32];
    __shared__ int ri[32];
    __shared__ E prow[kLuNB], tmp[kLuNB];
    __shared__ int s_p;
    E* M = A + (long long)mat * stride;
    int* pv = piv + (long long)mat * n;
    const int r0 = k0 + rank * R, r1 = min(n, r0 + R), rows = max(0, r1 - r0);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int e = threadIdx.x; e < rows * nb; e += blockDim.x)
        P[(e % rows) + (e / rows) * R] = M[(r0 + e % rows) + (long long)(k0 + e / rows) * n];
    __syncthreads();
    for (int j = 0; j < nb; ++j) {
        const int c = k0 + j;
        double best = -1.;
        int bi = n;
        for (int i = max(c, r0) + threadIdx.x; i < r1; i += blockDim.x) {
            const double a = norm2(P[(i - r0) + j * R]);
            if (a > best) { best = a; bi = i; }
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
            for (int w = 1; w < nw; ++w)
                if (rv[w] > b || (rv[w] == b && ri[w] < p)) { b = rv[w]; p = ri[w]; }
            cand_v = b;
            cand_i = p;
        }
        cl.sync();                                                   // (1) candidates posted
        if (threadIdx.x == 0) {
            double b = -1.;
            int p = n;
            for (int q = 0; q < ncta; ++q) {
                const double v = *cl.map_shared_rank(&cand_v, q);
                const int i = *cl.map_shared_rank(&cand_i, q);
                if (v > b || (v == b && i < p)) { b = v; p = i; }
            }
            s_p = p;
            if (rank == 0) {
                pv[c] = p;
                if (b == 0. && info[mat] == 0) info[mat] = c + 1;
            }
        }
        __syncthreads();
        const int p = s_p;
        const int rp = (p - k0) / R, rc = (c - k0) / R;
        if (threadIdx.x < nb) {
            const E* Pp = cl.map_shared_rank(P, rp);
            prow[threadIdx.x] = Pp[(p - (k0 + rp * R)) + threadIdx.x * R];
            if (rank == rp && p != c) {
                const E* Pc = cl.map_shared_rank(P, rc);
                tmp[threadIdx.x] = Pc[(c - (k0 + rc * R)) + threadIdx.x * R];
            }
        }
        cl.sync();                                                   // (2) rows c and p read
        if (threadIdx.x < nb && p != c) {
            if (rank == rc) P[(c - r0) + threadIdx.x * R] = prow[threadIdx.x];
            if (rank == rp) P[(p - r0) + threadIdx.x * R] = tmp[threadIdx.x];
        }
        __syncthreads();
        const E d = prow[j];
        const bool nz = norm2(d) > 0;
        const E id = nz ? cdiv(Elem<E>::one(), d) : Elem<E>::zero();
        for (int i = max(c + 1, r0) + threadIdx.x; i < r1; i += blockDim.x) {
            E l = P[(i - r0) + j * R];
            if (nz) { l = l * id; P[(i - r0) + j * R] = l; }
            for (int cc = j + 1; cc < nb; ++cc) cfms(P[(i - r0) + cc * R], l, prow[cc]);
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < rows * nb; e += blockDim.x)
        M[(r0 + e % rows) + (long long)(k0 + e / rows) * n] = P[(e % rows) + (e / rows) * R];
    cl.sync();   // no CTA leaves while another may still read its shared memory
}

// grid (ceil(n/32), nmat): column block b covers columns [32 b, 32 b + 32).  Columns
// from cmax on are left alone (the two-level factorisation exchanges and solves them
// once per 128-column block, k_lu_swap_trsm_block).
template <class E>
__global__ void __launch_bounds__(256) k_lu_swap_trsm(int n, int k0, int nb, E* A, long long stride,
                                                      const int* piv, int cmax) {
    const int col0 = blockIdx.x * kLuNB;
    if (col0 == k0 || col0 >= cmax) return;            // the panel itself, or deferred
    E* M = A + (long long)blockIdx.y * stride;
    const int* pv = piv + (long long)blockIdx.y * n;
    const int ncols = min(kLuNB, n - col0);
    __shared__ int sp[kLuNB];
    __shared__ E L11[kLuNB][kLuNB + 1];
    if (threadIdx.x < nb) sp[threadIdx.x] = pv[k0 + threadIdx.x];
    __syncthreads();
    if (threadIdx.x < ncols) {
        E* a = M + (long long)(col0 + threadIdx.x) * n;
        for (int j = 0; j < nb; ++j) {
            const int p = sp[j];
            if (p != k0 + j) {
                const E t = a[k0 + j];
                a[k0 + j] = a[p];
                a[p] = t;
            }
        }
    }
    if (col0 < k0) return;                             // left of the panel: exchanges only
    for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) {
        const int r = e % nb, k = e / nb;
        L11[r][k] = M[(k0 + r) + (long long)(k0 + k) * n];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int cc = warp; cc < ncols; cc += (blockDim.x >> 5)) {
        E* a = M + (long long)(col0 + cc) * n + k0;
        E x = lane < nb ? a[lane] : Elem<E>::zero();
        for (int k = 0; k < nb; ++k) {
            E xk;
            xk.re = __shfl_sync(0xffffffffu, x.re, k);
            xk.im = __shfl_sync(0xffffffffu, x.im, k);
            if (lane > k && lane < nb) cfms(x, L11[lane][k], xk);
        }
        if (lane < nb) a[lane] = x;
    }
}

// Two-level factorisation, after the kb (<= 128) columns from K0 are factored: the
// row exchanges of those columns applied, in order, to the columns right of them
// (cbase on), and the block row solved with the kb x kb unit lower triangle,
// U12 = L11^-1 A12.  grid (ceil((n - cbase) / 32), nmat); L11 in shared memory
// (kb x (kb + 1)); a warp per column, lane l holding rows l, l + 32, l + 64, l + 96.
constexpr int kLuBlock = 128;
template <class E>
__global__ void __launch_bounds__(256) k_lu_swap_trsm_block(int n, int K0, int kb, E* A, long long stride,
                                                            const int* piv) {
    extern __shared__ double blk_sm[];
    E* L = reinterpret_cast<E*>(blk_sm);                  // [r][k], leading dimension kb + 1
    __shared__ int sp[kLuBlock];
    const int cbase = K0 + kb;
    const int col0 = cbase + blockIdx.x * kLuNB;
    E* M = A + (long long)blockIdx.y * stride;
    const int* pv = piv + (long long)blockIdx.y * n;
    const int ncols = min(kLuNB, n - col0);
    for (int j = threadIdx.x; j < kb; j += blockDim.x) sp[j] = pv[K0 + j];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, k = e / kb;
        L[r * (kb + 1) + k] = M[(K0 + r) + (long long)(K0 + k) * n];
    }
    __syncthreads();
    if (threadIdx.x < ncols) {
        E* a = M + (long long)(col0 + threadIdx.x) * n;
        for (int j = 0; j < kb; ++j) {
            const int p = sp[j];
            if (p != K0 + j) {
                const E t = a[K0 + j];
                a[K0 + j] = a[p];
                a[p] = t;
            }
        }
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int cc = warp; cc < ncols; cc += (blockDim.x >> 5)) {
        E* a = M + (long long)(col0 + cc) * n + K0;
        E x[kLuBlock / 32];
#pragma unroll
        for (int s = 0; s < kLuBlock / 32; ++s) {
            const int r = lane + 32 * s;
            x[s] = r < kb ? a[r] : Elem<E>::zero();
        }
#pragma unroll
        for (int s0 = 0; s0 < kLuBlock / 32; ++s0) {
            for (int kk = 0; kk < 32; ++kk) {
                const int k = 32 * s0 + kk;
                if (k >= kb) break;
                E xk;
                xk.re = __shfl_sync(0xffffffffu, x[s0].re, kk);
                xk.im = __shfl_sync(0xffffffffu, x[s0].im, kk);
#pragma unroll
                for (int s = 0; s < kLuBlock / 32; ++s) {
                    const int r = lane + 32 * s;
                    if (s >= s0 && r > k && r < kb) cfms(x[s], L[r * (kb + 1) + k], xk);
                }
            }
        }
#pragma unroll
        for (int s = 0; s < kLuBlock / 32; ++s) {
            const int r = lane + 32 * s;
            if (r < kb) a[r] = x[s];
        }
    }
}

// grid (tiles over trailing rows, tiles over trailing columns below cend, nmat)
template <class E>
__global__ void __launch_bounds__(256) k_lu_gemm(int n, int k0, int nb, E* A, long long stride, int cend) {
    extern __shared__ double lu_smem[];
    E* La = reinterpret_cast<E*>(lu_smem);                // [k][i], 32 x 64
    E* Ub = La + kLuNB * kLuTile;                         // [k][j], 32 x 64
    const int t0 = k0 + nb;
    const int r0 = t0 + blockIdx.x * kLuTile, c0 = t0 + blockIdx.y * kLuTile;
    E* M = A + (long long)blockIdx.z * stride;
    for (int e = threadIdx.x; e < kLuNB * kLuTile; e += blockDim.x) {
        const int i = e % kLuTile, k = e / kLuTile;
        La[k * kLuTile + i] = (k < nb && r0 + i < n) ? M[(r0 + i) + (long long)(k0 + k) * n] : Elem<E>::zero();
        const int kk = e % kLuNB, j = e / kLuNB;
        Ub[kk * kLuTile + j] = (kk < nb && c0 + j < cend) ? M[(k0 + kk) + (long long)(c0 + j) * n] : Elem<E>::zero();
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    E acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = Elem<E>::zero();
    for (int k = 0; k < nb; ++k) {
        E av[4], bv[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) av[a] = La[k * kLuTile + tx + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; ++b) bv[b] = Ub[k * kLuTile + ty + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                acc[a][b].re = fma(av[a].re, bv[b].re, fma(-av[a].im, bv[b].im, acc[a][b].re));
                acc[a][b].im = fma(av[a].re, bv[b].im, fma(av[a].im, bv[b].re, acc[a][b].im));
            }
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int j = c0 + ty + 16 * b;
        if (j >= cend) continue;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int i = r0 + tx + 16 * a;
            if (i < n) M[i + (long long)j * n] -= acc[a][b];
        }
    }
}

// perm from the exchange sequence: one CTA per matrix, the exchanges applied in
// shared memory by one thread.
__global__ void k_lu_perm(int n, const int* piv, int* perm) {
    extern __shared__ int pm[];
    const int* pv = piv + (long long)blockIdx.x * n;
    for (int i = threadIdx.x; i < n; i += blockDim.x) pm[i] = i;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int k = 0; k < n; ++k) {
            const int p = pv[k];
            if (p != k) { const int t = pm[k]; pm[k] = pm[p]; pm[p] = t; }
        }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) perm[(long long)blockIdx.x * n + i] = pm[i];
}

size_t lu_solve_smem_bytes(int n, size_t esz) {
    return ((size_t)n + (size_t)kLuNB * (kLuNB + 1) + (size_t)kLuNB * kLuSolveChunk) * esz;
}

// Row permutation of the s columns of X in place through a shared-memory column
// buffer: forward (X <- P X) or inverse (X <- P^T X).
template <class E>
__device__ void permute_rows(E* X, int n, int s, const int* perm, E* buf, bool inverse) {
    for (int c = 0; c < s; ++c) {
        E* x = X + (long long)c * n;
        for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = x[i];
        __syncthreads();
        if (!inverse)
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = buf[perm[i]];
        else
            for (int i = threadIdx.x; i < n; i += blockDim.x) x[perm[i]] = buf[i];
        __syncthreads();
    }
}

// X <- T^-1 X (s columns), P T = L U stored in M.  Right-looking by 32-row blocks.
template <class E, int CH>
__device__ void lu_solve_n(const E* M, const int* perm, int n, E* X, int s, E* sm) {
    E* buf = sm;
    E (*D)[kLuNB + 1] = reinterpret_cast<E (*)[kLuNB + 1]>(sm + n);
    E* xb = sm + n + kLuNB * (kLuNB + 1);            // [c][k], CH x 32
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    permute_rows(X, n, s, perm, buf, false);
    for (int b0 = 0; b0 < n; b0 += kLuNB) {
        const int bs = min(kLuNB, n - b0);
        for (int e = threadIdx.x; e < bs * bs; e += blockDim.x) {
            const int r = e % bs, k = e / bs;
            D[r][k] = M[(b0 + r) + (long long)(b0 + k) * n];
        }
        __syncthreads();
        for (int cb = 0; cb < s; cb += CH) {
            const int cs = min(CH, s - cb);
            for (int c = warp; c < cs; c += nw) {
                E* x = X + (long long)(cb + c) * n + b0;
                E v = lane < bs ? x[lane] : Elem<E>::zero();
                for (int k = 0; k < bs; ++k) {
                    E vk;
                    vk.re = __shfl_sync(0xffffffffu, v.re, k);
                    vk.im = __shfl_sync(0xffffffffu, v.im, k);
                    if (lane > k && lane < bs) cfms(v, D[lane][k], vk);
                }
                if (lane < bs) { x[lane] = v; xb[c * kLuNB + lane] = v; }
            }
            __syncthreads();
            for (int i = b0 + bs + threadIdx.x; i < n; i += blockDim.x) {
                E acc[CH];
#pragma unroll
                for (int c = 0; c < CH; ++c) acc[c] = Elem<E>::zero();
                for (int k = 0; k < bs; ++k) {
                    const E l = M[i + (long long)(b0 + k) * n];
#pragma unroll
                    for (int c = 0; c < CH; ++c)
                        if (c < cs) cfma(acc[c], l, xb[c * kLuNB + k]);
                }
#pragma unroll
                for (int c = 0; c < CH; ++c)
                    if (c < cs) X[i + (long long)(cb + c) * n] -= acc[c];
            }
            __syncthreads();
        }
    }
    for (int b0 = ((n - 1) / kLuNB) * kLuNB; b0 >= 0; b0 -= kLuNB) {
        const int bs = min(kLuNB, n - b0);
        for (int e = threadIdx.x; e < bs * bs; e += blockDim.x) {
            const int r = e % bs, k = e / bs;
            D[r][k] = M[(b0 + r) + (long long)(b0 + k) * n];
        }
        __syncthreads();
        for (int cb = 0; cb < s; cb += CH) {
            const int cs = min(CH, s - cb);
            for (int c = warp; c < cs; c += nw) {
                E* x = X + (long long)(cb + c) * n + b0;
                E v = lane < bs ? x[lane] : Elem<E>::zero();
                for (int k = bs - 1; k >= 0; --k) {
                    if (lane == k) v = cdiv(v, D[k][k]);
                    E vk;
                    vk.re = __shfl_sync(0xffffffffu, v.re, k);
                    vk.im = __shfl_sync(0xffffffffu, v.im, k);
                    if (lane < k) cfms(v, D[lane][k], vk);
                }
                if (lane < bs) { x[lane] = v; xb[c * kLuNB + lane] = v; }
            }
            __syncthreads();
            for (int i = threadIdx.x; i < b0; i += blockDim.x) {
                E acc[CH];
#pragma unroll
                for (int c = 0; c < CH; ++c) acc[c] = Elem<E>::zero();
                for (int k = 0; k < bs; ++k) {
                    const E u = M[i + (long long)(b0 + k) * n];
#pragma unroll
                    for (int c = 0; c < CH; ++c)
                        if (c < cs) cfma(acc[c], u, xb[c * kLuNB + k]);
                }
#pragma unroll
                for (int c = 0; c < CH; ++c)
                    if (c < cs) X[i + (long long)(cb + c) * n] -= acc[c];
            }
            __syncthreads();
        }
    }
}

// Warp-wide dot products sum_{k in [k_lo, k_hi)} conj(a[k]) X[k, c] for the cs
// columns of a chunk; the sums end up in every lane.
template <class E, int CH>
__device__ __forceinline__ void warp_dots_h(const E* a, const E* X, int n, int k_lo, int k_hi, int cs,
                                            E (&acc)[CH]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < CH; ++c) acc[c] = Elem<E>::zero();
    for (int k = k_lo + lane; k < k_hi; k += 32) {
        const E u = conj(a[k]);
#pragma unroll
        for (int c = 0; c < CH; ++c)
            if (c < cs) cfma(acc[c], u, X[k + (long long)c * n]);
    }
#pragma unroll
    for (int c = 0; c < CH; ++c) {
        if (c >= cs) break;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc[c].re += __shfl_xor_sync(0xffffffffu, acc[c].re, o);
            acc[c].im += __shfl_xor_sync(0xffffffffu, acc[c].im, o);
        }
    }
}

// X <- T^-H X:  T^H = U^H L^H P, so x = P^T L^-H U^-H b.  Left-looking by 32-row
// blocks (the sums run down columns of U and L, which are contiguous).
template <class E, int CH>
__device__ void lu_solve_h(const E* M, const int* perm, int n, E* X, int s, E* sm) {
    E* buf = sm;
    E (*D)[kLuNB + 1] = reinterpret_cast<E (*)[kLuNB + 1]>(sm + n);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int b0 = 0; b0 < n; b0 += kLuNB) {               // U^H y = b
        const int bs = min(kLuNB, n - b0);
        for (int e = threadIdx.x; e < bs * bs; e += blockDim.x) {
            const int r = e % bs, k = e / bs;
            D[r][k] = M[(b0 + r) + (long long)(b0 + k) * n];
        }
        for (int cb = 0; cb < s; cb += CH) {
            const int cs = min(CH, s - cb);
            E* Xc = X + (long long)cb * n;
            if (b0 > 0)
                for (int r = warp; r < bs; r += nw) {
                    E acc[CH];
                    warp_dots_h<E, CH>(M + (long long)(b0 + r) * n, Xc, n, 0, b0, cs, acc);
                    if (lane == 0)
#pragma unroll
                        for (int c = 0; c < CH; ++c)
                            if (c < cs) Xc[b0 + r + (long long)c * n] -= acc[c];
                }
            __syncthreads();
            for (int c = warp; c < cs; c += nw) {
                E* x = Xc + (long long)c * n + b0;
                E v = lane < bs ? x[lane] : Elem<E>::zero();
                for (int k = 0; k < bs; ++k) {
                    if (lane == k) v = cdiv(v, conj(D[k][k]));
                    E vk;
                    vk.re = __shfl_sync(0xffffffffu, v.re, k);
                    vk.im = __shfl_sync(0xffffffffu, v.im, k);
                    if (lane > k && lane < bs) cfms_c(v, D[k][lane], vk);
                }
                if (lane < bs) x[lane] = v;
            }
            __syncthreads();
        }
    }
    for (int b0 = ((n - 1) / kLuNB) * kLuNB; b0 >= 0; b0 -= kLuNB) {   // L^H z = y
        const int bs = min(kLuNB, n - b0);
        for (int e = threadIdx.x; e < bs * bs; e += blockDim.x) {
            const int r = e % bs, k = e / bs;
            D[r][k] = M[(b0 + r) + (long long)(b0 + k) * n];
        }
        for (int cb = 0; cb < s; cb += CH) {
            const int cs = min(CH, s - cb);
            E* Xc = X + (long long)cb * n;
            if (b0 + bs < n)
                for (int r = warp; r < bs; r += nw) {
                    E acc[CH];
                    warp_dots_h<E, CH>(M + (long long)(b0 + r) * n, Xc, n, b0 + bs, n, cs, acc);
                    if (lane == 0)
#pragma unroll
                        for (int c = 0; c < CH; ++c)
                            if (c < cs) Xc[b0 + r + (long long)c * n] -= acc[c];
                }
            __syncthreads();
            for (int c = warp; c < cs; c += nw) {
                E* x = Xc + (long long)c * n + b0;
                E v = lane < bs ? x[lane] : Elem<E>::zero();
                for (int k = bs - 1; k >= 0; --k) {
                    E vk;
                    vk.re = __shfl_sync(0xffffffffu, v.re, k);
                    vk.im = __shfl_sync(0xffffffffu, v.im, k);
                    if (lane < k) cfms_c(v, D[k][lane], vk);
                }
                if (lane < bs) x[lane] = v;
            }
            __syncthreads();
        }
    }
    permute_rows(X, n, s, perm, buf, true);
}

// One CTA per matrix: X_m <- T_m^-1 X_m (trans = 0) or T_m^-H X_m (trans = 1).
// grid (column groups, nmat): CTA (g, m) solves columns [g cpc, g cpc + cpc) of X_m,
// so that small batches still occupy the GPU (the factors are then re-read from L2).
template <class E, int CH>
__global__ void __launch_bounds__(kLuSolveThreads) k_lu_solve(int n, int s, int cpc, int trans, const E* LU,
                                                              long long stride, const int* perm, E* X,
                                                              long long xstride) {
    extern __shared__ double lu_solve_sm[];
    E* sm = reinterpret_cast<E*>(lu_solve_sm);
    const int c0 = blockIdx.x * cpc, cs = min(cpc, s - c0);
    if (cs <= 0) return;
    const E* M = LU + (long long)blockIdx.y * stride;
    const int* pm = perm + (long long)blockIdx.y * n;
    E* Xm = X + (long long)blockIdx.y * xstride + (long long)c0 * n;
    if (trans) lu_solve_h<E, CH>(M, pm, n, Xm, cs, sm);
    else lu_solve_n<E, CH>(M, pm, n, Xm, cs, sm);
}

constexpr size_t kLuSmemLimit = 220 * 1024;

bool lu_solve_supported(int n) { return lu_solve_smem_bytes(n, sizeof(cplx)) <= kLuSmemLimit; }
bool lu_solve_supported_f32(int n) { return lu_solve_smem_bytes(n, sizeof(cplxf)) <= kLuSmemLimit; }

cudaError_t lu_perm_from_piv(int n, int nmat, const int* piv, int* perm, cudaStream_t st) {
    if (n < 1 || nmat < 1 || (size_t)n * sizeof(int) > kLuSmemLimit) return cudaErrorInvalidValue;
    if ((size_t)n * sizeof(int) > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_lu_perm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLuSmemLimit);
        if (e != cudaSuccess) return e;
    }
    k_lu_perm<<<nmat, 256, (size_t)n * sizeof(int), st>>>(n, piv, perm);
    return cudaGetLastError();
}

constexpr size_t kPanelClusterSmem = 200 * 1024;
int g_lu_cluster_panels = 1;   // 0: tall panels in global memory (kept for comparison tests)
int g_lu_tensor_cores = 1;     // complex64 trailing updates on the tensor cores

void lu_set_cluster_panels(int on) { g_lu_cluster_panels = on ? 1 : 0; }
void lu_set_tensor_cores(int on) { g_lu_tensor_cores = on ? 1 : 0; }
int lu_get_cluster_panels() { return g_lu_cluster_panels; }
int lu_get_tensor_cores() { return g_lu_tensor_cores; }

cudaError_t launch_cgemm_f32(int m, int n, int k, const cplxf* A, long long lda, long long sa, const cplxf* B,
                             long long ldb, long long sb, cplxf* C, long long ldc, long long sc, int nmat,
                             int use_tc, int* err, cudaStream_t st);

// Cluster launch of the panel factorisation when the panel is too tall for one CTA.
// Returns with *launched = false (nothing launched) when no cluster size up to 16
// holds the panel or the device cannot co-schedule such a cluster.
template <class E>
cudaError_t launch_panel_cluster(int n, int k0, int nb, int nmat, E* A, long long stride, int* piv, int* info,
                                 cudaStream_t st, bool* launched) {
    *launched = false;
    const int m = n - k0;
    int cs = 2, ci = 0;
    size_t R = 0, smem = 0;
    for (; cs <= 16; cs *= 2, ++ci) {
        R = (m + cs - 1) / cs;
        smem = R * nb * sizeof(E);
        if (smem <= kPanelClusterSmem) break;
    }
    if (cs > 16 || (long long)nmat * cs > 0x7fffffffLL) return cudaSuccess;
    static int ok[4] = {-1, -1, -1, -1};     // per cluster size 2, 4, 8, 16: unknown / no / yes
    cudaError_t e = cudaFuncSetAttribute(k_lu_panel_cluster<E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kPanelClusterSmem);
    if (e != cudaSuccess) return e;
    if (cs == 16) {
        e = cudaFuncSetAttribute(k_lu_panel_cluster<E>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return cudaSuccess;
        }
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(nmat * cs));
    cfg.blockDim = dim3(kLuPanelThreads);
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cs;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (ok[ci] < 0) {
        cfg.dynamicSmemBytes = kPanelClusterSmem;
        int ncl = 0;
        e = cudaOccupancyMaxActiveClusters(&ncl, k_lu_panel_cluster<E>, &cfg);
        if (e != cudaSuccess) cudaGetLastError();
        ok[ci] = (e == cudaSuccess && ncl > 0) ? 1 : 0;
    }
    if (!ok[ci]) return cudaSuccess;
    cfg.dynamicSmemBytes = smem;
    e = cudaLaunchKernelEx(&cfg, k_lu_panel_cluster<E>, n, k0, nb, (int)R, A, stride, piv, info);
    *launched = e == cudaSuccess;
    return e;
}

template <class E>
cudaError_t lu_factor_impl(int n, int nmat, E* A, long long stride, int* piv, int* perm, int* info, cudaStream_t st,
                           long long* launches, int* tc_err) {
    if (n < 1 || nmat < 1 || nmat > 65535 || (size_t)n * sizeof(int) > kLuSmemLimit) return cudaErrorInvalidValue;
    const size_t gemm_smem = 2 * (size_t)kLuNB * kLuTile * sizeof(E);
    cudaError_t e = cudaFuncSetAttribute(k_lu_gemm<E>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_lu_panel<E, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLuSmemLimit);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(info, 0, (size_t)nmat * sizeof(int), st);
    if (e != cudaSuccess) return e;
    long long nl = 0;
    const int ncb = (n + kLuNB - 1) / kLuNB;
    // one 32-column panel: factor, exchange and solve the columns below cmax, update
    // the trailing columns below cend
    auto panel_step = [&](int k0, int nb, int cmax, int cend) -> cudaError_t {
        const size_t psm = (size_t)(n - k0) * nb * sizeof(E);
        if (psm <= kLuSmemLimit) {
            k_lu_panel<E, true><<<nmat, kLuPanelThreads, psm, st>>>(n, k0, nb, A, stride, piv, info);
        } else {
            bool launched = false;
            if (g_lu_cluster_panels) {
                cudaError_t e2 = launch_panel_cluster<E>(n, k0, nb, nmat, A, stride, piv, info, st, &launched);
                if (e2 != cudaSuccess) return e2;
            }
            if (!launched) k_lu_panel<E, false><<<nmat, kLuPanelThreads, 0, st>>>(n, k0, nb, A, stride, piv, info);
        }
        ++nl;
        if (ncb > 1) {
            k_lu_swap_trsm<E><<<dim3(ncb, nmat), 256, 0, st>>>(n, k0, nb, A, stride, piv, cmax);
            ++nl;
        }
        const int t0 = k0 + nb;
        if (t0 < n && cend > t0) {
            const int rt = (n - t0 + kLuTile - 1) / kLuTile, ct = (cend - t0 + kLuTile - 1) / kLuTile;
            k_lu_gemm<E><<<dim3(rt, ct, nmat), 256, gemm_smem, st>>>(n, k0, nb, A, stride, cend);
            ++nl;
        }
        return cudaGetLastError();
    };
    bool two_level = false;
    if constexpr (std::is_same<E, cplxf>::value) two_level = tc_err && g_lu_tensor_cores && n >= 2 * kLuBlock;
    if (two_level) {
        // complex64 with tensor cores: 128-column blocks.  Inside a block its four
        // panels update only the block's own columns; then the block's exchanges and
        // triangular solve reach the columns right of it once, and the trailing matrix
        // takes one update of depth 128 on the tensor cores (3xTF32), instead of four
        // of depth 32 -- a quarter of the trailing matrix's reads and writes.
        if constexpr (std::is_same<E, cplxf>::value) {
            const size_t blk_smem = (size_t)kLuBlock * (kLuBlock + 1) * sizeof(E);
            e = cudaFuncSetAttribute(k_lu_swap_trsm_block<E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)blk_smem);
            if (e != cudaSuccess) return e;
            for (int K0 = 0; K0 < n; K0 += kLuBlock) {
                const int kb = min(kLuBlock, n - K0), cmax = K0 + kb;
                for (int k0 = K0; k0 < cmax; k0 += kLuNB) {
                    e = panel_step(k0, min(kLuNB, cmax - k0), cmax, cmax);
                    if (e != cudaSuccess) return e;
                }
                const int m = n - cmax;
                if (m > 0) {
                    const size_t sm = (size_t)kb * (kb + 1) * sizeof(E);
                    k_lu_swap_trsm_block<E><<<dim3((m + kLuNB - 1) / kLuNB, nmat), 256, sm, st>>>(n, K0, kb, A, stride,
                                                                                                   piv);
                    ++nl;
                    e = launch_cgemm_f32(m, m, kb, A + cmax + (long long)K0 * n, n, stride, A + K0 + (long long)cmax * n,
                                         n, stride, A + cmax + (long long)cmax * n, n, stride, nmat, 1, tc_err, st);
                    if (e != cudaSuccess) return e;
                    ++nl;
                }
            }
        }
    } else {
        for (int k0 = 0; k0 < n; k0 += kLuNB) {
            const int nb = min(kLuNB, n - k0);
            const size_t psm = (size_t)(n - k0) * nb * sizeof(E);
            if (psm <= kLuSmemLimit) {
                k_lu_panel<E, true><<<nmat, kLuPanelThreads, psm, st>>>(n, k0, nb, A, stride, piv, info);
            } else {
                bool launched = false;
                if (g_lu_cluster_panels) {
                    e = launch_panel_cluster<E>(n, k0, nb, nmat, A, stride, piv, info, st, &launched);
                    if (e != cudaSuccess) return e;
                }
                if (!launched) k_lu_panel<E, false><<<nmat, kLuPanelThreads, 0, st>>>(n, k0, nb, A, stride, piv, info);
            }
            ++nl;
            if (ncb > 1) {
                k_lu_swap_trsm<E><<<dim3(ncb, nmat), 256, 0, st>>>(n, k0, nb, A, stride, piv, n);
                ++nl;
            }
            const int m = n - k0 - nb;
            if (m > 0) {
                bool done = false;
                if constexpr (std::is_same<E, cplxf>::value) {
                    // complex64: A22 -= L21 U12 on the tensor cores (3xTF32) once the trailing
                    // block spans at least one 128-row tile
                    if (tc_err && g_lu_tensor_cores && m >= 128) {
                        const int t0 = k0 + nb;
                        e = launch_cgemm_f32(m, m, nb, A + t0 + (long long)k0 * n, n, stride, A + k0 + (long long)t0 * n,
                                             n, stride, A + t0 + (long long)t0 * n, n, stride, nmat, 1, tc_err, st);
                        if (e != cudaSuccess) return e;
                        done = true;
                    }
                }
                if (!done) {
                    const int tiles = (m + kLuTile - 1) / kLuTile;
                    k_lu_gemm<E><<<dim3(tiles, tiles, nmat), 256, gemm_smem, st>>>(n, k0, nb, A, stride, n);
                }
                ++nl;
            }
        }
    }
    e = lu_perm_from_piv(n, nmat, piv, perm, st);
    ++nl;
    if (launches) *launches += nl;
    if (e != cudaSuccess) return e;
    return cudaGetLastError();
}

template <class E>
cudaError_t lu_solve_impl(int n, int nmat, int trans, const E* LU, long long stride, const int* perm, int s, E* X,
                          long long xstride, cudaStream_t st) {
    const size_t smem = lu_solve_smem_bytes(n, sizeof(E));
    if (n < 1 || nmat < 1 || nmat > 65535 || s < 1 || smem > kLuSmemLimit) return cudaErrorInvalidValue;
    // columns per CTA: a power of two <= 16 (the register chunk is exactly that wide,
    // so no lane computes for absent columns), the widest that still gives about two
    // CTAs per SM of the 152, which re-reads the factors least
    int cpc = 16;
    while (cpc > 1 && (long long)nmat * ((s + cpc - 1) / cpc) < 304) cpc >>= 1;
    while (cpc > 1 && cpc / 2 >= s) cpc >>= 1;
    const int ng = (s + cpc - 1) / cpc;
    const dim3 grid(ng, nmat);
    cudaError_t e = cudaSuccess;
    switch (cpc) {
#define HB_SOLVE_CASE(CHV)                                                                                       \
    case CHV:                                                                                                    \
        e = cudaFuncSetAttribute(k_lu_solve<E, CHV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLuSmemLimit); \
        if (e != cudaSuccess) return e;                                                                          \
        k_lu_solve<E, CHV><<<grid, kLuSolveThreads, smem, st>>>(n, s, cpc, trans, LU, stride, perm, X, xstride); \
        break;
        HB_SOLVE_CASE(1)
        HB_SOLVE_CASE(2)
        HB_SOLVE_CASE(4)
        HB_SOLVE_CASE(8)
        HB_SOLVE_CASE(16)
#undef HB_SOLVE_CASE
    }
    return cudaGetLastError();
}

cudaError_t lu_factor_batched(int n, int nmat, cplx* A, long long stride, int* piv, int* perm, int* info,
                              cudaStream_t st, long long* launches) {
    return lu_factor_impl<cplx>(n, nmat, A, stride, piv, perm, info, st, launches, nullptr);
}
cudaError_t lu_factor_batched_f32(int n, int nmat, cplxf* A, long long stride, int* piv, int* perm, int* info,
                                  cudaStream_t st, long long* launches, int* tc_err) {
    return lu_factor_impl<cplxf>(n, nmat, A, stride, piv, perm, info, st, launches, tc_err);
}
cudaError_t lu_solve_batched(int n, int nmat, int trans, const cplx* LU, long long stride, const int* perm, int s,
                             cplx* X, long long xstride, cudaStream_t st) {
    return lu_solve_impl<cplx>(n, nmat, trans, LU, stride, perm, s, X, xstride, st);
}
cudaError_t lu_solve_batched_f32(int n, int nmat, int trans, const cplxf* LU, long long stride, const int* perm,
                                 int s, cplxf* X, long long xstride, cudaStream_t st) {
    return lu_solve_impl<cplxf>(n, nmat, trans, LU, stride, perm, s, X, xstride, st);
}

}  // namespace hbem
