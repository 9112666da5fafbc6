// Galerkin panel-pair quadrature kernels (see assemble.cuh for the layout).
//
// Formulas follow the reference's GalerkinBuilder
// (source/galerkin_builder.cpp:237-832); per quadrature point with
// v = gamma_i(x) - gamma_j(y), ks = k sqrt(c), h0/h1 = H0/H1(ks |v|):
//   V   : |tau_i||tau_j| f f w * { h0, h1|v|, h1|v|/ks - h0|v|^2 }      scale {1, -sqrt c, c}
//   K   : (v x tau_j)|tau_i| f g w * { ks h1/|v|, h0, h0 - ks|v| h1 }   scale {1, k c, c}
//   K^T : (tau_i x v)|tau_j| f g w * (same kernels)
//   W   : cf = b'b' w - (ks^2/2) temp, temp = 2 (tau_i.tau_j) f f w
//         { cf h0, h1|v| cf + ks h0 temp,
//           (h0|v|^2 - h1|v|/ks) cf - temp (2 ks h1|v| - h0) }           scale {1, -sqrt c, -c}
// and every matrix is finally multiplied by i/4.
#include "assemble.cuh"

namespace hbem {

struct KConst {
    cplx k, ks, k2ch, ks_inv, ks_two;
    double c, sqrtc;
    double ks_re_inv, lg_ks;   // real k: 1 / ks, log(ks / 2) + gamma
};

__device__ __forceinline__ KConst make_kconst(const Job& jb) {
    KConst K;
    K.c = jb.c;
    K.sqrtc = sqrt(jb.c);
    K.k = mk(jb.kre, jb.kim);
    K.ks = K.sqrtc * K.k;
    K.k2ch = 0.5 * (K.ks * K.ks);
    K.ks_inv = cdiv(mk(1.), K.ks);
    K.ks_two = 2.0 * K.ks;
    K.ks_re_inv = K.ks.re > 0. ? 1.0 / K.ks.re : 0.;
    K.lg_ks = K.ks.re > 0. ? log(0.5 * K.ks.re) + kEulerGamma : 0.;
    return K;
}

// Moment accumulators.  With P1 shape functions every local entry is
// sum_pts w phi_a(x) psi_b(y) kappa for a kernel value kappa and shape functions
// linear in the two panel parameters x (panel i) and y (panel j), so four
// moments per kernel value suffice:  [0] sum w k, [1] sum w x k, [2] sum w y k,
// [3] sum w x y k.  Kernel values per derivative order t:
//   s[t]  : {h0, h1|v|, q}   q = |v|^2 h0 - h1|v|/ks   (single layer, hypersingular)
//   w[t]  : 2 (tau_i.tau_j) {h0, h1|v|, q}              (hypersingular, curved panels)
//   dl[t] : (v x tau_j)|tau_i| {m1, h0, m3}             (double layer)
//   dlt[t]: (tau_i x v)|tau_j| {m1, h0, m3}             (transposed double layer)
// with m1 = ks h1/|v|, m3 = h0 - ks |v| h1.  For straight panels 2 tau_i.tau_j is
// constant per pair and w is folded into s when the blocks are formed.
template <int D, bool CURVED>
struct Acc {
    cplx s[D + 1][4], dl[D + 1][4], dlt[D + 1][4], w[CURVED ? D + 1 : 1][4];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int t = 0; t <= D; ++t)
#pragma unroll
            for (int e = 0; e < 4; ++e) s[t][e] = dl[t][e] = dlt[t][e] = mk(0.);
#pragma unroll
        for (int t = 0; t < (CURVED ? D + 1 : 1); ++t)
#pragma unroll
            for (int e = 0; e < 4; ++e) w[t][e] = mk(0.);
    }
};

// H0, H1 at ks |v| with 1/|v| given (real k: no division for 1/x)
template <bool RK>
__device__ __forceinline__ void hankel_at_ix(const KConst& K, double vn, double ivn, cplx& h0, cplx& h1) {
    if (RK) {
        if (vn > 0.) hankel01_real_ix(K.ks.re * vn, K.ks_re_inv * ivn, h0, h1);
        else hankel01_real(0., h0, h1);
    } else {
        hankel01_cplx(vn * K.ks.re, vn * K.ks.im, h0, h1);
    }
}

// H0, H1 at ks |v| with 1/|v| and log|v| given (k-independent point data): for real k
// the series branch needs neither a division nor a logarithm
template <bool RK>
__device__ __forceinline__ void hankel_at_pre(const KConst& K, double vn, double ivn, double lvn, cplx& h0,
                                              cplx& h1) {
    if (RK) {
        if (vn > 0.) hankel01_real_pre(K.ks.re * vn, K.ks_re_inv * ivn, K.lg_ks + lvn, h0, h1);
        else hankel01_real(0., h0, h1);
    } else {
        hankel01_cplx(vn * K.ks.re, vn * K.ks.im, h0, h1);
    }
}

// complex scalar times complex, specialised for real ks
template <bool RK>
__device__ __forceinline__ cplx kmul(cplx a, cplx z) { return RK ? a.re * z : a * z; }

// Kernel values of one quadrature point (see Acc).
template <int D, bool RK>
struct KVals {
    cplx s[D + 1], d[D + 1];
};

template <int D, bool RK>
__device__ __forceinline__ KVals<D, RK> kernel_values(const KConst& K, double vn, double vn2, double ivn, cplx h0,
                                                      cplx h1) {
    KVals<D, RK> kv;
    kv.s[0] = h0;
    kv.d[0] = vn > 0. ? kmul<RK>(K.ks, ivn * h1) : mk(0.);
    if (D > 0) {
        cplx hv = vn * h1;
        kv.s[1] = hv;
        kv.d[1] = h0;
        if (D > 1) {
            kv.s[2] = vn2 * h0 - kmul<RK>(K.ks_inv, hv);
            kv.d[2] = h0 - kmul<RK>(K.ks, hv);
        }
    }
    return kv;
}

__device__ __forceinline__ void moments4(cplx (&m)[4], const double wm[4], cplx k) {
#pragma unroll
    for (int e = 0; e < 4; ++e) axpy(m[e], wm[e], k);
}

// single layer / hypersingular moments (weights wm = {w, w x, w y, w x y})
template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void acc_s(Acc<D, CURVED>& A, const double wm[4], const KVals<D, RK>& kv, double tdt,
                                      bool with_w) {
#pragma unroll
    for (int t = 0; t <= D; ++t) moments4(A.s[t], wm, kv.s[t]);
    if (CURVED && with_w) {
#pragma unroll
        for (int t = 0; t <= D; ++t) moments4(A.w[CURVED ? t : 0], wm, tdt * kv.s[t]);
    }
}

template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void acc_dl(Acc<D, CURVED>& A, const double wm[4], const KVals<D, RK>& kv, double vd) {
#pragma unroll
    for (int t = 0; t <= D; ++t) moments4(A.dl[t], wm, vd * kv.d[t]);
}

template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void acc_dlt(Acc<D, CURVED>& A, const double wm[4], const KVals<D, RK>& kv, double vdt) {
#pragma unroll
    for (int t = 0; t <= D; ++t) moments4(A.dlt[t], wm, vdt * kv.d[t]);
}

__device__ __forceinline__ void mom_weights(double w, double x, double y, double wm[4]) {
    wm[0] = w;
    wm[1] = w * x;
    wm[2] = w * y;
    wm[3] = wm[1] * y;
}

// P1 shape function a on [0,1] as alpha + beta u: forward (t, 1-t) or reversed (1-t, t)
__device__ __forceinline__ void shape_ab(int a, bool reversed, double& al, double& be) {
    if ((a == 0) != reversed) { al = 0.; be = 1.; }
    else { al = 1.; be = -1.; }
}

// entry of sum w phi_a(x) psi_b(y) k from the moments
__device__ __forceinline__ cplx entry_xy(const cplx (&m)[4], int a, bool rx, int b, bool ry) {
    double ax, bx, ay, by;
    shape_ab(a, rx, ax, bx);
    shape_ab(b, ry, ay, by);
    return (ax * ay) * m[0] + (bx * ay) * m[1] + (ax * by) * m[2] + (bx * by) * m[3];
}
// entry of sum w phi_a(y) psi_b(x) k (test function on the y panel)
__device__ __forceinline__ cplx entry_yx(const cplx (&m)[4], int a, bool ry, int b, bool rx) {
    double ay, by, ax, bx;
    shape_ab(a, ry, ay, by);
    shape_ab(b, rx, ax, bx);
    return (ay * ax) * m[0] + (ay * bx) * m[1] + (by * ax) * m[2] + (by * bx) * m[3];
}

// Form the local blocks from the moments, scale the derivative orders and store.
//   rx, ry : shape functions on panel i (x) / panel j (y) reversed (adjacent pairs)
//   ttp    : |tau_i||tau_j| (constant per pair: lines and circular arcs)
//   tdt    : 2 tau_i.tau_j for straight panels (constant per pair); ignored when CURVED
//   tz     : the tangent product vanishes for the pair -> no k^2 term in W
// The entries of shape-function pair (a, b) of every layer and derivative order.
template <int D, bool CURVED>
__device__ __forceinline__ void store_local_ab(const Acc<D, CURVED>& A, const KConst& K, bool rx, bool ry, double ttp,
                                               double tdt, bool tz, cplx* dst, int a, int b) {
    const cplx kc = K.c * K.k;
    const int e = 2 * a + b;
    const double dd = (a == b) ? 1. : -1.;   // b'_a b'_b for P1 (+1, -1)
    cplx T[D + 1], S[D + 1];
#pragma unroll
    for (int t = 0; t <= D; ++t) {
        S[t] = A.s[t][0];
        if (tz) T[t] = mk(0.);
        else if (CURVED) T[t] = entry_xy(A.w[CURVED ? t : 0], a, rx, b, ry);
        else T[t] = tdt * entry_xy(A.s[t], a, rx, b, ry);
    }
#pragma unroll
    for (int t = 0; t <= D; ++t) {
        cplx dl = entry_xy(A.dl[t], a, rx, b, ry);
        cplx dlt = entry_yx(A.dlt[t], a, ry, b, rx);
        cplx sl = ttp * entry_xy(A.s[t], a, rx, b, ry);
        cplx hy = dd * S[t] - K.k2ch * T[t];
        if (t == 1) hy += K.ks * T[0];
        if (t == 2) hy -= K.ks_two * T[1] - T[0];
        if (t == 1) {
            dl = dl * kc; dlt = dlt * kc;
            hy = -K.sqrtc * hy; sl = -K.sqrtc * sl;
        } else if (t == 2) {
            dl = K.c * dl; dlt = K.c * dlt;
            hy = -K.c * hy; sl = -K.c * sl;   // single layer: c * (-q)
        }
        dst[t * kLocPerD + 0 + e] = dl;
        dst[t * kLocPerD + 4 + e] = dlt;
        dst[t * kLocPerD + 8 + e] = hy;
        dst[t * kLocPerD + 12 + e] = sl;
    }
}

template <int D, bool CURVED>
__device__ __forceinline__ void store_local(const Acc<D, CURVED>& A, const KConst& K, bool rx, bool ry, double ttp,
                                            double tdt, bool tz, cplx* dst) {
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b) store_local_ab<D, CURVED>(A, K, rx, ry, ttp, tdt, tz, dst, a, b);
}

__device__ __forceinline__ bool close100eps(cplx a, cplx b) { return hypot(a.re - b.re, a.im - b.im) < 100. * kEps; }

// ------------------------------------------------------------------ panel maps (device)

__device__ __forceinline__ cplx pan_op01(const double* P, int kind, double t, cplx* tan, double* tn) {
    if (kind == 0) {
        cplx d = mk(P[2] - P[0], P[3] - P[1]);
        *tan = d;
        *tn = hypot(d.re, d.im);
        return mk(fma(d.re, t, P[0]), fma(d.im, t, P[1]));
    }
    double dphi = P[4] - P[3], s, c;
    sincos(fma(t, dphi, P[3]), &s, &c);
    *tan = mk(-P[2] * dphi * s, P[2] * dphi * c);
    *tn = P[2] * fabs(dphi);
    return mk(P[0] + P[2] * c, P[1] + P[2] * s);
}

// reversed map; the tangent returned is the forward tangent at the reflected point
// (Derivative_01_swapped with neg = true)
__device__ __forceinline__ cplx pan_swapped(const double* P, int kind, double t, cplx* tan, double* tn) {
    if (kind == 0) {
        cplx d = mk(P[2] - P[0], P[3] - P[1]);
        *tan = d;
        *tn = hypot(d.re, d.im);
        return mk(fma(-d.re, t, P[2]), fma(-d.im, t, P[3]));
    }
    double dphi = P[3] - P[4], s, c;
    sincos(fma(t, dphi, P[4]), &s, &c);
    *tan = mk(P[2] * dphi * s, -P[2] * dphi * c);
    *tn = P[2] * fabs(dphi);
    return mk(P[0] + P[2] * c, P[1] + P[2] * s);
}

// ------------------------------------------------------------------ flags (k independent)

// General pairs: zero tests of galerkin_builder.cpp:475-499 and 834-870.
__global__ void k_flags_general(DevMesh M, uint8_t* flags) {
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long npair = (long long)M.n * (M.n + 1) / 2;
    if (q >= npair) return;
    uint8_t f = flags[q];
    if (f & 0x80) return;   // singular pair (set by the host)
    long long i = (long long)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while (i * (i + 1) / 2 > q) --i;
    while ((i + 1) * (i + 2) / 2 <= q) ++i;
    long long j = q - i * (i + 1) / 2;
    const int p = M.p;
    bool zr = true, zrt = true, tz = true;
    for (int a = 0; a < p; ++a) {
        cplx xi = M.gpt[i * p + a], ti = M.gtan[i * p + a];
        for (int b = 0; b < p; ++b) {
            cplx v = xi - M.gpt[j * p + b], tj = M.gtan[j * p + b];
            if (fabs(v.re * tj.im - v.im * tj.re) >= kEps) zr = false;
            if (fabs(v.im * ti.re - v.re * ti.im) >= kEps) zrt = false;
            if (fabs(ti.im * tj.im + ti.re * tj.re) >= kEps) tz = false;
        }
    }
    f = 0;
    if (zr) f |= PF_DL0_ZERO;
    if (zrt) f |= PF_DLT0_ZERO;
    if (tz) f |= PF_TDT0_ZERO;
    flags[q] = f;
}

// Point geometry of a singular pair (coincident or adjacent set K).
struct SPoint {
    cplx v, ti, tj;
    double tin, tjn, x, y;
};

__device__ __forceinline__ void singular_point(const DevMesh& M, const SingularTask& T, int K, double a_node,
                                               double b_node, SPoint& P) {
    const double* Pi = M.par + 5 * T.i;
    const double* Pj = M.par + 5 * T.j;
    int ki = M.kind[T.i], kj = M.kind[T.j];
    if (T.kind == PK_COINC) {
        // t = xc[b], s = t (1 - xc[a]); set 0: x = s, y = t; set 1 swaps the roles
        double t = b_node, s = t * (1. - a_node);
        cplx ts, tt;
        double tns, tnt;
        cplx ps = pan_op01(Pi, ki, s, &ts, &tns), pt = pan_op01(Pi, ki, t, &tt, &tnt);
        if (K == 0) { P.v = ps - pt; P.ti = ts; P.tin = tns; P.tj = tt; P.tjn = tnt; P.x = s; P.y = t; }
        else { P.v = pt - ps; P.ti = tt; P.tin = tnt; P.tj = ts; P.tjn = tns; P.x = t; P.y = s; }
        // the reference uses v = gamma(s) - gamma(t) for both sets; only its sign differs here
        return;
    }
    // adjacent: t = xc[a], s = t xc[b]; set 0: (x, y) = (s, t), set 1: (t, s)
    double ta = a_node, sa = ta * b_node;
    double x = K == 0 ? sa : ta, y = K == 0 ? ta : sa;
    cplx pi, pj;
    if (!T.swap) {
        pi = pan_swapped(Pi, ki, x, &P.ti, &P.tin);
        pj = pan_op01(Pj, kj, y, &P.tj, &P.tjn);
    } else {
        pi = pan_op01(Pi, ki, x, &P.ti, &P.tin);
        pj = pan_swapped(Pj, kj, y, &P.tj, &P.tjn);
    }
    P.v = pi - pj;
    P.x = x;
    P.y = y;
}

// Singular pairs: zero tests (galerkin_builder.cpp:366-375, 409-418, 834-853), one CTA per pair.
__global__ void k_flags_singular(DevMesh M, const SingularTask* tasks, uint8_t* flags) {
    SingularTask T = tasks[blockIdx.x];
    int nc = M.nc, tot = nc * nc;
    int nz[6] = {0, 0, 0, 0, 0, 0};   // counts of |value| >= eps per test
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        int a = e % nc, b = e / nc;
        for (int K = 0; K < 2; ++K) {
            SPoint P;
            singular_point(M, T, K, M.xc[a], M.xc[b], P);
            // v x tau_j |tau_i| (set K), tau_i x v |tau_j|; for coincident pairs the
            // reference multiplies the norm in before its zero test as well
            double vd = (P.v.re * P.tj.im - P.v.im * P.tj.re) * P.tin;
            double vdt = (P.v.im * P.ti.re - P.v.re * P.ti.im) * P.tjn;
            double td = P.ti.im * P.tj.im + P.ti.re * P.tj.re;
            if (fabs(vd) >= kEps) nz[K == 0 ? 0 : 2]++;
            if (fabs(vdt) >= kEps) nz[K == 0 ? 1 : 3]++;
            if (fabs(td) >= kEps) nz[K == 0 ? 4 : 5]++;
        }
    }
    __shared__ int s_nz[6];
    if (threadIdx.x < 6) s_nz[threadIdx.x] = 0;
    __syncthreads();
    for (int c = 0; c < 6; ++c)
        if (nz[c]) atomicAdd(&s_nz[c], nz[c]);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint8_t f = 0x80;
        if (!s_nz[0]) f |= PF_DL0_ZERO;
        if (!s_nz[1]) f |= PF_DLT0_ZERO;
        if (!s_nz[2]) f |= PF_DL1_ZERO;
        if (!s_nz[3]) f |= PF_DLT1_ZERO;
        if (!s_nz[4]) f |= PF_TDT0_ZERO;
        if (!s_nz[5]) f |= PF_TDT1_ZERO;
        if (M.lines) {   // lines: one tangent product for both sets (compute_tdottp on K = 0)
            f = (f & ~PF_TDT1_ZERO) | ((f & PF_TDT0_ZERO) ? PF_TDT1_ZERO : 0);
        }
        flags[tri_index(T.i, T.j)] = f;
    }
}

// ------------------------------------------------------------------ local-block kernels

// General pair number q (strictly lower pairs, in the builder's distance order when
// it made one) of mesh M for one job: p x p Gauss points, the pair's local blocks
// written to locj (the job's block array).
template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void general_pair(const DevMesh& M, const KConst& K, long long q, const double* sx,
                                             const double* sw, cplx* locj) {
    // neighbouring threads take pairs of similar panel distance, so a warp's lanes
    // mostly follow the same Hankel branch and series length
    if (M.gorder) q = M.gorder[q];
    long long i = (long long)((1.0 + sqrt(8.0 * (double)q + 1.0)) * 0.5);
    while (i * (i - 1) / 2 > q) --i;
    while ((i + 1) * i / 2 <= q) ++i;
    long long j = q - i * (i - 1) / 2;
    long long pid = tri_index(i, j);
    uint8_t fl = M.flags[pid];
    if (fl & 0x80) return;   // coincident / adjacent: singular kernel
    const bool use_dl = !(fl & PF_DL0_ZERO), use_dlt = !(fl & PF_DLT0_ZERO), tz = (fl & PF_TDT0_ZERO) != 0;
    const int p = M.p;
    const cplx* pti = M.gpt + i * p;
    const cplx* ptj = M.gpt + j * p;
    const cplx* tgi = M.gtan + i * p;
    const cplx* tgj = M.gtan + j * p;
    const double* tni = M.gtn + i * p;
    const double* tnj = M.gtn + j * p;
    Acc<D, CURVED> A;
    A.zero();
    for (int a = 0; a < p; ++a) {
        const cplx xi = pti[a], ti = tgi[a];
        const double tin = tni[a], s = sx[a], wa = sw[a];
        for (int b = 0; b < p; ++b) {
            const cplx yj = ptj[b], tj = tgj[b];
            const double tjn = tnj[b];
            const cplx v = xi - yj;
            const double vn2 = norm2(v), vn = sqrt(vn2);
            const double ivn = vn > 0. ? 1.0 / vn : 0.;
            cplx h0, h1;
            hankel_at_ix<RK>(K, vn, ivn, h0, h1);
            const KVals<D, RK> kv = kernel_values<D, RK>(K, vn, vn2, ivn, h0, h1);
            double wm[4];
            mom_weights(wa * sw[b], s, sx[b], wm);
            acc_s<D, RK, CURVED>(A, wm, kv, 2. * (ti.im * tj.im + ti.re * tj.re), !tz);
            // general: zero test on v x tau_j before the norm (galerkin_builder.cpp:475-499)
            if (use_dl) acc_dl<D, RK, CURVED>(A, wm, kv, (v.re * tj.im - v.im * tj.re) * tin);
            if (use_dlt) acc_dlt<D, RK, CURVED>(A, wm, kv, (v.im * ti.re - v.re * ti.im) * tjn);
        }
    }
    const cplx t0i = tgi[0], t0j = tgj[0];
    store_local<D, CURVED>(A, K, false, false, tni[0] * tnj[0], 2. * (t0i.im * t0j.im + t0i.re * t0j.re), tz,
                           locj + pid * (D + 1) * kLocPerD);
}

// General pairs, one thread per pair.
template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_general(DevMesh M, const Job* jobs, cplx* loc, long long npair) {
    __shared__ double sx[64], sw[64];
    for (int t = threadIdx.x; t < M.p; t += blockDim.x) { sx[t] = M.xg[t]; sw[t] = M.wg[t]; }
    __syncthreads();
    long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long nlow = (long long)M.n * (M.n - 1) / 2;   // strictly lower pairs
    if (q >= nlow) return;
    const int job = blockIdx.y;
    KConst K = make_kconst(jobs[job]);
    general_pair<D, RK, CURVED>(M, K, q, sx, sw, loc + (long long)job * npair * (D + 1) * kLocPerD);
}

template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_general_w(DevMesh M, const Job* jobs, cplx* loc, long long npair, int ppw) {
    __shared__ double sx[64], sw[64];
    for (int t = threadIdx.x; t < M.p; t += blockDim.x) { sx[t] = M.xg[t]; sw[t] = M.wg[t]; }
    __syncthreads();
    // k_general with one warp per pair, its lanes over the p x p Gauss points: for
    // launches with few pairs x media (the Newton rounds of a small scatterer) a thread
    // per pair leaves most of the GPU idle.  Each warp takes ppw consecutive pairs.
    const int lane = threadIdx.x & 31;
    const long long nlow = (long long)M.n * (M.n - 1) / 2;   // strictly lower pairs
    const long long q0 = (blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5)) * ppw;
    if (q0 >= nlow) return;   // whole warp
    const int job = blockIdx.y;
    const KConst K = make_kconst(jobs[job]);
    const int p = M.p;
    for (long long q = q0; q < q0 + ppw && q < nlow; ++q) {
        long long i = (long long)((1.0 + sqrt(8.0 * (double)q + 1.0)) * 0.5);
        while (i * (i - 1) / 2 > q) --i;
        while ((i + 1) * i / 2 <= q) ++i;
        const long long j = q - i * (i - 1) / 2;
        const long long pid = tri_index(i, j);
        const uint8_t fl = M.flags[pid];
        if (fl & 0x80) continue;   // coincident / adjacent: singular kernel (whole warp)
        const bool use_dl = !(fl & PF_DL0_ZERO), use_dlt = !(fl & PF_DLT0_ZERO), tz = (fl & PF_TDT0_ZERO) != 0;
        const cplx* pti = M.gpt + i * p;
        const cplx* ptj = M.gpt + j * p;
        const cplx* tgi = M.gtan + i * p;
        const cplx* tgj = M.gtan + j * p;
        const double* tni = M.gtn + i * p;
        const double* tnj = M.gtn + j * p;
        Acc<D, CURVED> A;
        A.zero();
        for (int e = lane; e < p * p; e += 32) {
            const int a = e / p, b = e - a * p;
            const cplx xi = pti[a], ti = tgi[a];
            const double tin = tni[a], s = sx[a], wa = sw[a];
            const cplx yj = ptj[b], tj = tgj[b];
            const double tjn = tnj[b];
            const cplx v = xi - yj;
            const double vn2 = norm2(v), vn = sqrt(vn2);
            const double ivn = vn > 0. ? 1.0 / vn : 0.;
            cplx h0, h1;
            hankel_at_ix<RK>(K, vn, ivn, h0, h1);
            const KVals<D, RK> kv = kernel_values<D, RK>(K, vn, vn2, ivn, h0, h1);
            double wm[4];
            mom_weights(wa * sw[b], s, sx[b], wm);
            acc_s<D, RK, CURVED>(A, wm, kv, 2. * (ti.im * tj.im + ti.re * tj.re), !tz);
            // general: zero test on v x tau_j before the norm (galerkin_builder.cpp:475-499)
            if (use_dl) acc_dl<D, RK, CURVED>(A, wm, kv, (v.re * tj.im - v.im * tj.re) * tin);
            if (use_dlt) acc_dlt<D, RK, CURVED>(A, wm, kv, (v.im * ti.re - v.re * ti.im) * tjn);
        }
        constexpr int NV = (int)(sizeof(Acc<D, CURVED>) / sizeof(double));
        double* av = reinterpret_cast<double*>(&A);
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double x = av[v];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            av[v] = x;
        }
        if (lane == 0) {
            const cplx t0i = tgi[0], t0j = tgj[0];
            store_local<D, CURVED>(A, K, false, false, tni[0] * tnj[0], 2. * (t0i.im * t0j.im + t0i.re * t0j.re),
                                   tz, loc + ((long long)job * npair + pid) * (D + 1) * kLocPerD);
        }
    }
}

template <class AccT>
__device__ __forceinline__ void block_reduce(AccT& A, double* red /* [nwarps][sizeof(AccT)/8] */) {
    constexpr int NV = (int)(sizeof(AccT) / sizeof(double));
    double* a = reinterpret_cast<double*>(&A);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        double x = a[v];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp * NV + v] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0.;
        for (int w = 0; w < nw; ++w) s += red[w * NV + threadIdx.x];
        red[threadIdx.x] = s;   // row 0 is read only by this thread before
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int v = 0; v < NV; ++v) a[v] = red[v];
    }
}

// Point data of a singular pair (see kSGeoFields): the geometry part of the
// quadrature, the same for every wavenumber and medium.
__device__ __forceinline__ void singular_fields(const DevMesh& M, const SingularTask& T, int Kset, double xa, double xb,
                                                double wa, double wb, double* f) {
    SPoint P;
    singular_point(M, T, Kset, xa, xb, P);
    const double wab = wa * wb;
    f[0] = norm2(P.v);
    f[1] = sqrt(f[0]);
    f[2] = 2. * (P.ti.im * P.tj.im + P.ti.re * P.tj.re);
    // v x tau_j |tau_i| and tau_i x v |tau_j|; for a coincident pair the second is the
    // double layer of set 1 (the reference uses v = gamma(s) - gamma(t) for both sets)
    f[3] = (P.v.re * P.tj.im - P.v.im * P.tj.re) * P.tin;
    f[4] = (P.v.im * P.ti.re - P.v.re * P.ti.im) * P.tjn;
    f[5] = (T.kind == PK_COINC ? xb : xa) * wab;
    f[6] = P.x;
    f[7] = P.y;
    f[8] = f[1] > 0. ? 1.0 / f[1] : 0.;
    f[9] = f[1] > 0. ? log(f[1]) : 0.;
}

// Tabulate singular_fields for every task, set and point: [task][set][field][point].
__global__ void __launch_bounds__(256) k_singular_geo(DevMesh M, const SingularTask* tasks, double* geo) {
    const SingularTask T = tasks[blockIdx.x];
    const int nc = M.nc, tot = nc * nc;
    double* G = geo + (long long)blockIdx.x * 2 * kSGeoFields * tot;
    const int nset = T.kind == PK_COINC ? 1 : 2;
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int a = e % nc, b = e / nc;
        for (int Kset = 0; Kset < nset; ++Kset) {
            double f[kSGeoFields];
            singular_fields(M, T, Kset, M.xc[a], M.xc[b], M.wc[a], M.wc[b], f);
#pragma unroll
            for (int q = 0; q < kSGeoFields; ++q) G[((long long)Kset * kSGeoFields + q) * tot + e] = f[q];
        }
    }
}

// Kernel values and moment updates of one point of a singular pair from its fields.
template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void singular_accumulate(Acc<D, CURVED>& A, const KConst& K, int kind, uint8_t fl,
                                                    int Kset, const double* f) {
    const double vn2 = f[0], vn = f[1];
    cplx h0, h1;
    hankel_at_pre<RK>(K, vn, f[8], f[9], h0, h1);
    const KVals<D, RK> kv = kernel_values<D, RK>(K, vn, vn2, f[8], h0, h1);
    double wm[4];
    if (kind == PK_COINC) {
        // one point serves both triangles: set 0 has (x, y) = (s, t), set 1 (t, s);
        // V and W kernels are symmetric in s <-> t: both sets in one moment update
        const double w = f[5], s = f[6], t = f[7];
        const double wsym[4] = {2. * w, w * (s + t), w * (s + t), 2. * w * s * t};
        acc_s<D, RK, CURVED>(A, wsym, kv, f[2], !(fl & PF_TDT0_ZERO));
        if (!(fl & PF_DL0_ZERO)) {
            mom_weights(w, s, t, wm);
            acc_dl<D, RK, CURVED>(A, wm, kv, f[3]);
        }
        if (!(fl & PF_DL1_ZERO)) {
            mom_weights(w, t, s, wm);
            acc_dl<D, RK, CURVED>(A, wm, kv, f[4]);
        }
    } else {
        const uint8_t dlz = Kset == 0 ? PF_DL0_ZERO : PF_DL1_ZERO;
        const uint8_t dltz = Kset == 0 ? PF_DLT0_ZERO : PF_DLT1_ZERO;
        const uint8_t tdz = Kset == 0 ? PF_TDT0_ZERO : PF_TDT1_ZERO;
        mom_weights(f[5], f[6], f[7], wm);
        acc_s<D, RK, CURVED>(A, wm, kv, f[2], !(fl & tdz));
        if (!(fl & dlz)) acc_dl<D, RK, CURVED>(A, wm, kv, f[3]);
        if (!(fl & dltz)) acc_dlt<D, RK, CURVED>(A, wm, kv, f[4]);
    }
}

// One coincident / adjacent pair (task index ti of mesh M) for one job, reduced over
// the CTA: its local blocks written to out.  sxc, swc: the composite nodes and
// weights in shared memory; red: reduction space.
template <int D, bool RK, bool CURVED>
__device__ __forceinline__ void singular_pair(const DevMesh& M, const SingularTask& T, int ti, const KConst& K,
                                              const double* sxc, const double* swc, double* red, cplx* out) {
    const long long pid = tri_index(T.i, T.j);
    const uint8_t fl = M.flags[pid];
    const int nc = M.nc, tot = nc * nc;
    const int nset = T.kind == PK_COINC ? 1 : 2;
    // point data from the table when the builder made one, else computed here
    const double* G = M.sgeo ? M.sgeo + (long long)ti * 2 * kSGeoFields * tot : nullptr;
    Acc<D, CURVED> A;
    A.zero();
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int a = e % nc, b = e / nc;
#pragma unroll 1
        for (int Kset = 0; Kset < nset; ++Kset) {
            double f[kSGeoFields];
            if (G) {
#pragma unroll
                for (int q = 0; q < kSGeoFields; ++q) f[q] = __ldg(G + ((long long)Kset * kSGeoFields + q) * tot + e);
            } else {
                singular_fields(M, T, Kset, sxc[a], sxc[b], swc[a], swc[b], f);
            }
            singular_accumulate<D, RK, CURVED>(A, K, T.kind, fl, Kset, f);
        }
    }
    block_reduce(A, red);
    if (threadIdx.x == 0) {
        // per-pair constants: tangent norms (constant on lines and arcs) and, for
        // straight panels, the tangent product
        SPoint P;
        singular_point(M, T, 0, sxc[0], sxc[0], P);
        const bool adj = T.kind == PK_ADJ;
        const bool tz = CURVED ? false : (fl & PF_TDT0_ZERO) != 0;
        store_local<D, CURVED>(A, K, adj && !T.swap, adj && T.swap, P.tin * P.tjn,
                               2. * (P.ti.im * P.tj.im + P.ti.re * P.tj.re), tz, out + pid * (D + 1) * kLocPerD);
    }
}

// (the per-pair code of singular_pair, kept inline here: the order-0 instance keeps
// its register allocation of 128 per thread)
template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_singular(DevMesh M, const SingularTask* tasks, const Job* jobs, cplx* loc,
                                                  long long npair) {
    extern __shared__ double sm[];
    double* sxc = sm;
    double* swc = sm + M.nc;
    double* red = sm + 2 * M.nc;
    for (int t = threadIdx.x; t < M.nc; t += blockDim.x) { sxc[t] = M.xc[t]; swc[t] = M.wc[t]; }
    __syncthreads();
    const SingularTask T = tasks[blockIdx.x];
    const int job = blockIdx.y;
    KConst K = make_kconst(jobs[job]);
    const long long pid = tri_index(T.i, T.j);
    const uint8_t fl = M.flags[pid];
    const int nc = M.nc, tot = nc * nc;
    const int nset = T.kind == PK_COINC ? 1 : 2;
    // point data from the table when the builder made one, else computed here
    const double* G = M.sgeo ? M.sgeo + (long long)blockIdx.x * 2 * kSGeoFields * tot : nullptr;
    Acc<D, CURVED> A;
    A.zero();
    for (int e = threadIdx.x; e < tot; e += blockDim.x) {
        const int a = e % nc, b = e / nc;
#pragma unroll 1
        for (int Kset = 0; Kset < nset; ++Kset) {
            double f[kSGeoFields];
            if (G) {
#pragma unroll
                for (int q = 0; q < kSGeoFields; ++q) f[q] = __ldg(G + ((long long)Kset * kSGeoFields + q) * tot + e);
            } else {
                singular_fields(M, T, Kset, sxc[a], sxc[b], swc[a], swc[b], f);
            }
            singular_accumulate<D, RK, CURVED>(A, K, T.kind, fl, Kset, f);
        }
    }
    block_reduce(A, red);
    if (threadIdx.x == 0) {
        // per-pair constants: tangent norms (constant on lines and arcs) and, for
        // straight panels, the tangent product
        SPoint P;
        singular_point(M, T, 0, sxc[0], sxc[0], P);
        const bool adj = T.kind == PK_ADJ;
        const bool tz = CURVED ? false : (fl & PF_TDT0_ZERO) != 0;
        store_local<D, CURVED>(A, K, adj && !T.swap, adj && T.swap, P.tin * P.tjn,
                               2. * (P.ti.im * P.tj.im + P.ti.re * P.tj.re), tz,
                               loc + ((long long)job * npair + pid) * (D + 1) * kLocPerD);
    }
}

// ------------------------------------------------------------------ launches of few jobs
//
// A launch of a few wavenumbers (one Newton point of the plain search: 2 media) has
// fewer singular CTAs than 4 per SM, and an adjacent pair's CTA (two point sets) takes
// twice a coincident pair's time, so k_singular ends in a tail on part of the GPU.
// Here each (pair, job) is split into CTAs of 1/q of a point set each: q parts for a
// coincident pair, 2q for an adjacent one (blocks 2q t .. 2q t + 2q - 1 of pair t,
// the upper q of a coincident pair empty), so that every CTA has the same work.  Their block sums go to `part`
// ([job][pair x 2q][NV] doubles) and k_singular_join adds them in part order and forms
// the pair blocks.

template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_singular_part(DevMesh M, const SingularTask* tasks, const Job* jobs, int q,
                                                       double* part) {
    extern __shared__ double sm[];
    double* sxc = sm;
    double* swc = sm + M.nc;
    double* red = sm + 2 * M.nc;
    for (int t = threadIdx.x; t < M.nc; t += blockDim.x) { sxc[t] = M.xc[t]; swc[t] = M.wc[t]; }
    __syncthreads();
    const int task = blockIdx.x / (2 * q), sub = blockIdx.x - task * 2 * q;
    const SingularTask T = tasks[task];
    const int nset = T.kind == PK_COINC ? 1 : 2;
    if (sub >= nset * q) return;   // whole CTA, before any barrier
    const int job = blockIdx.y;
    KConst K = make_kconst(jobs[job]);
    const uint8_t fl = M.flags[tri_index(T.i, T.j)];
    const int nc = M.nc, tot = nc * nc;
    const long long W = (long long)nset * tot;
    const long long w0 = W * sub / (nset * q), w1 = W * (sub + 1) / (nset * q);
    const double* G = M.sgeo ? M.sgeo + (long long)task * 2 * kSGeoFields * tot : nullptr;
    Acc<D, CURVED> A;
    A.zero();
    for (long long w = w0 + threadIdx.x; w < w1; w += blockDim.x) {
        const int Kset = (int)(w / tot), e = (int)(w - (long long)Kset * tot);
        double f[kSGeoFields];
        if (G) {
#pragma unroll
            for (int q = 0; q < kSGeoFields; ++q) f[q] = __ldg(G + ((long long)Kset * kSGeoFields + q) * tot + e);
        } else {
            const int a = e % nc, b = e / nc;
            singular_fields(M, T, Kset, sxc[a], sxc[b], swc[a], swc[b], f);
        }
        singular_accumulate<D, RK, CURVED>(A, K, T.kind, fl, Kset, f);
    }
    block_reduce(A, red);
    constexpr int NV = (int)(sizeof(Acc<D, CURVED>) / sizeof(double));
    if (threadIdx.x == 0) {
        const double* av = reinterpret_cast<const double*>(&A);
        double* dst = part + ((long long)job * gridDim.x + blockIdx.x) * NV;
#pragma unroll
        for (int v = 0; v < NV; ++v) dst[v] = av[v];
    }
}

// one warp per (pair, job): its lanes add the pair's partial sums (each lane some of
// the moments, the parts in order), then four lanes form the blocks of one
// shape-function pair each
template <int D, bool CURVED>
__global__ void __launch_bounds__(128) k_singular_join(DevMesh M, const SingularTask* tasks, const Job* jobs,
                                                       int ntasks, int q, const double* part, cplx* loc,
                                                       long long npair) {
    constexpr int NV = (int)(sizeof(Acc<D, CURVED>) / sizeof(double));
    __shared__ double sacc[4][NV];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int task = blockIdx.x * 4 + warp;
    if (task >= ntasks) return;   // whole warp
    const int job = blockIdx.y;
    const SingularTask T = tasks[task];
    const int nparts = (T.kind == PK_COINC ? 1 : 2) * q;
    const double* src = part + ((long long)job * ntasks + task) * 2 * q * NV;
    for (int v = lane; v < NV; v += 32) {
        double x = 0.;
        for (int u = 0; u < nparts; ++u) x += src[(long long)u * NV + v];
        sacc[warp][v] = x;
    }
    __syncwarp();
    if (lane >= 4) return;
    Acc<D, CURVED> A;
    double* av = reinterpret_cast<double*>(&A);
#pragma unroll
    for (int v = 0; v < NV; ++v) av[v] = sacc[warp][v];
    const KConst K = make_kconst(jobs[job]);
    const long long pid = tri_index(T.i, T.j);
    const uint8_t fl = M.flags[pid];
    SPoint P;
    singular_point(M, T, 0, M.xc[0], M.xc[0], P);
    const bool adj = T.kind == PK_ADJ;
    const bool tz = CURVED ? false : (fl & PF_TDT0_ZERO) != 0;
    store_local_ab<D, CURVED>(A, K, adj && !T.swap, adj && T.swap, P.tin * P.tjn,
                              2. * (P.ti.im * P.tj.im + P.ti.re * P.tj.re), tz,
                              loc + ((long long)job * npair + pid) * (D + 1) * kLocPerD, lane >> 1, lane & 1);
}

// ------------------------------------------------------------------ many meshes in one launch
//
// The batching path: the jobs of several meshes (scatterers of uneven panel counts,
// each with its wavenumbers and media) in one general-pair launch and one
// singular-pair launch.  Each CTA finds its job by a binary search over the jobs'
// first block numbers, copies that job's mesh view to shared memory and runs the
// same per-pair code as the single-mesh kernels.  The meshes of one launch share
// the panel kind (all lines or all curved) and the wavenumber kind (real or not).

// index of the job whose blocks [start[j], start[j + 1]) hold block b
__device__ __forceinline__ int job_of_block(const long long* start, int njobs, long long b) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_general_multi(const MultiMesh* meshes, const MultiJob* jobs,
                                                       const long long* start, int njobs, cplx* loc) {
    __shared__ DevMesh sM;
    __shared__ double sx[64], sw[64];
    __shared__ int sjob;
    if (threadIdx.x == 0) {
        sjob = job_of_block(start, njobs, blockIdx.x);
        sM = meshes[jobs[sjob].mesh].M;
    }
    __syncthreads();
    const int job = sjob;
    for (int t = threadIdx.x; t < sM.p; t += blockDim.x) { sx[t] = sM.xg[t]; sw[t] = sM.wg[t]; }
    __syncthreads();
    const long long q = (blockIdx.x - start[job]) * (long long)blockDim.x + threadIdx.x;
    const long long nlow = (long long)sM.n * (sM.n - 1) / 2;
    if (q >= nlow) return;
    const MultiJob J = jobs[job];
    const KConst K = make_kconst(J.job);
    general_pair<D, RK, CURVED>(sM, K, q, sx, sw, loc + J.loc);
}

template <int D, bool RK, bool CURVED>
__global__ void __launch_bounds__(128) k_singular_multi(const MultiMesh* meshes, const MultiJob* jobs,
                                                        const long long* start, int njobs, cplx* loc) {
    extern __shared__ double sm[];
    __shared__ DevMesh sM;
    __shared__ int sjob;
    __shared__ SingularTask sT;
    if (threadIdx.x == 0) {
        sjob = job_of_block(start, njobs, blockIdx.x);
        const MultiMesh& MM = meshes[jobs[sjob].mesh];
        sM = MM.M;
        sT = MM.tasks[blockIdx.x - start[sjob]];
    }
    __syncthreads();
    const int nc = sM.nc;
    double* sxc = sm;
    double* swc = sm + nc;
    double* red = sm + 2 * nc;
    for (int t = threadIdx.x; t < nc; t += blockDim.x) { sxc[t] = sM.xc[t]; swc[t] = sM.wc[t]; }
    __syncthreads();
    const MultiJob J = jobs[sjob];
    const KConst K = make_kconst(J.job);
    const SingularTask T = sT;
    singular_pair<D, RK, CURVED>(sM, T, (int)(blockIdx.x - start[sjob]), K, sxc, swc, red, loc + J.loc);
}

// ------------------------------------------------------------------ gather

// P1 dof m touches panel m-1 through local function 0 (t) and panel m through local
// function 1 (1-t)  (continuous_space.hpp:38-47).
__device__ __forceinline__ int p1_panel(int m, int a, int N) { return a == 0 ? (m == 0 ? N - 1 : m - 1) : m; }

// Spaces of a layer matrix.  `sp` bit 0: the test space is P0, bit 1: the trial space
// is P0 (DiscontinuousSpace<0>, discontinuous_space.hpp:33-127: one dof per panel,
// LocGlobMap(1, n, N) = n, shape function 1).  The pair blocks hold the integrals of
// the two P1 local functions t and 1 - t of each panel; since t + (1 - t) = 1 (and
// the derivatives, +1 and -1, sum to 0), the P0 integral of a panel is the sum of its
// two P1 entries: a P0 dof m takes both local functions of panel m.
__device__ __forceinline__ int dof_panel(int m, int a, int N, bool p0) { return p0 ? m : p1_panel(m, a, N); }

// row / column spaces of layer L (galerkin_builder.cpp:936-946): the double layer is
// test x trial, the hypersingular trial x trial, the single layer test x test
__device__ __forceinline__ bool row_p0(int L, int sp) { return L == 1 ? (sp & 2) != 0 : (sp & 1) != 0; }
__device__ __forceinline__ bool col_p0(int L, int sp) { return L == 2 ? (sp & 1) != 0 : (sp & 2) != 0; }

// the P1 local entry (a on panel i, b on panel j) of layer L from the pair blocks
__device__ __forceinline__ cplx pair_entry(const cplx* locj, int L, int t, int D1, int i, int j, int a, int b) {
    const cplx* blk;
    int e;
    if (L == 0) {
        if (i >= j) { blk = locj + tri_index(i, j) * D1 * kLocPerD + t * kLocPerD + 0; e = 2 * a + b; }
        else { blk = locj + tri_index(j, i) * D1 * kLocPerD + t * kLocPerD + 4; e = 2 * a + b; }
    } else {
        int off = (L == 1) ? 8 : 12;
        if (i >= j) { blk = locj + tri_index(i, j) * D1 * kLocPerD + t * kLocPerD + off; e = 2 * a + b; }
        else { blk = locj + tri_index(j, i) * D1 * kLocPerD + t * kLocPerD + off; e = 2 * b + a; }
    }
    return blk[e];
}

// layer value (before the i/4 factor) at dofs (m, n): L = 0 double layer, 1 hypersingular, 2 single layer
__device__ __forceinline__ cplx layer_entry(const cplx* locj, int N, int L, int t, int D1, int m, int n, int sp) {
    cplx s = mk(0.);
    const bool rp0 = row_p0(L, sp), cp0 = col_p0(L, sp);
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        int i = dof_panel(m, a, N, rp0);
#pragma unroll
        for (int b = 0; b < 2; ++b) {
            int j = dof_panel(n, b, N, cp0);
            s += pair_entry(locj, L, t, D1, i, j, a, b);
        }
    }
    return s;
}

// The same with the sub-matrix rule of GalerkinBuilder::assembleDense(k, c, layers, d,
// row, col, rows, cols) (galerkin_builder.cpp:918-1009): only panel pairs {i, j} with
// i in [row, row + rows) and j in [col, col + cols) (either order) contribute, in both
// orientations, to the dof block [row, row + rows) x [col, col + cols).  With test !=
// trial spaces the double layer takes ordered pairs only (row panel i in the row
// range, column panel j in the column range; galerkin_builder.cpp:966-971,997-1001).
__device__ __forceinline__ bool in_sub(int i, int j, int row, int rows, int col, int cols) {
    return (i >= row && i < row + rows && j >= col && j < col + cols) ||
           (j >= row && j < row + rows && i >= col && i < col + cols);
}

__device__ __forceinline__ cplx layer_entry_sub(const cplx* locj, int N, int L, int t, int D1, int m, int n, int row,
                                                int rows, int col, int cols, int sp) {
    cplx s = mk(0.);
    const bool rp0 = row_p0(L, sp), cp0 = col_p0(L, sp);
    const bool ordered = L == 0 && (sp == 1 || sp == 2);
    for (int a = 0; a < 2; ++a) {
        int i = dof_panel(m, a, N, rp0);
        for (int b = 0; b < 2; ++b) {
            int j = dof_panel(n, b, N, cp0);
            const bool take = ordered ? (i >= row && i < row + rows && j >= col && j < col + cols)
                                      : in_sub(i, j, row, rows, col, cols);
            if (take) s += pair_entry(locj, L, t, D1, i, j, a, b);
        }
    }
    return s;
}

// sub-matrix layers: out[L][t] rows x cols col-major, x i/4
__global__ void k_gather_layers_sub(int N, int D1, int layers, const cplx* loc, long long npair, int job, int row,
                                    int rows, int col, int cols, int sp, cplx* out) {
    long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long tot = (long long)rows * cols;
    if (idx >= tot) return;
    const int m = row + (int)(idx % rows), n = col + (int)(idx / rows);
    const cplx* lj = loc + (long long)job * npair * D1 * kLocPerD;
    int slot = 0;
    const int lbit[3] = {1, 4, 2};   // K, W, V
    for (int L = 0; L < 3; ++L) {
        if (!(layers & lbit[L])) continue;
        for (int t = 0; t < D1; ++t) {
            cplx v = layer_entry_sub(lj, N, L, t, D1, m, n, row, rows, col, cols, sp);
            out[(long long)(slot * D1 + t) * tot + idx] = mk(-0.25 * v.im, 0.25 * v.re);
        }
        ++slot;
    }
}

// T(k) and its derivatives for nk wavenumbers; jobs are (k, c_i), (k, c_o) interleaved.
// T is column-major 2N x 2N per (k, t); blocks (gen_sol_op.cpp:59-74):
//   T11 = K_i - K_o + M,  T12 = V_o - V_i,  T21 = W_o - W_i,  T22 = K_o - K_i + M^T
__global__ void k_gather_T(int N, int D1, const cplx* loc, long long npair, const double* Mmass, int sp, cplx* T) {
    const long long n2 = 2LL * N;
    long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n2 * n2) return;
    const int kk = blockIdx.y;
    const int m = (int)(idx % n2), n = (int)(idx / n2);
    const int bm = m >= N, bn = n >= N, mm = m - bm * N, nn = n - bn * N;
    const cplx* li = loc + (2LL * kk) * npair * D1 * kLocPerD;       // inner medium
    const cplx* lo = loc + (2LL * kk + 1) * npair * D1 * kLocPerD;   // outer medium
    int L;
    double sgn;
    if (!bm && !bn) { L = 0; sgn = 1.; }          // K_i - K_o
    else if (!bm && bn) { L = 2; sgn = -1.; }     // V_o - V_i
    else if (bm && !bn) { L = 1; sgn = -1.; }     // W_o - W_i
    else { L = 0; sgn = -1.; }                    // K_o - K_i
    for (int t = 0; t < D1; ++t) {
        cplx vi = layer_entry(li, N, L, t, D1, mm, nn, sp);
        cplx vo = layer_entry(lo, N, L, t, D1, mm, nn, sp);
        cplx d = sgn * (vi - vo);
        cplx val = mk(-0.25 * d.im, 0.25 * d.re);   // x i/4
        if (t == 0 && bm == bn) val.re += bm ? Mmass[nn + (long long)mm * N] : Mmass[mm + (long long)nn * N];
        T[((long long)kk * D1 + t) * n2 * n2 + idx] = val;
    }
}

// Separate layer matrices (GalerkinBuilder getters) for job `job`: out[L][t] N x N col-major, x i/4.
__global__ void k_gather_layers(int N, int D1, int layers, const cplx* loc, long long npair, int job, int sp,
                                cplx* out) {
    long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long nn2 = (long long)N * N;
    if (idx >= nn2) return;
    const int m = (int)(idx % N), n = (int)(idx / N);
    const cplx* lj = loc + (long long)job * npair * D1 * kLocPerD;
    int slot = 0;
    const int lbit[3] = {1, 4, 2};   // K, W, V
    for (int L = 0; L < 3; ++L) {
        if (!(layers & lbit[L])) continue;
        for (int t = 0; t < D1; ++t) {
            cplx v = layer_entry(lj, N, L, t, D1, m, n, sp);
            out[(long long)(slot * D1 + t) * nn2 + idx] = mk(-0.25 * v.im, 0.25 * v.re);
        }
        ++slot;
    }
}

// ------------------------------------------------------------------ Hankel evaluation

__global__ void k_hankel01(int n, const cplx* z, int complex_arg, cplx* h0, cplx* h1) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cplx a, b;
    if (complex_arg) hankel01_cplx(z[i].re, z[i].im, a, b);
    else hankel01_real(z[i].re, a, b);
    h0[i] = a;
    h1[i] = b;
}

cudaError_t launch_hankel01(int n, const cplx* z, int complex_arg, cplx* h0, cplx* h1, cudaStream_t st) {
    k_hankel01<<<(n + 127) / 128, 128, 0, st>>>(n, z, complex_arg, h0, h1);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ launchers

// General-pair layout of a launch: kLayoutAuto picks by size (a thread per pair
// once pairs x jobs fill the GPU, else a warp per pair with ppw pairs per warp);
// 0 forces a thread per pair, ppw > 0 a warp per pair with that many pairs.
constexpr int kLayoutAuto = -1;

// Parts per point set (q) of the split singular launch: about four CTAs per SM (152
// SMs) counting an adjacent pair's two sets, at most 8; 0 when the launch has that
// many CTAs without splitting.
int singular_parts(int ntasks, int njobs) {
    const long long ctas = (long long)ntasks * njobs, want = 4LL * 152;
    if (ntasks <= 0 || njobs <= 0 || ctas >= want) return 0;
    return (int)std::min<long long>(8, (want + 2 * ctas - 1) / (2 * ctas));
}

size_t singular_part_bytes(int ntasks, int njobs, int d, bool curved) {
    const int nparts = 2 * singular_parts(ntasks, njobs);
    size_t nv = 0;
    if (d == 0) nv = curved ? sizeof(Acc<0, true>) : sizeof(Acc<0, false>);
    else if (d == 1) nv = curved ? sizeof(Acc<1, true>) : sizeof(Acc<1, false>);
    else nv = curved ? sizeof(Acc<2, true>) : sizeof(Acc<2, false>);
    return (size_t)nparts * ntasks * njobs * nv;
}

// part: scratch of singular_part_bytes for the split singular launch of few jobs, or
// null (one CTA per pair and job)
template <int D, bool RK, bool CURVED>
static cudaError_t launch_local_c(const DevMesh& M, const SingularTask* tasks, int ntasks, const Job* jobs, int njobs,
                                  cplx* loc, cudaStream_t st, int layout, int which, double* part) {
    long long npair = (long long)M.n * (M.n + 1) / 2;
    long long nlow = (long long)M.n * (M.n - 1) / 2;
    constexpr int NV = (int)(sizeof(Acc<D, CURVED>) / sizeof(double));
    const size_t ssmem = (2 * (size_t)M.nc + 4 * NV) * sizeof(double);
    const int q = (part && (which & 2)) ? singular_parts(ntasks, njobs) : 0;
    if (q > 0)
        k_singular_part<D, RK, CURVED><<<dim3(ntasks * 2 * q, njobs), 128, ssmem, st>>>(M, tasks, jobs, q, part);
    if (nlow > 0 && (which & 1)) {
        int ppw = layout;
        if (layout == kLayoutAuto) {
            if (nlow * njobs >= 152LL * 16 * 32) ppw = 0;   // enough pairs x media for a thread per pair
            else ppw = (int)std::min(16LL, std::max(1LL, nlow * njobs / 8192));   // ~8k warps in the launch
        }
        if (ppw == 0) {
            dim3 g((unsigned)((nlow + 127) / 128), njobs);
            k_general<D, RK, CURVED><<<g, 128, 0, st>>>(M, jobs, loc, npair);
        } else {
            const long long per_cta = 4LL * ppw;
            dim3 g((unsigned)((nlow + per_cta - 1) / per_cta), njobs);
            k_general_w<D, RK, CURVED><<<g, 128, 0, st>>>(M, jobs, loc, npair, ppw);
        }
    }
    if (q > 0) {
        k_singular_join<D, CURVED><<<dim3((ntasks + 3) / 4, njobs), 128, 0, st>>>(M, tasks, jobs, ntasks, q, part, loc,
                                                                                   npair);
    } else if (ntasks > 0 && (which & 2)) {
        dim3 g(ntasks, njobs);
        k_singular<D, RK, CURVED><<<g, 128, ssmem, st>>>(M, tasks, jobs, loc, npair);
    }
    return cudaGetLastError();
}

template <int D, bool RK>
static cudaError_t launch_local_t(const DevMesh& M, const SingularTask* tasks, int ntasks, const Job* jobs, int njobs,
                                  cplx* loc, cudaStream_t st, int layout, int which, double* part) {
    if (M.lines) return launch_local_c<D, RK, false>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
    return launch_local_c<D, RK, true>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
}

size_t singular_geo_bytes(int nc, int ntasks) {
    return (size_t)ntasks * 2 * kSGeoFields * (size_t)nc * nc * sizeof(double);
}

cudaError_t launch_singular_geo(const DevMesh& M, const SingularTask* tasks, int ntasks, double* geo,
                                cudaStream_t st) {
    if (ntasks > 0) k_singular_geo<<<ntasks, 256, 0, st>>>(M, tasks, geo);
    return cudaGetLastError();
}

cudaError_t launch_flags(const DevMesh& M, const SingularTask* tasks, int ntasks, uint8_t* flags, cudaStream_t st) {
    long long npair = (long long)M.n * (M.n + 1) / 2;
    k_flags_general<<<(unsigned)((npair + 127) / 128), 128, 0, st>>>(M, flags);
    if (ntasks > 0) k_flags_singular<<<ntasks, 128, 0, st>>>(M, tasks, flags);
    return cudaGetLastError();
}

template <int D, bool RK, bool CURVED>
static cudaError_t launch_multi_c(const MultiMesh* meshes, const MultiJob* jobs, int njobs, const long long* gstart,
                                  long long gblocks, const long long* sstart, long long sblocks, int max_nc, cplx* loc,
                                  cudaStream_t st) {
    if (gblocks > 0) k_general_multi<D, RK, CURVED><<<(unsigned)gblocks, 128, 0, st>>>(meshes, jobs, gstart, njobs, loc);
    if (sblocks > 0) {
        constexpr int NV = (int)(sizeof(Acc<D, CURVED>) / sizeof(double));
        const size_t smem = (2 * (size_t)max_nc + 4 * NV) * sizeof(double);
        k_singular_multi<D, RK, CURVED><<<(unsigned)sblocks, 128, smem, st>>>(meshes, jobs, sstart, njobs, loc);
    }
    return cudaGetLastError();
}

// The pair blocks of njobs jobs over several meshes in two launches (see the
// many-mesh kernels): gstart / sstart (njobs + 1 entries, device) are the jobs'
// first CTA numbers of the general and singular launch.
cudaError_t launch_local_multi(const MultiMesh* meshes, const MultiJob* jobs, int njobs, const long long* gstart,
                               long long gblocks, const long long* sstart, long long sblocks, int max_nc, bool curved,
                               bool real_k, int d, cplx* loc, cudaStream_t st) {
    if (gblocks > 0x7fffffffLL || sblocks > 0x7fffffffLL) return cudaErrorInvalidValue;
#define HB_MULTI(D_, RK_)                                                                                        \
    return curved ? launch_multi_c<D_, RK_, true>(meshes, jobs, njobs, gstart, gblocks, sstart, sblocks, max_nc, \
                                                  loc, st)                                                       \
                  : launch_multi_c<D_, RK_, false>(meshes, jobs, njobs, gstart, gblocks, sstart, sblocks, max_nc, \
                                                   loc, st)
    if (real_k) {
        if (d == 0) HB_MULTI(0, true);
        if (d == 1) HB_MULTI(1, true);
        HB_MULTI(2, true);
    }
    if (d == 0) HB_MULTI(0, false);
    if (d == 1) HB_MULTI(1, false);
    HB_MULTI(2, false);
#undef HB_MULTI
}

// layout: kLayoutAuto or a forced general-pair layout (see launch_local_c); which:
// bit 0 the general pairs, bit 1 the singular pairs; part: see launch_local_c
cudaError_t launch_local(const DevMesh& M, const SingularTask* tasks, int ntasks, const Job* jobs, int njobs,
                         bool real_k, int d, cplx* loc, cudaStream_t st, int layout, int which, double* part) {
    if (real_k) {
        if (d == 0) return launch_local_t<0, true>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
        if (d == 1) return launch_local_t<1, true>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
        return launch_local_t<2, true>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
    }
    if (d == 0) return launch_local_t<0, false>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
    if (d == 1) return launch_local_t<1, false>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
    return launch_local_t<2, false>(M, tasks, ntasks, jobs, njobs, loc, st, layout, which, part);
}

cudaError_t launch_gather_T(int N, int d, const cplx* loc, const double* Mmass, int nk, int sp, cplx* T,
                            cudaStream_t st) {
    long long npair = (long long)N * (N + 1) / 2;
    long long tot = 4LL * N * N;
    dim3 g((unsigned)((tot + 255) / 256), nk);
    k_gather_T<<<g, 256, 0, st>>>(N, d + 1, loc, npair, Mmass, sp, T);
    return cudaGetLastError();
}

cudaError_t launch_gather_layers_sub(int N, int d, int layers, const cplx* loc, int job, int row, int rows, int col,
                                     int cols, int sp, cplx* out, cudaStream_t st) {
    long long npair = (long long)N * (N + 1) / 2;
    long long tot = (long long)rows * cols;
    k_gather_layers_sub<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, d + 1, layers, loc, npair, job, row, rows,
                                                                       col, cols, sp, out);
    return cudaGetLastError();
}

cudaError_t launch_gather_layers(int N, int d, int layers, const cplx* loc, int job, int sp, cplx* out,
                                 cudaStream_t st) {
    long long npair = (long long)N * (N + 1) / 2;
    long long tot = (long long)N * N;
    k_gather_layers<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(N, d + 1, layers, loc, npair, job, sp, out);
    return cudaGetLastError();
}

}  // namespace hbem
