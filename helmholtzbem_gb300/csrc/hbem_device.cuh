// Device-side building blocks: a small complex<double> type and the Hankel
// functions H0^(1), H1^(1) for real and complex argument.
#pragma once
#include <cuda_runtime.h>
#include <math_constants.h>

#include "hankel_tables.h"

namespace hbem {

struct cplx {
    double re, im;
};

__host__ __device__ __forceinline__ cplx mk(double r, double i = 0.) { cplx z; z.re = r; z.im = i; return z; }
__host__ __device__ __forceinline__ cplx operator+(cplx a, cplx b) { return mk(a.re + b.re, a.im + b.im); }
__host__ __device__ __forceinline__ cplx operator-(cplx a, cplx b) { return mk(a.re - b.re, a.im - b.im); }
__host__ __device__ __forceinline__ cplx operator-(cplx a) { return mk(-a.re, -a.im); }
__host__ __device__ __forceinline__ cplx operator*(cplx a, cplx b) {
    return mk(fma(a.re, b.re, -a.im * b.im), fma(a.re, b.im, a.im * b.re));
}
__host__ __device__ __forceinline__ cplx operator*(double s, cplx a) { return mk(s * a.re, s * a.im); }
__host__ __device__ __forceinline__ cplx operator*(cplx a, double s) { return mk(s * a.re, s * a.im); }
__host__ __device__ __forceinline__ cplx& operator+=(cplx& a, cplx b) { a.re += b.re; a.im += b.im; return a; }
__host__ __device__ __forceinline__ cplx& operator-=(cplx& a, cplx b) { a.re -= b.re; a.im -= b.im; return a; }
__host__ __device__ __forceinline__ cplx conj(cplx a) { return mk(a.re, -a.im); }
__host__ __device__ __forceinline__ double norm2(cplx a) { return fma(a.re, a.re, a.im * a.im); }
__device__ __forceinline__ double cabs(cplx a) { return hypot(a.re, a.im); }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
    double d = 1.0 / norm2(b);
    return mk((a.re * b.re + a.im * b.im) * d, (a.im * b.re - a.re * b.im) * d);
}
// acc += s * z  (s real)
__device__ __forceinline__ void axpy(cplx& acc, double s, cplx z) {
    acc.re = fma(s, z.re, acc.re);
    acc.im = fma(s, z.im, acc.im);
}
__device__ __forceinline__ cplx cexp_i(double t) { double s, c; sincos(t, &s, &c); return mk(c, s); }
__device__ __forceinline__ cplx clog(cplx z) { return mk(log(hypot(z.re, z.im)), atan2(z.im, z.re)); }
__device__ __forceinline__ cplx csqrt(cplx z) {
    double r = hypot(z.re, z.im);
    if (r == 0.) return mk(0., 0.);
    double t = sqrt(0.5 * (r + fabs(z.re)));
    if (z.re >= 0.) return mk(t, 0.5 * z.im / t);
    return mk(0.5 * fabs(z.im) / t, z.im >= 0. ? t : -t);
}
__device__ __forceinline__ cplx cexp(cplx z) { double e = exp(z.re), s, c; sincos(z.im, &s, &c); return mk(e * c, e * s); }

// complex<float> for the single-precision LU of the dense tail
struct cplxf {
    float re, im;
};
__host__ __device__ __forceinline__ cplxf mkf(float r, float i = 0.f) { cplxf z; z.re = r; z.im = i; return z; }
__host__ __device__ __forceinline__ cplxf operator+(cplxf a, cplxf b) { return mkf(a.re + b.re, a.im + b.im); }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a, cplxf b) { return mkf(a.re - b.re, a.im - b.im); }
__host__ __device__ __forceinline__ cplxf operator-(cplxf a) { return mkf(-a.re, -a.im); }
__host__ __device__ __forceinline__ cplxf operator*(cplxf a, cplxf b) {
    return mkf(fmaf(a.re, b.re, -a.im * b.im), fmaf(a.re, b.im, a.im * b.re));
}
__host__ __device__ __forceinline__ cplxf operator*(float s, cplxf a) { return mkf(s * a.re, s * a.im); }
__host__ __device__ __forceinline__ cplxf& operator+=(cplxf& a, cplxf b) { a.re += b.re; a.im += b.im; return a; }
__host__ __device__ __forceinline__ cplxf& operator-=(cplxf& a, cplxf b) { a.re -= b.re; a.im -= b.im; return a; }
__host__ __device__ __forceinline__ cplxf conj(cplxf a) { return mkf(a.re, -a.im); }
__host__ __device__ __forceinline__ float norm2(cplxf a) { return fmaf(a.re, a.re, a.im * a.im); }
__device__ __forceinline__ cplxf cdiv(cplxf a, cplxf b) {
    // scaled so that |b|^2 cannot overflow or underflow in single precision
    const float s = fmaxf(fabsf(b.re), fabsf(b.im));
    if (s == 0.f) return mkf(a.re / s, a.im / s);
    const float br = b.re / s, bi = b.im / s, ar = a.re / s, ai = a.im / s;
    const float d = 1.f / (br * br + bi * bi);
    return mkf((ar * br + ai * bi) * d, (ai * br - ar * bi) * d);
}

// Fused complex multiply-accumulate: four FMAs instead of the two multiplies, two
// FMAs and two adds of acc += a * b (the compiler may not reassociate the latter).
__device__ __forceinline__ void cfma(cplx& acc, cplx a, cplx b) {      // acc += a b
    acc.re = fma(a.re, b.re, fma(-a.im, b.im, acc.re));
    acc.im = fma(a.re, b.im, fma(a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfms(cplx& acc, cplx a, cplx b) {      // acc -= a b
    acc.re = fma(-a.re, b.re, fma(a.im, b.im, acc.re));
    acc.im = fma(-a.re, b.im, fma(-a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfma_c(cplx& acc, cplx a, cplx b) {    // acc += conj(a) b
    acc.re = fma(a.re, b.re, fma(a.im, b.im, acc.re));
    acc.im = fma(a.re, b.im, fma(-a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfms_c(cplx& acc, cplx a, cplx b) {    // acc -= conj(a) b
    acc.re = fma(-a.re, b.re, fma(-a.im, b.im, acc.re));
    acc.im = fma(-a.re, b.im, fma(a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfma(cplxf& acc, cplxf a, cplxf b) {
    acc.re = fmaf(a.re, b.re, fmaf(-a.im, b.im, acc.re));
    acc.im = fmaf(a.re, b.im, fmaf(a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfms(cplxf& acc, cplxf a, cplxf b) {
    acc.re = fmaf(-a.re, b.re, fmaf(a.im, b.im, acc.re));
    acc.im = fmaf(-a.re, b.im, fmaf(-a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfma_c(cplxf& acc, cplxf a, cplxf b) {
    acc.re = fmaf(a.re, b.re, fmaf(a.im, b.im, acc.re));
    acc.im = fmaf(a.re, b.im, fmaf(-a.im, b.re, acc.im));
}
__device__ __forceinline__ void cfms_c(cplxf& acc, cplxf a, cplxf b) {
    acc.re = fmaf(-a.re, b.re, fmaf(-a.im, b.im, acc.re));
    acc.im = fmaf(-a.re, b.im, fmaf(a.im, b.re, acc.im));
}

// element-type helpers for code templated on cplx / cplxf
template <class E> struct Elem;
template <> struct Elem<cplx> {
    typedef double real;
    __device__ __forceinline__ static cplx zero() { return mk(0.); }
    __device__ __forceinline__ static cplx one() { return mk(1.); }
};
template <> struct Elem<cplxf> {
    typedef float real;
    __device__ __forceinline__ static cplxf zero() { return mkf(0.f); }
    __device__ __forceinline__ static cplxf one() { return mkf(1.f); }
};

constexpr double kEps = 2.220446049250313e-16;
constexpr double kEulerGamma = 0.57721566490153286061;
constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------- real argument
//
// H0 = J0 + i Y0, H1 = J1 + i Y1 for real x, with the branch structure of the
// reference's vectorised evaluator (Hankel1Real01::jy_01, cbessel.cpp:1858-1997):
//   x <= 0        J0 = 1, everything else 0
//   x < 1e-8      limiting forms (DLMF 10.7.2-4)
//   x < 2         ascending series with harmonic numbers (DLMF 10.8.1-2)
//   2 <= x < 8    Taylor polynomials of degree 17 about 2.25, 2.75, ..., 7.75
//                 (the reference uses the series up to 8; the polynomials avoid its
//                 cancellation and cost a quarter of its operations there)
//   x <= 1e6      modulus/phase amplitudes P, Q in w = 64/x^2 (DLMF 10.17; degree 14
//                 on 8 <= x < 16, degree 8 beyond),
//                 phases through sin x +- cos x so the argument is used exactly
//   x > 1e6       leading-order asymptotic form (DLMF 10.17.3, first term)
__device__ __forceinline__ double horner_pq(const double* c, double w) {
    double r = c[HBEM_PQ_DEG];
#pragma unroll
    for (int k = HBEM_PQ_DEG - 1; k >= 0; --k) r = fma(r, w, c[k]);
    return r;
}
__device__ __forceinline__ double horner_pq_far(const double* c, double w) {
    double r = c[HBEM_PQ_DEG_FAR];
#pragma unroll
    for (int k = HBEM_PQ_DEG_FAR - 1; k >= 0; --k) r = fma(r, w, c[k]);
    return r;
}

// PRE: the caller supplies ix = 1/x and lg = log(x/2) + gamma (the assembly has them
// from k-independent tables: log(x/2) = log(k sqrt(c)/2) + log|v|), which saves the
// logarithm and the division of the ascending-series branch.
template <bool PRE, bool PRE_IX = PRE>
static __device__ __forceinline__ void hankel01_real_t(double x, double ix_in, double lg_in, cplx& h0, cplx& h1) {
    double j0, j1, y0, y1;
    if (x <= 0.) {
        h0 = mk(1., 0.); h1 = mk(0., 0.);
        return;
    }
    if (x < 1e-8) {
        j0 = 1.; j1 = 0.5 * x;
        y0 = (2. / kPi) * (PRE ? lg_in : (log(j1) + kEulerGamma));
        y1 = PRE_IX ? -(2. / kPi) * ix_in : -(2. / kPi) / x;
    } else if (x >= 2. && x < 8.) {
        // Taylor polynomials about the centre of the x's quarter-width interval
        // (coefficients from mpmath; no logarithm, no division)
        const int iv = min(HBEM_TAY_N - 1, (int)((x - 2.) * 2.));
        const double h = x - (2.25 + 0.5 * iv);
        const double2* c = reinterpret_cast<const double2*>(&HBEM_TAY[iv][0][0]);
        double2 a = __ldg(c + 2 * HBEM_TAY_DEG), b = __ldg(c + 2 * HBEM_TAY_DEG + 1);
        j0 = a.x; y0 = a.y; j1 = b.x; y1 = b.y;
#pragma unroll
        for (int m = HBEM_TAY_DEG - 1; m >= 0; --m) {
            a = __ldg(c + 2 * m);
            b = __ldg(c + 2 * m + 1);
            j0 = fma(j0, h, a.x);
            y0 = fma(y0, h, a.y);
            j1 = fma(j1, h, b.x);
            y1 = fma(y1, h, b.y);
        }
    } else if (x < 8.) {
        const double mx2_4 = -0.25 * x * x;
        double t = 1.;
        j0 = 1.; j1 = 1.; y0 = 0.; y1 = 0.;
        // terms t_k = (-x^2/4)^k/(k!)^2 with tabulated 1/k^2, H_k, 1/(k+1), H_k/(k+1);
        // stop once |t_k| < 2^-55, i.e. H_k |t_k| < eps for every k used (x < 8 needs < 40)
        for (int k = 1; k <= HBEM_SER_N; ++k) {
            t *= mx2_4 * HBEM_SER_IK2[k];
            j0 += t;
            y0 = fma(-HBEM_SER_H[k], t, y0);
            j1 = fma(t, HBEM_SER_IK1[k], j1);
            y1 = fma(-HBEM_SER_HK1[k], t, y1);
            if ((__double2hiint(t) & 0x7fffffff) < ((1023 - 55) << 20)) break;
        }
        const double ix = PRE_IX ? ix_in : 1.0 / x;
        j1 *= 0.5 * x;
        const double lg = PRE ? lg_in : log(0.5 * x) + kEulerGamma;
        y0 = (2. / kPi) * fma(lg, j0, y0);
        y1 = (1. / kPi) * (y1 * x + 2.0 * (lg * j1 + (j0 - 2.0) * ix));
    } else if (x <= 1e6) {
        double ix = PRE_IX ? ix_in : 1.0 / x, w = 64. * ix * ix;
        double P0, Q0, P1, Q1;
        if (x >= 16.) {   // w <= 1/4: the degree-8 fit of the same amplitudes
            P0 = 1. + horner_pq_far(HBEM_F0F, w);
            Q0 = (horner_pq_far(HBEM_G0F, w) - 0.125) * ix;
            P1 = 1. + horner_pq_far(HBEM_F1F, w);
            Q1 = (horner_pq_far(HBEM_G1F, w) + 0.375) * ix;
        } else {
            P0 = 1. + horner_pq(HBEM_F0, w);
            Q0 = (horner_pq(HBEM_G0, w) - 0.125) * ix;
            P1 = 1. + horner_pq(HBEM_F1, w);
            Q1 = (horner_pq(HBEM_G1, w) + 0.375) * ix;
        }
        double sx, cx;
        sincos(x, &sx, &cx);
        double r = rsqrt(kPi * x);
        double cc = (sx + cx) * r, ss = (sx - cx) * r;
        j0 = P0 * cc - Q0 * ss;
        y0 = P0 * ss + Q0 * cc;
        j1 = P1 * ss + Q1 * cc;
        y1 = Q1 * ss - P1 * cc;
    } else {
        double r = sqrt(2. / (kPi * x)), s0, c0, s1, c1;
        sincos(x - 0.25 * kPi, &s0, &c0);
        sincos(x - 0.75 * kPi, &s1, &c1);
        j0 = r * c0; y0 = r * s0; j1 = r * c1; y1 = r * s1;
    }
    h0 = mk(j0, y0);
    h1 = mk(j1, y1);
}

static __device__ __noinline__ void hankel01_real(double x, cplx& h0, cplx& h1) {
    hankel01_real_t<false>(x, 0., 0., h0, h1);
}

// x > 0 with ix = 1/x and lg = log(x/2) + gamma given
static __device__ __noinline__ void hankel01_real_pre(double x, double ix, double lg, cplx& h0, cplx& h1) {
    hankel01_real_t<true>(x, ix, lg, h0, h1);
}

// x > 0 with ix = 1/x given (the logarithm, needed only below x = 2, computed here)
static __device__ __noinline__ void hankel01_real_ix(double x, double ix, cplx& h0, cplx& h1) {
    hankel01_real_t<false, true>(x, ix, 0., h0, h1);
}

// ---------------------------------------------------------------- complex argument
//
// H0, H1 for complex z (the reference calls an Amos-method routine,
// cbessel.cpp:1210-1287).  Published methods of that family:
//   |z| <= 2       ascending series (principal log)
//   2 < |z| < 20   Miller's backward recurrence for J_n normalised by
//                  J0 + 2 sum J_2k = 1, with Neumann's series for Y0 and its
//                  derivative for Y1, all accumulated during the recurrence
//   |z| >= 20      Hankel's asymptotic expansion (DLMF 10.17.5)
// Non-finite values are replaced by 0 (galerkin_builder.cpp:216-235).
static __device__ __forceinline__ void hankel01_cplx(double zre, double zim, cplx& h0, cplx& h1) {
    const cplx I = mk(0., 1.);
    const cplx z = mk(zre, zim);
    double az = hypot(z.re, z.im);
    cplx j0, j1, y0, y1;
    if (az == 0.) {
        h0 = mk(0., 0.); h1 = mk(0., 0.);
        return;
    }
    if (az <= 2.) {
        cplx x2_4 = 0.25 * (z * z), t = mk(1.);
        double Hk = 0., k = 1.;
        j0 = mk(1.); j1 = mk(1.); y0 = mk(0.); y1 = mk(0.);
        for (int it = 0; it < 60; ++it) {
            t = t * x2_4 * (-1.0 / (k * k));
            Hk += 1.0 / k;
            j0 += t;
            y0 -= Hk * t;
            k += 1.0;
            j1 += t * (1.0 / k);
            y1 -= (Hk / k) * t;
            if (Hk * hypot(t.re, t.im) <= 0.1 * kEps) break;
        }
        j1 = j1 * (0.5 * z);
        cplx lg = clog(0.5 * z) + mk(kEulerGamma);
        y0 = (2. / kPi) * (y0 + lg * j0);
        y1 = (1. / kPi) * (y1 * z + 2.0 * (lg * j1 + cdiv(j0 - mk(2.0), z)));
    } else if (az < 20.) {
        int nstart = 2 * (int)((az + 40.) * 0.5);
        cplx iz2 = cdiv(mk(2.), z);           // 2/z
        cplx Jn1 = mk(0.), Jn = mk(1e-30);    // J_{n+1}, J_n (unnormalised)
        cplx S = mk(0.), sy0 = mk(0.), sy1 = mk(0.);

        // walk n = nstart .. 1 computing J_{n-1}; accumulate sums on the fly
        // even indices contribute to S and sy0; odd ones feed sy1

        for (int n = nstart; n >= 1; --n) {
            cplx Jm1 = (double)n * (iz2 * Jn) - Jn1;   // J_{n-1}
            // J_n is known here: use it
            if ((n & 1) == 0) {
                int kk = n / 2;
                double sg = (kk & 1) ? -1. : 1.;
                S += 2.0 * Jn;
                sy0 += (sg / kk) * Jn;
                // (J_{2k-1} - J_{2k+1})/k with J_{2k-1} = Jm1, J_{2k+1} = Jn1
                sy1 += (sg / kk) * (Jm1 - Jn1);
            }
            Jn1 = Jn;
            Jn = Jm1;
            double mag = fabs(Jn.re) + fabs(Jn.im);
            if (mag > 1e200) {
                Jn = 1e-200 * Jn; Jn1 = 1e-200 * Jn1;
                S = 1e-200 * S; sy0 = 1e-200 * sy0; sy1 = 1e-200 * sy1;
            }
        }

        // now Jn = J_0, Jn1 = J_1 (unnormalised)
        S += Jn;
        cplx iS = cdiv(mk(1.), S);
        j0 = Jn * iS; j1 = Jn1 * iS;
        sy0 = sy0 * iS; sy1 = sy1 * iS;
        cplx lg = clog(0.5 * z) + mk(kEulerGamma);
        y0 = (2. / kPi) * (lg * j0) - (4. / kPi) * sy0;
        y1 = (2. / kPi) * (lg * j1) - (2. / kPi) * cdiv(j0, z) + (2. / kPi) * sy1;
    } else {
        // sum_k i^k a_k(nu) / z^k for nu = 0 and nu = 1 in one loop (no local arrays)
        cplx iiz = I * cdiv(mk(1.), z);
        cplx s0 = mk(1.), s1 = mk(1.), t0 = mk(1.), t1 = mk(1.);
        bool d0 = false, d1 = false;
        for (int k = 1; k < 200 && !(d0 && d1); ++k) {
            double odd2 = (2. * k - 1.) * (2. * k - 1.);
            if (!d0) {
                t0 = t0 * ((-odd2 / (k * 8.)) * iiz);
                s0 += t0;
                d0 = hypot(t0.re, t0.im) < 0.25 * kEps;
            }
            if (!d1) {
                t1 = t1 * (((4. - odd2) / (k * 8.)) * iiz);
                s1 += t1;
                d1 = hypot(t1.re, t1.im) < 0.25 * kEps;
            }
        }
        cplx r = csqrt(cdiv(mk(2. / kPi), z));
        j0 = r * cexp(I * (z - mk(0.25 * kPi))) * s0;   // holds H0 itself
        j1 = r * cexp(I * (z - mk(0.75 * kPi))) * s1;   // holds H1 itself
        y0 = mk(0.);
        y1 = mk(0.);
    }
    cplx a = j0 + I * y0, b = j1 + I * y1;
    if (!isfinite(a.re) || !isfinite(a.im)) a = mk(0.);
    if (!isfinite(b.re) || !isfinite(b.im)) b = mk(0.);
    h0 = a;
    h1 = b;
}

}  // namespace hbem
