// Point functions of the MHD hot path: reconstruction, characteristic
// projection and Riemann fluxes, as __host__ __device__ templates.
//
// They restate the reference's include/interp.h, include/mhd_eigen.h and
// include/mhd_flux.h with the same parameter meaning.  For T=double, compiled
// with --fmad=false (or -ffp-contract=off on the host), every expression keeps
// the reference's evaluation order, so results are the reference's bit for
// bit.  The one deliberate difference: products with a structurally zero
// eigenvector entry are skipped in the projections (the reference multiplies
// by 0.0 and adds).  For finite data that changes at most the sign of an exact
// zero, never a value.
//
// For T=float the same code is the reconstruction/flux core of the
// FP32-split precision mode; that translation unit is built with fast float
// division and square root.
#pragma once

#ifdef __CUDACC__
#define MLAU_HD __host__ __device__ __forceinline__
#else
#define MLAU_HD inline
#include <cmath>
#if defined(__GNUC__)
// host compilers see the device loops' unroll hints
#pragma GCC diagnostic push
#pragma GCC diagnostic ignored "-Wunknown-pragmas"
#define MLAU_POINT_DIAG_PUSHED
#endif
#endif

namespace mlau {

template <class T> MLAU_HD T tsqrt(T x) { return sqrt(x); }
template <> MLAU_HD float tsqrt<float>(float x) { return sqrtf(x); }
template <class T> MLAU_HD T tabs(T x) { return fabs(x); }
template <> MLAU_HD float tabs<float>(float x) { return fabsf(x); }

// Epsilon of the WCNS nonlinear weights (interp.h:154,194).  In FP32 the
// reference's 1e-40 is a denormal that flush-to-zero removes, so FP32 uses a
// normal number far below any weight that matters.
template <class T> MLAU_HD T wcns_eps() { return T(1e-40); }
template <> MLAU_HD float wcns_eps<float>() { return 1e-30f; }

// funcs.h:23-43: ties go to a in max and to b in min.
template <class T> MLAU_HD T vmax(T a, T b) { return (a >= b) ? a : b; }
template <class T> MLAU_HD T vmin(T a, T b) { return (a >= b) ? b : a; }
template <class T> MLAU_HD T minmod(T a, T b)
{
    return vmin(vmax(a, b), T(0)) + vmax(vmin(a, b), T(0));
}

// ---------------------------------------------------------------------------
// Reconstruction: value at the left of face i+1/2 (fl) and at the right of
// face i-1/2 (fr) from the stencil f[0..4] centred on cell i.
// ---------------------------------------------------------------------------
// interp.h:30-37
template <class T> MLAU_HD void muscl_mm_lr(T f1, T f2, T f3, T &fl, T &fr)
{
    T df = T(0.5) * minmod(f2 - f1, f3 - f2);
    fl = f2 + df;
    fr = f2 - df;
}

// minmod3 (funcs.h:39-43)
template <class T> MLAU_HD T minmod3(T a, T b, T c)
{
    return vmin(vmax(vmax(a, b), c), T(0)) + vmax(vmin(vmin(a, b), c), T(0));
}

// interp.h:45-51: MUSCL with the MC limiter (alpha 2), the limiter of
// 2D/MPI/MRX/mhd_fd_ct_2d.c:107
template <class T> MLAU_HD void muscl_mc_lr(T f1, T f2, T f3, T &fl, T &fr)
{
    const T alpha = T(2.0);
    T df = T(0.5) * minmod(alpha * minmod(f2 - f1, f3 - f2), T(0.5) * (f3 - f1));
    fl = f2 + df;
    fr = f2 - df;
}

// interp.h:61-72: MUSCL with the Koren limiter
template <class T> MLAU_HD void muscl_kr_lr(T f1, T f2, T f3, T &fl, T &fr)
{
    const T d1 = T(2.0) * (f2 - f1);
    const T d2 = T(2.0) * (f3 - f2);
    const T dl = T(0.5) * minmod3(d1, d2, (T(0.5) * d1 + d2) / T(3.0));
    const T dr = T(0.5) * minmod3(d1, d2, (d1 + T(0.5) * d2) / T(3.0));
    fl = f2 + dl;
    fr = f2 - dr;
}

// Reconstruction codes: 1-4 are the drivers' ODR; 5 and 6 are 2nd-order MUSCL
// with the MC and Koren limiters in calc_flr's ODR 2 branch.  Every other
// order-dependent operation follows ODR 2 for them.
MLAU_HD int lin_odr(int odr) { return odr > 4 ? 2 : odr; }

// interp.h:106-146
template <class T> MLAU_HD void wcns3_lr(T f0, T f1, T f2, T &fl, T &fr)
{
    const T eps = wcns_eps<T>();
    T d0 = f0 - f1, d1 = f2 - f1;
    T s0 = d0 * d0, s1 = d1 * d1;
    T t = f2 - T(2.0) * f1 + f0;
    t = t * t;
    s0 = (T(1.0) + t / (s0 + eps));
    s1 = (T(1.0) + t / (s1 + eps));
    T a = T(0.25) * s0, b = T(0.75) * s1;
    a /= (a + b);
    b = T(1.0) - a;
    fl = T(0.5) * (a * (-f0 + T(3.0) * f1) + b * (f1 + f2));
    a = T(0.75) * s0;
    b = T(0.25) * s1;
    a /= (a + b);
    b = T(1.0) - a;
    fr = T(0.5) * (b * (-f2 + T(3.0) * f1) + a * (f1 + f0));
}

// interp.h:186-238
template <class T> MLAU_HD void wcns4_lr(T f0, T f1, T f2, T f3, T f4, T &fl, T &fr)
{
    const T eps = wcns_eps<T>();
    T p, q, s0, s1, s2;
    p = f0 - T(4.0) * f1 + T(3.0) * f2;
    q = f0 - T(2.0) * f1 + f2;
    s0 = T(13. / 12.) * q * q + T(0.25) * p * p;
    p = f1 - f3;
    q = f1 - T(2.0) * f2 + f3;
    s1 = T(13. / 12.) * q * q + T(0.25) * p * p;
    p = f4 - T(4.0) * f3 + T(3.0) * f2;
    q = f4 - T(2.0) * f3 + f2;
    s2 = T(13. / 12.) * q * q + T(0.25) * p * p;
    s0 = T(1.0) / (s0 * s0 + eps);
    s1 = T(1.0) / (s1 * s1 + eps);
    s2 = T(1.0) / (s2 * s2 + eps);
    // The three candidate stencils are shared by both sides.
    const T pa = T(3.0) * f0 - T(10.0) * f1 + T(15.0) * f2;
    const T pb = -f1 + T(6.0) * f2 + T(3.0) * f3;
    const T pc = +T(3.0) * f2 + T(6.0) * f3 - f4;
    T w0 = T(0.075) * s0, w1 = T(0.650) * s1, w2 = T(0.275) * s2;
    T r = T(1.0) / (w0 + w1 + w2);
    w0 *= r;
    w1 *= r;
    w2 = T(1.0) - w0 - w1;
    fl = T(0.125) * (+w0 * pa + w1 * pb + w2 * pc);
    const T qa = T(3.0) * f4 - T(10.0) * f3 + T(15.0) * f2;
    const T qb = -f3 + T(6.0) * f2 + T(3.0) * f1;
    const T qc = +T(3.0) * f2 + T(6.0) * f1 - f0;
    w0 = T(0.275) * s0;
    w1 = T(0.650) * s1;
    w2 = T(0.075) * s2;
    r = T(1.0) / (w0 + w1 + w2);
    w0 *= r;
    w1 *= r;
    w2 = T(1.0) - w0 - w1;
    fr = T(0.125) * (+w2 * qa + w1 * qb + w0 * qc);
}

// One-sided face values of include/interp.h - the value between f0 and fd
// (MUSCL, :25-28, :39-43, :55-60) or between f and fdn (WCNS, :75-104,
// :148-184).  No driver calls them; they complete the header's interface.
template <class T> MLAU_HD T muscl_mm_f(T fu, T f0, T fd)
{
    return f0 - T(0.5) * minmod(fu - f0, f0 - fd);
}
template <class T> MLAU_HD T muscl_mc_f(T fu, T f0, T fd)
{
    const T alpha = T(2.0);
    return f0 - T(0.5) * minmod(alpha * minmod(fu - f0, f0 - fd), T(0.5) * (fu - fd));
}
template <class T> MLAU_HD T muscl_kr_f(T fu, T f0, T fd)
{
    const T d1 = T(2.0) * (fu - f0);
    const T d2 = T(2.0) * (f0 - fd);
    return f0 - T(0.5) * minmod3(d1, d2, (T(0.5) * d1 + d2) / T(3.0));
}
template <class T> MLAU_HD T wcns3_f(T fup, T f, T fdn)
{
    const T eps = wcns_eps<T>();
    T d0 = fup - f, d1 = fdn - f;
    T s0 = d0 * d0, s1 = d1 * d1;
    T t = fup - T(2.0) * f + fdn;
    t = t * t;
    T a = T(0.25) * (T(1.0) + t / (s0 + eps));
    T b = T(0.75) * (T(1.0) + t / (s1 + eps));
    a /= (a + b);
    b = T(1.0) - a;
    return T(0.5) * (a * (-fup + T(3.0) * f) + b * (f + fdn));
}
template <class T> MLAU_HD T wcns4_f(T fuu, T fup, T f, T fdn, T fdd)
{
    const T eps = wcns_eps<T>();
    T p, q, s0, s1, s2;
    p = fuu - T(4.0) * fup + T(3.0) * f;
    q = fuu - T(2.0) * fup + f;
    s0 = T(13. / 12.) * q * q + T(0.25) * p * p;
    p = fup - fdn;
    q = fup - T(2.0) * f + fdn;
    s1 = T(13. / 12.) * q * q + T(0.25) * p * p;
    p = T(3.0) * f - T(4.0) * fdn + fdd;
    q = f - T(2.0) * fdn + fdd;
    s2 = T(13. / 12.) * q * q + T(0.25) * p * p;
    T w0 = T(0.075) / (s0 * s0 + eps);
    T w1 = T(0.650) / (s1 * s1 + eps);
    T w2 = T(0.275) / (s2 * s2 + eps);
    const T den = T(1.0) / (w0 + w1 + w2);
    w0 *= den;
    w1 *= den;
    w2 = T(1.0) - w0 - w1;
    return T(0.125) * (+w0 * (T(3.0) * fuu - T(10.0) * fup + T(15.0) * f)
                       + w1 * (-fup + T(6.0) * f + T(3.0) * fdn)
                       + w2 * (+T(3.0) * f + T(6.0) * fdn - fdd));
}

// calc_flr of the drivers (3D/MPI/OTvortex/mhd_fd_ct_3d.c:65-78).
template <class T> MLAU_HD void rec_lr(int odr, const T *f, T &fl, T &fr)
{
    if (odr == 4) wcns4_lr(f[0], f[1], f[2], f[3], f[4], fl, fr);
    else if (odr == 2) muscl_mm_lr(f[1], f[2], f[3], fl, fr);
    else if (odr == 3) wcns3_lr(f[1], f[2], f[3], fl, fr);
    else if (odr == 5) muscl_mc_lr(f[1], f[2], f[3], fl, fr);
    else if (odr == 6) muscl_kr_lr(f[1], f[2], f[3], fl, fr);
    else { fl = f[2]; fr = f[2]; }
}

// lcal_flr (mhd_fd_ct_3d.c:48-63): linear face interpolation, left value.
template <class T> MLAU_HD T lin_l(int odr, T f0, T f1, T f2, T f3, T f4)
{
    odr = lin_odr(odr);
    if (odr == 4)
        return T(0.003125) * (T(9.0) * f0 - T(56.0) * f1 + T(234.0) * f2 + T(144.0) * f3
                              - T(11.0) * f4);
    if (odr == 2) return T(0.25) * (-f1 + T(4.0) * f2 + f3);
    if (odr == 3) return T(0.125) * (-f1 + T(6.0) * f2 + T(3.0) * f3);
    return f2;
}
// ... and the right value (mirror stencil).
template <class T> MLAU_HD T lin_r(int odr, T f0, T f1, T f2, T f3, T f4)
{
    odr = lin_odr(odr);
    if (odr == 4)
        return T(0.003125) * (T(9.0) * f4 - T(56.0) * f3 + T(234.0) * f2 + T(144.0) * f1
                              - T(11.0) * f0);
    if (odr == 2) return T(0.25) * (-f3 + T(4.0) * f2 + f1);
    if (odr == 3) return T(0.125) * (-f3 + T(6.0) * f2 + T(3.0) * f1);
    return f2;
}

// calc_bc (mhd_fd_ct_3d.c:38-46)
template <class T> MLAU_HD T face2cen(int odr, T f0, T f1, T f2, T f3)
{
    if (lin_odr(odr) <= 2) return T(0.5) * (f1 + f2);
    return T(0.0625) * (T(9.0) * (f1 + f2) - (f0 + f3));
}

// calc_df (mhd_fd_ct_3d.c:80-88)
template <class T> MLAU_HD T fdiff(int odr, T f0, T f1, T f2, T f3)
{
    if (lin_odr(odr) <= 2) return f2 - f1;
    return (T(27.0) * (f2 - f1) - (f3 - f0)) / T(24.0);
}

// ---------------------------------------------------------------------------
// Characteristic reconstruction: q[k][m] = variable k at stencil point m,
// k = (ro, vn, vt, vu, bt, bu, pr).  Outputs ul (left of i+1/2), ur (right of
// i-1/2).  mhd_eigen.h:455-530 (full, mhd_eigen_st) and :609-684 (Alfven +
// entropy, mhd_eigen_ae).
// ---------------------------------------------------------------------------
template <class T>
MLAU_HD void zero_guard(const T q[7][5], T ul[7], T ur[7])
{
#pragma unroll
    for (int k = 1; k <= 5; k++) {
        bool z = (q[k][0] == T(0)) && (q[k][1] == T(0)) && (q[k][2] == T(0)) &&
                 (q[k][3] == T(0)) && (q[k][4] == T(0));
        if (z) { ul[k] = T(0); ur[k] = T(0); }
    }
}

// Alfven/entropy projection of the stencil q (variables x points) with the
// eigenvectors of the centre state qc.  Linear in q: the FP32-split mode
// passes perturbations from the cell centre here.
template <class T>
MLAU_HD void reconst_alfven_core(int odr, const T q[7][5], const T qc[7], T bn, T gamma, T ul[7],
                                 T ur[7])
{
    const T ro = qc[0], by = qc[4], bz = qc[5], pr = qc[6];
    T iro = T(1.0) / ro;
    T cs2 = gamma * pr * iro;
    T ca2 = bn * bn * iro;
    T ct2 = (by * by + bz * bz) * iro;
    T cb2 = cs2 + ca2 + ct2;
    T cf2 = T(0.5) * (cb2 + tsqrt(tabs(cb2 * cb2 - T(4.0) * cs2 * ca2)));
    T sro = tsqrt(ro);
    T isroh = T(0.5) / sro;
    T icf2 = T(1.0) / cf2;
    T byh = T(0.5) * by, bzh = T(0.5) * bz;

    T w[7][5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const T r = q[0][m], vx = q[1][m], vy = q[2][m], vz = q[3][m];
        const T b1 = q[4][m], b2 = q[5][m], p = q[6][m];
        w[0][m] = vx;
        w[1][m] = cf2 * r + (-by) * b1 + (-bz) * b2 - p;
        w[2][m] = by * b1 + bz * b2 + p;
        const T sy = sro * vy, sz = sro * vz;
        w[3][m] = sy + b1;
        w[4][m] = sy - b1;
        w[5][m] = sz + b2;
        w[6][m] = sz - b2;
    }
    T wl[7], wr[7];
#pragma unroll
    for (int n = 0; n < 7; n++) rec_lr(odr, w[n], wl[n], wr[n]);
    ul[0] = icf2 * wl[1] + icf2 * wl[2];
    ul[1] = wl[0];
    ul[2] = isroh * wl[3] + isroh * wl[4];
    ul[3] = isroh * wl[5] + isroh * wl[6];
    ul[4] = T(0.5) * wl[3] - T(0.5) * wl[4];
    ul[5] = T(0.5) * wl[5] - T(0.5) * wl[6];
    ul[6] = wl[2] - byh * wl[3] + byh * wl[4] - bzh * wl[5] + bzh * wl[6];
    ur[0] = icf2 * wr[1] + icf2 * wr[2];
    ur[1] = wr[0];
    ur[2] = isroh * wr[3] + isroh * wr[4];
    ur[3] = isroh * wr[5] + isroh * wr[6];
    ur[4] = T(0.5) * wr[3] - T(0.5) * wr[4];
    ur[5] = T(0.5) * wr[5] - T(0.5) * wr[6];
    ur[6] = wr[2] - byh * wr[3] + byh * wr[4] - bzh * wr[5] + bzh * wr[6];
}

template <class T>
MLAU_HD void reconst_alfven(int odr, const T q[7][5], T bn, T gamma, T ul[7], T ur[7])
{
    const T qc[7] = {q[0][2], q[1][2], q[2][2], q[3][2], q[4][2], q[5][2], q[6][2]};
    reconst_alfven_core(odr, q, qc, bn, gamma, ul, ur);
    zero_guard(q, ul, ur);
}

// Full 7-wave system (mhd_eigen_st, mhd_eigen.h:24-192).  Returns the row
// coefficients needed by the sparse projections below.
template <class T> struct Eigen7 {
    T a[7];  // fast row -cfaf*den, ... (l1 of the reference), a[0] unused
    T b[6];  // Alfven row (l2), b[2..5]
    T c[7];  // slow row (l3)
    T d6;    // entropy row pressure coefficient -1/a2
    T r[7], s[6], t[7];  // right eigenvectors: fast, Alfven, slow
    T lam[7];
};

template <class T>
MLAU_HD void eigen_full(T ro, T vx, T bx, T by, T bz, T pr, T gamma, Eigen7<T> &E)
{
    const T eps = T(1e-12);
    T sqrt2 = tsqrt(T(2.0));
    T iro = T(1.0) / ro;
    T sro = tsqrt(ro);
    T isro = T(1.0) / sro;
    T bxsr = bx * isro, bysr = by * isro, bzsr = bz * isro;
    T bx2 = bxsr * bxsr;
    T bt2 = bysr * bysr + bzsr * bzsr;
    T b2 = bx2 + bt2;
    T a2 = tabs(gamma * pr / ro);
    T aa = tsqrt(a2);
    T ca2 = bx2;
    T ca = tsqrt(ca2);
    T disc = tsqrt(tabs((a2 + b2) * (a2 + b2) - T(4.0) * a2 * ca2));
    T cf2 = tabs(T(0.5) * (a2 + b2 + disc));
    T cf = tsqrt(cf2);
    T cs2 = tabs(T(0.5) * (a2 + b2 - disc));
    T cs = tsqrt(cs2);
    bx2 = bx * bx;
    bt2 = by * by + bz * bz;
    b2 = bx2 + bt2;
    T den = T(1.0) / tsqrt(bt2);
    bool flag = (bt2 > eps * b2);
    T bey = flag ? (by * den) : (T(0.5) * sqrt2);
    T bez = flag ? (bz * den) : (T(0.5) * sqrt2);
    den = T(1.0) / tsqrt(tabs(cf2 - cs2));
    flag = ((bt2 > eps * b2) || (tabs(gamma * pr - bx2) > eps * gamma * pr));
    T af = flag ? (tsqrt(tabs(a2 - cs2)) * den) : T(1.0);
    T as = flag ? (tsqrt(tabs(cf2 - a2)) * den) : T(0.0);
    T sg = (bx > T(0)) ? T(1.0) : T(-1.0);
    T cfaf = cf * af, csas = cs * as, aaaf = aa * af, aaas = aa * as;
    den = T(0.5) / a2;
    E.lam[0] = vx - cf; E.lam[1] = vx - ca; E.lam[2] = vx - cs; E.lam[3] = vx;
    E.lam[4] = vx + cs; E.lam[5] = vx + ca; E.lam[6] = vx + cf;
    E.a[1] = -cfaf * den;
    E.a[2] = +csas * den * sg * bey;
    E.a[3] = +csas * den * sg * bez;
    E.a[4] = +aaas * den * isro * bey;
    E.a[5] = +aaas * den * isro * bez;
    E.a[6] = af * den * iro;
    E.b[2] = T(-0.5) * bez;
    E.b[3] = T(+0.5) * bey;
    E.b[4] = T(-0.5) * isro * bez * sg;
    E.b[5] = T(+0.5) * isro * bey * sg;
    E.c[1] = -csas * den;
    E.c[2] = -cfaf * den * sg * bey;
    E.c[3] = -cfaf * den * sg * bez;
    E.c[4] = -aaaf * den * isro * bey;
    E.c[5] = -aaaf * den * isro * bez;
    E.c[6] = as * den * iro;
    E.d6 = T(-1.0) / a2;
    E.r[0] = ro * af;
    E.r[1] = -cfaf;
    E.r[2] = +csas * sg * bey;
    E.r[3] = +csas * sg * bez;
    E.r[4] = +aaas * sro * bey;
    E.r[5] = +aaas * sro * bez;
    E.r[6] = af * gamma * pr;
    E.s[2] = -bez;
    E.s[3] = +bey;
    E.s[4] = -sro * bez * sg;
    E.s[5] = +sro * bey * sg;
    E.t[0] = ro * as;
    E.t[1] = -csas;
    E.t[2] = -cfaf * sg * bey;
    E.t[3] = -cfaf * sg * bez;
    E.t[4] = -aaaf * sro * bey;
    E.t[5] = -aaaf * sro * bez;
    E.t[6] = as * gamma * pr;
}

// Project one primitive vector on the 7 characteristic fields (rows ordered
// fast-, Alfven-, slow-, entropy, slow+, Alfven+, fast+).  Mirror rows share
// the odd (velocity) partial sums with their partners.
template <class T>
MLAU_HD void proj_full(const Eigen7<T> &E, T r, T vn, T vt, T vu, T bt, T bu, T p, T w[7])
{
    T oa = E.a[1] * vn + E.a[2] * vt + E.a[3] * vu;
    T pa4 = E.a[4] * bt, pa5 = E.a[5] * bu, pa6 = E.a[6] * p;
    w[0] = oa + pa4 + pa5 + pa6;
    w[6] = (-oa) + pa4 + pa5 + pa6;
    T ob = E.b[2] * vt + E.b[3] * vu;
    T pb4 = E.b[4] * bt, pb5 = E.b[5] * bu;
    w[1] = ob + pb4 + pb5;
    w[5] = (-ob) + pb4 + pb5;
    T oc = E.c[1] * vn + E.c[2] * vt + E.c[3] * vu;
    T pc4 = E.c[4] * bt, pc5 = E.c[5] * bu, pc6 = E.c[6] * p;
    w[2] = oc + pc4 + pc5 + pc6;
    w[4] = (-oc) + pc4 + pc5 + pc6;
    w[3] = r + E.d6 * p;
}

template <class T>
MLAU_HD void back_full(const Eigen7<T> &E, const T wl[7], T ul[7])
{
    ul[0] = E.r[0] * wl[0] + E.t[0] * wl[2] + wl[3] + E.t[0] * wl[4] + E.r[0] * wl[6];
    ul[1] = E.r[1] * wl[0] + E.t[1] * wl[2] - E.t[1] * wl[4] - E.r[1] * wl[6];
#pragma unroll
    for (int k = 2; k <= 3; k++)
        ul[k] = E.r[k] * wl[0] + E.s[k] * wl[1] + E.t[k] * wl[2] - E.t[k] * wl[4]
                - E.s[k] * wl[5] - E.r[k] * wl[6];
#pragma unroll
    for (int k = 4; k <= 5; k++)
        ul[k] = E.r[k] * wl[0] + E.s[k] * wl[1] + E.t[k] * wl[2] + E.t[k] * wl[4]
                + E.s[k] * wl[5] + E.r[k] * wl[6];
    ul[6] = E.r[6] * wl[0] + E.t[6] * wl[2] + E.t[6] * wl[4] + E.r[6] * wl[6];
}

template <class T>
MLAU_HD void reconst_full_core(int odr, const T q[7][5], const T qc[7], T bn, T gamma, T ul[7],
                               T ur[7])
{
    Eigen7<T> E;
    eigen_full(qc[0], qc[1], bn, qc[4], qc[5], qc[6], gamma, E);
    T w[7][5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        T wm[7];
        proj_full(E, q[0][m], q[1][m], q[2][m], q[3][m], q[4][m], q[5][m], q[6][m], wm);
#pragma unroll
        for (int n = 0; n < 7; n++) w[n][m] = wm[n];
    }
    T wl[7], wr[7];
#pragma unroll
    for (int n = 0; n < 7; n++) rec_lr(odr, w[n], wl[n], wr[n]);
    back_full(E, wl, ul);
    back_full(E, wr, ur);
}

template <class T>
MLAU_HD void reconst_full(int odr, const T q[7][5], T bn, T gamma, T ul[7], T ur[7])
{
    const T qc[7] = {q[0][2], q[1][2], q[2][2], q[3][2], q[4][2], q[5][2], q[6][2]};
    reconst_full_core(odr, q, qc, bn, gamma, ul, ur);
    zero_guard(q, ul, ur);
}

// The eigen-systems as include/mhd_eigen.h returns them: eigenvalues al[7]
// (the full system only; the others leave al untouched, as the reference's
// do), left eigenvectors as rows L[n][k] and right eigenvectors as R[n][k]
// (l_{n+1}[k] and r_{n+1}[k] in the header's 1-based names), every entry -
// zeros and their signs included - set as the header sets it.  The sparse
// projections above use the same coefficients without the zeros.
template <class T> MLAU_HD void mirror_row(const T a[7], T b[7])
{
    b[0] = a[0]; b[1] = -a[1]; b[2] = -a[2]; b[3] = -a[3];
    b[4] = a[4]; b[5] = a[5]; b[6] = a[6];
}

// mhd_eigen_st (mhd_eigen.h:24-192): fast, Alfven and slow pairs, entropy.
template <class T>
MLAU_HD void eigen_st_dense(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma, T al[7],
                            T L[7][7], T R[7][7])
{
    (void)vy;
    (void)vz;
    Eigen7<T> E;
    eigen_full(ro, vx, bx, by, bz, pr, gamma, E);
    const T z = T(0);
#pragma unroll
    for (int n = 0; n < 7; n++) al[n] = E.lam[n];
    L[0][0] = z;
    L[1][0] = z; L[1][1] = z; L[1][6] = z;
    L[2][0] = z;
#pragma unroll
    for (int k = 1; k < 7; k++) { L[0][k] = E.a[k]; L[2][k] = E.c[k]; }
#pragma unroll
    for (int k = 2; k < 6; k++) L[1][k] = E.b[k];
    L[3][0] = T(1.0);
    L[3][1] = z; L[3][2] = z; L[3][3] = z; L[3][4] = z; L[3][5] = z;
    L[3][6] = E.d6;
    R[1][0] = z; R[1][1] = z; R[1][6] = z;
#pragma unroll
    for (int k = 0; k < 7; k++) { R[0][k] = E.r[k]; R[2][k] = E.t[k]; }
#pragma unroll
    for (int k = 2; k < 6; k++) R[1][k] = E.s[k];
    R[3][0] = T(1.0);
#pragma unroll
    for (int k = 1; k < 7; k++) R[3][k] = z;
    mirror_row(L[0], L[6]); mirror_row(L[1], L[5]); mirror_row(L[2], L[4]);
    mirror_row(R[0], R[6]); mirror_row(R[1], R[5]); mirror_row(R[2], R[4]);
}

// Fast-speed quantities shared by the Alfven/entropy and Miyoshi systems
// (mhd_eigen.h:206-212, :337-343).
template <class T> MLAU_HD T fast_speed2(T ro, T bx, T by, T bz, T pr, T gamma)
{
    const T iro = T(1.0) / ro;
    const T cs2 = gamma * pr * iro;
    const T ca2 = bx * bx * iro;
    const T ct2 = (by * by + bz * bz) * iro;
    const T cb2 = cs2 + ca2 + ct2;
    return T(0.5) * (cb2 + tsqrt(tabs(cb2 * cb2 - T(4.0) * cs2 * ca2)));
}

// mhd_eigen_ae (mhd_eigen.h:326-453): Alfven and entropy modes.
template <class T>
MLAU_HD void eigen_ae_dense(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma, T al[7],
                            T L[7][7], T R[7][7])
{
    (void)vx; (void)vy; (void)vz; (void)al;
    const T cf2 = fast_speed2(ro, bx, by, bz, pr, gamma);
    const T sro = tsqrt(ro);
    const T isroh = T(0.5) / sro;
    const T icf2 = T(1.0) / cf2;
    const T byh = T(0.5) * by, bzh = T(0.5) * bz;
    const T z = T(0), one = T(1.0), h = T(0.5);
    const T l[7][7] = {{z, +one, z, z, z, z, z},
                       {cf2, z, z, z, -by, -bz, T(-1.0)},
                       {z, z, z, z, +by, +bz, +one},
                       {z, z, +sro, z, +one, z, z},
                       {z, z, +sro, z, T(-1.0), z, z},
                       {z, z, z, +sro, z, +one, z},
                       {z, z, z, +sro, z, T(-1.0), z}};
    const T r[7][7] = {{z, +one, z, z, z, z, z},
                       {+icf2, z, z, z, z, z, z},
                       {+icf2, z, z, z, z, z, +one},
                       {z, z, +isroh, z, +h, z, -byh},
                       {z, z, +isroh, z, T(-0.5), z, +byh},
                       {z, z, z, +isroh, z, +h, -bzh},
                       {z, z, z, +isroh, z, T(-0.5), +bzh}};
#pragma unroll
    for (int n = 0; n < 7; n++)
#pragma unroll
        for (int k = 0; k < 7; k++) { L[n][k] = l[n][k]; R[n][k] = r[n][k]; }
}

// mhd_eigen_mi (mhd_eigen.h:194-324): Miyoshi's fast and Alfven modes (the
// slow mode is ignored).
template <class T>
MLAU_HD void eigen_mi_dense(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma, T al[7],
                            T L[7][7], T R[7][7])
{
    (void)vx; (void)vy; (void)vz; (void)al;
    const T cf2 = fast_speed2(ro, bx, by, bz, pr, gamma);
    const T cf = tsqrt(cf2);
    const T rcf = ro * cf;
    const T sro = tsqrt(ro);
    const T isroh = T(0.5) / sro;
    const T icf2 = T(1.0) / cf2;
    const T icf2h = T(0.5) * icf2;
    const T ircfh = T(0.5) / rcf;
    const T byh = T(0.5) * by, bzh = T(0.5) * bz;
    const T z = T(0), one = T(1.0);
    const T l[7][7] = {{z, -rcf, z, z, +by, +bz, +one},
                       {cf2, z, z, z, -by, -bz, -one},
                       {z, +rcf, z, z, +by, +bz, +one},
                       {z, z, +sro, z, +one, z, z},
                       {z, z, +sro, z, -one, z, z},
                       {z, z, z, +sro, z, +one, z},
                       {z, z, z, +sro, z, -one, z}};
    const T r[7][7] = {{+icf2h, -ircfh, z, z, z, z, T(0.5)},
                       {+icf2, z, z, z, z, z, z},
                       {+icf2h, +ircfh, z, z, z, z, T(0.5)},
                       {z, z, +isroh, z, T(0.5), z, -byh},
                       {z, z, +isroh, z, T(-0.5), z, +byh},
                       {z, z, z, +isroh, z, T(0.5), -bzh},
                       {z, z, z, +isroh, z, T(-0.5), +bzh}};
#pragma unroll
    for (int n = 0; n < 7; n++)
#pragma unroll
        for (int k = 0; k < 7; k++) { L[n][k] = l[n][k]; R[n][k] = r[n][k]; }
}

// Fast + Alfven projection of Miyoshi (mhd_m_reconst with mhd_eigen_mi,
// mhd_eigen.h:194-324, 532-607; the slow mode is ignored), the header's
// alternative to the full system.  The reference multiplies the dense 7x7
// rows, zeros included, in index order; so does this (the zero products
// decide signed zeros).
template <class T>
MLAU_HD void reconst_miyoshi(int odr, const T q[7][5], T bn, T gamma, T ul[7], T ur[7])
{
    T al[7], L[7][7], R[7][7];
    eigen_mi_dense(q[0][2], q[1][2], q[2][2], q[3][2], bn, q[4][2], q[5][2], q[6][2], gamma, al,
                   L, R);
    T w[7][5];
#pragma unroll
    for (int n = 0; n < 7; n++)
#pragma unroll
        for (int m = 0; m < 5; m++)
            w[n][m] = (+L[n][0] * q[0][m] + L[n][1] * q[1][m] + L[n][2] * q[2][m]
                       + L[n][3] * q[3][m] + L[n][4] * q[4][m] + L[n][5] * q[5][m]
                       + L[n][6] * q[6][m]);
    T wl[7], wr[7];
#pragma unroll
    for (int n = 0; n < 7; n++) rec_lr(odr, w[n], wl[n], wr[n]);
#pragma unroll
    for (int n = 0; n < 7; n++) {
        ul[n] = R[0][n] * wl[0] + R[1][n] * wl[1] + R[2][n] * wl[2] + R[3][n] * wl[3]
                + R[4][n] * wl[4] + R[5][n] * wl[5] + R[6][n] * wl[6];
        ur[n] = R[0][n] * wr[0] + R[1][n] * wr[1] + R[2][n] * wr[2] + R[3][n] * wr[3]
                + R[4][n] * wr[4] + R[5][n] * wr[5] + R[6][n] * wr[6];
    }
    zero_guard(q, ul, ur);
}

// The eigen-system of a face: the full system (or Miyoshi's, eig = 1) where
// the largest sonic Mach^2 of the three central cells is at least 1, the
// Alfven + entropy system elsewhere (mhd_fd_ct_3d.c:416-420).
enum { EIG_FULL = 0, EIG_MIYOSHI = 1 };
template <class T>
MLAU_HD void reconst_face(int odr, int eig, T mach2, const T q[7][5], T bn, T gamma, T ul[7],
                          T ur[7])
{
    if (mach2 >= T(1.0)) {
        if (eig == EIG_MIYOSHI) reconst_miyoshi(odr, q, bn, gamma, ul, ur);
        else reconst_full(odr, q, bn, gamma, ul, ur);
    } else {
        reconst_alfven(odr, q, bn, gamma, ul, ur);
    }
}

// Characteristic reconstruction of an s-point stencil with any eigen-system
// and any face interpolation, as include/mhd_eigen.h's mhd_c_reconst /
// mhd_a_reconst / mhd_m_reconst compute it (:455-684): eigenvectors of the
// centre point s/2 (identity where the system leaves an entry unset), dense
// projection w = L q, func_lr on each characteristic field, back-projection
// with R, then the exact-zero guard on the transverse velocities and fields.
// eig: eigen_st_dense, eigen_ae_dense or eigen_mi_dense.  s is at most
// kMaxStencil (the drivers use 5); a larger s returns NaN faces.
constexpr int kMaxStencil = 8;

template <class T, class EIG, class LR>
MLAU_HD void reconst_dense(EIG eig, const T *ro, const T *vx, const T *vy, const T *vz,
                           const T *by, const T *bz, const T *pr, T bx, T gamma, int s, T *ul,
                           T *ur, LR func_lr)
{
    if (s < 1 || s > kMaxStencil) {
        for (int n = 0; n < 7; n++) { ul[n] = T(NAN); ur[n] = T(NAN); }
        return;
    }
    T al[7], L[7][7], R[7][7];
    for (int n = 0; n < 7; n++)
        for (int k = 0; k < 7; k++) { L[n][k] = (n == k) ? T(1.0) : T(0); R[n][k] = L[n][k]; }
    const int c = s / 2;
    eig(ro[c], vx[c], vy[c], vz[c], bx, by[c], bz[c], pr[c], gamma, al, L, R);
    T w[7][kMaxStencil], wl[7], wr[7];
    for (int m = 0; m < s; m++)
        for (int n = 0; n < 7; n++)
            w[n][m] = (+L[n][0] * ro[m] + L[n][1] * vx[m] + L[n][2] * vy[m] + L[n][3] * vz[m]
                       + L[n][4] * by[m] + L[n][5] * bz[m] + L[n][6] * pr[m]);
    for (int n = 0; n < 7; n++) func_lr(&w[n][0], &wl[n], &wr[n]);
    for (int n = 0; n < 7; n++)
        ul[n] = R[0][n] * wl[0] + R[1][n] * wl[1] + R[2][n] * wl[2] + R[3][n] * wl[3]
                + R[4][n] * wl[4] + R[5][n] * wl[5] + R[6][n] * wl[6];
    for (int n = 0; n < 7; n++)
        ur[n] = R[0][n] * wr[0] + R[1][n] * wr[1] + R[2][n] * wr[2] + R[3][n] * wr[3]
                + R[4][n] * wr[4] + R[5][n] * wr[5] + R[6][n] * wr[6];
    const T *tr[5] = {vx, vy, vz, by, bz};
    for (int k = 0; k < 5; k++) {
        bool z = true;
        for (int m = 0; m < s; m++) z = z && (tr[k][m] == T(0));
        if (z) { ul[k + 1] = T(0); ur[k + 1] = T(0); }
    }
}

// mhd_reconst (mhd_eigen.h:686-724): func_lr on the primitives themselves.
template <class T, class LR>
MLAU_HD void reconst_prim(const T *ro, const T *vx, const T *vy, const T *vz, const T *by,
                          const T *bz, const T *pr, int s, T *ul, T *ur, LR func_lr)
{
    if (s < 1 || s > kMaxStencil) {
        for (int n = 0; n < 7; n++) { ul[n] = T(NAN); ur[n] = T(NAN); }
        return;
    }
    const T *q[7] = {ro, vx, vy, vz, by, bz, pr};
    T w[kMaxStencil];
    for (int n = 0; n < 7; n++) {
        for (int m = 0; m < s; m++) w[m] = q[n][m];
        func_lr(w, &ul[n], &ur[n]);
    }
}

// ---------------------------------------------------------------------------
// Riemann solvers (include/mhd_flux.h).  l/r: (ro, vn, vt, vu, bt, bu, pr),
// bn: face-normal B, dv[2]: shock sensor (MLAU, LHLLD).  f: (ro, mn, mt, mu,
// bt, bu, en) fluxes.
// ---------------------------------------------------------------------------
enum { FLUX_MLAU = 0, FLUX_LHLLD = 1, FLUX_HLLD = 2, FLUX_ROE = 3 };

// calc_flux_mlau, mhd_flux.h:26-213.  With JUMPS, the total-pressure jump
// ptr-ptl (jp) and normal-velocity jump vnr-vnl (jv) come from the caller,
// formed from split (base + perturbation) parts instead of rounded values.
template <class T, bool JUMPS = false>
MLAU_HD void flux_mlau(const T *L, const T *R, T bnc, T gamma, T dv0, T dv1, T *f, T jp = T(0),
                       T jv = T(0))
{
    const T EPS = T(1e-8);
    const T rol = L[0], vnl = L[1], vtl = L[2], vul = L[3], btl = L[4], bul = L[5], prl = L[6];
    const T ror = R[0], vnr = R[1], vtr = R[2], vur = R[3], btr = R[4], bur = R[5], prr = R[6];
    T gm1i = T(1.0) / (gamma - T(1.0));
    T bnc2 = bnc * bnc;
    T sgn = (bnc > T(0)) ? T(1.0) : T(-1.0);
    T bnca = sgn * bnc;
    T roli = T(1.0) / rol;
    T vl2 = vnl * vnl + vtl * vtl + vul * vul;
    T pml = T(0.5) * (btl * btl + bul * bul);
    T ptl = prl + pml;
    T enl = gm1i * prl + pml + T(0.5) * rol * vl2;
    T hnl = (enl + ptl) * roli;
    T rori = T(1.0) / ror;
    T vr2 = vnr * vnr + vtr * vtr + vur * vur;
    T pmr = T(0.5) * (btr * btr + bur * bur);
    T ptr = prr + pmr;
    T enr = gm1i * prr + pmr + T(0.5) * ror * vr2;
    T hnr = (enr + ptr) * rori;
    T cl2 = gamma * prl * roli, cr2 = gamma * prr * rori;
    T cal2 = bnc2 * roli, car2 = bnc2 * rori;
    T cbl2 = cl2 + cal2 + T(2.0) * pml * roli;
    T cbr2 = cr2 + car2 + T(2.0) * pmr * rori;
    T cfl2 = T(0.5) * (cbl2 + tsqrt(tabs(cbl2 * cbl2 - T(4.0) * cl2 * cal2)));
    T cfr2 = T(0.5) * (cbr2 + tsqrt(tabs(cbr2 * cbr2 - T(4.0) * cr2 * car2)));
    cbl2 = vl2 + cal2 + T(2.0) * pml * roli;
    cbr2 = vr2 + car2 + T(2.0) * pmr * rori;
    T ccl2 = T(0.5) * (cbl2 + tsqrt(tabs(cbl2 * cbl2 - T(4.0) * vl2 * cal2)));
    T ccr2 = T(0.5) * (cbr2 + tsqrt(tabs(cbr2 * cbr2 - T(4.0) * vr2 * car2)));
    T cmax = tsqrt(vmax(cfl2, cfr2));
    T cfn = cmax;
    T cfni = T(1.0) / cfn;
    T sl = vmin(T(0.0), vmin(vnl, vnr) - cmax);
    T sr = vmax(T(0.0), vmax(vnl, vnr) + cmax);
    T mal = vnl * cfni, mar = vnr * cfni;
    T snl = (mal > T(0)) ? T(1.0) : T(-1.0);
    T snr = (mar > T(0)) ? T(1.0) : T(-1.0);
    T theta = vmin(T(1.0), (cfn - vmin(dv0, T(0.0))) / (cfn - vmin(dv1, T(0.0))));
    theta *= theta;
    theta *= theta;
    const T alpha = T(0.1875), beta = T(0.125);
    T malp1 = mal + T(1.0), marm1 = mar - T(1.0);
    T mal2m1 = mal * mal - T(1.0), mar2m1 = mar * mar - T(1.0);
    T bfl, ffl, bfr, ffr;
    if (snl * mal > T(1.0)) {
        bfl = T(0.5) * (T(1.0) + snl);
        ffl = bfl * mal;
    } else {
        bfl = +T(0.25) * malp1 * malp1 * (T(2.0) - mal) + alpha * mal * mal2m1 * mal2m1;
        ffl = +T(0.25) * malp1 * malp1 + beta * mal2m1 * mal2m1;
    }
    if (snr * mar > T(1.0)) {
        bfr = T(0.5) * (T(1.0) - snr);
        ffr = bfr * mar;
    } else {
        bfr = +T(0.25) * marm1 * marm1 * (T(2.0) + mar) - alpha * mar * mar2m1 * mar2m1;
        ffr = -T(0.25) * marm1 * marm1 - beta * mar2m1 * mar2m1;
    }
    T mnc = ffl + ffr;
    T mflux = mnc * cfn;
    const T dpt = JUMPS ? jp : (ptr - ptl);
    const T dvn = JUMPS ? jv : (vnr - vnl);
    mflux -= vmax(T(1.0) - tabs(mnc), T(0)) * theta * cfni * dpt / (rol + ror);
    T dir = (mflux > T(0)) ? T(1.0) : T(-1.0);
    T dirl = T(0.5) * (T(1.0) + dir);
    T dirr = T(1.0) - dirl;
    mflux *= (dirl * rol + dirr * ror);
    T mfl = mflux * dirl;
    T mfr = mflux - mfl;
    T ptot = bfl * ptl + bfr * ptr;
    T cfmod = tsqrt(vmax(ccl2, ccr2));
    ptot -= T(0.25) * bfl * bfr * (rol + ror) * cfmod * dvn;
    ptot -= T(0.5) * (T(1.0) - cfmod * cfni) * (bfl + bfr - T(1.0)) * (ptl + ptr);
    T slvl = sl - vnl, srvr = sr - vnr;
    T snc = dirl * sl + dirr * sr;
    T vndnm = mflux + dirl * rol * slvl + dirr * ror * srvr;
    T vnc = ((tabs(vndnm) > EPS) && (snc != T(0))) ? (mflux * snc / vndnm)
                                                    : (dirl * vnl + dirr * vnr);
    T slvc = sl - vnc, srvc = sr - vnc;
    T slvci = T(1.0) / slvc, srvci = T(1.0) / srvc;
    T rhdl = rol * slvl * slvc - bnc2;
    T rhdr = ror * srvr * srvc - bnc2;
    T dvtl = T(0.0), dvul = T(0.0), dbtl = T(0.0), dbul = T(0.0);
    T dvtr = T(0.0), dvur = T(0.0), dbtr = T(0.0), dbur = T(0.0);
    if (tabs(rhdl) > EPS) {
        T g = (vnc - vnl) / rhdl;
        dvtl = -bnc * btl * g;
        dvul = -bnc * bul * g;
        dbtl = bnc2 * btl * g * slvci;
        dbul = bnc2 * bul * g * slvci;
    }
    if (tabs(rhdr) > EPS) {
        T g = (vnc - vnr) / rhdr;
        dvtr = -bnc * btr * g;
        dvur = -bnc * bur * g;
        dbtr = bnc2 * btr * g * srvci;
        dbur = bnc2 * bur * g * srvci;
    }
    T cmpl = slvl * slvci, cmpr = srvr * srvci;
    T ro2l = rol * cmpl;
    T srol = tsqrt(ro2l);
    T vt2l = dvtl + vtl, vu2l = dvul + vul;
    T bt2l = dbtl + btl * cmpl, bu2l = dbul + bul * cmpl;
    T ro2r = ror * cmpr;
    T sror = tsqrt(ro2r);
    T vt2r = dvtr + vtr, vu2r = dvur + vur;
    T bt2r = dbtr + btr * cmpr, bu2r = dbur + bur * cmpr;
    T sroi = T(1.0) / (srol + sror);
    T srollri = srol * sroi, srorlri = sror * sroi;
    T bnflb = sgn * vmin(vmax(T(0.0), srollri * (bnca + sror * vnc)), bnca);
    T bnfrb = sgn * vmin(vmax(T(0.0), srorlri * (bnca - srol * vnc)), bnca);
    T bnflv = sgn * vmin(vmax(T(0.0), srorlri * (bnca + mflux / sror)), bnca);
    T bnfrv = sgn * vmin(vmax(T(0.0), srollri * (bnca - mflux / srol)), bnca);
    T bnsrv = vmax(bnca - dir * vnc * (dirl * srol + dirr * sror), T(0.0));
    T ccb = sroi * bnsrv;
    T ccv = srol * sror * ccb;
    T bnvt = bnflb * vt2l + bnfrb * vt2r + ccb * (bt2r - bt2l);
    T bnvu = bnflb * vu2l + bnfrb * vu2r + ccb * (bu2r - bu2l);
    T bnbt = bnflv * bt2l + bnfrv * bt2r + ccv * (vt2r - vt2l);
    T bnbu = bnflv * bu2l + bnfrv * bu2r + ccv * (vu2r - vu2l);
    bnvt -= vnc * (dirl * dbtl + dirr * dbtr);
    bnvu -= vnc * (dirl * dbul + dirr * dbur);
    bnbt -= mflux * (dirl * dvtl + dirr * dvtr);
    bnbu -= mflux * (dirl * dvul + dirr * dvur);
    f[0] = mflux;
    f[1] = mfl * vnl + mfr * vnr + ptot - T(0.5) * bnc2;
    f[2] = mfl * vtl + mfr * vtr - bnbt;
    f[3] = mfl * vul + mfr * vur - bnbu;
    f[4] = mfl * btl * roli + mfr * btr * rori - bnvt;
    f[5] = mfl * bul * roli + mfr * bur * rori - bnvu;
    T vb1 = dirl * (vtl * btl + vul * bul) + dirr * (vtr * btr + vur * bur);
    T vb2 = dirl * (vt2l * bt2l + vu2l * bu2l) + dirr * (vt2r * bt2r + vu2r * bu2r);
    T rv2b2 = (mflux * vnc - bnc2);
    rv2b2 *= rv2b2;
    T vb3 = T(0.0);
    if (rv2b2 > EPS * EPS) {
        vb3 = (+(f[2] * vnc + f[4] * bnc) * (f[2] * bnc + f[4] * mflux)
               + (f[3] * vnc + f[5] * bnc) * (f[3] * bnc + f[5] * mflux)) / rv2b2;
    }
    T bnvb = sgn * (bnca * (snc * vb2 - vnc * vb1) * (dirl * slvci + dirr * srvci)
                    + bnsrv * (vb3 - vb2));
    f[6] = mfl * hnl + mfr * hnr - bnvb;
}

// calc_flux_hlld (mhd_flux.h:456-582, LOWDISS=false) and calc_flux_lhlld
// (mhd_flux.h:584-719, LOWDISS=true).
template <class T, bool LOWDISS, bool JUMPS = false>
MLAU_HD void flux_hlld(const T *L, const T *R, T bnc, T gamma, T dv0, T dv1, T *f, T jp = T(0),
                       T jv = T(0))
{
    const T EPS = T(1e-8);
    const T rol = L[0], vnl = L[1], vtl = L[2], vul = L[3], btl = L[4], bul = L[5], prl = L[6];
    const T ror = R[0], vnr = R[1], vtr = R[2], vur = R[3], btr = R[4], bur = R[5], prr = R[6];
    T gm1i = T(1.0) / (gamma - T(1.0));
    T bnc2 = bnc * bnc;
    T sgn = (bnc > T(0)) ? T(1.0) : T(-1.0);
    T roli = T(1.0) / rol;
    T pml = T(0.5) * (btl * btl + bul * bul);
    T ptl = prl + pml;
    T vl2 = vnl * vnl + vtl * vtl + vul * vul;
    T enl = gm1i * prl + pml + T(0.5) * rol * vl2;
    T vbl = vtl * btl + vul * bul;
    T rori = T(1.0) / ror;
    T pmr = T(0.5) * (btr * btr + bur * bur);
    T ptr = prr + pmr;
    T vr2 = vnr * vnr + vtr * vtr + vur * vur;
    T enr = gm1i * prr + pmr + T(0.5) * ror * vr2;
    T vbr = vtr * btr + vur * bur;
    T cl2 = gamma * prl * roli, cr2 = gamma * prr * rori;
    T cal2 = bnc2 * roli, car2 = bnc2 * rori;
    T cbl2 = cl2 + cal2 + T(2.0) * pml * roli;
    T cbr2 = cr2 + car2 + T(2.0) * pmr * rori;
    T cfl2 = T(0.5) * (cbl2 + tsqrt(tabs(cbl2 * cbl2 - T(4.0) * cl2 * cal2)));
    T cfr2 = T(0.5) * (cbr2 + tsqrt(tabs(cbr2 * cbr2 - T(4.0) * cr2 * car2)));
    T cmax, vnc, ptc, slvl, srvr, rslvl, rsrvr, drsvi, sl, sr;
    if (!LOWDISS) {
        cmax = vmax(tsqrt(cfl2), tsqrt(cfr2));
        sl = vmin(T(0.0), vmin(vnl, vnr) - cmax);
        sr = vmax(T(0.0), vmax(vnl, vnr) + cmax);
        slvl = sl - vnl;
        srvr = sr - vnr;
        rslvl = rol * slvl;
        rsrvr = ror * srvr;
        drsvi = T(1.0) / (rsrvr - rslvl);
        if (JUMPS) {
            vnc = (rsrvr * vnr - rslvl * vnl - jp) * drsvi;
            ptc = (rsrvr * ptl - rslvl * ptr + rsrvr * rslvl * jv) * drsvi;
        } else {
            vnc = (rsrvr * vnr - rslvl * vnl - ptr + ptl) * drsvi;
            ptc = (rsrvr * ptl - rslvl * ptr + rsrvr * rslvl * (vnr - vnl)) * drsvi;
        }
    } else {
        cbl2 = vl2 + cal2 + T(2.0) * pml * roli;
        cbr2 = vr2 + car2 + T(2.0) * pmr * rori;
        T ccl2 = T(0.5) * (cbl2 + tsqrt(tabs(cbl2 * cbl2 - T(4.0) * vl2 * cal2)));
        T ccr2 = T(0.5) * (cbr2 + tsqrt(tabs(cbr2 * cbr2 - T(4.0) * vr2 * car2)));
        cmax = tsqrt(vmax(cfl2, cfr2));
        sl = vmin(T(0.0), vmin(vnl, vnr) - cmax);
        sr = vmax(T(0.0), vmax(vnl, vnr) + cmax);
        slvl = sl - vnl;
        srvr = sr - vnr;
        rslvl = rol * slvl;
        rsrvr = ror * srvr;
        drsvi = T(1.0) / (rsrvr - rslvl);
        T theta = vmin(T(1.0), (cmax - vmin(dv0, T(0.0))) / (cmax - vmin(dv1, T(0.0))));
        theta *= theta;
        theta *= theta;
        vnc = (rsrvr * vnr - rslvl * vnl - theta * (JUMPS ? jp : (ptr - ptl))) * drsvi;
        T mcc = vmin(T(1.0), tsqrt(vmax(ccl2, ccr2)) / cmax);
        ptc = (rsrvr * ptl - rslvl * ptr
               + (mcc * (T(2.0) - mcc)) * rsrvr * rslvl * (JUMPS ? jv : (vnr - vnl)))
              * drsvi;
    }
    T slvc = sl - vnc, srvc = sr - vnc;
    T ro2l = rslvl / slvc, ro2r = rsrvr / srvc;
    T rhdl = rslvl * slvc - bnc2, rhdr = rsrvr * srvc - bnc2;
    T vt2l, vu2l, bt2l, bu2l, vt2r, vu2r, bt2r, bu2r;
    if (tabs(rhdl) > EPS) {
        T rhdli = T(1.0) / rhdl;
        T rhnvl = (vnl - vnc) * bnc;
        T rhnbl = rslvl * slvl - bnc2;
        vt2l = vtl + rhnvl * rhdli * btl;
        vu2l = vul + rhnvl * rhdli * bul;
        bt2l = rhnbl * rhdli * btl;
        bu2l = rhnbl * rhdli * bul;
    } else {
        vt2l = vtl; vu2l = vul; bt2l = btl; bu2l = bul;
    }
    if (tabs(rhdr) > EPS) {
        T rhdri = T(1.0) / rhdr;
        T rhnvr = (vnr - vnc) * bnc;
        T rhnbr = rsrvr * srvr - bnc2;
        vt2r = vtr + rhnvr * rhdri * btr;
        vu2r = vur + rhnvr * rhdri * bur;
        bt2r = rhnbr * rhdri * btr;
        bu2r = rhnbr * rhdri * bur;
    } else {
        vt2r = vtr; vu2r = vur; bt2r = btr; bu2r = bur;
    }
    T vb2l = vt2l * bt2l + vu2l * bu2l;
    T vb2r = vt2r * bt2r + vu2r * bu2r;
    T en2l = (slvl * enl - ptl * vnl + ptc * vnc + bnc * (vbl - vb2l)) / slvc;
    T en2r = (srvr * enr - ptr * vnr + ptc * vnc + bnc * (vbr - vb2r)) / srvc;
    T rro2l = tsqrt(ro2l), rro2r = tsqrt(ro2r);
    T rro2i = T(1.0) / (rro2r + rro2l);
    T vt3m = (rro2r * vt2r + rro2l * vt2l + (bt2r - bt2l) * sgn) * rro2i;
    T vu3m = (rro2r * vu2r + rro2l * vu2l + (bu2r - bu2l) * sgn) * rro2i;
    T bt3m = (rro2l * bt2r + rro2r * bt2l + rro2r * rro2l * (vt2r - vt2l) * sgn) * rro2i;
    T bu3m = (rro2l * bu2r + rro2r * bu2l + rro2r * rro2l * (vu2r - vu2l) * sgn) * rro2i;
    T vb3m = vt3m * bt3m + vu3m * bu3m;
    T en3l = en2l - rro2l * (vb2l - vb3m) * sgn;
    T en3r = en2r + rro2r * (vb2r - vb3m) * sgn;
    T hl = (vnc > T(0)) ? T(1.0) : T(0.0);
    T hr = T(1.0) - hl;
    T h2l = (vnc - tabs(bnc) / rro2l > T(0)) ? T(1.0) : T(0.0);
    T h3l = (T(1.0) - h2l) * hl;
    T h2r = (vnc + tabs(bnc) / rro2r > T(0)) ? T(0.0) : T(1.0);
    T h3r = (T(1.0) - h2r) * hr;
    T rou = ro2l * hl + ro2r * hr;
    T vtu = vt2l * h2l + vt3m * (h3l + h3r) + vt2r * h2r;
    T vuu = vu2l * h2l + vu3m * (h3l + h3r) + vu2r * h2r;
    T btu = bt2l * h2l + bt3m * (h3l + h3r) + bt2r * h2r;
    T buu = bu2l * h2l + bu3m * (h3l + h3r) + bu2r * h2r;
    T enu = en2l * h2l + en3l * h3l + en3r * h3r + en2r * h2r;
    f[0] = rou * vnc;
    f[1] = rou * vnc * vnc + ptc - bnc2 * T(0.5);
    f[2] = rou * vtu * vnc - bnc * btu;
    f[3] = rou * vuu * vnc - bnc * buu;
    f[4] = btu * vnc - bnc * vtu;
    f[5] = buu * vnc - bnc * vuu;
    f[6] = (enu + ptc) * vnc - bnc * (vtu * btu + vuu * buu);
}

// calc_flux_roe, mhd_flux.h:215-454 (dv unused).
template <class T>
MLAU_HD void flux_roe(const T *L, const T *R, T bnc, T gamma, T *f)
{
    const T EPS = T(1e-8);
    const T rol = L[0], vnl = L[1], vtl = L[2], vul = L[3], btl = L[4], bul = L[5], prl = L[6];
    const T ror = R[0], vnr = R[1], vtr = R[2], vur = R[3], btr = R[4], bur = R[5], prr = R[6];
    T gm1 = gamma - T(1.0), gm2 = gamma - T(2.0), gm1i = T(1.0) / gm1;
    T roli = T(1.0) / rol, rori = T(1.0) / ror;
    T rrol = tsqrt(rol), rror = tsqrt(ror);
    T rroi = T(1.0) / (rrol + rror);
    T robar = rrol * rror;
    T robari = T(1.0) / robar;
    T rrobar = tsqrt(robar);
    T rrobai = tsqrt(robari);
    T vnbar = (rrol * vnl + rror * vnr) * rroi;
    T vtbar = (rrol * vtl + rror * vtr) * rroi;
    T vubar = (rrol * vul + rror * vur) * rroi;
    T bnbar = bnc;
    T btbar = (rrol * btr + rror * btl) * rroi;
    T bubar = (rrol * bur + rror * bul) * rroi;
    T hl = (+gamma * gm1i * prl * roli + T(0.5) * (vnl * vnl + vtl * vtl + vul * vul)
            + (bnbar * bnbar + btl * btl + bul * bul) * roli);
    T hr = (+gamma * gm1i * prr * rori + T(0.5) * (vnr * vnr + vtr * vtr + vur * vur)
            + (bnbar * bnbar + btr * btr + bur * bur) * rori);
    T hbar = (rrol * hl + rror * hr) * rroi;
    T btave = T(0.5) * (btl + btr), buave = T(0.5) * (bul + bur);
    T sgn = (bnbar > T(0)) ? T(1.0) : T(-1.0);
    T db2 = T(0.5) * gm2 * gm1i * ((btr - btl) * (btr - btl) + (bur - bul) * (bur - bul))
            * rroi * rroi;
    T kin = T(0.5) * (vnbar * vnbar + vtbar * vtbar + vubar * vubar);
    T bb = (bnbar * bnbar + btbar * btbar + bubar * bubar);
    T c2 = gm1 * (+hbar - kin - db2 - bb * robari);
    T a2 = (gm1 * (+hbar - kin - db2) - gm2 * bb * robari);
    T ca2 = bnbar * bnbar * robari;
    T cb2 = (btbar * btbar + bubar * bubar) * robari;
    T cf2 = T(0.5) * (a2 + tsqrt(cb2 * (a2 + c2 + ca2) + (c2 - ca2) * (c2 - ca2)));
    T cs2 = c2 * ca2 / cf2;
    T cf = tsqrt(cf2), cs = tsqrt(cs2), ca = tsqrt(ca2), c = tsqrt(c2);
    T cfi = T(1.0) / cf;
    T sgr1 = btbar * btbar + bubar * bubar - EPS;
    T sf11 = (sgr1 > T(0)) ? T(1.0) : T(0.0);
    T sf21 = T(1.0) - sf11;
    T beti = T(1.0) / tsqrt(btbar * btbar + bubar * bubar + sf21);
    T bett = sf11 * btbar * beti + sf21 * tsqrt(T(0.5));
    T betu = sf11 * bubar * beti + sf21 * tsqrt(T(0.5));
    T sgr2 = (btbar * btbar + bubar * bubar) * robari + tabs(ca2 - c2) - EPS;
    T sf12 = (sgr2 > T(0)) ? T(1.0) : T(0.0);
    T sf22 = T(1.0) - sf12;
    T cfca = vmax(T(0.0), cf2 - ca2);
    T cfcs = vmax(T(0.0), cf2 - cs2);
    T cfa = vmax(T(0.0), cf2 - c2);
    T alpi = T(1.0) / tsqrt(cfcs + sf22);
    T alpf = sf12 * tsqrt(cfca) * alpi + sf22;
    T alps = sf12 * tsqrt(cfa) * alpi;
    const T eeps = T(0.0);
    T ev[7];
    ev[0] = vmax(tabs(vnbar + cf), eeps);
    ev[1] = vmax(tabs(vnbar - cf), eeps);
    ev[2] = vmax(tabs(vnbar + cs), eeps);
    ev[3] = vmax(tabs(vnbar - cs), eeps);
    ev[4] = vmax(tabs(vnbar + ca), eeps);
    ev[5] = vmax(tabs(vnbar - ca), eeps);
    ev[6] = vmax(tabs(vnbar), eeps);
    T dltro = ror - rol;
    T dltmn = robar * (vnr - vnl), dltmt = robar * (vtr - vtl), dltmu = robar * (vur - vul);
    T dltbt = btr - btl, dltbu = bur - bul;
    T t1 = bett * dltbt + betu * dltbu;
    T t2 = (prr - prl + (btave * dltbt + buave * dltbu) + gm2 * (btbar * dltbt + bubar * dltbu))
           * gm1i;
    T t3 = betu * dltbt - bett * dltbu;
    T s1 = dltmn;
    T s2 = bett * dltmt + betu * dltmu;
    T s3 = betu * dltmt - bett * dltmu;
    T p11 = alps * cf * rrobai;
    T p12 = -alpf * c2 * cfi * rrobai;
    T p21 = alpf * (cf2 - c2 * gm2 * gm1i);
    T p22 = alps * (cs2 - c2 * gm2 * gm1i);
    T q11 = alpf * cf, q12 = alps * cs;
    T q21 = -alps * ca * sgn, q22 = alpf * c * sgn;
    T detpi = T(1.0) / (p11 * p22 - p12 * p21);
    T detqi = T(1.0) / (q11 * q22 - q12 * q21);
    T wv[7];
    T pa = (p22 * t1 - p12 * t2) * detpi, qa = (q22 * s1 - q12 * s2) * detqi;
    T pb = (-p21 * t1 + p11 * t2) * detpi, qb = (-q21 * s1 + q11 * s2) * detqi;
    wv[0] = T(0.5) * (pa + qa);
    wv[1] = T(0.5) * (pa - qa);
    wv[2] = T(0.5) * (pb + qb);
    wv[3] = T(0.5) * (pb - qb);
    wv[4] = T(0.5) * (rrobar * t3 - sgn * s3);
    wv[5] = T(0.5) * (rrobar * t3 + sgn * s3);
    wv[6] = dltro - alpf * (wv[0] + wv[1]) - alps * (wv[2] + wv[3]);
    T FL[7], FR[7];
    FL[0] = rol * vnl;
    FL[1] = rol * vnl * vnl + prl + T(0.5) * (-bnbar * bnbar + btl * btl + bul * bul);
    FL[2] = rol * vnl * vtl - bnbar * btl;
    FL[3] = rol * vnl * vul - bnbar * bul;
    FL[4] = vnl * btl - vtl * bnbar;
    FL[5] = vnl * bul - vul * bnbar;
    FL[6] = rol * vnl * hl - bnbar * (bnbar * vnl + btl * vtl + bul * vul);
    FR[0] = ror * vnr;
    FR[1] = ror * vnr * vnr + prr + T(0.5) * (-bnbar * bnbar + btr * btr + bur * bur);
    FR[2] = ror * vnr * vtr - bnbar * btr;
    FR[3] = ror * vnr * vur - bnbar * bur;
    FR[4] = vnr * btr - vtr * bnbar;
    FR[5] = vnr * bur - vur * bnbar;
    FR[6] = ror * vnr * hr - bnbar * (bnbar * vnr + btr * vtr + bur * vur);
    // right eigenvectors (conservative), waves: +f, -f, +s, -s, +a, -a, 0
    T ek[7][7];
    T h0 = kin + db2;
    T vbt = bett * vtbar + betu * vubar;
    ek[0][0] = alpf;
    ek[0][1] = alpf * (vnbar + cf);
    ek[0][2] = alpf * vtbar - alps * bett * ca * sgn;
    ek[0][3] = alpf * vubar - alps * betu * ca * sgn;
    ek[0][4] = alps * bett * cf * rrobai;
    ek[0][5] = alps * betu * cf * rrobai;
    ek[0][6] = alpf * (h0 + cf * vnbar + cf2 * gm1i + (cf2 - c2) * gm2 * gm1i)
               - alps * ca * vbt * sgn;
    ek[1][0] = alpf;
    ek[1][1] = alpf * (vnbar - cf);
    ek[1][2] = alpf * vtbar + alps * bett * ca * sgn;
    ek[1][3] = alpf * vubar + alps * betu * ca * sgn;
    ek[1][4] = ek[0][4];
    ek[1][5] = ek[0][5];
    ek[1][6] = alpf * (h0 - cf * vnbar + cf2 * gm1i + (cf2 - c2) * gm2 * gm1i)
               + alps * ca * vbt * sgn;
    ek[2][0] = alps;
    ek[2][1] = alps * (vnbar + cs);
    ek[2][2] = alps * vtbar + c * sgn * alpf * bett;
    ek[2][3] = alps * vubar + c * sgn * alpf * betu;
    ek[2][4] = -rrobai * c2 * alpf * bett * cfi;
    ek[2][5] = -rrobai * c2 * alpf * betu * cfi;
    ek[2][6] = alps * (h0 + cs * vnbar + cs2 * gm1i + (cs2 - c2) * gm2 * gm1i)
               + alpf * c * vbt * sgn;
    ek[3][0] = alps;
    ek[3][1] = alps * (vnbar - cs);
    ek[3][2] = alps * vtbar - c * sgn * alpf * bett;
    ek[3][3] = alps * vubar - c * sgn * alpf * betu;
    ek[3][4] = ek[2][4];
    ek[3][5] = ek[2][5];
    ek[3][6] = alps * (h0 - cs * vnbar + cs2 * gm1i + (cs2 - c2) * gm2 * gm1i)
               - alpf * c * vbt * sgn;
    ek[4][0] = T(0.0);
    ek[4][1] = T(0.0);
    ek[4][2] = -sgn * betu;
    ek[4][3] = sgn * bett;
    ek[4][4] = rrobai * betu;
    ek[4][5] = -rrobai * bett;
    ek[4][6] = -(betu * vtbar - bett * vubar) * sgn;
    ek[5][0] = T(0.0);
    ek[5][1] = T(0.0);
    ek[5][2] = -ek[4][2];
    ek[5][3] = -ek[4][3];
    ek[5][4] = ek[4][4];
    ek[5][5] = ek[4][5];
    ek[5][6] = -ek[4][6];
    ek[6][0] = T(1.0);
    ek[6][1] = vnbar;
    ek[6][2] = vtbar;
    ek[6][3] = vubar;
    ek[6][4] = T(0.0);
    ek[6][5] = T(0.0);
    ek[6][6] = h0;
#pragma unroll
    for (int k = 0; k < 7; k++) {
        T s = FL[k] + FR[k];
#pragma unroll
        for (int w = 0; w < 7; w++) s = s - ev[w] * wv[w] * ek[w][k];
        f[k] = T(0.5) * s;
    }
}

template <class T>
MLAU_HD void riemann(int which, const T *L, const T *R, T bn, T gamma, T dv0, T dv1, T *f)
{
    switch (which) {
    case FLUX_MLAU: flux_mlau(L, R, bn, gamma, dv0, dv1, f); break;
    case FLUX_LHLLD: flux_hlld<T, true>(L, R, bn, gamma, dv0, dv1, f); break;
    case FLUX_HLLD: flux_hlld<T, false>(L, R, bn, gamma, dv0, dv1, f); break;
    default: flux_roe(L, R, bn, gamma, f); break;
    }
}

// Riemann solver with caller-formed jumps (FP32-split mode); Roe has no
// jump-compensated form and uses the rounded face states.
template <class T>
MLAU_HD void riemann_jumps(int which, const T *L, const T *R, T bn, T gamma, T dv0, T dv1, T *f,
                           T jp, T jv)
{
    switch (which) {
    case FLUX_MLAU: flux_mlau<T, true>(L, R, bn, gamma, dv0, dv1, f, jp, jv); break;
    case FLUX_LHLLD: flux_hlld<T, true, true>(L, R, bn, gamma, dv0, dv1, f, jp, jv); break;
    case FLUX_HLLD: flux_hlld<T, false, true>(L, R, bn, gamma, dv0, dv1, f, jp, jv); break;
    default: flux_roe(L, R, bn, gamma, f); break;
    }
}

// hall_flux_lf (mhd_flux.h:734-766): Lax-Friedrichs fluxes of the Hall
// term's tangential B and energy; v is the Hall velocity, smax the maximum
// speed.  No driver of the ideal step calls it.
template <class T>
MLAU_HD void hall_lf(T vnl, T vtl, T vul, T btl, T bul, T vnr, T vtr, T vur, T btr, T bur, T bnc,
                     T smax, T *fbt, T *fbu, T *fen)
{
    const T pml = T(0.5) * (bnc * bnc + btl * btl + bul * bul);
    const T vbl = vnl * bnc + vtl * btl + vul * bul;
    const T pmr = T(0.5) * (bnc * bnc + btr * btr + bur * bur);
    const T vbr = vnr * bnc + vtr * btr + vur * bur;
    const T fbtl = btl * vnl - bnc * vtl, fbul = bul * vnl - bnc * vul;
    const T fenl = T(2.0) * pml * vnl - bnc * vbl;
    const T fbtr = btr * vnr - bnc * vtr, fbur = bur * vnr - bnc * vur;
    const T fenr = T(2.0) * pmr * vnr - bnc * vbr;
    *fbt = T(0.5) * (fbtl + fbtr - smax * (btr - btl));
    *fbu = T(0.5) * (fbul + fbur - smax * (bur - bul));
    *fen = T(0.5) * (fenl + fenr - smax * (pmr - pml));
}

}  // namespace mlau

#ifdef MLAU_POINT_DIAG_PUSHED
#pragma GCC diagnostic pop
#undef MLAU_POINT_DIAG_PUSHED
#endif
