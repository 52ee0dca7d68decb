/*
 * Point functions of the CPU oracle.  TEST INFRASTRUCTURE ONLY (see
 * mlau_oracle.h).  Each function keeps the reference's evaluation order; the
 * file must be compiled with -ffp-contract=off and without -ffast-math.
 */
#ifndef ORACLE_POINT_H
#define ORACLE_POINT_H

#include <math.h>

/* include/funcs.h:23-43: ties go to a in max and to b in min. */
static inline double o_max(double a, double b) { return (a >= b) ? a : b; }
static inline double o_min(double a, double b) { return (a >= b) ? b : a; }
static inline double o_minmod(double a, double b)
{
    return o_min(o_max(a, b), 0.0) + o_max(o_min(a, b), 0.0);
}

/* include/interp.h:30-37 (2nd-order MUSCL, minmod limiter). */
static inline void o_muscl_mm(double f1, double f2, double f3, double *fl, double *fr)
{
    double df = 0.5 * o_minmod(f2 - f1, f3 - f2);
    *fl = f2 + df;
    *fr = f2 - df;
}

/* minmod3 (include/funcs.h:39-43). */
static inline double o_minmod3(double a, double b, double c)
{
    return o_min(o_max(o_max(a, b), c), 0.0) + o_max(o_min(o_min(a, b), c), 0.0);
}

/* include/interp.h:45-51 (2nd-order MUSCL, MC limiter with alpha 2; the
   limiter of 2D/MPI/MRX/mhd_fd_ct_2d.c:107). */
static inline void o_muscl_mc(double f1, double f2, double f3, double *fl, double *fr)
{
    const double alpha = 2.0;
    double df = 0.5 * o_minmod(alpha * o_minmod(f2 - f1, f3 - f2), 0.5 * (f3 - f1));
    *fl = f2 + df;
    *fr = f2 - df;
}

/* include/interp.h:61-72 (2nd-order MUSCL, Koren limiter). */
static inline void o_muscl_kr(double f1, double f2, double f3, double *fl, double *fr)
{
    double d1 = 2.0 * (f2 - f1);
    double d2 = 2.0 * (f3 - f2);
    double dl = 0.5 * o_minmod3(d1, d2, (0.5 * d1 + d2) / 3.0);
    double dr = 0.5 * o_minmod3(d1, d2, (d1 + 0.5 * d2) / 3.0);
    *fl = f2 + dl;
    *fr = f2 - dr;
}

/* Reconstruction codes: 1-4 are the drivers' ODR; 5 and 6 are 2nd-order
   MUSCL with the MC and Koren limiters in calc_flr's ODR 2 branch (the
   alternatives include/interp.h ships).  Every other order-dependent
   operation (linear interpolation, calc_bc, calc_df) follows ODR 2 for them. */
static inline int o_lin_odr(int odr) { return odr > 4 ? 2 : odr; }

/* include/interp.h:106-146 (3rd-order WCNS, ESWENO3 weights). */
static inline void o_wcns3(double f0, double f1, double f2, double *fl, double *fr)
{
    const double tiny = 1e-40;
    double d0 = f0 - f1, d1 = f2 - f1;
    double s0 = d0 * d0, s1 = d1 * d1;
    double t = f2 - 2.0 * f1 + f0;
    t = t * t;
    s0 = (1.0 + t / (s0 + tiny));
    s1 = (1.0 + t / (s1 + tiny));
    double a = 0.25 * s0, b = 0.75 * s1;
    a /= (a + b);
    b = 1.0 - a;
    *fl = 0.5 * (a * (-f0 + 3.0 * f1) + b * (f1 + f2));
    a = 0.75 * s0;
    b = 0.25 * s1;
    a /= (a + b);
    b = 1.0 - a;
    *fr = 0.5 * (b * (-f2 + 3.0 * f1) + a * (f1 + f0));
}

/* include/interp.h:186-238 (4th-order WCNS, linear weights 0.075/0.65/0.275). */
static inline void o_wcns4(double f0, double f1, double f2, double f3, double f4,
                           double *fl, double *fr)
{
    const double tiny = 1e-40;
    double p, q, s[3];
    p = f0 - 4.0 * f1 + 3.0 * f2;
    q = f0 - 2.0 * f1 + f2;
    s[0] = (13. / 12.) * q * q + 0.25 * p * p;
    p = f1 - f3;
    q = f1 - 2.0 * f2 + f3;
    s[1] = (13. / 12.) * q * q + 0.25 * p * p;
    p = f4 - 4.0 * f3 + 3.0 * f2;
    q = f4 - 2.0 * f3 + f2;
    s[2] = (13. / 12.) * q * q + 0.25 * p * p;
    s[0] = 1.0 / (s[0] * s[0] + tiny);
    s[1] = 1.0 / (s[1] * s[1] + tiny);
    s[2] = 1.0 / (s[2] * s[2] + tiny);

    double w0 = 0.075 * s[0], w1 = 0.650 * s[1], w2 = 0.275 * s[2];
    double r = 1.0 / (w0 + w1 + w2);
    w0 *= r;
    w1 *= r;
    w2 = 1.0 - w0 - w1;
    *fl = 0.125 * (+w0 * (3.0 * f0 - 10.0 * f1 + 15.0 * f2)
                   + w1 * (-f1 + 6.0 * f2 + 3.0 * f3)
                   + w2 * (+3.0 * f2 + 6.0 * f3 - f4));

    w0 = 0.275 * s[0];
    w1 = 0.650 * s[1];
    w2 = 0.075 * s[2];
    r = 1.0 / (w0 + w1 + w2);
    w0 *= r;
    w1 *= r;
    w2 = 1.0 - w0 - w1;
    *fr = 0.125 * (+w2 * (3.0 * f4 - 10.0 * f3 + 15.0 * f2)
                   + w1 * (-f3 + 6.0 * f2 + 3.0 * f1)
                   + w0 * (+3.0 * f2 + 6.0 * f1 - f0));
}

/* calc_flr of the drivers (3D/MPI/OTvortex/mhd_fd_ct_3d.c:65-78). */
static inline void o_rec_lr(int odr, const double *f, double *fl, double *fr)
{
    switch (odr) {
    case 1: *fl = f[2]; *fr = f[2]; break;
    case 2: o_muscl_mm(f[1], f[2], f[3], fl, fr); break;
    case 3: o_wcns3(f[1], f[2], f[3], fl, fr); break;
    case 5: o_muscl_mc(f[1], f[2], f[3], fl, fr); break;
    case 6: o_muscl_kr(f[1], f[2], f[3], fl, fr); break;
    default: o_wcns4(f[0], f[1], f[2], f[3], f[4], fl, fr); break;
    }
}

/* lcal_flr of the drivers (mhd_fd_ct_3d.c:48-63): linear face interpolation. */
static inline void o_lin_lr(int odr, const double *f, double *fl, double *fr)
{
    switch (o_lin_odr(odr)) {
    case 1: *fl = f[2]; *fr = f[2]; break;
    case 2:
        *fl = 0.25 * (-f[1] + 4.0 * f[2] + f[3]);
        *fr = 0.25 * (-f[3] + 4.0 * f[2] + f[1]);
        break;
    case 3:
        *fl = 0.125 * (-f[1] + 6.0 * f[2] + 3.0 * f[3]);
        *fr = 0.125 * (-f[3] + 6.0 * f[2] + 3.0 * f[1]);
        break;
    default:
        *fl = 0.003125 * (9.0 * f[0] - 56.0 * f[1] + 234.0 * f[2] + 144.0 * f[3] - 11.0 * f[4]);
        *fr = 0.003125 * (9.0 * f[4] - 56.0 * f[3] + 234.0 * f[2] + 144.0 * f[1] - 11.0 * f[0]);
        break;
    }
}

/* calc_bc (mhd_fd_ct_3d.c:38-46): face B to cell centre. */
static inline double o_face2cen(int odr, double f0, double f1, double f2, double f3)
{
    if (o_lin_odr(odr) <= 2) return 0.5 * (f1 + f2);
    return 0.0625 * (9.0 * (f1 + f2) - (f0 + f3));
}

/* calc_df (mhd_fd_ct_3d.c:80-88): face-to-centre first difference. */
static inline double o_diff(int odr, double f0, double f1, double f2, double f3)
{
    if (o_lin_odr(odr) <= 2) return f2 - f1;
    return (27.0 * (f2 - f1) - (f3 - f0)) / 24.0;
}

/*
 * Eigen-systems of the primitive MHD equations (include/mhd_eigen.h).
 * L[n][k] is row n of the left eigenvector matrix, R[n][k] is component k of
 * right eigenvector n; variables k = (ro, vn, vt, vu, bt, bu, pr).
 */
/* mhd_eigen_st, include/mhd_eigen.h:24-192 (full 7-wave system, Athena). */
static void o_eigen_full(double ro, double vx, double vy, double vz, double bx, double by,
                         double bz, double pr, double gamma, double lam[7],
                         double L[7][7], double R[7][7])
{
    const double eps = 1e-12;
    double sqrt2 = sqrt(2.0);
    double iro = 1.0 / ro;
    double sro = sqrt(ro);
    double isro = 1.0 / sro;
    double bxsr = bx * isro, bysr = by * isro, bzsr = bz * isro;
    double bx2 = bxsr * bxsr;
    double bt2 = bysr * bysr + bzsr * bzsr;
    double b2 = bx2 + bt2;
    double a2 = fabs(gamma * pr / ro);
    double aa = sqrt(a2);
    double ca2 = bx2;
    double ca = sqrt(ca2);
    double disc = sqrt(fabs((a2 + b2) * (a2 + b2) - 4.0 * a2 * ca2));
    double cf2 = fabs(0.5 * (a2 + b2 + disc));
    double cf = sqrt(cf2);
    double cs2 = fabs(0.5 * (a2 + b2 - disc));
    double cs = sqrt(cs2);

    bx2 = bx * bx;
    bt2 = by * by + bz * bz;
    b2 = bx2 + bt2;
    double den = 1.0 / sqrt(bt2);
    int flag = (bt2 > eps * b2);
    double bey = flag ? (by * den) : (0.5 * sqrt2);
    double bez = flag ? (bz * den) : (0.5 * sqrt2);
    den = 1.0 / sqrt(fabs(cf2 - cs2));
    flag = ((bt2 > eps * b2) || (fabs(gamma * pr - bx2) > eps * gamma * pr));
    double af = flag ? (sqrt(fabs(a2 - cs2)) * den) : 1.0;
    double as = flag ? (sqrt(fabs(cf2 - a2)) * den) : 0.0;
    double sg = (bx > 0) ? (1.0) : (-1.0);
    double cfaf = cf * af, csas = cs * as, aaaf = aa * af, aaas = aa * as;
    den = 0.5 / a2;

    lam[0] = vx - cf; lam[1] = vx - ca; lam[2] = vx - cs; lam[3] = vx;
    lam[4] = vx + cs; lam[5] = vx + ca; lam[6] = vx + cf;

    /* fast, slow and Alfven rows; the +speed rows mirror the -speed rows */
    double *l;
    l = L[0];
    l[0] = 0; l[1] = -cfaf * den; l[2] = +csas * den * sg * bey; l[3] = +csas * den * sg * bez;
    l[4] = +aaas * den * isro * bey; l[5] = +aaas * den * isro * bez; l[6] = af * den * iro;
    l = L[1];
    l[0] = 0; l[1] = 0; l[2] = -0.5 * bez; l[3] = +0.5 * bey;
    l[4] = -0.5 * isro * bez * sg; l[5] = +0.5 * isro * bey * sg; l[6] = 0;
    l = L[2];
    l[0] = 0; l[1] = -csas * den; l[2] = -cfaf * den * sg * bey; l[3] = -cfaf * den * sg * bez;
    l[4] = -aaaf * den * isro * bey; l[5] = -aaaf * den * isro * bez; l[6] = as * den * iro;
    l = L[3];
    l[0] = 1.0; l[1] = 0; l[2] = 0; l[3] = 0; l[4] = 0; l[5] = 0; l[6] = -1.0 / a2;
    for (int m = 0; m < 3; m++) {
        double *s = L[m], *t = L[6 - m];
        t[0] = +s[0]; t[1] = -s[1]; t[2] = -s[2]; t[3] = -s[3];
        t[4] = +s[4]; t[5] = +s[5]; t[6] = +s[6];
    }
    double *r;
    r = R[0];
    r[0] = ro * af; r[1] = -cfaf; r[2] = +csas * sg * bey; r[3] = +csas * sg * bez;
    r[4] = +aaas * sro * bey; r[5] = +aaas * sro * bez; r[6] = af * gamma * pr;
    r = R[1];
    r[0] = 0; r[1] = 0; r[2] = -bez; r[3] = +bey;
    r[4] = -sro * bez * sg; r[5] = +sro * bey * sg; r[6] = 0;
    r = R[2];
    r[0] = ro * as; r[1] = -csas; r[2] = -cfaf * sg * bey; r[3] = -cfaf * sg * bez;
    r[4] = -aaaf * sro * bey; r[5] = -aaaf * sro * bez; r[6] = as * gamma * pr;
    r = R[3];
    r[0] = 1.0; r[1] = 0; r[2] = 0; r[3] = 0; r[4] = 0; r[5] = 0; r[6] = 0;
    for (int m = 0; m < 3; m++) {
        double *s = R[m], *t = R[6 - m];
        t[0] = +s[0]; t[1] = -s[1]; t[2] = -s[2]; t[3] = -s[3];
        t[4] = +s[4]; t[5] = +s[5]; t[6] = +s[6];
    }
}

/* mhd_eigen_mi, include/mhd_eigen.h:194-324 (Miyoshi's fast + Alfven
 * projection; the slow mode is ignored). */
static void o_eigen_miyoshi(double ro, double bx, double by, double bz, double pr,
                            double gamma, double L[7][7], double R[7][7])
{
    double iro = 1.0 / ro;
    double cs2 = gamma * pr * iro;
    double ca2 = bx * bx * iro;
    double ct2 = (by * by + bz * bz) * iro;
    double cb2 = cs2 + ca2 + ct2;
    double cf2 = 0.5 * (cb2 + sqrt(fabs(cb2 * cb2 - 4.0 * cs2 * ca2)));
    double cf = sqrt(cf2);
    double rcf = ro * cf, sro = sqrt(ro), isroh = 0.5 / sro;
    double icf2 = 1.0 / cf2, icf2h = 0.5 * icf2, ircfh = 0.5 / rcf;
    double byh = 0.5 * by, bzh = 0.5 * bz;
    const double Lt[7][7] = {
        {0, -rcf, 0, 0, +by, +bz, +1.0},
        {cf2, 0, 0, 0, -by, -bz, -1.0},
        {0, +rcf, 0, 0, +by, +bz, +1.0},
        {0, 0, +sro, 0, +1.0, 0, 0},
        {0, 0, +sro, 0, -1.0, 0, 0},
        {0, 0, 0, +sro, 0, +1.0, 0},
        {0, 0, 0, +sro, 0, -1.0, 0}};
    const double Rt[7][7] = {
        {+icf2h, -ircfh, 0, 0, 0, 0, +0.5},
        {+icf2, 0, 0, 0, 0, 0, 0},
        {+icf2h, +ircfh, 0, 0, 0, 0, +0.5},
        {0, 0, +isroh, 0, +0.5, 0, -byh},
        {0, 0, +isroh, 0, -0.5, 0, +byh},
        {0, 0, 0, +isroh, 0, +0.5, -bzh},
        {0, 0, 0, +isroh, 0, -0.5, +bzh}};
    for (int n = 0; n < 7; n++)
        for (int k = 0; k < 7; k++) { L[n][k] = Lt[n][k]; R[n][k] = Rt[n][k]; }
}

/* mhd_eigen_ae, include/mhd_eigen.h:326-453 (Alfven + entropy projection). */
static void o_eigen_alfven(double ro, double bx, double by, double bz, double pr,
                           double gamma, double L[7][7], double R[7][7])
{
    double iro = 1.0 / ro;
    double cs2 = gamma * pr * iro;
    double ca2 = bx * bx * iro;
    double ct2 = (by * by + bz * bz) * iro;
    double cb2 = cs2 + ca2 + ct2;
    double cf2 = 0.5 * (cb2 + sqrt(fabs(cb2 * cb2 - 4.0 * cs2 * ca2)));
    double sro = sqrt(ro);
    double isroh = 0.5 / sro;
    double icf2 = 1.0 / cf2;
    double byh = 0.5 * by, bzh = 0.5 * bz;
    const double Lt[7][7] = {
        {0, +1.0, 0, 0, 0, 0, 0},
        {cf2, 0, 0, 0, -by, -bz, -1.0},
        {0, 0, 0, 0, +by, +bz, +1.0},
        {0, 0, +sro, 0, +1.0, 0, 0},
        {0, 0, +sro, 0, -1.0, 0, 0},
        {0, 0, 0, +sro, 0, +1.0, 0},
        {0, 0, 0, +sro, 0, -1.0, 0}};
    const double Rt[7][7] = {
        {0, +1.0, 0, 0, 0, 0, 0},
        {+icf2, 0, 0, 0, 0, 0, 0},
        {+icf2, 0, 0, 0, 0, 0, +1.0},
        {0, 0, +isroh, 0, +0.5, 0, -byh},
        {0, 0, +isroh, 0, -0.5, 0, +byh},
        {0, 0, 0, +isroh, 0, +0.5, -bzh},
        {0, 0, 0, +isroh, 0, -0.5, +bzh}};
    for (int n = 0; n < 7; n++)
        for (int k = 0; k < 7; k++) { L[n][k] = Lt[n][k]; R[n][k] = Rt[n][k]; }
}

/* mhd_c_reconst / mhd_a_reconst / mhd_m_reconst (include/mhd_eigen.h:455-530,
 * 609-684, 532-607): project the 5-point stencil on characteristic fields,
 * reconstruct each field, project back, and keep identically-zero v and B at
 * zero.  full: 0 Alfven + entropy, 1 full 7-wave, 2 Miyoshi.
 * q[k][m]: variable k at stencil point m; ul at i+1/2, ur at i-1/2. */
static void o_reconst(int full, int odr, const double q[7][5], double bn, double gamma,
                      double ul[7], double ur[7])
{
    double L[7][7], R[7][7], lam[7];
    if (full == 2)
        o_eigen_miyoshi(q[0][2], bn, q[4][2], q[5][2], q[6][2], gamma, L, R);
    else if (full)
        o_eigen_full(q[0][2], q[1][2], q[2][2], q[3][2], bn, q[4][2], q[5][2], q[6][2],
                     gamma, lam, L, R);
    else
        o_eigen_alfven(q[0][2], bn, q[4][2], q[5][2], q[6][2], gamma, L, R);

    double w[7][5], wl[7], wr[7];
    for (int m = 0; m < 5; m++)
        for (int n = 0; n < 7; n++)
            w[n][m] = (+L[n][0] * q[0][m] + L[n][1] * q[1][m] + L[n][2] * q[2][m]
                       + L[n][3] * q[3][m] + L[n][4] * q[4][m] + L[n][5] * q[5][m]
                       + L[n][6] * q[6][m]);
    for (int n = 0; n < 7; n++) o_rec_lr(odr, w[n], &wl[n], &wr[n]);
    for (int k = 0; k < 7; k++)
        ul[k] = R[0][k] * wl[0] + R[1][k] * wl[1] + R[2][k] * wl[2] + R[3][k] * wl[3]
                + R[4][k] * wl[4] + R[5][k] * wl[5] + R[6][k] * wl[6];
    for (int k = 0; k < 7; k++)
        ur[k] = R[0][k] * wr[0] + R[1][k] * wr[1] + R[2][k] * wr[2] + R[3][k] * wr[3]
                + R[4][k] * wr[4] + R[5][k] * wr[5] + R[6][k] * wr[6];

    /* variables 1..5 (vn, vt, vu, bt, bu) that vanish on the whole stencil */
    for (int k = 1; k <= 5; k++) {
        int zero = 1;
        for (int m = 0; m < 5; m++)
            if (q[k][m] != 0.0) zero = 0;
        if (zero) ul[k] = ur[k] = 0.0;
    }
}

/*
 * Riemann solvers (include/mhd_flux.h).  Arguments: left/right primitives
 * (ro, vn, vt, vu, bt, bu, pr), the face-normal B, gamma, the shock sensor
 * dv[2] (MLAU and LHLLD only); outputs the 7 fluxes (ro, mn, mt, mu, bt, bu, en).
 */
#define O_EPS (1e-8)

/* calc_flux_mlau, include/mhd_flux.h:26-213. */
static void o_flux_mlau(double rol, double vnl, double vtl, double vul, double btl, double bul,
                        double prl, double ror, double vnr, double vtr, double vur, double btr,
                        double bur, double prr, double bnc, double gamma, const double *dv,
                        double *f)
{
    double gm1i = 1.0 / (gamma - 1.0);
    double bnc2 = bnc * bnc;
    double sgn = (bnc > 0) ? (1.0) : (-1.0);
    double bnca = sgn * bnc;

    double roli = 1.0 / rol;
    double vl2 = vnl * vnl + vtl * vtl + vul * vul;
    double pml = 0.5 * (btl * btl + bul * bul);
    double ptl = prl + pml;
    double enl = gm1i * prl + pml + 0.5 * rol * vl2;
    double hnl = (enl + ptl) * roli;

    double rori = 1.0 / ror;
    double vr2 = vnr * vnr + vtr * vtr + vur * vur;
    double pmr = 0.5 * (btr * btr + bur * bur);
    double ptr = prr + pmr;
    double enr = gm1i * prr + pmr + 0.5 * ror * vr2;
    double hnr = (enr + ptr) * rori;

    double cl2 = gamma * prl * roli, cr2 = gamma * prr * rori;
    double cal2 = bnc2 * roli, car2 = bnc2 * rori;
    double cbl2 = cl2 + cal2 + 2.0 * pml * roli;
    double cbr2 = cr2 + car2 + 2.0 * pmr * rori;
    double cfl2 = 0.5 * (cbl2 + sqrt(fabs(cbl2 * cbl2 - 4.0 * cl2 * cal2)));
    double cfr2 = 0.5 * (cbr2 + sqrt(fabs(cbr2 * cbr2 - 4.0 * cr2 * car2)));
    cbl2 = vl2 + cal2 + 2.0 * pml * roli;
    cbr2 = vr2 + car2 + 2.0 * pmr * rori;
    double ccl2 = 0.5 * (cbl2 + sqrt(fabs(cbl2 * cbl2 - 4.0 * vl2 * cal2)));
    double ccr2 = 0.5 * (cbr2 + sqrt(fabs(cbr2 * cbr2 - 4.0 * vr2 * car2)));
    double cmax = sqrt(o_max(cfl2, cfr2));
    double cfn = cmax;
    double cfni = 1.0 / cfn;
    double sl = o_min(0.0, o_min(vnl, vnr) - cmax);
    double sr = o_max(0.0, o_max(vnl, vnr) + cmax);

    double mal = vnl * cfni, mar = vnr * cfni;
    double snl = (mal > 0) ? 1.0 : (-1.0);
    double snr = (mar > 0) ? 1.0 : (-1.0);
    double theta = o_min(1.0, (cfn - o_min(dv[0], 0.0)) / (cfn - o_min(dv[1], 0.0)));
    theta *= theta;
    theta *= theta;
    const double alpha = 0.1875, beta = 0.125;
    double malp1 = mal + 1.0, marm1 = mar - 1.0;
    double mal2m1 = mal * mal - 1.0, mar2m1 = mar * mar - 1.0;
    double bfl, ffl, bfr, ffr;
    if (snl * mal > 1.0) {
        bfl = 0.5 * (1.0 + snl);
        ffl = bfl * mal;
    } else {
        bfl = +0.25 * malp1 * malp1 * (2.0 - mal) + alpha * mal * mal2m1 * mal2m1;
        ffl = +0.25 * malp1 * malp1 + beta * mal2m1 * mal2m1;
    }
    if (snr * mar > 1.0) {
        bfr = 0.5 * (1.0 - snr);
        ffr = bfr * mar;
    } else {
        bfr = +0.25 * marm1 * marm1 * (2.0 + mar) - alpha * mar * mar2m1 * mar2m1;
        ffr = -0.25 * marm1 * marm1 - beta * mar2m1 * mar2m1;
    }

    double mnc = ffl + ffr;
    double mflux = mnc * cfn;
    mflux -= o_max(1.0 - fabs(mnc), 0.0) * theta * cfni * (ptr - ptl) / (rol + ror);
    double dir = (mflux > 0) ? 1.0 : (-1.0);
    double dirl = 0.5 * (1.0 + dir);
    double dirr = 1.0 - dirl;
    mflux *= (dirl * rol + dirr * ror);
    double mfl = mflux * dirl;
    double mfr = mflux - mfl;
    double ptot = bfl * ptl + bfr * ptr;
    double cfmod = sqrt(o_max(ccl2, ccr2));
    ptot -= 0.25 * bfl * bfr * (rol + ror) * cfmod * (vnr - vnl);
    ptot -= 0.5 * (1.0 - cfmod * cfni) * (bfl + bfr - 1.0) * (ptl + ptr);

    double slvl = sl - vnl, srvr = sr - vnr;
    double snc = dirl * sl + dirr * sr;
    double vndnm = mflux + dirl * rol * slvl + dirr * ror * srvr;
    double vnc = ((fabs(vndnm) > O_EPS) && (snc != 0)) ? (mflux * snc / vndnm)
                                                        : (dirl * vnl + dirr * vnr);

    double slvc = sl - vnc, srvc = sr - vnc;
    double slvci = 1.0 / slvc, srvci = 1.0 / srvc;
    double rhdl = rol * slvl * slvc - bnc2;
    double rhdr = ror * srvr * srvc - bnc2;
    double dvtl = 0.0, dvul = 0.0, dbtl = 0.0, dbul = 0.0;
    double dvtr = 0.0, dvur = 0.0, dbtr = 0.0, dbur = 0.0;
    if (fabs(rhdl) > O_EPS) {
        double g = (vnc - vnl) / rhdl;
        dvtl = -bnc * btl * g;
        dvul = -bnc * bul * g;
        dbtl = bnc2 * btl * g * slvci;
        dbul = bnc2 * bul * g * slvci;
    }
    if (fabs(rhdr) > O_EPS) {
        double g = (vnc - vnr) / rhdr;
        dvtr = -bnc * btr * g;
        dvur = -bnc * bur * g;
        dbtr = bnc2 * btr * g * srvci;
        dbur = bnc2 * bur * g * srvci;
    }
    double cmpl = slvl * slvci, cmpr = srvr * srvci;
    double ro2l = rol * cmpl;
    double srol = sqrt(ro2l);
    double vt2l = dvtl + vtl, vu2l = dvul + vul;
    double bt2l = dbtl + btl * cmpl, bu2l = dbul + bul * cmpl;
    double ro2r = ror * cmpr;
    double sror = sqrt(ro2r);
    double vt2r = dvtr + vtr, vu2r = dvur + vur;
    double bt2r = dbtr + btr * cmpr, bu2r = dbur + bur * cmpr;

    double sroi = 1.0 / (srol + sror);
    double srollri = srol * sroi, srorlri = sror * sroi;
    double bnflb = sgn * o_min(o_max(0.0, srollri * (bnca + sror * vnc)), bnca);
    double bnfrb = sgn * o_min(o_max(0.0, srorlri * (bnca - srol * vnc)), bnca);
    double bnflv = sgn * o_min(o_max(0.0, srorlri * (bnca + mflux / sror)), bnca);
    double bnfrv = sgn * o_min(o_max(0.0, srollri * (bnca - mflux / srol)), bnca);
    double bnsrv = o_max(bnca - dir * vnc * (dirl * srol + dirr * sror), 0.0);
    double ccb = sroi * bnsrv;
    double ccv = srol * sror * ccb;
    double bnvt = bnflb * vt2l + bnfrb * vt2r + ccb * (bt2r - bt2l);
    double bnvu = bnflb * vu2l + bnfrb * vu2r + ccb * (bu2r - bu2l);
    double bnbt = bnflv * bt2l + bnfrv * bt2r + ccv * (vt2r - vt2l);
    double bnbu = bnflv * bu2l + bnfrv * bu2r + ccv * (vu2r - vu2l);
    bnvt -= vnc * (dirl * dbtl + dirr * dbtr);
    bnvu -= vnc * (dirl * dbul + dirr * dbur);
    bnbt -= mflux * (dirl * dvtl + dirr * dvtr);
    bnbu -= mflux * (dirl * dvul + dirr * dvur);

    f[0] = mflux;
    f[1] = mfl * vnl + mfr * vnr + ptot - 0.5 * bnc2;
    f[2] = mfl * vtl + mfr * vtr - bnbt;
    f[3] = mfl * vul + mfr * vur - bnbu;
    f[4] = mfl * btl * roli + mfr * btr * rori - bnvt;
    f[5] = mfl * bul * roli + mfr * bur * rori - bnvu;

    double vb1 = dirl * (vtl * btl + vul * bul) + dirr * (vtr * btr + vur * bur);
    double vb2 = dirl * (vt2l * bt2l + vu2l * bu2l) + dirr * (vt2r * bt2r + vu2r * bu2r);
    double rv2b2 = (mflux * vnc - bnc2);
    rv2b2 *= rv2b2;
    double vb3 = 0.0;
    if (rv2b2 > O_EPS * O_EPS) {
        vb3 = (+(f[2] * vnc + f[4] * bnc) * (f[2] * bnc + f[4] * mflux)
               + (f[3] * vnc + f[5] * bnc) * (f[3] * bnc + f[5] * mflux)) / rv2b2;
    }
    double bnvb = sgn * (bnca * (snc * vb2 - vnc * vb1) * (dirl * slvci + dirr * srvci)
                         + bnsrv * (vb3 - vb2));
    f[6] = mfl * hnl + mfr * hnr - bnvb;
}

/* calc_flux_hlld (include/mhd_flux.h:456-582) and calc_flux_lhlld
 * (:584-719); lowdiss selects the low-dissipation all-speed variant. */
static void o_flux_hlld(int lowdiss, double rol, double vnl, double vtl, double vul,
                        double btl, double bul, double prl, double ror, double vnr,
                        double vtr, double vur, double btr, double bur, double prr,
                        double bnc, double gamma, const double *dv, double *f)
{
    double gm1i = 1.0 / (gamma - 1.0);
    double bnc2 = bnc * bnc;
    double sgn = (bnc > 0) ? (1.0) : (-1.0);
    double roli = 1.0 / rol;
    double pml = 0.5 * (btl * btl + bul * bul);
    double ptl = prl + pml;
    double vl2 = vnl * vnl + vtl * vtl + vul * vul;
    double enl = gm1i * prl + pml + 0.5 * rol * vl2;
    double vbl = vtl * btl + vul * bul;
    double rori = 1.0 / ror;
    double pmr = 0.5 * (btr * btr + bur * bur);
    double ptr = prr + pmr;
    double vr2 = vnr * vnr + vtr * vtr + vur * vur;
    double enr = gm1i * prr + pmr + 0.5 * ror * vr2;
    double vbr = vtr * btr + vur * bur;
    double cl2 = gamma * prl * roli, cr2 = gamma * prr * rori;
    double cal2 = bnc2 * roli, car2 = bnc2 * rori;
    double cbl2 = cl2 + cal2 + 2.0 * pml * roli;
    double cbr2 = cr2 + car2 + 2.0 * pmr * rori;
    double cfl2 = 0.5 * (cbl2 + sqrt(fabs(cbl2 * cbl2 - 4.0 * cl2 * cal2)));
    double cfr2 = 0.5 * (cbr2 + sqrt(fabs(cbr2 * cbr2 - 4.0 * cr2 * car2)));
    double cmax, vnc, ptc, slvl, srvr, rslvl, rsrvr, drsvi, sl, sr;
    if (!lowdiss) {
        double cfl = sqrt(cfl2), cfr = sqrt(cfr2);
        cmax = o_max(cfl, cfr);
        sl = o_min(0.0, o_min(vnl, vnr) - cmax);
        sr = o_max(0.0, o_max(vnl, vnr) + cmax);
        slvl = sl - vnl;
        srvr = sr - vnr;
        rslvl = rol * slvl;
        rsrvr = ror * srvr;
        drsvi = 1.0 / (rsrvr - rslvl);
        vnc = (rsrvr * vnr - rslvl * vnl - ptr + ptl) * drsvi;
        ptc = (rsrvr * ptl - rslvl * ptr + rsrvr * rslvl * (vnr - vnl)) * drsvi;
    } else {
        cbl2 = vl2 + cal2 + 2.0 * pml * roli;
        cbr2 = vr2 + car2 + 2.0 * pmr * rori;
        double ccl2 = 0.5 * (cbl2 + sqrt(fabs(cbl2 * cbl2 - 4.0 * vl2 * cal2)));
        double ccr2 = 0.5 * (cbr2 + sqrt(fabs(cbr2 * cbr2 - 4.0 * vr2 * car2)));
        cmax = sqrt(o_max(cfl2, cfr2));
        sl = o_min(0.0, o_min(vnl, vnr) - cmax);
        sr = o_max(0.0, o_max(vnl, vnr) + cmax);
        slvl = sl - vnl;
        srvr = sr - vnr;
        rslvl = rol * slvl;
        rsrvr = ror * srvr;
        drsvi = 1.0 / (rsrvr - rslvl);
        double theta = o_min(1.0, (cmax - o_min(dv[0], 0.0)) / (cmax - o_min(dv[1], 0.0)));
        theta *= theta;
        theta *= theta;
        vnc = (rsrvr * vnr - rslvl * vnl - theta * (ptr - ptl)) * drsvi;
        double mcc = o_min(1.0, sqrt(o_max(ccl2, ccr2)) / cmax);
        ptc = (rsrvr * ptl - rslvl * ptr + (mcc * (2.0 - mcc)) * rsrvr * rslvl * (vnr - vnl))
              * drsvi;
    }
    double slvc = sl - vnc, srvc = sr - vnc;
    double ro2l = rslvl / slvc, ro2r = rsrvr / srvc;
    double rhdl = rslvl * slvc - bnc2, rhdr = rsrvr * srvc - bnc2;
    double vt2l, vu2l, bt2l, bu2l, vt2r, vu2r, bt2r, bu2r;
    if (fabs(rhdl) > O_EPS) {
        double rhdli = 1.0 / rhdl;
        double rhnvl = (vnl - vnc) * bnc;
        double rhnbl = rslvl * slvl - bnc2;
        vt2l = vtl + rhnvl * rhdli * btl;
        vu2l = vul + rhnvl * rhdli * bul;
        bt2l = rhnbl * rhdli * btl;
        bu2l = rhnbl * rhdli * bul;
    } else {
        vt2l = vtl; vu2l = vul; bt2l = btl; bu2l = bul;
    }
    if (fabs(rhdr) > O_EPS) {
        double rhdri = 1.0 / rhdr;
        double rhnvr = (vnr - vnc) * bnc;
        double rhnbr = rsrvr * srvr - bnc2;
        vt2r = vtr + rhnvr * rhdri * btr;
        vu2r = vur + rhnvr * rhdri * bur;
        bt2r = rhnbr * rhdri * btr;
        bu2r = rhnbr * rhdri * bur;
    } else {
        vt2r = vtr; vu2r = vur; bt2r = btr; bu2r = bur;
    }
    double vb2l = vt2l * bt2l + vu2l * bu2l;
    double vb2r = vt2r * bt2r + vu2r * bu2r;
    double en2l = (slvl * enl - ptl * vnl + ptc * vnc + bnc * (vbl - vb2l)) / slvc;
    double en2r = (srvr * enr - ptr * vnr + ptc * vnc + bnc * (vbr - vb2r)) / srvc;
    double rro2l = sqrt(ro2l), rro2r = sqrt(ro2r);
    double rro2i = 1.0 / (rro2r + rro2l);
    double vt3m = (rro2r * vt2r + rro2l * vt2l + (bt2r - bt2l) * sgn) * rro2i;
    double vu3m = (rro2r * vu2r + rro2l * vu2l + (bu2r - bu2l) * sgn) * rro2i;
    double bt3m = (rro2l * bt2r + rro2r * bt2l + rro2r * rro2l * (vt2r - vt2l) * sgn) * rro2i;
    double bu3m = (rro2l * bu2r + rro2r * bu2l + rro2r * rro2l * (vu2r - vu2l) * sgn) * rro2i;
    double vb3m = vt3m * bt3m + vu3m * bu3m;
    double en3l = en2l - rro2l * (vb2l - vb3m) * sgn;
    double en3r = en2r + rro2r * (vb2r - vb3m) * sgn;
    double hl = (vnc > 0) ? (1.0) : (0.0);
    double hr = 1.0 - hl;
    double h2l = (vnc - fabs(bnc) / rro2l > 0) ? (1.0) : (0.0);
    double h3l = (1.0 - h2l) * hl;
    double h2r = (vnc + fabs(bnc) / rro2r > 0) ? (0.0) : (1.0);
    double h3r = (1.0 - h2r) * hr;
    double rou = ro2l * hl + ro2r * hr;
    double vtu = vt2l * h2l + vt3m * (h3l + h3r) + vt2r * h2r;
    double vuu = vu2l * h2l + vu3m * (h3l + h3r) + vu2r * h2r;
    double btu = bt2l * h2l + bt3m * (h3l + h3r) + bt2r * h2r;
    double buu = bu2l * h2l + bu3m * (h3l + h3r) + bu2r * h2r;
    double enu = en2l * h2l + en3l * h3l + en3r * h3r + en2r * h2r;
    f[0] = rou * vnc;
    f[1] = rou * vnc * vnc + ptc - bnc2 * 0.5;
    f[2] = rou * vtu * vnc - bnc * btu;
    f[3] = rou * vuu * vnc - bnc * buu;
    f[4] = btu * vnc - bnc * vtu;
    f[5] = buu * vnc - bnc * vuu;
    f[6] = (enu + ptc) * vnc - bnc * (vtu * btu + vuu * buu);
}

/* calc_flux_roe, include/mhd_flux.h:215-454 (dv unused). */
static void o_flux_roe(double rol, double vnl, double vtl, double vul, double btl, double bul,
                       double prl, double ror, double vnr, double vtr, double vur, double btr,
                       double bur, double prr, double bnc, double gamma, double *f)
{
    double gm1 = gamma - 1.0, gm2 = gamma - 2.0, gm1i = 1.0 / gm1;
    double roli = 1.0 / rol, rori = 1.0 / ror;
    double rrol = sqrt(rol), rror = sqrt(ror);
    double rroi = 1.0 / (rrol + rror);
    double robar = rrol * rror;
    double robari = 1.0 / robar;
    double rrobar = sqrt(robar);
    double rrobai = sqrt(robari);
    double vnbar = (rrol * vnl + rror * vnr) * rroi;
    double vtbar = (rrol * vtl + rror * vtr) * rroi;
    double vubar = (rrol * vul + rror * vur) * rroi;
    double bnbar = bnc;
    double btbar = (rrol * btr + rror * btl) * rroi;
    double bubar = (rrol * bur + rror * bul) * rroi;
    double hl = (+gamma * gm1i * prl * roli + 0.5 * (vnl * vnl + vtl * vtl + vul * vul)
                 + (bnbar * bnbar + btl * btl + bul * bul) * roli);
    double hr = (+gamma * gm1i * prr * rori + 0.5 * (vnr * vnr + vtr * vtr + vur * vur)
                 + (bnbar * bnbar + btr * btr + bur * bur) * rori);
    double hbar = (rrol * hl + rror * hr) * rroi;
    double btave = 0.5 * (btl + btr), buave = 0.5 * (bul + bur);
    double sgn = (bnbar > 0) ? (1.0) : (-1.0);
    double db2 = 0.5 * gm2 * gm1i * ((btr - btl) * (btr - btl) + (bur - bul) * (bur - bul))
                 * rroi * rroi;
    double vbar2 = vnbar * vnbar + vtbar * vtbar + vubar * vubar;
    double c2 = gm1 * (+hbar - 0.5 * (vnbar * vnbar + vtbar * vtbar + vubar * vubar) - db2
                       - (bnbar * bnbar + btbar * btbar + bubar * bubar) * robari);
    double a2 = (gm1 * (+hbar - 0.5 * (vnbar * vnbar + vtbar * vtbar + vubar * vubar) - db2)
                 - gm2 * (bnbar * bnbar + btbar * btbar + bubar * bubar) * robari);
    (void)vbar2;
    double ca2 = bnbar * bnbar * robari;
    double cb2 = (btbar * btbar + bubar * bubar) * robari;
    double cf2 = 0.5 * (a2 + sqrt(cb2 * (a2 + c2 + ca2) + (c2 - ca2) * (c2 - ca2)));
    double cs2 = c2 * ca2 / cf2;
    double cf = sqrt(cf2), cs = sqrt(cs2), ca = sqrt(ca2), c = sqrt(c2);
    double cfi = 1.0 / cf;
    double sgr1 = btbar * btbar + bubar * bubar - O_EPS;
    double sf11 = (sgr1 > 0) ? 1.0 : 0.0;
    double sf21 = 1.0 - sf11;
    double beti = 1.0 / sqrt(btbar * btbar + bubar * bubar + sf21);
    double bett = sf11 * btbar * beti + sf21 * sqrt(0.5);
    double betu = sf11 * bubar * beti + sf21 * sqrt(0.5);
    double sgr2 = (btbar * btbar + bubar * bubar) * robari + fabs(ca2 - c2) - O_EPS;
    double sf12 = (sgr2 > 0) ? 1.0 : 0.0;
    double sf22 = 1.0 - sf12;
    double cfca = o_max(0.0, cf2 - ca2);
    double cfcs = o_max(0.0, cf2 - cs2);
    double cfa = o_max(0.0, cf2 - c2);
    double alpi = 1.0 / sqrt(cfcs + sf22);
    double alpf = sf12 * sqrt(cfca) * alpi + sf22;
    double alps = sf12 * sqrt(cfa) * alpi;
    const double eeps = 0.0;
    double evpf = o_max(fabs(vnbar + cf), eeps), evmf = o_max(fabs(vnbar - cf), eeps);
    double evps = o_max(fabs(vnbar + cs), eeps), evms = o_max(fabs(vnbar - cs), eeps);
    double evpa = o_max(fabs(vnbar + ca), eeps), evma = o_max(fabs(vnbar - ca), eeps);
    double ev00 = o_max(fabs(vnbar), eeps);
    double dltro = ror - rol;
    double dltmn = robar * (vnr - vnl), dltmt = robar * (vtr - vtl), dltmu = robar * (vur - vul);
    double dltbt = btr - btl, dltbu = bur - bul;
    double t1 = bett * dltbt + betu * dltbu;
    double t2 = (prr - prl + (btave * dltbt + buave * dltbu) + gm2 * (btbar * dltbt + bubar * dltbu))
                * gm1i;
    double t3 = betu * dltbt - bett * dltbu;
    double s1 = dltmn;
    double s2 = bett * dltmt + betu * dltmu;
    double s3 = betu * dltmt - bett * dltmu;
    double p11 = alps * cf * rrobai;
    double p12 = -alpf * c2 * cfi * rrobai;
    double p21 = alpf * (cf2 - c2 * gm2 * gm1i);
    double p22 = alps * (cs2 - c2 * gm2 * gm1i);
    double q11 = alpf * cf, q12 = alps * cs;
    double q21 = -alps * ca * sgn, q22 = alpf * c * sgn;
    double detpi = 1.0 / (p11 * p22 - p12 * p21);
    double detqi = 1.0 / (q11 * q22 - q12 * q21);
    double wvpf = 0.5 * ((p22 * t1 - p12 * t2) * detpi + (q22 * s1 - q12 * s2) * detqi);
    double wvmf = 0.5 * ((p22 * t1 - p12 * t2) * detpi - (q22 * s1 - q12 * s2) * detqi);
    double wvps = 0.5 * ((-p21 * t1 + p11 * t2) * detpi + (-q21 * s1 + q11 * s2) * detqi);
    double wvms = 0.5 * ((-p21 * t1 + p11 * t2) * detpi - (-q21 * s1 + q11 * s2) * detqi);
    double wvpa = 0.5 * (rrobar * t3 - sgn * s3);
    double wvma = 0.5 * (rrobar * t3 + sgn * s3);
    double wv00 = dltro - alpf * (wvpf + wvmf) - alps * (wvps + wvms);
    /* one-sided fluxes */
    double FL[7], FR[7];
    FL[0] = rol * vnl;
    FL[1] = rol * vnl * vnl + prl + 0.5 * (-bnbar * bnbar + btl * btl + bul * bul);
    FL[2] = rol * vnl * vtl - bnbar * btl;
    FL[3] = rol * vnl * vul - bnbar * bul;
    FL[4] = vnl * btl - vtl * bnbar;
    FL[5] = vnl * bul - vul * bnbar;
    FL[6] = rol * vnl * hl - bnbar * (bnbar * vnl + btl * vtl + bul * vul);
    FR[0] = ror * vnr;
    FR[1] = ror * vnr * vnr + prr + 0.5 * (-bnbar * bnbar + btr * btr + bur * bur);
    FR[2] = ror * vnr * vtr - bnbar * btr;
    FR[3] = ror * vnr * vur - bnbar * bur;
    FR[4] = vnr * btr - vtr * bnbar;
    FR[5] = vnr * bur - vur * bnbar;
    FR[6] = ror * vnr * hr - bnbar * (bnbar * vnr + btr * vtr + bur * vur);
    /* right eigenvectors in conservative variables (7 waves x 7 components) */
    double kin = 0.5 * (vnbar * vnbar + vtbar * vtbar + vubar * vubar);
    double ev[7][7];
    ev[0][0] = alpf;
    ev[0][1] = alpf * (vnbar + cf);
    ev[0][2] = alpf * vtbar - alps * bett * ca * sgn;
    ev[0][3] = alpf * vubar - alps * betu * ca * sgn;
    ev[0][4] = alps * bett * cf * rrobai;
    ev[0][5] = alps * betu * cf * rrobai;
    ev[0][6] = alpf * (kin + db2 + cf * vnbar + cf2 * gm1i + (cf2 - c2) * gm2 * gm1i)
               - alps * ca * (bett * vtbar + betu * vubar) * sgn;
    ev[1][0] = alpf;
    ev[1][1] = alpf * (vnbar - cf);
    ev[1][2] = alpf * vtbar + alps * bett * ca * sgn;
    ev[1][3] = alpf * vubar + alps * betu * ca * sgn;
    ev[1][4] = ev[0][4];
    ev[1][5] = ev[0][5];
    ev[1][6] = alpf * (kin + db2 - cf * vnbar + cf2 * gm1i + (cf2 - c2) * gm2 * gm1i)
               + alps * ca * (bett * vtbar + betu * vubar) * sgn;
    ev[2][0] = alps;
    ev[2][1] = alps * (vnbar + cs);
    ev[2][2] = alps * vtbar + c * sgn * alpf * bett;
    ev[2][3] = alps * vubar + c * sgn * alpf * betu;
    ev[2][4] = -rrobai * c2 * alpf * bett * cfi;
    ev[2][5] = -rrobai * c2 * alpf * betu * cfi;
    ev[2][6] = alps * (kin + db2 + cs * vnbar + cs2 * gm1i + (cs2 - c2) * gm2 * gm1i)
               + alpf * c * (bett * vtbar + betu * vubar) * sgn;
    ev[3][0] = alps;
    ev[3][1] = alps * (vnbar - cs);
    ev[3][2] = alps * vtbar - c * sgn * alpf * bett;
    ev[3][3] = alps * vubar - c * sgn * alpf * betu;
    ev[3][4] = ev[2][4];
    ev[3][5] = ev[2][5];
    ev[3][6] = alps * (kin + db2 - cs * vnbar + cs2 * gm1i + (cs2 - c2) * gm2 * gm1i)
               - alpf * c * (bett * vtbar + betu * vubar) * sgn;
    ev[4][0] = 0.0;
    ev[4][1] = 0.0;
    ev[4][2] = -sgn * betu;
    ev[4][3] = sgn * bett;
    ev[4][4] = rrobai * betu;
    ev[4][5] = -rrobai * bett;
    ev[4][6] = -(betu * vtbar - bett * vubar) * sgn;
    ev[5][0] = 0.0;
    ev[5][1] = 0.0;
    ev[5][2] = -ev[4][2];
    ev[5][3] = -ev[4][3];
    ev[5][4] = ev[4][4];
    ev[5][5] = ev[4][5];
    ev[5][6] = -ev[4][6];
    ev[6][0] = 1.0;
    ev[6][1] = vnbar;
    ev[6][2] = vtbar;
    ev[6][3] = vubar;
    ev[6][4] = 0.0;
    ev[6][5] = 0.0;
    ev[6][6] = kin + db2;
    const double eval[7] = {evpf, evmf, evps, evms, evpa, evma, ev00};
    const double wamp[7] = {wvpf, wvmf, wvps, wvms, wvpa, wvma, wv00};
    for (int k = 0; k < 7; k++) {
        double s = FL[k] + FR[k];
        for (int w = 0; w < 7; w++) s = s - eval[w] * wamp[w] * ev[w][k];
        f[k] = 0.5 * s;
    }
}

static inline void o_flux(int which, const double *l, const double *r, double bn,
                          double gamma, const double *dv, double *f)
{
    switch (which) {
    case 0:
        o_flux_mlau(l[0], l[1], l[2], l[3], l[4], l[5], l[6], r[0], r[1], r[2], r[3], r[4],
                    r[5], r[6], bn, gamma, dv, f);
        break;
    case 1:
        o_flux_hlld(1, l[0], l[1], l[2], l[3], l[4], l[5], l[6], r[0], r[1], r[2], r[3], r[4],
                    r[5], r[6], bn, gamma, dv, f);
        break;
    case 2:
        o_flux_hlld(0, l[0], l[1], l[2], l[3], l[4], l[5], l[6], r[0], r[1], r[2], r[3], r[4],
                    r[5], r[6], bn, gamma, dv, f);
        break;
    default:
        o_flux_roe(l[0], l[1], l[2], l[3], l[4], l[5], l[6], r[0], r[1], r[2], r[3], r[4],
                   r[5], r[6], bn, gamma, f);
        break;
    }
}

#endif
