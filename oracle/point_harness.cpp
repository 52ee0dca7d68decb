// Batch drivers of the point functions, for tests.  TEST INFRASTRUCTURE ONLY.
//
// The same source is compiled twice: with -DMLAU_POINT_REF against the
// reference's include/interp.h, mhd_eigen.h and mhd_flux.h, and without it
// against this library's include/mlau_point.h, which declares the same
// functions under the same names.  The two builds are compared value for
// value on seeded inputs (tests/test_point_api.py) and the reference build
// writes the golden vectors (tests/golden/make_point_golden.py).
//
// Layouts (rows of doubles, one per call):
//   ph_flux     in  rol vnl vtl vul btl bul prl ror vnr vtr vur btr bur prr
//                   bnc gamma dv0 dv1                                (18)
//               out fro fmn fmt fmu fbt fbu fen                       (7)
//   ph_interp   in  f0..f4 (5)  out fl fr (2; one-sided forms: f, 0)
//   ph_eigen    in  ro vx vy vz bx by bz pr gamma (9)
//               out al1..al7, l1..l7 (7 each), r1..r7 (7 each)       (105)
//   ph_reconst  in  ro[5] vx[5] vy[5] vz[5] by[5] bz[5] pr[5] bx gamma (37)
//               out ul[7] ur[7]                                       (14)
#include <math.h>
#ifdef MLAU_POINT_REF
#include "interp.h"
#include "mhd_eigen.h"
#include "mhd_flux.h"
#else
#include "mlau_point.h"
#endif

namespace {

typedef void (*FluxFn)(double, double, double, double, double, double, double, double, double,
                       double, double, double, double, double, double, double, double *,
                       double *, double *, double *, double *, double *, double *, double *);
typedef void (*ReconstFn)(const double *, const double *, const double *, const double *,
                          const double *, const double *, const double *, double, double,
                          const int, double *, double *,
                          void (*)(const double *, double *, double *));
typedef void (*EigenFn)(double, double, double, double, double, double, double, double, double,
                        double *, double *, double *, double *, double *, double *, double *,
                        double *, double *, double *, double *, double *, double *, double *,
                        double *, double *, double *, double *, double *, double *, double *);

// the drivers' calc_flr (3D/MPI/OTvortex/mhd_fd_ct_3d.c:65-78) with the
// reconstruction code chosen at run time: 1-4 ODR, 5 MC and 6 Koren MUSCL
int g_odr = 4;
void flr(const double *f, double *fl, double *fr)
{
    switch (g_odr) {
    case 1: *fl = f[2]; *fr = f[2]; break;
    case 2: muscl_mm_cal_flr(f[1], f[2], f[3], fl, fr); break;
    case 3: wcns3_cal_flr(f[1], f[2], f[3], fl, fr); break;
    case 5: muscl_mc_cal_flr(f[1], f[2], f[3], fl, fr); break;
    case 6: muscl_kr_cal_flr(f[1], f[2], f[3], fl, fr); break;
    default: wcns4_cal_flr(f[0], f[1], f[2], f[3], f[4], fl, fr); break;
    }
}

}  // namespace

extern "C" {

int ph_flux(int which, long n, const double *in, double *out)
{
    static const FluxFn fns[5] = {&calc_flux_mlau, &calc_flux_lhlld, &calc_flux_hlld,
                                  &calc_flux_roe, &calc_flux_hl3d2};
    if (which < 0 || which > 4) return -1;
    const FluxFn fn = fns[which];
    for (long t = 0; t < n; t++) {
        const double *q = in + 18 * t;
        double *o = out + 7 * t;
        double dv[2] = {q[16], q[17]};
        fn(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], q[10], q[11], q[12], q[13],
           q[14], q[15], dv, o, o + 1, o + 2, o + 3, o + 4, o + 5, o + 6);
    }
    return 0;
}

int ph_interp(int which, long n, const double *in, double *out)
{
    for (long t = 0; t < n; t++) {
        const double *f = in + 5 * t;
        double *o = out + 2 * t;
        o[1] = 0.0;
        switch (which) {
        case 0: muscl_mm_cal_flr(f[0], f[1], f[2], o, o + 1); break;
        case 1: muscl_mc_cal_flr(f[0], f[1], f[2], o, o + 1); break;
        case 2: muscl_kr_cal_flr(f[0], f[1], f[2], o, o + 1); break;
        case 3: wcns3_cal_flr(f[0], f[1], f[2], o, o + 1); break;
        case 4: wcns4_cal_flr(f[0], f[1], f[2], f[3], f[4], o, o + 1); break;
        case 5: o[0] = muscl_mm_cal_f(f[0], f[1], f[2]); break;
        case 6: o[0] = muscl_mc_cal_f(f[0], f[1], f[2]); break;
        case 7: o[0] = muscl_kr_cal_f(f[0], f[1], f[2]); break;
        case 8: o[0] = wcns3_cal_f(f[0], f[1], f[2]); break;
        case 9: o[0] = wcns4_cal_f(f[0], f[1], f[2], f[3], f[4]); break;
        case 10: o[0] = minmod(f[0], f[1]); break;
        case 11: o[0] = minmod3(f[0], f[1], f[2]); break;
        case 12: o[0] = max(f[0], f[1]); break;
        case 13: o[0] = min(f[0], f[1]); break;
        default: return -1;
        }
    }
    return 0;
}

int ph_eigen(int which, long n, const double *in, double *out)
{
    static const EigenFn fns[3] = {&mhd_eigen_st, &mhd_eigen_mi, &mhd_eigen_ae};
    if (which < 0 || which > 2) return -1;
    const EigenFn fn = fns[which];
    for (long t = 0; t < n; t++) {
        const double *q = in + 9 * t;
        double *a = out + 105 * t, *l = a + 7, *r = a + 56;
        // entries a system leaves unset keep these markers
        for (int k = 0; k < 7; k++) a[k] = 7.25;
        for (int k = 0; k < 49; k++) { l[k] = 3.5; r[k] = -3.5; }
        fn(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], a, a + 1, a + 2, a + 3, a + 4,
           a + 5, a + 6, l, l + 7, l + 14, l + 21, l + 28, l + 35, l + 42, r, r + 7, r + 14,
           r + 21, r + 28, r + 35, r + 42);
    }
    return 0;
}

int ph_reconst(int which, int odr, long n, const double *in, double *out)
{
    static const ReconstFn fns[4] = {&mhd_c_reconst, &mhd_m_reconst, &mhd_a_reconst,
                                     &mhd_reconst};
    if (which < 0 || which > 3 || odr < 1 || odr > 6) return -1;
    g_odr = odr;
    const ReconstFn fn = fns[which];
    for (long t = 0; t < n; t++) {
        const double *q = in + 37 * t;
        double *o = out + 14 * t;
        fn(q, q + 5, q + 10, q + 15, q + 20, q + 25, q + 30, q[35], q[36], 5, o, o + 7, &flr);
    }
    return 0;
}

#ifndef MLAU_POINT_REF
// The float overloads (the FP32-split form's arithmetic) on the same rows.
int ph_flux_f(int which, long n, const double *in, double *out)
{
    typedef void (*FluxFnF)(float, float, float, float, float, float, float, float, float, float,
                            float, float, float, float, float, float, float *, float *, float *,
                            float *, float *, float *, float *, float *);
    static const FluxFnF fns[5] = {&calc_flux_mlau, &calc_flux_lhlld, &calc_flux_hlld,
                                   &calc_flux_roe, &calc_flux_hl3d2};
    if (which < 0 || which > 4) return -1;
    for (long t = 0; t < n; t++) {
        float q[18], o[7];
        for (int k = 0; k < 18; k++) q[k] = (float)in[18 * t + k];
        float dv[2] = {q[16], q[17]};
        fns[which](q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], q[10], q[11],
                   q[12], q[13], q[14], q[15], dv, o, o + 1, o + 2, o + 3, o + 4, o + 5, o + 6);
        for (int k = 0; k < 7; k++) out[7 * t + k] = o[k];
    }
    return 0;
}
#endif

}  // extern "C"
