/* The reference's point-function interface on this library's point functions.
 *
 * A program written against the reference's include/funcs.h, interp.h,
 * mhd_eigen.h and mhd_flux.h includes this header in their place and compiles
 * unchanged, on the host (any C++ compiler) and in CUDA device code (nvcc):
 * every function keeps the reference's name, parameter list and argument
 * meaning, as an inline __host__ __device__ adapter over the templates of
 * mlau_gb300/csrc/point.cuh.  With double arguments, built without
 * floating-point contraction (-ffp-contract=off on the host, --fmad=false
 * under nvcc) as the reference is built, the results are the reference
 * headers' bit for bit, signed zeros included.  Each function also has a
 * float overload with the same parameter list in float: the arithmetic of the
 * FP32-split form.
 *
 *   reference                               replaced by (double / float)
 *   funcs.h:23-31      max, min             host compilers only (see below)
 *   funcs.h:33-43      minmod, minmod3
 *   interp.h:25-72     muscl_{mm,mc,kr}_cal_f, muscl_{mm,mc,kr}_cal_flr
 *   interp.h:75-146    wcns3_cal_f, wcns3_cal_flr
 *   interp.h:148-238   wcns4_cal_f, wcns4_cal_flr
 *   mhd_eigen.h:24-453 mhd_eigen_st, mhd_eigen_mi, mhd_eigen_ae
 *   mhd_eigen.h:455-724 mhd_c_reconst, mhd_m_reconst, mhd_a_reconst, mhd_reconst
 *   mhd_flux.h:26-213  calc_flux_mlau       (the 25-argument flux type of the
 *   mhd_flux.h:215-454 calc_flux_roe         drivers' func_flux pointer,
 *   mhd_flux.h:456-582 calc_flux_hlld        3D/MPI/OTvortex/mhd_fd_ct_3d.c:
 *   mhd_flux.h:584-719 calc_flux_lhlld       130-137)
 *   mhd_flux.h:722-732 calc_flux_hl3d2      (LHLLD, as in the reference)
 *   mhd_flux.h:734-766 hall_flux_lf
 *
 * Differences, all outside the reference's own use:
 *   - max and min are defined for host compilers only.  Under nvcc the CUDA
 *     math headers already define max/min(double, double) for host and
 *     device code; they agree with funcs.h's (a >= b) ? a : b except when
 *     the second argument is NaN or the two are zeros of opposite sign.
 *   - the mhd_*_reconst stencil length s is at most 8 (the drivers use 5);
 *     a longer stencil returns NaN faces.  The reference sizes its scratch
 *     with a variable-length array, which device code cannot.
 *   - the reference's EPS macro (mhd_flux.h:24) is not defined.
 *   - calc_flux_roe, calc_flux_hlld and hall_flux_lf do not read dv, as in
 *     the reference, so it may be a null pointer there.
 */
#ifndef MLAU_POINT_H
#define MLAU_POINT_H

#include "../mlau_gb300/csrc/point.cuh"

#define MLAU_POINT_MAX_STENCIL 8

/* funcs.h:23-43 */
#ifndef __CUDACC__
inline double max(double a, double b) { return mlau::vmax(a, b); }
inline double min(double a, double b) { return mlau::vmin(a, b); }
inline float max(float a, float b) { return mlau::vmax(a, b); }
inline float min(float a, float b) { return mlau::vmin(a, b); }
#endif
MLAU_HD double minmod(double a, double b) { return mlau::minmod(a, b); }
MLAU_HD float minmod(float a, float b) { return mlau::minmod(a, b); }
MLAU_HD double minmod3(double a, double b, double c) { return mlau::minmod3(a, b, c); }
MLAU_HD float minmod3(float a, float b, float c) { return mlau::minmod3(a, b, c); }

/* interp.h: one-sided values and face pairs.  The _flr forms return the
 * value left of face i+1/2 in *fl and right of face i-1/2 in *fr. */
#define MLAU_POINT_INTERP(T)                                                                  \
    MLAU_HD T muscl_mm_cal_f(T fu, T f0, T fd) { return mlau::muscl_mm_f(fu, f0, fd); }     \
    MLAU_HD T muscl_mc_cal_f(T fu, T f0, T fd) { return mlau::muscl_mc_f(fu, f0, fd); }     \
    MLAU_HD T muscl_kr_cal_f(T fu, T f0, T fd) { return mlau::muscl_kr_f(fu, f0, fd); }     \
    MLAU_HD void muscl_mm_cal_flr(T f1, T f2, T f3, T *fl, T *fr)                            \
    {                                                                                         \
        mlau::muscl_mm_lr(f1, f2, f3, *fl, *fr);                                              \
    }                                                                                         \
    MLAU_HD void muscl_mc_cal_flr(T f1, T f2, T f3, T *fl, T *fr)                            \
    {                                                                                         \
        mlau::muscl_mc_lr(f1, f2, f3, *fl, *fr);                                              \
    }                                                                                         \
    MLAU_HD void muscl_kr_cal_flr(T f1, T f2, T f3, T *fl, T *fr)                            \
    {                                                                                         \
        mlau::muscl_kr_lr(f1, f2, f3, *fl, *fr);                                              \
    }                                                                                         \
    MLAU_HD T wcns3_cal_f(T fup, T f, T fdn) { return mlau::wcns3_f(fup, f, fdn); }         \
    MLAU_HD void wcns3_cal_flr(T f0, T f1, T f2, T *fl, T *fr)                               \
    {                                                                                         \
        mlau::wcns3_lr(f0, f1, f2, *fl, *fr);                                                 \
    }                                                                                         \
    MLAU_HD T wcns4_cal_f(T fuu, T fup, T f, T fdn, T fdd)                                    \
    {                                                                                         \
        return mlau::wcns4_f(fuu, fup, f, fdn, fdd);                                          \
    }                                                                                         \
    MLAU_HD void wcns4_cal_flr(T f0, T f1, T f2, T f3, T f4, T *fl, T *fr)                   \
    {                                                                                         \
        mlau::wcns4_lr(f0, f1, f2, f3, f4, *fl, *fr);                                         \
    }
MLAU_POINT_INTERP(double)
MLAU_POINT_INTERP(float)
#undef MLAU_POINT_INTERP

/* mhd_eigen.h:24-453: eigenvalues al1..al7 (mhd_eigen_st only; the others
 * leave them untouched), left eigenvectors l1..l7 (rows) and right
 * eigenvectors r1..r7 (columns), 7 entries each. */
namespace mlau {
template <class T> struct EigenOut {
    T *al[7], *l[7], *r[7];
    template <class F> MLAU_HD void fill(F eig, T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr,
                                         T gamma) const
    {
        T a[7], L[7][7], R[7][7];
        eig(ro, vx, vy, vz, bx, by, bz, pr, gamma, a, L, R);
        for (int n = 0; n < 7; n++)
            for (int k = 0; k < 7; k++) { l[n][k] = L[n][k]; r[n][k] = R[n][k]; }
    }
    template <class F> MLAU_HD void fill_al(F eig, T ro, T vx, T vy, T vz, T bx, T by, T bz,
                                            T pr, T gamma) const
    {
        T a[7], L[7][7], R[7][7];
        eig(ro, vx, vy, vz, bx, by, bz, pr, gamma, a, L, R);
        for (int n = 0; n < 7; n++) {
            *al[n] = a[n];
            for (int k = 0; k < 7; k++) { l[n][k] = L[n][k]; r[n][k] = R[n][k]; }
        }
    }
};
template <class T> struct EigSt {
    MLAU_HD void operator()(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T g, T a[7],
                            T L[7][7], T R[7][7]) const
    {
        eigen_st_dense(ro, vx, vy, vz, bx, by, bz, pr, g, a, L, R);
    }
};
template <class T> struct EigAe {
    MLAU_HD void operator()(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T g, T a[7],
                            T L[7][7], T R[7][7]) const
    {
        eigen_ae_dense(ro, vx, vy, vz, bx, by, bz, pr, g, a, L, R);
    }
};
template <class T> struct EigMi {
    MLAU_HD void operator()(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T g, T a[7],
                            T L[7][7], T R[7][7]) const
    {
        eigen_mi_dense(ro, vx, vy, vz, bx, by, bz, pr, g, a, L, R);
    }
};
}  // namespace mlau

#define MLAU_POINT_EIGEN(T)                                                                   \
    MLAU_HD void mhd_eigen_st(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma,       \
                              T *al1, T *al2, T *al3, T *al4, T *al5, T *al6, T *al7, T *l1, \
                              T *l2, T *l3, T *l4, T *l5, T *l6, T *l7, T *r1, T *r2, T *r3, \
                              T *r4, T *r5, T *r6, T *r7)                                    \
    {                                                                                         \
        const mlau::EigenOut<T> o{{al1, al2, al3, al4, al5, al6, al7},                        \
                                  {l1, l2, l3, l4, l5, l6, l7},                               \
                                  {r1, r2, r3, r4, r5, r6, r7}};                              \
        o.fill_al(mlau::EigSt<T>(), ro, vx, vy, vz, bx, by, bz, pr, gamma);                   \
    }                                                                                         \
    MLAU_HD void mhd_eigen_mi(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma,       \
                              T *al1, T *al2, T *al3, T *al4, T *al5, T *al6, T *al7, T *l1, \
                              T *l2, T *l3, T *l4, T *l5, T *l6, T *l7, T *r1, T *r2, T *r3, \
                              T *r4, T *r5, T *r6, T *r7)                                    \
    {                                                                                         \
        const mlau::EigenOut<T> o{{al1, al2, al3, al4, al5, al6, al7},                        \
                                  {l1, l2, l3, l4, l5, l6, l7},                               \
                                  {r1, r2, r3, r4, r5, r6, r7}};                              \
        o.fill(mlau::EigMi<T>(), ro, vx, vy, vz, bx, by, bz, pr, gamma);                      \
    }                                                                                         \
    MLAU_HD void mhd_eigen_ae(T ro, T vx, T vy, T vz, T bx, T by, T bz, T pr, T gamma,       \
                              T *al1, T *al2, T *al3, T *al4, T *al5, T *al6, T *al7, T *l1, \
                              T *l2, T *l3, T *l4, T *l5, T *l6, T *l7, T *r1, T *r2, T *r3, \
                              T *r4, T *r5, T *r6, T *r7)                                    \
    {                                                                                         \
        const mlau::EigenOut<T> o{{al1, al2, al3, al4, al5, al6, al7},                        \
                                  {l1, l2, l3, l4, l5, l6, l7},                               \
                                  {r1, r2, r3, r4, r5, r6, r7}};                              \
        o.fill(mlau::EigAe<T>(), ro, vx, vy, vz, bx, by, bz, pr, gamma);                      \
    }
MLAU_POINT_EIGEN(double)
MLAU_POINT_EIGEN(float)
#undef MLAU_POINT_EIGEN

/* mhd_eigen.h:455-724: reconstruction of the 7 primitives (ro, vx, vy, vz,
 * by, bz, pr; x is the face normal) from an s-point stencil centred on s/2,
 * with func_lr the face interpolation of one field (the drivers pass their
 * calc_flr).  ul: left of face i+1/2; ur: right of face i-1/2. */
#define MLAU_POINT_RECONST(T)                                                                 \
    MLAU_HD void mhd_c_reconst(const T *ro, const T *vx, const T *vy, const T *vz,            \
                               const T *by, const T *bz, const T *pr, T bx, T gamma,          \
                               const int s, T *ul, T *ur,                                     \
                               void (*func_lr)(const T *, T *, T *))                          \
    {                                                                                         \
        mlau::reconst_dense(mlau::EigSt<T>(), ro, vx, vy, vz, by, bz, pr, bx, gamma, s, ul,   \
                            ur, func_lr);                                                     \
    }                                                                                         \
    MLAU_HD void mhd_m_reconst(const T *ro, const T *vx, const T *vy, const T *vz,            \
                               const T *by, const T *bz, const T *pr, T bx, T gamma,          \
                               const int s, T *ul, T *ur,                                     \
                               void (*func_lr)(const T *, T *, T *))                          \
    {                                                                                         \
        mlau::reconst_dense(mlau::EigMi<T>(), ro, vx, vy, vz, by, bz, pr, bx, gamma, s, ul,   \
                            ur, func_lr);                                                     \
    }                                                                                         \
    MLAU_HD void mhd_a_reconst(const T *ro, const T *vx, const T *vy, const T *vz,            \
                               const T *by, const T *bz, const T *pr, T bx, T gamma,          \
                               const int s, T *ul, T *ur,                                     \
                               void (*func_lr)(const T *, T *, T *))                          \
    {                                                                                         \
        mlau::reconst_dense(mlau::EigAe<T>(), ro, vx, vy, vz, by, bz, pr, bx, gamma, s, ul,   \
                            ur, func_lr);                                                     \
    }                                                                                         \
    MLAU_HD void mhd_reconst(const T *ro, const T *vx, const T *vy, const T *vz, const T *by, \
                             const T *bz, const T *pr, T bx, T gamma, const int s, T *ul,     \
                             T *ur, void (*func_lr)(const T *, T *, T *))                     \
    {                                                                                         \
        (void)bx;                                                                             \
        (void)gamma;                                                                          \
        mlau::reconst_prim(ro, vx, vy, vz, by, bz, pr, s, ul, ur, func_lr);                   \
    }
MLAU_POINT_RECONST(double)
MLAU_POINT_RECONST(float)
#undef MLAU_POINT_RECONST

/* mhd_flux.h: numerical fluxes at a face from the left (..l) and right (..r)
 * primitives (ro, vn, vt, vu, bt, bu, pr), the face-normal field bnc and
 * gamma; dv[0] is the normal velocity jump across the face and dv[1] the
 * smallest transverse one (the MLAU and LHLLD shock sensor).  Outputs: the
 * fluxes of ro, mn, mt, mu, bt, bu, en. */
namespace mlau {
template <class T> struct FluxOut {
    T *p[7];
    MLAU_HD void put(const T f[7]) const
    {
        for (int n = 0; n < 7; n++) *p[n] = f[n];
    }
};
}  // namespace mlau
#define MLAU_POINT_FLUX_ARGS(T)                                                               \
    T rol, T vnl, T vtl, T vul, T btl, T bul, T prl, T ror, T vnr, T vtr, T vur, T btr, T bur, \
        T prr, T bnc, T gamma, T *dv, T *fro, T *fmn, T *fmt, T *fmu, T *fbt, T *fbu, T *fen
#define MLAU_POINT_FLUX(T)                                                                    \
    MLAU_HD void calc_flux_mlau(MLAU_POINT_FLUX_ARGS(T))                                      \
    {                                                                                         \
        const T L[7] = {rol, vnl, vtl, vul, btl, bul, prl};                                   \
        const T R[7] = {ror, vnr, vtr, vur, btr, bur, prr};                                   \
        T f[7];                                                                               \
        mlau::flux_mlau(L, R, bnc, gamma, dv[0], dv[1], f);                                   \
        mlau::FluxOut<T>{{fro, fmn, fmt, fmu, fbt, fbu, fen}}.put(f);                         \
    }                                                                                         \
    MLAU_HD void calc_flux_lhlld(MLAU_POINT_FLUX_ARGS(T))                                     \
    {                                                                                         \
        const T L[7] = {rol, vnl, vtl, vul, btl, bul, prl};                                   \
        const T R[7] = {ror, vnr, vtr, vur, btr, bur, prr};                                   \
        T f[7];                                                                               \
        mlau::flux_hlld<T, true>(L, R, bnc, gamma, dv[0], dv[1], f);                          \
        mlau::FluxOut<T>{{fro, fmn, fmt, fmu, fbt, fbu, fen}}.put(f);                         \
    }                                                                                         \
    MLAU_HD void calc_flux_hlld(MLAU_POINT_FLUX_ARGS(T))                                      \
    {                                                                                         \
        (void)dv;                                                                             \
        const T L[7] = {rol, vnl, vtl, vul, btl, bul, prl};                                   \
        const T R[7] = {ror, vnr, vtr, vur, btr, bur, prr};                                   \
        T f[7];                                                                               \
        mlau::flux_hlld<T, false>(L, R, bnc, gamma, T(0), T(0), f);                           \
        mlau::FluxOut<T>{{fro, fmn, fmt, fmu, fbt, fbu, fen}}.put(f);                         \
    }                                                                                         \
    MLAU_HD void calc_flux_roe(MLAU_POINT_FLUX_ARGS(T))                                       \
    {                                                                                         \
        (void)dv;                                                                             \
        const T L[7] = {rol, vnl, vtl, vul, btl, bul, prl};                                   \
        const T R[7] = {ror, vnr, vtr, vur, btr, bur, prr};                                   \
        T f[7];                                                                               \
        mlau::flux_roe(L, R, bnc, gamma, f);                                                  \
        mlau::FluxOut<T>{{fro, fmn, fmt, fmu, fbt, fbu, fen}}.put(f);                         \
    }                                                                                         \
    MLAU_HD void calc_flux_hl3d2(MLAU_POINT_FLUX_ARGS(T))                                     \
    {                                                                                         \
        calc_flux_lhlld(rol, vnl, vtl, vul, btl, bul, prl, ror, vnr, vtr, vur, btr, bur, prr, \
                        bnc, gamma, dv, fro, fmn, fmt, fmu, fbt, fbu, fen);                   \
    }                                                                                         \
    MLAU_HD void hall_flux_lf(T rol, T vnl, T vtl, T vul, T btl, T bul, T enl, T ror, T vnr,  \
                              T vtr, T vur, T btr, T bur, T enr, T bnc, T smax, T *fbt,       \
                              T *fbu, T *fen)                                                 \
    {                                                                                         \
        (void)rol;                                                                            \
        (void)enl;                                                                            \
        (void)ror;                                                                            \
        (void)enr;                                                                            \
        mlau::hall_lf(vnl, vtl, vul, btl, bul, vnr, vtr, vur, btr, bur, bnc, smax, fbt, fbu,  \
                      fen);                                                                   \
    }
MLAU_POINT_FLUX(double)
MLAU_POINT_FLUX(float)
#undef MLAU_POINT_FLUX
#undef MLAU_POINT_FLUX_ARGS

#endif /* MLAU_POINT_H */
