/*
 * CPU oracle for the MLAU per-step hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference solver's step drivers and point
 * functions, used by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline as the checker.  The GPU product never links, loads or calls it.
 *
 * Every function keeps the reference's arithmetic in the same evaluation order
 * and is built with -ffp-contract=off, so on identical inputs it reproduces the
 * reference bit for bit.  That claim is pinned by tests that compare it with the
 * reference itself (compiled from its own sources by oracle/build_ref.sh) and
 * with committed golden vectors made by that build (tests/golden/).
 *
 * Layout (as in the reference): one array per variable, x fastest,
 * index = nx*(ny*k+j)+i, ghost depth xoff=yoff=zoff (4 for ODR 4).
 * Boundaries: periodic in every direction (the reference's single-rank
 * periodic branch of mpi_sdrv3d / bc2d / prdc_1d), or the 1D characteristic
 * open boundary of 1D/SERIAL/shock/openbc1d_mhd.c.
 */
#ifndef MLAU_ORACLE_H
#define MLAU_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Riemann solver selector (include/mhd_flux.h of the reference). */
enum { ORACLE_FLUX_MLAU = 0, ORACLE_FLUX_LHLLD = 1, ORACLE_FLUX_HLLD = 2, ORACLE_FLUX_ROE = 3 };
/* 1D boundary selector. */
enum { ORACLE_BC1D_OPEN = 0, ORACLE_BC1D_PERIODIC = 1 };

/* One full SSP-RK step of 3D ideal MHD with CT, in place, periodic.
 * Restates 3D/MPI/OTvortex/mhd_fd_ct_3d.c:99-1198 (single rank). */
void oracle_fd_ct_3d(double *ro, double *mx, double *my, double *mz,
                     double *en, double *bx, double *by, double *bz,
                     double dt, double dx, double dy, double dz,
                     int nx, int ny, int nz, int xoff, int yoff, int zoff,
                     double gamma, int odr, int flux, int nrk);

/* One full SSP-RK step of 2D ideal MHD with CT, in place, periodic.
 * Restates 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-660. */
void oracle_fd_ct_2d(double *ro, double *mx, double *my, double *mz,
                     double *en, double *bx, double *by, double *bz,
                     double dt, double dx, double dy,
                     int nx, int ny, int xoff, int yoff,
                     double gamma, int odr, int flux, int nrk);
/* The problems' setbc: the boundary tables applied to the conserved arrays. */
void oracle_bc2d_state(double *ro, double *mx, double *my, double *mz,
                       double *en, double *bx, double *by, double *bz,
                       int nx, int ny, int xoff, int yoff, const int *dnx, const int *dny);
/* Same with the problem's boundary tables dnx[8]/dny[8] (global.hpp dnxs /
 * dnys, variable order ro mx my mz en bx by bz; 0 periodic, -1 Dirichlet,
 * +1 Neumann); NULL tables are periodic. */
void oracle_fd_ct_2d_bc(double *ro, double *mx, double *my, double *mz,
                        double *en, double *bx, double *by, double *bz,
                        double dt, double dx, double dy,
                        int nx, int ny, int xoff, int yoff,
                        double gamma, int odr, int flux, int nrk,
                        const int *dnx, const int *dny);

/* One full SSP-RK step of 1D MHD (7 variables, constant bx), in place.
 * Restates 1D/SERIAL/shock/mhd_fd4c_1d.c:60-271 (bc=OPEN, open boundary at
 * stage 0 via openbc1d_mhd.c:21-175) and 1D/SERIAL/wave/mhd_fd4c_1d.c
 * (bc=PERIODIC, prdc_1d after each stage). */
void oracle_fd4c_1d(double *ro, double *mx, double *my, double *mz,
                    double *en, double *by, double *bz,
                    double bx, double dt, double dx, int nx, int xoff,
                    double gamma, int odr, int flux, int nrk, int bc);

/* CFL time step.  Return the new dt (or dt_old when vmax is not finite).
 * 3D: 3D/MPI/OTvortex/cflcheck.hpp:1-39, 2D: 2D/SERIAL/OTvortex/cflcheck.hpp,
 * 1D: 1D/SERIAL/shock/main.cpp:113-128. vmax_out may be NULL. */
double oracle_cfl_3d(const double *ro, const double *mx, const double *my, const double *mz,
                     const double *en, const double *bx, const double *by, const double *bz,
                     int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma,
                     double cfl, double dr, double vfast, double dt_old, double *vmax_out);
double oracle_cfl_2d(const double *ro, const double *mx, const double *my, const double *mz,
                     const double *en, const double *bx, const double *by, const double *bz,
                     int nx, int ny, int xoff, int yoff, double gamma,
                     double cfl, double dr, double vfast, double dt_old, double *vmax_out);
double oracle_dt_1d(const double *ro, const double *mx, const double *my, const double *mz,
                    const double *en, const double *by, const double *bz, double bx,
                    int nx, double gamma, double cfl, double dx, double vfloor);

/* Point functions, exported for known-answer tests.
 * rec_lr: include/interp.h via the drivers' calc_flr (odr 1..4).
 * flux:   include/mhd_flux.h calc_flux_{mlau,lhlld,hlld,roe}; in[16] = 7 left
 *         primitives, 7 right primitives, bn, gamma; dv[2]; out[7]. */
void oracle_rec_lr(int odr, const double *f5, double *fl, double *fr);
void oracle_flux(int flux, const double *in16, const double *dv, double *out7);
/* Characteristic reconstruction (include/mhd_eigen.h mhd_c_reconst /
 * mhd_a_reconst): prim[7][5] stencils of (ro,vn,vt,vu,bt,bu,pr). */
void oracle_reconst(int full, int odr, const double *prim35, double bn, double gamma,
                    double *ul7, double *ur7);

#ifdef __cplusplus
}
#endif
/* 2D MRX operators (2D/MPI/MRX/mhd_fd_ct_2d.c:726-1174) for one rank:
 * resistive diffusion of the CT field (uniform eta0, energy updated by the
 * resistive Poynting flux) and the viscous term (uniform kinematic nu0).
 * odr/nrk as the driver file's ODR / R_K; dnx/dny the problem's dnxs/dnys
 * (NULL: periodic), with the MPI drivers' single-rank boundary routines. */
void oracle_diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0,
                           double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                           double gamma, int odr, int nrk, const int *dnx, const int *dny);
void oracle_ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en,
                          double nu0, double dt, double dx, double dy, int nx, int ny, int xoff,
                          int yoff, double gamma, int odr, int nrk, const int *dnx,
                          const int *dny);
/* The RMI problem's inflow (inj_ro, 2D/MPI/RMI/inj_ro.hpp:1-58) and the
 * periodic exchange its main loop runs after it; noise: the random() / RAND_MAX
 * draws in loop order, or NULL. */
void oracle_inj_ro(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                   double *by, double *bz, int nx, int ny, int xoff, int yoff, double ro_3,
                   double dro3, double vy_1, double bx_1, double by_1, double bz_1, double pr_1,
                   double vref, double gam, const double *noise, const int *dnx,
                   const int *dny);
/* The 3D step with the problem's tables dnxs/dnys/dnzs (NULL: periodic),
 * filled as the MPI driver's single-rank routines do. */
void oracle_fd_ct_3d_bc(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                        double *by, double *bz, double dt, double dx, double dy, double dz,
                        int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma,
                        int odr, int flx, int nrk, const int *dnx, const int *dny,
                        const int *dnz);
/* Eigen-system of the oracle's steps where Mach^2 >= 1: 0 the drivers' full
 * 7-wave system, 1 Miyoshi's (the driver with mhd_c_reconst swapped for
 * mhd_m_reconst). */
void oracle_set_eigen(int miyoshi);
/* Anisotropic heat conduction along B (t_conduction with diffusion2d_ani,
 * 2D/MPI/MRX/mhd_fd_ct_2d.c:1176-1456): implicit Crank-Nicolson in p/rho by
 * six-colour Gauss-Seidel; returns the sweep count, *err = -1 when cmax
 * sweeps did not converge (the reference's CMAX is 2048). */
int oracle_t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                        double *en, const double *bx, const double *by, const double *bz,
                        double kk0, double dt, double dx, double dy, int nx, int ny, int xoff,
                        int yoff, double gamma, int odr, const int *dnx, const int *dny,
                        int cmax, int *err);

#endif
