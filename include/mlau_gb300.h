/*
 * mlau_gb300.h - C ABI of the GB300 (sm_103a) MHD step library
 * (libmlau_gb300.so).
 *
 * Two layers:
 *
 * 1. Drop-in step drivers with the reference solver's names and parameter
 *    lists.  Each call copies the caller's host arrays to the GPU, advances
 *    one full SSP-RK step there, and copies them back, in place, like the
 *    reference's OpenMP drivers.  The library exports each one twice: with C
 *    linkage (the names below) and with the reference's own C++ linkage, so
 *    that an unmodified problem main.cpp relinks against this library in
 *    place of the driver object file.
 *
 * 2. A handle API that keeps a simulation resident in HBM across steps (the
 *    fast path): create / upload / step / cfl / download / destroy.
 *
 * Arrays: one float64 array per variable, x fastest, index nx*(ny*k+j)+i,
 * ghost cells included (the reference layout).  Face-centred bx[i] sits at
 * x_{i-1/2}, by[j] at y_{j-1/2}, bz[k] at z_{k-1/2}.  Boundaries: periodic.
 *
 * Errors: status-returning calls return 0 on success and a negative MLAU_ERR_*
 * code otherwise; mlau_last_error() gives the message.  The void drop-in
 * drivers keep the reference's void signature; on error they leave the
 * arrays untouched, print the message to stderr and record it.
 */
#ifndef MLAU_GB300_H
#define MLAU_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MLAU_OK = 0,
    MLAU_ERR_ARG = -1,         /* invalid argument or unsupported configuration */
    MLAU_ERR_CUDA = -2,        /* CUDA runtime error */
    MLAU_ERR_NOMEM = -3,       /* device memory exhausted / over budget */
    MLAU_ERR_STATE = -4,       /* NaN or non-positive density/pressure seen */
    MLAU_ERR_TIMEOUT = -5,     /* a bounded device-side wait gave up */
    MLAU_ERR_CONVERGE = -6     /* an iterative solve ran out of sweeps */
};

/* Riemann solvers of include/mhd_flux.h. */
enum { MLAU_FLUX_MLAU = 0, MLAU_FLUX_LHLLD = 1, MLAU_FLUX_HLLD = 2, MLAU_FLUX_ROE = 3 };
/* Arithmetic of the step.  MLAU_FP64: the reference's, bit for bit.
 * MLAU_FP32_SPLIT: reconstruction, Riemann solver, edge EMFs, CT weights and
 * shock sensors in FP32; the conserved state stays FP64, and its RK
 * accumulation, the pressure recovery and the CT curl run in float-float
 * (hi + lo FP32 pairs, ~48 bits) on the FP32 pipe.  MLAU_FP32_SPLIT_F64: the
 * same FP32 parts, with those three steps in FP64 arithmetic instead (3D). */
enum { MLAU_FP64 = 0, MLAU_FP32_SPLIT = 1, MLAU_FP32_SPLIT_F64 = 2 };
/* 1D boundaries. */
enum { MLAU_BC1D_OPEN = 0, MLAU_BC1D_PERIODIC = 1 };
/* Eigen-system of the characteristic projection where the largest sonic
 * Mach^2 of the face's three central cells is at least 1 (elsewhere the
 * Alfven + entropy system): the drivers' full 7-wave system
 * (mhd_c_reconst, mhd_eigen.h:455-530) or Miyoshi's fast + Alfven system
 * (mhd_m_reconst, mhd_eigen.h:532-607), the header's alternative. */
enum { MLAU_EIGEN_FULL = 0, MLAU_EIGEN_MIYOSHI = 1 };

/* Output file formats (mlau_sim_outdat). */
enum { MLAU_OUT_F64 = 0, MLAU_OUT_F32_RANK = 1 };

/* ---------------------------------------------------------------------- */
/* 1. Drop-in drivers                                                      */
/* ---------------------------------------------------------------------- */

/* Replaces mhd_fd_ct_3d (3D/MPI/OTvortex/mhd_fd_ct_3d.c:99-103, prototype
 * 3D/MPI/OTvortex/myfunc.h:48-52, caller 3D/MPI/OTvortex/main.cpp:48-50).
 * Single GPU: mpi_numx = mpi_numy = mpi_numz = 1 and mpi_rank = 0 are
 * required.  The problem's tables dnxs / dnys / dnzs apply (each axis all
 * zero or all nonzero; non-periodic ones with the FP64 form). */
void mhd_fd_ct_3d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, double dz, int nx,
                  int ny, int nz, int xoff, int yoff, int zoff, double gamma, int mpi_rank,
                  int mpi_numx, int mpi_numy, int mpi_numz);

/* Replaces the serial mhd_fd_ct_2d (2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-94,
 * caller 2D/SERIAL/OTvortex/main.cpp:30-31).  The problem's boundary tables
 * dnxs / dnys (periodic, Dirichlet or Neumann per array and axis) apply. */
void mhd_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma);

/* Replaces the MPI form of mhd_fd_ct_2d (2D/MPI/OTvortex/mhd_fd_ct_2d.c:95-99,
 * caller 2D/MPI/OTvortex/main.cpp:48-50; the same driver serves
 * 2D/MPI/KHI with reflecting y walls); C++ callers reach it under the
 * reference's overloaded name.  mpi_numx = mpi_numy = 1 required; each
 * axis's table entries must be all zero or all nonzero. */
void mhd_fd_ct_2d_mpi(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                      double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                      int xoff, int yoff, double gamma, int mpi_rank, int mpi_numx,
                      int mpi_numy);

/* Replaces mhd_fd4c_1d (1D/SERIAL/shock/mhd_fd4c_1d.c:60-63, caller
 * 1D/SERIAL/shock/main.cpp:166-167).  Boundary: mlau_set_bc_1d (default
 * open, as the shock driver; periodic as 1D/SERIAL/wave). */
void mhd_fd4c_1d(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                 double *bz, double bx, double dt, double dx, int nx, int xoff, double gamma);

/* Replace the MRX problem's resistive diffusion of the CT field (uniform
 * resistivity eta0; energy updated by the resistive Poynting flux) and its
 * viscous term (uniform kinematic viscosity nu0), 2D/MPI/MRX/myfunc.h:12-22,
 * 2D/MPI/MRX/mhd_fd_ct_2d.c:726-1174, caller 2D/MPI/MRX/main.cpp:52-68.
 * Each is an explicit SSP-RK update with the 2D drop-in's scheme (odr, nrk)
 * and the problem's tables (each axis all zero or all nonzero); the MRX
 * hyperbolic step itself is mhd_fd_ct_2d_mpi with reconstruction code 5.
 * mpi_numx = mpi_numy = 1 required. */
void diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0, double dt,
                    double dx, double dy, int nx, int ny, int xoff, int yoff, double gamma,
                    int mpi_rank, int mpi_numx, int mpi_numy);
void ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en, double nu0,
                   double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                   double gamma, int mpi_rank, int mpi_numx, int mpi_numy);
/* Replaces the MRX problem's anisotropic heat conduction along B (conductivity
 * kk0; 2D/MPI/MRX/myfunc.h:34-39, mhd_fd_ct_2d.c:1176-1456): Crank-Nicolson
 * in p/rho solved by six-colour Gauss-Seidel sweeps (at most 2048, the
 * reference's CMAX).  Like the reference, it halts the process (messages on
 * stdout, exit status 255) when the sweeps do not converge; the handle API
 * returns MLAU_ERR_CONVERGE instead. */
void t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                  double *en, const double *bx, const double *by, const double *bz, double kk0,
                  double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                  double gamma, int mpi_rank, int mpi_numx, int mpi_numy);

/* The reference fixes the spatial order (ODR), Runge-Kutta order (R_K) and
 * Riemann solver (func_flux=) at compile time in each driver copy
 * (mhd_fd_ct_3d.c:25-27,131-138).  The drop-in drivers read them from here
 * (dim = 1, 2 or 3).  Defaults are those of the shipped driver files:
 * 3D and 2D odr=2, nrk=3, LHLLD; 1D odr=1, nrk=2, LHLLD.  The environment
 * variables MLAU_ODR, MLAU_RK and MLAU_FLUX (mlau|lhlld|hlld|roe) override
 * the defaults at first use.
 * Reconstruction codes (odr): 1-4 as the drivers' ODR (1 first order,
 * 2 MUSCL minmod, 3 WCNS3, 4 WCNS4); 5 and 6 are second-order MUSCL with the
 * MC limiter (include/interp.h:45-51, the limiter of
 * 2D/MPI/MRX/mhd_fd_ct_2d.c:107) and the Koren limiter (interp.h:61-72), the
 * calc_flr alternatives the headers ship; everything else follows ODR 2. */
int mlau_set_scheme(int dim, int odr, int flux, int nrk);
/* Eigen-system of the drop-in drivers (MLAU_EIGEN_*; default full, or the
 * environment variable MLAU_EIGEN=miyoshi at first use): the reference's
 * driver with its mhd_c_reconst call replaced by mhd_m_reconst. */
int mlau_set_eigen(int dim, int eig);
int mlau_set_bc_1d(int bc);
/* The boundary tables the drop-in drivers see: the problem program's own
 * dnxs / dnys / dnzs when it defines them (the library's weak all-zero
 * tables give way to them at load time), else zeros. */
int mlau_boundary_tables(int *dnx, int *dny, int *dnz);
/* Arithmetic of the drop-in 3D driver: MLAU_FP64 (default; the reference's
 * arithmetic bit for bit), MLAU_FP32_SPLIT or MLAU_FP32_SPLIT_F64. */
int mlau_set_precision(int dim, int precision);
/* Free the device memory cached by the drop-in drivers (it is kept between
 * calls so that a time loop does not reallocate every step). */
void mlau_release_dropin(void);
const char *mlau_last_error(void);
void mlau_clear_error(void);

/* ---------------------------------------------------------------------- */
/* 2. Device-resident handle API                                           */
/* ---------------------------------------------------------------------- */
typedef struct mlau_sim mlau_sim;

/* dim 3: nx,ny,nz padded sizes; dim 2: nz = 1; dim 1: ny = nz = 1.
 * xoff/yoff/zoff: ghost depth (>= 4, as the reference fixes it).  Interior width
 * must be at least the ghost depth.  odr 1..6, flux MLAU_FLUX_*, nrk 1..3,
 * precision MLAU_FP64, or MLAU_FP32_SPLIT / MLAU_FP32_SPLIT_F64 (3D only). */
int mlau_sim_create(mlau_sim **out, int dim, int nx, int ny, int nz, int xoff, int yoff,
                    int zoff, double dx, double dy, double dz, double gamma, int odr, int flux,
                    int nrk, int precision);
int mlau_sim_destroy(mlau_sim *sim);
/* Host arrays in the order (ro, mx, my, mz, en, bx, by, bz); in 1D bx is
 * unused (set it with mlau_sim_set_bx_1d).  A null entry is skipped. */
int mlau_sim_upload(mlau_sim *sim, const double *const *host8);
int mlau_sim_download(mlau_sim *sim, double *const *host8);
int mlau_sim_set_bx_1d(mlau_sim *sim, double bx);
int mlau_sim_set_bc_1d(mlau_sim *sim, int bc);
/* Boundary tables of a 3D simulation (dnxs / dnys / dnzs of the problem,
 * 3D/MPI/OTvortex/global.hpp:22-24; order ro mx my mz en bx by bz; 0
 * periodic, -1 Dirichlet, +1 Neumann mirror as mpi_xbc3d / _ybc3d / _zbc3d,
 * 3D/MPI/OTvortex/boundary.c:227-309, at the driver's three fill sites).
 * Each axis's entries all zero or all nonzero; non-periodic tables need the
 * FP64 form.  All zero (the default) is periodic. */
int mlau_sim_set_bc_3d(mlau_sim *sim, const int *dnx, const int *dny, const int *dnz);
/* Eigen-system where Mach^2 >= 1 (MLAU_EIGEN_*; FP64 simulations). */
int mlau_sim_set_eigen(mlau_sim *sim, int eig);
/* Boundary tables of a 2D FP64 simulation: dnx[8] / dny[8] as the problem's
 * dnxs / dnys (2D/MPI/KHI/global.hpp:21-22; order ro mx my mz en bx by bz;
 * 0 periodic, -1 Dirichlet, +1 Neumann mirror), each array's ghosts filled by
 * its own entry as bc2d (2D/SERIAL/OTvortex/boundary.c:18-74), including the
 * shock-sensor and cell-B fills inside the step.  All zero (the default) is
 * periodic.  The drop-in 2D drivers apply the problem's own tables. */
int mlau_sim_set_bc_2d(mlau_sim *sim, const int *dnx, const int *dny);
/* The MRX operators on a device-resident 2D FP64 state (the simulation's
 * odr and nrk, its tables; each axis's entries all zero or all nonzero):
 * resistive diffusion of B with energy, and viscosity of the velocity with
 * energy.  Enqueued on the simulation's stream like a step. */
int mlau_sim_resistive_2d(mlau_sim *sim, double eta0, double dt);
int mlau_sim_viscous_2d(mlau_sim *sim, double nu0, double dt);
/* Anisotropic heat conduction along B over dt (energy updated; 2D FP64, same
 * table rule).  *sweeps (may be NULL) receives the Gauss-Seidel sweep count;
 * MLAU_ERR_CONVERGE after 2048 sweeps without convergence, with the energy
 * as the reference leaves it.  Synchronises the simulation's stream once per
 * 8 sweeps to test convergence. */
int mlau_sim_conduction_2d(mlau_sim *sim, double kk0, double dt, int *sweeps);
/* The RMI problem's inflow through the upper boundary (inj_ro,
 * 2D/MPI/RMI/inj_ro.hpp:1-58, called before each step, main.cpp:48-54):
 * rows [ny-yoff, ny) take density ro3 (+ dro3 (2u - 1) with noise[k] = u,
 * the yoff*nx draws random()/RAND_MAX in row order, or no perturbation when
 * noise is NULL), velocity (0, vy1 - vref, 0), B (bx1, by1, bz1) - By on the
 * face row ny-yoff kept - and pressure pr1; then the main loop's periodic
 * exchange of the 8 arrays along axes whose table entry 0 is zero.  2D FP64;
 * noise is a host array, copied before the call returns. */
int mlau_sim_inject_2d(mlau_sim *sim, double ro3, double dro3, double vy1, double bx1,
                       double by1, double bz1, double pr1, double vref, const double *noise);
/* nsteps full RK steps with fixed dt, enqueued on the simulation's stream. */
int mlau_sim_step(mlau_sim *sim, double dt, int nsteps);
/* CFL time step (3D/MPI/OTvortex/cflcheck.hpp:1-39, 2D cflcheck.hpp,
 * 1D/SERIAL/shock/main.cpp:113-128): dt = cfl*dr/max(vfast, max fast speed),
 * dt_old kept when that maximum is not finite.  Synchronizes the stream. */
int mlau_sim_cfl(mlau_sim *sim, double cfl, double dr, double vfast, double dt_old,
                 double *dt_out, double *vmax_out);
int mlau_sim_sync(mlau_sim *sim);
/* cudaStream_t of the simulation, for callers that time or order work. */
void *mlau_sim_stream(mlau_sim *sim);
/* Device pointer of variable v (same order as upload). */
int mlau_sim_device_ptr(mlau_sim *sim, int v, double **ptr);
/* Per-kernel CUDA-event timing (off by default).  kind: 0 prim, 1 aux,
 * 2 reconstruction, 3 flux, 4 emf, 5 update, 6 copy, 7 cfl, 8 split sweep,
 * 9 split prep, 10 split update. */
int mlau_sim_set_timing(mlau_sim *sim, int on);
int mlau_sim_timing(mlau_sim *sim, int kind, long *count, double *total_ms);
/* Device bytes held by the simulation. */
long long mlau_sim_device_bytes(mlau_sim *sim);
/* Number of kernel launches one mlau_sim_step(sim, dt, 1) issues. */
int mlau_sim_launches_per_step(mlau_sim *sim);
/* Enqueue nsteps steps between two CUDA events recorded on the simulation's
 * stream and return the elapsed device time in milliseconds. */
int mlau_sim_time_steps(mlau_sim *sim, double dt, int nsteps, double *ms);

/* Checkpoint and output files in the reference's formats, written from and
 * read into the device-resident state (2D/3D checkpoints; outputs in all
 * dimensions), so runs restart across the reference and this library and the
 * reference's readers take its output.
 * Checkpoint - replaces bkup_save / bkup_load (3D/MPI/OTvortex/bkup.hpp:4-76,
 * 2D/MPI/OTvortex/bkup.hpp): <dir>/bkup_stamp.dat ("%d %d\n" step, output count) and
 * bkup_time.dat (3 doubles: time, dt, next output time) from rank 0, and
 * bkup_data_%05d.dat (FP64 ro, mx, my, mz, bx, by, bz, en, ghosts included)
 * per rank.  mlau_sim_bkup_load returns 1 and changes nothing when there is
 * no stamp file (the reference's fresh start). */
int mlau_sim_bkup_save(mlau_sim *sim, const char *dir, int n, int cnt, double tim, double dt,
                       double trec, int rank);
int mlau_sim_bkup_load(mlau_sim *sim, const char *dir, int *n, int *cnt, double *tim, double *dt,
                       double *trec, int rank);
/* Output - replaces the state part of dataio (3D/MPI/OTvortex/dataio.hpp:62-80,
 * MLAU_OUT_F32_RANK: outdat_%05d_%05d.dat, FP32 ro mx my mz en bx by bz per
 * rank; 2D/SERIAL/OTvortex/dataio.hpp:28-38, MLAU_OUT_F64: outdat_%05d.dat,
 * FP64; in 1D the 1D driver's outdat_%05d.dat of ro mx my mz en by bz,
 * 1D/SERIAL/shock/main.cpp:171-184).  FP32 conversion happens on the device. */
int mlau_sim_outdat(mlau_sim *sim, const char *dir, int cnt, int rank, int format);
/* The run's metadata as the same routines write them: first != 0 writes
 * params.dat and offsets.dat (1D: params "bx gamma", xoff.dat) and starts
 * t.dat; otherwise appends tim to t.dat.  Grid coordinate files are the
 * problem's own and are not written. */
int mlau_outdat_meta(const char *dir, int dim, int first, double tim, double gamma, double bx,
                     int xoff, int yoff, int zoff);

/* ---------------------------------------------------------------------- */
/* 5. Batched 2D engine                                                    */
/* ---------------------------------------------------------------------- */
/* Many independent 2D instances (the 2D driver's scheme,
 * 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c, RK3) in slots of one engine, each with
 * its own grid size (nx, ny padded), cell sizes, gamma, Riemann solver, CFL
 * number and end time.  One persistent cooperative kernel per step walks a
 * per-instance tile table; each instance takes its own CFL dt every step
 * (clipped to land on its end time) and retires when it gets there.
 * Instances are periodic unless mlau_batch_set_bc gives them tables.
 * Precision per engine: MLAU_FP64 (each instance bit-identical to
 * mhd_fd_ct_2d, with its boundary tables) or MLAU_FP32_SPLIT.  Instances join and leave between runs
 * (continuous batching).  No reference counterpart (the reference runs one
 * problem per process). */
typedef struct mlau_batch mlau_batch;
/* Engine with pools of capacity_cells cells and max_inst slots. */
int mlau_batch_open(mlau_batch **out, int precision, long long capacity_cells, int max_inst,
                    int off, int odr);
/* Admit an instance with its initial state (8 host arrays); MLAU_ERR_NOMEM
 * when no slot or pool space is free (retry after a removal). */
int mlau_batch_add(mlau_batch *b, int nx, int ny, double dx, double dy, double gamma, int flux,
                   double cfl, double t_end, const double *const *host8, int *slot);
int mlau_batch_remove(mlau_batch *b, int slot);
/* FP32-split engine sized for and filled with ninst instances (zero state;
 * upload each). */
int mlau_batch_create(mlau_batch **out, int ninst, const int *nx, const int *ny, int off,
                      const double *dx, const double *dy, const double *gamma, const int *flux,
                      const double *cfl, const double *t_end, int odr);
int mlau_batch_destroy(mlau_batch *b);
int mlau_batch_upload(mlau_batch *b, int inst, const double *const *host8);
int mlau_batch_download(mlau_batch *b, int inst, double *const *host8);
/* dt > 0: fixed time step for that instance instead of its CFL step. */
int mlau_batch_set_fixed_dt(mlau_batch *b, int inst, double dt);
/* Boundary tables of a 2D instance - the problem's dnxs / dnys
 * (2D/SERIAL/OTvortex/global.hpp:22-29, 0 periodic, -1 Dirichlet, +1 Neumann
 * per variable ro mx my mz en bx by bz), applied as mhd_fd_ct_2d applies
 * them (bc2d, 2D/SERIAL/OTvortex/boundary.c:18-74); all zero (the default) is
 * periodic.  Set between runs, before the instance's next step. */
int mlau_batch_set_bc(mlau_batch *b, int inst, const int *dnx, const int *dny);
/* Tile shape TW x TH (= 256 threads, TW a multiple of 16). */
int mlau_batch_set_tile(mlau_batch *b, int tw, int th);
/* Grid of the persistent step kernel: nblocks co-resident blocks (clamped to
 * what fits, returned), or 0 for all that fit.  Several engines stepping at
 * once on one GPU each take a share, so that their grids are co-resident
 * together.  mlau_batch_max_grid: the blocks that fit at the current tile. */
int mlau_batch_set_grid(mlau_batch *b, int nblocks);
int mlau_batch_max_grid(mlau_batch *b);
/* Time `steps` steps per candidate tile shape on the live state and keep the
 * fastest (the tuning steps advance the simulation). */
int mlau_batch_autotune(mlau_batch *b, int steps, int *tw, int *th, double *ms);
/* Advance until every instance has retired or max_steps steps were taken;
 * steps_per_graph > 0 replays a captured CUDA graph of that many steps. */
int mlau_batch_run(mlau_batch *b, int max_steps, int steps_per_graph, int *active_left,
                   double *ms);
int mlau_batch_info(mlau_batch *b, int inst, double *t, int *steps, int *active);
/* MLAU_ERR_STATE when the instance retired early because its state held a NaN
 * or a non-positive density or pressure (the other instances carry on). */
int mlau_batch_status(mlau_batch *b, int inst);
long long mlau_batch_cells(mlau_batch *b);
long long mlau_batch_device_bytes(mlau_batch *b);
/* Kernel launches issued so far (graph replays counted per step). */
long long mlau_batch_launches(mlau_batch *b);
/* 1D engine (FP64): independent 1D problems, each stepped bit-identically to
 * mhd_fd4c_1d (1D/SERIAL/shock/mhd_fd4c_1d.c:60-271; open boundary
 * openbc1d_mhd.c:21-175, or periodic).  Each instance's dt is fixed once from
 * its initial state, dt = cfl*dx/max(1, max|vx|+cf), as the 1D driver's main
 * does (1D/SERIAL/shock/main.cpp:113-128), unless mlau_batch_set_fixed_dt
 * gives one; it retires after the step that reaches t_end (the last step is
 * not clipped).  The other mlau_batch_* calls apply; tiles are 64, 128 or
 * 256 cells by 1. */
int mlau_batch1d_open(mlau_batch **out, long long capacity_cells, int max_inst, int off, int odr);
/* host8: slots 0 ro, 1 mx, 2 my, 3 mz, 4 en, 6 by, 7 bz (slot 5 unused). */
int mlau_batch1d_add(mlau_batch *b, int nx, double dx, double bx, double gamma, int flux, int nrk,
                     int bc, double cfl, double t_end, const double *const *host8, int *slot);

/* ---------------------------------------------------------------------- */
/* 4. Allocation-free 1D step                                              */
/* ---------------------------------------------------------------------- */
/* No counterpart in the reference (its drivers malloc scratch on every call).
 * For callers that cannot allocate device memory - code inside a host
 * framework that owns every device allocation, or a service holding a fixed
 * device-memory budget: one 1D step like mhd_fd4c_1d (odr/flux/nrk/bc as in
 * the handle API) on arrays the caller already holds in device-accessible
 * memory, updated in place, with no allocation.  Its scratch is one static
 * device array of 32*(MLAU_NOALLOC_1D_MAX_NX+1) doubles (4.2 MB) that every
 * GPU loading the library holds until the process exits; nx above
 * MLAU_NOALLOC_1D_MAX_NX is rejected.  The first call on a device resolves
 * that array's device address (cudaGetSymbolAddress) - make it before any
 * stream capture.  The work is enqueued on `stream` (NULL: the legacy default
 * stream) and the call returns without waiting.  All calls share the one
 * array: calls that overlap on the GPU (different streams, no ordering) race
 * on it.  Nothing in the scratch needs clearing between calls: every element
 * a step reads is written earlier in the same step (ghost depth xoff >= 4, as
 * the reference fixes it; smaller depths are rejected).  The resolved address
 * is cached per device for the life of the process, so cudaDeviceReset is not
 * supported once this entry point has run on that device. */
#define MLAU_NOALLOC_1D_MAX_NX 16392
int mlau_fd4c_1d_noalloc(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                         double *bz, double bx, double dt, double dx, int nx, int xoff,
                         double gamma, int odr, int flux, int nrk, int bc, void *stream);

/* ---------------------------------------------------------------------- */
/* 3. Measurement helpers                                                  */
/* ---------------------------------------------------------------------- */
/* FMA throughput of the current device in flop/s (2 flops per FMA), FP64 and
 * FP32: the pipe rates that bound the plain and the split step. */
int mlau_measure_fma_peaks(double *fp64_flops, double *fp32_flops);
/* Page-lock (pin) / release caller-owned host memory, so that the drop-in
 * drivers' host<->device copies run at full link speed. */
int mlau_pin_host(void *ptr, long long bytes);
int mlau_unpin_host(void *ptr);
/* Select the CUDA device used by this host thread's later calls. */
int mlau_set_device(int device);
/* PCI bus id of a device ("domain:bus:device.function"), e.g. to find the
 * host CPUs and memory node next to it, where host arrays that cross the
 * link every step belong. */
int mlau_device_pci_bus_id(int device, char *buf, int len);

#ifdef __cplusplus
}
#endif
#endif
