/* Reference-oracle harness.  TEST INFRASTRUCTURE ONLY.
 *
 * Compiled by oracle/build.py together with sed-patched copies of the
 * reference's own step driver and boundary sources (read from the reference
 * tree, written only into oracle/_ref/), one shared library per scheme
 * variant.  It defines the problem-side boundary tables the drivers read
 * (3D/MPI/OTvortex/global.hpp:22-29: all periodic) and exports the drivers
 * under C names with the MPI arguments fixed to a single rank. */
#ifndef REF_DIM
#error "REF_DIM must be 1, 2 or 3"
#endif

int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnys[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnzs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int stxs[8] = {0, 0, 0, 0, 0, 1, 0, 0};
int stys[8] = {0, 0, 0, 0, 0, 0, 1, 0};
int stzs[8] = {0, 0, 0, 0, 0, 0, 0, 1};

#if REF_DIM == 3
void mhd_fd_ct_3d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, double dz, int nx,
                  int ny, int nz, int xoff, int yoff, int zoff, double gamma, int mpi_rank,
                  int mpi_numx, int mpi_numy, int mpi_numz);
extern "C" void ref_step(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                         double *by, double *bz, double dt, double dx, double dy, double dz,
                         int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma)
{
    mhd_fd_ct_3d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, dz, nx, ny, nz, xoff, yoff, zoff,
                 gamma, 0, 1, 1, 1);
}
#elif REF_DIM == 2
void mhd_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma);
extern "C" void ref_step(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                         double *by, double *bz, double dt, double dx, double dy, double dz,
                         int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma)
{
    (void)dz; (void)nz; (void)zoff;
    mhd_fd_ct_2d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma);
}
#else
void mhd_fd4c_1d(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                 double *bz, double bx, double dt, double dx, int nx, int xoff, double gamma);
extern "C" void ref_step_1d(double *ro, double *mx, double *my, double *mz, double *en,
                            double *by, double *bz, double bx, double dt, double dx, int nx,
                            int xoff, double gamma)
{
    mhd_fd4c_1d(ro, mx, my, mz, en, by, bz, bx, dt, dx, nx, xoff, gamma);
}
#endif
