// The reference compiles its drivers as C++ (Makefile.inc: mpic++/g++ on .c
// files), so problem programs reference them by their C++ (mangled) names.
// These definitions give the library those exact symbols, forwarding to the
// C-linkage entry points of api.cu, so an unmodified main.cpp links against
// libmlau_gb300.so in place of the driver object file.
//
// A C++ function cannot share a name with a C-linkage declaration in one
// translation unit, so the C entry points are declared here under other
// identifiers bound to their symbols with asm labels.

extern "C" void mlau_c_fd_ct_3d(double *, double *, double *, double *, double *, double *,
                                double *, double *, double, double, double, double, int, int,
                                int, int, int, int, double, int, int, int, int)
    __asm__("mhd_fd_ct_3d");
extern "C" void mlau_c_fd_ct_2d(double *, double *, double *, double *, double *, double *,
                                double *, double *, double, double, double, int, int, int, int,
                                double) __asm__("mhd_fd_ct_2d");
extern "C" void mlau_c_fd_ct_2d_mpi(double *, double *, double *, double *, double *, double *,
                                    double *, double *, double, double, double, int, int, int,
                                    int, double, int, int, int) __asm__("mhd_fd_ct_2d_mpi");
extern "C" void mlau_c_diff_ctfield_e(double *, double *, double *, double *, double, double,
                                      double, double, int, int, int, int, double, int, int, int)
    __asm__("diff_ctfield_e");
extern "C" void mlau_c_ns_viscous_2d(const double *, double *, double *, double *, double *,
                                     double, double, double, double, int, int, int, int, double,
                                     int, int, int) __asm__("ns_viscous_2d");
extern "C" void mlau_c_t_conduction(const double *, const double *, const double *,
                                    const double *, double *, const double *, const double *,
                                    const double *, double, double, double, double, int, int,
                                    int, int, double, int, int, int) __asm__("t_conduction");
extern "C" void mlau_c_fd4c_1d(double *, double *, double *, double *, double *, double *,
                               double *, double, double, double, int, int, double)
    __asm__("mhd_fd4c_1d");

// 3D/MPI/OTvortex/myfunc.h:48-52
void mhd_fd_ct_3d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, double dz, int nx,
                  int ny, int nz, int xoff, int yoff, int zoff, double gamma, int mpi_rank,
                  int mpi_numx, int mpi_numy, int mpi_numz)
{
    mlau_c_fd_ct_3d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, dz, nx, ny, nz, xoff, yoff, zoff,
                    gamma, mpi_rank, mpi_numx, mpi_numy, mpi_numz);
}

// 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-94
void mhd_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma)
{
    mlau_c_fd_ct_2d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma);
}

// 2D/MPI/OTvortex/mhd_fd_ct_2d.c:95-99 (the MPI overload)
void mhd_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma, int mpi_rank, int mpi_numx, int mpi_numy)
{
    mlau_c_fd_ct_2d_mpi(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma,
                        mpi_rank, mpi_numx, mpi_numy);
}

// 2D/MPI/MRX/myfunc.h:12-16
void diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0, double dt,
                    double dx, double dy, int nx, int ny, int xoff, int yoff, double gamma,
                    int mpi_rank, int mpi_numx, int mpi_numy)
{
    mlau_c_diff_ctfield_e(en, bx, by, bz, eta0, dt, dx, dy, nx, ny, xoff, yoff, gamma, mpi_rank,
                          mpi_numx, mpi_numy);
}

// 2D/MPI/MRX/myfunc.h:17-22
void ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en, double nu0,
                   double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                   double gamma, int mpi_rank, int mpi_numx, int mpi_numy)
{
    mlau_c_ns_viscous_2d(ro, mx, my, mz, en, nu0, dt, dx, dy, nx, ny, xoff, yoff, gamma, mpi_rank,
                         mpi_numx, mpi_numy);
}

// 2D/MPI/MRX/myfunc.h:34-39
void t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                  double *en, const double *bx, const double *by, const double *bz, double kk0,
                  double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                  double gamma, int mpi_rank, int mpi_numx, int mpi_numy)
{
    mlau_c_t_conduction(ro, mx, my, mz, en, bx, by, bz, kk0, dt, dx, dy, nx, ny, xoff, yoff, gamma,
                        mpi_rank, mpi_numx, mpi_numy);
}

// 1D/SERIAL/shock/mhd_fd4c_1d.c:60-63
void mhd_fd4c_1d(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                 double *bz, double bx, double dt, double dx, int nx, int xoff, double gamma)
{
    mlau_c_fd4c_1d(ro, mx, my, mz, en, by, bz, bx, dt, dx, nx, xoff, gamma);
}

// Boundary tables of the problem program (3D/MPI/OTvortex/global.hpp:22-29,
// 2D/MPI/KHI/global.hpp:21-22; order ro mx my mz en bx by bz, 0 periodic).
// Defined here, all zero, as weak symbols with default visibility: a problem
// program that defines its own tables (every reference problem does, in
// global.hpp) overrides these when it is loaded - the linker exports an
// executable's definition of a symbol that a linked library also defines.
extern "C" {
__attribute__((weak, visibility("default"))) int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
__attribute__((weak, visibility("default"))) int dnys[8] = {0, 0, 0, 0, 0, 0, 0, 0};
__attribute__((weak, visibility("default"))) int dnzs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
}
