// A problem program in the shape of 2D/MPI/MRX, compiled as C++ like the
// reference's: it defines the MRX boundary tables (2D/MPI/MRX/global.hpp:22-23),
// declares the driver-file functions with the reference's prototypes
// (2D/MPI/MRX/myfunc.h:6-39, C++ linkage) and runs the main loop's sequence
// (main.cpp:48-68) for one rank: step, resistive diffusion, viscosity, heat
// conduction.  Usage: mrx_dropin in.bin out.bin nx ny dt dx dy gamma eta0 nu0
// kk0 nloop (in/out: ro mx my mz en bx by bz, FP64, nx*ny each).
#include <cstdio>
#include <cstdlib>
#include <vector>

int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnys[8] = {+1, +1, -1, +1, +1, +1, -1, +1};

void mhd_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma, int mpi_rank, int mpi_numx, int mpi_numy);
void diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0, double dt,
                    double dx, double dy, int nx, int ny, int xoff, int yoff, double gamma,
                    int mpi_rank, int mpi_numx, int mpi_numy);
void ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en, double nu0,
                   double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                   double gamma, int mpi_rank, int mpi_numx, int mpi_numy);
void t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                  double *en, const double *bx, const double *by, const double *bz, double kk0,
                  double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                  double gamma, int mpi_rank, int mpi_numx, int mpi_numy);
extern "C" int mlau_set_scheme(int dim, int odr, int flux, int nrk);
extern "C" const char *mlau_last_error(void);

int main(int argc, char **argv)
{
    if (argc != 13) return 2;
    const int nx = atoi(argv[3]), ny = atoi(argv[4]), nloop = atoi(argv[12]);
    const double dt = atof(argv[5]), dx = atof(argv[6]), dy = atof(argv[7]), gam = atof(argv[8]);
    const double eta0 = atof(argv[9]), nu0 = atof(argv[10]), kk0 = atof(argv[11]);
    const size_t n = (size_t)nx * ny;
    std::vector<double> a(8 * n);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(a.data(), sizeof(double), 8 * n, f) != 8 * n) return 3;
    fclose(f);
    double *ro = &a[0], *mx = ro + n, *my = mx + n, *mz = my + n, *en = mz + n, *bx = en + n,
           *by = bx + n, *bz = by + n;
    mlau_set_scheme(2, 5, 1, 3);  // the MRX driver file: ODR 2 with the MC limiter, LHLLD, RK3
    for (int k = 0; k < nloop; k++) {
        mhd_fd_ct_2d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, 4, 4, gam, 0, 1, 1);
        if (eta0 != 0) diff_ctfield_e(en, bx, by, bz, eta0, dt, dx, dy, nx, ny, 4, 4, gam, 0, 1, 1);
        if (nu0 != 0) ns_viscous_2d(ro, mx, my, mz, en, nu0, dt, dx, dy, nx, ny, 4, 4, gam, 0, 1, 1);
        if (kk0 != 0)
            t_conduction(ro, mx, my, mz, en, bx, by, bz, kk0, dt, dx, dy, nx, ny, 4, 4, gam, 0, 1, 1);
    }
    if (mlau_last_error()[0]) {
        fprintf(stderr, "%s\n", mlau_last_error());
        return 4;
    }
    f = fopen(argv[2], "wb");
    if (!f || fwrite(a.data(), sizeof(double), 8 * n, f) != 8 * n) return 5;
    fclose(f);
    return 0;
}
