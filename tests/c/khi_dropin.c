/* A problem program in the shape of 2D/MPI/KHI: it defines the boundary
 * tables (2D/MPI/KHI/global.hpp:21-22) and calls the reference-named MPI 2D
 * driver for one rank.  Usage: khi_dropin in.bin out.bin nx ny dt dx dy gamma
 * nsteps (in/out: ro mx my mz en bx by bz, FP64, nx*ny each). */
#include <stdio.h>
#include <stdlib.h>

int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnys[8] = {+1, +1, -1, +1, +1, +1, -1, +1};

void mhd_fd_ct_2d_mpi(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                      double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                      int xoff, int yoff, double gamma, int mpi_rank, int mpi_numx, int mpi_numy);
const char *mlau_last_error(void);

int main(int argc, char **argv)
{
    if (argc != 10) return 2;
    const int nx = atoi(argv[3]), ny = atoi(argv[4]), nsteps = atoi(argv[9]);
    const double dt = atof(argv[5]), dx = atof(argv[6]), dy = atof(argv[7]), gamma = atof(argv[8]);
    const size_t n = (size_t)nx * ny;
    double *a = malloc(sizeof(double) * 8 * n);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(a, sizeof(double), 8 * n, f) != 8 * n) return 3;
    fclose(f);
    for (int k = 0; k < nsteps; k++)
        mhd_fd_ct_2d_mpi(a, a + n, a + 2 * n, a + 3 * n, a + 4 * n, a + 5 * n, a + 6 * n, a + 7 * n,
                         dt, dx, dy, nx, ny, 4, 4, gamma, 0, 1, 1);
    if (mlau_last_error()[0]) {
        fprintf(stderr, "%s\n", mlau_last_error());
        return 4;
    }
    f = fopen(argv[2], "wb");
    if (!f || fwrite(a, sizeof(double), 8 * n, f) != 8 * n) return 5;
    fclose(f);
    free(a);
    return 0;
}
