// Byte-format oracle for the checkpoint and output files: compiles the
// reference's own checkpoint (3D/MPI/OTvortex/bkup.hpp) and output routines
// (3D/MPI/OTvortex/dataio.hpp - FP32 per rank; 2D/SERIAL/OTvortex/dataio.hpp -
// FP64 serial) against globals defined here, and exports them with C
// linkage.  TEST INFRASTRUCTURE ONLY: built by oracle/build.py::build_ref_io
// from the reference tree (include path = the reference root); never part of
// the library.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace r3 {
char fildir[512];
int nx, ny, nz, xoff, yoff, zoff, mpi_numx = 1, mpi_numy = 1;
double gam;
double *x, *y, *z, *ro, *mx, *my, *mz, *en, *bx, *by, *bz;
#include "3D/MPI/OTvortex/bkup.hpp"
#include "3D/MPI/OTvortex/dataio.hpp"
}  // namespace r3

namespace r2 {
char fildir[512];
int nx, ny, xoff, yoff;
double gam;
double *ro, *mx, *my, *mz, *en, *bx, *by, *bz;
#include "2D/SERIAL/OTvortex/dataio.hpp"
}  // namespace r2

extern "C" {

// st: ro, mx, my, mz, en, bx, by, bz (the library's order)
void ref_bkup_save(const char *dir, int n, int cnt, double tim, double dt, double trec, int nall,
                   int rank, double **st)
{
    std::snprintf(r3::fildir, sizeof(r3::fildir), "%s", dir);
    r3::ro = st[0]; r3::mx = st[1]; r3::my = st[2]; r3::mz = st[3];
    r3::en = st[4]; r3::bx = st[5]; r3::by = st[6]; r3::bz = st[7];
    r3::bkup_save(n, cnt, tim, dt, trec, nall, rank);
}

void ref_bkup_load(const char *dir, int *n, int *cnt, double *tim, double *dt, double *trec,
                   int nall, int rank, double **st)
{
    std::snprintf(r3::fildir, sizeof(r3::fildir), "%s", dir);
    r3::ro = st[0]; r3::mx = st[1]; r3::my = st[2]; r3::mz = st[3];
    r3::en = st[4]; r3::bx = st[5]; r3::by = st[6]; r3::bz = st[7];
    r3::bkup_load(n, cnt, tim, dt, trec, nall, rank);
}

void ref_dataio_3d(const char *dir, int n, int cnt, double tim, int rank, int nx, int ny, int nz,
                   int xoff, int yoff, int zoff, double gam, double **st, double *x, double *y,
                   double *z)
{
    std::snprintf(r3::fildir, sizeof(r3::fildir), "%s", dir);
    r3::nx = nx; r3::ny = ny; r3::nz = nz;
    r3::xoff = xoff; r3::yoff = yoff; r3::zoff = zoff;
    r3::gam = gam;
    r3::x = x; r3::y = y; r3::z = z;
    r3::ro = st[0]; r3::mx = st[1]; r3::my = st[2]; r3::mz = st[3];
    r3::en = st[4]; r3::bx = st[5]; r3::by = st[6]; r3::bz = st[7];
    r3::dataio(n, cnt, tim, rank);
}

void ref_dataio_2d(const char *dir, int n, int cnt, double tim, int nx, int ny, int xoff,
                   int yoff, double gam, double **st)
{
    std::snprintf(r2::fildir, sizeof(r2::fildir), "%s", dir);
    r2::nx = nx; r2::ny = ny; r2::xoff = xoff; r2::yoff = yoff;
    r2::gam = gam;
    r2::ro = st[0]; r2::mx = st[1]; r2::my = st[2]; r2::mz = st[3];
    r2::en = st[4]; r2::bx = st[5]; r2::by = st[6]; r2::bz = st[7];
    r2::dataio(n, cnt, tim);
}

}  // extern "C"
