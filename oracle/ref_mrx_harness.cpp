// Reference-oracle harness for the 2D MRX operators.  TEST INFRASTRUCTURE ONLY.
//
// Compiled by oracle/build.py::build_ref_mrx with a patched copy of the
// reference's 2D/MPI/MRX/mhd_fd_ct_2d.c (its ODR/R_K lines; written only into
// oracle/_ref/) and 2D/MPI/MRX/boundary.c, against the single-rank mpi.h stub.
// It defines the boundary tables the sources read (settable by the caller)
// and exports the MRX step, the resistive and viscous operators and the
// anisotropic heat conduction under C names with one MPI rank.

int dnxs[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int dnys[8] = {0, 0, 0, 0, 0, 0, 0, 0};
int stxs[8] = {0, 0, 0, 0, 0, 1, 0, 0};
int stys[8] = {0, 0, 0, 0, 0, 0, 1, 0};

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

extern "C" {

void ref_mrx_step(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                  double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                  int xoff, int yoff, double gamma)
{
    mhd_fd_ct_2d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma, 0, 1, 1);
}

void ref_diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0, double dt,
                        double dx, double dy, int nx, int ny, int xoff, int yoff, double gamma)
{
    diff_ctfield_e(en, bx, by, bz, eta0, dt, dx, dy, nx, ny, xoff, yoff, gamma, 0, 1, 1);
}

void ref_ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en,
                       double nu0, double dt, double dx, double dy, int nx, int ny, int xoff,
                       int yoff, double gamma)
{
    ns_viscous_2d(ro, mx, my, mz, en, nu0, dt, dx, dy, nx, ny, xoff, yoff, gamma, 0, 1, 1);
}

void ref_t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                      double *en, const double *bx, const double *by, const double *bz,
                      double kk0, double dt, double dx, double dy, int nx, int ny, int xoff,
                      int yoff, double gamma)
{
    t_conduction(ro, mx, my, mz, en, bx, by, bz, kk0, dt, dx, dy, nx, ny, xoff, yoff, gamma, 0, 1,
                 1);
}

}  // extern "C"
