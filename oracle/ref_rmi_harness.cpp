// Reference-oracle harness for the RMI problem's inflow routine.  TEST
// INFRASTRUCTURE ONLY.
//
// Compiled by oracle/build.py::build_ref_rmi with the reference's own
// 2D/MPI/RMI/inj_ro.hpp (included from where it lies) against the
// single-rank mpi.h stub.  The routine reads the problem's globals gam and
// vref and its RANDOM switch; they are defined here (RANDOM on: with dro3 = 0
// the density is ro_3 exactly).  The routine seeds random() itself on its
// first call; ref_inj_ro primes that once on scratch arrays and then reseeds
// with the caller's seed, so the draws are those of srandom(seed).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mpi.h"

#define RANDOM (1)
static double gam = 5.0 / 3.0;
static double vref = 0.0;

#include "inj_ro.hpp"

extern "C" {

void ref_inj_ro(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                double *by, double *bz, int nx, int ny, int xoff, int yoff, double ro_3,
                double dro3, double vy_1, double bx_1, double by_1, double bz_1, double pr_1,
                double vref_, double gam_, unsigned seed)
{
    static bool primed = false;
    gam = gam_;
    vref = vref_;
    const size_t n = (size_t)nx * ny;
    if (!primed) {
        std::vector<double> t(8 * n, 1.0);
        double *p = t.data();
        inj_ro(p, p + n, p + 2 * n, p + 3 * n, p + 4 * n, p + 5 * n, p + 6 * n, p + 7 * n, ro_3,
               dro3, vy_1, bx_1, by_1, bz_1, pr_1, nx, ny, xoff, yoff, 0, 1, 1);
        primed = true;
    }
    srandom(seed);
    inj_ro(ro, mx, my, mz, en, bx, by, bz, ro_3, dro3, vy_1, bx_1, by_1, bz_1, pr_1, nx, ny, xoff,
           yoff, 0, 1, 1);
}

}  // extern "C"
