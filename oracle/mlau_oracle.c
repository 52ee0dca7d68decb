/*
 * CPU oracle for the MLAU per-step hot path.  TEST INFRASTRUCTURE ONLY: it is
 * the checker that tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline run; the GPU product never links or calls it.
 *
 * Restates the reference step drivers (file:line cited per function) in plain
 * C.  Arithmetic keeps the reference's evaluation order; build with
 * -O2 -fopenmp -ffp-contract=off (oracle/Makefile), never -ffast-math.
 * Scratch layout differs from the reference (struct-of-arrays instead of the
 * reference's stride-8 array-of-structs); the numbers do not.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "mlau_oracle.h"
#include "oracle_point.h"

/* Eigen-system where the drivers use the full one: 1 (mhd_c_reconst, the
   drivers' choice) or 2 (Miyoshi's mhd_m_reconst swapped in). */
static int o_full = 1;

static const int o_zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};

void oracle_set_eigen(int miyoshi) { o_full = miyoshi ? 2 : 1; }

/* Phase hook of the op-counting build (oracle/opcount.cpp); no-op here.
 * 0 cell B + primitives, 1 CT weights + shock sensors, 2 reconstruction,
 * 3 Riemann flux, 4 edge EMF, 5 RK update + CT curl. */
#ifndef ORACLE_PHASE
#define ORACLE_PHASE(p) ((void)0)
#endif

#define IDX3(i, j, k) ((long)nx * ((long)ny * (k) + (j)) + (i))

static double *alloc_d(long n)
{
    double *p = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (!p) abort();
    return p;
}

/* RK coefficients rk_fac (mhd_fd_ct_3d.c:120): U <- a U^n + b (U - dt L(U)). */
static void rk_coef(int nrk, int stage, double *a, double *b)
{
    const double t[3][2] = {{0.0, 1.0},
                            {0.5 + (nrk - 2) * 0.25, 0.5 - (nrk - 2) * 0.25},
                            {1. / 3., 2. / 3.}};
    *a = t[stage][0];
    *b = t[stage][1];
}

/* Ghost fill of one 3D array as the MPI driver leaves it for one rank
 * (3D/MPI/OTvortex/boundary.c): the periodic exchange along each axis whose
 * table entry 0 (dn0) is zero (mpi_sdrv3d), then the X, Y and Z mirrors by
 * dn (mpi_xbc3d / _ybc3d / _zbc3d, :227-309): dn -1 Dirichlet, +1 Neumann,
 * 0 nothing; st 1 marks a face-centred axis (its right boundary face is
 * kept). */
static void fill3d_bc(double *f, int nx, int ny, int nz, int xoff, int yoff, int zoff,
                      const int dn0[3], const int st[3], const int dn[3])
{
    if (dn0[0] == 0)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < xoff; i++) {
                    f[IDX3(nx - 1 - i, j, k)] = f[IDX3(2 * xoff - 1 - i, j, k)];
                    f[IDX3(i, j, k)] = f[IDX3(nx - 2 * xoff + i, j, k)];
                }
    if (dn0[1] == 0)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < yoff; j++)
                for (int i = 0; i < nx; i++) {
                    f[IDX3(i, ny - 1 - j, k)] = f[IDX3(i, 2 * yoff - 1 - j, k)];
                    f[IDX3(i, j, k)] = f[IDX3(i, ny - 2 * yoff + j, k)];
                }
    if (dn0[2] == 0)
        for (int k = 0; k < zoff; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    f[IDX3(i, j, nz - 1 - k)] = f[IDX3(i, j, 2 * zoff - 1 - k)];
                    f[IDX3(i, j, k)] = f[IDX3(i, j, nz - 2 * zoff + k)];
                }
    if (dn[0] != 0)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                for (int i = 0; i < xoff; i++)
                    f[IDX3(i, j, k)] = dn[0] * f[IDX3((2 * xoff - 1 + st[0]) - i, j, k)];
                for (int i = 0; i < xoff - st[0]; i++)
                    f[IDX3(nx - 1 - i, j, k)] = dn[0] * f[IDX3((nx - 2 * xoff + st[0]) + i, j, k)];
            }
    if (dn[1] != 0)
        for (int k = 0; k < nz; k++) {
            for (int j = 0; j < yoff; j++)
                for (int i = 0; i < nx; i++)
                    f[IDX3(i, j, k)] = dn[1] * f[IDX3(i, (2 * yoff - 1 + st[1]) - j, k)];
            for (int j = 0; j < yoff - st[1]; j++)
                for (int i = 0; i < nx; i++)
                    f[IDX3(i, ny - 1 - j, k)] = dn[1] * f[IDX3(i, (ny - 2 * yoff + st[1]) + j, k)];
        }
    if (dn[2] != 0) {
        for (int k = 0; k < zoff; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++)
                    f[IDX3(i, j, k)] = dn[2] * f[IDX3(i, j, (2 * zoff - 1 + st[2]) - k)];
        for (int k = 0; k < zoff - st[2]; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++)
                    f[IDX3(i, j, nz - 1 - k)] = dn[2] * f[IDX3(i, j, (nz - 2 * zoff + st[2]) + k)];
    }
}

/* bc2d, 2D/SERIAL/OTvortex/boundary.c:18-74: one array, X then Y; dn 0 is
   periodic, -1 Dirichlet (antisymmetric mirror), +1 Neumann (mirror); st 1
   marks a face-centred array along that axis (its right boundary face is
   computed by the update, not filled). */
static void bc2d_o(double *f, int nx, int ny, int xoff, int yoff, int stx, int dnx, int sty,
                   int dny)
{
    if (dnx == 0) {
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < xoff; i++) {
                f[(long)nx * j + (nx - 1 - i)] = f[(long)nx * j + (2 * xoff - 1 - i)];
                f[(long)nx * j + i] = f[(long)nx * j + (nx - 2 * xoff + i)];
            }
    } else {
        for (int j = 0; j < ny; j++) {
            for (int i = 0; i < xoff; i++)
                f[(long)nx * j + i] = dnx * f[(long)nx * j + (2 * xoff - 1 + stx) - i];
            for (int i = 0; i < xoff - stx; i++)
                f[(long)nx * j + (nx - 1 - i)] = dnx * f[(long)nx * j + (nx - 2 * xoff + stx) + i];
        }
    }
    if (dny == 0) {
        for (int j = 0; j < yoff; j++)
            for (int i = 0; i < nx; i++) {
                f[(long)nx * (ny - 1 - j) + i] = f[(long)nx * (2 * yoff - 1 - j) + i];
                f[(long)nx * j + i] = f[(long)nx * (ny - 2 * yoff + j) + i];
            }
    } else {
        for (int j = 0; j < yoff; j++)
            for (int i = 0; i < nx; i++)
                f[(long)nx * j + i] = dny * f[(long)nx * ((2 * yoff - 1 + sty) - j) + i];
        for (int j = 0; j < yoff - sty; j++)
            for (int i = 0; i < nx; i++)
                f[(long)nx * (ny - 1 - j) + i] = dny * f[(long)nx * ((ny - 2 * yoff + sty) + j) + i];
    }
}

/*
 * One face sweep of the 3D/2D drivers along an axis with element stride `st`
 * (mhd_fd_ct_3d.c:379-493 for X, :587-701 Y, :795-909 Z; 2D :273-362 and
 * :404-493).  Variables are passed already rotated to (normal, t, u) order:
 * vn/vt/vu velocities, cn/ct/cu cell-centred B, bface = face-centred normal B.
 * dvt/dvu: transverse shock sensors (dvu NULL in 2D).  split_t / split_u
 * select which tangential B fluxes get the central/upwind split (ql/qr).
 * Pencils: `npen` lines, line p starts at base[p], with `len` cells along the
 * axis.  Outputs flux fl[7 arrays] ordered (ro, mn, mt, mu, bt, bu, en) at
 * face index i (face i-1/2) for i in [3, len-2), and central parts fct/fcu.
 */
typedef struct {
    const double *ro, *vn, *vt, *vu, *cn, *ct, *cu, *pr, *m2, *bface, *dvt, *dvu;
    int split_t, split_u;
} sweep_in;

static void sweep_pencil(const sweep_in *S, long base, long st, int len, int odr, int flx,
                         double gamma, double *const fl[7], double *fct, double *fcu,
                         double *ul, double *ur, double *qlt, double *qrt, double *qlu,
                         double *qru)
{
    ORACLE_PHASE(2);
    for (int i = 2; i < len - 2; i++) {
        long c = base + st * i;
        double q[7][5];
        for (int m = 0; m < 5; m++) {
            long s = c + st * (m - 2);
            q[0][m] = S->ro[s];
            q[1][m] = S->vn[s];
            q[2][m] = S->vt[s];
            q[3][m] = S->vu[s];
            q[4][m] = S->ct[s];
            q[5][m] = S->cu[s];
            q[6][m] = S->pr[s];
        }
        double vl[7], vr[7];
        int full = (o_max(S->m2[c - st], o_max(S->m2[c], S->m2[c + st])) >= 1.0) ? o_full : 0;
        o_reconst(full, odr, q, S->cn[c], gamma, vl, vr);
        for (int v = 0; v < 7; v++) {
            ul[7 * (i + 1) + v] = vl[v];
            ur[7 * i + v] = vr[v];
        }
        double bl = S->bface[c + st], br = S->bface[c];
        if (S->split_t) {
            double a5[5], b5[5], la, ra, lb, rb;
            for (int m = 0; m < 5; m++) {
                long s = c + st * (m - 2);
                a5[m] = S->ct[s] * S->vn[s];
                b5[m] = S->vt[s];
            }
            o_lin_lr(odr, a5, &la, &ra);
            o_lin_lr(odr, b5, &lb, &rb);
            qlt[i + 1] = la - bl * lb;
            qrt[i] = ra - br * rb;
        }
        if (S->split_u) {
            double a5[5], b5[5], la, ra, lb, rb;
            for (int m = 0; m < 5; m++) {
                long s = c + st * (m - 2);
                a5[m] = S->cu[s] * S->vn[s];
                b5[m] = S->vu[s];
            }
            o_lin_lr(odr, a5, &la, &ra);
            o_lin_lr(odr, b5, &lb, &rb);
            qlu[i + 1] = la - bl * lb;
            qru[i] = ra - br * rb;
        }
    }
    ORACLE_PHASE(3);
    for (int i = 3; i < len - 2; i++) {
        long c = base + st * i;
        double bn = 0.5 * (S->bface[c] + S->bface[c]);
        double dvtm = S->dvu ? o_min(o_min(S->dvt[c - st], S->dvt[c]),
                                     o_min(S->dvu[c - st], S->dvu[c]))
                             : o_min(S->dvt[c - st], S->dvt[c]);
        double dv[2] = {(S->vn[c] - S->vn[c - st]), dvtm};
        double f[7];
        o_flux(flx, &ul[7 * i], &ur[7 * i], bn, gamma, dv, f);
        for (int v = 0; v < 7; v++) fl[v][c] = f[v];
        if (S->split_t) {
            fct[c] = 0.5 * (qlt[i] + qrt[i]);
            fl[4][c] -= fct[c];
        }
        if (S->split_u) {
            fcu[c] = 0.5 * (qlu[i] + qru[i]);
            fl[5][c] -= fcu[c];
        }
    }
}

/* Corner (edge) EMF contribution along an axis with stride st (one pencil):
 * the linear face interpolations of the upwind (fu) and central (fc) parts are
 * formed once per window j in [2, len-2), then for edges j in [3, len-2)
 * ``e += (+-0.5)*((ul0+ur0) + w*(ul1+ur1))`` with w = ct or 1-ct
 * (mhd_fd_ct_3d.c:494-585 and siblings). */
static void emf_pencil(const double *fu, const double *fc, const double *ctw, int one_minus,
                       double sgn, double *e, long base, long st, int len, int odr)
{
    double *buf = alloc_d(4L * (len + 1));
    double *ul0 = buf, *ur0 = buf + (len + 1), *ul1 = buf + 2 * (len + 1), *ur1 = buf + 3 * (len + 1);
    for (int j = 2; j < len - 2; j++) {
        long c = base + st * j;
        double a[5], b[5];
        for (int m = 0; m < 5; m++) {
            a[m] = fu[c + st * (m - 2)];
            b[m] = fc[c + st * (m - 2)];
        }
        o_lin_lr(odr, a, &ul0[j + 1], &ur0[j]);
        o_lin_lr(odr, b, &ul1[j + 1], &ur1[j]);
    }
    const double h = (sgn > 0) ? 0.5 : -0.5;
    for (int j = 3; j < len - 2; j++) {
        long c = base + st * j;
        double w = one_minus ? (1.0 - ctw[c]) : ctw[c];
        e[c] += h * ((ul0[j] + ur0[j]) + w * (ul1[j] + ur1[j]));
    }
    free(buf);
}

/* ------------------------------------------------------------------------ */
/* 3D driver: 3D/MPI/OTvortex/mhd_fd_ct_3d.c:99-1198, one rank, with the    */
/* problem's tables dnxs/dnys/dnzs (NULL: periodic).                          */
/* ------------------------------------------------------------------------ */
void oracle_fd_ct_3d_bc(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                        double *by, double *bz, double dt, double dx, double dy, double dz,
                        int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma,
                        int odr, int flx, int nrk, const int *tx_in, const int *ty_in,
                        const int *tz_in)
{
    const int *tx = tx_in ? tx_in : o_zero8, *ty = ty_in ? ty_in : o_zero8,
              *tz = tz_in ? tz_in : o_zero8;
    const int dn0[3] = {tx[0], ty[0], tz[0]}, st0[3] = {0, 0, 0};
    const long n = (long)nx * ny * nz;
    const double dtdx = dt / dx, dtdy = dt / dy, dtdz = dt / dz;
    double *state[8] = {ro, mx, my, mz, bx, by, bz, en};
    double *u0 = alloc_d(8 * n);
    for (int v = 0; v < 8; v++) memcpy(u0 + v * n, state[v], sizeof(double) * n);

    double *vx = alloc_d(n), *vy = alloc_d(n), *vz = alloc_d(n), *pr = alloc_d(n);
    double *cx = alloc_d(n), *cy = alloc_d(n), *cz = alloc_d(n), *m2 = alloc_d(n);
    double *ex = alloc_d(n), *ey = alloc_d(n), *ez = alloc_d(n);
    double *ct0 = alloc_d(n), *ct1 = alloc_d(n), *ct2 = alloc_d(n);
    double *dvx = alloc_d(n), *dvy = alloc_d(n), *dvz = alloc_d(n);
    double *F[3][7], *FC[3][2];
    for (int d = 0; d < 3; d++) {
        for (int v = 0; v < 7; v++) F[d][v] = alloc_d(n);
        FC[d][0] = alloc_d(n);
        FC[d][1] = alloc_d(n);
    }
    const long sy = nx, sz = (long)nx * ny;

    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, &ra, &rb);

        ORACLE_PHASE(0);
        /* cell-centred B (:186-220) and its periodic fill (:221-238) */
#pragma omp parallel for
        for (int k = 0; k < nz; k++) {
            for (int j = 0; j < ny; j++)
                for (int i = 1; i < nx - 2; i++) {
                    long s = IDX3(i, j, k);
                    cx[s] = o_face2cen(odr, bx[s - 1], bx[s], bx[s + 1], bx[s + 2]);
                }
            for (int j = 1; j < ny - 2; j++)
                for (int i = 0; i < nx; i++) {
                    long s = IDX3(i, j, k);
                    cy[s] = o_face2cen(odr, by[s - sy], by[s], by[s + sy], by[s + 2 * sy]);
                }
        }
#pragma omp parallel for
        for (int k = 1; k < nz - 2; k++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    long s = IDX3(i, j, k);
                    cz[s] = o_face2cen(odr, bz[s - sz], bz[s], bz[s + sz], bz[s + 2 * sz]);
                }
        {
            const int d5[3] = {tx[5], ty[5], tz[5]}, d6[3] = {tx[6], ty[6], tz[6]},
                      d7[3] = {tx[7], ty[7], tz[7]};
            fill3d_bc(cx, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d5);
            fill3d_bc(cy, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d6);
            fill3d_bc(cz, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d7);
        }

        /* primitives (:240-262) */
#pragma omp parallel for
        for (long s = 0; s < n; s++) {
            double iro = 1.0 / ro[s];
            vx[s] = mx[s] * iro;
            vy[s] = my[s] * iro;
            vz[s] = mz[s] * iro;
            double v2 = (vx[s] * vx[s] + vy[s] * vy[s] + vz[s] * vz[s]);
            double b2 = (cx[s] * cx[s] + cy[s] * cy[s] + cz[s] * cz[s]);
            pr[s] = (gamma - 1) * (en[s] - 0.5 * (ro[s] * v2 + b2));
            m2[s] = v2 / (gamma * pr[s] * iro);
            ex[s] = ey[s] = ez[s] = 0.0;
            ct0[s] = ct1[s] = ct2[s] = 0.5;
        }

        ORACLE_PHASE(1);
        /* Alfven-upwind CT weights (:264-340) */
        const double eps = 1e-6;
#pragma omp parallel for
        for (int k = 0; k < nz; k++)
            for (int j = 1; j < ny; j++)
                for (int i = 1; i < nx; i++) {
                    long s = IDX3(i, j, k);
                    double va = 0.25 * (vx[s - sy - 1] + vx[s - sy] + vx[s - 1] + vx[s]);
                    double vb = 0.25 * (vy[s - sy - 1] + vy[s - sy] + vy[s - 1] + vy[s]);
                    double rc = 0.25 * (ro[s - sy - 1] + ro[s - sy] + ro[s - 1] + ro[s]);
                    rc = 1.0 / sqrt(rc);
                    double ba = 0.5 * (bx[s - sy] + bx[s]);
                    double bb = 0.5 * (by[s - 1] + by[s]);
                    va = fabs(va) + fabs(ba * rc);
                    vb = fabs(vb) + fabs(bb * rc);
                    ct0[s] = (va + 0.5 * eps) / (va + vb + eps);
                }
#pragma omp parallel for
        for (int k = 1; k < nz; k++) {
            for (int j = 1; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    long s = IDX3(i, j, k);
                    double va = 0.25 * (vy[s - sz - sy] + vy[s - sz] + vy[s - sy] + vy[s]);
                    double vb = 0.25 * (vz[s - sz - sy] + vz[s - sz] + vz[s - sy] + vz[s]);
                    double rc = 0.25 * (ro[s - sz - sy] + ro[s - sz] + ro[s - sy] + ro[s]);
                    rc = 1.0 / sqrt(rc);
                    double ba = 0.5 * (by[s - sz] + by[s]);
                    double bb = 0.5 * (bz[s - sy] + bz[s]);
                    va = fabs(va) + fabs(ba * rc);
                    vb = fabs(vb) + fabs(bb * rc);
                    ct1[s] = (va + 0.5 * eps) / (va + vb + eps);
                }
            for (int j = 0; j < ny; j++)
                for (int i = 1; i < nx; i++) {
                    long s = IDX3(i, j, k);
                    double va = 0.25 * (vz[s - sz - 1] + vz[s - sz] + vz[s - 1] + vz[s]);
                    double vb = 0.25 * (vx[s - sz - 1] + vx[s - sz] + vx[s - 1] + vx[s]);
                    double rc = 0.25 * (ro[s - sz - 1] + ro[s - sz] + ro[s - 1] + ro[s]);
                    rc = 1.0 / sqrt(rc);
                    double ba = 0.5 * (bz[s - 1] + bz[s]);
                    double bb = 0.5 * (bx[s - sz] + bx[s]);
                    va = fabs(va) + fabs(ba * rc);
                    vb = fabs(vb) + fabs(bb * rc);
                    ct2[s] = (va + 0.5 * eps) / (va + vb + eps);
                }
        }

        /* shock sensors (:342-377) */
#pragma omp parallel for
        for (int k = 1; k < nz - 1; k++)
            for (int j = 1; j < ny - 1; j++)
                for (int i = 1; i < nx - 1; i++) {
                    long s = IDX3(i, j, k);
                    dvx[s] = o_min((vx[s + 1] - vx[s]), (vx[s] - vx[s - 1]));
                    dvy[s] = o_min((vy[s + sy] - vy[s]), (vy[s] - vy[s - sy]));
                    dvz[s] = o_min((vz[s + sz] - vz[s]), (vz[s] - vz[s - sz]));
                }
        {
            /* the sensors' sign flips (:367-376) */
            const int d1[3] = {-tx[1], +ty[1], +tz[1]}, d2[3] = {+tx[2], -ty[2], +tz[2]},
                      d3[3] = {+tx[3], +ty[3], -tz[3]};
            fill3d_bc(dvx, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d1);
            fill3d_bc(dvy, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d2);
            fill3d_bc(dvz, nx, ny, nz, xoff, yoff, zoff, dn0, st0, d3);
        }

        /* three face sweeps; rotated variables (:379-493, :587-701, :795-909) */
        sweep_in SX = {ro, vx, vy, vz, cx, cy, cz, pr, m2, bx, dvy, dvz, 1, 1};
        sweep_in SY = {ro, vy, vz, vx, cy, cz, cx, pr, m2, by, dvz, dvx, 1, 1};
        sweep_in SZ = {ro, vz, vx, vy, cz, cx, cy, pr, m2, bz, dvx, dvy, 1, 1};
        const sweep_in *SW[3] = {&SX, &SY, &SZ};
        const int lens[3] = {nx, ny, nz};
        const long strides[3] = {1, sy, sz};
        for (int d = 0; d < 3; d++) {
            int len = lens[d];
            long st = strides[d];
            long npen = n / len;
#pragma omp parallel
            {
                double *ul = alloc_d(7 * (len + 1)), *ur = alloc_d(7 * (len + 1));
                double *q = alloc_d(4 * (len + 1));
#pragma omp for
                for (long p = 0; p < npen; p++) {
                    long base;
                    if (d == 0) base = p * nx;
                    else if (d == 1) base = (p / nx) * sz + (p % nx);
                    else base = p;
                    sweep_pencil(SW[d], base, st, len, odr, flx, gamma, F[d], FC[d][0],
                                 FC[d][1], ul, ur, q, q + (len + 1), q + 2 * (len + 1),
                                 q + 3 * (len + 1));
                }
                free(ul);
                free(ur);
                free(q);
            }
        }

        ORACLE_PHASE(4);
        /* edge EMFs (:494-585, :702-793, :910-1001).  F[d][4] is the flux of
         * the first tangential B (t), F[d][5] of the second (u):
         *   X: t=y, u=z;  Y: t=z, u=x;  Z: t=x, u=y. */
#pragma omp parallel for
        for (int k = 0; k < nz; k++)
            for (int i = 3; i < nx - 2; i++)
                emf_pencil(F[0][4], FC[0][0], ct0, 1, -1.0, ez, IDX3(i, 0, k), sy, ny, odr);
#pragma omp parallel for
        for (int j = 0; j < ny; j++)
            for (int i = 3; i < nx - 2; i++)
                emf_pencil(F[0][5], FC[0][1], ct2, 0, +1.0, ey, IDX3(i, j, 0), sz, nz, odr);
#pragma omp parallel for
        for (int j = 3; j < ny - 2; j++)
            for (int i = 0; i < nx; i++)
                emf_pencil(F[1][4], FC[1][0], ct1, 1, -1.0, ex, IDX3(i, j, 0), sz, nz, odr);
#pragma omp parallel for
        for (int k = 0; k < nz; k++)
            for (int j = 3; j < ny - 2; j++)
                emf_pencil(F[1][5], FC[1][1], ct0, 0, +1.0, ez, IDX3(0, j, k), 1, nx, odr);
#pragma omp parallel for
        for (int k = 3; k < nz - 2; k++)
            for (int j = 0; j < ny; j++)
                emf_pencil(F[2][4], FC[2][0], ct2, 1, -1.0, ey, IDX3(0, j, k), 1, nx, odr);
#pragma omp parallel for
        for (int k = 3; k < nz - 2; k++)
            for (int i = 0; i < nx; i++)
                emf_pencil(F[2][5], FC[2][1], ct1, 0, +1.0, ex, IDX3(i, 0, k), sy, ny, odr);

        ORACLE_PHASE(5);
        /* cell-centred update (:1003-1078).  Flux component per direction
         * for (ro, mx, my, mz, en): X (0,1,2,3,6), Y (0,3,1,2,6), Z (0,2,3,1,6). */
        static const int cmp[3][5] = {{0, 1, 2, 3, 6}, {0, 3, 1, 2, 6}, {0, 2, 3, 1, 6}};
        double *cons[5] = {ro, mx, my, mz, en};
        const int u0v[5] = {0, 1, 2, 3, 7};
#pragma omp parallel for
        for (int k = zoff; k < nz - zoff; k++)
            for (int j = yoff; j < ny - yoff; j++)
                for (int i = xoff; i < nx - xoff; i++) {
                    long s = IDX3(i, j, k);
                    for (int v = 0; v < 5; v++) {
                        const double *fx = F[0][cmp[0][v]], *fy = F[1][cmp[1][v]],
                                     *fz = F[2][cmp[2][v]];
                        double d0 = o_diff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
                        double d1 = o_diff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
                        double d2 = o_diff(odr, fz[s - sz], fz[s], fz[s + sz], fz[s + 2 * sz]);
                        cons[v][s] = ra * u0[u0v[v] * n + s]
                                     + rb * (cons[v][s] - dtdx * d0 - dtdy * d1 - dtdz * d2);
                    }
                }
        /* CT update of face B (:1079-1157) */
#pragma omp parallel for
        for (int k = zoff; k < nz - zoff; k++) {
            for (int j = yoff; j < ny - yoff; j++)
                for (int i = xoff; i < nx - xoff + 1; i++) {
                    long s = IDX3(i, j, k);
                    double d0 = o_diff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
                    double d1 = o_diff(odr, ey[s - sz], ey[s], ey[s + sz], ey[s + 2 * sz]);
                    bx[s] = ra * u0[4 * n + s] + rb * (bx[s] - dtdy * d0 + dtdz * d1);
                }
            for (int j = yoff; j < ny - yoff + 1; j++)
                for (int i = xoff; i < nx - xoff; i++) {
                    long s = IDX3(i, j, k);
                    double d0 = o_diff(odr, ex[s - sz], ex[s], ex[s + sz], ex[s + 2 * sz]);
                    double d1 = o_diff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
                    by[s] = ra * u0[5 * n + s] + rb * (by[s] - dtdz * d0 + dtdx * d1);
                }
        }
#pragma omp parallel for
        for (int k = zoff; k < nz - zoff + 1; k++)
            for (int j = yoff; j < ny - yoff; j++)
                for (int i = xoff; i < nx - xoff; i++) {
                    long s = IDX3(i, j, k);
                    double d0 = o_diff(odr, ey[s - 1], ey[s], ey[s + 1], ey[s + 2]);
                    double d1 = o_diff(odr, ex[s - sy], ex[s], ex[s + sy], ex[s + 2 * sy]);
                    bz[s] = ra * u0[6 * n + s] + rb * (bz[s] - dtdx * d0 + dtdy * d1);
                }
        /* boundary of the 8 conserved arrays (:1161-1175); state[] holds
           ro mx my mz bx by bz en, the tables ro mx my mz en bx by bz */
        for (int v = 0; v < 8; v++) {
            const int t = (v < 4) ? v : (v == 7 ? 4 : v + 1);
            const int st[3] = {t == 5, t == 6, t == 7}, dn[3] = {tx[t], ty[t], tz[t]};
            fill3d_bc(state[v], nx, ny, nz, xoff, yoff, zoff, dn0, st, dn);
        }
    }

    free(u0);
    double *tmp[] = {vx, vy, vz, pr, cx, cy, cz, m2, ex, ey, ez, ct0, ct1, ct2, dvx, dvy, dvz};
    for (unsigned t = 0; t < sizeof(tmp) / sizeof(tmp[0]); t++) free(tmp[t]);
    for (int d = 0; d < 3; d++) {
        for (int v = 0; v < 7; v++) free(F[d][v]);
        free(FC[d][0]);
        free(FC[d][1]);
    }
}

/* ------------------------------------------------------------------------ */
/* 2D driver: 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-660; boundary tables     */
/* dnx/dny as the problem's dnxs/dnys (global.hpp), NULL = periodic.        */
/* ------------------------------------------------------------------------ */
void oracle_fd_ct_2d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                     double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                     int xoff, int yoff, double gamma, int odr, int flx, int nrk)
{
    oracle_fd_ct_2d_bc(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma,
                       odr, flx, nrk, NULL, NULL);
}

/* The problems' setbc (2D/SERIAL/OTvortex/setbc.hpp:1-6): bc2d on the eight
   conserved arrays with the boundary tables. */
void oracle_bc2d_state(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                       double *by, double *bz, int nx, int ny, int xoff, int yoff,
                       const int *dnx, const int *dny)
{
    static const int stx[8] = {0, 0, 0, 0, 0, 1, 0, 0}, sty[8] = {0, 0, 0, 0, 0, 0, 1, 0};
    double *p[8] = {ro, mx, my, mz, en, bx, by, bz};
    for (int v = 0; v < 8; v++) bc2d_o(p[v], nx, ny, xoff, yoff, stx[v], dnx[v], sty[v], dny[v]);
}

void oracle_fd_ct_2d_bc(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                        double *by, double *bz, double dt, double dx, double dy, int nx, int ny,
                        int xoff, int yoff, double gamma, int odr, int flx, int nrk,
                        const int *dnx_in, const int *dny_in)
{
    static const int zero8[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    static const int stx[8] = {0, 0, 0, 0, 0, 1, 0, 0}, sty[8] = {0, 0, 0, 0, 0, 0, 1, 0};
    const int *dnx = dnx_in ? dnx_in : zero8, *dny = dny_in ? dny_in : zero8;
    const long n = (long)nx * ny;
    const double dtdx = dt / dx, dtdy = dt / dy;
    double *state[8] = {ro, mx, my, mz, bx, by, bz, en};
    double *u0 = alloc_d(8 * n);
    for (int v = 0; v < 8; v++) memcpy(u0 + v * n, state[v], sizeof(double) * n);
    double *vx = alloc_d(n), *vy = alloc_d(n), *vz = alloc_d(n), *pr = alloc_d(n);
    double *cx = alloc_d(n), *cy = alloc_d(n), *m2 = alloc_d(n), *ez = alloc_d(n);
    double *ctw = alloc_d(n), *dvx = alloc_d(n), *dvy = alloc_d(n);
    double *FX[7], *FY[7], *fcx = alloc_d(n), *fcy = alloc_d(n);
    for (int v = 0; v < 7; v++) { FX[v] = alloc_d(n); FY[v] = alloc_d(n); }
    const long sy = nx;

    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, &ra, &rb);
        ORACLE_PHASE(0);
        /* cell-centred B (:172-201) */
#pragma omp parallel for
        for (int j = 0; j < ny; j++)
            for (int i = 1; i < nx - 2; i++) {
                long s = (long)nx * j + i;
                cx[s] = o_face2cen(odr, bx[s - 1], bx[s], bx[s + 1], bx[s + 2]);
            }
#pragma omp parallel for
        for (int j = 1; j < ny - 2; j++)
            for (int i = 0; i < nx; i++) {
                long s = (long)nx * j + i;
                cy[s] = o_face2cen(odr, by[s - sy], by[s], by[s + sy], by[s + 2 * sy]);
            }
        bc2d_o(cx, nx, ny, xoff, yoff, 0, dnx[5], 0, dny[5]);
        bc2d_o(cy, nx, ny, xoff, yoff, 0, dnx[6], 0, dny[6]);
        /* primitives (:203-223) */
#pragma omp parallel for
        for (long s = 0; s < n; s++) {
            double iro = 1.0 / ro[s];
            vx[s] = mx[s] * iro;
            vy[s] = my[s] * iro;
            vz[s] = mz[s] * iro;
            double v2 = (vx[s] * vx[s] + vy[s] * vy[s] + vz[s] * vz[s]);
            double b2 = (cx[s] * cx[s] + cy[s] * cy[s] + bz[s] * bz[s]);
            pr[s] = (gamma - 1) * (en[s] - 0.5 * (ro[s] * v2 + b2));
            m2[s] = v2 / (gamma * pr[s] * iro);
            ez[s] = 0.0;
            ctw[s] = 0.5;
        }
        ORACLE_PHASE(1);
        /* CT weights (:224-249) */
        const double eps = 1e-6;
#pragma omp parallel for
        for (int j = 1; j < ny; j++)
            for (int i = 1; i < nx; i++) {
                long s = (long)nx * j + i;
                double va = 0.25 * (vx[s - sy - 1] + vx[s - sy] + vx[s - 1] + vx[s]);
                double vb = 0.25 * (vy[s - sy - 1] + vy[s - sy] + vy[s - 1] + vy[s]);
                double rc = 0.25 * (ro[s - sy - 1] + ro[s - sy] + ro[s - 1] + ro[s]);
                rc = 1.0 / sqrt(rc);
                double ba = 0.5 * (bx[s - sy] + bx[s]);
                double bb = 0.5 * (by[s - 1] + by[s]);
                va = fabs(va) + fabs(ba * rc);
                vb = fabs(vb) + fabs(bb * rc);
                ctw[s] = (va + 0.5 * eps) / (va + vb + eps);
            }
        /* shock sensors (:251-271) */
#pragma omp parallel for
        for (int j = 1; j < ny - 1; j++)
            for (int i = 1; i < nx - 1; i++) {
                long s = (long)nx * j + i;
                dvx[s] = o_min((vx[s + 1] - vx[s]), (vx[s] - vx[s - 1]));
                dvy[s] = o_min((vy[s + sy] - vy[s]), (vy[s] - vy[s - sy]));
            }
        bc2d_o(dvx, nx, ny, xoff, yoff, 0, -dnx[1], 0, +dny[1]);
        bc2d_o(dvy, nx, ny, xoff, yoff, 0, +dnx[2], 0, -dny[2]);

        /* X faces (:273-362): (vn,vt,vu)=(vx,vy,vz), (bt,bu)=(cy,bz); only the
         * By flux is split.  Y faces (:404-493): (vy,vz,vx), (bz,cx); only Bx. */
        sweep_in SX = {ro, vx, vy, vz, cx, cy, bz, pr, m2, bx, dvy, NULL, 1, 0};
        sweep_in SY = {ro, vy, vz, vx, cy, bz, cx, pr, m2, by, dvx, NULL, 0, 1};
#pragma omp parallel
        {
            int L = (nx > ny ? nx : ny) + 1;
            double *ul = alloc_d(7 * L), *ur = alloc_d(7 * L), *q = alloc_d(4 * L);
#pragma omp for
            for (int j = 0; j < ny; j++)
                sweep_pencil(&SX, (long)nx * j, 1, nx, odr, flx, gamma, FX, fcx, NULL, ul, ur,
                             q, q + L, q + 2 * L, q + 3 * L);
#pragma omp for
            for (int i = 0; i < nx; i++)
                sweep_pencil(&SY, i, sy, ny, odr, flx, gamma, FY, NULL, fcy, ul, ur, q, q + L,
                             q + 2 * L, q + 3 * L);
            free(ul);
            free(ur);
            free(q);
        }
        ORACLE_PHASE(4);
        /* Ez from x-faces along Y (:364-402) and from y-faces along X (:495-533).
         * The 2D reference restricts the x-face part to rows j in [3,ny-2) via
         * its loops; emf_pencil covers the same edges. */
#pragma omp parallel for
        for (int i = 3; i < nx - 2; i++)
            emf_pencil(FX[4], fcx, ctw, 1, -1.0, ez, i, sy, ny, odr);
#pragma omp parallel for
        for (int j = 3; j < ny - 2; j++)
            emf_pencil(FY[5], fcy, ctw, 0, +1.0, ez, (long)nx * j, 1, nx, odr);

        ORACLE_PHASE(5);
        /* cell-centred update incl. Bz (:535-592).  Components per direction
         * for (ro, mx, my, mz, bz, en): X (0,1,2,3,5,6), Y (0,3,1,2,4,6). */
        static const int cx2[6] = {0, 1, 2, 3, 5, 6}, cy2[6] = {0, 3, 1, 2, 4, 6};
        double *cons[6] = {ro, mx, my, mz, bz, en};
        const int u0v[6] = {0, 1, 2, 3, 6, 7};
#pragma omp parallel for
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                long s = (long)nx * j + i;
                for (int v = 0; v < 6; v++) {
                    const double *fx = FX[cx2[v]], *fy = FY[cy2[v]];
                    double d0 = o_diff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
                    double d1 = o_diff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
                    cons[v][s] = ra * u0[u0v[v] * n + s] + rb * (cons[v][s] - dtdx * d0 - dtdy * d1);
                }
            }
        /* CT Bx, By (:593-632) */
#pragma omp parallel for
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff + 1; i++) {
                long s = (long)nx * j + i;
                double d = o_diff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
                bx[s] = ra * u0[4 * n + s] + rb * (bx[s] - dtdy * d);
            }
#pragma omp parallel for
        for (int j = yoff; j < ny - yoff + 1; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                long s = (long)nx * j + i;
                double d = o_diff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
                by[s] = ra * u0[5 * n + s] + rb * (by[s] + dtdx * d);
            }
        /* boundary of the 8 conserved arrays (:636-638), in the reference's order */
        double *p[8] = {ro, mx, my, mz, en, bx, by, bz};
        for (int v = 0; v < 8; v++) bc2d_o(p[v], nx, ny, xoff, yoff, stx[v], dnx[v], sty[v], dny[v]);
    }
    free(u0);
    double *tmp[] = {vx, vy, vz, pr, cx, cy, m2, ez, ctw, dvx, dvy, fcx, fcy};
    for (unsigned t = 0; t < sizeof(tmp) / sizeof(tmp[0]); t++) free(tmp[t]);
    for (int v = 0; v < 7; v++) { free(FX[v]); free(FY[v]); }
}

/* ------------------------------------------------------------------------ */
/* 1D driver: 1D/SERIAL/shock/mhd_fd4c_1d.c:60-271 and the wave variant.     */
/* ------------------------------------------------------------------------ */

/* openbc1d_mhd, 1D/SERIAL/shock/openbc1d_mhd.c:21-175: characteristic
 * advection of the boundary data across the domain edge, both sides. */
static void open_bc_1d(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                       double *bz, double bx, double dx, double dt, int nx, int xoff,
                       double gamma)
{
    const double bx2 = bx * bx, dtdx = dt / dx;
    for (int side = 0; side <= 1; side++) {
        int sgn = side ? -1 : 1;
        int si = side ? (nx - xoff - 1) : xoff;
        int so = si - sgn;
        double q[2][7];
        for (int t = 0; t < 2; t++) {
            int s = t ? so : si;
            double r = ro[s], iro = 1.0 / r;
            double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
            double v2 = vx * vx + vy * vy + vz * vz;
            double b2 = bx * bx + by[s] * by[s] + bz[s] * bz[s];
            q[t][0] = r;
            q[t][1] = vx;
            q[t][2] = vy;
            q[t][3] = vz;
            q[t][4] = by[s];
            q[t][5] = bz[s];
            q[t][6] = (gamma - 1) * (en[s] - 0.5 * (r * v2 + b2));
        }
        double L[7][7], R[7][7], lam[7];
        o_eigen_full(0.5 * (q[0][0] + q[1][0]), 0.5 * (q[0][1] + q[1][1]),
                     0.5 * (q[0][2] + q[1][2]), 0.5 * (q[0][3] + q[1][3]), 0.5 * (bx + bx),
                     0.5 * (q[0][4] + q[1][4]), 0.5 * (q[0][5] + q[1][5]),
                     0.5 * (q[0][6] + q[1][6]), gamma, lam, L, R);
        double w[7][2];
        for (int t = 0; t < 2; t++)
            for (int m = 0; m < 7; m++)
                w[m][t] = (+L[m][0] * q[t][0] + L[m][1] * q[t][1] + L[m][2] * q[t][2]
                           + L[m][3] * q[t][3] + L[m][4] * q[t][4] + L[m][5] * q[t][5]
                           + L[m][6] * q[t][6]);
        for (int m = 0; m < 7; m++) {
            double c = sgn * lam[m];
            w[m][1] = (c > 0) ? w[m][1] : (1 + c * dtdx) * w[m][1] - c * dtdx * w[m][0];
        }
        double p[7];
        for (int k = 0; k < 7; k++)
            p[k] = R[0][k] * w[0][1] + R[1][k] * w[1][1] + R[2][k] * w[2][1] + R[3][k] * w[3][1]
                   + R[4][k] * w[4][1] + R[5][k] * w[5][1] + R[6][k] * w[6][1];
        ro[so] = p[0];
        mx[so] = p[1];
        my[so] = p[2];
        mz[so] = p[3];
        by[so] = p[4];
        bz[so] = p[5];
        en[so] = p[6];
        double v2 = mx[so] * mx[so] + my[so] * my[so] + mz[so] * mz[so];
        double b2 = bx2 + by[so] * by[so] + bz[so] * bz[so];
        en[so] = en[so] / (gamma - 1.0) + 0.5 * (ro[so] * v2 + b2);
        mx[so] *= ro[so];
        my[so] *= ro[so];
        mz[so] *= ro[so];
        for (int j = 0; j < xoff - 1; j++) {
            int s = side * (nx - 1) + sgn * j;
            ro[s] = ro[so];
            mx[s] = mx[so];
            my[s] = my[so];
            mz[s] = mz[so];
            by[s] = by[so];
            bz[s] = bz[so];
            en[s] = en[so];
        }
    }
}

static void fill1d(double *f, int nx, int xoff)
{
    for (int i = 0; i < xoff; i++) {
        f[nx - 1 - i] = f[2 * xoff - 1 - i];
        f[i] = f[nx - 2 * xoff + i];
    }
}

void oracle_fd4c_1d(double *ro, double *mx, double *my, double *mz, double *en, double *by,
                    double *bz, double bx, double dt, double dx, int nx, int xoff, double gamma,
                    int odr, int flx, int nrk, int bc)
{
    const double dtdx = dt / dx, bx2 = bx * bx;
    double *state[7] = {ro, mx, my, mz, by, bz, en};
    double *u0 = alloc_d(7L * nx);
    for (int v = 0; v < 7; v++) memcpy(u0 + (long)v * nx, state[v], sizeof(double) * nx);
    double *vx = alloc_d(nx), *vy = alloc_d(nx), *vz = alloc_d(nx), *pr = alloc_d(nx);
    double *ul = alloc_d(7L * (nx + 1)), *ur = alloc_d(7L * (nx + 1)), *fx = alloc_d(7L * nx);

    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, &ra, &rb);
        for (int i = 0; i < nx; i++) {
            double iro = 1.0 / ro[i];
            vx[i] = mx[i] * iro;
            vy[i] = my[i] * iro;
            vz[i] = mz[i] * iro;
            double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
            double b2 = bx2 + by[i] * by[i] + bz[i] * bz[i];
            pr[i] = (gamma - 1) * (en[i] - 0.5 * (ro[i] * v2 + b2));
        }
        /* faces (:133-186); full eigen-system where any of the three central
         * cells is sonic-supersonic */
        for (int i = 2; i < nx - 2; i++) {
            double q[7][5];
            for (int m = 0; m < 5; m++) {
                int s = i + m - 2;
                q[0][m] = ro[s];
                q[1][m] = vx[s];
                q[2][m] = vy[s];
                q[3][m] = vz[s];
                q[4][m] = by[s];
                q[5][m] = bz[s];
                q[6][m] = pr[s];
            }
            double mach[3];
            for (int t = 0; t < 3; t++) {
                double c2 = gamma * q[6][1 + t] / q[0][1 + t];
                double v2 = q[1][1 + t] * q[1][1 + t] + q[2][1 + t] * q[2][1 + t]
                            + q[3][1 + t] * q[3][1 + t];
                mach[t] = v2 / c2;
            }
            int full = (o_max(mach[0], o_max(mach[1], mach[2])) >= 1.0) ? o_full : 0;
            double vl[7], vr[7];
            o_reconst(full, odr, q, bx, gamma, vl, vr);
            for (int v = 0; v < 7; v++) {
                ul[7 * (i + 1) + v] = vl[v];
                ur[7 * i + v] = vr[v];
            }
        }
        for (int i = 3; i < nx - 2; i++) {
            double dv[2] = {(vx[i] - vx[i - 1]), 0.0};
            o_flux(flx, &ul[7 * i], &ur[7 * i], bx, gamma, dv, &fx[7 * i]);
        }
        if (bc == ORACLE_BC1D_OPEN && rk == 0)
            open_bc_1d(ro, mx, my, mz, en, by, bz, bx, dx, dt, nx, xoff, gamma);
        /* update (:220-255): flux order (ro, mx, my, mz, by, bz, en) */
        for (int i = 4; i < nx - 4; i++)
            for (int v = 0; v < 7; v++) {
                double d = o_diff(odr, fx[7 * (i - 1) + v], fx[7 * i + v], fx[7 * (i + 1) + v],
                                  fx[7 * (i + 2) + v]);
                state[v][i] = ra * u0[(long)v * nx + i] + rb * (state[v][i] - dtdx * d);
            }
        if (bc == ORACLE_BC1D_PERIODIC)
            for (int v = 0; v < 7; v++) fill1d(state[v], nx, xoff);
    }
    free(u0);
    free(vx);
    free(vy);
    free(vz);
    free(pr);
    free(ul);
    free(ur);
    free(fx);
}

/* ------------------------------------------------------------------------ */
/* CFL dt                                                                    */
/* ------------------------------------------------------------------------ */
double oracle_cfl_3d(const double *ro, const double *mx, const double *my, const double *mz,
                     const double *en, const double *bx, const double *by, const double *bz,
                     int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma,
                     double cfl, double dr, double vfast, double dt_old, double *vmax_out)
{
    double vmax = vfast;
    for (int k = zoff; k < nz - zoff; k++)
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                long s = IDX3(i, j, k);
                double iro = 1.0 / ro[s];
                double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
                double bxc = 0.5 * (bx[s] + bx[s + 1]);
                double byc = 0.5 * (by[s] + by[s + nx]);
                double bzc = 0.5 * (bz[s] + bz[s + (long)nx * ny]);
                double v2 = vx * vx + vy * vy + vz * vz;
                double b2 = bxc * bxc + byc * byc + bzc * bzc;
                double p = (gamma - 1) * (en[s] - 0.5 * (ro[s] * v2 + b2));
                double cf = sqrt((0.5 * gamma * (2.0 * p) + b2) / (ro[s]));
                double vt = sqrt(v2) + cf;
                if (vt > vmax) vmax = vt;
            }
    if (vmax_out) *vmax_out = vmax;
    return isfinite(vmax) ? cfl * dr / vmax : dt_old;
}

double oracle_cfl_2d(const double *ro, const double *mx, const double *my, const double *mz,
                     const double *en, const double *bx, const double *by, const double *bz,
                     int nx, int ny, int xoff, int yoff, double gamma, double cfl, double dr,
                     double vfast, double dt_old, double *vmax_out)
{
    double vmax = vfast;
    for (int j = yoff; j < ny - yoff; j++)
        for (int i = xoff; i < nx - xoff; i++) {
            long s = (long)nx * j + i;
            double iro = 1.0 / ro[s];
            double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
            double bxc = 0.5 * (bx[s] + bx[s + 1]);
            double byc = 0.5 * (by[s] + by[s + nx]);
            double bzc = bz[s];
            double v2 = vx * vx + vy * vy + vz * vz;
            double b2 = bxc * bxc + byc * byc + bzc * bzc;
            double p = (gamma - 1) * (en[s] - 0.5 * (ro[s] * v2 + b2));
            double cf = sqrt((0.5 * gamma * (2.0 * p) + b2) / (ro[s]));
            double vt = sqrt(vx * vx + vy * vy) + cf;
            if (vt > vmax) vmax = vt;
        }
    if (vmax_out) *vmax_out = vmax;
    return isfinite(vmax) ? cfl * dr / vmax : dt_old;
}

double oracle_dt_1d(const double *ro, const double *mx, const double *my, const double *mz,
                    const double *en, const double *by, const double *bz, double bx, int nx,
                    double gamma, double cfl, double dx, double vfloor)
{
    double vmax = vfloor;
    for (int i = 0; i < nx; i++) {
        double iro = 1.0 / ro[i];
        double vx = mx[i] * iro, vy = my[i] * iro, vz = mz[i] * iro;
        double v2 = vx * vx + vy * vy + vz * vz;
        double b2 = bx * bx + by[i] * by[i] + bz[i] * bz[i];
        double p = (gamma - 1) * (en[i] - 0.5 * (ro[i] * v2 + b2));
        double cf = sqrt((gamma * p + b2) * iro);
        double vt = fabs(vx) + cf;
        if (vt > vmax) vmax = vt;
    }
    return cfl * dx / vmax;
}

/* ------------------------------------------------------------------------ */
void oracle_rec_lr(int odr, const double *f5, double *fl, double *fr) { o_rec_lr(odr, f5, fl, fr); }

void oracle_flux(int flx, const double *in, const double *dv, double *out)
{
    o_flux(flx, in, in + 7, in[14], in[15], dv, out);
}

void oracle_reconst(int full, int odr, const double *prim35, double bn, double gamma,
                    double *ul, double *ur)
{
    double q[7][5];
    for (int k = 0; k < 7; k++)
        for (int m = 0; m < 5; m++) q[k][m] = prim35[5 * k + m];
    o_reconst(full, odr, q, bn, gamma, ul, ur);
}

/* ------------------------------------------------------------------------ */
/* 2D MRX operators: 2D/MPI/MRX/mhd_fd_ct_2d.c:726-1174, one rank.           */
/* ------------------------------------------------------------------------ */

/* Ghost fill of arrays p[0..nn) by the MPI 2D drivers' single-rank boundary
   routines (2D/MPI/MRX/boundary.c): mpi_sdrv2d - periodic along an axis whose
   table entry 0 is zero, X then Y, every array - then per array mpi_xbc2d and
   mpi_ybc2d, mirroring where the array's own entry is nonzero. */
static void o_bc2d_mpi(double **p, int nn, const int *stx, const int *sty, const int *dnx,
                       const int *dny, int dnx0, int dny0, int nx, int ny, int xoff, int yoff)
{
    if (dnx0 == 0)
        for (int n = 0; n < nn; n++)
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < xoff; i++) {
                    p[n][(long)nx * j + (nx - 1 - i)] = p[n][(long)nx * j + (2 * xoff - 1 - i)];
                    p[n][(long)nx * j + i] = p[n][(long)nx * j + (nx - 2 * xoff + i)];
                }
    if (dny0 == 0)
        for (int n = 0; n < nn; n++)
            for (int j = 0; j < yoff; j++)
                for (int i = 0; i < nx; i++) {
                    p[n][(long)nx * (ny - 1 - j) + i] = p[n][(long)nx * (2 * yoff - 1 - j) + i];
                    p[n][(long)nx * j + i] = p[n][(long)nx * (ny - 2 * yoff + j) + i];
                }
    for (int n = 0; n < nn; n++) {
        double *f = p[n];
        if (dnx[n] != 0) {
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < xoff; i++)
                    f[(long)nx * j + i] = dnx[n] * f[(long)nx * j + (2 * xoff - 1 + stx[n]) - i];
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < xoff - stx[n]; i++)
                    f[(long)nx * j + (nx - 1 - i)] =
                        dnx[n] * f[(long)nx * j + (nx - 2 * xoff + stx[n]) + i];
        }
        if (dny[n] != 0) {
            for (int j = 0; j < yoff; j++)
                for (int i = 0; i < nx; i++)
                    f[(long)nx * j + i] = dny[n] * f[(long)nx * ((2 * yoff - 1 + sty[n]) - j) + i];
            for (int j = 0; j < yoff - sty[n]; j++)
                for (int i = 0; i < nx; i++)
                    f[(long)nx * (ny - 1 - j) + i] =
                        dny[n] * f[(long)nx * ((ny - 2 * yoff + sty[n]) + j) + i];
        }
    }
}


/* diff_ctfield_e (2D/MPI/MRX/mhd_fd_ct_2d.c:726-950): resistive diffusion of
   the CT field with uniform resistivity eta0, energy updated by the
   resistive Poynting flux. */
void oracle_diff_ctfield_e(double *en, double *bx, double *by, double *bz, double eta0,
                           double dt, double dx, double dy, int nx, int ny, int xoff, int yoff,
                           double gamma, int odr, int nrk, const int *dnx_in, const int *dny_in)
{
    (void)gamma;
    const int *dnx = dnx_in ? dnx_in : o_zero8, *dny = dny_in ? dny_in : o_zero8;
    static const int stx[8] = {0, 0, 0, 0, 0, 1, 0, 0}, sty[8] = {0, 0, 0, 0, 0, 0, 1, 0};
    const long n = (long)nx * ny;
    const double dtdx = dt / dx, dtdy = dt / dy, idx = 1. / dx, idy = 1. / dy;
    double *ut = alloc_d(4 * n), *fx = alloc_d(n), *fy = alloc_d(n);
    double *ex = alloc_d(n), *ey = alloc_d(n), *ez = alloc_d(n);
    memcpy(ut, bx, sizeof(double) * n);
    memcpy(ut + n, by, sizeof(double) * n);
    memcpy(ut + 2 * n, bz, sizeof(double) * n);
    memcpy(ut + 3 * n, en, sizeof(double) * n);
#define S2(i, j) ((long)nx * (j) + (i))
    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, &ra, &rb);
        /* resistive E = eta0 * J (:772-801) */
        for (int j = 2; j < ny - 1; j++)
            for (int i = 2; i < nx - 1; i++) {
                const long s = S2(i, j);
                double jx = +o_diff(odr, bz[S2(i, j - 2)], bz[S2(i, j - 1)], bz[S2(i, j)], bz[S2(i, j + 1)]) * idy;
                double jy = -o_diff(odr, bz[S2(i - 2, j)], bz[S2(i - 1, j)], bz[S2(i, j)], bz[S2(i + 1, j)]) * idx;
                double jz = +o_diff(odr, by[S2(i - 2, j)], by[S2(i - 1, j)], by[S2(i, j)], by[S2(i + 1, j)]) * idx
                            - o_diff(odr, bx[S2(i, j - 2)], bx[S2(i, j - 1)], bx[S2(i, j)], bx[S2(i, j + 1)]) * idy;
                ex[s] = eta0 * jx;
                ey[s] = eta0 * jy;
                ez[s] = eta0 * jz;
            }
        /* energy flux along X (:802-826) */
        for (int j = 2; j < ny - 2; j++)
            for (int i = 2; i < nx - 1; i++) {
                const long s = S2(i, j);
                double ep = ey[s];
                double bp = o_face2cen(odr, bz[S2(i - 2, j)], bz[S2(i - 1, j)], bz[S2(i, j)], bz[S2(i + 1, j)]);
                double em = 0.5 * (ez[s] + ez[S2(i, j + 1)]);
                double bm = 0.5 * (o_face2cen(odr, by[S2(i - 2, j)], by[S2(i - 1, j)], by[S2(i, j)], by[S2(i + 1, j)])
                                   + o_face2cen(odr, by[S2(i - 2, j + 1)], by[S2(i - 1, j + 1)], by[S2(i, j + 1)], by[S2(i + 1, j + 1)]));
                fx[s] = ep * bp - em * bm;
            }
        /* energy flux along Y (:827-852) */
        for (int j = 2; j < ny - 1; j++)
            for (int i = 2; i < nx - 2; i++) {
                const long s = S2(i, j);
                double ep = 0.5 * (ez[s] + ez[S2(i + 1, j)]);
                double bp = 0.5 * (o_face2cen(odr, bx[S2(i, j - 2)], bx[S2(i, j - 1)], bx[S2(i, j)], bx[S2(i, j + 1)])
                                   + o_face2cen(odr, bx[S2(i + 1, j - 2)], bx[S2(i + 1, j - 1)], bx[S2(i + 1, j)], bx[S2(i + 1, j + 1)]));
                double em = ex[s];
                double bm = o_face2cen(odr, bz[S2(i, j - 2)], bz[S2(i, j - 1)], bz[S2(i, j)], bz[S2(i, j + 1)]);
                fy[s] = ep * bp - em * bm;
            }
        /* CT Bx, By (:854-889) */
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff + 1; i++) {
                const long s = S2(i, j);
                double du = o_diff(odr, ez[S2(i, j - 1)], ez[s], ez[S2(i, j + 1)], ez[S2(i, j + 2)]);
                bx[s] = ra * ut[s] + rb * (bx[s] - dtdy * du);
            }
        for (int j = yoff; j < ny - yoff + 1; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                const long s = S2(i, j);
                double du = o_diff(odr, ez[S2(i - 1, j)], ez[s], ez[S2(i + 1, j)], ez[S2(i + 2, j)]);
                by[s] = ra * ut[n + s] + rb * (by[s] + dtdx * du);
            }
        /* Bz and energy (:890-921) */
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                const long s = S2(i, j);
                double d00 = o_diff(odr, ey[S2(i - 1, j)], ey[s], ey[S2(i + 1, j)], ey[S2(i + 2, j)]);
                double d01 = o_diff(odr, fx[S2(i - 1, j)], fx[s], fx[S2(i + 1, j)], fx[S2(i + 2, j)]);
                double d10 = o_diff(odr, ex[S2(i, j - 1)], ex[s], ex[S2(i, j + 1)], ex[S2(i, j + 2)]);
                double d11 = o_diff(odr, fy[S2(i, j - 1)], fy[s], fy[S2(i, j + 1)], fy[S2(i, j + 2)]);
                bz[s] = ra * ut[2 * n + s] + rb * (bz[s] - dtdx * d00 + dtdy * d10);
                en[s] = ra * ut[3 * n + s] + rb * (en[s] - dtdx * d01 - dtdy * d11);
            }
        double *p[3] = {bx, by, bz};
        o_bc2d_mpi(p, 3, stx + 5, sty + 5, dnx + 5, dny + 5, dnx[0], dny[0], nx, ny, xoff, yoff);
    }
    o_bc2d_mpi(&en, 1, stx + 4, sty + 4, dnx + 4, dny + 4, dnx[0], dny[0], nx, ny, xoff, yoff);
    free(ut); free(fx); free(fy); free(ex); free(ey); free(ez);
}

/* ns_viscous_2d (2D/MPI/MRX/mhd_fd_ct_2d.c:952-1174): viscous term of the 2D
   Navier-Stokes equation with uniform kinematic viscosity nu0. */
void oracle_ns_viscous_2d(const double *ro, double *mx, double *my, double *mz, double *en,
                          double nu0, double dt, double dx, double dy, int nx, int ny, int xoff,
                          int yoff, double gamma, int odr, int nrk, const int *dnx_in,
                          const int *dny_in)
{
    (void)gamma;
    const int *dnx = dnx_in ? dnx_in : o_zero8, *dny = dny_in ? dny_in : o_zero8;
    static const int st0[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const long n = (long)nx * ny;
    const double idx = 1. / dx, idy = 1. / dy, dtdx = dt * idx, dtdy = dt * idy;
    const double c2 = 2. / 3., c4 = 4. / 3.;
    double *ir = alloc_d(n), *ut = alloc_d(4 * n), *fx = alloc_d(4 * n), *fy = alloc_d(4 * n);
    for (long s = 0; s < n; s++) {
        ir[s] = 1.0 / ro[s];
        mx[s] *= ir[s];
        my[s] *= ir[s];
        mz[s] *= ir[s];
        ut[s] = mx[s];
        ut[n + s] = my[s];
        ut[2 * n + s] = mz[s];
        ut[3 * n + s] = en[s];
    }
    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, &ra, &rb);
        /* flux along X (:999-1043) */
        for (int j = 1; j < ny - 1; j++)
            for (int i = 2; i < nx - 1; i++) {
                const long s = S2(i, j);
                double ro0 = 0.5 * (ro[S2(i, j)] + ro[S2(i - 1, j)]);
                double rnu = ro0 * nu0;
                double vx0 = o_face2cen(odr, mx[S2(i - 2, j)], mx[S2(i - 1, j)], mx[s], mx[S2(i + 1, j)]);
                double vy0 = o_face2cen(odr, my[S2(i - 2, j)], my[S2(i - 1, j)], my[s], my[S2(i + 1, j)]);
                double vz0 = o_face2cen(odr, mz[S2(i - 2, j)], mz[S2(i - 1, j)], mz[s], mz[S2(i + 1, j)]);
                double dvxdx = o_diff(odr, mx[S2(i - 2, j)], mx[S2(i - 1, j)], mx[s], mx[S2(i + 1, j)]) * idx;
                double dvydx = o_diff(odr, my[S2(i - 2, j)], my[S2(i - 1, j)], my[s], my[S2(i + 1, j)]) * idx;
                double dvzdx = o_diff(odr, mz[S2(i - 2, j)], mz[S2(i - 1, j)], mz[s], mz[S2(i + 1, j)]) * idx;
                double dv[4];
                for (int m = 0; m < 4; m++)
                    dv[m] = 0.5 * (mx[S2(i - 2 + m, j + 1)] - mx[S2(i - 2 + m, j - 1)]);
                double dvxdy = o_face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idy;
                for (int m = 0; m < 4; m++)
                    dv[m] = 0.5 * (my[S2(i - 2 + m, j + 1)] - my[S2(i - 2 + m, j - 1)]);
                double dvydy = o_face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idy;
                fx[s] = -rnu * (c4 * dvxdx - c2 * dvydy);
                fx[n + s] = -rnu * (dvydx + dvxdy);
                fx[2 * n + s] = -rnu * (dvzdx);
                fx[3 * n + s] = fx[s] * vx0 + fx[n + s] * vy0 + fx[2 * n + s] * vz0;
            }
        /* flux along Y (:1045-1089) */
        for (int j = 2; j < ny - 1; j++)
            for (int i = 1; i < nx - 1; i++) {
                const long s = S2(i, j);
                double ro0 = 0.5 * (ro[S2(i, j)] + ro[S2(i, j - 1)]);
                double rnu = ro0 * nu0;
                double vx0 = o_face2cen(odr, mx[S2(i, j - 2)], mx[S2(i, j - 1)], mx[s], mx[S2(i, j + 1)]);
                double vy0 = o_face2cen(odr, my[S2(i, j - 2)], my[S2(i, j - 1)], my[s], my[S2(i, j + 1)]);
                double vz0 = o_face2cen(odr, mz[S2(i, j - 2)], mz[S2(i, j - 1)], mz[s], mz[S2(i, j + 1)]);
                double dvxdy = o_diff(odr, mx[S2(i, j - 2)], mx[S2(i, j - 1)], mx[s], mx[S2(i, j + 1)]) * idy;
                double dvydy = o_diff(odr, my[S2(i, j - 2)], my[S2(i, j - 1)], my[s], my[S2(i, j + 1)]) * idy;
                double dvzdy = o_diff(odr, mz[S2(i, j - 2)], mz[S2(i, j - 1)], mz[s], mz[S2(i, j + 1)]) * idy;
                double dv[4];
                for (int m = 0; m < 4; m++)
                    dv[m] = 0.5 * (mx[S2(i + 1, j - 2 + m)] - mx[S2(i - 1, j - 2 + m)]);
                double dvxdx = o_face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idx;
                for (int m = 0; m < 4; m++)
                    dv[m] = 0.5 * (my[S2(i + 1, j - 2 + m)] - my[S2(i - 1, j - 2 + m)]);
                double dvydx = o_face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idx;
                fy[s] = -rnu * (dvxdy + dvydx);
                fy[n + s] = -rnu * (c4 * dvydy - c2 * dvxdx);
                fy[2 * n + s] = -rnu * (dvzdy);
                fy[3 * n + s] = fy[s] * vx0 + fy[n + s] * vy0 + fy[2 * n + s] * vz0;
            }
        /* update (:1091-1139) */
        double *vel[3] = {mx, my, mz};
        for (int j = yoff; j < ny - yoff; j++)
            for (int i = xoff; i < nx - xoff; i++) {
                const long s = S2(i, j);
                double du[2][4];
                for (int c = 0; c < 4; c++) {
                    du[0][c] = o_diff(odr, fx[c * n + S2(i - 1, j)], fx[c * n + s], fx[c * n + S2(i + 1, j)], fx[c * n + S2(i + 2, j)]);
                    du[1][c] = o_diff(odr, fy[c * n + S2(i, j - 1)], fy[c * n + s], fy[c * n + S2(i, j + 1)], fy[c * n + S2(i, j + 2)]);
                }
                for (int c = 0; c < 3; c++)
                    vel[c][s] = ra * ut[c * n + s] + rb * (vel[c][s] - (dtdx * du[0][c] + dtdy * du[1][c]) * ir[s]);
                en[s] = ra * ut[3 * n + s] + rb * (en[s] - (dtdx * du[0][3] + dtdy * du[1][3]));
            }
        o_bc2d_mpi(vel, 3, st0, st0, dnx + 1, dny + 1, dnx[0], dny[0], nx, ny, xoff, yoff);
    }
    o_bc2d_mpi(&en, 1, st0, st0, dnx + 4, dny + 4, dnx[0], dny[0], nx, ny, xoff, yoff);
    for (long s = 0; s < n; s++) {
        mx[s] *= ro[s];
        my[s] *= ro[s];
        mz[s] *= ro[s];
    }
    free(ir); free(ut); free(fx); free(fy);
}
#undef S2

/* ---- anisotropic thermal conduction (2D/MPI/MRX/mhd_fd_ct_2d.c:1176-1456) ---- */

/* Periodic ghost exchange of one rank (mpi_sdrv2d, 2D/MPI/MRX/boundary.c:31-141):
   along an axis whose table entry 0 is zero. */
static void o_sdrv2d(double **p, int nn, int dnx0, int dny0, int nx, int ny, int xoff, int yoff)
{
    static const int z[8] = {0, 0, 0, 0, 0, 0, 0, 0};  /* no mirrors: periodic fills only */
    o_bc2d_mpi(p, nn, z, z, z, z, dnx0, dny0, nx, ny, xoff, yoff);
}

/* Mirror of one array along x / y (mpi_xbc2d / mpi_ybc2d, boundary.c:143-185):
   nothing when dn is zero. */
static void o_xbc2d(double *f, int nx, int ny, int xoff, int st, int dn)
{
    if (dn == 0) return;
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < xoff; i++) f[(long)nx * j + i] = dn * f[(long)nx * j + (2 * xoff - 1 + st) - i];
    for (int j = 0; j < ny; j++)
        for (int i = 0; i < xoff - st; i++)
            f[(long)nx * j + (nx - 1 - i)] = dn * f[(long)nx * j + (nx - 2 * xoff + st) + i];
}

static void o_ybc2d(double *f, int nx, int ny, int yoff, int st, int dn)
{
    if (dn == 0) return;
    for (int j = 0; j < yoff; j++)
        for (int i = 0; i < nx; i++) f[(long)nx * j + i] = dn * f[(long)nx * ((2 * yoff - 1 + st) - j) + i];
    for (int j = 0; j < yoff - st; j++)
        for (int i = 0; i < nx; i++)
            f[(long)nx * (ny - 1 - j) + i] = dn * f[(long)nx * ((ny - 2 * yoff + st) + j) + i];
}

/* mhd_e2p (:1176-1219): total energy -> pressure (direc +1) or back (-1) over
   [1, nx-2) x [1, ny-2), then the energy's boundary fill. */
static void o_e2p(const double *ro, const double *mx, const double *my, const double *mz,
                  double *en, const double *bx, const double *by, const double *bz, int nx,
                  int ny, int xoff, int yoff, double gamma, int direc, int odr, const int *dnx,
                  const int *dny)
{
    for (int j = 1; j < ny - 2; j++)
        for (int i = 1; i < nx - 2; i++) {
            const long s = (long)nx * j + i;
            const double iro = 1.0 / ro[s];
            const double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
            const double bxc = o_face2cen(odr, bx[s - 1], bx[s], bx[s + 1], bx[s + 2]);
            const double byc = o_face2cen(odr, by[s - nx], by[s], by[s + nx], by[s + 2 * nx]);
            const double bzc = bz[s];
            const double v2 = (vx * vx + vy * vy + vz * vz);
            const double b2 = (bxc * bxc + byc * byc + bzc * bzc);
            const double t0 = (gamma - 1) * (en[s] - 0.5 * (ro[s] * v2 + b2));
            const double t1 = en[s] / (gamma - 1) + 0.5 * (ro[s] * v2 + b2);
            en[s] = 0.5 * ((1 + direc) * t0 + (1 - direc) * t1);
        }
    o_sdrv2d(&en, 1, dnx[0], dny[0], nx, ny, xoff, yoff);
    o_xbc2d(en, nx, ny, xoff, 0, dnx[4]);
    o_ybc2d(en, nx, ny, yoff, 0, dny[4]);
}

/* diffusion2d_ani (:1221-1378): Crank-Nicolson step of
   g df/dt = div(g K grad f) with the full tensor K, solved by six-colour
   Gauss-Seidel sweeps until the summed |residual| falls below 1e-6 of the
   summed |rhs/denominator| or cmax sweeps ran.  The colours are independent
   sets of the stencil, so the sweep equals the reference's loop order.
   Returns the number of sweeps; *err = -1 when it reached cmax. */
static int o_diffusion2d_ani(double *f, const double *g, double *kxx, double *kyy, double *kxy,
                             double dt0, double dx, double dy, int nx, int ny, int xoff, int yoff,
                             int stx, int dnx, int sty, int dny, int dnx0, int dny0, int odr,
                             int cmax, int *err)
{
    const int od4 = (o_lin_odr(odr) - 1) / 2;
    const double idx2 = 1.0 / (dx * dx), idy2 = 1.0 / (dy * dy), idxy = 1.0 / (dx * dy);
    const double alpha = 0.5, beta = 1.0 - alpha, omega = 1.0, eps = 1e-6;
    const double d1 = 1.0 + 0.25 * od4, d2 = 1.0 * od4 / 12.0;
    const long n = (long)nx * ny;
    double *denom = alloc_d(n), *ig = alloc_d(n), *rhs = alloc_d(n);
    double anorm, anorm_f = 0.0;
    int cnt = 0;
    for (long s = 0; s < n; s++) {
        ig[s] = 1.0 / g[s];
        kxx[s] *= g[s];
        kyy[s] *= g[s];
        kxy[s] *= g[s];
    }
#define F(a, b) f[(long)nx * (b) + (a)]
    for (int j = 2; j < ny - 2; j++)
        for (int i = 2; i < nx - 2; i++) {
            const long s = (long)nx * j + i, sim = s - 1, sip = s + 1, sjm = s - nx, sjp = s + nx;
            const double k0 = 0.5 * (kxx[sim] + kxx[s]), k1 = 0.5 * (kxx[sip] + kxx[s]);
            const double k2 = 0.5 * (kyy[sjm] + kyy[s]), k3 = 0.5 * (kyy[sjp] + kyy[s]);
            const double dt = dt0 * ig[s];
            denom[s] = 1.0 / (1.0 + alpha * dt * d1 * (idx2 * (k0 + k1) + idy2 * (k2 + k3)));
            rhs[s] = f[s] + beta * dt *
                     ((+idx2 * (+k0 * (d1 * (f[sim] - f[s]) - d2 * (f[s - 2] - f[sip]))
                                + k1 * (d1 * (f[sip] - f[s]) - d2 * (f[s + 2] - f[sim])))
                       + idy2 * (+k2 * (d1 * (f[sjm] - f[s]) - d2 * (f[s - 2 * nx] - f[sjp]))
                                 + k3 * (d1 * (f[sjp] - f[s]) - d2 * (f[s + 2 * nx] - f[sjm]))))
                      + 0.25 * (+idxy * (+kxy[sjm] * (F(i - 1, j - 1) - F(i + 1, j - 1))
                                         + kxy[sjp] * (F(i + 1, j + 1) - F(i - 1, j + 1))
                                         + kxy[sim] * (F(i - 1, j - 1) - F(i - 1, j + 1))
                                         + kxy[sip] * (F(i + 1, j + 1) - F(i + 1, j - 1)))));
            anorm_f += fabs(rhs[s] * denom[s]);
        }
    do {
        anorm = 0.0;
        for (int py = 0; py < 2; py++)
            for (int px = 0; px < 3; px++)
                for (int j = 2 + py; j < ny - 2; j += 2)
                    for (int i = 4 - ((j + px) % 3); i < nx - 2; i += 3) {
                        const long s = (long)nx * j + i, sim = s - 1, sip = s + 1, sjm = s - nx,
                                   sjp = s + nx;
                        const double k0 = 0.5 * (kxx[sim] + kxx[s]), k1 = 0.5 * (kxx[sip] + kxx[s]);
                        const double k2 = 0.5 * (kyy[sjm] + kyy[s]), k3 = 0.5 * (kyy[sjp] + kyy[s]);
                        const double dt = dt0 * ig[s];
                        const double resid =
                            (alpha * dt *
                                 ((+idx2 * (+k0 * (d1 * f[sim] - d2 * (f[s - 2] - f[sip]))
                                            + k1 * (d1 * f[sip] - d2 * (f[s + 2] - f[sim])))
                                   + idy2 * (+k2 * (d1 * f[sjm] - d2 * (f[s - 2 * nx] - f[sjp]))
                                             + k3 * (d1 * f[sjp] - d2 * (f[s + 2 * nx] - f[sjm]))))
                                  + 0.25 * (+idxy * (+kxy[sjm] * (F(i - 1, j - 1) - F(i + 1, j - 1))
                                                     + kxy[sjp] * (F(i + 1, j + 1) - F(i - 1, j + 1))
                                                     + kxy[sim] * (F(i - 1, j - 1) - F(i - 1, j + 1))
                                                     + kxy[sip] * (F(i + 1, j + 1) - F(i + 1, j - 1)))))
                             + rhs[s]) * denom[s] - f[s];
                        anorm += fabs(resid);
                        f[s] += omega * resid;
                    }
        o_sdrv2d(&f, 1, dnx0, dny0, nx, ny, xoff, yoff);
        o_xbc2d(f, nx, ny, xoff, stx, dnx);
        o_ybc2d(f, nx, ny, yoff, sty, dny);
        cnt++;
    } while ((anorm > eps * anorm_f) && (cnt < cmax));
#undef F
    for (long s = 0; s < n; s++) {
        kxx[s] *= ig[s];
        kyy[s] *= ig[s];
        kxy[s] *= ig[s];
    }
    if (cnt == cmax) *err = -1;
    free(denom); free(ig); free(rhs);
    return cnt;
}

/* t_conduction (:1380-1456): anisotropic heat conduction along B with
   conductivity kk0, implicit (Crank-Nicolson) in the temperature p/rho.
   Returns the Gauss-Seidel sweep count; *err = -1 when it did not converge
   within cmax sweeps (the reference then aborts the run). */
int oracle_t_conduction(const double *ro, const double *mx, const double *my, const double *mz,
                        double *en, const double *bx, const double *by, const double *bz,
                        double kk0, double dt, double dx, double dy, int nx, int ny, int xoff,
                        int yoff, double gamma, int odr, const int *dnx_in, const int *dny_in,
                        int cmax, int *err)
{
    const int *dnx = dnx_in ? dnx_in : o_zero8, *dny = dny_in ? dny_in : o_zero8;
    const long n = (long)nx * ny;
    const double eps = 1e-6;
    double *kxx = alloc_d(n), *kyy = alloc_d(n), *kxy = alloc_d(n);
    *err = 0;
    for (int j = 1; j < ny - 2; j++)
        for (int i = 1; i < nx - 2; i++) {
            const long s = (long)nx * j + i;
            const double bxc = o_face2cen(odr, bx[s - 1], bx[s], bx[s + 1], bx[s + 2]);
            const double byc = o_face2cen(odr, by[s - nx], by[s], by[s + nx], by[s + 2 * nx]);
            const double bzc = bz[s];
            const double ib2 = 1.0 / (bxc * bxc + byc * byc + bzc * bzc + eps);
            kxx[s] = kk0 * (bxc * bxc + eps) * ib2;
            kyy[s] = kk0 * (byc * byc + eps) * ib2;
            kxy[s] = kk0 * (bxc * byc) * ib2;
        }
    double *p[3] = {kxx, kyy, kxy};
    o_sdrv2d(p, 3, dnx[0], dny[0], nx, ny, xoff, yoff);
    o_xbc2d(kxx, nx, ny, xoff, 0, dnx[5] * dnx[5]);
    o_xbc2d(kyy, nx, ny, xoff, 0, dnx[6] * dnx[6]);
    o_xbc2d(kxy, nx, ny, xoff, 0, dnx[5] * dnx[6]);
    o_ybc2d(kxx, nx, ny, yoff, 0, dny[5] * dny[5]);
    o_ybc2d(kyy, nx, ny, yoff, 0, dny[6] * dny[6]);
    o_ybc2d(kxy, nx, ny, yoff, 0, dny[5] * dny[6]);
    o_e2p(ro, mx, my, mz, en, bx, by, bz, nx, ny, xoff, yoff, gamma, +1, odr, dnx, dny);
    for (long s = 0; s < n; s++) en[s] /= ro[s];
    const int cnt = o_diffusion2d_ani(en, ro, kxx, kyy, kxy, dt, dx, dy, nx, ny, xoff, yoff, 0, +0,
                                      0, +1, dnx[0], dny[0], odr, cmax, err);
    for (long s = 0; s < n; s++) en[s] *= ro[s];
    o_e2p(ro, mx, my, mz, en, bx, by, bz, nx, ny, xoff, yoff, gamma, -1, odr, dnx, dny);
    free(kxx); free(kyy); free(kxy);
    return cnt;
}

/* inj_ro (2D/MPI/RMI/inj_ro.hpp:1-58): the RMI problem's inflow through the
   upper boundary, set before each step on the rows [ny-yoff, ny) of the top
   rank: uniform upstream state (velocity vy_1 - vref), density ro_3 plus
   dro3 * (2u - 1) with u the draws (double)random()/RAND_MAX in loop order
   (noise, or none when NULL); By on the boundary face row j = ny-yoff keeps
   its value (CT spacing).  Then the main loop's periodic exchange
   (mpi_sdrv2d of the 8 arrays, main.cpp:50-54). */
void oracle_inj_ro(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                   double *by, double *bz, int nx, int ny, int xoff, int yoff, double ro_3,
                   double dro3, double vy_1, double bx_1, double by_1, double bz_1, double pr_1,
                   double vref, double gam, const double *noise, const int *dnx_in,
                   const int *dny_in)
{
    const int *dnx = dnx_in ? dnx_in : o_zero8, *dny = dny_in ? dny_in : o_zero8;
    long k = 0;
    for (int j = ny - yoff; j < ny; j++) {
        const int ctyflg = (j == (ny - yoff));
        for (int i = 0; i < nx; i++) {
            const long ss = (long)nx * j + i;
            ro[ss] = ro_3;
            if (noise) ro[ss] += dro3 * (noise[k++] - 0.5) * 2.0;
            double vx = 0, vy = vy_1, vz = 0;
            vy -= vref;
            double bxc, byc, bzc;
            bx[ss] = bxc = bx_1;
            by[ss] = ctyflg ? by[ss] : by_1;
            byc = by_1;
            bz[ss] = bzc = bz_1;
            const double b2 = bxc * bxc + byc * byc + bzc * bzc;
            const double pr = pr_1;
            mx[ss] = ro[ss] * vx;
            my[ss] = ro[ss] * vy;
            mz[ss] = ro[ss] * vz;
            en[ss] = pr / (gam - 1) + 0.5 * (ro[ss] * (vx * vx + vy * vy + vz * vz) + b2);
        }
    }
    double *p[8] = {ro, mx, my, mz, en, bx, by, bz};
    o_sdrv2d(p, 8, dnx[0], dny[0], nx, ny, xoff, yoff);
}

void oracle_fd_ct_3d(double *ro, double *mx, double *my, double *mz, double *en, double *bx,
                     double *by, double *bz, double dt, double dx, double dy, double dz,
                     int nx, int ny, int nz, int xoff, int yoff, int zoff, double gamma,
                     int odr, int flx, int nrk)
{
    oracle_fd_ct_3d_bc(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, dz, nx, ny, nz, xoff, yoff,
                       zoff, gamma, odr, flx, nrk, NULL, NULL, NULL);
}

