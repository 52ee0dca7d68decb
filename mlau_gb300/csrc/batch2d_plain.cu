// Batched 2D engine, plain FP64 arithmetic: each phase evaluates exactly the
// expressions of the single-instance plain 2D kernels (plain2d.cu), so every
// instance advances bit for bit like mhd_fd_ct_2d (2D/SERIAL/OTvortex/
// mhd_fd_ct_2d.c:91-660) with the CFL dt of 2D/SERIAL/OTvortex/cflcheck.hpp.
// Built with --fmad=false like the other plain kernels.
#include "batch2d.cuh"
#include "stencil.cuh"

namespace mlau {
namespace {

__device__ void pp_cfl(const BArgs &A, int nt, const BTile *tiles)
{
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const BTile tl = tiles[t];
        BInst &I = A.inst[tl.inst];
        double vt = 0.0;
        if (I.active) {
            const int i = tl.x0 + threadIdx.x, j = tl.y0 + threadIdx.y;
            if (i >= I.off && i < I.nx - I.off && j >= I.off && j < I.ny - I.off) {
                const long long s = I.base + (long long)I.nx * j + i;
                const double *const *S = A.a.s;
                const double ro = S[0][s];
                const double iro = 1.0 / ro;
                const double vx = S[1][s] * iro, vy = S[2][s] * iro, vz = S[3][s] * iro;
                const double v2 = vx * vx + vy * vy + vz * vz;
                const double bxc = 0.5 * (S[5][s] + S[5][s + 1]);
                const double byc = 0.5 * (S[6][s] + S[6][s + I.nx]);
                const double bzc = S[7][s];
                const double b2 = bxc * bxc + byc * byc + bzc * bzc;
                const double pr = (I.gamma - 1) * (S[4][s] - 0.5 * (ro * v2 + b2));
                const double cf = sqrt((0.5 * I.gamma * (2.0 * pr) + b2) / (ro));
                const double v = sqrt(vx * vx + vy * vy) + cf;
                vt = (v == v && I.dt_fixed <= 0.0) ? v : 0.0;
                batch_check(I, ro, pr);
            }
        }
        batch_vmax(I, vt);
    }
}

__device__ void pp_prep(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const long long sy = I.nx;
        // cell B from the face stencils at the cell's boundary source (with the
        // tables: each component at its own source, times its sign)
        long long wx, wy;
        double gx = 1.0, gy = 1.0;
        if (I.walls) {
            wx = bsrc(I, i, j, 0, 0, I.bcx[5], I.bcy[5], &gx);
            wy = bsrc(I, i, j, 0, 0, I.bcx[6], I.bcy[6], &gy);
        } else {
            wx = wy = I.base + sy * bwrap(j, I.ny, I.off) + bwrap(i, I.nx, I.off);
        }
        const double *bx = a.s[5], *by = a.s[6];
        const double cx = gx * face2cen(A.odr, bx[wx - 1], bx[wx], bx[wx + 1], bx[wx + 2]);
        const double cy = gy * face2cen(A.odr, by[wy - sy], by[wy], by[wy + sy], by[wy + 2 * sy]);
        const double ro = a.s[0][c];
        const double iro = 1.0 / ro;
        const double vx = a.s[1][c] * iro, vy = a.s[2][c] * iro, vz = a.s[3][c] * iro;
        const double bz = a.s[7][c];
        const double v2 = (vx * vx + vy * vy + vz * vz);
        const double b2 = (cx * cx + cy * cy + bz * bz);
        const double pr = (I.gamma - 1) * (a.s[4][c] - 0.5 * (ro * v2 + b2));
        a.vx[c] = vx;
        a.vy[c] = vy;
        a.vz[c] = vz;
        a.pr[c] = pr;
        a.m2[c] = v2 / (I.gamma * pr * iro);
        a.cx[c] = cx;
        a.cy[c] = cy;
        if (rk == 0)
            for (int v = 0; v < 8; v++) a.u0[v][c] = a.s[v][c];
    });
}

__device__ void pp_aux(const BArgs &A, int nt, const BTile *tl)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const long long sy = I.nx;
        a.ct[c] = (i >= 1 && j >= 1) ? ct_weight(a.vx, a.vy, a.s[0], a.s[5], a.s[6], c, sy, 1, sy, 1)
                                     : 0.5;
        if (I.walls) {  // signs of the sensors' fill (mhd_fd_ct_2d.c:262-271)
            double g0 = 1.0, g1 = 1.0;
            const long long w0 = bsrc(I, i, j, 0, 0, -I.bcx[1], I.bcy[1], &g0);
            const long long w1 = bsrc(I, i, j, 0, 0, I.bcx[2], -I.bcy[2], &g1);
            a.dv[0][c] = g0 * vmin((a.vx[w0 + 1] - a.vx[w0]), (a.vx[w0] - a.vx[w0 - 1]));
            a.dv[1][c] = g1 * vmin((a.vy[w1 + sy] - a.vy[w1]), (a.vy[w1] - a.vy[w1 - sy]));
            return;
        }
        const long long w = I.base + sy * bwrap(j, I.ny, I.off) + bwrap(i, I.nx, I.off);
        a.dv[0][c] = vmin((a.vx[w + 1] - a.vx[w]), (a.vx[w] - a.vx[w - 1]));
        a.dv[1][c] = vmin((a.vy[w + sy] - a.vy[w]), (a.vy[w] - a.vy[w - sy]));
    });
}

// X (D=0): (vn, vt, vu) = (vx, vy, vz), (bt, bu) = (cy, bz), By flux split.
// Y (D=1): (vy, vz, vx), (bz, cx), Bx flux split.
__device__ void pp_rec(const BArgs &A, int nt, const BTile *tl, int D)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const int len = D == 0 ? I.nx : I.ny, pos = D == 0 ? i : j;
        if (pos < 2 || pos >= len - 2) return;
        const long long st = D == 0 ? 1 : I.nx;
        const double *vn = D == 0 ? a.vx : a.vy, *vt = D == 0 ? a.vy : a.vz,
                     *vu = D == 0 ? a.vz : a.vx;
        const double *cn = D == 0 ? a.cx : a.cy, *ct = D == 0 ? a.cy : a.s[7],
                     *cu = D == 0 ? a.s[7] : a.cx;
        const double *bface = D == 0 ? a.s[5] : a.s[6];
        double q[7][5];
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const long long s = c + st * (m - 2);
            q[0][m] = a.s[0][s];
            q[1][m] = vn[s];
            q[2][m] = vt[s];
            q[3][m] = vu[s];
            q[4][m] = ct[s];
            q[5][m] = cu[s];
            q[6][m] = a.pr[s];
        }
        double ul[7], ur[7];
        if (vmax(a.m2[c - st], vmax(a.m2[c], a.m2[c + st])) >= 1.0)
            reconst_full(A.odr, q, cn[c], I.gamma, ul, ur);
        else
            reconst_alfven(A.odr, q, cn[c], I.gamma, ul, ur);
#pragma unroll
        for (int n = 0; n < 7; n++) {
            a.ul[n][c + st] = ul[n];
            a.ur[n][c] = ur[n];
        }
        const double *bt = D == 1 ? cu : ct, *vv = D == 1 ? vu : vt;
        double a5[5], t5[5];
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const long long s = c + st * (m - 2);
            a5[m] = bt[s] * vn[s];
            t5[m] = vv[s];
        }
        a.ul[7][c + st] = lin_l(A.odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                          - bface[c + st] * lin_l(A.odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
        a.ur[7][c] = lin_r(A.odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                     - bface[c] * lin_r(A.odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
    });
}

__device__ void pp_flux(const BArgs &A, int nt, const BTile *tl, int D)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const int len = D == 0 ? I.nx : I.ny, pos = D == 0 ? i : j;
        if (pos < 3 || pos >= len - 2) return;
        const long long st = D == 0 ? 1 : I.nx;
        const double *vn = D == 0 ? a.vx : a.vy, *dvt = D == 0 ? a.dv[1] : a.dv[0];
        const double *bface = D == 0 ? a.s[5] : a.s[6];
        double L[7], R[7], F[7];
#pragma unroll
        for (int n = 0; n < 7; n++) {
            L[n] = a.ul[n][c];
            R[n] = a.ur[n][c];
        }
        const double bn = 0.5 * (bface[c] + bface[c]);
        riemann(I.flux, L, R, bn, I.gamma, (vn[c] - vn[c - st]), vmin(dvt[c - st], dvt[c]), F);
        const double fc = 0.5 * (a.ul[7][c] + a.ur[7][c]);
        F[4 + D] -= fc;
#pragma unroll
        for (int n = 0; n < 7; n++) a.F[D][n][c] = F[n];
        a.FC[D][c] = fc;
    });
}

__device__ void pp_emf(const BArgs &A, int nt, const BTile *tl)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        double ez = 0.0;
        if (i >= 3 && i < I.nx - 2 && j >= 3 && j < I.ny - 2) {
            const double w = a.ct[c];
            ez = (0.0 + emf_part(a.F[0][4], a.FC[0], (1.0 - w), -1.0, c, I.nx, A.odr))
                 + emf_part(a.F[1][5], a.FC[1], w, +1.0, c, 1, A.odr);
        }
        a.ez[c] = ez;
    });
}

__device__ void pp_update(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    // rk_fac of the reference for R_K=3 (mhd_fd_ct_2d.c:110)
    const double rkf[3][2] = {{0.0, 1.0}, {0.5 + (3 - 2) * 0.25, 0.5 - (3 - 2) * 0.25},
                              {1. / 3., 2. / 3.}};
    const double ra = rkf[rk][0], rb = rkf[rk][1];
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        if (i < I.off || i >= I.nx - I.off || j < I.off || j >= I.ny - I.off) return;
        const long long sy = I.nx;
        const double dtdx = I.dt / I.dx, dtdy = I.dt / I.dy;
        const int sv[6] = {0, 1, 2, 3, 7, 4};
        const int cX[6] = {0, 1, 2, 3, 5, 6}, cY[6] = {0, 3, 1, 2, 4, 6};
        double out[8];
#pragma unroll
        for (int v = 0; v < 6; v++) {
            const double *fx = a.F[0][cX[v]], *fy = a.F[1][cY[v]];
            const double d0 = fdiff(A.odr, fx[c - 1], fx[c], fx[c + 1], fx[c + 2]);
            const double d1 = fdiff(A.odr, fy[c - sy], fy[c], fy[c + sy], fy[c + 2 * sy]);
            out[sv[v]] = ra * a.u0[sv[v]][c] + rb * (a.s[sv[v]][c] - dtdx * d0 - dtdy * d1);
        }
        const double *ez = a.ez;
        {
            const double dd = fdiff(A.odr, ez[c - sy], ez[c], ez[c + sy], ez[c + 2 * sy]);
            out[5] = ra * a.u0[5][c] + rb * (a.s[5][c] - dtdy * dd);
        }
        {
            const double dd = fdiff(A.odr, ez[c - 1], ez[c], ez[c + 1], ez[c + 2]);
            out[6] = ra * a.u0[6][c] + rb * (a.s[6][c] + dtdx * dd);
        }
        if (I.walls) {  // the boundary phases fill the ghosts
#pragma unroll
            for (int v = 0; v < 8; v++) a.s[v][c] = out[v];
            return;
        }
        const int Nx = I.nx - 2 * I.off, Ny = I.ny - 2 * I.off;
        const int is[3] = {i, i < 2 * I.off ? i + Nx : -1, i >= Nx ? i - Nx : -1};
        const int js[3] = {j, j < 2 * I.off ? j + Ny : -1, j >= Ny ? j - Ny : -1};
        for (int bb = 0; bb < 3; bb++) {
            if (js[bb] < 0) continue;
            for (int aa = 0; aa < 3; aa++) {
                if (is[aa] < 0) continue;
                const long long t = I.base + sy * js[bb] + is[aa];
#pragma unroll
                for (int v = 0; v < 8; v++) a.s[v][t] = out[v];
            }
        }
    });
}

// Instances with tables: the right boundary faces the 2D driver's CT loops
// also update (Bx at i = nx-off, By at j = ny-off, mhd_fd_ct_2d.c:593-632),
// where that axis mirrors the face array ...
__device__ void pp_face(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    const double rkf[3][2] = {{0.0, 1.0}, {0.5 + (3 - 2) * 0.25, 0.5 - (3 - 2) * 0.25},
                              {1. / 3., 2. / 3.}};
    const double ra = rkf[rk][0], rb = rkf[rk][1];
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        if (!I.walls) return;
        const long long sy = I.nx;
        const double *ez = a.ez;
        if (I.bcx[5] != 0 && i == I.nx - I.off && j >= I.off && j < I.ny - I.off) {
            const double dd = fdiff(A.odr, ez[c - sy], ez[c], ez[c + sy], ez[c + 2 * sy]);
            a.s[5][c] = ra * a.u0[5][c] + rb * (a.s[5][c] - (I.dt / I.dy) * dd);
        }
        if (I.bcy[6] != 0 && j == I.ny - I.off && i >= I.off && i < I.nx - I.off) {
            const double dd = fdiff(A.odr, ez[c - 1], ez[c], ez[c + 1], ez[c + 2]);
            a.s[6][c] = ra * a.u0[6][c] + rb * (a.s[6][c] + (I.dt / I.dx) * dd);
        }
    });
}

// ... then every ghost takes its boundary source times the signs (:636-638).
__device__ void pp_bc(const BArgs &A, int nt, const BTile *tl)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        if (!I.walls) return;
        if (i >= I.off && i < I.nx - I.off && j >= I.off && j < I.ny - I.off) return;
#pragma unroll
        for (int v = 0; v < 8; v++) {
            double g = 1.0;
            const long long w = bsrc(I, i, j, v == 5, v == 6, I.bcx[v], I.bcy[v], &g);
            if (w != c) a.s[v][c] = g * a.s[v][w];
        }
    });
}

__global__ void __launch_bounds__(256) kb_step_plain(BArgs A)
{
    const int nt = A.sync->ntiles;
    const BTile *tl = A.sync->tiles;
    pp_cfl(A, nt, tl);
    if (grid_barrier(A.sync, A.nblocks)) return;
    batch_dt(A);
    if (grid_barrier(A.sync, A.nblocks)) return;
    for (int rk = 0; rk < 3; rk++) {
        pp_prep(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        pp_aux(A, nt, tl);
        if (grid_barrier(A.sync, A.nblocks)) return;
        for (int D = 0; D < 2; D++) {
            pp_rec(A, nt, tl, D);
            if (grid_barrier(A.sync, A.nblocks)) return;
            pp_flux(A, nt, tl, D);
            if (grid_barrier(A.sync, A.nblocks)) return;
        }
        pp_emf(A, nt, tl);
        if (grid_barrier(A.sync, A.nblocks)) return;
        pp_update(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        if (A.sync->walls) {
            pp_face(A, nt, tl, rk);
            if (grid_barrier(A.sync, A.nblocks)) return;
            pp_bc(A, nt, tl);
            if (grid_barrier(A.sync, A.nblocks)) return;
        }
    }
    batch_advance(A);
}

}  // namespace

const void *batch2d_plain_kernel() { return (const void *)kb_step_plain; }

}  // namespace mlau
