// Batched 1D instances, plain FP64: every phase evaluates exactly the
// expressions of the single-instance 1D kernels (plain1d.cu), so each
// instance advances bit for bit like mhd_fd4c_1d (1D/SERIAL/shock/
// mhd_fd4c_1d.c:60-271, open boundaries via openbc1d_mhd.c:21-175, or the
// periodic boundaries of 1D/SERIAL/wave).  As in 1D/SERIAL/shock/main.cpp:
// 113-128 the time step is fixed once, from the initial state
// (cfl*dx/max(1, max|vx|+cf) over all cells); an instance retires after the
// step that reaches its end time (the last step is not clipped).
//
// 1D instances use the engine's host side (batch2d.cu) with tiles of TW
// cells along x (ny = 1).  State slots: 0 ro, 1 mx, 2 my, 3 mz, 4 en, 6 by,
// 7 bz.  Each instance has its own flux, boundary, RK stage count (1-3), Bx,
// gamma, CFL number and end time; the reconstruction order is the batch's.
#include "batch2d.cuh"
#include "stencil.cuh"

namespace mlau {
namespace {

__device__ __forceinline__ double bx_of(const BInst &I) { return I.bx; }

// one-off dt of the reference 1D driver's main, at an instance's first step
__device__ void q_dt0(const BArgs &A, int nt, const BTile *tiles)
{
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const BTile tl = tiles[t];
        BInst &I = A.inst[tl.inst];
        double vt = 0.0;
        if (I.active && I.steps == 0 && I.dt_fixed <= 0.0) {
            const int i = tl.x0 + threadIdx.x;
            if (i < I.nx) {
                const long long s = I.base + i;
                const double *const *S = A.a.s;
                const double bx = bx_of(I);
                const double iro = 1.0 / S[0][s];
                const double vx = S[1][s] * iro, vy = S[2][s] * iro, vz = S[3][s] * iro;
                const double v2 = vx * vx + vy * vy + vz * vz;
                const double b2 = bx * bx + S[6][s] * S[6][s] + S[7][s] * S[7][s];
                const double pr = (I.gamma - 1) * (S[4][s] - 0.5 * (S[0][s] * v2 + b2));
                const double cf = sqrt((I.gamma * pr + b2) * iro);
                const double v = fabs(vx) + cf;
                vt = (v == v) ? v : 0.0;
            }
        }
        batch_vmax(I, vt);
    }
}

__device__ void q_dt(const BArgs &A)
{
    const int g = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    for (int n = g; n < A.ninst; n += gridDim.x * blockDim.x * blockDim.y) {
        BInst &I = A.inst[n];
        if (!I.active) continue;
        if (I.steps == 0 && I.dt_fixed <= 0.0) {
            const double vm = __longlong_as_double((long long)I.vkey);
            const double vmax = (vm > 1.0) ? vm : 1.0;  // floor 1.0 as in the reference main
            I.dt_fixed = I.cfl * I.dx / vmax;
        }
        I.dt = I.dt_fixed;
    }
}

// Visit the cells of every active instance that has RK stage `rk`.
template <class Body>
__device__ __forceinline__ void for_cells1(const BArgs &A, int nt, const BTile *tiles, int rk,
                                           Body body)
{
    for (int t = blockIdx.x; t < nt; t += gridDim.x) {
        const BTile tl = tiles[t];
        const BInst &I = A.inst[tl.inst];
        if (!I.active || rk >= I.nrk) continue;
        const int i = tl.x0 + threadIdx.x;
        if (i >= I.nx) continue;
        body(I, i, I.base);
    }
}

__device__ void q_prim(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells1(A, nt, tl, rk, [&](const BInst &cI, int i, long long b) {
        BInst &I = const_cast<BInst &>(cI);
        const long long s = b + i;
        const double bx = bx_of(I);
        const double ro = a.s[0][s], iro = 1.0 / ro;
        const double vx = a.s[1][s] * iro, vy = a.s[2][s] * iro, vz = a.s[3][s] * iro;
        const double by = a.s[6][s], bz = a.s[7][s];
        const double v2 = vx * vx + vy * vy + vz * vz;
        const double b2 = bx * bx + by * by + bz * bz;
        a.vx[s] = vx;
        a.vy[s] = vy;
        a.vz[s] = vz;
        a.pr[s] = (I.gamma - 1) * (a.s[4][s] - 0.5 * (ro * v2 + b2));
        if (rk == 0 && i >= I.off && i < I.nx - I.off) batch_check(I, ro, a.pr[s]);
        if (rk == 0)
            for (int v = 0; v < 8; v++)
                if (v != 5) a.u0[v][s] = a.s[v][s];
    });
}

__device__ void q_rec(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells1(A, nt, tl, rk, [&](const BInst &I, int i, long long b) {
        if (i < 2 || i >= I.nx - 2) return;
        const double bx = bx_of(I);
        double q[7][5];
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const long long s = b + i + m - 2;
            q[0][m] = a.s[0][s];
            q[1][m] = a.vx[s];
            q[2][m] = a.vy[s];
            q[3][m] = a.vz[s];
            q[4][m] = a.s[6][s];
            q[5][m] = a.s[7][s];
            q[6][m] = a.pr[s];
        }
        double mach[3];
#pragma unroll
        for (int t = 0; t < 3; t++) {
            const double c2 = I.gamma * q[6][1 + t] / q[0][1 + t];
            const double v2 = q[1][1 + t] * q[1][1 + t] + q[2][1 + t] * q[2][1 + t]
                              + q[3][1 + t] * q[3][1 + t];
            mach[t] = v2 / c2;
        }
        double ul[7], ur[7];
        if (vmax(mach[0], vmax(mach[1], mach[2])) >= 1.0) reconst_full(A.odr, q, bx, I.gamma, ul, ur);
        else reconst_alfven(A.odr, q, bx, I.gamma, ul, ur);
        // face states: ul at index b+i+1 (left of face i+1/2), ur at b+i
#pragma unroll
        for (int n = 0; n < 7; n++) {
            a.ul[n][b + i + 1] = ul[n];
            a.ur[n][b + i] = ur[n];
        }
    });
}

__device__ void q_flux(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells1(A, nt, tl, rk, [&](const BInst &I, int i, long long b) {
        if (i < 3 || i >= I.nx - 2) return;
        const long long s = b + i;
        double L[7], R[7], F[7];
#pragma unroll
        for (int n = 0; n < 7; n++) {
            L[n] = a.ul[n][s];
            R[n] = a.ur[n][s];
        }
        riemann(I.flux, L, R, bx_of(I), I.gamma, (a.vx[s] - a.vx[s - 1]), 0.0, F);
#pragma unroll
        for (int n = 0; n < 7; n++) a.F[0][n][s] = F[n];
    });
}

// openbc1d_mhd at stage 0 (1D/SERIAL/shock/openbc1d_mhd.c:21-175); one
// thread per instance, both sides, in the reference's order.
__device__ void q_openbc(const BArgs &A)
{
    const int g = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    for (int n = g; n < A.ninst; n += gridDim.x * blockDim.x * blockDim.y) {
        const BInst &I = A.inst[n];
        if (!I.active || I.bc != MLAU_BC1D_OPEN) continue;
        const long long b = I.base;
        double *ro = A.a.s[0] + b, *mx = A.a.s[1] + b, *my = A.a.s[2] + b, *mz = A.a.s[3] + b,
               *en = A.a.s[4] + b, *by = A.a.s[6] + b, *bz = A.a.s[7] + b;
        const int nx = I.nx, xoff = I.off;
        const double bx = bx_of(I), bx2 = bx * bx, dtdx = I.dt / I.dx, gamma = I.gamma;
        for (int side = 0; side <= 1; side++) {
            const int sgn = side ? -1 : 1;
            const int si = side ? (nx - xoff - 1) : xoff;
            const int so = si - sgn;
            double q[2][7];
            for (int t = 0; t < 2; t++) {
                const int s = t ? so : si;
                const double r = ro[s], iro = 1.0 / r;
                const double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
                const double v2 = vx * vx + vy * vy + vz * vz;
                const double b2 = bx * bx + by[s] * by[s] + bz[s] * bz[s];
                q[t][0] = r;
                q[t][1] = vx;
                q[t][2] = vy;
                q[t][3] = vz;
                q[t][4] = by[s];
                q[t][5] = bz[s];
                q[t][6] = (gamma - 1) * (en[s] - 0.5 * (r * v2 + b2));
            }
            Eigen7<double> E;
            eigen_full(0.5 * (q[0][0] + q[1][0]), 0.5 * (q[0][1] + q[1][1]), 0.5 * (bx + bx),
                       0.5 * (q[0][4] + q[1][4]), 0.5 * (q[0][5] + q[1][5]),
                       0.5 * (q[0][6] + q[1][6]), gamma, E);
            double w0[7], w1[7];
            proj_full(E, q[0][0], q[0][1], q[0][2], q[0][3], q[0][4], q[0][5], q[0][6], w0);
            proj_full(E, q[1][0], q[1][1], q[1][2], q[1][3], q[1][4], q[1][5], q[1][6], w1);
            for (int m = 0; m < 7; m++) {
                const double c = sgn * E.lam[m];
                w1[m] = (c > 0) ? w1[m] : (1 + c * dtdx) * w1[m] - c * dtdx * w0[m];
            }
            double p[7];
            back_full(E, w1, p);
            ro[so] = p[0];
            mx[so] = p[1];
            my[so] = p[2];
            mz[so] = p[3];
            by[so] = p[4];
            bz[so] = p[5];
            en[so] = p[6];
            const double v2 = mx[so] * mx[so] + my[so] * my[so] + mz[so] * mz[so];
            const double b2 = bx2 + by[so] * by[so] + bz[so] * bz[so];
            en[so] = en[so] / (gamma - 1.0) + 0.5 * (ro[so] * v2 + b2);
            mx[so] *= ro[so];
            my[so] *= ro[so];
            mz[so] *= ro[so];
            for (int j = 0; j < xoff - 1; j++) {
                const int s = side * (nx - 1) + sgn * j;
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
}

__device__ void q_update(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells1(A, nt, tl, rk, [&](const BInst &I, int i, long long b) {
        if (i < I.off || i >= I.nx - I.off) return;
        // SSP-RK coefficients of stage rk for an nrk-stage scheme
        const double ra = (rk == 0) ? 0.0 : (rk == 1) ? 0.5 + (I.nrk - 2) * 0.25 : 1. / 3.;
        const double rb = (rk == 0) ? 1.0 : (rk == 1) ? 0.5 - (I.nrk - 2) * 0.25 : 2. / 3.;
        const long long s = b + i;
        const double dtdx = I.dt / I.dx;
        const int sv[7] = {0, 1, 2, 3, 6, 7, 4};  // flux order (ro, mx, my, mz, by, bz, en)
        double out[7];
#pragma unroll
        for (int v = 0; v < 7; v++) {
            const double *fx = a.F[0][v];
            const double dd = fdiff(A.odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
            out[v] = ra * a.u0[sv[v]][s] + rb * (a.s[sv[v]][s] - dtdx * dd);
        }
        const bool periodic = I.bc == MLAU_BC1D_PERIODIC;
        const int N = I.nx - 2 * I.off;
        const int im[3] = {i, (periodic && i < 2 * I.off) ? i + N : -1,
                           (periodic && i >= N) ? i - N : -1};
        for (int k = 0; k < 3; k++) {
            if (im[k] < 0) continue;
#pragma unroll
            for (int v = 0; v < 7; v++) a.s[sv[v]][b + im[k]] = out[v];
        }
    });
}

__device__ void q_advance(const BArgs &A)
{
    const int g = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    for (int n = g; n < A.ninst; n += gridDim.x * blockDim.x * blockDim.y) {
        BInst &I = A.inst[n];
        I.vkey = 0;
        if (!I.active) continue;
        I.t += I.dt;
        I.steps += 1;
        // the last step is not clipped; a bad state retires the instance
        if (I.t >= I.t_end || !(I.dt > 0.0) || I.status) {
            I.active = 0;
            atomicSub(&A.sync->active_left, 1);
        }
    }
}

__global__ void __launch_bounds__(256) kb_step_1d(BArgs A)
{
    const int nt = A.sync->ntiles;
    const BTile *tl = A.sync->tiles;
    // the host sets `fresh` when some instance still needs its one-off dt;
    // every block reads it before the first barrier, block 0 clears it after
    const int fresh = *(volatile int *)&A.sync->fresh;
    if (fresh) {
        q_dt0(A, nt, tl);
        if (grid_barrier(A.sync, A.nblocks)) return;
        if (blockIdx.x == 0 && threadIdx.x == 0) A.sync->fresh = 0;
    }
    q_dt(A);  // writes dt only; the first reader (open BC) is three barriers on
    for (int rk = 0; rk < 3; rk++) {
        q_prim(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        q_rec(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        q_flux(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        if (rk == 0) {
            q_openbc(A);
            if (grid_barrier(A.sync, A.nblocks)) return;
        }
        q_update(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
    }
    q_advance(A);
}

}  // namespace

const void *batch1d_plain_kernel() { return (const void *)kb_step_1d; }

}  // namespace mlau
