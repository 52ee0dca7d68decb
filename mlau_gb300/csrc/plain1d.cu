// Plain FP64 1D step: one SSP-RK step of 1D MHD (7 variables, constant Bx),
// the GPU form of 1D/SERIAL/shock/mhd_fd4c_1d.c:60-271 with either the
// characteristic open boundary of 1D/SERIAL/shock/openbc1d_mhd.c:21-175
// (applied once, at stage 0, between the fluxes and the update) or the
// periodic boundary of 1D/SERIAL/wave (prdc_1d after each stage).
// Compiled with --fmad=false: bit-for-bit the reference's arithmetic.
//
// State slots: 0 ro, 1 mx, 2 my, 3 mz, 4 en, 6 by, 7 bz (slot 5 unused).
#include "stencil.cuh"

namespace mlau {
namespace {

// Primitives; at the first stage also the copy of the state U^n (seven small
// copies would cost more than the kernel).
__global__ void k_prim1(PlainFields f, int nx, double bx, double gamma, int save_u0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    if (save_u0)
        for (int v = 0; v < 8; v++)
            if (v != 5) f.u0[v][i] = f.s[v][i];
    const double ro = f.s[0][i], iro = 1.0 / ro;
    const double vx = f.s[1][i] * iro, vy = f.s[2][i] * iro, vz = f.s[3][i] * iro;
    const double by = f.s[6][i], bz = f.s[7][i];
    const double v2 = vx * vx + vy * vy + vz * vz;
    const double b2 = bx * bx + by * by + bz * bz;
    f.vx[i] = vx;
    f.vy[i] = vy;
    f.vz[i] = vz;
    f.pr[i] = (gamma - 1) * (f.s[4][i] - 0.5 * (ro * v2 + b2));
}

// Face states (:133-186): full characteristic system where any of the three
// central cells has sonic Mach^2 >= 1.
__global__ void k_rec1(PlainFields f, int nx, int odr, int eig, double bx, double gamma)
{
    const int i = 2 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx - 2) return;
    double q[7][5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const int s = i + m - 2;
        q[0][m] = f.s[0][s];
        q[1][m] = f.vx[s];
        q[2][m] = f.vy[s];
        q[3][m] = f.vz[s];
        q[4][m] = f.s[6][s];
        q[5][m] = f.s[7][s];
        q[6][m] = f.pr[s];
    }
    double mach[3];
#pragma unroll
    for (int t = 0; t < 3; t++) {
        const double c2 = gamma * q[6][1 + t] / q[0][1 + t];
        const double v2 = q[1][1 + t] * q[1][1 + t] + q[2][1 + t] * q[2][1 + t]
                          + q[3][1 + t] * q[3][1 + t];
        mach[t] = v2 / c2;
    }
    double ul[7], ur[7];
    reconst_face(odr, eig, vmax(mach[0], vmax(mach[1], mach[2])), q, bx, gamma, ul, ur);
#pragma unroll
    for (int n = 0; n < 7; n++) {
        f.ul[n][i + 1] = ul[n];
        f.ur[n][i] = ur[n];
    }
}

__global__ void k_flux1(PlainFields f, int nx, int which, double bx, double gamma)
{
    const int i = 3 + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx - 2) return;
    double L[7], R[7], F[7];
#pragma unroll
    for (int n = 0; n < 7; n++) {
        L[n] = f.ul[n][i];
        R[n] = f.ur[n][i];
    }
    riemann(which, L, R, bx, gamma, (f.vx[i] - f.vx[i - 1]), 0.0, F);
#pragma unroll
    for (int n = 0; n < 7; n++) f.F[0][n][i] = F[n];
}

// openbc1d_mhd (1D/SERIAL/shock/openbc1d_mhd.c:21-175).  The two sides read
// and write disjoint cells (interior width >= ghost depth), so each runs in
// its own block: block 0 the left side, block 1 the right.
__global__ void k_openbc1(PlainFields f, int nx, int xoff, double bx, double dtdx, double gamma)
{
    if (threadIdx.x != 0 || blockIdx.x > 1) return;
    double *ro = f.s[0], *mx = f.s[1], *my = f.s[2], *mz = f.s[3], *en = f.s[4], *by = f.s[6],
           *bz = f.s[7];
    const double bx2 = bx * bx;
    {
        const int side = blockIdx.x;
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
                   0.5 * (q[0][4] + q[1][4]), 0.5 * (q[0][5] + q[1][5]), 0.5 * (q[0][6] + q[1][6]),
                   gamma, E);
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

// Update (:220-255); with periodic boundaries each cell also writes its ghost
// images (prdc_1d, 1D/SERIAL/wave/prdc_1d.c).
__global__ void k_update1(PlainFields f, int nx, int xoff, int odr, double ra, double rb,
                          double dtdx, int periodic)
{
    const int i = xoff + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx - xoff) return;
    const int sv[7] = {0, 1, 2, 3, 6, 7, 4};  // flux order (ro, mx, my, mz, by, bz, en)
    double out[7];
#pragma unroll
    for (int v = 0; v < 7; v++) {
        const double *fx = f.F[0][v];
        const double dd = fdiff(odr, fx[i - 1], fx[i], fx[i + 1], fx[i + 2]);
        out[v] = ra * f.u0[sv[v]][i] + rb * (f.s[sv[v]][i] - dtdx * dd);
    }
    const int N = nx - 2 * xoff;
    const int im[3] = {i, (periodic && i < 2 * xoff) ? i + N : -1, (periodic && i >= N) ? i - N : -1};
    for (int a = 0; a < 3; a++) {
        if (im[a] < 0) continue;
#pragma unroll
        for (int v = 0; v < 7; v++) f.s[sv[v]][im[a]] = out[v];
    }
}

}  // namespace

int plain1d_alloc(Sim *s)
{
    PlainFields &f = s->f;
    const long long n = s->g.n;
    int rc = 0;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, &f.s[v], n) | dalloc(s, &f.u0[v], n);
    double **singles[] = {&f.vx, &f.vy, &f.vz, &f.pr};
    for (auto p : singles) rc |= dalloc(s, p, n);
    for (int v = 0; v < 7; v++)
        rc |= dalloc(s, &f.ul[v], n + 1) | dalloc(s, &f.ur[v], n + 1) | dalloc(s, &f.F[0][v], n);
    return rc ? MLAU_ERR_NOMEM : MLAU_OK;
}

// 1D grids hold a few thousand cells, each cell a long chain of FP64
// operations: blocks of 32 threads spread a 2048-cell problem over 64 SMs
// instead of 16 (0.208 instead of 0.222 ms per step at 2048 cells; the rest
// is each warp's own FP64 chain and the launches).
constexpr int T1D = 32;

int plain1d_step(Sim *s, double dt)
{
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const int nx = g.nx, off = g.ox;
    const double dtdx = dt / g.dx;
    const int T = T1D;
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        {
            TimedLaunch tl(&s->timer, KK_PRIM);
            k_prim1<<<blocks_for(nx, T), T, 0, st>>>(f, nx, s->bx1d, s->gamma, rk == 0);
        }
        {
            TimedLaunch tl(&s->timer, KK_REC);
            k_rec1<<<blocks_for(nx - 4, T), T, 0, st>>>(f, nx, s->odr, s->eig, s->bx1d, s->gamma);
        }
        {
            TimedLaunch tl(&s->timer, KK_FLUX);
            k_flux1<<<blocks_for(nx - 5, T), T, 0, st>>>(f, nx, s->flux, s->bx1d, s->gamma);
        }
        if (s->bc1d == MLAU_BC1D_OPEN && rk == 0) {
            TimedLaunch tl(&s->timer, KK_AUX);
            k_openbc1<<<2, 1, 0, st>>>(f, nx, off, s->bx1d, dtdx, s->gamma);
        }
        {
            TimedLaunch tl(&s->timer, KK_UPDATE);
            k_update1<<<blocks_for(nx - 2 * off, T), T, 0, st>>>(
                f, nx, off, s->odr, ra, rb, dtdx, s->bc1d == MLAU_BC1D_PERIODIC);
        }
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau

namespace mlau {

// Enqueue one 1D step on `st` for caller-provided fields (state and scratch
// already placed); used by the allocation-free entry point.  Same kernels and
// launch sequence as plain1d_step.
int plain1d_enqueue(const PlainFields &f, int nx, int off, int odr, int flux, int nrk, int bc,
                    double bx, double dt, double dx, double gamma, cudaStream_t st)
{
    const double dtdx = dt / dx;
    const int T = T1D;
    for (int rk = 0; rk < nrk; rk++) {
        double ra, rb;
        rk_coef(nrk, rk, ra, rb);
        k_prim1<<<blocks_for(nx, T), T, 0, st>>>(f, nx, bx, gamma, rk == 0);
        k_rec1<<<blocks_for(nx - 4, T), T, 0, st>>>(f, nx, odr, EIG_FULL, bx, gamma);
        k_flux1<<<blocks_for(nx - 5, T), T, 0, st>>>(f, nx, flux, bx, gamma);
        if (bc == MLAU_BC1D_OPEN && rk == 0) k_openbc1<<<2, 1, 0, st>>>(f, nx, off, bx, dtdx, gamma);
        k_update1<<<blocks_for(nx - 2 * off, T), T, 0, st>>>(f, nx, off, odr, ra, rb, dtdx,
                                                            bc == MLAU_BC1D_PERIODIC);
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau
