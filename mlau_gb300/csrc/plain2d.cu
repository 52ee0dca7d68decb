// Plain FP64 2D step: one SSP-RK step of ideal MHD with constrained transport,
// the GPU form of 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-660, with the problem's
// boundary tables (periodic, or Dirichlet / Neumann mirrors per array and
// axis as bc2d, 2D/SERIAL/OTvortex/boundary.c:18-74).
// Bz is cell-centred and advanced with the fluxes; Bx, By live on faces and
// are advanced by the curl of the corner EMF Ez.  Compiled with --fmad=false
// so the arithmetic is the reference's, bit for bit.
#include <algorithm>

#include "stencil.cuh"

namespace mlau {
namespace {

// Cell-centred B: computed at the cell itself or, in the ghost frame, at its
// boundary source times the table's sign (calc_bc then bc2d with dnxs[5..6],
// :186-200).
__global__ void __launch_bounds__(TPB)
k_prim2(PlainFields f, Dims d, Box b, int odr, double gamma, Bc2 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx;
    double gx = 1.0, gy = 1.0;
    const int ix = bc_src(i, d.nx, d.ox, 0, bc.x[5], &gx), jx = bc_src(j, d.ny, d.oy, 0, bc.y[5], &gx);
    const int iy = bc_src(i, d.nx, d.ox, 0, bc.x[6], &gy), jy = bc_src(j, d.ny, d.oy, 0, bc.y[6], &gy);
    const long long wx = d.at(ix, jx, 0), wy = d.at(iy, jy, 0);
    const double *bx = f.s[5], *by = f.s[6];
    const double cx = gx * face2cen(odr, bx[wx - 1], bx[wx], bx[wx + 1], bx[wx + 2]);
    const double cy = gy * face2cen(odr, by[wy - sy], by[wy], by[wy + sy], by[wy + 2 * sy]);
    const long long s = d.at(i, j, 0);
    const double ro = f.s[0][s];
    const double iro = 1.0 / ro;
    const double vx = f.s[1][s] * iro, vy = f.s[2][s] * iro, vz = f.s[3][s] * iro;
    const double bz = f.s[7][s];
    const double v2 = (vx * vx + vy * vy + vz * vz);
    const double b2 = (cx * cx + cy * cy + bz * bz);
    const double pr = (gamma - 1) * (f.s[4][s] - 0.5 * (ro * v2 + b2));
    f.vx[s] = vx;
    f.vy[s] = vy;
    f.vz[s] = vz;
    f.pr[s] = pr;
    f.m2[s] = v2 / (gamma * pr * iro);
    f.cx[s] = cx;
    f.cy[s] = cy;
}

// Shock sensors, with the sign rules of their ghost fill (:262-271): dvx
// takes -dnxs[1] along x and +dnys[1] along y, dvy +dnxs[2] and -dnys[2].
__global__ void __launch_bounds__(TPB) k_aux2(PlainFields f, Dims d, Box b, Bc2 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx;
    const long long s = d.at(i, j, 0);
    f.ct[0][s] = (i >= 1 && j >= 1) ? ct_weight(f.vx, f.vy, f.s[0], f.s[5], f.s[6], s, sy, 1, sy, 1)
                                    : 0.5;
    double g0 = 1.0, g1 = 1.0;
    const int i0 = bc_src(i, d.nx, d.ox, 0, -bc.x[1], &g0), j0 = bc_src(j, d.ny, d.oy, 0, bc.y[1], &g0);
    const int i1 = bc_src(i, d.nx, d.ox, 0, bc.x[2], &g1), j1 = bc_src(j, d.ny, d.oy, 0, -bc.y[2], &g1);
    const long long w0 = d.at(i0, j0, 0), w1 = d.at(i1, j1, 0);
    f.dv[0][s] = g0 * vmin((f.vx[w0 + 1] - f.vx[w0]), (f.vx[w0] - f.vx[w0 - 1]));
    f.dv[1][s] = g1 * vmin((f.vy[w1 + sy] - f.vy[w1]), (f.vy[w1] - f.vy[w1 - sy]));
}

// Sweep along x (D=0): (vn, vt, vu) = (vx, vy, vz), (bt, bu) = (cy, bz), the
// By flux is split.  Along y (D=1): (vy, vz, vx), (bz, cx), the Bx flux is split.
struct View2 {
    const double *vn, *vt, *vu, *cn, *ct, *cu, *bface, *dvt;
    int split_u;  // 0: split the bt flux; 1: split the bu flux
};

View2 make_view2(const PlainFields &f, int D)
{
    if (D == 0) return {f.vx, f.vy, f.vz, f.cx, f.cy, f.s[7], f.s[5], f.dv[1], 0};
    return {f.vy, f.vz, f.vx, f.cy, f.s[7], f.cx, f.s[6], f.dv[0], 1};
}

__global__ void __launch_bounds__(TPB)
k_rec2(PlainFields f, View2 v, Dims d, Box b, long long st, int odr, int eig, double gamma)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long c = d.at(i, j, 0);
    double q[7][5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const long long s = c + st * (m - 2);
        q[0][m] = f.s[0][s];
        q[1][m] = v.vn[s];
        q[2][m] = v.vt[s];
        q[3][m] = v.vu[s];
        q[4][m] = v.ct[s];
        q[5][m] = v.cu[s];
        q[6][m] = f.pr[s];
    }
    double ul[7], ur[7];
    reconst_face(odr, eig, vmax(f.m2[c - st], vmax(f.m2[c], f.m2[c + st])), q, v.cn[c], gamma,
                 ul, ur);
#pragma unroll
    for (int n = 0; n < 7; n++) {
        f.ul[n][c + st] = ul[n];
        f.ur[n][c] = ur[n];
    }
    const double *bt = v.split_u ? v.cu : v.ct, *vt = v.split_u ? v.vu : v.vt;
    double a5[5], t5[5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const long long s = c + st * (m - 2);
        a5[m] = bt[s] * v.vn[s];
        t5[m] = vt[s];
    }
    f.ql[0][c + st] = lin_l(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                      - v.bface[c + st] * lin_l(odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
    f.qr[0][c] = lin_r(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                 - v.bface[c] * lin_r(odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
}

__global__ void __launch_bounds__(TPB)
k_flux2(PlainFields f, View2 v, Dims d, Box b, long long st, int D, int which, double gamma)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long c = d.at(i, j, 0);
    double L[7], R[7], F[7];
#pragma unroll
    for (int n = 0; n < 7; n++) {
        L[n] = f.ul[n][c];
        R[n] = f.ur[n][c];
    }
    const double bn = 0.5 * (v.bface[c] + v.bface[c]);
    riemann(which, L, R, bn, gamma, (v.vn[c] - v.vn[c - st]), vmin(v.dvt[c - st], v.dvt[c]), F);
    const double fc = 0.5 * (f.ql[0][c] + f.qr[0][c]);
    F[4 + v.split_u] -= fc;
#pragma unroll
    for (int n = 0; n < 7; n++) f.F[D][n][c] = F[n];
    f.FC[D][0][c] = fc;
}

__global__ void __launch_bounds__(TPB) k_emf2(PlainFields f, Dims d, Box b, int odr)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long c = d.at(i, j, 0);
    double ez = 0.0;
    if (i >= 3 && i < d.nx - 2 && j >= 3 && j < d.ny - 2) {
        const double w = f.ct[0][c];
        ez = (0.0 + emf_part(f.F[0][4], f.FC[0][0], (1.0 - w), -1.0, c, d.nx, odr))
             + emf_part(f.F[1][5], f.FC[1][0], w, +1.0, c, 1, odr);
    }
    f.e[2][c] = ez;
}

// RK combine + CT curl of the interior.  With periodic tables each cell also
// writes its periodic images; otherwise k_face2 and k_bc2 follow.
__global__ void __launch_bounds__(TPB)
k_update2(PlainFields f, Dims d, Box b, int odr, double ra, double rb, double dtdx, double dtdy,
          int images)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx;
    const long long s = d.at(i, j, 0);
    // (ro, mx, my, mz, bz, en): state slot and flux component per direction
    const int sv[6] = {0, 1, 2, 3, 7, 4};
    const int cX[6] = {0, 1, 2, 3, 5, 6}, cY[6] = {0, 3, 1, 2, 4, 6};
    double out[8];
#pragma unroll
    for (int v = 0; v < 6; v++) {
        const double *fx = f.F[0][cX[v]], *fy = f.F[1][cY[v]];
        const double d0 = fdiff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
        const double d1 = fdiff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
        out[sv[v]] = ra * f.u0[sv[v]][s] + rb * (f.s[sv[v]][s] - dtdx * d0 - dtdy * d1);
    }
    const double *ez = f.e[2];
    {
        const double dd = fdiff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
        out[5] = ra * f.u0[5][s] + rb * (f.s[5][s] - dtdy * dd);
    }
    {
        const double dd = fdiff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
        out[6] = ra * f.u0[6][s] + rb * (f.s[6][s] + dtdx * dd);
    }
    if (!images) {
#pragma unroll
        for (int v = 0; v < 8; v++) f.s[v][s] = out[v];
        return;
    }
    const int Nx = d.nx - 2 * d.ox, Ny = d.ny - 2 * d.oy;
    int is[3] = {i, i < 2 * d.ox ? i + Nx : -1, i >= Nx ? i - Nx : -1};
    int js[3] = {j, j < 2 * d.oy ? j + Ny : -1, j >= Ny ? j - Ny : -1};
    for (int bb = 0; bb < 3; bb++) {
        if (js[bb] < 0) continue;
        for (int a = 0; a < 3; a++) {
            if (is[a] < 0) continue;
            const long long t = d.at(is[a], js[bb], 0);
#pragma unroll
            for (int v = 0; v < 8; v++) f.s[v][t] = out[v];
        }
    }
}

// The right boundary faces the CT loops also update (:593-632 run one face
// further, i < nx-xoff+1 for Bx and j < ny-yoff+1 for By); they survive the
// boundary fill only where that axis mirrors the face array.
__global__ void __launch_bounds__(TPB)
k_face2(PlainFields f, Dims d, int odr, double ra, double rb, double dtdx, double dtdy, int do_x,
        int do_y)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const long long sy = d.nx;
    const double *ez = f.e[2];
    const int ny_in = d.ny - 2 * d.oy, nx_in = d.nx - 2 * d.ox;
    if (do_x && t < ny_in) {  // Bx at i = nx - xoff
        const long long s = d.at(d.nx - d.ox, d.oy + t, 0);
        const double dd = fdiff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
        f.s[5][s] = ra * f.u0[5][s] + rb * (f.s[5][s] - dtdy * dd);
    }
    if (do_y && t < nx_in) {  // By at j = ny - yoff
        const long long s = d.at(d.ox + t, d.ny - d.oy, 0);
        const double dd = fdiff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
        f.s[6][s] = ra * f.u0[6][s] + rb * (f.s[6][s] + dtdx * dd);
    }
}

// Ghost fill of the conserved arrays with the tables (:636-638): each ghost
// takes its boundary source (periodic image or mirror, composed over the two
// axes) times the signs.  Sources are interior cells or computed faces.
__global__ void __launch_bounds__(TPB) k_bc2(PlainFields f, Dims d, Box b, Bc2 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    if (i >= d.ox && i < d.nx - d.ox && j >= d.oy && j < d.ny - d.oy) return;
    const long long s = d.at(i, j, 0);
#pragma unroll
    for (int v = 0; v < 8; v++) {
        double g = 1.0;
        const int si = bc_src(i, d.nx, d.ox, v == 5, bc.x[v], &g);
        const int sj = bc_src(j, d.ny, d.oy, v == 6, bc.y[v], &g);
        if (si == i && sj == j) continue;
        f.s[v][s] = g * f.s[v][d.at(si, sj, 0)];
    }
}

}  // namespace

int plain2d_alloc(Sim *s)
{
    PlainFields &f = s->f;
    const long long n = s->g.n;
    int rc = 0;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, &f.s[v], n) | dalloc(s, &f.u0[v], n);
    double **singles[] = {&f.vx, &f.vy, &f.vz, &f.pr, &f.m2, &f.cx, &f.cy, &f.dv[0], &f.dv[1],
                          &f.ct[0], &f.ql[0], &f.qr[0], &f.e[2]};
    for (auto p : singles) rc |= dalloc(s, p, n);
    for (int v = 0; v < 7; v++) rc |= dalloc(s, &f.ul[v], n) | dalloc(s, &f.ur[v], n);
    for (int D = 0; D < 2; D++) {
        for (int v = 0; v < 7; v++) rc |= dalloc(s, &f.F[D][v], n);
        rc |= dalloc(s, &f.FC[D][0], n);
    }
    return rc ? MLAU_ERR_NOMEM : MLAU_OK;
}

int plain2d_step(Sim *s, double dt)
{
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, 1, g.ox, g.oy, 0};
    {
        TimedLaunch tl(&s->timer, KK_COPY);
        for (int v = 0; v < 8; v++)
            MLAU_CUDA(cudaMemcpyAsync(f.u0[v], f.s[v], sizeof(double) * g.n,
                                      cudaMemcpyDeviceToDevice, st));
    }
    const Box all{0, 0, 0, g.nx, g.ny, 1};
    const Box inner{g.ox, g.oy, 0, g.nx - 2 * g.ox, g.ny - 2 * g.oy, 1};
    const double dtdx = dt / g.dx, dtdy = dt / g.dy;
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        {
            TimedLaunch tl(&s->timer, KK_PRIM);
            k_prim2<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->odr, s->gamma,
                                                                  s->bc2);
        }
        {
            TimedLaunch tl(&s->timer, KK_AUX);
            k_aux2<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->bc2);
        }
        for (int D = 0; D < 2; D++) {
            const View2 v = make_view2(f, D);
            const long long stride = D == 0 ? 1 : g.nx;
            Box rb_ = all, fb = all;
            if (D == 0) { rb_.lo0 = 2; rb_.e0 = g.nx - 4; fb.lo0 = 3; fb.e0 = g.nx - 5; }
            else { rb_.lo1 = 2; rb_.e1 = g.ny - 4; fb.lo1 = 3; fb.e1 = g.ny - 5; }
            {
                TimedLaunch tl(&s->timer, KK_REC);
                k_rec2<<<blocks_for(rb_.count(), TPB), TPB, 0, st>>>(f, v, d, rb_, stride, s->odr,
                                                                     s->eig, s->gamma);
            }
            {
                TimedLaunch tl(&s->timer, KK_FLUX);
                k_flux2<<<blocks_for(fb.count(), TPB), TPB, 0, st>>>(f, v, d, fb, stride, D,
                                                                     s->flux, s->gamma);
            }
        }
        {
            TimedLaunch tl(&s->timer, KK_EMF);
            k_emf2<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->odr);
        }
        {
            TimedLaunch tl(&s->timer, KK_UPDATE);
            k_update2<<<blocks_for(inner.count(), TPB), TPB, 0, st>>>(f, d, inner, s->odr, ra, rb,
                                                                      dtdx, dtdy, !s->walls2d);
            if (s->walls2d) {
                const int n = std::max(g.nx, g.ny);
                k_face2<<<blocks_for(n, TPB), TPB, 0, st>>>(f, d, s->odr, ra, rb, dtdx, dtdy,
                                                            s->bc2.x[5] != 0, s->bc2.y[6] != 0);
                k_bc2<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->bc2);
            }
        }
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau
