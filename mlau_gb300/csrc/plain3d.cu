// Plain FP64 3D step: one SSP-RK step of ideal MHD with constrained transport,
// the GPU form of the reference driver 3D/MPI/OTvortex/mhd_fd_ct_3d.c:99-1198
// (single rank), with the problem's boundary tables dnxs/dnys/dnzs: periodic
// along an axis whose entries are zero, Dirichlet / Neumann mirrors
// (3D/MPI/OTvortex/boundary.c:227-309) where they are -1 / +1.
//
// Compiled with --fmad=false: every floating-point expression is evaluated
// as in the reference (same operands, same order, IEEE division and square
// root), so the result equals the reference's bit for bit.
//
// Per RK stage, each kernel reads the reference's own index sets:
//   prim     cell-centred B (ghosts at their boundary sources, :186-238) + primitives (:240-262)
//   aux      CT upwind weights (:264-340) + shock sensors, ghosts at their sources (:342-377)
//   rec<D>   characteristic reconstruction of each cell along axis D (:394-454)
//   flux<D>  Riemann flux at each face along D, CT central/upwind split (:457-487)
//   emf      edge EMFs ex, ey, ez from the face fluxes (:494-585, :702-793, :910-1001)
//   update   RK combine of cell-centred variables (:1003-1078) and CT curl of
//            face B (:1079-1157); on a periodic box each thread also writes its
//            periodic ghost images, which is exactly the reference's fill
//            (:1161-1175); with walls, face + bc follow (the right boundary faces
//            the CT loops reach, then the ghost fill with the tables).
// A ghost's boundary source composes, axis by axis, the periodic image or the
// mirror with the product of the signs: the result of the reference's
// periodic exchange followed by its X, Y and Z mirrors.
#include <algorithm>

#include "sim.cuh"
#include "point.cuh"
#include "stencil.cuh"

namespace mlau {
namespace {

// Source of cell (i, j, k) of a cell-centred ghost-filled array whose x/y/z
// table entries are dx/dy/dz (sign into *g).
__device__ __forceinline__ long long src3(const Dims &d, int i, int j, int k, int dx, int dy,
                                          int dz, double *g)
{
    return d.at(bc_src(i, d.nx, d.ox, 0, dx, g), bc_src(j, d.ny, d.oy, 0, dy, g),
                bc_src(k, d.nz, d.oz, 0, dz, g));
}

__global__ void __launch_bounds__(TPB)
k_prim3(PlainFields f, Dims d, Box b, int odr, double gamma, Bc3 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    double gx = 1.0, gy = 1.0, gz = 1.0;
    const long long wx = src3(d, i, j, k, bc.x[5], bc.y[5], bc.z[5], &gx);
    const long long wy = src3(d, i, j, k, bc.x[6], bc.y[6], bc.z[6], &gy);
    const long long wz = src3(d, i, j, k, bc.x[7], bc.y[7], bc.z[7], &gz);
    const double *bx = f.s[5], *by = f.s[6], *bz = f.s[7];
    const double cx = gx * face2cen(odr, bx[wx - 1], bx[wx], bx[wx + 1], bx[wx + 2]);
    const double cy = gy * face2cen(odr, by[wy - sy], by[wy], by[wy + sy], by[wy + 2 * sy]);
    const double cz = gz * face2cen(odr, bz[wz - sz], bz[wz], bz[wz + sz], bz[wz + 2 * sz]);
    const long long s = d.at(i, j, k);
    const double ro = f.s[0][s];
    const double iro = 1.0 / ro;
    const double vx = f.s[1][s] * iro, vy = f.s[2][s] * iro, vz = f.s[3][s] * iro;
    const double v2 = (vx * vx + vy * vy + vz * vz);
    const double b2 = (cx * cx + cy * cy + cz * cz);
    const double pr = (gamma - 1) * (f.s[4][s] - 0.5 * (ro * v2 + b2));
    f.vx[s] = vx;
    f.vy[s] = vy;
    f.vz[s] = vz;
    f.pr[s] = pr;
    f.m2[s] = v2 / (gamma * pr * iro);
    f.cx[s] = cx;
    f.cy[s] = cy;
    f.cz[s] = cz;
}

// CT weights, and the shock sensors with the sign rules of their ghost fill
// (:367-376): dvx takes -dnxs[1] along x, dvy -dnys[2] along y, dvz -dnzs[3]
// along z, the table entries along the other axes.
__global__ void __launch_bounds__(TPB) k_aux3(PlainFields f, Dims d, Box b, Bc3 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long s = d.at(i, j, k);
    const double *ro = f.s[0];
    // ct0: x-y plane (Ez), a=x, b=y; ct1: y-z (Ex), a=y, b=z; ct2: z-x (Ey), a=z, b=x
    f.ct[0][s] = (i >= 1 && j >= 1) ? ct_weight(f.vx, f.vy, ro, f.s[5], f.s[6], s, sy, 1, sy, 1)
                                    : 0.5;
    f.ct[1][s] = (j >= 1 && k >= 1) ? ct_weight(f.vy, f.vz, ro, f.s[6], f.s[7], s, sz, sy, sz, sy)
                                    : 0.5;
    f.ct[2][s] = (k >= 1 && i >= 1) ? ct_weight(f.vz, f.vx, ro, f.s[7], f.s[5], s, sz, 1, 1, sz)
                                    : 0.5;
    double g0 = 1.0, g1 = 1.0, g2 = 1.0;
    const long long w0 = src3(d, i, j, k, -bc.x[1], bc.y[1], bc.z[1], &g0);
    const long long w1 = src3(d, i, j, k, bc.x[2], -bc.y[2], bc.z[2], &g1);
    const long long w2 = src3(d, i, j, k, bc.x[3], bc.y[3], -bc.z[3], &g2);
    f.dv[0][s] = g0 * vmin((f.vx[w0 + 1] - f.vx[w0]), (f.vx[w0] - f.vx[w0 - 1]));
    f.dv[1][s] = g1 * vmin((f.vy[w1 + sy] - f.vy[w1]), (f.vy[w1] - f.vy[w1 - sy]));
    f.dv[2][s] = g2 * vmin((f.vz[w2 + sz] - f.vz[w2]), (f.vz[w2] - f.vz[w2 - sz]));
}

// Rotated views of the primitives for a sweep along axis D.
struct SweepView {
    const double *vn, *vt, *vu, *cn, *ct, *cu, *bface, *dvt, *dvu;
};

__host__ SweepView make_view(const PlainFields &f, int D)
{
    if (D == 0) return {f.vx, f.vy, f.vz, f.cx, f.cy, f.cz, f.s[5], f.dv[1], f.dv[2]};
    if (D == 1) return {f.vy, f.vz, f.vx, f.cy, f.cz, f.cx, f.s[6], f.dv[2], f.dv[0]};
    return {f.vz, f.vx, f.vy, f.cz, f.cx, f.cy, f.s[7], f.dv[0], f.dv[1]};
}

__global__ void __launch_bounds__(TPB)
k_rec3(PlainFields f, SweepView v, Dims d, Box b, long long st, int odr, int eig, double gamma)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long c = d.at(i, j, k);
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
    // Linear interpolation of the central (B_t v_n - B_n v_t) part of the two
    // tangential B fluxes (:441-453).
    const double bl = v.bface[c + st], br = v.bface[c];
    double a5[5], t5[5], u5[5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const long long s = c + st * (m - 2);
        a5[m] = v.ct[s] * v.vn[s];
        t5[m] = v.vt[s];
    }
    f.ql[0][c + st] = lin_l(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                      - bl * lin_l(odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
    f.qr[0][c] = lin_r(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                 - br * lin_r(odr, t5[0], t5[1], t5[2], t5[3], t5[4]);
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const long long s = c + st * (m - 2);
        a5[m] = v.cu[s] * v.vn[s];
        u5[m] = v.vu[s];
    }
    f.ql[1][c + st] = lin_l(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                      - bl * lin_l(odr, u5[0], u5[1], u5[2], u5[3], u5[4]);
    f.qr[1][c] = lin_r(odr, a5[0], a5[1], a5[2], a5[3], a5[4])
                 - br * lin_r(odr, u5[0], u5[1], u5[2], u5[3], u5[4]);
}

__global__ void __launch_bounds__(TPB)
k_flux3(PlainFields f, SweepView v, Dims d, Box b, long long st, int D, int which, double gamma)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long c = d.at(i, j, k);
    double L[7], R[7], F[7];
#pragma unroll
    for (int n = 0; n < 7; n++) {
        L[n] = f.ul[n][c];
        R[n] = f.ur[n][c];
    }
    const double bn = 0.5 * (v.bface[c] + v.bface[c]);
    const double dvtm = vmin(vmin(v.dvt[c - st], v.dvt[c]), vmin(v.dvu[c - st], v.dvu[c]));
    riemann(which, L, R, bn, gamma, (v.vn[c] - v.vn[c - st]), dvtm, F);
    const double fct = 0.5 * (f.ql[0][c] + f.qr[0][c]);
    const double fcu = 0.5 * (f.ql[1][c] + f.qr[1][c]);
    F[4] -= fct;
    F[5] -= fcu;
#pragma unroll
    for (int n = 0; n < 7; n++) f.F[D][n][c] = F[n];
    f.FC[D][0][c] = fct;
    f.FC[D][1][c] = fcu;
}

__global__ void __launch_bounds__(TPB) k_emf3(PlainFields f, Dims d, Box b, int odr)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long c = d.at(i, j, k);
    const bool xi = (i >= 3 && i < d.nx - 2), yj = (j >= 3 && j < d.ny - 2),
               zk = (k >= 3 && k < d.nz - 2);
    // F[d][4]/F[d][5] are the fluxes of the first/second tangential B:
    //   X: (By, Bz), Y: (Bz, Bx), Z: (Bx, By).
    double ez = 0.0, ex = 0.0, ey = 0.0;
    if (xi && yj) {
        const double w = f.ct[0][c];
        ez = (0.0 + emf_part(f.F[0][4], f.FC[0][0], (1.0 - w), -1.0, c, sy, odr))
             + emf_part(f.F[1][5], f.FC[1][1], w, +1.0, c, 1, odr);
    }
    if (yj && zk) {
        const double w = f.ct[1][c];
        ex = (0.0 + emf_part(f.F[1][4], f.FC[1][0], (1.0 - w), -1.0, c, sz, odr))
             + emf_part(f.F[2][5], f.FC[2][1], w, +1.0, c, sy, odr);
    }
    if (zk && xi) {
        const double w = f.ct[2][c];
        ey = (0.0 + emf_part(f.F[0][5], f.FC[0][1], w, +1.0, c, sz, odr))
             + emf_part(f.F[2][4], f.FC[2][0], (1.0 - w), -1.0, c, 1, odr);
    }
    f.e[0][c] = ex;
    f.e[1][c] = ey;
    f.e[2][c] = ez;
}

__global__ void __launch_bounds__(TPB)
k_update3(PlainFields f, Dims d, Box b, int odr, double ra, double rb, double dtdx, double dtdy,
          double dtdz, int images)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long s = d.at(i, j, k);
    // flux component per direction for (ro, mx, my, mz, en)
    const int cX[5] = {0, 1, 2, 3, 6}, cY[5] = {0, 3, 1, 2, 6}, cZ[5] = {0, 2, 3, 1, 6};
    double out[8];
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double *fx = f.F[0][cX[v]], *fy = f.F[1][cY[v]], *fz = f.F[2][cZ[v]];
        const double d0 = fdiff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
        const double d1 = fdiff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
        const double d2 = fdiff(odr, fz[s - sz], fz[s], fz[s + sz], fz[s + 2 * sz]);
        out[v] = ra * f.u0[v][s] + rb * (f.s[v][s] - dtdx * d0 - dtdy * d1 - dtdz * d2);
    }
    const double *ex = f.e[0], *ey = f.e[1], *ez = f.e[2];
    {
        const double d0 = fdiff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
        const double d1 = fdiff(odr, ey[s - sz], ey[s], ey[s + sz], ey[s + 2 * sz]);
        out[5] = ra * f.u0[5][s] + rb * (f.s[5][s] - dtdy * d0 + dtdz * d1);
    }
    {
        const double d0 = fdiff(odr, ex[s - sz], ex[s], ex[s + sz], ex[s + 2 * sz]);
        const double d1 = fdiff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
        out[6] = ra * f.u0[6][s] + rb * (f.s[6][s] - dtdz * d0 + dtdx * d1);
    }
    {
        const double d0 = fdiff(odr, ey[s - 1], ey[s], ey[s + 1], ey[s + 2]);
        const double d1 = fdiff(odr, ex[s - sy], ex[s], ex[s + sy], ex[s + 2 * sy]);
        out[7] = ra * f.u0[7][s] + rb * (f.s[7][s] - dtdx * d0 + dtdy * d1);
    }
    if (!images) {
#pragma unroll
        for (int v = 0; v < 8; v++) f.s[v][s] = out[v];
        return;
    }
    // periodic images: i+N for i < 2*off, i-N for i >= N (N interior width)
    const int Nx = d.nx - 2 * d.ox, Ny = d.ny - 2 * d.oy, Nz = d.nz - 2 * d.oz;
    int is[3] = {i, i < 2 * d.ox ? i + Nx : -1, i >= Nx ? i - Nx : -1};
    int js[3] = {j, j < 2 * d.oy ? j + Ny : -1, j >= Ny ? j - Ny : -1};
    int ks[3] = {k, k < 2 * d.oz ? k + Nz : -1, k >= Nz ? k - Nz : -1};
    for (int c = 0; c < 3; c++) {
        if (ks[c] < 0) continue;
        for (int bb = 0; bb < 3; bb++) {
            if (js[bb] < 0) continue;
            for (int a = 0; a < 3; a++) {
                if (is[a] < 0) continue;
                const long long t = d.at(is[a], js[bb], ks[c]);
#pragma unroll
                for (int v = 0; v < 8; v++) f.s[v][t] = out[v];
            }
        }
    }
}

// The right boundary faces the CT loops also update (:1079-1157 run one face
// further: Bx at i = nx-xoff, By at j = ny-yoff, Bz at k = nz-zoff); they
// survive the ghost fill only where that axis mirrors the face array.  One
// thread per face of the three planes.
__global__ void __launch_bounds__(TPB)
k_face3(PlainFields f, Dims d, int odr, double ra, double rb, double dtdx, double dtdy,
        double dtdz, int do_x, int do_y, int do_z)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const int Nx = d.nx - 2 * d.ox, Ny = d.ny - 2 * d.oy, Nz = d.nz - 2 * d.oz;
    const double *ex = f.e[0], *ey = f.e[1], *ez = f.e[2];
    if (do_x && t < (long long)Ny * Nz) {  // Bx at i = nx - xoff
        const long long s = d.at(d.nx - d.ox, d.oy + (int)(t % Ny), d.oz + (int)(t / Ny));
        const double d0 = fdiff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
        const double d1 = fdiff(odr, ey[s - sz], ey[s], ey[s + sz], ey[s + 2 * sz]);
        f.s[5][s] = ra * f.u0[5][s] + rb * (f.s[5][s] - dtdy * d0 + dtdz * d1);
    }
    if (do_y && t < (long long)Nx * Nz) {  // By at j = ny - yoff
        const long long s = d.at(d.ox + (int)(t % Nx), d.ny - d.oy, d.oz + (int)(t / Nx));
        const double d0 = fdiff(odr, ex[s - sz], ex[s], ex[s + sz], ex[s + 2 * sz]);
        const double d1 = fdiff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
        f.s[6][s] = ra * f.u0[6][s] + rb * (f.s[6][s] - dtdz * d0 + dtdx * d1);
    }
    if (do_z && t < (long long)Nx * Ny) {  // Bz at k = nz - zoff
        const long long s = d.at(d.ox + (int)(t % Nx), d.oy + (int)(t / Nx), d.nz - d.oz);
        const double d0 = fdiff(odr, ey[s - 1], ey[s], ey[s + 1], ey[s + 2]);
        const double d1 = fdiff(odr, ex[s - sy], ex[s], ex[s + sy], ex[s + 2 * sy]);
        f.s[7][s] = ra * f.u0[7][s] + rb * (f.s[7][s] - dtdx * d0 + dtdy * d1);
    }
}

// Ghost fill of the conserved arrays with the tables (:1161-1175): each
// ghost takes its boundary source composed over the three axes, times the
// signs.  Sources are interior cells or computed faces.
__global__ void __launch_bounds__(TPB) k_bc3(PlainFields f, Dims d, Box b, Bc3 bc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    if (i >= d.ox && i < d.nx - d.ox && j >= d.oy && j < d.ny - d.oy && k >= d.oz &&
        k < d.nz - d.oz)
        return;
    const long long s = d.at(i, j, k);
#pragma unroll
    for (int v = 0; v < 8; v++) {
        double g = 1.0;
        const int si = bc_src(i, d.nx, d.ox, v == 5, bc.x[v], &g);
        const int sj = bc_src(j, d.ny, d.oy, v == 6, bc.y[v], &g);
        const int sk = bc_src(k, d.nz, d.oz, v == 7, bc.z[v], &g);
        if (si == i && sj == j && sk == k) continue;
        f.s[v][s] = g * f.s[v][d.at(si, sj, sk)];
    }
}

}  // namespace

int plain3d_alloc(Sim *s)
{
    PlainFields &f = s->f;
    const long long n = s->g.n;
    int rc = 0;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, &f.s[v], n) | dalloc(s, &f.u0[v], n);
    double **singles[] = {&f.vx, &f.vy, &f.vz, &f.pr, &f.m2, &f.cx, &f.cy, &f.cz,
                          &f.dv[0], &f.dv[1], &f.dv[2], &f.ct[0], &f.ct[1], &f.ct[2],
                          &f.ql[0], &f.ql[1], &f.qr[0], &f.qr[1], &f.e[0], &f.e[1], &f.e[2]};
    for (auto p : singles) rc |= dalloc(s, p, n);
    for (int v = 0; v < 7; v++) rc |= dalloc(s, &f.ul[v], n) | dalloc(s, &f.ur[v], n);
    for (int D = 0; D < 3; D++) {
        for (int v = 0; v < 7; v++) rc |= dalloc(s, &f.F[D][v], n);
        rc |= dalloc(s, &f.FC[D][0], n) | dalloc(s, &f.FC[D][1], n);
    }
    return rc ? MLAU_ERR_NOMEM : MLAU_OK;
}

// Ghost fill of the FP64 state with the simulation's 3D tables (also the
// last act of an FP32-split stage with non-periodic tables).
int plain3d_fill_ghosts(Sim *s)
{
    const Geometry &g = s->g;
    const Dims d{g.nx, g.ny, g.nz, g.ox, g.oy, g.oz};
    const Box all{0, 0, 0, g.nx, g.ny, g.nz};
    k_bc3<<<blocks_for(all.count(), TPB), TPB, 0, s->stream>>>(s->f, d, all, s->bc3);
    return MLAU_OK;
}

int plain3d_step(Sim *s, double dt)
{
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, g.nz, g.ox, g.oy, g.oz};
    const long long sy = g.nx, sz = (long long)g.nx * g.ny;
    {
        TimedLaunch tl(&s->timer, KK_COPY);
        for (int v = 0; v < 8; v++)
            MLAU_CUDA(cudaMemcpyAsync(f.u0[v], f.s[v], sizeof(double) * g.n,
                                      cudaMemcpyDeviceToDevice, st));
    }
    const Box all{0, 0, 0, g.nx, g.ny, g.nz};
    const Box inner{g.ox, g.oy, g.oz, g.nx - 2 * g.ox, g.ny - 2 * g.oy, g.nz - 2 * g.oz};
    const long long strides[3] = {1, sy, sz};
    const double dtdx = dt / g.dx, dtdy = dt / g.dy, dtdz = dt / g.dz;
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        {
            TimedLaunch tl(&s->timer, KK_PRIM);
            k_prim3<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->odr, s->gamma,
                                                                  s->bc3);
        }
        {
            TimedLaunch tl(&s->timer, KK_AUX);
            k_aux3<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->bc3);
        }
        for (int D = 0; D < 3; D++) {
            const SweepView v = make_view(f, D);
            Box rb_ = all, fb = all;
            int *lo_r[3] = {&rb_.lo0, &rb_.lo1, &rb_.lo2}, *e_r[3] = {&rb_.e0, &rb_.e1, &rb_.e2};
            int *lo_f[3] = {&fb.lo0, &fb.lo1, &fb.lo2}, *e_f[3] = {&fb.e0, &fb.e1, &fb.e2};
            const int len = (D == 0) ? g.nx : (D == 1 ? g.ny : g.nz);
            *lo_r[D] = 2;
            *e_r[D] = len - 4;  // cells [2, len-2)
            *lo_f[D] = 3;
            *e_f[D] = len - 5;  // faces [3, len-2)
            {
                TimedLaunch tl(&s->timer, KK_REC);
                k_rec3<<<blocks_for(rb_.count(), TPB), TPB, 0, st>>>(f, v, d, rb_, strides[D],
                                                                     s->odr, s->eig, s->gamma);
            }
            {
                TimedLaunch tl(&s->timer, KK_FLUX);
                k_flux3<<<blocks_for(fb.count(), TPB), TPB, 0, st>>>(f, v, d, fb, strides[D], D,
                                                                     s->flux, s->gamma);
            }
        }
        {
            TimedLaunch tl(&s->timer, KK_EMF);
            k_emf3<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->odr);
        }
        {
            TimedLaunch tl(&s->timer, KK_UPDATE);
            k_update3<<<blocks_for(inner.count(), TPB), TPB, 0, st>>>(f, d, inner, s->odr, ra, rb,
                                                                      dtdx, dtdy, dtdz, !s->walls3d);
            if (s->walls3d) {
                const long long n = std::max({(long long)g.ny * g.nz, (long long)g.nx * g.nz,
                                              (long long)g.nx * g.ny});
                k_face3<<<blocks_for(n, TPB), TPB, 0, st>>>(f, d, s->odr, ra, rb, dtdx, dtdy, dtdz,
                                                            s->bc3.x[5] != 0, s->bc3.y[6] != 0,
                                                            s->bc3.z[7] != 0);
                k_bc3<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(f, d, all, s->bc3);
            }
        }
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau
