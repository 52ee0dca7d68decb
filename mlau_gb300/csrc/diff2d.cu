// 2D problem operators on the device, run between hyperbolic steps as the
// problems' main loops do.
//
// MRX (2D/MPI/MRX/main.cpp:48-68, mhd_fd_ct_2d.c:726-1456): resistive
// diffusion of the CT field with uniform resistivity (diff_ctfield_e, energy
// updated by the resistive Poynting flux), the viscous term with uniform
// kinematic viscosity (ns_viscous_2d) - explicit SSP-RK updates of their own -
// and anisotropic heat conduction along B (t_conduction, implicit, solved by
// colour Gauss-Seidel sweeps).  RMI (2D/MPI/RMI/main.cpp:48-54): the inflow
// injected at the upper boundary before each step (inj_ro).
//
// Plain FP64, built with --fmad=false and the reference's evaluation order:
// bit for bit the reference's results.  The boundary fills follow the MPI 2D
// drivers' single-rank routines (periodic along an axis whose table entry 0
// is zero, then mirrors where an entry is nonzero); tables must be all zero
// or all nonzero per axis.  Scratch reuses the 2D step's arrays.
#include "stencil.cuh"

namespace mlau {
namespace {

__device__ __forceinline__ long long at2(const Dims &d, int i, int j)
{
    return (long long)d.nx * j + i;
}

// ---- resistive diffusion ------------------------------------------------------
struct Res {
    double *bx, *by, *bz, *en;  // state
    double *ut[4];              // bx, by, bz, en at the start
    double *ex, *ey, *ez, *fx, *fy;
};

// E = eta0 * J over [2, nx-1) x [2, ny-1) (:772-801)
__global__ void __launch_bounds__(TPB) k_res_e(Res r, Dims d, Box b, int odr, double eta0,
                                               double idx, double idy)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double *bx = r.bx, *by = r.by, *bz = r.bz;
    const double jx = +fdiff(odr, bz[s - 2 * sy], bz[s - sy], bz[s], bz[s + sy]) * idy;
    const double jy = -fdiff(odr, bz[s - 2], bz[s - 1], bz[s], bz[s + 1]) * idx;
    const double jz = +fdiff(odr, by[s - 2], by[s - 1], by[s], by[s + 1]) * idx
                      - fdiff(odr, bx[s - 2 * sy], bx[s - sy], bx[s], bx[s + sy]) * idy;
    r.ex[s] = eta0 * jx;
    r.ey[s] = eta0 * jy;
    r.ez[s] = eta0 * jz;
}

// Energy fluxes: along X over [2, nx-1) x [2, ny-2), along Y over
// [2, nx-2) x [2, ny-1) (:802-852)
__global__ void __launch_bounds__(TPB) k_res_flux(Res r, Dims d, Box b, int odr)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double *bx = r.bx, *by = r.by, *bz = r.bz, *ez = r.ez;
    if (j < d.ny - 2) {
        const double ep = r.ey[s];
        const double bp = face2cen(odr, bz[s - 2], bz[s - 1], bz[s], bz[s + 1]);
        const double em = 0.5 * (ez[s] + ez[s + sy]);
        const double bm = 0.5 * (face2cen(odr, by[s - 2], by[s - 1], by[s], by[s + 1])
                                 + face2cen(odr, by[s + sy - 2], by[s + sy - 1], by[s + sy],
                                            by[s + sy + 1]));
        r.fx[s] = ep * bp - em * bm;
    }
    if (i < d.nx - 2) {
        const double ep = 0.5 * (ez[s] + ez[s + 1]);
        const double bp = 0.5 * (face2cen(odr, bx[s - 2 * sy], bx[s - sy], bx[s], bx[s + sy])
                                 + face2cen(odr, bx[s + 1 - 2 * sy], bx[s + 1 - sy], bx[s + 1],
                                            bx[s + 1 + sy]));
        const double em = r.ex[s];
        const double bm = face2cen(odr, bz[s - 2 * sy], bz[s - sy], bz[s], bz[s + sy]);
        r.fy[s] = ep * bp - em * bm;
    }
}

// CT Bx over [xoff, nx-xoff] x [yoff, ny-yoff), By over [xoff, nx-xoff) x
// [yoff, ny-yoff], Bz and energy over the interior (:854-921)
__global__ void __launch_bounds__(TPB)
k_res_update(Res r, Dims d, Box b, int odr, double ra, double rb, double dtdx, double dtdy)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double *ez = r.ez, *ex = r.ex, *ey = r.ey, *fx = r.fx, *fy = r.fy;
    const bool in_x = i < d.nx - d.ox, in_y = j < d.ny - d.oy;
    if (in_y) {
        const double du = fdiff(odr, ez[s - sy], ez[s], ez[s + sy], ez[s + 2 * sy]);
        r.bx[s] = ra * r.ut[0][s] + rb * (r.bx[s] - dtdy * du);
    }
    if (in_x) {
        const double du = fdiff(odr, ez[s - 1], ez[s], ez[s + 1], ez[s + 2]);
        r.by[s] = ra * r.ut[1][s] + rb * (r.by[s] + dtdx * du);
    }
    if (in_x && in_y) {
        const double d00 = fdiff(odr, ey[s - 1], ey[s], ey[s + 1], ey[s + 2]);
        const double d01 = fdiff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
        const double d10 = fdiff(odr, ex[s - sy], ex[s], ex[s + sy], ex[s + 2 * sy]);
        const double d11 = fdiff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
        r.bz[s] = ra * r.ut[2][s] + rb * (r.bz[s] - dtdx * d00 + dtdy * d10);
        r.en[s] = ra * r.ut[3][s] + rb * (r.en[s] - dtdx * d01 - dtdy * d11);
    }
}

// ---- viscosity ----------------------------------------------------------------
struct Visc {
    const double *ro;
    double *v[3], *en;  // mx, my, mz hold velocities while the operator runs
    double *ut[4];      // vx, vy, vz, en at the start
    double *ir;         // 1 / rho
    double *fx[4], *fy[4];
};

__global__ void __launch_bounds__(TPB) k_visc_begin(Visc q, long long n)
{
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double ir = 1.0 / q.ro[s];
    q.ir[s] = ir;
    for (int c = 0; c < 3; c++) {
        q.v[c][s] *= ir;
        q.ut[c][s] = q.v[c][s];
    }
    q.ut[3][s] = q.en[s];
}

__global__ void __launch_bounds__(TPB) k_visc_end(Visc q, long long n)
{
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    for (int c = 0; c < 3; c++) q.v[c][s] *= q.ro[s];
}

// Fluxes: along X over [2, nx-1) x [1, ny-1), along Y over [1, nx-1) x
// [2, ny-1) (:999-1089)
__global__ void __launch_bounds__(TPB)
k_visc_flux(Visc q, Dims d, Box b, int odr, double nu0, double idx, double idy)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double c2 = 2. / 3., c4 = 4. / 3.;
    const double *vx = q.v[0], *vy = q.v[1], *vz = q.v[2], *ro = q.ro;
    if (i >= 2) {
        const double ro0 = 0.5 * (ro[s] + ro[s - 1]);
        const double rnu = ro0 * nu0;
        const double vx0 = face2cen(odr, vx[s - 2], vx[s - 1], vx[s], vx[s + 1]);
        const double vy0 = face2cen(odr, vy[s - 2], vy[s - 1], vy[s], vy[s + 1]);
        const double vz0 = face2cen(odr, vz[s - 2], vz[s - 1], vz[s], vz[s + 1]);
        const double dvxdx = fdiff(odr, vx[s - 2], vx[s - 1], vx[s], vx[s + 1]) * idx;
        const double dvydx = fdiff(odr, vy[s - 2], vy[s - 1], vy[s], vy[s + 1]) * idx;
        const double dvzdx = fdiff(odr, vz[s - 2], vz[s - 1], vz[s], vz[s + 1]) * idx;
        double dv[4];
#pragma unroll
        for (int m = 0; m < 4; m++) dv[m] = 0.5 * (vx[s - 2 + m + sy] - vx[s - 2 + m - sy]);
        const double dvxdy = face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idy;
#pragma unroll
        for (int m = 0; m < 4; m++) dv[m] = 0.5 * (vy[s - 2 + m + sy] - vy[s - 2 + m - sy]);
        const double dvydy = face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idy;
        const double f0 = -rnu * (c4 * dvxdx - c2 * dvydy);
        const double f1 = -rnu * (dvydx + dvxdy);
        const double f2 = -rnu * (dvzdx);
        q.fx[0][s] = f0;
        q.fx[1][s] = f1;
        q.fx[2][s] = f2;
        q.fx[3][s] = f0 * vx0 + f1 * vy0 + f2 * vz0;
    }
    if (j >= 2) {
        const double ro0 = 0.5 * (ro[s] + ro[s - sy]);
        const double rnu = ro0 * nu0;
        const double vx0 = face2cen(odr, vx[s - 2 * sy], vx[s - sy], vx[s], vx[s + sy]);
        const double vy0 = face2cen(odr, vy[s - 2 * sy], vy[s - sy], vy[s], vy[s + sy]);
        const double vz0 = face2cen(odr, vz[s - 2 * sy], vz[s - sy], vz[s], vz[s + sy]);
        const double dvxdy = fdiff(odr, vx[s - 2 * sy], vx[s - sy], vx[s], vx[s + sy]) * idy;
        const double dvydy = fdiff(odr, vy[s - 2 * sy], vy[s - sy], vy[s], vy[s + sy]) * idy;
        const double dvzdy = fdiff(odr, vz[s - 2 * sy], vz[s - sy], vz[s], vz[s + sy]) * idy;
        double dv[4];
#pragma unroll
        for (int m = 0; m < 4; m++)
            dv[m] = 0.5 * (vx[s + (m - 2) * sy + 1] - vx[s + (m - 2) * sy - 1]);
        const double dvxdx = face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idx;
#pragma unroll
        for (int m = 0; m < 4; m++)
            dv[m] = 0.5 * (vy[s + (m - 2) * sy + 1] - vy[s + (m - 2) * sy - 1]);
        const double dvydx = face2cen(odr, dv[0], dv[1], dv[2], dv[3]) * idx;
        const double g0 = -rnu * (dvxdy + dvydx);
        const double g1 = -rnu * (c4 * dvydy - c2 * dvxdx);
        const double g2 = -rnu * (dvzdy);
        q.fy[0][s] = g0;
        q.fy[1][s] = g1;
        q.fy[2][s] = g2;
        q.fy[3][s] = g0 * vx0 + g1 * vy0 + g2 * vz0;
    }
}

// Update of the interior (:1091-1139)
__global__ void __launch_bounds__(TPB)
k_visc_update(Visc q, Dims d, Box b, int odr, double ra, double rb, double dtdx, double dtdy)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    double du[2][4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const double *fx = q.fx[c], *fy = q.fy[c];
        du[0][c] = fdiff(odr, fx[s - 1], fx[s], fx[s + 1], fx[s + 2]);
        du[1][c] = fdiff(odr, fy[s - sy], fy[s], fy[s + sy], fy[s + 2 * sy]);
    }
#pragma unroll
    for (int c = 0; c < 3; c++)
        q.v[c][s] = ra * q.ut[c][s] + rb * (q.v[c][s] - (dtdx * du[0][c] + dtdy * du[1][c]) * q.ir[s]);
    q.en[s] = ra * q.ut[3][s] + rb * (q.en[s] - (dtdx * du[0][3] + dtdy * du[1][3]));
}

// ---- boundary fill of up to four arrays ----------------------------------------
// Ghost fill of one axis: none, periodic image, or mirror (st: face-centred
// along the axis, dn: +1 Neumann / -1 Dirichlet), as the MPI drivers'
// single-rank routines (mpi_sdrv2d, mpi_xbc2d, mpi_ybc2d in
// 2D/MPI/MRX/boundary.c) leave it.
enum { AX_NONE = 0, AX_PERIODIC = 1, AX_MIRROR = 2 };
struct Axis {
    int mode, st, dn;
};

__device__ __forceinline__ int ax_src(int i, int n, int off, Axis a, double *g)
{
    if (a.mode == AX_PERIODIC) return wrap_idx(i, n, off);
    if (a.mode == AX_MIRROR) return bc_src(i, n, off, a.st, a.dn, g);
    return i;
}

struct Fill {
    double *a[4];
    int n;
    Axis x[4], y[4];
};

// Each ghost takes its source along each axis composed over the two axes,
// times the signs: the result of the reference's periodic exchange followed
// by its x and y mirrors, in one pass (every source is a cell this pass does
// not write).
__global__ void __launch_bounds__(TPB) k_fill2(Fill fl, Dims d, Box b, const int *skip)
{
    if (skip && *skip) return;
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    if (i >= d.ox && i < d.nx - d.ox && j >= d.oy && j < d.ny - d.oy) return;
    const long long s = at2(d, i, j);
#pragma unroll
    for (int v = 0; v < 4; v++) {
        if (v >= fl.n) break;
        double g = 1.0;
        const int si = ax_src(i, d.nx, d.ox, fl.x[v], &g);
        const int sj = ax_src(j, d.ny, d.oy, fl.y[v], &g);
        if (si == i && sj == j) continue;
        fl.a[v][s] = g * fl.a[v][at2(d, si, sj)];
    }
}

// Axis after the reference's sequence: the periodic exchange where the
// axis's table entry 0 is zero, then a mirror by `dn` where it is nonzero.
Axis ax_of(int dn0, int dn, int st)
{
    if (dn != 0) return Axis{AX_MIRROR, st, dn};
    return dn0 == 0 ? Axis{AX_PERIODIC, 0, 0} : Axis{AX_NONE, 0, 0};
}

Fill make_fill(const Sim *s, std::initializer_list<std::pair<double *, int>> arrs)
{
    Fill f{};
    f.n = 0;
    for (auto &p : arrs) {
        const int v = p.second;  // table index (ro mx my mz en bx by bz)
        f.a[f.n] = p.first;
        f.x[f.n] = ax_of(s->bc2.x[0], s->bc2.x[v], v == 5);
        f.y[f.n] = ax_of(s->bc2.y[0], s->bc2.y[v], v == 6);
        f.n++;
    }
    return f;
}

void launch_fill(const Fill &fl, const Dims &d, cudaStream_t st, const int *skip = nullptr)
{
    const Box all{0, 0, 0, d.nx, d.ny, 1};
    k_fill2<<<blocks_for(all.count(), TPB), TPB, 0, st>>>(fl, d, all, skip);
}

// ---- anisotropic heat conduction ------------------------------------------------
// t_conduction with diffusion2d_ani (2D/MPI/MRX/mhd_fd_ct_2d.c:1176-1456):
// conductivity kk0 along B (tensor K from cell B), Crank-Nicolson in the
// temperature T = p/rho, solved by six-colour Gauss-Seidel sweeps.  A colour
// (row parity, column residue mod 3 shifted by the row) is an independent set
// of the 9-point stencil, so one launch per colour reproduces the reference's
// loop order exactly.  The sweeps stop when the summed |residual| is at most
// 1e-6 of the summed |rhs/denominator|, or after cmax sweeps.

struct CondState {
    double anorm_f, anorm;
    int cnt, done, err, pad;
};
constexpr int kRedBlocks = 256;  // fixed reduction grid: sums in a fixed order
constexpr int kRedThreads = 256;
constexpr int kSweepChunk = 8;   // sweeps per captured graph launch
struct CondBuf {
    CondState st;
    double part[kRedBlocks];
};

struct Cond {
    const double *ro, *mx, *my, *mz, *bx, *by, *bz;
    double *en;  // energy -> pressure -> temperature and back
    double *kxx, *kyy, *kxy, *ig, *denom, *rhs, *adt, *res;
    CondBuf *cb;
};

struct CondCoef {
    double d1, d2, idx2, idy2, idxy, alpha, beta, omega;
};

// Conductivity tensor over [1, nx-2) x [1, ny-2) (:1402-1420)
__global__ void __launch_bounds__(TPB) k_cond_tensor(Cond c, Dims d, Box b, int odr, double kk0)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double eps = 1e-6;
    const double bxc = face2cen(odr, c.bx[s - 1], c.bx[s], c.bx[s + 1], c.bx[s + 2]);
    const double byc = face2cen(odr, c.by[s - sy], c.by[s], c.by[s + sy], c.by[s + 2 * sy]);
    const double bzc = c.bz[s];
    const double ib2 = 1.0 / (bxc * bxc + byc * byc + bzc * bzc + eps);
    c.kxx[s] = kk0 * (bxc * bxc + eps) * ib2;
    c.kyy[s] = kk0 * (byc * byc + eps) * ib2;
    c.kxy[s] = kk0 * (bxc * byc) * ib2;
}

// Energy <-> pressure over [1, nx-2) x [1, ny-2) (mhd_e2p, :1176-1219)
__global__ void __launch_bounds__(TPB) k_e2p(Cond c, Dims d, Box b, int odr, double gamma, int direc)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), sy = d.nx;
    const double iro = 1.0 / c.ro[s];
    const double vx = c.mx[s] * iro, vy = c.my[s] * iro, vz = c.mz[s] * iro;
    const double bxc = face2cen(odr, c.bx[s - 1], c.bx[s], c.bx[s + 1], c.bx[s + 2]);
    const double byc = face2cen(odr, c.by[s - sy], c.by[s], c.by[s + sy], c.by[s + 2 * sy]);
    const double bzc = c.bz[s];
    const double v2 = (vx * vx + vy * vy + vz * vz);
    const double b2 = (bxc * bxc + byc * byc + bzc * bzc);
    const double e = c.en[s];
    const double t0 = (gamma - 1) * (e - 0.5 * (c.ro[s] * v2 + b2));
    const double t1 = e / (gamma - 1) + 0.5 * (c.ro[s] * v2 + b2);
    c.en[s] = 0.5 * ((double)(1 + direc) * t0 + (double)(1 - direc) * t1);
}

// Pressure -> temperature, 1/rho and rho-weighted conductivities, every cell
__global__ void __launch_bounds__(TPB) k_cond_prep(Cond c, long long n)
{
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double g = c.ro[s];
    c.en[s] /= g;
    c.ig[s] = 1.0 / g;
    c.kxx[s] *= g;
    c.kyy[s] *= g;
    c.kxy[s] *= g;
}

__global__ void __launch_bounds__(TPB) k_cond_post(Cond c, long long n)
{
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    c.en[s] *= c.ro[s];
}

// The explicit half of the step and the diagonal, over [2, nx-2) x [2, ny-2)
// (:1262-1296)
__global__ void __launch_bounds__(TPB) k_cond_rhs(Cond c, Dims d, Box b, CondCoef q, double dt0)
{
    int i, j, k;
    if (!b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) return;
    const long long s = at2(d, i, j), nx = d.nx;
    const double *f = c.en, *kxx = c.kxx, *kyy = c.kyy, *kxy = c.kxy;
    const long long sim = s - 1, sip = s + 1, sjm = s - nx, sjp = s + nx;
    const double k0 = 0.5 * (kxx[sim] + kxx[s]), k1 = 0.5 * (kxx[sip] + kxx[s]);
    const double k2 = 0.5 * (kyy[sjm] + kyy[s]), k3 = 0.5 * (kyy[sjp] + kyy[s]);
    const double dt = dt0 * c.ig[s];
    const double adt = q.alpha * dt;
    const double den =
        1.0 / (1.0 + adt * q.d1 * (q.idx2 * (k0 + k1) + q.idy2 * (k2 + k3)));
    const double d1 = q.d1, d2 = q.d2;
    const double r =
        f[s] + q.beta * dt *
                   ((+q.idx2 * (+k0 * (d1 * (f[sim] - f[s]) - d2 * (f[s - 2] - f[sip]))
                                + k1 * (d1 * (f[sip] - f[s]) - d2 * (f[s + 2] - f[sim])))
                     + q.idy2 * (+k2 * (d1 * (f[sjm] - f[s]) - d2 * (f[s - 2 * nx] - f[sjp]))
                                 + k3 * (d1 * (f[sjp] - f[s]) - d2 * (f[s + 2 * nx] - f[sjm]))))
                    + 0.25 * (+q.idxy * (+kxy[sjm] * (f[sjm - 1] - f[sjm + 1])
                                         + kxy[sjp] * (f[sjp + 1] - f[sjp - 1])
                                         + kxy[sim] * (f[sjm - 1] - f[sjp - 1])
                                         + kxy[sip] * (f[sjp + 1] - f[sjm + 1]))));
    c.denom[s] = den;
    c.rhs[s] = r;
    c.adt[s] = adt;
    c.res[s] = fabs(r * den);
}

// One colour of a Gauss-Seidel sweep (:1305-1351): rows j = 2 + py + 2a,
// columns i = 4 - ((j + px) % 3) + 3b, inside [2, nx-2) x [2, ny-2).
__global__ void __launch_bounds__(TPB)
k_cond_colour(Cond c, Dims d, CondCoef q, int py, int px, int nb, long long total)
{
    if (c.cb->st.done) return;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total) return;
    const int j = 2 + py + 2 * (int)(t / nb);
    const int i = 4 - ((j + px) % 3) + 3 * (int)(t % nb);
    if (j >= d.ny - 2 || i >= d.nx - 2) return;
    const long long s = at2(d, i, j), nx = d.nx;
    double *f = c.en;
    const double *kxx = c.kxx, *kyy = c.kyy, *kxy = c.kxy;
    const long long sim = s - 1, sip = s + 1, sjm = s - nx, sjp = s + nx;
    const double k0 = 0.5 * (kxx[sim] + kxx[s]), k1 = 0.5 * (kxx[sip] + kxx[s]);
    const double k2 = 0.5 * (kyy[sjm] + kyy[s]), k3 = 0.5 * (kyy[sjp] + kyy[s]);
    const double d1 = q.d1, d2 = q.d2;
    const double resid =
        (c.adt[s] *
             ((+q.idx2 * (+k0 * (d1 * f[sim] - d2 * (f[s - 2] - f[sip]))
                          + k1 * (d1 * f[sip] - d2 * (f[s + 2] - f[sim])))
               + q.idy2 * (+k2 * (d1 * f[sjm] - d2 * (f[s - 2 * nx] - f[sjp]))
                           + k3 * (d1 * f[sjp] - d2 * (f[s + 2 * nx] - f[sjm]))))
              + 0.25 * (+q.idxy * (+kxy[sjm] * (f[sjm - 1] - f[sjm + 1])
                                   + kxy[sjp] * (f[sjp + 1] - f[sjp - 1])
                                   + kxy[sim] * (f[sjm - 1] - f[sjp - 1])
                                   + kxy[sip] * (f[sjp + 1] - f[sjm + 1]))))
         + c.rhs[s]) * c.denom[s] - f[s];
    c.res[s] = fabs(resid);
    f[s] += q.omega * resid;
}

// Block partial sums of res over [2, nx-2) x [2, ny-2): each thread strides
// in a fixed order, then a fixed tree; deterministic for a geometry.  In a
// sweep (gated) it returns at once when the sweeps have stopped.
__global__ void __launch_bounds__(kRedThreads) k_cond_sum(Cond c, Dims d, Box b, int gated)
{
    __shared__ double sh[kRedThreads];
    if (gated && c.cb->st.done) return;
    double acc = 0.0;
    const long long tot = (long long)b.e0 * b.e1 * b.e2;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < tot;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        b.decode(t, i, j, k);
        acc += c.res[at2(d, i, j)];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = kRedThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) c.cb->part[blockIdx.x] = sh[0];
}

// Total of the partial sums; first = 1: the norm of rhs/denominator, which
// also resets the sweep state; else the sweep's residual norm, its count and
// the stopping test (:1353-1369).
__global__ void __launch_bounds__(kRedBlocks) k_cond_check(Cond c, int first, int cmax)
{
    __shared__ double sh[kRedBlocks];
    CondState &st = c.cb->st;
    if (!first && st.done) return;
    sh[threadIdx.x] = c.cb->part[threadIdx.x];
    __syncthreads();
    for (int w = kRedBlocks / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double eps = 1e-6;
    if (first) {
        st.anorm_f = sh[0];
        st.anorm = 0.0;
        st.cnt = 0;
        st.done = 0;
        st.err = 0;
        return;
    }
    st.anorm = sh[0];
    st.cnt += 1;
    if (!((st.anorm > eps * st.anorm_f) && (st.cnt < cmax))) st.done = 1;
    if (st.cnt == cmax) st.err = -1;
}

// ---- RMI inflow ------------------------------------------------------------------
// inj_ro (2D/MPI/RMI/inj_ro.hpp:1-58): rows [ny-yoff, ny), every column, take
// the upstream state; density ro_3 plus dro3 (2u - 1) with the draws u in loop
// order (noise may be null); By on the face row j = ny-yoff keeps its value.
struct Inflow {
    double ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, gam;
};

__global__ void __launch_bounds__(TPB)
k_inject2(PlainFields f, Dims d, Inflow q, const double *noise)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long cnt = (long long)d.oy * d.nx;
    if (t >= cnt) return;
    const int j = d.ny - d.oy + (int)(t / d.nx), i = (int)(t % d.nx);
    const long long s = at2(d, i, j);
    double ro = q.ro3;
    if (noise) ro += q.dro3 * (noise[t] - 0.5) * 2.0;
    const double vx = 0, vz = 0;
    double vy = q.vy1;
    vy -= q.vref;
    const double bxc = q.bx1, byc = q.by1, bzc = q.bz1;
    const double b2 = bxc * bxc + byc * byc + bzc * bzc;
    f.s[0][s] = ro;
    f.s[5][s] = bxc;
    if (j != d.ny - d.oy) f.s[6][s] = q.by1;
    f.s[7][s] = bzc;
    f.s[1][s] = ro * vx;
    f.s[2][s] = ro * vy;
    f.s[3][s] = ro * vz;
    f.s[4][s] = q.pr1 / (q.gam - 1) + 0.5 * (ro * (vx * vx + vy * vy + vz * vz) + b2);
}

int check_2d(Sim *s, const char *what)
{
    if (s->g.dim != 2 || s->precision != MLAU_FP64) {
        set_error("%s: 2D FP64 simulations only", what);
        return MLAU_ERR_ARG;
    }
    for (const int *t : {s->bc2.x, s->bc2.y}) {
        int nz = 0;
        for (int v = 0; v < 8; v++) nz += t[v] != 0;
        if (nz != 0 && nz != 8) {
            set_error("%s: each axis's boundary entries must be all zero or all nonzero", what);
            return MLAU_ERR_ARG;
        }
    }
    return MLAU_OK;
}

}  // namespace

int diff2d_resistive(Sim *s, double eta0, double dt)
{
    int rc = check_2d(s, "resistive diffusion");
    if (rc) return rc;
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, 1, g.ox, g.oy, 0};
    Res r{f.s[5], f.s[6], f.s[7], f.s[4], {f.u0[5], f.u0[6], f.u0[7], f.u0[4]},
          f.ul[0], f.ul[1], f.e[2], f.ur[0], f.ur[1]};
    for (int c = 0; c < 4; c++)
        MLAU_CUDA(cudaMemcpyAsync(r.ut[c], c == 3 ? r.en : (c == 0 ? r.bx : c == 1 ? r.by : r.bz),
                                  sizeof(double) * g.n, cudaMemcpyDeviceToDevice, st));
    const double dtdx = dt / g.dx, dtdy = dt / g.dy, idx = 1. / g.dx, idy = 1. / g.dy;
    const Box e{2, 2, 0, g.nx - 3, g.ny - 3, 1};
    const Box up{g.ox, g.oy, 0, g.nx - 2 * g.ox + 1, g.ny - 2 * g.oy + 1, 1};
    const Fill fb = make_fill(s, {{f.s[5], 5}, {f.s[6], 6}, {f.s[7], 7}});
    const Fill fe = make_fill(s, {{f.s[4], 4}});
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        k_res_e<<<blocks_for(e.count(), TPB), TPB, 0, st>>>(r, d, e, s->odr, eta0, idx, idy);
        k_res_flux<<<blocks_for(e.count(), TPB), TPB, 0, st>>>(r, d, e, s->odr);
        k_res_update<<<blocks_for(up.count(), TPB), TPB, 0, st>>>(r, d, up, s->odr, ra, rb, dtdx,
                                                                  dtdy);
        launch_fill(fb, d, st);
        MLAU_CUDA(cudaGetLastError());
    }
    launch_fill(fe, d, st);
    MLAU_CUDA(cudaGetLastError());
    return MLAU_OK;
}

int diff2d_viscous(Sim *s, double nu0, double dt)
{
    int rc = check_2d(s, "viscosity");
    if (rc) return rc;
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, 1, g.ox, g.oy, 0};
    Visc q{f.s[0], {f.s[1], f.s[2], f.s[3]}, f.s[4], {f.u0[1], f.u0[2], f.u0[3], f.u0[4]}, f.pr,
           {f.F[0][0], f.F[0][1], f.F[0][2], f.F[0][3]}, {f.F[1][0], f.F[1][1], f.F[1][2], f.F[1][3]}};
    const double idx = 1. / g.dx, idy = 1. / g.dy, dtdx = dt * idx, dtdy = dt * idy;
    const Box fl{1, 1, 0, g.nx - 2, g.ny - 2, 1};
    const Box in{g.ox, g.oy, 0, g.nx - 2 * g.ox, g.ny - 2 * g.oy, 1};
    const Fill fv = make_fill(s, {{f.s[1], 1}, {f.s[2], 2}, {f.s[3], 3}});
    const Fill fe = make_fill(s, {{f.s[4], 4}});
    k_visc_begin<<<blocks_for(g.n, TPB), TPB, 0, st>>>(q, g.n);
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        k_visc_flux<<<blocks_for(fl.count(), TPB), TPB, 0, st>>>(q, d, fl, s->odr, nu0, idx, idy);
        k_visc_update<<<blocks_for(in.count(), TPB), TPB, 0, st>>>(q, d, in, s->odr, ra, rb, dtdx,
                                                                   dtdy);
        launch_fill(fv, d, st);
        MLAU_CUDA(cudaGetLastError());
    }
    launch_fill(fe, d, st);
    k_visc_end<<<blocks_for(g.n, TPB), TPB, 0, st>>>(q, g.n);
    MLAU_CUDA(cudaGetLastError());
    return MLAU_OK;
}

namespace {

long long cond_key(const Sim *s, int cmax)
{
    // FNV-1a over the parameters a captured sweep graph bakes in
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *b = (const unsigned char *)p;
        for (size_t k = 0; k < n; k++) h = (h ^ b[k]) * 1099511628211ull;
    };
    mix(&s->odr, sizeof(int));
    mix(&s->g.dx, sizeof(double));
    mix(&s->g.dy, sizeof(double));
    mix(s->bc2.x, sizeof(s->bc2.x));
    mix(s->bc2.y, sizeof(s->bc2.y));
    mix(&cmax, sizeof(int));
    return (long long)(h & 0x7fffffffffffffffull);
}

// One Gauss-Seidel sweep: six colours, the temperature's ghost fill, the
// residual norm and the stopping test; every launch returns at once when an
// earlier sweep has stopped.
void enqueue_sweep(Sim *s, const Cond &c, const Dims &d, const CondCoef &q, const Fill &ft,
                   int cmax, cudaStream_t st)
{
    const int nb = (d.nx - 4 + 2) / 3;
    for (int py = 0; py < 2; py++) {
        const long long rows = (d.ny - 4 - py + 1) / 2;
        for (int px = 0; px < 3; px++) {
            const long long total = rows * nb;
            k_cond_colour<<<blocks_for(total, TPB), TPB, 0, st>>>(c, d, q, py, px, nb, total);
        }
    }
    launch_fill(ft, d, st, &c.cb->st.done);
    const Box in{2, 2, 0, d.nx - 4, d.ny - 4, 1};
    k_cond_sum<<<kRedBlocks, kRedThreads, 0, st>>>(c, d, in, 1);
    k_cond_check<<<1, kRedBlocks, 0, st>>>(c, 0, cmax);
}

}  // namespace

void diff2d_free(Sim *s)
{
    if (s->cond_exec) cudaGraphExecDestroy(s->cond_exec);
    if (s->d_cond) cudaFree(s->d_cond);
    if (s->h_cond) cudaFreeHost(s->h_cond);
    s->cond_exec = nullptr;
    s->d_cond = s->h_cond = nullptr;
}

int diff2d_conduction(Sim *s, double kk0, double dt, int *sweeps)
{
    int rc = check_2d(s, "heat conduction");
    if (rc) return rc;
    const int cmax = 2048;  // CMAX, 2D/MPI/MRX/mhd_fd_ct_2d.c:30
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, 1, g.ox, g.oy, 0};
    if (!s->d_cond) {
        MLAU_CUDA(cudaMalloc(&s->d_cond, sizeof(CondBuf)));
        MLAU_CUDA(cudaMallocHost(&s->h_cond, sizeof(CondState)));
    }
    // a fresh sweep state (the first reduction below then sets it up)
    MLAU_CUDA(cudaMemsetAsync(s->d_cond, 0, sizeof(CondState), st));
    const Cond c{f.s[0], f.s[1], f.s[2], f.s[3], f.s[5], f.s[6], f.s[7], f.s[4],
                 f.ul[0], f.ul[1], f.ul[2], f.ul[3], f.ul[4], f.ul[5], f.ul[6], f.ur[0],
                 (CondBuf *)s->d_cond};
    const int od4 = (lin_odr(s->odr) - 1) / 2;
    CondCoef q;
    q.d1 = 1.0 + 0.25 * od4;
    q.d2 = 1.0 * od4 / 12.0;
    q.idx2 = 1.0 / (g.dx * g.dx);
    q.idy2 = 1.0 / (g.dy * g.dy);
    q.idxy = 1.0 / (g.dx * g.dy);
    q.alpha = 0.5;
    q.beta = 1.0 - q.alpha;
    q.omega = 1.0;
    const int *tx = s->bc2.x, *ty = s->bc2.y;
    // tensor: its own mirrors (products of the B entries), then the
    // energy -> pressure -> temperature conversion
    Fill fk{};
    fk.n = 3;
    fk.a[0] = c.kxx; fk.a[1] = c.kyy; fk.a[2] = c.kxy;
    fk.x[0] = ax_of(tx[0], tx[5] * tx[5], 0);
    fk.x[1] = ax_of(tx[0], tx[6] * tx[6], 0);
    fk.x[2] = ax_of(tx[0], tx[5] * tx[6], 0);
    fk.y[0] = ax_of(ty[0], ty[5] * ty[5], 0);
    fk.y[1] = ax_of(ty[0], ty[6] * ty[6], 0);
    fk.y[2] = ax_of(ty[0], ty[5] * ty[6], 0);
    Fill fe{};
    fe.n = 1;
    fe.a[0] = c.en;
    fe.x[0] = ax_of(tx[0], tx[4], 0);
    fe.y[0] = ax_of(ty[0], ty[4], 0);
    // the temperature during the sweeps: x as the exchange leaves it, y
    // Neumann mirror (diffusion2d_ani's call, :1437)
    Fill ft{};
    ft.n = 1;
    ft.a[0] = c.en;
    ft.x[0] = ax_of(tx[0], 0, 0);
    ft.y[0] = ax_of(ty[0], +1, 0);
    const Box cen{1, 1, 0, g.nx - 3, g.ny - 3, 1};
    const Box in{2, 2, 0, g.nx - 4, g.ny - 4, 1};
    k_cond_tensor<<<blocks_for(cen.count(), TPB), TPB, 0, st>>>(c, d, cen, s->odr, kk0);
    launch_fill(fk, d, st);
    k_e2p<<<blocks_for(cen.count(), TPB), TPB, 0, st>>>(c, d, cen, s->odr, s->gamma, +1);
    launch_fill(fe, d, st);
    k_cond_prep<<<blocks_for(g.n, TPB), TPB, 0, st>>>(c, g.n);
    k_cond_rhs<<<blocks_for(in.count(), TPB), TPB, 0, st>>>(c, d, in, q, dt);
    k_cond_sum<<<kRedBlocks, kRedThreads, 0, st>>>(c, d, in, 0);
    k_cond_check<<<1, kRedBlocks, 0, st>>>(c, 1, cmax);
    MLAU_CUDA(cudaGetLastError());
    // the sweeps, kSweepChunk per graph launch, until the state says stop
    const long long key = cond_key(s, cmax);
    if (!s->cond_exec || s->cond_key != key) {
        if (s->cond_exec) {
            cudaGraphExecDestroy(s->cond_exec);
            s->cond_exec = nullptr;
        }
        cudaGraph_t gr = nullptr;
        MLAU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kSweepChunk; k++) enqueue_sweep(s, c, d, q, ft, cmax, st);
        const cudaError_t e = cudaStreamEndCapture(st, &gr);
        if (e != cudaSuccess) {
            set_error("sweep graph capture: %s", cudaGetErrorString(e));
            return MLAU_ERR_CUDA;
        }
        const cudaError_t ei = cudaGraphInstantiate(&s->cond_exec, gr, 0);
        cudaGraphDestroy(gr);
        if (ei != cudaSuccess) {
            s->cond_exec = nullptr;
            set_error("sweep graph instantiate: %s", cudaGetErrorString(ei));
            return MLAU_ERR_CUDA;
        }
        s->cond_key = key;
    }
    CondState *hs = (CondState *)s->h_cond;
    for (int launched = 0; launched < cmax; launched += kSweepChunk) {
        MLAU_CUDA(cudaGraphLaunch(s->cond_exec, st));
        MLAU_CUDA(cudaMemcpyAsync(hs, s->d_cond, sizeof(CondState), cudaMemcpyDeviceToHost, st));
        MLAU_CUDA(cudaStreamSynchronize(st));
        if (hs->done) break;
    }
    k_cond_post<<<blocks_for(g.n, TPB), TPB, 0, st>>>(c, g.n);
    k_e2p<<<blocks_for(cen.count(), TPB), TPB, 0, st>>>(c, d, cen, s->odr, s->gamma, -1);
    launch_fill(fe, d, st);
    MLAU_CUDA(cudaGetLastError());
    if (sweeps) *sweeps = hs->cnt;
    if (hs->err) {
        set_error("heat conduction did not converge within %d sweeps", cmax);
        return MLAU_ERR_CONVERGE;
    }
    return MLAU_OK;
}

int diff2d_inject(Sim *s, double ro3, double dro3, double vy1, double bx1, double by1, double bz1,
                  double pr1, double vref, const double *noise)
{
    if (s->g.dim != 2 || s->precision != MLAU_FP64) {
        set_error("inflow injection: 2D FP64 simulations only");
        return MLAU_ERR_ARG;
    }
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const Dims d{g.nx, g.ny, 1, g.ox, g.oy, 0};
    const long long cnt = (long long)g.oy * g.nx;
    double *dn = nullptr;
    if (noise) {
        dn = f.ur[6];  // scratch of n >= cnt cells
        MLAU_CUDA(cudaMemcpyAsync(dn, noise, sizeof(double) * cnt, cudaMemcpyHostToDevice, st));
    }
    const Inflow q{ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, s->gamma};
    k_inject2<<<blocks_for(cnt, TPB), TPB, 0, st>>>(f, d, q, dn);
    // the main loop's periodic exchange of the 8 arrays (RMI main.cpp:50-54)
    for (int h = 0; h < 2; h++) {
        Fill fl{};
        fl.n = 4;
        for (int v = 0; v < 4; v++) {
            fl.a[v] = f.s[4 * h + v];
            fl.x[v] = ax_of(s->bc2.x[0], 0, 0);
            fl.y[v] = ax_of(s->bc2.y[0], 0, 0);
        }
        launch_fill(fl, d, st);
    }
    MLAU_CUDA(cudaGetLastError());
    if (noise) MLAU_CUDA(cudaStreamSynchronize(st));  // the host draws may be reused at once
    return MLAU_OK;
}

}  // namespace mlau
