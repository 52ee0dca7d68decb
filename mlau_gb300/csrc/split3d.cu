// FP32-split 3D step.  Same scheme and data layout as the plain FP64 step
// (3D/MPI/OTvortex/mhd_fd_ct_3d.c), with the arithmetic split by what needs
// FP64:
//
//   FP64  conserved state, its RK3 accumulation of flux differences, primitive
//         recovery p = (gamma-1)(E - rho v^2/2 - B^2/2) (cancellation at low
//         Mach and low beta), the CT curl update of face B (div B at round-off).
//   FP32  characteristic reconstruction and the Riemann solver, the edge EMFs,
//         the CT weights and shock sensors.
//
// Reconstruction works on perturbations from the cell centre, q_m - q_c, and
// WCNS/MUSCL/linear weights are translation invariant, so the face states
// keep FP32 relative accuracy in the perturbation, not in the absolute value.
// The Riemann solver receives its total-pressure and normal-velocity jumps
// formed the same way (centre difference + perturbation difference).
//
// The primitives leave the FP64 prep kernel as (hi, lo) float pairs with
// q = hi + lo to ~48 bits, so every later difference q_m - q_c is formed in
// FP32 as (hi_m - hi_c) + (lo_m - lo_c) without losing the perturbation.
// Flux differences are formed in FP32 (neighbouring fluxes of one sign
// subtract exactly) and added to the FP64 state in FP64.
//
// Kernels per RK stage: prep (FP64 primitive recovery -> float pairs), aux
// (FP32 CT weights and shock sensors), one fused reconstruction + flux kernel
// per direction (shared-memory tile: each thread reconstructs one cell, then
// each face thread solves one Riemann problem), emf (FP32), update (FP64 RK
// combine + CT curl + periodic ghost images).
#include "sim.cuh"
#include "point.cuh"

namespace mlau {

struct SplitFields {
    float2 *q[8];    // ro, vx, vy, vz, cx, cy, cz, pr as (hi, lo) pairs
    float *bf[3];    // face-centred bx, by, bz rounded to FP32
    float *F[3][7];
    float *FC[3][2];
    float *e[3];
    float *m2;
    float *ct[3];
    float *dv[3];
};

namespace {

struct Dims {
    int nx, ny, nz, ox, oy, oz;
    __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)nx * ((long long)ny * k + j) + i;
    }
};

// --- primitives (FP64 recovery, FP32-pair output) ------------------------
__device__ __forceinline__ float2 split2(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

__global__ void __launch_bounds__(256)
ks_prim(PlainFields f, SplitFields g, Dims d, int odr, double gamma)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.nx) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long w = d.at(wrap_idx(i, d.nx, d.ox), wrap_idx(j, d.ny, d.oy), wrap_idx(k, d.nz, d.oz));
    const double *bx = f.s[5], *by = f.s[6], *bz = f.s[7];
    const double cx = face2cen(odr, bx[w - 1], bx[w], bx[w + 1], bx[w + 2]);
    const double cy = face2cen(odr, by[w - sy], by[w], by[w + sy], by[w + 2 * sy]);
    const double cz = face2cen(odr, bz[w - sz], bz[w], bz[w + sz], bz[w + 2 * sz]);
    const long long s = d.at(i, j, k);
    const double ro = f.s[0][s];
    // Velocities and the kinetic energy in FP32: rho v^2/2 enters the pressure
    // as an additive term, so its FP32 rounding (1e-7 of itself) stays below
    // the pressure's own FP32 resolution at any Mach number; the cancelling
    // terms E and B^2/2 stay FP64.
    const float rof = (float)ro, irof = 1.0f / rof;
    const float vx = (float)f.s[1][s] * irof, vy = (float)f.s[2][s] * irof,
                vz = (float)f.s[3][s] * irof;
    const float v2 = vx * vx + vy * vy + vz * vz;
    const double b2 = cx * cx + cy * cy + cz * cz;
    const double pr = (gamma - 1) * (f.s[4][s] - 0.5 * ((double)(rof * v2) + b2));
    g.q[0][s] = split2(ro);
    g.q[1][s] = make_float2(vx, 0.f);
    g.q[2][s] = make_float2(vy, 0.f);
    g.q[3][s] = make_float2(vz, 0.f);
    g.q[4][s] = split2(cx);
    g.q[5][s] = split2(cy);
    g.q[6][s] = split2(cz);
    g.q[7][s] = split2(pr);
    g.bf[0][s] = (float)bx[s];
    g.bf[1][s] = (float)by[s];
    g.bf[2][s] = (float)bz[s];
    g.m2[s] = v2 / ((float)gamma * (float)pr * irof);
}

// --- CT weights and shock sensors (FP32) ----------------------------------
__device__ __forceinline__ float qf(const float2 *a, long long s) { return a[s].x + a[s].y; }
// difference a[s] - a[t] from the pairs
__device__ __forceinline__ float qd(const float2 *a, long long s, long long t)
{
    const float2 u = a[s], v = a[t];
    return (u.x - v.x) + (u.y - v.y);
}

__device__ __forceinline__ float ct_w(const float2 *va, const float2 *vb, const float2 *ro,
                                      const float *ba, const float *bbf, long long s, long long P,
                                      long long Q, long long oa, long long ob)
{
    const float eps = 1e-6f;
    float a = 0.25f * (qf(va, s - P - Q) + qf(va, s - P) + qf(va, s - Q) + qf(va, s));
    float c = 0.25f * (qf(vb, s - P - Q) + qf(vb, s - P) + qf(vb, s - Q) + qf(vb, s));
    float rc = 0.25f * (qf(ro, s - P - Q) + qf(ro, s - P) + qf(ro, s - Q) + qf(ro, s));
    rc = rsqrtf(rc);
    const float fa = 0.5f * (ba[s - oa] + ba[s]);
    const float fb = 0.5f * (bbf[s - ob] + bbf[s]);
    a = fabsf(a) + fabsf(fa * rc);
    c = fabsf(c) + fabsf(fb * rc);
    return (a + 0.5f * eps) / (a + c + eps);
}

__global__ void __launch_bounds__(256) ks_aux(SplitFields g, Dims d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.nx) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long s = d.at(i, j, k);
    const float2 *ro = g.q[0], *vx = g.q[1], *vy = g.q[2], *vz = g.q[3];
    g.ct[0][s] = (i >= 1 && j >= 1) ? ct_w(vx, vy, ro, g.bf[0], g.bf[1], s, sy, 1, sy, 1) : 0.5f;
    g.ct[1][s] = (j >= 1 && k >= 1) ? ct_w(vy, vz, ro, g.bf[1], g.bf[2], s, sz, sy, sz, sy) : 0.5f;
    g.ct[2][s] = (k >= 1 && i >= 1) ? ct_w(vz, vx, ro, g.bf[2], g.bf[0], s, sz, 1, 1, sz) : 0.5f;
    const long long w = d.at(wrap_idx(i, d.nx, d.ox), wrap_idx(j, d.ny, d.oy), wrap_idx(k, d.nz, d.oz));
    g.dv[0][s] = fminf(qd(vx, w + 1, w), qd(vx, w, w - 1));
    g.dv[1][s] = fminf(qd(vy, w + sy, w), qd(vy, w, w - sy));
    g.dv[2][s] = fminf(qd(vz, w + sz, w), qd(vz, w, w - sz));
}

// --- fused reconstruction + Riemann flux along axis D ----------------------
// Rotated views: normal/tangential velocity, cell B (normal, t, u), face B.
struct View {
    const float2 *vn, *vt, *vu, *cn, *ct, *cu;
    const float *bface, *dvt, *dvu;
};

// Tile: TA threads along the fast (x) axis x TB along the second axis.  For
// D=0 the sweep runs along x (TA cells per tile, TB rows); for D=1,2 it runs
// along the second axis (TB cells per tile, TA columns of x).  A tile of T
// cells yields T-1 faces; consecutive tiles overlap by one cell.
template <int D> struct Tile;
template <> struct Tile<0> { static constexpr int TA = 32, TB = 4; };
template <> struct Tile<1> { static constexpr int TA = 16, TB = 16; };
template <> struct Tile<2> { static constexpr int TA = 16, TB = 16; };

// Per-cell results in shared memory, stored variable-major ([var][TB][TA]) so
// that the lanes of a warp touch consecutive words (no bank conflicts):
//   sl - perturbation at the cell's right face (left state of face c+1) + 2 central parts
//   sr - at its left face (right state of face c) + 2 central parts
//   sb - the cell-centre state (ro, vn, vt, vu, bt, bu, pr) as (hi, lo)

template <int D>
__global__ void __launch_bounds__(Tile<D>::TA *Tile<D>::TB)
ks_sweep(SplitFields g, View v, Dims d, int odr, int which, float gamma)
{
    constexpr int TA = Tile<D>::TA, TB = Tile<D>::TB;
    constexpr int T = (D == 0) ? TA : TB;  // cells per tile along the sweep
    __shared__ float sl[9][TB][TA], sr[9][TB][TA];
    __shared__ float2 sb[7][TB][TA];
    const int ta = threadIdx.x, tb = threadIdx.y;
    const int p = (D == 0) ? ta : tb;  // position along the sweep inside the tile
    int i, j, k, len;
    long long st;
    if (D == 0) {
        len = d.nx;
        st = 1;
        i = 2 + blockIdx.x * (T - 1) + ta;
        const long long row = (long long)blockIdx.y * TB + tb;
        j = (int)(row % d.ny);
        k = (int)(row / d.ny);
        if (row >= (long long)d.ny * d.nz) k = d.nz;  // out of range
    } else if (D == 1) {
        len = d.ny;
        st = d.nx;
        i = blockIdx.x * TA + ta;
        j = 2 + blockIdx.y * (T - 1) + tb;
        k = blockIdx.z;
    } else {
        len = d.nz;
        st = (long long)d.nx * d.ny;
        i = blockIdx.x * TA + ta;
        k = 2 + blockIdx.y * (T - 1) + tb;
        j = blockIdx.z;
    }
    const int a = (D == 0) ? i : (D == 1 ? j : k);  // sweep coordinate
    const bool in_box = i < d.nx && j < d.ny && k < d.nz;
    const bool do_rec = in_box && a >= 2 && a < len - 2;
    const long long c = in_box ? d.at(i, j, k) : 0;

    if (do_rec) {
        const float2 *src[7] = {g.q[0], v.vn, v.vt, v.vu, v.ct, v.cu, g.q[7]};
        float dq[7][5], qc[7];
        unsigned zero = 0;
#pragma unroll
        for (int n = 0; n < 7; n++) {
            float2 h[5];
#pragma unroll
            for (int m = 0; m < 5; m++) h[m] = src[n][c + st * (m - 2)];
            qc[n] = h[2].x + h[2].y;
            bool z = true;
#pragma unroll
            for (int m = 0; m < 5; m++) {
                dq[n][m] = (h[m].x - h[2].x) + (h[m].y - h[2].y);
                z = z && (h[m].x == 0.f) && (h[m].y == 0.f);
            }
            if (z) zero |= 1u << n;
            sb[n][tb][ta] = h[2];
        }
        float ul[7], ur[7];
        const float bnc = qf(v.cn, c);
        const float mm = fmaxf(g.m2[c - st], fmaxf(g.m2[c], g.m2[c + st]));
        if (mm >= 1.0f) reconst_full_core(odr, dq, qc, bnc, gamma, ul, ur);
        else reconst_alfven_core(odr, dq, qc, bnc, gamma, ul, ur);
#pragma unroll
        for (int n = 1; n <= 5; n++)
            if (zero & (1u << n)) { ul[n] = 0.f; ur[n] = 0.f; }
#pragma unroll
        for (int n = 0; n < 7; n++) { sl[n][tb][ta] = ul[n]; sr[n][tb][ta] = ur[n]; }
        // central parts of the two tangential B fluxes: lin(bt vn) - bn_face lin(vt)
        const float bl = v.bface[c + st], br = v.bface[c];
#pragma unroll
        for (int t = 0; t < 2; t++) {
            const int kb = 4 + t, kv = 2 + t;
            const float a0 = (qc[kb]) * (qc[1]);
            float da[5];
#pragma unroll
            for (int m = 0; m < 5; m++)
                da[m] = (qc[kb] + dq[kb][m]) * (qc[1] + dq[1][m]) - a0;
            const float al = a0 + lin_l(odr, da[0], da[1], da[2], da[3], da[4]);
            const float ar = a0 + lin_r(odr, da[0], da[1], da[2], da[3], da[4]);
            const float vl = qc[kv] + lin_l(odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
            const float vr = qc[kv] + lin_r(odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
            sl[7 + t][tb][ta] = al - bl * vl;
            sr[7 + t][tb][ta] = ar - br * vr;
        }
    }
    __syncthreads();

    if (!in_box || p == 0 || a < 3 || a >= len - 2) return;
    const int tbl = (D == 0) ? tb : tb - 1, tal = (D == 0) ? ta - 1 : ta;
    float L[7], Rr[7];
#pragma unroll
    for (int n = 0; n < 7; n++) {
        L[n] = (sb[n][tbl][tal].x + sb[n][tbl][tal].y) + sl[n][tbl][tal];
        Rr[n] = (sb[n][tb][ta].x + sb[n][tb][ta].y) + sr[n][tb][ta];
    }
    // jumps from split parts: centre difference from the pairs, plus the
    // difference of the FP32 perturbations
    auto jump = [&](int n) {
        return ((sb[n][tb][ta].x - sb[n][tbl][tal].x) + (sb[n][tb][ta].y - sb[n][tbl][tal].y))
               + (sr[n][tb][ta] - sl[n][tbl][tal]);
    };
    const float jv = jump(1);
    const float jp = jump(6) + 0.5f * (jump(4) * (Rr[4] + L[4]) + jump(5) * (Rr[5] + L[5]));
    const float bn = v.bface[c];
    const float dv0 = (sb[1][tb][ta].x - sb[1][tbl][tal].x) + (sb[1][tb][ta].y - sb[1][tbl][tal].y);
    const float dvtm = fminf(fminf(v.dvt[c - st], v.dvt[c]), fminf(v.dvu[c - st], v.dvu[c]));
    float F[7];
    riemann_jumps(which, L, Rr, bn, gamma, dv0, dvtm, F, jp, jv);
    const float fct = 0.5f * (sl[7][tbl][tal] + sr[7][tb][ta]);
    const float fcu = 0.5f * (sl[8][tbl][tal] + sr[8][tb][ta]);
    F[4] -= fct;
    F[5] -= fcu;
#pragma unroll
    for (int n = 0; n < 7; n++) g.F[D][n][c] = F[n];
    g.FC[D][0][c] = fct;
    g.FC[D][1][c] = fcu;
}

// --- edge EMFs (FP32) --------------------------------------------------------
__device__ __forceinline__ float emf_part32(const float *fu, const float *fc, float w, float h,
                                            long long c, long long st, int odr)
{
    const float ul0 = lin_l(odr, fu[c - 3 * st], fu[c - 2 * st], fu[c - st], fu[c], fu[c + st]);
    const float ul1 = lin_l(odr, fc[c - 3 * st], fc[c - 2 * st], fc[c - st], fc[c], fc[c + st]);
    const float ur0 = lin_r(odr, fu[c - 2 * st], fu[c - st], fu[c], fu[c + st], fu[c + 2 * st]);
    const float ur1 = lin_r(odr, fc[c - 2 * st], fc[c - st], fc[c], fc[c + st], fc[c + 2 * st]);
    return h * ((ul0 + ur0) + w * (ul1 + ur1));
}

__global__ void __launch_bounds__(256) ks_emf(SplitFields g, Dims d, int odr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, k = blockIdx.z;
    if (i >= d.nx) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long c = d.at(i, j, k);
    const bool xi = (i >= 3 && i < d.nx - 2), yj = (j >= 3 && j < d.ny - 2),
               zk = (k >= 3 && k < d.nz - 2);
    float ez = 0.f, ex = 0.f, ey = 0.f;
    if (xi && yj) {
        const float w = g.ct[0][c];
        ez = emf_part32(g.F[0][4], g.FC[0][0], 1.f - w, -0.5f, c, sy, odr)
             + emf_part32(g.F[1][5], g.FC[1][1], w, 0.5f, c, 1, odr);
    }
    if (yj && zk) {
        const float w = g.ct[1][c];
        ex = emf_part32(g.F[1][4], g.FC[1][0], 1.f - w, -0.5f, c, sz, odr)
             + emf_part32(g.F[2][5], g.FC[2][1], w, 0.5f, c, sy, odr);
    }
    if (zk && xi) {
        const float w = g.ct[2][c];
        ey = emf_part32(g.F[0][5], g.FC[0][1], w, 0.5f, c, sz, odr)
             + emf_part32(g.F[2][4], g.FC[2][0], 1.f - w, -0.5f, c, 1, odr);
    }
    g.e[0][c] = ex;
    g.e[1][c] = ey;
    g.e[2][c] = ez;
}

// --- RK combine + CT curl ------------------------------------------------------
// The flux divergence dt/dx dF + dt/dy dG + dt/dz dH is formed in FP32 (each
// difference of neighbouring FP32 fluxes is exact when they share sign and
// magnitude) and accumulated into the FP64 state in FP64.
__device__ __forceinline__ float df32(int odr, const float *f, long long s, long long st)
{
    return fdiff(odr, f[s - st], f[s], f[s + st], f[s + 2 * st]);
}

// FP64 face-to-centre difference of FP32 edge EMFs; the 1/24 of the 4th-order
// stencil is a multiplication here (no FP64 division).
__device__ __forceinline__ double df64(int odr, const float *f, long long s, long long st)
{
    const double f0 = f[s - st], f1 = f[s], f2 = f[s + st], f3 = f[s + 2 * st];
    if (odr <= 2) return f2 - f1;
    return (27.0 * (f2 - f1) - (f3 - f0)) * (1.0 / 24.0);
}

__global__ void __launch_bounds__(256)
ks_update(PlainFields f, SplitFields g, Dims d, int odr, double ra, double rb, float dtdx,
          float dtdy, float dtdz, double dtdx_d, double dtdy_d, double dtdz_d)
{
    const int i = d.ox + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = d.oy + blockIdx.y, k = d.oz + blockIdx.z;
    if (i >= d.nx - d.ox) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long s = d.at(i, j, k);
    const int cX[5] = {0, 1, 2, 3, 6}, cY[5] = {0, 3, 1, 2, 6}, cZ[5] = {0, 2, 3, 1, 6};
    double out[8];
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const float div = dtdx * df32(odr, g.F[0][cX[v]], s, 1) + dtdy * df32(odr, g.F[1][cY[v]], s, sy)
                          + dtdz * df32(odr, g.F[2][cZ[v]], s, sz);
        out[v] = ra * f.u0[v][s] + rb * (f.s[v][s] - (double)div);
    }
    // CT curl in FP64: the differences of the FP32 edge EMFs are exact in
    // FP64, so the discrete divergence of the B increment cancels to FP64
    // round-off (in FP32, 27*(E2-E1) alone would need more than 24 bits).
    const double ddx = (double)dtdx_d, ddy = (double)dtdy_d, ddz = (double)dtdz_d;
    out[5] = ra * f.u0[5][s] + rb * (f.s[5][s] - ddy * df64(odr, g.e[2], s, sy)
                                     + ddz * df64(odr, g.e[1], s, sz));
    out[6] = ra * f.u0[6][s] + rb * (f.s[6][s] - ddz * df64(odr, g.e[0], s, sz)
                                     + ddx * df64(odr, g.e[2], s, 1));
    out[7] = ra * f.u0[7][s] + rb * (f.s[7][s] - ddx * df64(odr, g.e[1], s, 1)
                                     + ddy * df64(odr, g.e[0], s, sy));
    const int Nx = d.nx - 2 * d.ox, Ny = d.ny - 2 * d.oy, Nz = d.nz - 2 * d.oz;
    const int is[3] = {i, i < 2 * d.ox ? i + Nx : -1, i >= Nx ? i - Nx : -1};
    const int js[3] = {j, j < 2 * d.oy ? j + Ny : -1, j >= Ny ? j - Ny : -1};
    const int ks[3] = {k, k < 2 * d.oz ? k + Nz : -1, k >= Nz ? k - Nz : -1};
    for (int cc = 0; cc < 3; cc++) {
        if (ks[cc] < 0) continue;
        for (int bb = 0; bb < 3; bb++) {
            if (js[bb] < 0) continue;
            for (int aa = 0; aa < 3; aa++) {
                if (is[aa] < 0) continue;
                const long long t = d.at(is[aa], js[bb], ks[cc]);
#pragma unroll
                for (int v = 0; v < 8; v++) f.s[v][t] = out[v];
            }
        }
    }
}

View make_view(const SplitFields &g, int D)
{
    if (D == 0) return {g.q[1], g.q[2], g.q[3], g.q[4], g.q[5], g.q[6], g.bf[0], g.dv[1], g.dv[2]};
    if (D == 1) return {g.q[2], g.q[3], g.q[1], g.q[5], g.q[6], g.q[4], g.bf[1], g.dv[2], g.dv[0]};
    return {g.q[3], g.q[1], g.q[2], g.q[6], g.q[4], g.q[5], g.bf[2], g.dv[0], g.dv[1]};
}

int falloc(Sim *s, float **p, long long n)
{
    double *q = nullptr;
    int rc = dalloc(s, &q, (n + 1) / 2);
    *p = (float *)q;
    return rc;
}

}  // namespace

int split3d_alloc(Sim *s)
{
    if (s->g.dim != 3) { set_error("FP32-split mode is 3D only"); return MLAU_ERR_ARG; }
    PlainFields &f = s->f;
    const long long n = s->g.n;
    int rc = 0;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, &f.s[v], n) | dalloc(s, &f.u0[v], n);
    s->sp = new SplitFields();
    SplitFields &g = *s->sp;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, (double **)&g.q[v], n);
    for (int D = 0; D < 3; D++) rc |= falloc(s, &g.bf[D], n);
    for (int D = 0; D < 3; D++) {
        for (int v = 0; v < 7; v++) rc |= falloc(s, &g.F[D][v], n);
        rc |= falloc(s, &g.FC[D][0], n) | falloc(s, &g.FC[D][1], n);
        rc |= falloc(s, &g.e[D], n) | falloc(s, &g.ct[D], n) | falloc(s, &g.dv[D], n);
    }
    rc |= falloc(s, &g.m2, n);
    return rc ? MLAU_ERR_NOMEM : MLAU_OK;
}

void split3d_free(Sim *s)
{
    delete s->sp;
    s->sp = nullptr;
}

int split3d_step(Sim *s, double dt)
{
    const Geometry &G = s->g;
    PlainFields &f = s->f;
    SplitFields &g = *s->sp;
    cudaStream_t st = s->stream;
    const Dims d{G.nx, G.ny, G.nz, G.ox, G.oy, G.oz};
    {
        TimedLaunch tl(&s->timer, KK_COPY);
        for (int v = 0; v < 8; v++)
            MLAU_CUDA(cudaMemcpyAsync(f.u0[v], f.s[v], sizeof(double) * G.n,
                                      cudaMemcpyDeviceToDevice, st));
    }
    const dim3 cb(128), cg(blocks_for(G.nx, 128), G.ny, G.nz);
    const dim3 ug(blocks_for(G.nx - 2 * G.ox, 128), G.ny - 2 * G.oy, G.nz - 2 * G.oz);
    const float gam = (float)s->gamma;
    for (int rk = 0; rk < s->nrk; rk++) {
        const double t[3][2] = {{0.0, 1.0},
                                {0.5 + (s->nrk - 2) * 0.25, 0.5 - (s->nrk - 2) * 0.25},
                                {1. / 3., 2. / 3.}};
        const double ra = t[rk][0], rb = t[rk][1];
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_PREP);
            ks_prim<<<cg, cb, 0, st>>>(f, g, d, s->odr, s->gamma);
            ks_aux<<<cg, cb, 0, st>>>(g, d);
        }
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_SWEEP);
            {
                constexpr int T = Tile<0>::TA;
                dim3 b(Tile<0>::TA, Tile<0>::TB);
                dim3 gr(blocks_for(G.nx - 5, T - 1), blocks_for((long long)G.ny * G.nz, Tile<0>::TB));
                ks_sweep<0><<<gr, b, 0, st>>>(g, make_view(g, 0), d, s->odr, s->flux, gam);
            }
            {
                constexpr int T = Tile<1>::TB;
                dim3 b(Tile<1>::TA, Tile<1>::TB);
                dim3 gr(blocks_for(G.nx, Tile<1>::TA), blocks_for(G.ny - 5, T - 1), G.nz);
                ks_sweep<1><<<gr, b, 0, st>>>(g, make_view(g, 1), d, s->odr, s->flux, gam);
            }
            {
                constexpr int T = Tile<2>::TB;
                dim3 b(Tile<2>::TA, Tile<2>::TB);
                dim3 gr(blocks_for(G.nx, Tile<2>::TA), blocks_for(G.nz - 5, T - 1), G.ny);
                ks_sweep<2><<<gr, b, 0, st>>>(g, make_view(g, 2), d, s->odr, s->flux, gam);
            }
        }
        {
            TimedLaunch tl(&s->timer, KK_EMF);
            ks_emf<<<cg, cb, 0, st>>>(g, d, s->odr);
        }
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_UPDATE);
            ks_update<<<ug, cb, 0, st>>>(f, g, d, s->odr, ra, rb, (float)(dt / G.dx),
                                         (float)(dt / G.dy), (float)(dt / G.dz), dt / G.dx,
                                         dt / G.dy, dt / G.dz);
        }
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau
