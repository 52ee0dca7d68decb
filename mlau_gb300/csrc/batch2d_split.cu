// Batched 2D engine, FP32-split arithmetic: FP64 state, primitive recovery
// and CT curl; reconstruction on centre-relative perturbations (primitives as
// (hi, lo) float pairs), Riemann solver with split jumps and edge EMFs in
// FP32.  The per-instance numerics are the 2D driver's
// (2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-660) in the arithmetic of the 3D
// FP32-split step (split3d.cu).
#include "batch2d.cuh"
#include "split_conv.cuh"
#include "point_x2.cuh"

namespace mlau {
namespace {
__device__ __forceinline__ float pf(float2 v) { return v.x + v.y; }
__device__ __forceinline__ float pd(float2 u, float2 v) { return (u.x - v.x) + (u.y - v.y); }

// --- phases -------------------------------------------------------------------
__device__ void ph_cfl(const BArgs &A, int nt, const BTile *tiles)
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
                const double bxc = 0.5 * (S[5][s] + S[5][s + 1]);
                const double byc = 0.5 * (S[6][s] + S[6][s + I.nx]);
                const double bzc = S[7][s];
                const double b2 = bxc * bxc + byc * byc + bzc * bzc;
                const float ro = (float)S[0][s], iro = 1.f / ro;
                const float vx = (float)S[1][s] * iro, vy = (float)S[2][s] * iro,
                            vz = (float)S[3][s] * iro;
                const float v2 = vx * vx + vy * vy + vz * vz;
                const float pr = (float)((I.gamma - 1.0) * (S[4][s] - 0.5 * ((double)(ro * v2) + b2)));
                const float cf = sqrtf((0.5f * (float)I.gamma * (2.f * pr) + (float)b2) * iro);
                const float v = sqrtf(vx * vx + vy * vy) + cf;
                vt = (v == v && I.dt_fixed <= 0.0) ? (double)v : 0.0;
                batch_check(I, ro, pr);
            }
        }
        batch_vmax(I, vt);
    }
}

__device__ void ph_prep(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        long long wx, wy;
        double gx = 1.0, gy = 1.0;
        if (I.walls) {  // each component at its own boundary source, with its sign
            wx = bsrc(I, i, j, 0, 0, I.bcx[5], I.bcy[5], &gx);
            wy = bsrc(I, i, j, 0, 0, I.bcx[6], I.bcy[6], &gy);
        } else {
            wx = wy = I.base + (long long)I.nx * bwrap(j, I.ny, I.off) + bwrap(i, I.nx, I.off);
        }
        const double *bx = a.s[5], *by = a.s[6];
        const double cx = gx * face2cen(A.odr, bx[wx - 1], bx[wx], bx[wx + 1], bx[wx + 2]);
        const double cy =
            gy * face2cen(A.odr, by[wy - I.nx], by[wy], by[wy + I.nx], by[wy + 2 * I.nx]);
        const double bz = a.s[7][c];
        const double ro = a.s[0][c];
        const float2 ro2 = split2(ro);
        const float rof = ro2.x + ro2.y, irof = 1.f / rof;
        const float vx = to_f32(a.s[1][c]) * irof, vy = to_f32(a.s[2][c]) * irof,
                    vz = to_f32(a.s[3][c]) * irof;
        const float v2 = vx * vx + vy * vy + vz * vz;
        const double b2 = cx * cx + cy * cy + bz * bz;
        const double pr = (I.gamma - 1.0) * (a.s[4][c] - 0.5 * (to_f64(rof * v2) + b2));
        const float2 pr2 = split2(pr);
        a.q[0][c] = ro2;
        a.q[1][c] = make_float2(vx, 0.f);
        a.q[2][c] = make_float2(vy, 0.f);
        a.q[3][c] = make_float2(vz, 0.f);
        a.q[4][c] = split2(cx);
        a.q[5][c] = split2(cy);
        a.q[6][c] = split2(bz);
        a.q[7][c] = pr2;
        a.bf[0][c] = to_f32(bx[c]);
        a.bf[1][c] = to_f32(by[c]);
        a.m2f[c] = v2 / (to_f32(I.gamma) * (pr2.x + pr2.y) * irof);
        if (rk == 0)
            for (int v = 0; v < 8; v++) a.u0[v][c] = a.s[v][c];
    });
}

__device__ void ph_aux(const BArgs &A, int nt, const BTile *tl)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const long long nx = I.nx;
        float ctw = 0.5f;
        if (i >= 1 && j >= 1) {
            const float eps = 1e-6f;
            const long long P = nx, Q = 1;
            float va = 0.25f * (pf(a.q[1][c - P - Q]) + pf(a.q[1][c - P]) + pf(a.q[1][c - Q]) + pf(a.q[1][c]));
            float vb = 0.25f * (pf(a.q[2][c - P - Q]) + pf(a.q[2][c - P]) + pf(a.q[2][c - Q]) + pf(a.q[2][c]));
            float rc = 0.25f * (pf(a.q[0][c - P - Q]) + pf(a.q[0][c - P]) + pf(a.q[0][c - Q]) + pf(a.q[0][c]));
            rc = rsqrtf(rc);
            const float ba = 0.5f * (a.bf[0][c - nx] + a.bf[0][c]);
            const float bb = 0.5f * (a.bf[1][c - 1] + a.bf[1][c]);
            va = fabsf(va) + fabsf(ba * rc);
            vb = fabsf(vb) + fabsf(bb * rc);
            ctw = (va + 0.5f * eps) / (va + vb + eps);
        }
        a.ctf[c] = ctw;
        if (I.walls) {  // signs of the sensors' fill (mhd_fd_ct_2d.c:262-271)
            double g0 = 1.0, g1 = 1.0;
            const long long w0 = bsrc(I, i, j, 0, 0, -I.bcx[1], I.bcy[1], &g0);
            const long long w1 = bsrc(I, i, j, 0, 0, I.bcx[2], -I.bcy[2], &g1);
            a.dvf[0][c] =
                (float)g0 * fminf(pd(a.q[1][w0 + 1], a.q[1][w0]), pd(a.q[1][w0], a.q[1][w0 - 1]));
            a.dvf[1][c] = (float)g1 *
                          fminf(pd(a.q[2][w1 + nx], a.q[2][w1]), pd(a.q[2][w1], a.q[2][w1 - nx]));
            return;
        }
        const long long w = I.base + nx * bwrap(j, I.ny, I.off) + bwrap(i, I.nx, I.off);
        a.dvf[0][c] = fminf(pd(a.q[1][w + 1], a.q[1][w]), pd(a.q[1][w], a.q[1][w - 1]));
        a.dvf[1][c] = fminf(pd(a.q[2][w + nx], a.q[2][w]), pd(a.q[2][w], a.q[2][w - nx]));
    });
}

// Reconstruction along D (0: x, 1: y) of cells [2, len-2).
__device__ void ph_rec(const BArgs &A, int nt, const BTile *tl, int D)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const int len = D == 0 ? I.nx : I.ny, pos = D == 0 ? i : j;
        if (pos < 2 || pos >= len - 2) return;
        const long long st = D == 0 ? 1 : I.nx;
        // rotated variables: X (ro, vx, vy, vz, cy, bz, pr) / n=cx; Y (ro, vy, vz, vx, bz, cx, pr) / n=cy
        const float2 *src[7];
        src[0] = a.q[0];
        src[6] = a.q[7];
        if (D == 0) { src[1] = a.q[1]; src[2] = a.q[2]; src[3] = a.q[3]; src[4] = a.q[5]; src[5] = a.q[6]; }
        else { src[1] = a.q[2]; src[2] = a.q[3]; src[3] = a.q[1]; src[4] = a.q[6]; src[5] = a.q[4]; }
        const float2 *cn = D == 0 ? a.q[4] : a.q[5];
        const int kb = D == 0 ? 4 : 5, kv = D == 0 ? 2 : 3;
        const float *bface = a.bf[D];
        const float mm = fmaxf(a.m2f[c - st], fmaxf(a.m2f[c], a.m2f[c + st]));
        if (A.odr == 4 && mm < 1.f) {
            // WCNS4 below Mach 1: packed FP32x2 form on the outer / inner
            // point pairs of the perturbations (the centre one is zero)
            float2 O[7], In[7];
            float qc[7];
            unsigned zero = 0;
#pragma unroll
            for (int n = 0; n < 7; n++) {
                float2 h[5];
#pragma unroll
                for (int m = 0; m < 5; m++) h[m] = src[n][c + st * (m - 2)];
                qc[n] = pf(h[2]);
                const float2 t0 = x2sub(h[0], h[2]), t1 = x2sub(h[1], h[2]);
                const float2 t3 = x2sub(h[3], h[2]), t4 = x2sub(h[4], h[2]);
                O[n] = make_float2(t0.x + t0.y, t4.x + t4.y);
                In[n] = make_float2(t1.x + t1.y, t3.x + t3.y);
                bool z = true;
#pragma unroll
                for (int m = 0; m < 5; m++) z = z && h[m].x == 0.f && h[m].y == 0.f;
                if (z) zero |= 1u << n;
            }
            float2 LR[7];
            reconst_alfven_wcns4_x2(O, In, qc, pf(cn[c]), (float)I.gamma, LR);
#pragma unroll
            for (int n = 1; n <= 5; n++)
                if (zero & (1u << n)) LR[n] = make_float2(0.f, 0.f);
#pragma unroll
            for (int n = 0; n < 7; n++) {
                a.ulf[n][c + st] = LR[n].x;
                a.urf[n][c] = LR[n].y;
            }
            const float a0 = qc[kb] * qc[1];
            const float2 dao = x2fma(O[kb], x2add(x2k(qc[1]), O[1]), x2mul(x2k(qc[kb]), O[1]));
            const float2 dai = x2fma(In[kb], x2add(x2k(qc[1]), In[1]), x2mul(x2k(qc[kb]), In[1]));
            const float2 Av = lin4_pert_x2(dao, dai), V = lin4_pert_x2(O[kv], In[kv]);
            a.ulf[7][c + st] = (a0 + Av.x) - bface[c + st] * (qc[kv] + V.x);
            a.urf[7][c] = (a0 + Av.y) - bface[c] * (qc[kv] + V.y);
            return;
        }
        float dq[7][5], qc[7];
        unsigned zero = 0;
#pragma unroll
        for (int n = 0; n < 7; n++) {
            float2 h[5];
#pragma unroll
            for (int m = 0; m < 5; m++) h[m] = src[n][c + st * (m - 2)];
            qc[n] = pf(h[2]);
            bool z = true;
#pragma unroll
            for (int m = 0; m < 5; m++) {
                dq[n][m] = pd(h[m], h[2]);
                z = z && h[m].x == 0.f && h[m].y == 0.f;
            }
            if (z) zero |= 1u << n;
        }
        float ul[7], ur[7];
        if (mm >= 1.f) reconst_full_core(A.odr, dq, qc, pf(cn[c]), (float)I.gamma, ul, ur);
        else reconst_alfven_core(A.odr, dq, qc, pf(cn[c]), (float)I.gamma, ul, ur);
#pragma unroll
        for (int n = 1; n <= 5; n++)
            if (zero & (1u << n)) { ul[n] = 0.f; ur[n] = 0.f; }
#pragma unroll
        for (int n = 0; n < 7; n++) {
            a.ulf[n][c + st] = ul[n];
            a.urf[n][c] = ur[n];
        }
        // CT central part of the split tangential B flux:
        // X: By flux from (cy vx, vy); Y: Bx flux from (cx vy, vx)
        const float a0 = qc[kb] * qc[1];
        float da[5];
#pragma unroll
        for (int m = 0; m < 5; m++) da[m] = (qc[kb] + dq[kb][m]) * (qc[1] + dq[1][m]) - a0;
        const float al = a0 + lin_l(A.odr, da[0], da[1], da[2], da[3], da[4]);
        const float ar = a0 + lin_r(A.odr, da[0], da[1], da[2], da[3], da[4]);
        const float vl = qc[kv] + lin_l(A.odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
        const float vr = qc[kv] + lin_r(A.odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
        a.ulf[7][c + st] = al - bface[c + st] * vl;
        a.urf[7][c] = ar - bface[c] * vr;
    });
}

__device__ void ph_flux(const BArgs &A, int nt, const BTile *tl, int D)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        const int len = D == 0 ? I.nx : I.ny, pos = D == 0 ? i : j;
        if (pos < 3 || pos >= len - 2) return;
        const long long st = D == 0 ? 1 : I.nx;
        const float2 *src[7];
        src[0] = a.q[0];
        src[6] = a.q[7];
        if (D == 0) { src[1] = a.q[1]; src[2] = a.q[2]; src[3] = a.q[3]; src[4] = a.q[5]; src[5] = a.q[6]; }
        else { src[1] = a.q[2]; src[2] = a.q[3]; src[3] = a.q[1]; src[4] = a.q[6]; src[5] = a.q[4]; }
        float L[7], R[7], jmp[7];
#pragma unroll
        for (int n = 0; n < 7; n++) {
            const float2 bl = src[n][c - st], br = src[n][c];
            const float dl = a.ulf[n][c], dr = a.urf[n][c];
            L[n] = pf(bl) + dl;
            R[n] = pf(br) + dr;
            jmp[n] = pd(br, bl) + (dr - dl);
        }
        const float jp = jmp[6] + 0.5f * (jmp[4] * (R[4] + L[4]) + jmp[5] * (R[5] + L[5]));
        const float bn = a.bf[D][c];
        const float *dvt = a.dvf[D == 0 ? 1 : 0];
        float F[7];
        const float dv0 = pd(src[1][c], src[1][c - st]), dv1 = fminf(dvt[c - st], dvt[c]);
        if (I.flux == FLUX_MLAU) {
            float2 P[7];
#pragma unroll
            for (int n = 0; n < 7; n++) P[n] = make_float2(L[n], R[n]);
            flux_mlau_x2(P, bn, (float)I.gamma, dv0, dv1, F, jp, jmp[1]);
        } else {
            riemann_jumps(I.flux, L, R, bn, (float)I.gamma, dv0, dv1, F, jp, jmp[1]);
        }
        const float fc = 0.5f * (a.ulf[7][c] + a.urf[7][c]);
        F[4 + D] -= fc;
#pragma unroll
        for (int n = 0; n < 7; n++) a.Ff[D][n][c] = F[n];
        a.FCf[D][c] = fc;
    });
}

__device__ __forceinline__ float emf_p(const float *fu, const float *fc, float w, float h,
                                       long long c, long long st, int odr)
{
    const float ul0 = lin_l(odr, fu[c - 3 * st], fu[c - 2 * st], fu[c - st], fu[c], fu[c + st]);
    const float ul1 = lin_l(odr, fc[c - 3 * st], fc[c - 2 * st], fc[c - st], fc[c], fc[c + st]);
    const float ur0 = lin_r(odr, fu[c - 2 * st], fu[c - st], fu[c], fu[c + st], fu[c + 2 * st]);
    const float ur1 = lin_r(odr, fc[c - 2 * st], fc[c - st], fc[c], fc[c + st], fc[c + 2 * st]);
    return h * ((ul0 + ur0) + w * (ul1 + ur1));
}

__device__ void ph_emf(const BArgs &A, int nt, const BTile *tl)
{
    const BArrays &a = A.a;
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        float ez = 0.f;
        if (i >= 3 && i < I.nx - 2 && j >= 3 && j < I.ny - 2) {
            const float w = a.ctf[c];
            ez = emf_p(a.Ff[0][4], a.FCf[0], 1.f - w, -0.5f, c, I.nx, A.odr)
                 + emf_p(a.Ff[1][5], a.FCf[1], w, 0.5f, c, 1, A.odr);
        }
        a.ezf[c] = ez;
    });
}

__device__ void ph_update(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    const double rkf[3][2] = {{0.0, 1.0}, {0.75, 0.25}, {1. / 3., 2. / 3.}};
    const double ra = rkf[rk][0], rb = rkf[rk][1];
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        if (i < I.off || i >= I.nx - I.off || j < I.off || j >= I.ny - I.off) return;
        const long long nx = I.nx;
        const float dtdx = (float)(I.dt / I.dx), dtdy = (float)(I.dt / I.dy);
        const int sv[6] = {0, 1, 2, 3, 7, 4};
        const int cX[6] = {0, 1, 2, 3, 5, 6}, cY[6] = {0, 3, 1, 2, 4, 6};
        double out[8];
#pragma unroll
        for (int v = 0; v < 6; v++) {
            const float *fx = a.Ff[0][cX[v]], *fy = a.Ff[1][cY[v]];
            const float div = dtdx * fdiff(A.odr, fx[c - 1], fx[c], fx[c + 1], fx[c + 2])
                              + dtdy * fdiff(A.odr, fy[c - nx], fy[c], fy[c + nx], fy[c + 2 * nx]);
            out[sv[v]] = ra * a.u0[sv[v]][c] + rb * (a.s[sv[v]][c] - to_f64(div));
        }
        // CT curl in FP64 on the FP32 EMFs: the differences are exact; the
        // stencil's 1/24 rides on dt/dx
        const float *ez = a.ezf;
        const bool o4 = lin_odr(A.odr) > 2;
        const double c24 = o4 ? 1.0 / 24.0 : 1.0;
        const double ddx = I.dt / I.dx * c24, ddy = I.dt / I.dy * c24;
        auto d64 = [&](long long st) {
            const double f0 = to_f64(ez[c - st]), f1 = to_f64(ez[c]), f2 = to_f64(ez[c + st]),
                         f3 = to_f64(ez[c + 2 * st]);
            return o4 ? 27.0 * (f2 - f1) - (f3 - f0) : f2 - f1;
        };
        const double dy_ez = d64(nx), dx_ez = d64(1);
        out[5] = ra * a.u0[5][c] + rb * (a.s[5][c] - ddy * dy_ez);
        out[6] = ra * a.u0[6][c] + rb * (a.s[6][c] + ddx * dx_ez);
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
                const long long t = I.base + nx * js[bb] + is[aa];
#pragma unroll
                for (int v = 0; v < 8; v++) a.s[v][t] = out[v];
            }
        }
    });
}

// Instances with tables: the right boundary faces the 2D driver's CT loops
// also update (Bx at i = nx-off, By at j = ny-off, mhd_fd_ct_2d.c:593-632)
// where that axis mirrors the face array, with the FP64 curl of ph_update ...
__device__ void ph_face(const BArgs &A, int nt, const BTile *tl, int rk)
{
    const BArrays &a = A.a;
    const double rkf[3][2] = {{0.0, 1.0}, {0.75, 0.25}, {1. / 3., 2. / 3.}};
    const double ra = rkf[rk][0], rb = rkf[rk][1];
    for_cells(A, nt, tl, [&](const BInst &I, int i, int j, long long c) {
        if (!I.walls) return;
        const float *ez = a.ezf;
        const bool o4 = lin_odr(A.odr) > 2;
        const double c24 = o4 ? 1.0 / 24.0 : 1.0;
        auto d64 = [&](long long st) {
            const double f0 = to_f64(ez[c - st]), f1 = to_f64(ez[c]), f2 = to_f64(ez[c + st]),
                         f3 = to_f64(ez[c + 2 * st]);
            return o4 ? 27.0 * (f2 - f1) - (f3 - f0) : f2 - f1;
        };
        if (I.bcx[5] != 0 && i == I.nx - I.off && j >= I.off && j < I.ny - I.off)
            a.s[5][c] = ra * a.u0[5][c] + rb * (a.s[5][c] - I.dt / I.dy * c24 * d64(I.nx));
        if (I.bcy[6] != 0 && j == I.ny - I.off && i >= I.off && i < I.nx - I.off)
            a.s[6][c] = ra * a.u0[6][c] + rb * (a.s[6][c] + I.dt / I.dx * c24 * d64(1));
    });
}

// ... then every ghost takes its boundary source times the signs (:636-638).
__device__ void ph_bc(const BArgs &A, int nt, const BTile *tl)
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

// One full RK3 step of every active instance.
__global__ void __launch_bounds__(256, 3) kb_step_split(BArgs A)
{
    const int nt = A.sync->ntiles;
    const BTile *tl = A.sync->tiles;
    ph_cfl(A, nt, tl);
    if (grid_barrier(A.sync, A.nblocks)) return;
    batch_dt(A);
    if (grid_barrier(A.sync, A.nblocks)) return;
    for (int rk = 0; rk < 3; rk++) {
        ph_prep(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        ph_aux(A, nt, tl);
        if (grid_barrier(A.sync, A.nblocks)) return;
        for (int D = 0; D < 2; D++) {
            ph_rec(A, nt, tl, D);
            if (grid_barrier(A.sync, A.nblocks)) return;
            ph_flux(A, nt, tl, D);
            if (grid_barrier(A.sync, A.nblocks)) return;
        }
        ph_emf(A, nt, tl);
        if (grid_barrier(A.sync, A.nblocks)) return;
        ph_update(A, nt, tl, rk);
        if (grid_barrier(A.sync, A.nblocks)) return;
        if (A.sync->walls) {
            ph_face(A, nt, tl, rk);
            if (grid_barrier(A.sync, A.nblocks)) return;
            ph_bc(A, nt, tl);
            if (grid_barrier(A.sync, A.nblocks)) return;
        }
    }
    batch_advance(A);
}

}  // namespace

const void *batch2d_split_kernel() { return (const void *)kb_step_split; }

}  // namespace mlau
