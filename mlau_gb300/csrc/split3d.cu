// FP32-split 3D step.  Same scheme and data layout as the plain FP64 step
// (3D/MPI/OTvortex/mhd_fd_ct_3d.c), with the arithmetic split by what needs
// more than FP32:
//
//   FP64  the CT curl update of face B (div B at FP64 round-off); the state
//         is stored in FP64.
//   float-float (~48 bits, FP32 pipe)
//         the RK3 accumulation of flux differences into the cell-centred
//         state and primitive recovery p = (gamma-1)(E - rho v^2/2 - B^2/2)
//         with cell B (cancellation at low Mach and low beta); FP64 in the
//         MLAU_FP32_SPLIT_F64 form.
//   FP32  characteristic reconstruction and the Riemann solver, the edge EMFs,
//         the CT weights and shock sensors.
//
// On this part FP64 issues at 1/64 of the FP32 rate, so the 48-bit parts run
// as float-float arithmetic (ff.cuh) rather than FP64: 10-20 FP32 operations
// per FP64 one still leave the prep and update kernels near the memory roof.
// Measured over 200 steps at 256^3 the float-float and FP64 forms of these
// two parts give the same L1 error against the plain FP64 step.
//
// Reconstruction works on perturbations from the cell centre, q_m - q_c, and
// WCNS/MUSCL/linear weights are translation invariant, so the face states
// keep FP32 relative accuracy in the perturbation, not in the absolute value.
// The Riemann solver receives its total-pressure and normal-velocity jumps
// formed the same way (centre difference + perturbation difference).
//
// The primitives leave the prep kernel as (hi, lo) float pairs with
// q = hi + lo to ~48 bits, so every later difference q_m - q_c is formed in
// FP32 as (hi_m - hi_c) + (lo_m - lo_c) without losing the perturbation.
// Flux differences are formed in FP32 (neighbouring fluxes of one sign
// subtract exactly) and added to the state in float-float.
//
// Kernels per RK stage: prep (float-float primitive recovery -> float pairs),
// aux (FP32 CT weights and shock sensors), one fused reconstruction + flux
// kernel per direction, emf (FP32), update (float-float RK combine, FP64 CT
// curl, periodic ghost images).
//
// The fused sweep is a persistent kernel over tiles.  Each tile's inputs (the
// 5-point stencils of eight float-pair arrays and four float arrays, halo
// included) are staged in shared memory by the tensor memory accelerator
// (cp.async.bulk.tensor), double-buffered: while a block computes one tile,
// the copy of its next tile is in flight.  Then each thread reconstructs one
// cell into shared memory and, after a block barrier, each face thread solves
// one Riemann problem.
//
// Every FP32 scratch array uses a row pitch px = nx rounded up to a multiple
// of 4 elements, so that its rows start on 16-byte boundaries as the tensor
// maps require; the FP64 state keeps the reference layout.
#include "sim.cuh"
#include "point.cuh"
#include "tma.cuh"
#include "split_conv.cuh"
#include "ff.cuh"
#include "point_x2.cuh"
#include "slab_plan.h"

#include <algorithm>
#include <memory>
#include <vector>

namespace mlau {

int plain3d_fill_ghosts(Sim *s);  // plain3d.cu: ghost fill of the FP64 state with the tables

// Arrays staged for a sweep, in the sweep's rotated order: density, normal /
// tangential / third velocity, the two tangential cell B components,
// pressure, the normal cell B (float pairs); then Mach^2, the face B normal
// to the sweep, and the two tangential shock sensors (floats).
enum { SQ_RO, SQ_VN, SQ_VT, SQ_VU, SQ_BT, SQ_BU, SQ_PR, SQ_BN, NQ };
enum { SF_M2, SF_BF, SF_DVT, SF_DVU, NF };

struct SweepMaps {
    CUtensorMap q[NQ];
    CUtensorMap f[NF];
};

struct SplitPtrs {
    float2 *q[8];    // ro, vx, vy, vz, cx, cy, cz, pr as (hi, lo) pairs
    float *bf[3];    // face-centred bx, by, bz rounded to FP32
    float *F[3][7];
    float *FC[3][2];
    float *e[3];     // edge EMFs
    float *m2;
    float *ct[3];
    float *dv[3];
};

struct SplitFields {
    SplitPtrs p{};
    long long px = 0;       // row pitch of the FP32 scratch (elements)
    SweepMaps maps[3];      // per sweep direction
    int ntile[3][2] = {};   // tiles along the first two tile axes, per sweep
    int ntiles[3] = {};
    int nblocks[3] = {};    // persistent grid per sweep
    int spec = 0;           // sweep instance: 0 run-time scheme, 1 WCNS4 + MLAU, 2 WCNS4 + LHLLD
    int f64 = 0;            // state arithmetic in FP64 (MLAU_FP32_SPLIT_F64), else float-float
    int *d_err = nullptr;   // set when a bounded wait gave up
    // host-array steps (split3d_step_host): upload / download streams, the
    // plane schedule and its copy events
    cudaStream_t cs = nullptr, cd = nullptr;
    cudaEvent_t ev_start = nullptr;
    std::unique_ptr<SlabPlan> plan;
    int plan_nrk = 0;
    std::vector<cudaEvent_t> ev_up, ev_dn;
};

namespace {

struct Dims {
    int nx, ny, nz, ox, oy, oz;
    long long px;  // row pitch of the FP32 scratch
    // FP64 state (reference layout)
    __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)nx * ((long long)ny * k + j) + i;
    }
    // FP32 scratch (pitched rows)
    __device__ __forceinline__ long long ap(int i, int j, int k) const
    {
        return px * ((long long)ny * k + j) + i;
    }
};

// Cell of this thread for the plane kernels: one thread per cell of an x-y
// plane (flattened, so no block runs mostly past the row end), one grid row
// of blocks per z-plane, from plane k0.
__device__ __forceinline__ bool plane_cell(const Dims &d, int &i, int &j, int &k, int k0 = 0)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= d.nx * d.ny) return false;
    j = t / d.nx;
    i = t - j * d.nx;
    k = k0 + blockIdx.y;
    return true;
}

// A host double as a float-float pair (hi rounded, lo the rounded rest).
inline float2 host_ff(double x)
{
    const float h = (float)x;
    return make_float2(h, (float)(x - (double)h));
}

// --- primitives (float-float recovery, FP32-pair output) -----------------
// Face-to-centre B as the scheme's calc_bc, in float-float.
// b: the faces w - st, w, w + st, w + 2 st.
__device__ __forceinline__ ff face2cen_ff(int odr, const double b[4])
{
    const ff f1 = ff_from(b[1]), f2 = ff_from(b[2]);
    if (lin_odr(odr) <= 2) return ff_scale(ff_add(f1, f2), 0.5f);
    const ff f0 = ff_from(b[0]), f3 = ff_from(b[3]);
    return ff_scale(ff_sub(ff_mul_f(ff_add(f1, f2), 9.0f), ff_add(f0, f3)), 0.0625f);
}

// F64: pressure recovery and cell B in FP64 arithmetic (the split form with
// FP64 kept for the state arithmetic) instead of float-float; the primitives
// then leave as the (hi, lo) splits of their FP64 values, velocities included.
// WALLS: the boundary tables bc are not all periodic; each cell-B component
// then reads its face stencil at its own boundary source, with its sign
// (3D/MPI/OTvortex/mhd_fd_ct_3d.c:186-238, boundary.c:227-309).
template <bool F64, bool WALLS>
__global__ void __launch_bounds__(256)
ks_prim(PlainFields f, SplitPtrs g, Dims d, Bc3 bc, int odr, float2 gm1, double gm1d,
        float gamma_f, int save_u0, int k0)
{
    int i, j, k;
    if (!plane_cell(d, i, j, k, k0)) return;
    const long long sy = d.nx, sz = (long long)d.nx * d.ny;
    const long long s = d.at(i, j, k), sp = d.ap(i, j, k);
    // loads first, so that they are in flight together (the kernel waits on
    // memory otherwise); the face stencils are at the cell's boundary source
    long long w[3];
    double gb[3] = {1.0, 1.0, 1.0};
    if constexpr (WALLS) {
#pragma unroll
        for (int a = 0; a < 3; a++)
            w[a] = d.at(bc_src(i, d.nx, d.ox, 0, bc.x[5 + a], &gb[a]),
                        bc_src(j, d.ny, d.oy, 0, bc.y[5 + a], &gb[a]),
                        bc_src(k, d.nz, d.oz, 0, bc.z[5 + a], &gb[a]));
    } else {
        w[0] = d.at(wrap_idx(i, d.nx, d.ox), wrap_idx(j, d.ny, d.oy), wrap_idx(k, d.nz, d.oz));
        w[1] = w[0];
        w[2] = w[0];
    }
    double bs[3][4], u[8];
    const long long st[3] = {1, sy, sz};
#pragma unroll
    for (int a = 0; a < 3; a++)
#pragma unroll
        for (int m = 0; m < 4; m++) bs[a][m] = f.s[5 + a][w[a] + (m - 1) * st[a]];
#pragma unroll
    for (int v = 0; v < 8; v++) u[v] = f.s[v][s];
    if constexpr (F64) {
        // p = (gamma-1)(E - rho v^2/2 - B^2/2) and cell B in FP64
        const double ro = u[0], iro = 1.0 / ro;
        const double cx = gb[0] * face2cen(odr, bs[0][0], bs[0][1], bs[0][2], bs[0][3]);
        const double cy = gb[1] * face2cen(odr, bs[1][0], bs[1][1], bs[1][2], bs[1][3]);
        const double cz = gb[2] * face2cen(odr, bs[2][0], bs[2][1], bs[2][2], bs[2][3]);
        const double vx = u[1] * iro, vy = u[2] * iro, vz = u[3] * iro;
        const double pr = gm1d * (u[4] - 0.5 * (ro * (vx * vx + vy * vy + vz * vz)
                                                + (cx * cx + cy * cy + cz * cz)));
        const float2 ro2 = split2(ro), vx2 = split2(vx), vy2 = split2(vy), vz2 = split2(vz);
        const float2 pr2 = split2(pr);
        g.q[0][sp] = ro2;
        g.q[1][sp] = vx2;
        g.q[2][sp] = vy2;
        g.q[3][sp] = vz2;
        g.q[4][sp] = split2(cx);
        g.q[5][sp] = split2(cy);
        g.q[6][sp] = split2(cz);
        g.q[7][sp] = pr2;
        g.bf[0][sp] = to_f32(u[5]);
        g.bf[1][sp] = to_f32(u[6]);
        g.bf[2][sp] = to_f32(u[7]);
        if (save_u0)
#pragma unroll
            for (int v = 0; v < 8; v++) f.u0[v][s] = u[v];
        const float fx = vx2.x + vx2.y, fy = vy2.x + vy2.y, fz = vz2.x + vz2.y;
        g.m2[sp] = (fx * fx + fy * fy + fz * fz) / (gamma_f * (pr2.x + pr2.y) / (ro2.x + ro2.y));
        return;
    }
    // a mirror's sign (+-1) flips both parts exactly
    const ff cx = ff_scale(face2cen_ff(odr, bs[0]), (float)gb[0]);
    const ff cy = ff_scale(face2cen_ff(odr, bs[1]), (float)gb[1]);
    const ff cz = ff_scale(face2cen_ff(odr, bs[2]), (float)gb[2]);
    const double ro = u[0];
    // Velocities and the kinetic energy in FP32: rho v^2/2 enters the pressure
    // as an additive term, so its FP32 rounding (1e-7 of itself) stays below
    // the pressure's own FP32 resolution at any Mach number; the cancelling
    // terms E and B^2/2 are carried in float-float (48 bits).
    const float2 ro2 = split2(ro);
    const float rof = ro2.x + ro2.y, irof = 1.0f / rof;
    const float vx = to_f32(u[1]) * irof, vy = to_f32(u[2]) * irof, vz = to_f32(u[3]) * irof;
    const float v2 = vx * vx + vy * vy + vz * vz;
    const ff b2 = ff_add(ff_add(ff_sqr(cx), ff_sqr(cy)), ff_sqr(cz));
    const ff pr = ff_mul({gm1.x, gm1.y},
                         ff_sub(ff_from(u[4]), ff_scale(ff_add_f(b2, rof * v2), 0.5f)));
    const float2 pr2 = ff_pair(pr);
    g.q[0][sp] = ro2;
    g.q[1][sp] = make_float2(vx, 0.f);
    g.q[2][sp] = make_float2(vy, 0.f);
    g.q[3][sp] = make_float2(vz, 0.f);
    g.q[4][sp] = ff_pair(cx);
    g.q[5][sp] = ff_pair(cy);
    g.q[6][sp] = ff_pair(cz);
    g.q[7][sp] = pr2;
    g.bf[0][sp] = to_f32(u[5]);
    g.bf[1][sp] = to_f32(u[6]);
    g.bf[2][sp] = to_f32(u[7]);
    // the first stage keeps U^n for the later stages' RK combine (this
    // kernel has loaded every state value of the cell already)
    if (save_u0)
#pragma unroll
        for (int v = 0; v < 8; v++) f.u0[v][s] = u[v];
    g.m2[sp] = v2 / (gamma_f * (pr2.x + pr2.y) * irof);
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

// WALLS: each shock sensor is read at its own boundary source with its sign,
// as the reference fills them (mhd_fd_ct_3d.c:367-376: dvx takes -dnxs[1]
// along x, dvy -dnys[2] along y, dvz -dnzs[3] along z).
template <bool WALLS>
__global__ void __launch_bounds__(256) ks_aux(SplitPtrs g, Dims d, Bc3 bc, int k0)
{
    int i, j, k;
    if (!plane_cell(d, i, j, k, k0)) return;
    const long long sy = d.px, sz = d.px * d.ny;
    const long long s = d.ap(i, j, k);
    const float2 *ro = g.q[0], *vx = g.q[1], *vy = g.q[2], *vz = g.q[3];
    g.ct[0][s] = (i >= 1 && j >= 1) ? ct_w(vx, vy, ro, g.bf[0], g.bf[1], s, sy, 1, sy, 1) : 0.5f;
    g.ct[1][s] = (j >= 1 && k >= 1) ? ct_w(vy, vz, ro, g.bf[1], g.bf[2], s, sz, sy, sz, sy) : 0.5f;
    g.ct[2][s] = (k >= 1 && i >= 1) ? ct_w(vz, vx, ro, g.bf[2], g.bf[0], s, sz, 1, 1, sz) : 0.5f;
    if constexpr (WALLS) {
        double g0 = 1.0, g1 = 1.0, g2 = 1.0;
        const long long w0 = d.ap(bc_src(i, d.nx, d.ox, 0, -bc.x[1], &g0),
                                  bc_src(j, d.ny, d.oy, 0, bc.y[1], &g0),
                                  bc_src(k, d.nz, d.oz, 0, bc.z[1], &g0));
        const long long w1 = d.ap(bc_src(i, d.nx, d.ox, 0, bc.x[2], &g1),
                                  bc_src(j, d.ny, d.oy, 0, -bc.y[2], &g1),
                                  bc_src(k, d.nz, d.oz, 0, bc.z[2], &g1));
        const long long w2 = d.ap(bc_src(i, d.nx, d.ox, 0, bc.x[3], &g2),
                                  bc_src(j, d.ny, d.oy, 0, bc.y[3], &g2),
                                  bc_src(k, d.nz, d.oz, 0, -bc.z[3], &g2));
        g.dv[0][s] = (float)g0 * fminf(qd(vx, w0 + 1, w0), qd(vx, w0, w0 - 1));
        g.dv[1][s] = (float)g1 * fminf(qd(vy, w1 + sy, w1), qd(vy, w1, w1 - sy));
        g.dv[2][s] = (float)g2 * fminf(qd(vz, w2 + sz, w2), qd(vz, w2, w2 - sz));
    } else {
        const long long w =
            d.ap(wrap_idx(i, d.nx, d.ox), wrap_idx(j, d.ny, d.oy), wrap_idx(k, d.nz, d.oz));
        g.dv[0][s] = fminf(qd(vx, w + 1, w), qd(vx, w, w - 1));
        g.dv[1][s] = fminf(qd(vy, w + sy, w), qd(vy, w, w - sy));
        g.dv[2][s] = fminf(qd(vz, w + sz, w), qd(vz, w, w - sz));
    }
}

// --- fused reconstruction + Riemann flux along axis D ----------------------
// Tile geometry.  Threads: TA along x times TB along the second axis.  For D=0
// the sweep runs along x (TA = T cells per tile, TB rows of one z-plane); for
// D=1,2 along y or z (TB = T cells per tile, TA columns of x).  A tile of T
// cells yields T-1 faces; consecutive tiles along the sweep overlap by one
// cell.  The staged box (BX, BY, BZ elements, x fastest) covers the tile's
// stencils: 2 cells of halo on each side along the sweep; for D=0 its x
// origin is rounded down to a multiple of 4 elements (16-byte TMA rule), so
// the box is 40 wide and the tile starts at offset x0 - xs in it.
template <int D> struct SG;
template <> struct SG<0> {
    static constexpr int TA = 32, TB = 4, T = 32;
    static constexpr int BX = 40, BY = 4, BZ = 1;
};
template <> struct SG<1> {
    static constexpr int TA = 8, TB = 16, T = 16;
    static constexpr int BX = 8, BY = 20, BZ = 1;
};
template <> struct SG<2> {
    static constexpr int TA = 8, TB = 16, T = 16;
    static constexpr int BX = 8, BY = 1, BZ = 20;
};
template <int D> __host__ __device__ constexpr int box_elems() { return SG<D>::BX * SG<D>::BY * SG<D>::BZ; }
template <int D> __host__ __device__ constexpr unsigned stage_bytes()
{
    return (unsigned)(box_elems<D>() * (NQ * sizeof(float2) + NF * sizeof(float)));
}
template <int D> constexpr size_t sweep_dyn_smem() { return 2 * stage_bytes<D>() + 128; }

struct TileAt {
    int x, y, z;   // box origin (elements)
    int i0, j0, k0;  // cell of thread (0, 0)
    int off;       // D=0: x offset of the tile inside the box
};

// Tile t of a sweep: n0 tiles along the first tile axis, n1 along the second.
// A launch over part of the grid starts its z-planes (D = 0, 1) or its tile
// rows along z (D = 2) at base.
template <int D> __device__ __forceinline__ TileAt tile_at(int t, int n0, int n1, int base)
{
    constexpr int T = SG<D>::T;
    const int t0 = t % n0, r = t / n0, t1 = r % n1, t2 = r / n1;
    TileAt a;
    if (D == 0) {
        const int x0 = 2 + (T - 1) * t0;
        a.x = (x0 - 2) & ~3;
        a.y = SG<0>::TB * t1;
        a.z = base + t2;
        a.i0 = x0; a.j0 = a.y; a.k0 = a.z;
        a.off = x0 - a.x;
    } else if (D == 1) {
        const int y0 = 2 + (T - 1) * t1;
        a.x = SG<1>::TA * t0;
        a.y = y0 - 2;
        a.z = base + t2;
        a.i0 = a.x; a.j0 = y0; a.k0 = a.z;
        a.off = 0;
    } else {
        const int z0 = 2 + (T - 1) * (base + t1);
        a.x = SG<2>::TA * t0;
        a.y = t2;
        a.z = z0 - 2;
        a.i0 = a.x; a.j0 = t2; a.k0 = z0;
        a.off = 0;
    }
    return a;
}

// Box element of stencil point m (0..4, centre 2) of thread (ta, tb).
template <int D> __device__ __forceinline__ int bidx(const TileAt &a, int ta, int tb, int m)
{
    if (D == 0) return tb * SG<0>::BX + a.off + ta + (m - 2);
    return (tb + m) * SG<D>::TA + ta;
}

template <int D>
__device__ __forceinline__ void issue_tile(const SweepMaps &M, unsigned char *st, const TileAt &a,
                                           uint64_t *bar)
{
    constexpr int NB = box_elems<D>();
    mbar_expect_tx(bar, stage_bytes<D>());
#pragma unroll
    for (int n = 0; n < NQ; n++) tma_load_3d(st + n * NB * sizeof(float2), &M.q[n], a.x, a.y, a.z, bar);
#pragma unroll
    for (int n = 0; n < NF; n++)
        tma_load_3d(st + NQ * NB * sizeof(float2) + n * NB * sizeof(float), &M.f[n], a.x, a.y, a.z,
                    bar);
}

// Per-cell results of a sweep tile in shared memory: sl / sr - the face
// perturbations at the cell's right / left face plus the two central CT parts.
// (The cell-centre states the Riemann step needs are read from the staged
// tile itself: a face's two cells are its thread's stencil points 1 and 2.)
template <int D> struct CellSmem {
    float (&sl)[9][SG<D>::TB][SG<D>::TA];
    float (&sr)[9][SG<D>::TB][SG<D>::TA];
};

// Reconstruction of one cell, any scheme: characteristic projection of the
// stencil perturbations, the scheme's face interpolation, back-projection;
// the central parts lin(bt vn) - bn_face lin(vt) of the two tangential B
// fluxes.
template <int D>
__device__ __forceinline__ void rec_cell(const float2 *Q, const float *Fs, const TileAt &a, int ta,
                                         int tb, int odr, float gamma, const CellSmem<D> &c)
{
    constexpr int NB = box_elems<D>();
    auto QI = [&](int n, int m) { return Q[n * NB + bidx<D>(a, ta, tb, m)]; };
    auto FI = [&](int n, int m) { return Fs[n * NB + bidx<D>(a, ta, tb, m)]; };
    float dq[7][5], qc[7];
    unsigned zero = 0;
#pragma unroll
    for (int n = 0; n < 7; n++) {
        float2 h[5];
#pragma unroll
        for (int m = 0; m < 5; m++) h[m] = QI(n, m);
        qc[n] = h[2].x + h[2].y;
        bool z = true;
#pragma unroll
        for (int m = 0; m < 5; m++) {
            dq[n][m] = (h[m].x - h[2].x) + (h[m].y - h[2].y);
            z = z && (h[m].x == 0.f) && (h[m].y == 0.f);
        }
        if (z) zero |= 1u << n;
    }
    float ul[7], ur[7];
    const float2 bn2 = QI(SQ_BN, 2);
    const float bnc = bn2.x + bn2.y;
    const float mm = fmaxf(FI(SF_M2, 1), fmaxf(FI(SF_M2, 2), FI(SF_M2, 3)));
    if (mm >= 1.0f) reconst_full_core(odr, dq, qc, bnc, gamma, ul, ur);
    else reconst_alfven_core(odr, dq, qc, bnc, gamma, ul, ur);
#pragma unroll
    for (int n = 1; n <= 5; n++)
        if (zero & (1u << n)) { ul[n] = 0.f; ur[n] = 0.f; }
#pragma unroll
    for (int n = 0; n < 7; n++) { c.sl[n][tb][ta] = ul[n]; c.sr[n][tb][ta] = ur[n]; }
    const float bl = FI(SF_BF, 3), br = FI(SF_BF, 2);
#pragma unroll
    for (int tt = 0; tt < 2; tt++) {
        const int kb = 4 + tt, kv = 2 + tt;
        const float a0 = (qc[kb]) * (qc[1]);
        float da[5];
#pragma unroll
        for (int m = 0; m < 5; m++) da[m] = (qc[kb] + dq[kb][m]) * (qc[1] + dq[1][m]) - a0;
        const float al = a0 + lin_l(odr, da[0], da[1], da[2], da[3], da[4]);
        const float ar = a0 + lin_r(odr, da[0], da[1], da[2], da[3], da[4]);
        const float vl = qc[kv] + lin_l(odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
        const float vr = qc[kv] + lin_r(odr, dq[kv][0], dq[kv][1], dq[kv][2], dq[kv][3], dq[kv][4]);
        c.sl[7 + tt][tb][ta] = al - bl * vl;
        c.sr[7 + tt][tb][ta] = ar - br * vr;
    }
}

// The same for WCNS4, on packed FP32x2 pairs (point_x2.cuh): the stencil
// perturbations as outer (f0, f4) and inner (f1, f3) pairs - the centre one
// is zero - and the face values as (left, right) pairs.  The central CT parts
// take the product perturbation in expanded form, (qb + db)(qv + dv) - qb qv
// = db (qv + dv) + qb dv, which keeps it to FP32 relative accuracy.
template <int D>
__device__ __forceinline__ void rec_cell_wcns4(const float2 *Q, const float *Fs, const TileAt &a,
                                               int ta, int tb, int odr, float gamma,
                                               const CellSmem<D> &c)
{
    constexpr int NB = box_elems<D>();
    auto QI = [&](int n, int m) { return Q[n * NB + bidx<D>(a, ta, tb, m)]; };
    auto FI = [&](int n, int m) { return Fs[n * NB + bidx<D>(a, ta, tb, m)]; };
    float2 O[7], I[7];
    float qc[7];
    unsigned zero = 0;
#pragma unroll
    for (int n = 0; n < 7; n++) {
        float2 h[5];
#pragma unroll
        for (int m = 0; m < 5; m++) h[m] = QI(n, m);
        qc[n] = h[2].x + h[2].y;
        float dqm[5];
#pragma unroll
        for (int m = 0; m < 5; m++) {
            if (m == 2) continue;
            const float2 t = x2sub(h[m], h[2]);  // (hi_m - hi_c, lo_m - lo_c)
            dqm[m] = t.x + t.y;
        }
        O[n] = make_float2(dqm[0], dqm[4]);
        I[n] = make_float2(dqm[1], dqm[3]);
        bool z = true;
#pragma unroll
        for (int m = 0; m < 5; m++) z = z && (h[m].x == 0.f) && (h[m].y == 0.f);
        if (z) zero |= 1u << n;
    }
    const float2 bn2 = QI(SQ_BN, 2);
    const float bnc = bn2.x + bn2.y;
    const float mm = fmaxf(FI(SF_M2, 1), fmaxf(FI(SF_M2, 2), FI(SF_M2, 3)));
    float2 LR[7];
    if (mm >= 1.0f) {
        float dq[7][5], ul[7], ur[7];
#pragma unroll
        for (int n = 0; n < 7; n++) {
            dq[n][0] = O[n].x; dq[n][1] = I[n].x; dq[n][2] = 0.f; dq[n][3] = I[n].y; dq[n][4] = O[n].y;
        }
        reconst_full_core(odr, dq, qc, bnc, gamma, ul, ur);
#pragma unroll
        for (int n = 0; n < 7; n++) LR[n] = make_float2(ul[n], ur[n]);
    } else {
        reconst_alfven_wcns4_x2(O, I, qc, bnc, gamma, LR);
    }
#pragma unroll
    for (int n = 1; n <= 5; n++)
        if (zero & (1u << n)) LR[n] = make_float2(0.f, 0.f);
#pragma unroll
    for (int n = 0; n < 7; n++) { c.sl[n][tb][ta] = LR[n].x; c.sr[n][tb][ta] = LR[n].y; }
    const float bl = FI(SF_BF, 3), br = FI(SF_BF, 2);
#pragma unroll
    for (int tt = 0; tt < 2; tt++) {
        const int kb = 4 + tt, kv = 2 + tt;
        const float a0 = qc[kb] * qc[1];
        const float2 dao = x2fma(O[kb], x2add(x2k(qc[1]), O[1]), x2mul(x2k(qc[kb]), O[1]));
        const float2 dai = x2fma(I[kb], x2add(x2k(qc[1]), I[1]), x2mul(x2k(qc[kb]), I[1]));
        const float2 A = lin4_pert_x2(dao, dai), V = lin4_pert_x2(O[kv], I[kv]);
        c.sl[7 + tt][tb][ta] = (a0 + A.x) - bl * (qc[kv] + V.x);
        c.sr[7 + tt][tb][ta] = (a0 + A.y) - br * (qc[kv] + V.y);
    }
}

// ODR / WHICH > 0 / >= 0 fix the reconstruction code and the solver at
// compile time (the common schemes get their own instances: no run-time
// dispatch and some 18 fewer registers per thread); 0 / -1 read them from
// the arguments.
template <int D, int ODR = 0, int WHICH = -1>
__global__ void __launch_bounds__(SG<D>::TA *SG<D>::TB, ODR ? 5 : 1)
ks_sweep(const __grid_constant__ SweepMaps M, SplitPtrs g, Dims d, int odr_rt, int which_rt,
         float gamma, int n0, int n1, int ntiles, int base, int *err)
{
    const int odr = ODR ? ODR : odr_rt;
    const int which = WHICH >= 0 ? WHICH : which_rt;
    constexpr int TA = SG<D>::TA, TB = SG<D>::TB, NB = box_elems<D>();
    constexpr unsigned STAGE = stage_bytes<D>();
    extern __shared__ unsigned char dyn_smem[];
    unsigned char *stages =
        (unsigned char *)(((uintptr_t)dyn_smem + 127) & ~(uintptr_t)127);
    // per-cell results: sl/sr - perturbation at the cell's right / left face
    // + 2 central parts
    __shared__ float sl[9][TB][TA], sr[9][TB][TA];
    __shared__ uint64_t bar[2];
    const int ta = threadIdx.x, tb = threadIdx.y, tid = tb * TA + ta;
    const int p = (D == 0) ? ta : tb;  // position along the sweep inside the tile
    const int len = (D == 0) ? d.nx : (D == 1 ? d.ny : d.nz);

    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_async_shared();
    }
    __syncthreads();
    if (tid == 0 && (int)blockIdx.x < ntiles)
        issue_tile<D>(M, stages, tile_at<D>(blockIdx.x, n0, n1, base), &bar[0]);

    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, it++) {
        const int b = it & 1;
        const int tn = t + gridDim.x;
        if (tid == 0 && tn < ntiles) {
            // the other buffer was released by the barrier that ended the
            // previous iteration
            fence_async_shared();
            issue_tile<D>(M, stages + (b ^ 1) * STAGE, tile_at<D>(tn, n0, n1, base), &bar[b ^ 1]);
        }
        const bool ok = mbar_wait(&bar[b], (it >> 1) & 1);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(err, 1);
                if (tn < ntiles) mbar_wait(&bar[b ^ 1], ((it + 1) >> 1) & 1);
            }
            return;
        }
        const float2 *Q = (const float2 *)(stages + b * STAGE);
        const float *Fs = (const float *)(stages + b * STAGE + NQ * NB * sizeof(float2));
        const TileAt a = tile_at<D>(t, n0, n1, base);
        const int i = a.i0 + ta, j = a.j0 + ((D == 2) ? 0 : tb), k = a.k0 + ((D == 2) ? tb : 0);
        const int ac = (D == 0) ? i : (D == 1 ? j : k);  // sweep coordinate
        const bool in_box = i < d.nx && j < d.ny && k < d.nz;
        const bool do_rec = in_box && ac >= 2 && ac < len - 2;
        auto QI = [&](int n, int m) { return Q[n * NB + bidx<D>(a, ta, tb, m)]; };
        auto FI = [&](int n, int m) { return Fs[n * NB + bidx<D>(a, ta, tb, m)]; };

        if (do_rec) {
            const CellSmem<D> cs{sl, sr};
            if constexpr (ODR == 4) rec_cell_wcns4<D>(Q, Fs, a, ta, tb, odr, gamma, cs);
            else rec_cell<D>(Q, Fs, a, ta, tb, odr, gamma, cs);
        }
        __syncthreads();

        if (in_box && p >= 1 && ac >= 3 && ac < len - 2) {
            const int tbl = (D == 0) ? tb : tb - 1, tal = (D == 0) ? ta - 1 : ta;
            // the two cells' centre states: stencil points 1 (left) and 2 (right)
            float2 cl[7], cr[7];
            float L[7], Rr[7];
#pragma unroll
            for (int n = 0; n < 7; n++) {
                cl[n] = QI(n, 1);
                cr[n] = QI(n, 2);
                L[n] = (cl[n].x + cl[n].y) + sl[n][tbl][tal];
                Rr[n] = (cr[n].x + cr[n].y) + sr[n][tb][ta];
            }
            // jumps from split parts: centre difference from the pairs, plus
            // the difference of the FP32 perturbations
            auto jump = [&](int n) {
                return ((cr[n].x - cl[n].x) + (cr[n].y - cl[n].y)) + (sr[n][tb][ta] - sl[n][tbl][tal]);
            };
            const float jv = jump(1);
            const float jp = jump(6) + 0.5f * (jump(4) * (Rr[4] + L[4]) + jump(5) * (Rr[5] + L[5]));
            const float bn = FI(SF_BF, 2);
            const float dv0 = (cr[1].x - cl[1].x) + (cr[1].y - cl[1].y);
            const float dvtm = fminf(fminf(FI(SF_DVT, 1), FI(SF_DVT, 2)),
                                     fminf(FI(SF_DVU, 1), FI(SF_DVU, 2)));
            float F[7];
            if constexpr (ODR == 4 && WHICH == FLUX_MLAU) {
                float2 P[7];
#pragma unroll
                for (int n = 0; n < 7; n++) P[n] = make_float2(L[n], Rr[n]);
                flux_mlau_x2(P, bn, gamma, dv0, dvtm, F, jp, jv);
            } else {
                riemann_jumps(which, L, Rr, bn, gamma, dv0, dvtm, F, jp, jv);
            }
            const float fct = 0.5f * (sl[7][tbl][tal] + sr[7][tb][ta]);
            const float fcu = 0.5f * (sl[8][tbl][tal] + sr[8][tb][ta]);
            F[4] -= fct;
            F[5] -= fcu;
            const long long c = d.ap(i, j, k);
#pragma unroll
            for (int n = 0; n < 7; n++) g.F[D][n][c] = F[n];
            g.FC[D][0][c] = fct;
            g.FC[D][1][c] = fcu;
        }
        __syncthreads();  // the stage and the per-cell results are reused
    }
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

__global__ void __launch_bounds__(256) ks_emf(SplitPtrs g, Dims d, int odr, int k0)
{
    int i, j, k;
    if (!plane_cell(d, i, j, k, k0)) return;
    const long long sy = d.px, sz = d.px * d.ny;
    const long long c = d.ap(i, j, k);
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
// magnitude) and accumulated into the state in float-float.
//
// The kernel streams some 60 flux values, 24 edge EMFs and 16 state values
// per cell with little arithmetic between them, so it is bound by memory
// latency unless the loads are in flight together: every value is read into
// registers first (read-only data through the non-coherent path), and the
// arithmetic follows.

// The RK combine ra u0 + rb u in float-float (ra = 0, rb = 1 at the first stage).
struct RkFF {
    float2 ra, rb;
    int first;
};
__device__ __forceinline__ double rk_ff(const RkFF &c, double u0, ff u)
{
    if (c.first) return ff_to_double(u);
    return ff_to_double(ff_add(ff_mul({c.ra.x, c.ra.y}, ff_from(u0)), ff_mul({c.rb.x, c.rb.y}, u)));
}

// Stencil f[s - st], f[s], f[s + st], f[s + 2 st] of a read-only array.
__device__ __forceinline__ void ld4(float v[4], const float *f, long long s, long long st)
{
#pragma unroll
    for (int m = 0; m < 4; m++) v[m] = __ldg(f + s + (m - 1) * st);
}

// FP64 difference of the FP32 edge EMFs f0..f3 along one axis (the values
// converted exactly), without the 1/24 of the 4th-order stencil.
__device__ __forceinline__ double df_f64(int odr, const float e[4])
{
    const double e0 = to_f64(e[0]), e1 = to_f64(e[1]), e2 = to_f64(e[2]), e3 = to_f64(e[3]);
    if (lin_odr(odr) <= 2) return e2 - e1;
    return 27.0 * (e2 - e1) - (e3 - e0);
}

// F64: the RK combine of the cell-centred variables in FP64 arithmetic (the
// split form with FP64 kept for the state arithmetic), else in float-float;
// the flux divergence is formed in FP32 and the CT curl in FP64 in both.
// rd: (ra, rb) and (dt/dx, dt/dy, dt/dz) times the stencil's 1/24, as
// doubles.
struct RkF64 {
    double ra, rb, ddx, ddy, ddz;
};

template <bool F64>
__global__ void __launch_bounds__(128)
ks_update(PlainFields f, SplitPtrs g, Dims d, int odr, RkFF rk, RkF64 rd, float dtdx, float dtdy,
          float dtdz, int images, int k0)
{
    const int i = d.ox + blockIdx.x * blockDim.x + threadIdx.x;
    const int j = d.oy + blockIdx.y, k = k0 + blockIdx.z;
    if (i >= d.nx - d.ox) return;
    const long long sy = d.px, sz = d.px * d.ny;  // scratch strides
    const long long s = d.at(i, j, k), sp = d.ap(i, j, k);
    const int cX[5] = {0, 1, 2, 3, 6}, cY[5] = {0, 3, 1, 2, 6}, cZ[5] = {0, 2, 3, 1, 6};
    // loads
    float fx[5][4], fy[5][4], fz[5][4];
#pragma unroll
    for (int v = 0; v < 5; v++) {
        ld4(fx[v], g.F[0][cX[v]], sp, 1);
        ld4(fy[v], g.F[1][cY[v]], sp, sy);
        ld4(fz[v], g.F[2][cZ[v]], sp, sz);
    }
    float ezy[4], eyz[4], exz[4], ezx[4], eyx[4], exy[4];
    ld4(ezy, g.e[2], sp, sy);
    ld4(eyz, g.e[1], sp, sz);
    ld4(exz, g.e[0], sp, sz);
    ld4(ezx, g.e[2], sp, 1);
    ld4(eyx, g.e[1], sp, 1);
    ld4(exy, g.e[0], sp, sy);
    double u[8], u0[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
        u[v] = f.s[v][s];
        u0[v] = rk.first ? 0.0 : __ldg(f.u0[v] + s);
    }
    // arithmetic: the flux divergence of the cell-centred variables
    double out[8];
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const float div = dtdx * fdiff(odr, fx[v][0], fx[v][1], fx[v][2], fx[v][3])
                          + dtdy * fdiff(odr, fy[v][0], fy[v][1], fy[v][2], fy[v][3])
                          + dtdz * fdiff(odr, fz[v][0], fz[v][1], fz[v][2], fz[v][3]);
        if constexpr (F64) {
            const double w = u[v] - to_f64(div);
            out[v] = rk.first ? w : rd.ra * u0[v] + rd.rb * w;
        } else {
            // the first stage is u - div: one FP64 addition beats its float-float form
            out[v] = rk.first ? u[v] - to_f64(div)
                              : rk_ff(rk, u0[v], ff_add_f(ff_from(u[v]), -div));
        }
    }
    // CT curl of face B in FP64 in both forms: the EMF differences of the
    // converted FP32 values and their products with dt/dx are rounded to 53
    // bits, so the discrete divergence of the B increment cancels to FP64
    // round-off (float-float, 48 bits, let it grow some 30 times faster).
    const double b5 = u[5] - rd.ddy * df_f64(odr, ezy) + rd.ddz * df_f64(odr, eyz);
    const double b6 = u[6] - rd.ddz * df_f64(odr, exz) + rd.ddx * df_f64(odr, ezx);
    const double b7 = u[7] - rd.ddx * df_f64(odr, eyx) + rd.ddy * df_f64(odr, exy);
    out[5] = rk.first ? b5 : rd.ra * u0[5] + rd.rb * b5;
    out[6] = rk.first ? b6 : rd.ra * u0[6] + rd.rb * b6;
    out[7] = rk.first ? b7 : rd.ra * u0[7] + rd.rb * b7;
    if (!images) {  // non-periodic tables: the ghost fill follows
#pragma unroll
        for (int v = 0; v < 8; v++) f.s[v][s] = out[v];
        return;
    }
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

// The right boundary faces the reference's CT loops also update (Bx at
// i = nx-xoff, By at j = ny-yoff, Bz at k = nz-zoff; mhd_fd_ct_3d.c:1079-1157
// run one face further); with non-periodic tables they survive the ghost fill
// where that axis mirrors the face array.  Same FP64 curl as ks_update, one
// thread per face of the three planes.
__global__ void __launch_bounds__(128)
ks_face(PlainFields f, SplitPtrs g, Dims d, int odr, RkFF rk, RkF64 rd, int do_x, int do_y,
        int do_z)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long sy = d.px, sz = d.px * d.ny;  // scratch strides
    const int Nx = d.nx - 2 * d.ox, Ny = d.ny - 2 * d.oy, Nz = d.nz - 2 * d.oz;
    auto put = [&](int v, int i, int j, int k, double b) {
        const long long s = d.at(i, j, k);
        f.s[v][s] = rk.first ? b : rd.ra * f.u0[v][s] + rd.rb * b;
    };
    float e0[4], e1[4];
    if (do_x && t < (long long)Ny * Nz) {  // Bx at i = nx - xoff
        const int i = d.nx - d.ox, j = d.oy + (int)(t % Ny), k = d.oz + (int)(t / Ny);
        const long long sp = d.ap(i, j, k);
        ld4(e0, g.e[2], sp, sy);
        ld4(e1, g.e[1], sp, sz);
        put(5, i, j, k, f.s[5][d.at(i, j, k)] - rd.ddy * df_f64(odr, e0) + rd.ddz * df_f64(odr, e1));
    }
    if (do_y && t < (long long)Nx * Nz) {  // By at j = ny - yoff
        const int i = d.ox + (int)(t % Nx), j = d.ny - d.oy, k = d.oz + (int)(t / Nx);
        const long long sp = d.ap(i, j, k);
        ld4(e0, g.e[0], sp, sz);
        ld4(e1, g.e[2], sp, 1);
        put(6, i, j, k, f.s[6][d.at(i, j, k)] - rd.ddz * df_f64(odr, e0) + rd.ddx * df_f64(odr, e1));
    }
    if (do_z && t < (long long)Nx * Ny) {  // Bz at k = nz - zoff
        const int i = d.ox + (int)(t % Nx), j = d.oy + (int)(t / Nx), k = d.nz - d.oz;
        const long long sp = d.ap(i, j, k);
        ld4(e0, g.e[1], sp, 1);
        ld4(e1, g.e[0], sp, sy);
        put(7, i, j, k, f.s[7][d.at(i, j, k)] - rd.ddx * df_f64(odr, e0) + rd.ddy * df_f64(odr, e1));
    }
}

int falloc(Sim *s, float **p, long long n)
{
    double *q = nullptr;
    int rc = dalloc(s, &q, (n + 1) / 2);
    *p = (float *)q;
    return rc;
}

// Arrays staged by sweep D, in SQ_* / SF_* order.
void sweep_arrays(const SplitPtrs &g, int D, const void *q[NQ], const void *f[NF])
{
    static const int vq[3][NQ] = {{0, 1, 2, 3, 5, 6, 7, 4}, {0, 2, 3, 1, 6, 4, 7, 5},
                                  {0, 3, 1, 2, 4, 5, 7, 6}};
    static const int dvt[3] = {1, 2, 0}, dvu[3] = {2, 0, 1};
    for (int n = 0; n < NQ; n++) q[n] = g.q[vq[D][n]];
    f[SF_M2] = g.m2;
    f[SF_BF] = g.bf[D];
    f[SF_DVT] = g.dv[dvt[D]];
    f[SF_DVU] = g.dv[dvu[D]];
}

// Opt a sweep instance into its dynamic shared memory and return how many of
// its blocks fit on an SM.
template <class K> int sweep_occupancy(K kernel, int threads, size_t dyn, int *per_sm)
{
    MLAU_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    MLAU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, kernel, threads, dyn));
    return MLAU_OK;
}

template <int D> int setup_sweep(Sim *s, SplitFields &sf)
{
    const Geometry &G = s->g;
    constexpr int T = SG<D>::T;
    const void *q[NQ], *f[NF];
    sweep_arrays(sf.p, D, q, f);
    for (int n = 0; n < NQ; n++) {
        int rc = tma_map_3d(&sf.maps[D].q[n], q[n], sizeof(float2), G.nx, G.ny, G.nz, sf.px,
                            SG<D>::BX, SG<D>::BY, SG<D>::BZ);
        if (rc) return rc;
    }
    for (int n = 0; n < NF; n++) {
        int rc = tma_map_3d(&sf.maps[D].f[n], f[n], sizeof(float), G.nx, G.ny, G.nz, sf.px,
                            SG<D>::BX, SG<D>::BY, SG<D>::BZ);
        if (rc) return rc;
    }
    int n0, n1, n2;
    if (D == 0) {
        n0 = (int)blocks_for(G.nx - 5, T - 1);
        n1 = (int)blocks_for(G.ny, SG<0>::TB);
        n2 = G.nz;
    } else if (D == 1) {
        n0 = (int)blocks_for(G.nx, SG<1>::TA);
        n1 = (int)blocks_for(G.ny - 5, T - 1);
        n2 = G.nz;
    } else {
        n0 = (int)blocks_for(G.nx, SG<2>::TA);
        n1 = (int)blocks_for(G.nz - 5, T - 1);
        n2 = G.ny;
    }
    sf.ntile[D][0] = n0;
    sf.ntile[D][1] = n1;
    sf.ntiles[D] = n0 * n1 * n2;
    int per_sm = 0;
    const int ro = sf.spec == 1   ? sweep_occupancy(ks_sweep<D, 4, FLUX_MLAU>, SG<D>::TA * SG<D>::TB,
                                              sweep_dyn_smem<D>(), &per_sm)
             : sf.spec == 2 ? sweep_occupancy(ks_sweep<D, 4, FLUX_LHLLD>, SG<D>::TA * SG<D>::TB,
                                              sweep_dyn_smem<D>(), &per_sm)
                            : sweep_occupancy(ks_sweep<D>, SG<D>::TA * SG<D>::TB,
                                              sweep_dyn_smem<D>(), &per_sm);
    if (ro) return ro;
    int dev = 0, sms = 0;
    MLAU_CUDA(cudaGetDevice(&dev));
    MLAU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (per_sm < 1) {
        set_error("FP32-split sweep %d does not fit on an SM", D);
        return MLAU_ERR_CUDA;
    }
    sf.nblocks[D] = std::max(1, std::min(sf.ntiles[D], sms * per_sm));
    return MLAU_OK;
}

// Sweep D over the whole grid (count < 0), or over z-planes [base, base +
// count) (D = 0, 1) / tile rows along z [base, base + count) (D = 2).
template <int D>
void launch_sweep(Sim *s, SplitFields &sf, const Dims &d, float gam, int base = 0,
                  int count = -1)
{
    const dim3 b(SG<D>::TA, SG<D>::TB);
    const size_t dyn = sweep_dyn_smem<D>();
    const int n0 = sf.ntile[D][0];
    int n1 = sf.ntile[D][1], ntiles = sf.ntiles[D];
    if (count >= 0) {
        if (D == 2) {
            n1 = count;
            ntiles = n0 * count * d.ny;
        } else {
            ntiles = n0 * n1 * count;
        }
    }
    if (ntiles <= 0) return;
    const int nb = std::min(ntiles, sf.nblocks[D]);
    if (sf.spec == 1)
        ks_sweep<D, 4, FLUX_MLAU><<<nb, b, dyn, s->stream>>>(
            sf.maps[D], sf.p, d, s->odr, s->flux, gam, n0, n1, ntiles, base, sf.d_err);
    else if (sf.spec == 2)
        ks_sweep<D, 4, FLUX_LHLLD><<<nb, b, dyn, s->stream>>>(
            sf.maps[D], sf.p, d, s->odr, s->flux, gam, n0, n1, ntiles, base, sf.d_err);
    else
        ks_sweep<D><<<nb, b, dyn, s->stream>>>(sf.maps[D], sf.p, d, s->odr, s->flux, gam, n0,
                                               n1, ntiles, base, sf.d_err);
}

}  // namespace

int tma_map_3d(CUtensorMap *map, const void *base, int elem_bytes, int nx, int ny, int nz,
               long long px, int bx, int by, int bz)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        MLAU_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                   cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !fn) {
            set_error("cuTensorMapEncodeTiled is not available from the driver");
            return MLAU_ERR_CUDA;
        }
        encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    const long long row = px * elem_bytes;
    if (((uintptr_t)base & 15) || (row & 15) || ((long long)bx * elem_bytes) % 16) {
        set_error("tensor map: base, row pitch or box width not 16-byte aligned");
        return MLAU_ERR_ARG;
    }
    const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {(cuuint64_t)row, (cuuint64_t)(row * ny)};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType ty =
        elem_bytes == 8 ? CU_TENSOR_MAP_DATA_TYPE_INT64 : CU_TENSOR_MAP_DATA_TYPE_INT32;
    const CUresult r = encode(map, ty, 3, const_cast<void *>(base), dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return MLAU_ERR_CUDA;
    }
    return MLAU_OK;
}

int split3d_alloc(Sim *s)
{
    if (s->g.dim != 3) { set_error("FP32-split mode is 3D only"); return MLAU_ERR_ARG; }
    PlainFields &f = s->f;
    const Geometry &G = s->g;
    const long long n = G.n;
    int rc = 0;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, &f.s[v], n) | dalloc(s, &f.u0[v], n);
    s->sp = new SplitFields();
    SplitFields &sf = *s->sp;
    sf.px = (G.nx + 3) / 4 * 4;
    const long long np = sf.px * G.ny * G.nz;
    SplitPtrs &g = sf.p;
    for (int v = 0; v < 8; v++) rc |= dalloc(s, (double **)&g.q[v], np);
    for (int D = 0; D < 3; D++) rc |= falloc(s, &g.bf[D], np);
    for (int D = 0; D < 3; D++) {
        for (int v = 0; v < 7; v++) rc |= falloc(s, &g.F[D][v], np);
        rc |= falloc(s, &g.FC[D][0], np) | falloc(s, &g.FC[D][1], np);
        rc |= falloc(s, &g.e[D], np) | falloc(s, &g.ct[D], np) | falloc(s, &g.dv[D], np);
    }
    rc |= falloc(s, &g.m2, np);
    double *flag = nullptr;
    rc |= dalloc(s, &flag, 1);
    if (rc) return MLAU_ERR_NOMEM;
    sf.d_err = (int *)flag;
    MLAU_CUDA(cudaMemset(sf.d_err, 0, sizeof(int)));
    // the sweeps read the arrays' ghost rows too: start from zeros
    for (int v = 0; v < 8; v++) MLAU_CUDA(cudaMemset(g.q[v], 0, sizeof(float2) * np));
    sf.spec = (s->odr == 4 && s->flux == FLUX_MLAU) ? 1 : (s->odr == 4 && s->flux == FLUX_LHLLD) ? 2 : 0;
    sf.f64 = s->precision == MLAU_FP32_SPLIT_F64;
    int r2 = setup_sweep<0>(s, sf);
    if (!r2) r2 = setup_sweep<1>(s, sf);
    if (!r2) r2 = setup_sweep<2>(s, sf);
    return r2;
}

void split3d_free(Sim *s)
{
    SplitFields *sf = s->sp;
    if (sf) {
        if (sf->cs) cudaStreamSynchronize(sf->cs);
        if (sf->cd) cudaStreamSynchronize(sf->cd);
        for (cudaEvent_t e : sf->ev_up) cudaEventDestroy(e);
        for (cudaEvent_t e : sf->ev_dn) cudaEventDestroy(e);
        if (sf->ev_start) cudaEventDestroy(sf->ev_start);
        if (sf->cs) cudaStreamDestroy(sf->cs);
        if (sf->cd) cudaStreamDestroy(sf->cd);
    }
    delete sf;
    s->sp = nullptr;
}

// MLAU_ERR_TIMEOUT when a sweep gave up waiting for its staged tile (the
// stream must be idle).
int split3d_check(Sim *s)
{
    if (!s->sp || !s->sp->d_err) return MLAU_OK;
    int e = 0;
    MLAU_CUDA(cudaMemcpy(&e, s->sp->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        set_error("FP32-split sweep: a bounded wait for a staged tile gave up");
        return MLAU_ERR_TIMEOUT;
    }
    return MLAU_OK;
}

namespace {

struct StepCtx {
    Sim *s;
    const Dims d;
    const dim3 cb, cg, ug;
    explicit StepCtx(Sim *sim)
        : s(sim), d{sim->g.nx, sim->g.ny, sim->g.nz, sim->g.ox, sim->g.oy, sim->g.oz, sim->sp->px},
          cb(128), cg(blocks_for((long long)sim->g.nx * sim->g.ny, 128), sim->g.nz),
          ug(blocks_for(sim->g.nx - 2 * sim->g.ox, 128), sim->g.ny - 2 * sim->g.oy,
             sim->g.nz - 2 * sim->g.oz)
    {
    }
    // primitive recovery of planes [k0, k0 + nk)
    void prim(int rk, int k0, int nk) const
    {
        const bool w = s->walls3d;
        auto kern = s->sp->f64 ? (w ? ks_prim<true, true> : ks_prim<true, false>)
                               : (w ? ks_prim<false, true> : ks_prim<false, false>);
        kern<<<dim3(cg.x, nk), cb, 0, s->stream>>>(s->f, s->sp->p, d, s->bc3, s->odr,
                                                   host_ff(s->gamma - 1), s->gamma - 1,
                                                   (float)s->gamma, rk == 0, k0);
    }
    // CT weights and shock sensors of planes [k0, k0 + nk)
    void aux(int k0, int nk) const
    {
        auto kern = s->walls3d ? ks_aux<true> : ks_aux<false>;
        kern<<<dim3(cg.x, nk), cb, 0, s->stream>>>(s->sp->p, d, s->bc3, k0);
    }
    void sweeps() const
    {
        const float gam = (float)s->gamma;
        launch_sweep<0>(s, *s->sp, d, gam);
        launch_sweep<1>(s, *s->sp, d, gam);
        launch_sweep<2>(s, *s->sp, d, gam);
    }
    // sweep D over planes (D = 0, 1) or tile rows along z (D = 2) [a, b)
    void sweep(int D, int a, int b) const
    {
        const float gam = (float)s->gamma;
        if (D == 0) launch_sweep<0>(s, *s->sp, d, gam, a, b - a);
        else if (D == 1) launch_sweep<1>(s, *s->sp, d, gam, a, b - a);
        else launch_sweep<2>(s, *s->sp, d, gam, a, b - a);
    }
    void emf(int k0, int nk) const
    {
        ks_emf<<<dim3(cg.x, nk), cb, 0, s->stream>>>(s->sp->p, d, s->odr, k0);
    }
    // RK combine + CT curl of the interior planes [k0, k0 + nk)
    void update(int rk, double dt, int k0, int nk) const
    {
        const Geometry &G = s->g;
        const double t[3][2] = {{0.0, 1.0},
                                {0.5 + (s->nrk - 2) * 0.25, 0.5 - (s->nrk - 2) * 0.25},
                                {1. / 3., 2. / 3.}};
        const double ra = t[rk][0], rb = t[rk][1];
        const double c24 = lin_odr(s->odr) > 2 ? 1.0 / 24.0 : 1.0;
        const RkFF c{host_ff(ra), host_ff(rb), ra == 0.0 && rb == 1.0};
        const RkF64 c64{ra, rb, dt / G.dx * c24, dt / G.dy * c24, dt / G.dz * c24};
        auto kern = s->sp->f64 ? ks_update<true> : ks_update<false>;
        kern<<<dim3(ug.x, ug.y, nk), cb, 0, s->stream>>>(
            s->f, s->sp->p, d, s->odr, c, c64, (float)(dt / G.dx), (float)(dt / G.dy),
            (float)(dt / G.dz), !s->walls3d, k0);
        if (s->walls3d && k0 + nk == G.nz - G.oz) {
            // after the last interior plane: the right boundary faces, then
            // the ghost fill with the tables
            const long long n = std::max({(long long)G.ny * G.nz, (long long)G.nx * G.nz,
                                          (long long)G.nx * G.ny});
            ks_face<<<blocks_for(n, 128), 128, 0, s->stream>>>(
                s->f, s->sp->p, d, s->odr, c, c64, s->bc3.x[5] != 0, s->bc3.y[6] != 0,
                s->bc3.z[7] != 0);
            plain3d_fill_ghosts(s);
        }
    }
};

}  // namespace

int split3d_step(Sim *s, double dt)
{
    const Geometry &G = s->g;
    const StepCtx x(s);
    for (int rk = 0; rk < s->nrk; rk++) {
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_PREP);
            x.prim(rk, 0, G.nz);
            x.aux(0, G.nz);
        }
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_SWEEP);
            x.sweeps();
        }
        {
            TimedLaunch tl(&s->timer, KK_EMF);
            x.emf(0, G.nz);
        }
        {
            TimedLaunch tl(&s->timer, KK_SPLIT_UPDATE);
            x.update(rk, dt, G.oz, G.nz - 2 * G.oz);
        }
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

// One step of a periodic state held in host arrays h[0..7] (the C-ABI
// drivers), in place: the same kernels and arithmetic as upload +
// split3d_step + download, run over z-plane ranges in the order of a
// SlabPlan (slab_plan.h), so that the upload overlaps the first RK stage and
// the download the last.  Uploads go in chunks of planes on one copy stream,
// each recorded by an event the compute stream waits on before the first
// kernel that reads those planes; downloads go on a second copy stream, each
// run of planes as soon as the update that writes it has been launched.
int split3d_step_host(Sim *s, double dt, double *const *h)
{
    const Geometry &G = s->g;
    SplitFields &sf = *s->sp;
    const int nz = G.nz, oz = G.oz, Nz = nz - 2 * oz;
    if (!sf.cs) MLAU_CUDA(cudaStreamCreateWithFlags(&sf.cs, cudaStreamNonBlocking));
    if (!sf.cd) MLAU_CUDA(cudaStreamCreateWithFlags(&sf.cd, cudaStreamNonBlocking));
    if (!sf.ev_start) MLAU_CUDA(cudaEventCreateWithFlags(&sf.ev_start, cudaEventDisableTiming));
    if (!sf.plan || sf.plan_nrk != s->nrk) {
        // the first and last stages are asked for in slabs of >= 16 interior
        // planes (at most 8); uploads of half a slab (tapered slab sizes and
        // 4-16 slabs measured within 2 % of this at 256^3).  The first stage
        // starts a quarter of the way up: 20.8 ms per 256^3 call against 21.3
        // starting at the bottom slab (whose periodic sources at the far end
        // must arrive first) and 21.2 starting half way.
        const int nslab = std::max(1, std::min(8, Nz / 16));
        const int chunk = std::max(4, (nz + 2 * nslab - 1) / (2 * nslab));
        sf.plan.reset(new SlabPlan(SlabGeom{nz, oz, SG<2>::T}, s->nrk, nslab, chunk, nslab / 4));
        sf.plan_nrk = s->nrk;
        int ndn = 0;
        for (const SlabOp &o : sf.plan->ops) ndn += o.kind == SP_DOWNLOAD;
        auto grow = [&](std::vector<cudaEvent_t> &v, size_t n) -> int {
            while (v.size() < n) {
                cudaEvent_t e = nullptr;
                if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) {
                    sf.plan.reset();  // the next call builds the plan and its events again
                    set_error("split3d_step_host: cudaEventCreate: %s",
                              cudaGetErrorString(cudaGetLastError()));
                    return MLAU_ERR_CUDA;
                }
                v.push_back(e);
            }
            return MLAU_OK;
        };
        if (int rc = grow(sf.ev_up, (size_t)sf.plan->uploads())) return rc;
        if (int rc = grow(sf.ev_dn, (size_t)ndn)) return rc;
    }
    const long long plane = (long long)G.nx * G.ny;
    auto copy = [&](cudaStream_t st, int k0, int k1, bool in) -> int {
        for (int v = 0; v < 8; v++) {
            double *dv = s->f.s[v] + k0 * plane, *hv = h[v] + k0 * plane;
            const size_t bytes = sizeof(double) * (size_t)(k1 - k0) * plane;
            MLAU_CUDA(in ? cudaMemcpyAsync(dv, hv, bytes, cudaMemcpyHostToDevice, st)
                         : cudaMemcpyAsync(hv, dv, bytes, cudaMemcpyDeviceToHost, st));
        }
        return MLAU_OK;
    };
    // the previous use of the state on the compute stream ends before the upload
    MLAU_CUDA(cudaEventRecord(sf.ev_start, s->stream));
    MLAU_CUDA(cudaStreamWaitEvent(sf.cs, sf.ev_start, 0));
    const StepCtx x(s);
    int nd = 0;
    for (const SlabOp &o : sf.plan->ops) {
        const int n = o.b - o.a;
        switch (o.kind) {
        case SP_UPLOAD:
            if (int rc = copy(sf.cs, o.a, o.b, true)) return rc;
            MLAU_CUDA(cudaEventRecord(sf.ev_up[o.n], sf.cs));
            break;
        case SP_WAIT: MLAU_CUDA(cudaStreamWaitEvent(s->stream, sf.ev_up[o.n], 0)); break;
        case SP_PRIM: x.prim(o.rk, o.a, n); break;
        case SP_AUX: x.aux(o.a, n); break;
        case SP_SWEEP_X: x.sweep(0, o.a, o.b); break;
        case SP_SWEEP_Y: x.sweep(1, o.a, o.b); break;
        case SP_SWEEP_Z: x.sweep(2, o.a, o.b); break;
        case SP_EMF: x.emf(o.a, n); break;
        case SP_UPDATE: x.update(o.rk, dt, o.a, n); break;
        case SP_DOWNLOAD:
            MLAU_CUDA(cudaEventRecord(sf.ev_dn[nd], s->stream));
            MLAU_CUDA(cudaStreamWaitEvent(sf.cd, sf.ev_dn[nd], 0));
            nd++;
            if (int rc = copy(sf.cd, o.a, o.b, false)) return rc;
            break;
        case SP_STAGE:
            x.prim(o.rk, 0, nz);
            x.aux(0, nz);
            x.sweeps();
            x.emf(0, nz);
            x.update(o.rk, dt, oz, Nz);
            break;
        default: set_error("split3d_step_host: bad plan op"); return MLAU_ERR_ARG;
        }
    }
    MLAU_CUDA(cudaGetLastError());
    MLAU_CUDA(cudaStreamSynchronize(sf.cd));
    MLAU_CUDA(cudaStreamSynchronize(sf.cs));
    return split3d_check(s);
}

}  // namespace mlau
