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

// Primitives of cell i from its conserved state (ro, mx, my, mz, by, bz, en).
__device__ __forceinline__ void put_prim1(const PlainFields &f, int i, double ro, double mx,
                                          double my, double mz, double by, double bz, double en,
                                          double bx, double gamma)
{
    const double iro = 1.0 / ro;
    const double vx = mx * iro, vy = my * iro, vz = mz * iro;
    const double v2 = vx * vx + vy * vy + vz * vz;
    const double b2 = bx * bx + by * by + bz * bz;
    f.vx[i] = vx;
    f.vy[i] = vy;
    f.vz[i] = vz;
    f.pr[i] = (gamma - 1) * (en - 0.5 * (ro * v2 + b2));
}

// Primitives and the copy of the state U^n, at the first stage of a step (the
// later stages take their primitives from the update before them).
__global__ void k_prim1(PlainFields f, int nx, double bx, double gamma, int save_u0)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx) return;
    if (save_u0)
        for (int v = 0; v < 8; v++)
            if (v != 5) f.u0[v][i] = f.s[v][i];
    put_prim1(f, i, f.s[0][i], f.s[1][i], f.s[2][i], f.s[3][i], f.s[6][i], f.s[7][i], f.s[4][i],
              bx, gamma);
}

// Face states (:133-186): full characteristic system where any of the three
// central cells has sonic Mach^2 >= 1, Alfven + entropy system elsewhere.
//
// A cell's work is spread over 8 lanes: on this part a warp's FP64
// instruction holds its sub-partition's FP64 pipe for 64 cycles, and a
// 2048-cell grid at one cell per thread is 64 warps running one long serial
// chain each.  Lane r (0..6) projects the stencil on characteristic field r,
// interpolates it and back-projects output r; lane 7 repeats field 6 and
// stores nothing.  Every lane evaluates the cell's eigen-system (the same
// values).  The projections and back-projections are the dense 7-term sums of
// include/mhd_eigen.h (:455-684) in its order, the same on every lane (no
// divergence), so the face values equal those of the one-lane form and the
// reference's; the lanes exchange the interpolated fields by warp shuffles.
constexpr int RLANES = 8;

// Left eigenvector n (Ln[k] = L[n][k]) and entry n of every right
// eigenvector (Rc[k] = R[k][n], the back-projection's coefficients of output
// n) from a dense fill, selected with unrolled predicated moves so that the
// 7x7 matrices stay in registers and their constant entries fold away;
// eigenvalue n into *lam.
template <class FILL>
__device__ __forceinline__ void eig_row(FILL fill, int n, double Ln[7], double Rc[7], double *lam)
{
    double al[7], L[7][7], R[7][7];
    fill(al, L, R);
#pragma unroll
    for (int k = 0; k < 7; k++) {
        Ln[k] = L[0][k];
        Rc[k] = R[k][0];
    }
    *lam = al[0];
#pragma unroll
    for (int j = 1; j < 7; j++) {
#pragma unroll
        for (int k = 0; k < 7; k++) {
            Ln[k] = (n == j) ? L[j][k] : Ln[k];
            Rc[k] = (n == j) ? R[k][j] : Rc[k];
        }
        *lam = (n == j) ? al[j] : *lam;
    }
}

__global__ void k_rec1(PlainFields f, int nx, int odr, int eig, double bx, double gamma)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = t & (RLANES - 1), i = 2 + t / RLANES;
    const bool live = i < nx - 2;
    const int ic = live ? i : nx - 3;  // every lane takes part in the shuffles
    const int n = r < 7 ? r : 6;
    double q[7][5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        const int s = ic + m - 2;
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
    for (int u = 0; u < 3; u++) {
        const double c2 = gamma * q[6][1 + u] / q[0][1 + u];
        const double v2 = q[1][1 + u] * q[1][1 + u] + q[2][1 + u] * q[2][1 + u]
                          + q[3][1 + u] * q[3][1 + u];
        mach[u] = v2 / c2;
    }
    // Ln: the lane's left eigenvector; Rc[j]: entry n of right eigenvector j
    // (the back-projection's coefficient of field j in output n)
    double Ln[7], Rc[7], lam;
    const double c0 = q[0][2], c1 = q[1][2], c2 = q[2][2], c3 = q[3][2], c4 = q[4][2],
                 c5 = q[5][2], c6 = q[6][2];
    if (vmax(mach[0], vmax(mach[1], mach[2])) >= 1.0) {
        if (eig == EIG_MIYOSHI)
            eig_row([&](double *a, double (*L)[7], double (*R)[7]) {
                eigen_mi_dense(c0, c1, c2, c3, bx, c4, c5, c6, gamma, a, L, R); }, n, Ln, Rc, &lam);
        else
            eig_row([&](double *a, double (*L)[7], double (*R)[7]) {
                eigen_st_dense(c0, c1, c2, c3, bx, c4, c5, c6, gamma, a, L, R); }, n, Ln, Rc, &lam);
    } else {
        eig_row([&](double *a, double (*L)[7], double (*R)[7]) {
            eigen_ae_dense(c0, c1, c2, c3, bx, c4, c5, c6, gamma, a, L, R); }, n, Ln, Rc, &lam);
    }
    double w[5];
#pragma unroll
    for (int m = 0; m < 5; m++)
        w[m] = (+Ln[0] * q[0][m] + Ln[1] * q[1][m] + Ln[2] * q[2][m] + Ln[3] * q[3][m]
                + Ln[4] * q[4][m] + Ln[5] * q[5][m] + Ln[6] * q[6][m]);
    double wl, wr;
    rec_lr(odr, w, wl, wr);
    // blocks of fewer than 32 threads are one partial warp
    const unsigned mask = blockDim.x >= 32 ? 0xffffffffu : (1u << blockDim.x) - 1u;
    const int g0 = (threadIdx.x & 31) & ~(RLANES - 1);
    double fl[7], fr[7];
#pragma unroll
    for (int k = 0; k < 7; k++) {
        fl[k] = __shfl_sync(mask, wl, g0 + k);
        fr[k] = __shfl_sync(mask, wr, g0 + k);
    }
    double ul = Rc[0] * fl[0] + Rc[1] * fl[1] + Rc[2] * fl[2] + Rc[3] * fl[3] + Rc[4] * fl[4]
                + Rc[5] * fl[5] + Rc[6] * fl[6];
    double ur = Rc[0] * fr[0] + Rc[1] * fr[1] + Rc[2] * fr[2] + Rc[3] * fr[3] + Rc[4] * fr[4]
                + Rc[5] * fr[5] + Rc[6] * fr[6];
    // exact-zero guard (mhd_eigen.h:516-529): output n of a field that is zero
    // across the stencil
    bool zero = false;
#pragma unroll
    for (int k = 1; k <= 5; k++) {
        const bool z = q[k][0] == 0.0 && q[k][1] == 0.0 && q[k][2] == 0.0 && q[k][3] == 0.0 &&
                       q[k][4] == 0.0;
        zero = (n == k) ? z : zero;
    }
    if (zero) {
        ul = 0.0;
        ur = 0.0;
    }
    if (live && r < 7) {
        f.ul[n][i + 1] = ul;
        f.ur[n][i] = ur;
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

// The MLAU flux (include/mhd_flux.h:26-213, point.cuh flux_mlau) of one face
// on a lane pair: lane side 0 evaluates the left state's quantities, side 1
// the right state's (energies, fast and "cc" speeds, the star-state
// corrections, the boundary-normal field splits), and the pair exchanges
// them by shuffles; the quantities that join both sides are evaluated by
// both lanes.  Every quantity keeps flux_mlau's expression and operand
// order, so the fluxes are its own bit for bit; a lane's chain of divisions
// and square roots is 11 long instead of 19.
__device__ __forceinline__ void flux_mlau_pair(const double *L, const double *R, double bnc,
                                               double gamma, double dv0, double dv1, int side,
                                               unsigned mask, double *f)
{
    const double EPS = 1e-8;
    const double *X = side ? R : L;  // this lane's state
    auto other = [&](double v) { return __shfl_xor_sync(mask, v, 1); };
    auto pick = [&](double own, double oth, int want) { return side == want ? own : oth; };
    const double rol = L[0], vnl = L[1], vtl = L[2], vul = L[3], btl = L[4], bul = L[5];
    const double ror = R[0], vnr = R[1], vtr = R[2], vur = R[3], btr = R[4], bur = R[5];
    const double gm1i = 1.0 / (gamma - 1.0);
    const double bnc2 = bnc * bnc;
    const double sgn = (bnc > 0) ? 1.0 : -1.0;
    const double bnca = sgn * bnc;
    // per side
    const double roi = 1.0 / X[0];
    const double v2 = X[1] * X[1] + X[2] * X[2] + X[3] * X[3];
    const double pm = 0.5 * (X[4] * X[4] + X[5] * X[5]);
    const double pt = X[6] + pm;
    const double en = gm1i * X[6] + pm + 0.5 * X[0] * v2;
    const double hn = (en + pt) * roi;
    const double c2 = gamma * X[6] * roi;
    const double ca2 = bnc2 * roi;
    double cb2 = c2 + ca2 + 2.0 * pm * roi;
    const double cf2 = 0.5 * (cb2 + sqrt(fabs(cb2 * cb2 - 4.0 * c2 * ca2)));
    cb2 = v2 + ca2 + 2.0 * pm * roi;
    const double cc2 = 0.5 * (cb2 + sqrt(fabs(cb2 * cb2 - 4.0 * v2 * ca2)));
    const double cf2o = other(cf2), cc2o = other(cc2), pto = other(pt), hno = other(hn),
                 roio = other(roi);
    const double cfl2 = pick(cf2, cf2o, 0), cfr2 = pick(cf2, cf2o, 1);
    const double ccl2 = pick(cc2, cc2o, 0), ccr2 = pick(cc2, cc2o, 1);
    const double ptl = pick(pt, pto, 0), ptr = pick(pt, pto, 1);
    const double hnl = pick(hn, hno, 0), hnr = pick(hn, hno, 1);
    const double roli = pick(roi, roio, 0), rori = pick(roi, roio, 1);
    // joint
    const double cmax = sqrt(vmax(cfl2, cfr2));
    const double cfn = cmax;
    const double cfni = 1.0 / cfn;
    const double sl = vmin(0.0, vmin(vnl, vnr) - cmax);
    const double sr = vmax(0.0, vmax(vnl, vnr) + cmax);
    const double mal = vnl * cfni, mar = vnr * cfni;
    const double snl = (mal > 0) ? 1.0 : -1.0;
    const double snr = (mar > 0) ? 1.0 : -1.0;
    double theta = vmin(1.0, (cfn - vmin(dv0, 0.0)) / (cfn - vmin(dv1, 0.0)));
    theta *= theta;
    theta *= theta;
    const double alpha = 0.1875, beta = 0.125;
    const double malp1 = mal + 1.0, marm1 = mar - 1.0;
    const double mal2m1 = mal * mal - 1.0, mar2m1 = mar * mar - 1.0;
    double bfl, ffl, bfr, ffr;
    if (snl * mal > 1.0) {
        bfl = 0.5 * (1.0 + snl);
        ffl = bfl * mal;
    } else {
        bfl = +0.25 * malp1 * malp1 * (2.0 - mal) + alpha * mal * mal2m1 * mal2m1;
        ffl = +0.25 * malp1 * malp1 + beta * mal2m1 * mal2m1;
    }
    if (snr * mar > 1.0) {
        bfr = 0.5 * (1.0 - snr);
        ffr = bfr * mar;
    } else {
        bfr = +0.25 * marm1 * marm1 * (2.0 + mar) - alpha * mar * mar2m1 * mar2m1;
        ffr = -0.25 * marm1 * marm1 - beta * mar2m1 * mar2m1;
    }
    const double mnc = ffl + ffr;
    double mflux = mnc * cfn;
    const double dpt = ptr - ptl;
    const double dvn = vnr - vnl;
    mflux -= vmax(1.0 - fabs(mnc), 0.0) * theta * cfni * dpt / (rol + ror);
    const double dir = (mflux > 0) ? 1.0 : -1.0;
    const double dirl = 0.5 * (1.0 + dir);
    const double dirr = 1.0 - dirl;
    mflux *= (dirl * rol + dirr * ror);
    const double mfl = mflux * dirl;
    const double mfr = mflux - mfl;
    double ptot = bfl * ptl + bfr * ptr;
    const double cfmod = sqrt(vmax(ccl2, ccr2));
    ptot -= 0.25 * bfl * bfr * (rol + ror) * cfmod * dvn;
    ptot -= 0.5 * (1.0 - cfmod * cfni) * (bfl + bfr - 1.0) * (ptl + ptr);
    const double slvl = sl - vnl, srvr = sr - vnr;
    const double snc = dirl * sl + dirr * sr;
    const double vndnm = mflux + dirl * rol * slvl + dirr * ror * srvr;
    const double vnc = ((fabs(vndnm) > EPS) && (snc != 0)) ? (mflux * snc / vndnm)
                                                          : (dirl * vnl + dirr * vnr);
    const double slvc = sl - vnc, srvc = sr - vnc;
    // per side: star-state corrections
    const double svX = side ? srvr : slvl, svc = side ? srvc : slvc;
    const double svci = 1.0 / svc;
    const double rhd = X[0] * svX * svc - bnc2;
    double dvt = 0.0, dvu = 0.0, dbt = 0.0, dbu = 0.0;
    if (fabs(rhd) > EPS) {
        const double g = (vnc - X[1]) / rhd;
        dvt = -bnc * X[4] * g;
        dvu = -bnc * X[5] * g;
        dbt = bnc2 * X[4] * g * svci;
        dbu = bnc2 * X[5] * g * svci;
    }
    const double cmp = svX * svci;
    const double ro2 = X[0] * cmp;
    const double sro = sqrt(ro2);
    const double vt2 = dvt + X[2], vu2 = dvu + X[3];
    const double bt2 = dbt + X[4] * cmp, bu2 = dbu + X[5] * cmp;
    const double o_svci = other(svci), o_sro = other(sro), o_vt2 = other(vt2),
                 o_vu2 = other(vu2), o_bt2 = other(bt2), o_bu2 = other(bu2), o_dvt = other(dvt),
                 o_dvu = other(dvu), o_dbt = other(dbt), o_dbu = other(dbu);
    const double slvci = pick(svci, o_svci, 0), srvci = pick(svci, o_svci, 1);
    const double srol = pick(sro, o_sro, 0), sror = pick(sro, o_sro, 1);
    const double vt2l = pick(vt2, o_vt2, 0), vt2r = pick(vt2, o_vt2, 1);
    const double vu2l = pick(vu2, o_vu2, 0), vu2r = pick(vu2, o_vu2, 1);
    const double bt2l = pick(bt2, o_bt2, 0), bt2r = pick(bt2, o_bt2, 1);
    const double bu2l = pick(bu2, o_bu2, 0), bu2r = pick(bu2, o_bu2, 1);
    const double dvtl = pick(dvt, o_dvt, 0), dvtr = pick(dvt, o_dvt, 1);
    const double dvul = pick(dvu, o_dvu, 0), dvur = pick(dvu, o_dvu, 1);
    const double dbtl = pick(dbt, o_dbt, 0), dbtr = pick(dbt, o_dbt, 1);
    const double dbul = pick(dbu, o_dbu, 0), dbur = pick(dbu, o_dbu, 1);
    // joint
    const double sroi = 1.0 / (srol + sror);
    const double srollri = srol * sroi, srorlri = sror * sroi;
    const double bnflb = sgn * vmin(vmax(0.0, srollri * (bnca + sror * vnc)), bnca);
    const double bnfrb = sgn * vmin(vmax(0.0, srorlri * (bnca - srol * vnc)), bnca);
    // the two velocity-side splits, one per lane
    const double bnfv = side ? sgn * vmin(vmax(0.0, srollri * (bnca - mflux / srol)), bnca)
                             : sgn * vmin(vmax(0.0, srorlri * (bnca + mflux / sror)), bnca);
    const double o_bnfv = other(bnfv);
    const double bnflv = pick(bnfv, o_bnfv, 0), bnfrv = pick(bnfv, o_bnfv, 1);
    const double bnsrv = vmax(bnca - dir * vnc * (dirl * srol + dirr * sror), 0.0);
    const double ccb = sroi * bnsrv;
    const double ccv = srol * sror * ccb;
    double bnvt = bnflb * vt2l + bnfrb * vt2r + ccb * (bt2r - bt2l);
    double bnvu = bnflb * vu2l + bnfrb * vu2r + ccb * (bu2r - bu2l);
    double bnbt = bnflv * bt2l + bnfrv * bt2r + ccv * (vt2r - vt2l);
    double bnbu = bnflv * bu2l + bnfrv * bu2r + ccv * (vu2r - vu2l);
    bnvt -= vnc * (dirl * dbtl + dirr * dbtr);
    bnvu -= vnc * (dirl * dbul + dirr * dbur);
    bnbt -= mflux * (dirl * dvtl + dirr * dvtr);
    bnbu -= mflux * (dirl * dvul + dirr * dvur);
    f[0] = mflux;
    f[1] = mfl * vnl + mfr * vnr + ptot - 0.5 * bnc2;
    f[2] = mfl * vtl + mfr * vtr - bnbt;
    f[3] = mfl * vul + mfr * vur - bnbu;
    f[4] = mfl * btl * roli + mfr * btr * rori - bnvt;
    f[5] = mfl * bul * roli + mfr * bur * rori - bnvu;
    const double vb1 = dirl * (vtl * btl + vul * bul) + dirr * (vtr * btr + vur * bur);
    const double vb2 = dirl * (vt2l * bt2l + vu2l * bu2l) + dirr * (vt2r * bt2r + vu2r * bu2r);
    double rv2b2 = (mflux * vnc - bnc2);
    rv2b2 *= rv2b2;
    double vb3 = 0.0;
    if (rv2b2 > EPS * EPS) {
        vb3 = (+(f[2] * vnc + f[4] * bnc) * (f[2] * bnc + f[4] * mflux)
               + (f[3] * vnc + f[5] * bnc) * (f[3] * bnc + f[5] * mflux)) / rv2b2;
    }
    const double bnvb = sgn * (bnca * (snc * vb2 - vnc * vb1) * (dirl * slvci + dirr * srvci)
                               + bnsrv * (vb3 - vb2));
    f[6] = mfl * hnl + mfr * hnr - bnvb;
}

// MLAU faces on lane pairs (flux_mlau_pair); the other solvers keep one
// face per thread (k_flux1).
__global__ void k_flux1_mlau(PlainFields f, int nx, double bx, double gamma)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int side = t & 1, i = 3 + t / 2;
    const bool live = i < nx - 2;
    const int ic = live ? i : nx - 3;  // both lanes of a pair take part in the shuffles
    const unsigned mask = blockDim.x >= 32 ? 0xffffffffu : (1u << blockDim.x) - 1u;
    double L[7], R[7], F[7];
#pragma unroll
    for (int n = 0; n < 7; n++) {
        L[n] = f.ul[n][ic];
        R[n] = f.ur[n][ic];
    }
    flux_mlau_pair(L, R, bx, gamma, (f.vx[ic] - f.vx[ic - 1]), 0.0, side, mask, F);
    if (!live) return;
#pragma unroll
    for (int n = 0; n < 7; n++)
        if ((n < 4) == (side == 0)) f.F[0][n][i] = F[n];
}

// openbc1d_mhd (1D/SERIAL/shock/openbc1d_mhd.c:21-175).  The two sides read
// and write disjoint cells (interior width >= ghost depth), so each runs in
// its own block of 8 lanes: block 0 the left side, block 1 the right.  Lane r
// (0..6) projects both cells on characteristic field r and applies its
// outflow condition; the back-projection of primitive r follows the dense
// 7-term sums of the header, with the fields exchanged by shuffles; lane 0
// converts to conserved variables and fills the ghost cells.
__global__ void k_openbc1(PlainFields f, int nx, int xoff, double bx, double dtdx, double gamma)
{
    const int r = threadIdx.x;
    if (blockIdx.x > 1 || r >= 8) return;  // launched with 8 threads per block
    const int n = r < 7 ? r : 6;
    const double *ro = f.s[0], *mx = f.s[1], *my = f.s[2], *mz = f.s[3], *en = f.s[4],
                 *by = f.s[6], *bz = f.s[7];
    const double bx2 = bx * bx;
    const int side = blockIdx.x;
    const int sgn = side ? -1 : 1;
    const int si = side ? (nx - xoff - 1) : xoff;
    const int so = si - sgn;
    double q[2][7];
    for (int t = 0; t < 2; t++) {
        const int s = t ? so : si;
        const double rr = ro[s], iro = 1.0 / rr;
        const double vx = mx[s] * iro, vy = my[s] * iro, vz = mz[s] * iro;
        const double v2 = vx * vx + vy * vy + vz * vz;
        const double b2 = bx * bx + by[s] * by[s] + bz[s] * bz[s];
        q[t][0] = rr;
        q[t][1] = vx;
        q[t][2] = vy;
        q[t][3] = vz;
        q[t][4] = by[s];
        q[t][5] = bz[s];
        q[t][6] = (gamma - 1) * (en[s] - 0.5 * (rr * v2 + b2));
    }
    double Ln[7], Rc[7], lam;
    eig_row([&](double *a, double (*L)[7], double (*R)[7]) {
        eigen_st_dense(0.5 * (q[0][0] + q[1][0]), 0.5 * (q[0][1] + q[1][1]), 0.0, 0.0,
                       0.5 * (bx + bx), 0.5 * (q[0][4] + q[1][4]), 0.5 * (q[0][5] + q[1][5]),
                       0.5 * (q[0][6] + q[1][6]), gamma, a, L, R); }, n, Ln, Rc, &lam);
    double w[2];
    for (int t = 0; t < 2; t++)
        w[t] = (+Ln[0] * q[t][0] + Ln[1] * q[t][1] + Ln[2] * q[t][2] + Ln[3] * q[t][3]
                + Ln[4] * q[t][4] + Ln[5] * q[t][5] + Ln[6] * q[t][6]);
    const double c = sgn * lam;
    const double w1 = (c > 0) ? w[1] : (1 + c * dtdx) * w[1] - c * dtdx * w[0];
    double wv[7];
    for (int k = 0; k < 7; k++) wv[k] = __shfl_sync(0xffu, w1, k, 8);
    const double pn = Rc[0] * wv[0] + Rc[1] * wv[1] + Rc[2] * wv[2] + Rc[3] * wv[3]
                      + Rc[4] * wv[4] + Rc[5] * wv[5] + Rc[6] * wv[6];
    double p[7];
    for (int k = 0; k < 7; k++) p[k] = __shfl_sync(0xffu, pn, k, 8);
    if (r != 0) return;
    // conserved ghost state, in the reference's order of operations
    const double v2 = p[1] * p[1] + p[2] * p[2] + p[3] * p[3];
    const double b2 = bx2 + p[4] * p[4] + p[5] * p[5];
    double *o = f.obc + 7 * side;
    o[0] = p[0];
    o[1] = p[1] * p[0];
    o[2] = p[2] * p[0];
    o[3] = p[3] * p[0];
    o[4] = p[4];
    o[5] = p[5];
    o[6] = p[6] / (gamma - 1.0) + 0.5 * (p[0] * v2 + b2);
}

// Update (:220-255); with periodic boundaries each cell also writes its ghost
// images (prdc_1d, 1D/SERIAL/wave/prdc_1d.c).  openbc: the first stage of an
// open-boundary step, whose ghost cells take the states k_openbc1 left in
// f.obc (every ghost cell of a side the same, openbc1d_mhd.c:160-175); the
// first and last interior threads write them.  Every cell written also gets
// its primitives (k_prim1's arithmetic), which the next stage reads; ghost
// cells an open boundary leaves alone keep those of the first stage.
__global__ void k_update1(PlainFields f, int nx, int xoff, int odr, double ra, double rb,
                          double dtdx, int periodic, int openbc, double bx, double gamma)
{
    const int i = xoff + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nx - xoff) return;
    const int sv[7] = {0, 1, 2, 3, 6, 7, 4};  // flux order (ro, mx, my, mz, by, bz, en)
    if (openbc && (i == xoff || i == nx - xoff - 1)) {
        const int side = i == xoff ? 0 : 1;
        const int g0 = side ? nx - xoff : 0;
        double g[7];
        for (int v = 0; v < 7; v++) {
            g[v] = f.obc[7 * side + v];
            for (int j = 0; j < xoff; j++) f.s[sv[v]][g0 + j] = g[v];
        }
        for (int j = 0; j < xoff; j++)
            put_prim1(f, g0 + j, g[0], g[1], g[2], g[3], g[4], g[5], g[6], bx, gamma);
    }
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
        put_prim1(f, im[a], out[0], out[1], out[2], out[3], out[4], out[5], out[6], bx, gamma);
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
    rc |= dalloc(s, &f.obc, 14);
    if (rc) return MLAU_ERR_NOMEM;
    // created here, not at the first step, which may be inside a graph capture
    MLAU_CUDA(cudaStreamCreateWithFlags(&s->stream2, cudaStreamNonBlocking));
    MLAU_CUDA(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
    MLAU_CUDA(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    return MLAU_OK;
}

// 1D grids hold a few thousand cells, each cell a long chain of FP64
// operations: blocks of 32 threads spread a 2048-cell problem over 64 SMs
// instead of 16 at 128 threads.  Smaller blocks measured slower (16: 0.181,
// 8: 0.282 ms per step against 0.151): a partial warp's FP64 instruction
// holds the pipe as long as a full one.
constexpr int T1D = 32;

int plain1d_step(Sim *s, double dt)
{
    const Geometry &g = s->g;
    PlainFields &f = s->f;
    cudaStream_t st = s->stream;
    const int nx = g.nx, off = g.ox;
    const double dtdx = dt / g.dx;
    const int T = T1D;
    const bool open = s->bc1d == MLAU_BC1D_OPEN;
    // The open boundary reads only the state of its two end cells, which no
    // kernel of the first stage writes before the update: it runs on a second
    // stream beside the stage (forked here, joined before the update; one
    // stream when the kernels are timed one by one).
    const bool fork = open && !s->timer.on && s->stream2;
    for (int rk = 0; rk < s->nrk; rk++) {
        double ra, rb;
        rk_coef(s->nrk, rk, ra, rb);
        if (fork && rk == 0) {
            MLAU_CUDA(cudaEventRecord(s->ev_fork, st));
            MLAU_CUDA(cudaStreamWaitEvent(s->stream2, s->ev_fork, 0));
            k_openbc1<<<2, 8, 0, s->stream2>>>(f, nx, off, s->bx1d, dtdx, s->gamma);
            MLAU_CUDA(cudaEventRecord(s->ev_join, s->stream2));
        }
        if (rk == 0) {
            TimedLaunch tl(&s->timer, KK_PRIM);
            k_prim1<<<blocks_for(nx, T), T, 0, st>>>(f, nx, s->bx1d, s->gamma, 1);
        }
        {
            TimedLaunch tl(&s->timer, KK_REC);
            k_rec1<<<blocks_for((long long)(nx - 4) * RLANES, T), T, 0, st>>>(f, nx, s->odr, s->eig,
                                                                            s->bx1d, s->gamma);
        }
        {
            TimedLaunch tl(&s->timer, KK_FLUX);
            if (s->flux == FLUX_MLAU)
                k_flux1_mlau<<<blocks_for((long long)(nx - 5) * 2, T), T, 0, st>>>(f, nx, s->bx1d,
                                                                                s->gamma);
            else
                k_flux1<<<blocks_for(nx - 5, T), T, 0, st>>>(f, nx, s->flux, s->bx1d, s->gamma);
        }
        if (open && rk == 0) {
            if (fork) {
                MLAU_CUDA(cudaStreamWaitEvent(st, s->ev_join, 0));
            } else {
                TimedLaunch tl(&s->timer, KK_AUX);
                k_openbc1<<<2, 8, 0, st>>>(f, nx, off, s->bx1d, dtdx, s->gamma);
            }
        }
        {
            TimedLaunch tl(&s->timer, KK_UPDATE);
            k_update1<<<blocks_for(nx - 2 * off, T), T, 0, st>>>(
                f, nx, off, s->odr, ra, rb, dtdx, s->bc1d == MLAU_BC1D_PERIODIC, open && rk == 0,
                s->bx1d, s->gamma);
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
        if (rk == 0) k_prim1<<<blocks_for(nx, T), T, 0, st>>>(f, nx, bx, gamma, 1);
        k_rec1<<<blocks_for((long long)(nx - 4) * RLANES, T), T, 0, st>>>(f, nx, odr, EIG_FULL,
                                                                        bx, gamma);
        if (flux == FLUX_MLAU)
            k_flux1_mlau<<<blocks_for((long long)(nx - 5) * 2, T), T, 0, st>>>(f, nx, bx, gamma);
        else
            k_flux1<<<blocks_for(nx - 5, T), T, 0, st>>>(f, nx, flux, bx, gamma);
        if (bc == MLAU_BC1D_OPEN && rk == 0) k_openbc1<<<2, 8, 0, st>>>(f, nx, off, bx, dtdx, gamma);
        k_update1<<<blocks_for(nx - 2 * off, T), T, 0, st>>>(f, nx, off, odr, ra, rb, dtdx,
                                                            bc == MLAU_BC1D_PERIODIC,
                                                            bc == MLAU_BC1D_OPEN && rk == 0, bx,
                                                            gamma);
        MLAU_CUDA(cudaGetLastError());
    }
    return MLAU_OK;
}

}  // namespace mlau
