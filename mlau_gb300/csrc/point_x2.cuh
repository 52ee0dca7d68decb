// Packed-FP32 forms of the WCNS4 characteristic reconstruction, for the
// FP32-split sweeps.
//
// The sweeps reconstruct perturbations from the cell centre, so the centre
// value of every 5-point stencil is exactly zero and its terms drop out.  What
// remains is mirror-symmetric: the left face value of a stencil f0..f4 is the
// right face value of f4..f0.  Values are therefore carried as float2 pairs -
// the outer points (f0, f4), the inner points (f1, f3), the two face values
// (left, right) - and computed with the packed FP32x2 operations of the
// sm_100 family (__ffma2_rn, __fadd2_rn, __fmul2_rn: one instruction for both
// lanes), which halves the issue slots of the arithmetic that dominates the
// sweep.
//
// Same formulas as wcns4_lr and reconst_alfven_core in point.cuh
// (include/interp.h:186-238, include/mhd_eigen.h:609-684) up to FP32
// rounding, with two rescalings that cancel in the normalised weights: the
// smoothness indicators carry a factor 4 (and the weight epsilon 16) and the
// candidate stencils the 1/8.
#pragma once

#include <cuda_runtime.h>

#include "point.cuh"

namespace mlau {

__device__ __forceinline__ float2 x2k(float c) { return make_float2(c, c); }
__device__ __forceinline__ float2 x2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 x2sub(float2 a, float2 b) { return __ffma2_rn(b, x2k(-1.f), a); }
__device__ __forceinline__ float2 x2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 x2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// WCNS4 of the stencil (o.x, i.x, 0, i.y, o.y): o holds the outer points
// (f0, f4), i the inner points (f1, f3).  Returns (value at the right face
// i+1/2 from the left, value at the left face i-1/2 from the right), the fl and
// fr of wcns4_lr.
//
// Lanes: pa / qa and the weights of stencils 0 / 2 are computed in the direct
// lanes (left, right); pc / qc come out in swapped lanes (right, left), as do
// the 3 f3 / 3 f1 parts of pb / qb, and the two accumulators are added across
// lanes at the end.
__device__ __forceinline__ float2 wcns4_pert_x2(float2 o, float2 i)
{
    // the indicators below are 4 x the reference's, so their squares are 16 x:
    // the epsilon is scaled with them (16 x the FP32 epsilon of wcns4_lr)
    const float eps = 16e-30f;
    // 4 x the smoothness indicators of the outer stencils: (s0, s2)
    const float2 p = x2fma(x2k(-4.f), i, o);
    const float2 q = x2fma(x2k(-2.f), i, o);
    float2 s = x2fma(x2mul(x2k(13.f / 3.f), q), q, x2mul(p, p));
    s = x2fma(s, s, x2k(eps));
    const float2 is = make_float2(1.f / s.x, 1.f / s.y);
    // ... and of the centre stencil
    const float p1 = i.x - i.y, q1 = i.x + i.y;
    const float s1 = fmaf((13.f / 3.f) * q1, q1, p1 * p1);
    const float wb = 0.65f / fmaf(s1, s1, eps);
    const float2 wa = x2mul(x2k(0.075f), is);  // pa (left) / qa (right)
    const float2 wc = x2mul(x2k(0.275f), is);  // qc (right) / pc (left): swapped lanes
    // candidate stencils / 8 without their centre terms
    const float2 pa = x2fma(x2k(-1.25f), i, x2mul(x2k(0.375f), o));    // (pa, qa)
    const float2 pcs = x2fma(x2k(0.75f), i, x2mul(x2k(-0.125f), o));   // (qc, pc)
    const float2 nd = x2fma(wa, pa, x2mul(x2k(-0.125f * wb), i));      // -f1 of pb, -f3 of qb
    const float2 ns = x2fma(wc, pcs, x2mul(x2k(0.375f * wb), i));      // 3 f1 of qb, 3 f3 of pb
    const float2 dd = x2add(wa, x2k(wb));
    return make_float2((nd.x + ns.y) / (dd.x + wc.y), (nd.y + ns.x) / (dd.y + wc.x));
}

// lcal_flr's 4th-order linear interpolation (left, right) of the stencil
// (o.x, i.x, 0, i.y, o.y) (3D/MPI/OTvortex/mhd_fd_ct_3d.c:48-63).
__device__ __forceinline__ float2 lin4_pert_x2(float2 o, float2 i)
{
    const float2 d = x2fma(x2k(-56.f * 0.003125f), i, x2mul(x2k(9.f * 0.003125f), o));
    const float2 w = x2fma(x2k(144.f * 0.003125f), i, x2mul(x2k(-11.f * 0.003125f), o));
    return make_float2(d.x + w.y, d.y + w.x);
}

// reconst_alfven_core for WCNS4 on perturbations: O[n] = (dq[n][0], dq[n][4]),
// I[n] = (dq[n][1], dq[n][3]) of the seven fields (ro, vx, vy, vz, by, bz,
// pr), qc the cell-centre values.  Returns LR[n] = (ul[n], ur[n]).
__device__ __forceinline__ void reconst_alfven_wcns4_x2(const float2 O[7], const float2 I[7],
                                                        const float qc[7], float bn, float gamma,
                                                        float2 LR[7])
{
    const float ro = qc[0], by = qc[4], bz = qc[5], pr = qc[6];
    const float iro = 1.f / ro;
    const float cs2 = gamma * pr * iro;
    const float ca2 = bn * bn * iro;
    const float ct2 = (by * by + bz * bz) * iro;
    const float cb2 = cs2 + ca2 + ct2;
    const float cf2 = 0.5f * (cb2 + sqrtf(fabsf(cb2 * cb2 - 4.f * cs2 * ca2)));
    const float sro = sqrtf(ro);
    const float isroh = 0.5f / sro;
    const float icf2 = 1.f / cf2;
    // characteristic variables of the outer and inner point pairs; w1 is
    // carried with the opposite sign (-w1 = w2 - cf2 r), which WCNS preserves
    float2 w[7][2];
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const float2 *P = h ? I : O;
        w[0][h] = P[1];
        w[2][h] = x2fma(x2k(by), P[4], x2fma(x2k(bz), P[5], P[6]));
        w[1][h] = x2fma(x2k(-cf2), P[0], w[2][h]);
        const float2 sy = x2mul(x2k(sro), P[2]), sz = x2mul(x2k(sro), P[3]);
        w[3][h] = x2add(sy, P[4]);
        w[4][h] = x2sub(sy, P[4]);
        w[5][h] = x2add(sz, P[5]);
        w[6][h] = x2sub(sz, P[5]);
    }
    float2 W[7];
#pragma unroll
    for (int n = 0; n < 7; n++) W[n] = wcns4_pert_x2(w[n][0], w[n][1]);
    LR[0] = x2mul(x2k(icf2), x2sub(W[2], W[1]));
    LR[1] = W[0];
    LR[2] = x2mul(x2k(isroh), x2add(W[3], W[4]));
    LR[3] = x2mul(x2k(isroh), x2add(W[5], W[6]));
    LR[4] = x2mul(x2k(0.5f), x2sub(W[3], W[4]));
    LR[5] = x2mul(x2k(0.5f), x2sub(W[5], W[6]));
    LR[6] = x2fma(x2k(-bz), LR[5], x2fma(x2k(-by), LR[4], W[2]));
}

// calc_flux_mlau (include/mhd_flux.h:26-213) in its split-jump form
// (flux_mlau<float, true>), with the left and right states as the lanes of
// the pairs P[n] = (L[n], R[n]), n = ro, vn, vt, vu, bt, bu, pr.  The
// per-side quantities - energies, enthalpies, fast and "cc" speeds, the Mach
// polynomials, the star-state corrections - run as packed operations; the
// right side's Mach polynomials are those of the left side at -Mn, so both
// come from one evaluation at (Mn_l, -Mn_r).
__device__ __forceinline__ void flux_mlau_x2(const float2 P[7], float bnc, float gamma, float dv0,
                                             float dv1, float f[7], float jp, float jv)
{
    const float EPS = 1e-8f;
    const float2 ro = P[0], vn = P[1], vt = P[2], vu = P[3], bt = P[4], bu = P[5], pr = P[6];
    const float gm1i = 1.f / (gamma - 1.f);
    const float bnc2 = bnc * bnc;
    const float sgn = (bnc > 0.f) ? 1.f : -1.f;
    const float bnca = sgn * bnc;
    const float2 roi = make_float2(1.f / ro.x, 1.f / ro.y);
    const float2 v2 = x2fma(vu, vu, x2fma(vt, vt, x2mul(vn, vn)));
    const float2 pm = x2mul(x2k(0.5f), x2fma(bt, bt, x2mul(bu, bu)));
    const float2 pt = x2add(pr, pm);
    const float2 en = x2fma(x2mul(x2k(0.5f), ro), v2, x2fma(x2k(gm1i), pr, pm));
    const float2 hn = x2mul(x2add(en, pt), roi);
    const float2 c2 = x2mul(x2mul(x2k(gamma), pr), roi);
    const float2 ca2 = x2mul(x2k(bnc2), roi);
    const float2 pm2 = x2mul(x2mul(x2k(2.f), pm), roi);
    float2 cb2 = x2add(x2add(c2, ca2), pm2);
    float2 dsc = x2fma(cb2, cb2, x2mul(x2mul(x2k(-4.f), c2), ca2));
    const float2 cf2 = x2mul(x2k(0.5f), x2add(cb2, make_float2(sqrtf(fabsf(dsc.x)), sqrtf(fabsf(dsc.y)))));
    cb2 = x2add(x2add(v2, ca2), pm2);
    dsc = x2fma(cb2, cb2, x2mul(x2mul(x2k(-4.f), v2), ca2));
    const float2 cc2 = x2mul(x2k(0.5f), x2add(cb2, make_float2(sqrtf(fabsf(dsc.x)), sqrtf(fabsf(dsc.y)))));
    const float cmax = sqrtf(vmax(cf2.x, cf2.y));
    const float cfn = cmax;
    const float cfni = 1.f / cfn;
    const float sl = vmin(0.f, vmin(vn.x, vn.y) - cmax);
    const float sr = vmax(0.f, vmax(vn.x, vn.y) + cmax);
    float theta = vmin(1.f, (cfn - vmin(dv0, 0.f)) / (cfn - vmin(dv1, 0.f)));
    theta *= theta;
    theta *= theta;
    const float alpha = 0.1875f, beta = 0.125f;
    // Mach polynomials at m = (Mn_l, -Mn_r): lanes (bfl, bfr), (ffl, -ffr)
    const float2 m = x2mul(vn, make_float2(cfni, -cfni));
    const float2 mp1 = x2add(m, x2k(1.f));
    const float2 m2m1 = x2fma(m, m, x2k(-1.f));
    const float2 mp1s = x2mul(mp1, mp1), m2m1s = x2mul(m2m1, m2m1);
    const float2 bsub = x2fma(x2mul(x2k(alpha), m), m2m1s,
                              x2mul(x2mul(x2k(0.25f), mp1s), x2sub(x2k(2.f), m)));
    const float2 fsub = x2fma(x2k(beta), m2m1s, x2mul(x2k(0.25f), mp1s));
    // supersonic side (|Mn| > 1): bf = 1 moving away from the face, else 0; ff = bf Mn
    const bool supl = fabsf(m.x) > 1.f, supr = fabsf(m.y) > 1.f;
    const float bfl = supl ? (m.x > 0.f ? 1.f : 0.f) : bsub.x;
    const float bfr = supr ? (m.y > 0.f ? 1.f : 0.f) : bsub.y;
    const float ffl = supl ? bfl * m.x : fsub.x;
    const float ffr = supr ? bfr * (-m.y) : -fsub.y;
    const float mnc = ffl + ffr;
    float mflux = mnc * cfn;
    mflux -= vmax(1.f - fabsf(mnc), 0.f) * theta * cfni * jp / (ro.x + ro.y);
    const float dir = (mflux > 0.f) ? 1.f : -1.f;
    const float dirl = 0.5f * (1.f + dir);
    const float dirr = 1.f - dirl;
    mflux *= (dirl * ro.x + dirr * ro.y);
    const float mfl = mflux * dirl;
    const float mfr = mflux - mfl;
    float ptot = bfl * pt.x + bfr * pt.y;
    const float cfmod = sqrtf(vmax(cc2.x, cc2.y));
    ptot -= 0.25f * bfl * bfr * (ro.x + ro.y) * cfmod * jv;
    ptot -= 0.5f * (1.f - cfmod * cfni) * (bfl + bfr - 1.f) * (pt.x + pt.y);
    const float2 sv = x2sub(make_float2(sl, sr), vn);  // (sl - vnl, sr - vnr)
    const float snc = dirl * sl + dirr * sr;
    const float vndnm = mflux + dirl * ro.x * sv.x + dirr * ro.y * sv.y;
    const float vnc = ((fabsf(vndnm) > EPS) && (snc != 0.f)) ? (mflux * snc / vndnm)
                                                             : (dirl * vn.x + dirr * vn.y);
    const float2 svc = x2sub(make_float2(sl, sr), x2k(vnc));  // (sl - vnc, sr - vnc)
    const float2 svci = make_float2(1.f / svc.x, 1.f / svc.y);
    const float2 rhd = x2fma(x2mul(ro, sv), svc, x2k(-bnc2));
    const float2 gq = x2sub(x2k(vnc), vn);
    const float2 g = make_float2(fabsf(rhd.x) > EPS ? gq.x / rhd.x : 0.f,
                                 fabsf(rhd.y) > EPS ? gq.y / rhd.y : 0.f);
    const float2 dvt = x2mul(x2mul(x2k(-bnc), bt), g), dvu = x2mul(x2mul(x2k(-bnc), bu), g);
    const float2 gs = x2mul(g, svci);
    const float2 dbt = x2mul(x2mul(x2k(bnc2), bt), gs), dbu = x2mul(x2mul(x2k(bnc2), bu), gs);
    const float2 cmp = x2mul(sv, svci);
    const float2 ro2 = x2mul(ro, cmp);
    const float srol = sqrtf(ro2.x), sror = sqrtf(ro2.y);
    const float2 vt2 = x2add(dvt, vt), vu2 = x2add(dvu, vu);
    const float2 bt2 = x2fma(bt, cmp, dbt), bu2 = x2fma(bu, cmp, dbu);
    const float sroi = 1.f / (srol + sror);
    const float srollri = srol * sroi, srorlri = sror * sroi;
    const float bnflb = sgn * vmin(vmax(0.f, srollri * (bnca + sror * vnc)), bnca);
    const float bnfrb = sgn * vmin(vmax(0.f, srorlri * (bnca - srol * vnc)), bnca);
    const float bnflv = sgn * vmin(vmax(0.f, srorlri * (bnca + mflux / sror)), bnca);
    const float bnfrv = sgn * vmin(vmax(0.f, srollri * (bnca - mflux / srol)), bnca);
    const float bnsrv = vmax(bnca - dir * vnc * (dirl * srol + dirr * sror), 0.f);
    const float ccb = sroi * bnsrv;
    const float ccv = srol * sror * ccb;
    float bnvt = bnflb * vt2.x + bnfrb * vt2.y + ccb * (bt2.y - bt2.x);
    float bnvu = bnflb * vu2.x + bnfrb * vu2.y + ccb * (bu2.y - bu2.x);
    float bnbt = bnflv * bt2.x + bnfrv * bt2.y + ccv * (vt2.y - vt2.x);
    float bnbu = bnflv * bu2.x + bnfrv * bu2.y + ccv * (vu2.y - vu2.x);
    bnvt -= vnc * (dirl * dbt.x + dirr * dbt.y);
    bnvu -= vnc * (dirl * dbu.x + dirr * dbu.y);
    bnbt -= mflux * (dirl * dvt.x + dirr * dvt.y);
    bnbu -= mflux * (dirl * dvu.x + dirr * dvu.y);
    const float2 mf = make_float2(mfl, mfr);
    f[0] = mflux;
    const float2 a1 = x2mul(mf, vn), a2 = x2mul(mf, vt), a3 = x2mul(mf, vu);
    const float2 a4 = x2mul(x2mul(mf, bt), roi), a5 = x2mul(x2mul(mf, bu), roi);
    f[1] = a1.x + a1.y + ptot - 0.5f * bnc2;
    f[2] = a2.x + a2.y - bnbt;
    f[3] = a3.x + a3.y - bnbu;
    f[4] = a4.x + a4.y - bnvt;
    f[5] = a5.x + a5.y - bnvu;
    const float2 vb1s = x2fma(vt, bt, x2mul(vu, bu)), vb2s = x2fma(vt2, bt2, x2mul(vu2, bu2));
    const float vb1 = dirl * vb1s.x + dirr * vb1s.y;
    const float vb2 = dirl * vb2s.x + dirr * vb2s.y;
    float rv2b2 = (mflux * vnc - bnc2);
    rv2b2 *= rv2b2;
    float vb3 = 0.f;
    if (rv2b2 > EPS * EPS) {
        vb3 = (+(f[2] * vnc + f[4] * bnc) * (f[2] * bnc + f[4] * mflux)
               + (f[3] * vnc + f[5] * bnc) * (f[3] * bnc + f[5] * mflux)) / rv2b2;
    }
    const float bnvb = sgn * (bnca * (snc * vb2 - vnc * vb1) * (dirl * svci.x + dirr * svci.y)
                              + bnsrv * (vb3 - vb2));
    const float2 a6 = x2mul(mf, hn);
    f[6] = a6.x + a6.y - bnvb;
}

}  // namespace mlau
