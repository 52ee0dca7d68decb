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
// smoothness indicators carry a factor 4 and the candidate stencils the 1/8.
#pragma once

#include <cuda_runtime.h>

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
    const float eps = 1e-30f;
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

}  // namespace mlau
