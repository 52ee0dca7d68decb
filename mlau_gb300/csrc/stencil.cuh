// Device helpers shared by the plain FP64 step kernels (1D, 2D, 3D).
#pragma once

#include "sim.cuh"
#include "point.cuh"

namespace mlau {
namespace {

constexpr int TPB = 128;

struct Box {
    int lo0, lo1, lo2, e0, e1, e2;
    __device__ __forceinline__ bool decode(long long t, int &i, int &j, int &k) const
    {
        long long tot = (long long)e0 * e1 * e2;
        if (t >= tot) return false;
        int a = (int)(t % e0);
        long long r = t / e0;
        int b = (int)(r % e1);
        int c = (int)(r / e1);
        i = lo0 + a;
        j = lo1 + b;
        k = lo2 + c;
        return true;
    }
    long long count() const { return (long long)e0 * e1 * e2; }
};

struct Dims {
    int nx, ny, nz, ox, oy, oz;
    __device__ __forceinline__ long long at(int i, int j, int k) const
    {
        return (long long)nx * ((long long)ny * k + j) + i;
    }
};

// ---------------------------------------------------------------------------
// Alfven-upwind weight of one edge from the 4 surrounding cells, summed in
// the reference's order (s-P-Q, s-P, s-Q, s); face B averaged with the cell
// offset oa (first axis) and ob (second axis).  mhd_fd_ct_3d.c:277-289.
__device__ __forceinline__ double ct_weight(const double *va, const double *vb, const double *ro,
                                            const double *ba, const double *bbf, long long s,
                                            long long P, long long Q, long long oa, long long ob)
{
    const double eps = 1e-6;
    double a = 0.25 * (va[s - P - Q] + va[s - P] + va[s - Q] + va[s]);
    double c = 0.25 * (vb[s - P - Q] + vb[s - P] + vb[s - Q] + vb[s]);
    double rc = 0.25 * (ro[s - P - Q] + ro[s - P] + ro[s - Q] + ro[s]);
    rc = 1.0 / sqrt(rc);
    double fa = 0.5 * (ba[s - oa] + ba[s]);
    double fb = 0.5 * (bbf[s - ob] + bbf[s]);
    a = fabs(a) + fabs(fa * rc);
    c = fabs(c) + fabs(fb * rc);
    return (a + 0.5 * eps) / (a + c + eps);
}

// One edge contribution: sgn*0.5*((ul0+ur0) + w*(ul1+ur1)) with ul from the
// linear interpolation centred one edge below and ur centred on the edge.
__device__ __forceinline__ double emf_part(const double *fu, const double *fc, double w,
                                           double sgn, long long c, long long st, int odr)
{
    const double ul0 = lin_l(odr, fu[c - 3 * st], fu[c - 2 * st], fu[c - st], fu[c], fu[c + st]);
    const double ul1 = lin_l(odr, fc[c - 3 * st], fc[c - 2 * st], fc[c - st], fc[c], fc[c + st]);
    const double ur0 = lin_r(odr, fu[c - 2 * st], fu[c - st], fu[c], fu[c + st], fu[c + 2 * st]);
    const double ur1 = lin_r(odr, fc[c - 2 * st], fc[c - st], fc[c], fc[c + st], fc[c + 2 * st]);
    return sgn * 0.5 * ((ul0 + ur0) + w * (ul1 + ur1));
}

inline void rk_coef(int nrk, int stage, double &a, double &b)
{
    const double t[3][2] = {{0.0, 1.0},
                            {0.5 + (nrk - 2) * 0.25, 0.5 - (nrk - 2) * 0.25},
                            {1. / 3., 2. / 3.}};
    a = t[stage][0];
    b = t[stage][1];
}

}  // namespace
}  // namespace mlau
