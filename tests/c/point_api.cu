// Device code written against the reference's point-function signatures
// (include/mhd_flux.h's 25-argument flux type, interp.h's *_cal_flr,
// mhd_eigen.h's mhd_*_reconst taking the drivers' calc_flr), compiled with
// include/mlau_point.h in place of those headers.  Built by
// tests/test_gpu_point_api.py with nvcc --fmad=false (the reference is built
// without contraction) and run on inputs whose reference outputs are stored
// in tests/golden/point_api.npz.  Row layouts: oracle/point_harness.cpp.
#include <cuda_runtime.h>

#include "mlau_point.h"

typedef void (*FluxFn)(double, double, double, double, double, double, double, double, double,
                       double, double, double, double, double, double, double, double *,
                       double *, double *, double *, double *, double *, double *, double *);
typedef void (*LrFn)(const double *, double *, double *);
typedef void (*ReconstFn)(const double *, const double *, const double *, const double *,
                          const double *, const double *, const double *, double, double,
                          const int, double *, double *, LrFn);

// the drivers' calc_flr (3D/MPI/OTvortex/mhd_fd_ct_3d.c:65-78) at ODR 2 and 4
__device__ void calc_flr_2(const double *f, double *fl, double *fr)
{
    muscl_mm_cal_flr(f[1], f[2], f[3], fl, fr);
}
__device__ void calc_flr_4(const double *f, double *fl, double *fr)
{
    wcns4_cal_flr(f[0], f[1], f[2], f[3], f[4], fl, fr);
}

__global__ void k_flux(int which, long n, const double *in, double *out)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    FluxFn func_flux;
    switch (which) {
    case 0: func_flux = &calc_flux_mlau; break;
    case 1: func_flux = &calc_flux_lhlld; break;
    case 2: func_flux = &calc_flux_hlld; break;
    case 3: func_flux = &calc_flux_roe; break;
    default: func_flux = &calc_flux_hl3d2; break;
    }
    const double *q = in + 18 * t;
    double *o = out + 7 * t;
    double dv[2] = {q[16], q[17]};
    func_flux(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7], q[8], q[9], q[10], q[11], q[12],
              q[13], q[14], q[15], dv, o, o + 1, o + 2, o + 3, o + 4, o + 5, o + 6);
}

__global__ void k_interp(int which, long n, const double *in, double *out)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double *f = in + 5 * t;
    double *o = out + 2 * t;
    o[1] = 0.0;
    switch (which) {
    case 0: muscl_mm_cal_flr(f[0], f[1], f[2], o, o + 1); break;
    case 1: muscl_mc_cal_flr(f[0], f[1], f[2], o, o + 1); break;
    case 2: muscl_kr_cal_flr(f[0], f[1], f[2], o, o + 1); break;
    case 3: wcns3_cal_flr(f[0], f[1], f[2], o, o + 1); break;
    case 4: wcns4_cal_flr(f[0], f[1], f[2], f[3], f[4], o, o + 1); break;
    case 5: o[0] = muscl_mm_cal_f(f[0], f[1], f[2]); break;
    case 6: o[0] = muscl_mc_cal_f(f[0], f[1], f[2]); break;
    case 7: o[0] = muscl_kr_cal_f(f[0], f[1], f[2]); break;
    case 8: o[0] = wcns3_cal_f(f[0], f[1], f[2]); break;
    case 9: o[0] = wcns4_cal_f(f[0], f[1], f[2], f[3], f[4]); break;
    case 10: o[0] = minmod(f[0], f[1]); break;
    default: o[0] = minmod3(f[0], f[1], f[2]); break;
    }
}

__global__ void k_reconst(int which, int odr, long n, const double *in, double *out)
{
    const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const LrFn func_lr = (odr == 2) ? &calc_flr_2 : &calc_flr_4;
    ReconstFn rec;
    switch (which) {
    case 0: rec = &mhd_c_reconst; break;
    case 1: rec = &mhd_m_reconst; break;
    case 2: rec = &mhd_a_reconst; break;
    default: rec = &mhd_reconst; break;
    }
    const double *q = in + 37 * t;
    double *o = out + 14 * t;
    rec(q, q + 5, q + 10, q + 15, q + 20, q + 25, q + 30, q[35], q[36], 5, o, o + 7, func_lr);
}

// kind 0 flux, 1 interp, 2 reconst (odr 2 or 4); returns a cudaError_t.
extern "C" int point_api_run(int kind, int which, int odr, long n, const double *in, double *out)
{
    const int win[3] = {18, 5, 37}, wout[3] = {7, 2, 14};
    if (kind < 0 || kind > 2 || n <= 0) return (int)cudaErrorInvalidValue;
    double *d_in = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_in, sizeof(double) * win[kind] * n);
    if (e == cudaSuccess) e = cudaMalloc(&d_out, sizeof(double) * wout[kind] * n);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_in, in, sizeof(double) * win[kind] * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int b = 128;
        const long g = (n + b - 1) / b;
        if (kind == 0) k_flux<<<g, b>>>(which, n, d_in, d_out);
        else if (kind == 1) k_interp<<<g, b>>>(which, n, d_in, d_out);
        else k_reconst<<<g, b>>>(which, odr, n, d_in, d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d_out, sizeof(double) * wout[kind] * n, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_out);
    return (int)e;
}
