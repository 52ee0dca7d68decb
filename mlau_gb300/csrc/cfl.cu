// CFL maximum-speed reduction on the device: the GPU form of the reference's
// cflcheck (3D/MPI/OTvortex/cflcheck.hpp:1-39, 2D/SERIAL/OTvortex/
// cflcheck.hpp:1-32) and of the 1D one-off dt (1D/SERIAL/shock/main.cpp:113-128).
// Each thread evaluates one cell's fast speed; warp shuffles and a shared
// array reduce a block, and one 64-bit atomicMax per block folds the block
// maxima.  A maximum is exact and order-independent, so the result equals the
// reference's serial loop (NaN cells never win there, and never win here).
#include "stencil.cuh"

namespace mlau {
namespace {

// Order-preserving map of non-NaN doubles onto unsigned 64-bit integers.
__device__ __forceinline__ unsigned long long ord_enc(double x)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__host__ __device__ inline double ord_dec(unsigned long long u)
{
    unsigned long long b = (u >> 63) ? (u & 0x7fffffffffffffffULL) : ~u;
    double x;
    memcpy(&x, &b, sizeof(x));
    return x;
}

__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <int DIM>
__global__ void __launch_bounds__(256)
k_cfl(const PlainFields f, Dims d, Box b, double gamma, double bx1d, unsigned long long *out)
{
    __shared__ double red[8];
    int i, j, k;
    double vt = -INFINITY;
    if (b.decode((long long)blockIdx.x * blockDim.x + threadIdx.x, i, j, k)) {
        const long long s = d.at(i, j, k);
        const double ro = f.s[0][s];
        const double iro = 1.0 / ro;
        const double vx = f.s[1][s] * iro, vy = f.s[2][s] * iro, vz = f.s[3][s] * iro;
        const double v2 = vx * vx + vy * vy + vz * vz;
        if (DIM == 1) {
            const double b2 = bx1d * bx1d + f.s[6][s] * f.s[6][s] + f.s[7][s] * f.s[7][s];
            const double pr = (gamma - 1) * (f.s[4][s] - 0.5 * (ro * v2 + b2));
            const double cf = sqrt((gamma * pr + b2) * iro);
            vt = fabs(vx) + cf;
        } else {
            const double bxc = 0.5 * (f.s[5][s] + f.s[5][s + 1]);
            const double byc = 0.5 * (f.s[6][s] + f.s[6][s + d.nx]);
            const double bzc = (DIM == 3) ? 0.5 * (f.s[7][s] + f.s[7][s + (long long)d.nx * d.ny])
                                          : f.s[7][s];
            const double b2 = bxc * bxc + byc * byc + bzc * bzc;
            const double pr = (gamma - 1) * (f.s[4][s] - 0.5 * (ro * v2 + b2));
            const double cf = sqrt((0.5 * gamma * (2.0 * pr) + b2) / (ro));
            vt = ((DIM == 3) ? sqrt(v2) : sqrt(vx * vx + vy * vy)) + cf;
        }
        if (vt != vt) vt = -INFINITY;  // NaN never becomes the maximum
    }
    vt = warp_max(vt);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = vt;
    __syncthreads();
    if (wid == 0) {
        vt = (lane < (int)(blockDim.x >> 5)) ? red[lane] : -INFINITY;
        vt = warp_max(vt);
        if (lane == 0) atomicMax(out, ord_enc(vt));
    }
}

}  // namespace

int cfl_compute(Sim *s, double *vmax_out)
{
    const Geometry &g = s->g;
    const Dims d{g.nx, g.ny, g.nz, g.ox, g.oy, g.oz};
    unsigned long long *acc = (unsigned long long *)s->d_red;
    // -inf encodes to the smallest key of any non-NaN double
    double ninf = -INFINITY;
    unsigned long long b;
    memcpy(&b, &ninf, sizeof(b));
    const unsigned long long init = ~b;
    MLAU_CUDA(cudaMemcpyAsync(acc, &init, sizeof(init), cudaMemcpyHostToDevice, s->stream));
    {
        TimedLaunch tl(&s->timer, KK_CFL);
        if (g.dim == 3) {
            Box bx{g.ox, g.oy, g.oz, g.nx - 2 * g.ox, g.ny - 2 * g.oy, g.nz - 2 * g.oz};
            k_cfl<3><<<blocks_for(bx.count(), 256), 256, 0, s->stream>>>(s->f, d, bx, s->gamma, 0.0, acc);
        } else if (g.dim == 2) {
            Box bx{g.ox, g.oy, 0, g.nx - 2 * g.ox, g.ny - 2 * g.oy, 1};
            k_cfl<2><<<blocks_for(bx.count(), 256), 256, 0, s->stream>>>(s->f, d, bx, s->gamma, 0.0, acc);
        } else {
            Box bx{0, 0, 0, g.nx, 1, 1};  // the 1D dt scans every cell, ghosts included
            k_cfl<1><<<blocks_for(bx.count(), 256), 256, 0, s->stream>>>(s->f, d, bx, s->gamma,
                                                                         s->bx1d, acc);
        }
    }
    MLAU_CUDA(cudaGetLastError());
    unsigned long long h = 0;
    MLAU_CUDA(cudaMemcpyAsync(&h, acc, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
    MLAU_CUDA(cudaStreamSynchronize(s->stream));
    *vmax_out = ord_dec(h);
    return MLAU_OK;
}

}  // namespace mlau
