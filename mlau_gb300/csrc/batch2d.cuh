// Shared definitions of the batched engine (batch2d_split.cu,
// batch2d_plain.cu, batch1d_plain.cu, batch2d.cu).
//
// Many independent 2D instances live in pooled per-cell arrays;
// instance n owns cells [base_n, base_n + nx_n*ny_n) of every pool (x fastest,
// `off` ghost cells).  A tile table lists TW x TH cell blocks of the active
// instances.  One persistent cooperative kernel per RK3 step runs every phase
// over the whole table; phases are separated by a grid barrier whose spin has
// an iteration limit (on timeout the kernel records an error and every block
// leaves).  The tile table's pointer and length are read from device memory
// at each launch, so a captured graph stays valid while instances join and
// leave between runs.
#pragma once

#include "sim.cuh"
#include "point.cuh"

namespace mlau {

struct BInst {
    int nx, ny, off, flux;
    int bc, nrk;  // 1D instances only: boundary (MLAU_BC1D_*) and RK stages
    double gamma, cfl;
    double dx, dy;
    double bx;  // 1D instances only: the constant normal field
    double t, t_end, dt_fixed, dt;
    long long base;
    int active, steps;
    int status, pad;  // status: 1 once a NaN or non-positive density/pressure was seen
    unsigned long long vkey;  // order-preserving key of this step's max speed
    // 2D boundary tables (the problem's dnxs / dnys: 0 periodic, -1 Dirichlet,
    // +1 Neumann per variable), walls: some entry is not periodic
    int walls, pad2;
    signed char bcx[8], bcy[8];
};

struct BTile { int inst, x0, y0, pad; };

struct BSync {
    unsigned count, gen;
    int err, active_left;
    int ntiles, fresh;  // fresh: some 1D instance still needs its one-off dt
    BTile *tiles;
    int walls, pad;      // some active 2D instance has non-periodic tables
};

struct BArrays {
    double *s[8], *u0[8];
    // FP32-split workspace
    float2 *q[8];  // ro, vx, vy, vz, cx, cy, bz, pr as (hi, lo)
    float *bf[2], *m2f, *ctf, *dvf[2];
    float *ulf[8], *urf[8], *Ff[2][7], *FCf[2], *ezf;
    // FP64 plain workspace
    double *vx, *vy, *vz, *pr, *m2, *cx, *cy, *ct, *dv[2];
    double *ul[8], *ur[8], *F[2][7], *FC[2], *ez;
};

struct BArgs {
    BArrays a;
    BInst *inst;
    BSync *sync;
    int ninst;
    unsigned nblocks;
    int odr;
};

constexpr long long kBatchSpinLimit = 20000000;  // x ~100 ns sleep: a few seconds

// Grid-wide barrier with a bounded spin.  Returns true when the kernel must
// stop (a block timed out, or another block reported an error).
__device__ __forceinline__ bool grid_barrier(BSync *sy, unsigned nblocks)
{
    __shared__ int stop;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        stop = 0;
        volatile unsigned *vgen = &sy->gen;
        volatile int *verr = &sy->err;
        const unsigned g = *vgen;
        __threadfence();
        if (atomicAdd(&sy->count, 1u) == nblocks - 1) {
            sy->count = 0;
            __threadfence();
            atomicAdd(&sy->gen, 1u);
        } else {
            long long it = 0;
            while (*vgen == g) {
                if (*verr) { stop = 1; break; }
                if (++it > kBatchSpinLimit) {
                    atomicExch(&sy->err, 1);
                    stop = 1;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
        if (*verr) stop = 1;
    }
    __syncthreads();
    return stop != 0;
}

__device__ __forceinline__ int bwrap(int i, int n, int off)
{
    const int N = n - 2 * off;
    return (i < off) ? i + N : ((i >= n - off) ? i - N : i);
}

// Pool index of the boundary source of cell (i, j) of instance I for an
// array with x / y table entries dnx / dny (periodic image or mirror,
// composed over the two axes; the sign into *g), as the 2D driver's bc2d
// (2D/SERIAL/OTvortex/boundary.c:18-74).  stx / sty: face-centred along x / y.
__device__ __forceinline__ long long bsrc(const BInst &I, int i, int j, int stx, int sty, int dnx,
                                          int dny, double *g)
{
    return I.base + (long long)I.nx * bc_src(j, I.ny, I.off, sty, dny, g) +
           bc_src(i, I.nx, I.off, stx, dnx, g);
}

// Visit every cell of every active instance's tiles; body(I, i, j, c).
template <class Body>
__device__ __forceinline__ void for_cells(const BArgs &A, int ntiles, const BTile *tiles, Body body)
{
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const BTile tl = tiles[t];
        const BInst &I = A.inst[tl.inst];
        if (!I.active) continue;
        const int i = tl.x0 + tx, j = tl.y0 + ty;
        if (i >= I.nx || j >= I.ny) continue;
        body(I, i, j, I.base + (long long)I.nx * j + i);
    }
}

// Record a bad cell state (NaN, or density or pressure not positive).
__device__ __forceinline__ void batch_check(BInst &I, double ro, double pr)
{
    if (!(ro > 0.0) || !(pr > 0.0)) atomicOr(&I.status, 1);
}

// dt of every active instance: fixed, or cfl*min(dx,dy)/vmax; clipped to
// land on t_end.  vmax arrives as the order key of a non-negative double.
// An instance whose state went bad retires here, before it steps again.
__device__ __forceinline__ void batch_dt(const BArgs &A)
{
    const int g = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    for (int n = g; n < A.ninst; n += gridDim.x * blockDim.x * blockDim.y) {
        BInst &I = A.inst[n];
        if (!I.active) continue;
        if (I.status) {
            I.active = 0;
            atomicSub(&A.sync->active_left, 1);
            continue;
        }
        double dt = I.dt_fixed;
        if (dt <= 0.0) {
            const double vm = __longlong_as_double((long long)I.vkey);
            dt = (vm > 0.0) ? I.cfl * fmin(I.dx, I.dy) / vm : 0.0;
        }
        if (I.t + dt > I.t_end) dt = I.t_end - I.t;
        I.dt = dt;
    }
}

__device__ __forceinline__ void batch_advance(const BArgs &A)
{
    const int g = blockIdx.x * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x + threadIdx.x;
    for (int n = g; n < A.ninst; n += gridDim.x * blockDim.x * blockDim.y) {
        BInst &I = A.inst[n];
        I.vkey = 0;
        if (!I.active) continue;
        I.t += I.dt;
        I.steps += 1;
        if (I.t >= I.t_end * (1.0 - 1e-12) || !(I.dt > 0.0)) {
            I.active = 0;
            atomicSub(&A.sync->active_left, 1);
        }
    }
}

// Block max of a non-negative speed, folded into the instance's key.
__device__ __forceinline__ void batch_vmax(BInst &I, double vt)
{
    __shared__ double red[32];
    const int lin = threadIdx.y * blockDim.x + threadIdx.x;
    const int lane = lin & 31, wid = lin >> 5, nw = (blockDim.x * blockDim.y) >> 5;
    for (int o = 16; o > 0; o >>= 1) vt = fmax(vt, __shfl_xor_sync(0xffffffffu, vt, o));
    if (lane == 0) red[wid] = vt;
    __syncthreads();
    if (wid == 0) {
        vt = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) vt = fmax(vt, __shfl_xor_sync(0xffffffffu, vt, o));
        if (lane == 0 && vt > 0.0) atomicMax(&I.vkey, (unsigned long long)__double_as_longlong(vt));
    }
    __syncthreads();
}

// Kernel entry points (one per arithmetic), for the host launcher.
const void *batch2d_split_kernel();
const void *batch2d_plain_kernel();
const void *batch1d_plain_kernel();

}  // namespace mlau
