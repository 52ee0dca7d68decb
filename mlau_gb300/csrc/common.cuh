// Shared host/device helpers of the GB300 MHD step library.
#pragma once

#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/mlau_gb300.h"

namespace mlau {

// Last error message, per host thread (mlau_last_error()).
void set_error(const char *fmt, ...);

#define MLAU_CUDA(call)                                                              \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            ::mlau::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call,            \
                              cudaGetErrorString(e_));                               \
            return MLAU_ERR_CUDA;                                                    \
        }                                                                            \
    } while (0)

// Periodic image of a padded index along one axis: ghosts [0,off) and
// [n-off,n) map onto the interior [off, n-off) (interior width n-2*off >= off).
__host__ __device__ __forceinline__ int wrap_idx(int i, int n, int off)
{
    const int N = n - 2 * off;
    return (i < off) ? i + N : ((i >= n - off) ? i - N : i);
}

// Source of a possibly-ghost index along one axis under the reference's
// boundary rule for one array (bc2d, 2D/SERIAL/OTvortex/boundary.c:18-74):
// dn 0 periodic image; dn -1 (Dirichlet) / +1 (Neumann) mirror about the
// boundary, multiplying *sgn by dn.  st 1 marks a face-centred array along
// the axis: its right boundary face n-off is a computed value, not a ghost.
__host__ __device__ __forceinline__ int bc_src(int i, int n, int off, int st, int dn, double *sgn)
{
    if (dn == 0) return wrap_idx(i, n, off);
    if (i < off) { *sgn *= dn; return (2 * off - 1 + st) - i; }
    if (i >= n - off + st) { *sgn *= dn; return (n - 2 * off + st) + (n - 1 - i); }
    return i;
}

// Boundary tables of a 2D problem (the problem's dnxs/dnys, variable order
// ro mx my mz en bx by bz); all zero = periodic.
struct Bc2 {
    int x[8], y[8];
};

// Boundary tables of a 3D problem (dnxs/dnys/dnzs, same order).
struct Bc3 {
    int x[8], y[8], z[8];
};

// Kernel-kind identifiers for the optional per-kernel event timing.
enum KernelKind {
    KK_PRIM = 0, KK_AUX, KK_REC, KK_FLUX, KK_EMF, KK_UPDATE, KK_COPY, KK_CFL,
    KK_SPLIT_SWEEP, KK_SPLIT_PREP, KK_SPLIT_UPDATE, KK_COUNT
};

// Records a CUDA event pair around each launch when enabled.
struct KernelTimer {
    bool on = false;
    cudaStream_t stream = nullptr;
    struct Rec { int kind; cudaEvent_t a, b; };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    double total_ms[KK_COUNT] = {0};
    long count[KK_COUNT] = {0};

    cudaEvent_t ev();
    void begin(int kind, cudaEvent_t &a);
    void end(int kind, cudaEvent_t a);
    int flush();  // synchronize, accumulate, recycle events
    void reset();
    ~KernelTimer();
};

struct TimedLaunch {
    KernelTimer *t;
    int kind;
    cudaEvent_t a = nullptr;
    TimedLaunch(KernelTimer *t_, int k) : t(t_), kind(k) { if (t && t->on) t->begin(kind, a); }
    ~TimedLaunch() { if (t && t->on) t->end(kind, a); }
};

inline unsigned blocks_for(long long n, int threads)
{
    return (unsigned)((n + threads - 1) / threads);
}

}  // namespace mlau
