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
