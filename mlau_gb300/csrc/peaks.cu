// Arithmetic-pipe throughput probes.  The hot path is bound by FP64 (plain
// mode) or FP32 (split mode) issue, not by HBM or tensor cores, so its roofline
// needs the chip's own FMA rates, measured on the device in use.
#include "sim.cuh"

namespace mlau {
namespace {

constexpr int CHAINS = 8;

template <class T>
__global__ void __launch_bounds__(256) k_fma_probe(T *out, int iters, T a, T b)
{
    T acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++) acc[c] = T(threadIdx.x + c);
    for (int n = 0; n < iters; n++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) acc[c] = fma(acc[c], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < CHAINS; c++) s += acc[c];
    if (s == T(-1.2345)) out[0] = s;  // keeps the loop alive; never true
}

template <class T>
int probe(double *flops, int iters)
{
    int dev = 0, sms = 0;
    MLAU_CUDA(cudaGetDevice(&dev));
    MLAU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    T *out = nullptr;
    MLAU_CUDA(cudaMalloc(&out, sizeof(T)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = sms * 8, threads = 256;
    const T a = T(0.999999), b = T(1e-7);
    k_fma_probe<T><<<blocks, threads>>>(out, iters / 8, a, b);  // warm-up
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(e0);
        k_fma_probe<T><<<blocks, threads>>>(out, iters, a, b);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        best = ms < best ? ms : best;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) {
        set_error("peak probe: %s", cudaGetErrorString(e));
        return MLAU_ERR_CUDA;
    }
    *flops = 2.0 * CHAINS * (double)iters * blocks * threads / (best * 1e-3);
    return MLAU_OK;
}

}  // namespace
}  // namespace mlau

extern "C" int mlau_measure_fma_peaks(double *fp64_flops, double *fp32_flops)
{
    int rc = MLAU_OK;
    if (fp64_flops) rc = mlau::probe<double>(fp64_flops, 4096);
    if (rc == MLAU_OK && fp32_flops) rc = mlau::probe<float>(fp32_flops, 65536);
    return rc;
}
