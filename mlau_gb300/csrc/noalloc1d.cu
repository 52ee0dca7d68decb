// Allocation-free 1D step for callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at step time: code
// running inside a host framework that owns every device allocation (a
// caching allocator or a fixed memory pool that must not fragment), a
// long-running service that admits work under a fixed device-memory budget,
// or host code between graph captures that must not change the device memory
// map.  mlau_fd4c_1d_noalloc serves them: it advances one 1D step on arrays
// the caller already has on the device, and keeps its own scratch (the U^n
// copy, primitives, face states and fluxes) in one statically sized device
// array of this file, so it allocates nothing.
#include <mutex>

#include "sim.cuh"

namespace mlau {
int plain1d_enqueue(const PlainFields &f, int nx, int off, int odr, int flux, int nrk, int bc,
                    double bx, double dt, double dx, double gamma, cudaStream_t st);
}

namespace {

constexpr int kMaxNx = MLAU_NOALLOC_1D_MAX_NX;
// u0 (7 x nx) + vx, vy, vz, pr (4 x nx) + face states (14 x (nx+1)) + fluxes
// (7 x nx) + the open boundary's two ghost states (14): 32 nx + 28 doubles
constexpr long long kScratch = 32LL * (kMaxNx + 1);
static_assert(32LL * kMaxNx + 28 <= kScratch, "noalloc scratch too small");

// One array per process and device; it lives until the process exits.
static __device__ __align__(256) double g_noalloc_scratch[kScratch];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for the current device.  In host code
// the symbol g_noalloc_scratch is only a host-side handle, not a device
// address, so it is resolved once per device with cudaGetSymbolAddress while
// that device is current.
int scratch_for_current_device(double **out)
{
    int dev = 0;
    MLAU_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        mlau::set_error("mlau_fd4c_1d_noalloc: device %d out of range", dev);
        return MLAU_ERR_ARG;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            mlau::set_error("mlau_fd4c_1d_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
            return MLAU_ERR_CUDA;
        }
        g_addr[dev] = (double *)p;
    }
    *out = g_addr[dev];
    return MLAU_OK;
}

}  // namespace

extern "C" int mlau_fd4c_1d_noalloc(double *ro, double *mx, double *my, double *mz, double *en,
                                    double *by, double *bz, double bx, double dt, double dx,
                                    int nx, int xoff, double gamma, int odr, int flux, int nrk,
                                    int bc, void *stream)
{
    using namespace mlau;
    if (!ro || !mx || !my || !mz || !en || !by || !bz) {
        set_error("mlau_fd4c_1d_noalloc: null array");
        return MLAU_ERR_ARG;
    }
    if (nx > kMaxNx) {
        set_error("mlau_fd4c_1d_noalloc: nx=%d exceeds the static scratch limit of %d cells "
                  "(use the mlau_sim handle API for larger grids)", nx, kMaxNx);
        return MLAU_ERR_ARG;
    }
    if (xoff < 4 || nx - 2 * xoff < xoff || odr < 1 || odr > 6 || flux < 0 || flux > 3 ||
        nrk < 1 || nrk > 3 || (bc != MLAU_BC1D_OPEN && bc != MLAU_BC1D_PERIODIC) ||
        !(gamma > 1.0) || !(dx > 0)) {
        set_error("mlau_fd4c_1d_noalloc: bad geometry or scheme");
        return MLAU_ERR_ARG;
    }
    double *base = nullptr;
    int rc = scratch_for_current_device(&base);
    if (rc != MLAU_OK) return rc;
    PlainFields f{};
    f.s[0] = ro; f.s[1] = mx; f.s[2] = my; f.s[3] = mz; f.s[4] = en; f.s[6] = by; f.s[7] = bz;
    double *p = base;
    for (int v = 0; v < 8; v++) {
        if (v == 5) continue;
        f.u0[v] = p;
        p += nx;
    }
    f.vx = p; p += nx;
    f.vy = p; p += nx;
    f.vz = p; p += nx;
    f.pr = p; p += nx;
    for (int v = 0; v < 7; v++) { f.ul[v] = p; p += nx + 1; }
    for (int v = 0; v < 7; v++) { f.ur[v] = p; p += nx + 1; }
    for (int v = 0; v < 7; v++) { f.F[0][v] = p; p += nx; }
    f.obc = p;
    return plain1d_enqueue(f, nx, xoff, odr, flux, nrk, bc, bx, dt, dx, gamma,
                           (cudaStream_t)stream);
}
