// Internal simulation object behind the mlau_sim handle.
#pragma once

#include "common.cuh"

namespace mlau {

// Device fields of the plain FP64 step, one padded array each.
struct PlainFields {
    double *s[8];        // state ro, mx, my, mz, en, bx, by, bz
    double *u0[8];       // copy of the state at the start of the step (U^n)
    double *vx, *vy, *vz, *pr, *m2, *cx, *cy, *cz;
    double *dv[3];       // shock sensors dvx, dvy, dvz
    double *ct[3];       // CT Alfven-upwind weights at x-y (ct0), y-z (ct1), z-x (ct2) edges
    double *ul[7], *ur[7];     // face states (ro, vn, vt, vu, bt, bu, pr)
    double *ql[2], *qr[2];     // linear central parts of the two tangential B fluxes
    double *F[3][7];     // face fluxes per direction: (ro, mn, mt, mu, bt, bu, en)
    double *FC[3][2];    // central parts of the bt and bu fluxes
    double *e[3];        // edge EMFs ex, ey, ez
    double *obc;         // 1D open boundary: each side's ghost state (ro, mx, my, mz, by, bz, en)
};

struct Geometry {
    int dim;
    int nx, ny, nz, ox, oy, oz;
    long long n;  // nx*ny*nz
    double dx, dy, dz;
};

struct SplitFields;  // FP32-split workspace (split3d.cu)

// The two FP32-split forms share the workspace and the kernels.
inline bool is_split(int precision)
{
    return precision == MLAU_FP32_SPLIT || precision == MLAU_FP32_SPLIT_F64;
}

struct Sim {
    Geometry g;
    double gamma;
    int odr, flux, nrk, precision;
    int eig = 0;         // eigen-system where Mach^2 >= 1: 0 full 7-wave, 1 Miyoshi
    int bc1d = MLAU_BC1D_OPEN;
    double bx1d = 0.0;
    Bc2 bc2{};           // 2D boundary tables (all zero: periodic)
    bool walls2d = false;  // some 2D table entry is not periodic
    Bc3 bc3{};           // 3D boundary tables (all zero: periodic)
    bool walls3d = false;  // some 3D table entry is not periodic
    cudaStream_t stream = nullptr;
    // 1D open boundary: a second stream and fork / join events, so that the
    // boundary's serial chain runs beside the first stage's kernels
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    PlainFields f{};
    SplitFields *sp = nullptr;
    std::vector<void *> allocs;
    long long bytes = 0;
    double *d_red = nullptr;   // device scratch for reductions (2 doubles)
    int *d_flag = nullptr;     // device status flag
    KernelTimer timer;
    // steps replayed from a captured CUDA graph (small problems are launch bound)
    cudaGraphExec_t gexec = nullptr;
    double graph_dt = 0.0;
    int graph_steps = 0;
    // anisotropic conduction: device convergence state with its pinned host
    // copy, and the captured graph of a run of Gauss-Seidel sweeps with the
    // parameters it was captured for
    void *d_cond = nullptr;
    void *h_cond = nullptr;
    cudaGraphExec_t cond_exec = nullptr;
    long long cond_key = -1;
};

int plain3d_alloc(Sim *s);
int plain3d_step(Sim *s, double dt);
int plain2d_alloc(Sim *s);
int plain2d_step(Sim *s, double dt);
int plain1d_alloc(Sim *s);
int plain1d_step(Sim *s, double dt);
int split3d_alloc(Sim *s);
int split3d_step(Sim *s, double dt);
// one step of a state in host arrays (in place), copies overlapped with the step
int split3d_step_host(Sim *s, double dt, double *const *h);
void split3d_free(Sim *s);
int split3d_check(Sim *s);
int diff2d_resistive(Sim *s, double eta0, double dt);
int diff2d_viscous(Sim *s, double nu0, double dt);
int diff2d_conduction(Sim *s, double kk0, double dt, int *sweeps);
int diff2d_inject(Sim *s, double ro3, double dro3, double vy1, double bx1, double by1, double bz1,
                  double pr1, double vref, const double *noise);
void diff2d_free(Sim *s);
int cfl_compute(Sim *s, double *vmax_out);
int launches_per_step(const Sim *s);

// Allocate one padded array per call; recorded for release at destroy.
int dalloc(Sim *s, double **p, long long count);

}  // namespace mlau
