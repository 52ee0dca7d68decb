// Checkpoint and output files in the reference's formats, written from and
// read into a device-resident simulation, so that runs restart across the CPU
// reference and this library and the reference's readers consume GPU output.
//
//   checkpoint (3D/MPI/OTvortex/bkup.hpp:4-76, same in 2D/MPI):
//     <dir>/bkup_stamp.dat            text "%d %d\n" (step, output count), rank 0
//     <dir>/bkup_time.dat             3 raw doubles (time, dt, next output time), rank 0
//     <dir>/bkup_data_%05d.dat        raw FP64 ro, mx, my, mz, bx, by, bz, en (whole
//                                     padded arrays, ghosts included), per rank
//   output (MLAU_OUT_F32_RANK: 3D/MPI/OTvortex/dataio.hpp:62-80, 2D/MPI):
//     <dir>/outdat_%05d_%05d.dat      FP32 ro, mx, my, mz, en, bx, by, bz (cnt, rank)
//   output (MLAU_OUT_F64: 2D/SERIAL/OTvortex/dataio.hpp:28-38; 1D
//     1D/SERIAL/shock/main.cpp:136-147,171-184):
//     <dir>/outdat_%05d.dat           FP64 ro, mx, my, mz, en, bx, by, bz
//                                     (1D: ro, mx, my, mz, en, by, bz)
//   plus the run's metadata text files (params.dat, offsets.dat / xoff.dat,
//   t.dat) as the same routines write them at the first output.
//
// FP32 output is converted on the device (round to nearest, as the
// reference's (float) cast) so that half the bytes cross to the host.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>

#include "sim.cuh"

using namespace mlau;

struct mlau_sim : public Sim {};

namespace {

__global__ void k_d2f(const double *in, float *out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(in[i]);
}

// Host staging buffer (pinned) released on scope exit.
struct Pinned {
    void *p = nullptr;
    explicit Pinned(size_t bytes) { if (cudaMallocHost(&p, bytes) != cudaSuccess) p = nullptr; }
    ~Pinned() { if (p) cudaFreeHost(p); }
};

struct File {
    FILE *f = nullptr;
    File(const std::string &path, const char *mode) { f = std::fopen(path.c_str(), mode); }
    ~File() { if (f) std::fclose(f); }
};

std::string path_of(const char *dir, const char *fmt, int a = -1, int b = -1)
{
    char name[64];
    if (b >= 0) std::snprintf(name, sizeof(name), fmt, a, b);
    else if (a >= 0) std::snprintf(name, sizeof(name), fmt, a);
    else std::snprintf(name, sizeof(name), "%s", fmt);
    return std::string(dir) + "/" + name;
}

int open_err(const std::string &p)
{
    set_error("cannot open %s: %s", p.c_str(), std::strerror(errno));
    return MLAU_ERR_ARG;
}

// Device -> host -> file for the listed state slots, FP64 or FP32.
int write_arrays(Sim *s, FILE *f, const int *slots, int nslots, bool fp32)
{
    const long long n = s->g.n;
    const size_t esz = fp32 ? sizeof(float) : sizeof(double);
    Pinned host(esz * n);
    if (!host.p) { set_error("pinned staging buffer of %lld bytes", (long long)(esz * n)); return MLAU_ERR_NOMEM; }
    float *dev = nullptr;
    if (fp32) MLAU_CUDA(cudaMalloc(&dev, sizeof(float) * n));
    int rc = MLAU_OK;
    for (int k = 0; k < nslots && rc == MLAU_OK; k++) {
        const double *src = s->f.s[slots[k]];
        cudaError_t e;
        if (fp32) {
            k_d2f<<<1024, 256, 0, s->stream>>>(src, dev, n);
            e = cudaMemcpyAsync(host.p, dev, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream);
        } else {
            e = cudaMemcpyAsync(host.p, src, sizeof(double) * n, cudaMemcpyDeviceToHost, s->stream);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            set_error("output copy: %s", cudaGetErrorString(e));
            rc = MLAU_ERR_CUDA;
        } else if (std::fwrite(host.p, esz, (size_t)n, f) != (size_t)n) {
            set_error("short write");
            rc = MLAU_ERR_ARG;
        }
    }
    if (dev) cudaFree(dev);
    return rc;
}

int check_sim(Sim *s, const char *dir, bool dim23)
{
    if (!s || !dir) { set_error("null argument"); return 0; }
    if (dim23 && s->g.dim == 1) { set_error("the reference's checkpoint exists for 2D and 3D only"); return 0; }
    return 1;
}

}  // namespace

extern "C" {

int mlau_sim_bkup_save(mlau_sim *s, const char *dir, int n, int cnt, double tim, double dt,
                       double trec, int rank)
{
    if (!check_sim(s, dir, true) || rank < 0) return MLAU_ERR_ARG;
    MLAU_CUDA(cudaStreamSynchronize(s->stream));
    if (rank == 0) {
        const std::string ps = path_of(dir, "bkup_stamp.dat");
        File st(ps, "w");
        if (!st.f) return open_err(ps);
        std::fprintf(st.f, "%d %d\n", n, cnt);
        const std::string pt = path_of(dir, "bkup_time.dat");
        File ft(pt, "wb");
        if (!ft.f) return open_err(pt);
        const double v[3] = {tim, dt, trec};
        if (std::fwrite(v, sizeof(double), 3, ft.f) != 3) { set_error("short write"); return MLAU_ERR_ARG; }
    }
    const std::string pd = path_of(dir, "bkup_data_%05d.dat", rank);
    File fd(pd, "wb");
    if (!fd.f) return open_err(pd);
    static const int order[8] = {0, 1, 2, 3, 5, 6, 7, 4};  // ro mx my mz bx by bz en
    return write_arrays(s, fd.f, order, 8, false);
}

int mlau_sim_bkup_load(mlau_sim *s, const char *dir, int *n, int *cnt, double *tim, double *dt,
                       double *trec, int rank)
{
    if (!check_sim(s, dir, true) || rank < 0) return MLAU_ERR_ARG;
    const std::string ps = path_of(dir, "bkup_stamp.dat");
    File st(ps, "r");
    if (!st.f) return 1;  // no checkpoint: nothing loaded, as the reference
    int vi[2];
    if (std::fscanf(st.f, "%d %d", &vi[0], &vi[1]) != 2) { set_error("malformed %s", ps.c_str()); return MLAU_ERR_ARG; }
    const std::string pt = path_of(dir, "bkup_time.dat");
    File ft(pt, "rb");
    double vd[3];
    if (!ft.f) return open_err(pt);
    if (std::fread(vd, sizeof(double), 3, ft.f) != 3) { set_error("short read of %s", pt.c_str()); return MLAU_ERR_ARG; }
    const std::string pd = path_of(dir, "bkup_data_%05d.dat", rank);
    File fd(pd, "rb");
    if (!fd.f) return open_err(pd);
    const long long nn = s->g.n;
    Pinned host(sizeof(double) * nn);
    if (!host.p) { set_error("pinned staging buffer"); return MLAU_ERR_NOMEM; }
    static const int order[8] = {0, 1, 2, 3, 5, 6, 7, 4};
    for (int k = 0; k < 8; k++) {
        if (std::fread(host.p, sizeof(double), (size_t)nn, fd.f) != (size_t)nn) {
            set_error("%s holds fewer than 8 arrays of %lld cells", pd.c_str(), nn);
            return MLAU_ERR_ARG;
        }
        MLAU_CUDA(cudaMemcpyAsync(s->f.s[order[k]], host.p, sizeof(double) * nn,
                                  cudaMemcpyHostToDevice, s->stream));
        MLAU_CUDA(cudaStreamSynchronize(s->stream));
    }
    if (n) *n = vi[0];
    if (cnt) *cnt = vi[1];
    if (tim) *tim = vd[0];
    if (dt) *dt = vd[1];
    if (trec) *trec = vd[2];
    return MLAU_OK;
}

int mlau_sim_outdat(mlau_sim *s, const char *dir, int cnt, int rank, int format)
{
    if (!check_sim(s, dir, false) || cnt < 0) return MLAU_ERR_ARG;
    MLAU_CUDA(cudaStreamSynchronize(s->stream));
    static const int all8[8] = {0, 1, 2, 3, 4, 5, 6, 7};  // ro mx my mz en bx by bz
    static const int d1[7] = {0, 1, 2, 3, 4, 6, 7};       // ro mx my mz en by bz
    if (format == MLAU_OUT_F32_RANK) {
        if (s->g.dim == 1 || rank < 0) { set_error("FP32 per-rank output is the 2D/3D MPI format"); return MLAU_ERR_ARG; }
        const std::string p = path_of(dir, "outdat_%05d_%05d.dat", cnt, rank);
        File f(p, "wb");
        if (!f.f) return open_err(p);
        return write_arrays(s, f.f, all8, 8, true);
    }
    if (format == MLAU_OUT_F64) {
        const std::string p = path_of(dir, "outdat_%05d.dat", cnt);
        File f(p, "wb");
        if (!f.f) return open_err(p);
        return s->g.dim == 1 ? write_arrays(s, f.f, d1, 7, false)
                             : write_arrays(s, f.f, all8, 8, false);
    }
    set_error("unknown output format %d", format);
    return MLAU_ERR_ARG;
}

int mlau_outdat_meta(const char *dir, int dim, int first, double tim, double gamma, double bx,
                     int xoff, int yoff, int zoff)
{
    if (!dir || dim < 1 || dim > 3) { set_error("bad arguments"); return MLAU_ERR_ARG; }
    if (first) {
        const std::string pp = path_of(dir, "params.dat");
        File fp(pp, "w");
        if (!fp.f) return open_err(pp);
        if (dim == 1) std::fprintf(fp.f, "%.12f %.12f\n", bx, gamma);
        else std::fprintf(fp.f, "%f\n", gamma);
        const std::string po = path_of(dir, dim == 1 ? "xoff.dat" : "offsets.dat");
        File fo(po, "w");
        if (!fo.f) return open_err(po);
        if (dim == 1) std::fprintf(fo.f, "%d\n", xoff);
        else if (dim == 2) std::fprintf(fo.f, "%d %d\n", xoff, yoff);
        else std::fprintf(fo.f, "%d %d %d\n", xoff, yoff, zoff);
    }
    const std::string pt = path_of(dir, "t.dat");
    File ft(pt, first ? "w" : "a");
    if (!ft.f) return open_err(pt);
    if (dim == 1) std::fprintf(ft.f, "%.12f\n", tim);
    else std::fprintf(ft.f, "%f\n", tim);
    return MLAU_OK;
}

}  // extern "C"
