// Host side of the batched 2D engine (kernels: batch2d_split.cu,
// batch2d_plain.cu; shared definitions: batch2d.cuh).
//
// Instances occupy slots; their cells are carved from fixed-capacity pools by
// a first-fit allocator, so instances can join and leave between runs
// (continuous batching).  The tile table lives in device memory and the
// kernel reads its address and length at every launch, so a captured step
// graph survives membership changes.
#include <algorithm>
#include <cstring>
#include <map>
#include <vector>

#include "batch2d.cuh"

using namespace mlau;

struct mlau_batch {
    int dim = 2;
    int precision = MLAU_FP32_SPLIT, odr = 4, off = 4;
    int max_inst = 0;
    long long capacity = 0;
    std::vector<BInst> h_inst;
    std::vector<char> used;
    std::map<long long, long long> free_;  // start -> length (cells)
    BInst *d_inst = nullptr;
    BSync *d_sync = nullptr;
    BSync *h_sync = nullptr;
    BTile *d_tiles = nullptr;
    long long tiles_cap = 0;
    int ntiles = 0, tw = 32, th = 8;
    bool tiles_dirty = true;
    BArrays a{};
    std::vector<void *> allocs;
    long long bytes = 0;
    cudaStream_t stream = nullptr;
    unsigned nblocks = 0, max_blocks = 0, want_blocks = 0;  // want 0: all co-resident blocks
    cudaGraphExec_t gexec = nullptr;
    int graph_steps = 0;
    long long launches = 0;
    const void *kernel = nullptr;
};

namespace {

int balloc(mlau_batch *b, void **p, size_t bytes)
{
    cudaError_t e = cudaMalloc(p, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("batch: cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        return MLAU_ERR_NOMEM;
    }
    b->allocs.push_back(*p);
    b->bytes += (long long)bytes;
    return MLAU_OK;
}

long long carve(mlau_batch *b, long long n)
{
    for (auto it = b->free_.begin(); it != b->free_.end(); ++it) {
        if (it->second >= n) {
            const long long base = it->first, rest = it->second - n;
            b->free_.erase(it);
            if (rest > 0) b->free_[base + n] = rest;
            return base;
        }
    }
    return -1;
}

void release(mlau_batch *b, long long base, long long n)
{
    auto it = b->free_.emplace(base, n).first;
    auto nx = std::next(it);
    if (nx != b->free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        b->free_.erase(nx);
    }
    if (it != b->free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
            pv->second += it->second;
            b->free_.erase(it);
        }
    }
}

// The engine's stream has the highest priority: while blocks of its
// persistent kernel are still waiting for room, the block scheduler places
// them before blocks of ordinary kernels from other streams.
cudaError_t make_stream(cudaStream_t *st)
{
    int least = 0, greatest = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e != cudaSuccess) return e;
    return cudaStreamCreateWithPriority(st, cudaStreamNonBlocking, greatest);
}

int occupancy(mlau_batch *b)
{
    int dev = 0, sms = 0, per_sm = 0;
    MLAU_CUDA(cudaGetDevice(&dev));
    MLAU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MLAU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->kernel, b->tw * b->th, 0));
    if (per_sm < 1) { set_error("batch: step kernel does not fit on an SM"); return MLAU_ERR_ARG; }
    b->max_blocks = (unsigned)(sms * per_sm);
    b->nblocks = b->want_blocks ? std::min(b->want_blocks, b->max_blocks) : b->max_blocks;
    return MLAU_OK;
}

// Rebuild the tile table of the occupied slots (round-robin over instances so
// neighbouring blocks work on different instances).
int build_tiles(mlau_batch *b)
{
    std::vector<std::vector<BTile>> per;
    for (int n = 0; n < b->max_inst; n++) {
        if (!b->used[n] || !b->h_inst[n].active) continue;
        const BInst &I = b->h_inst[n];
        per.emplace_back();
        for (int y = 0; y < I.ny; y += b->th)
            for (int x = 0; x < I.nx; x += b->tw) per.back().push_back({n, x, y, 0});
    }
    std::vector<BTile> tiles;
    for (size_t k = 0;; k++) {
        bool more = false;
        for (auto &p : per)
            if (k < p.size()) { tiles.push_back(p[k]); more = true; }
        if (!more) break;
    }
    if ((long long)tiles.size() > b->tiles_cap) {
        if (b->d_tiles) {
            cudaFree(b->d_tiles);
            b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)b->d_tiles));
        }
        b->tiles_cap = (long long)tiles.size() * 2 + 64;
        int rc = balloc(b, (void **)&b->d_tiles, sizeof(BTile) * b->tiles_cap);
        if (rc) return rc;
    }
    if (!tiles.empty())
        MLAU_CUDA(cudaMemcpyAsync(b->d_tiles, tiles.data(), sizeof(BTile) * tiles.size(),
                                  cudaMemcpyHostToDevice, b->stream));
    b->ntiles = (int)tiles.size();
    b->tiles_dirty = false;
    return MLAU_OK;
}

BArgs make_args(mlau_batch *b)
{
    BArgs A;
    A.a = b->a;
    A.inst = b->d_inst;
    A.sync = b->d_sync;
    A.ninst = b->max_inst;
    A.nblocks = b->nblocks;
    A.odr = b->odr;
    return A;
}

int launch_step(mlau_batch *b)
{
    BArgs A = make_args(b);
    void *params[] = {&A};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->nblocks);
    cfg.blockDim = dim3(b->tw, b->th);
    cfg.stream = b->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    MLAU_CUDA(cudaLaunchKernelExC(&cfg, b->kernel, params));
    return MLAU_OK;
}

// Push the instance table, tile table and a fresh status word.
int push_table(mlau_batch *b)
{
    if (b->tiles_dirty) {
        int rc = build_tiles(b);
        if (rc) return rc;
    }
    MLAU_CUDA(cudaMemcpyAsync(b->d_inst, b->h_inst.data(), sizeof(BInst) * b->max_inst,
                              cudaMemcpyHostToDevice, b->stream));
    BSync s0{};
    for (int n = 0; n < b->max_inst; n++) {
        const BInst &I = b->h_inst[n];
        if (!b->used[n] || !I.active) continue;
        s0.active_left++;
        if (b->dim == 1 && I.steps == 0 && !(I.dt_fixed > 0.0)) s0.fresh = 1;
        if (b->dim == 2 && I.walls) s0.walls = 1;
    }
    s0.ntiles = b->ntiles;
    s0.tiles = b->d_tiles;
    *b->h_sync = s0;
    MLAU_CUDA(cudaMemcpyAsync(b->d_sync, b->h_sync, sizeof(BSync), cudaMemcpyHostToDevice,
                              b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    return MLAU_OK;
}

int pull_table(mlau_batch *b)
{
    MLAU_CUDA(cudaMemcpyAsync(b->h_inst.data(), b->d_inst, sizeof(BInst) * b->max_inst,
                              cudaMemcpyDeviceToHost, b->stream));
    MLAU_CUDA(cudaMemcpyAsync(b->h_sync, b->d_sync, sizeof(BSync), cudaMemcpyDeviceToHost,
                              b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    if (b->h_sync->err) {
        set_error("batch: a grid barrier gave up waiting (device timeout)");
        return MLAU_ERR_TIMEOUT;
    }
    return MLAU_OK;
}

int make_graph(mlau_batch *b, int steps)
{
    if (b->gexec && b->graph_steps == steps) return MLAU_OK;
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    cudaGraph_t g;
    MLAU_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = MLAU_OK;
    for (int k = 0; k < steps && rc == MLAU_OK; k++) rc = launch_step(b);
    cudaMemcpyAsync(b->h_sync, b->d_sync, sizeof(BSync), cudaMemcpyDeviceToHost, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != MLAU_OK) return rc;
    if (e != cudaSuccess) {
        set_error("batch: graph capture: %s", cudaGetErrorString(e));
        return MLAU_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&b->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        set_error("batch: graph instantiate: %s", cudaGetErrorString(e));
        return MLAU_ERR_CUDA;
    }
    b->graph_steps = steps;
    return MLAU_OK;
}

int check_inst(mlau_batch *b, int n)
{
    if (!b || n < 0 || n >= b->max_inst || !b->used[n]) {
        set_error("batch: slot %d is not in use", n);
        return 0;
    }
    return 1;
}

}  // namespace

extern "C" {

int mlau_batch_open(mlau_batch **out, int precision, long long capacity_cells, int max_inst,
                    int off, int odr)
{
    if (!out || capacity_cells <= 0 || max_inst <= 0 || off < 4 || odr < 1 || odr > 6 ||
        (precision != MLAU_FP64 && precision != MLAU_FP32_SPLIT)) {
        set_error("batch: bad arguments");
        return MLAU_ERR_ARG;
    }
    mlau_batch *b = new mlau_batch();
    b->precision = precision;
    b->odr = odr;
    b->off = off;
    b->max_inst = max_inst;
    b->capacity = capacity_cells;
    b->h_inst.assign(max_inst, BInst{});
    b->used.assign(max_inst, 0);
    b->free_[0] = capacity_cells;
    b->kernel = precision == MLAU_FP64 ? batch2d_plain_kernel() : batch2d_split_kernel();
    if (make_stream(&b->stream) != cudaSuccess) {
        set_error("batch: stream creation failed");
        delete b;
        return MLAU_ERR_CUDA;
    }
    const long long C = capacity_cells;
    const size_t n8 = sizeof(double) * C, n4 = sizeof(float) * C, nf2 = sizeof(float2) * C;
    BArrays &a = b->a;
    int rc = MLAU_OK;
    for (int v = 0; v < 8 && !rc; v++)
        rc |= balloc(b, (void **)&a.s[v], n8) | balloc(b, (void **)&a.u0[v], n8);
    if (precision == MLAU_FP32_SPLIT) {
        for (int v = 0; v < 8 && !rc; v++)
            rc |= balloc(b, (void **)&a.q[v], nf2) | balloc(b, (void **)&a.ulf[v], n4) |
                  balloc(b, (void **)&a.urf[v], n4);
        for (int D = 0; D < 2 && !rc; D++) {
            rc |= balloc(b, (void **)&a.bf[D], n4) | balloc(b, (void **)&a.dvf[D], n4) |
                  balloc(b, (void **)&a.FCf[D], n4);
            for (int v = 0; v < 7; v++) rc |= balloc(b, (void **)&a.Ff[D][v], n4);
        }
        if (!rc)
            rc |= balloc(b, (void **)&a.m2f, n4) | balloc(b, (void **)&a.ctf, n4) |
                  balloc(b, (void **)&a.ezf, n4);
    } else {
        double **singles[] = {&a.vx, &a.vy, &a.vz, &a.pr, &a.m2, &a.cx, &a.cy, &a.ct,
                              &a.dv[0], &a.dv[1], &a.ez, &a.FC[0], &a.FC[1]};
        for (auto p : singles)
            if (!rc) rc |= balloc(b, (void **)p, n8);
        for (int v = 0; v < 8 && !rc; v++)
            rc |= balloc(b, (void **)&a.ul[v], n8) | balloc(b, (void **)&a.ur[v], n8);
        for (int D = 0; D < 2 && !rc; D++)
            for (int v = 0; v < 7; v++) rc |= balloc(b, (void **)&a.F[D][v], n8);
    }
    if (!rc)
        rc |= balloc(b, (void **)&b->d_inst, sizeof(BInst) * max_inst) |
              balloc(b, (void **)&b->d_sync, sizeof(BSync));
    if (!rc && cudaMallocHost((void **)&b->h_sync, sizeof(BSync)) != cudaSuccess) {
        set_error("batch: pinned status buffer");
        rc = MLAU_ERR_NOMEM;
    }
    if (!rc) rc = occupancy(b);
    if (rc) {
        mlau_batch_destroy(b);
        return rc;
    }
    *out = b;
    return MLAU_OK;
}

int mlau_batch1d_open(mlau_batch **out, long long capacity_cells, int max_inst, int off, int odr)
{
    if (!out || capacity_cells <= 0 || max_inst <= 0 || off < 4 || odr < 1 || odr > 6) {
        set_error("batch1d: bad arguments");
        return MLAU_ERR_ARG;
    }
    mlau_batch *b = new mlau_batch();
    b->dim = 1;
    b->precision = MLAU_FP64;
    b->odr = odr;
    b->off = off;
    b->max_inst = max_inst;
    b->capacity = capacity_cells;
    b->tw = 256;
    b->th = 1;
    b->h_inst.assign(max_inst, BInst{});
    b->used.assign(max_inst, 0);
    b->free_[0] = capacity_cells;
    b->kernel = batch1d_plain_kernel();
    if (make_stream(&b->stream) != cudaSuccess) {
        set_error("batch1d: stream creation failed");
        delete b;
        return MLAU_ERR_CUDA;
    }
    const size_t n8 = sizeof(double) * capacity_cells;
    BArrays &a = b->a;
    int rc = MLAU_OK;
    for (int v = 0; v < 8 && !rc; v++) {
        if (v == 5) continue;
        rc |= balloc(b, (void **)&a.s[v], n8) | balloc(b, (void **)&a.u0[v], n8);
    }
    double **singles[] = {&a.vx, &a.vy, &a.vz, &a.pr};
    for (auto p : singles)
        if (!rc) rc |= balloc(b, (void **)p, n8);
    for (int v = 0; v < 7 && !rc; v++)
        rc |= balloc(b, (void **)&a.ul[v], n8) | balloc(b, (void **)&a.ur[v], n8) |
              balloc(b, (void **)&a.F[0][v], n8);
    if (!rc)
        rc |= balloc(b, (void **)&b->d_inst, sizeof(BInst) * max_inst) |
              balloc(b, (void **)&b->d_sync, sizeof(BSync));
    if (!rc && cudaMallocHost((void **)&b->h_sync, sizeof(BSync)) != cudaSuccess) {
        set_error("batch1d: pinned status buffer");
        rc = MLAU_ERR_NOMEM;
    }
    if (!rc) rc = occupancy(b);
    if (rc) {
        mlau_batch_destroy(b);
        return rc;
    }
    *out = b;
    return MLAU_OK;
}

int mlau_batch_destroy(mlau_batch *b)
{
    if (!b) return MLAU_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    for (void *p : b->allocs) cudaFree(p);
    if (b->h_sync) cudaFreeHost(b->h_sync);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MLAU_OK;
}

// Admit one instance: returns its slot, or MLAU_ERR_NOMEM when no slot or not
// enough pooled cells are free (the caller queues it and retries later).
int mlau_batch_add(mlau_batch *b, int nx, int ny, double dx, double dy, double gamma, int flux,
                   double cfl, double t_end, const double *const *host8, int *slot)
{
    if (b && b->dim != 2) {
        set_error("batch: a 1D batch takes mlau_batch1d_add");
        return MLAU_ERR_ARG;
    }
    if (!b || !host8 || !slot || nx - 2 * b->off < b->off || ny - 2 * b->off < b->off ||
        flux < 0 || flux > 3 || !(gamma > 1.0) || !(dx > 0) || !(dy > 0)) {
        set_error("batch: bad instance");
        return MLAU_ERR_ARG;
    }
    int n = -1;
    for (int k = 0; k < b->max_inst; k++)
        if (!b->used[k]) { n = k; break; }
    if (n < 0) { set_error("batch: no free slot"); return MLAU_ERR_NOMEM; }
    const long long cells = (long long)nx * ny;
    const long long base = carve(b, cells);
    if (base < 0) { set_error("batch: no room for %lld cells", cells); return MLAU_ERR_NOMEM; }
    BInst I{};
    I.nx = nx;
    I.ny = ny;
    I.off = b->off;
    I.flux = flux;
    I.gamma = gamma;
    I.cfl = cfl;
    I.dx = dx;
    I.dy = dy;
    I.t_end = t_end;
    I.base = base;
    I.active = 1;
    b->h_inst[n] = I;
    b->used[n] = 1;
    b->tiles_dirty = true;
    const size_t bytes = sizeof(double) * cells;
    for (int v = 0; v < 8; v++)
        MLAU_CUDA(cudaMemcpyAsync(b->a.s[v] + base, host8[v], bytes, cudaMemcpyHostToDevice,
                                  b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    *slot = n;
    return MLAU_OK;
}

int mlau_batch1d_add(mlau_batch *b, int nx, double dx, double bx, double gamma, int flux, int nrk,
                     int bc, double cfl, double t_end, const double *const *host8, int *slot)
{
    if (!b || b->dim != 1 || !host8 || !slot || nx - 2 * b->off < b->off || flux < 0 ||
        flux > 3 || nrk < 1 || nrk > 3 || (bc != MLAU_BC1D_OPEN && bc != MLAU_BC1D_PERIODIC) ||
        !(gamma > 1.0) || !(dx > 0) || !(cfl > 0)) {
        set_error("batch1d: bad instance");
        return MLAU_ERR_ARG;
    }
    for (int v = 0; v < 8; v++)
        if (v != 5 && !host8[v]) {
            set_error("batch1d: missing state array %d", v);
            return MLAU_ERR_ARG;
        }
    int n = -1;
    for (int k = 0; k < b->max_inst; k++)
        if (!b->used[k]) { n = k; break; }
    if (n < 0) { set_error("batch1d: no free slot"); return MLAU_ERR_NOMEM; }
    const long long base = carve(b, nx);
    if (base < 0) { set_error("batch1d: no room for %d cells", nx); return MLAU_ERR_NOMEM; }
    BInst I{};
    I.nx = nx;
    I.ny = 1;
    I.off = b->off;
    I.flux = flux;
    I.bc = bc;
    I.nrk = nrk;
    I.gamma = gamma;
    I.cfl = cfl;
    I.dx = dx;
    I.dy = dx;
    I.bx = bx;
    I.t_end = t_end;
    I.base = base;
    I.active = 1;
    b->h_inst[n] = I;
    b->used[n] = 1;
    b->tiles_dirty = true;
    for (int v = 0; v < 8; v++)
        if (v != 5)
            MLAU_CUDA(cudaMemcpyAsync(b->a.s[v] + base, host8[v], sizeof(double) * nx,
                                      cudaMemcpyHostToDevice, b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    *slot = n;
    return MLAU_OK;
}

int mlau_batch_remove(mlau_batch *b, int n)
{
    if (!check_inst(b, n)) return MLAU_ERR_ARG;
    release(b, b->h_inst[n].base, (long long)b->h_inst[n].nx * b->h_inst[n].ny);
    b->used[n] = 0;
    b->h_inst[n] = BInst{};
    b->tiles_dirty = true;
    return MLAU_OK;
}

int mlau_batch_create(mlau_batch **out, int ninst, const int *nx, const int *ny, int off,
                      const double *dx, const double *dy, const double *gamma, const int *flux,
                      const double *cfl, const double *t_end, int odr)
{
    if (!out || ninst <= 0 || !nx || !ny) { set_error("batch: bad arguments"); return MLAU_ERR_ARG; }
    long long cells = 0;
    for (int n = 0; n < ninst; n++) cells += (long long)nx[n] * ny[n];
    int rc = mlau_batch_open(out, MLAU_FP32_SPLIT, cells, ninst, off, odr);
    if (rc) return rc;
    mlau_batch *b = *out;
    std::vector<double> zero;
    for (int n = 0; n < ninst && !rc; n++) {
        zero.assign((size_t)nx[n] * ny[n], 0.0);
        const double *h[8];
        for (int v = 0; v < 8; v++) h[v] = zero.data();
        int slot;
        rc = mlau_batch_add(b, nx[n], ny[n], dx[n], dy[n], gamma[n], flux[n], cfl[n], t_end[n], h,
                            &slot);
    }
    if (rc) { mlau_batch_destroy(b); *out = nullptr; }
    return rc;
}

int mlau_batch_upload(mlau_batch *b, int n, const double *const *h)
{
    if (!check_inst(b, n) || !h) return MLAU_ERR_ARG;
    const BInst &I = b->h_inst[n];
    const size_t bytes = sizeof(double) * I.nx * I.ny;
    for (int v = 0; v < 8; v++)
        if (b->a.s[v] && h[v])
            MLAU_CUDA(cudaMemcpyAsync(b->a.s[v] + I.base, h[v], bytes, cudaMemcpyHostToDevice,
                                      b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    return MLAU_OK;
}

int mlau_batch_download(mlau_batch *b, int n, double *const *h)
{
    if (!check_inst(b, n) || !h) return MLAU_ERR_ARG;
    const BInst &I = b->h_inst[n];
    const size_t bytes = sizeof(double) * I.nx * I.ny;
    for (int v = 0; v < 8; v++)
        if (b->a.s[v] && h[v])
            MLAU_CUDA(cudaMemcpyAsync(h[v], b->a.s[v] + I.base, bytes, cudaMemcpyDeviceToHost,
                                      b->stream));
    MLAU_CUDA(cudaStreamSynchronize(b->stream));
    return MLAU_OK;
}

int mlau_batch_set_bc(mlau_batch *b, int n, const int *dnx, const int *dny)
{
    if (!check_inst(b, n)) return MLAU_ERR_ARG;
    if (b->dim != 2 || !dnx || !dny) {
        set_error("batch: boundary tables apply to 2D instances");
        return MLAU_ERR_ARG;
    }
    BInst &I = b->h_inst[n];
    int walls = 0;
    for (int v = 0; v < 8; v++) {
        if (dnx[v] < -1 || dnx[v] > 1 || dny[v] < -1 || dny[v] > 1) {
            set_error("boundary table entries are -1, 0 or +1");
            return MLAU_ERR_ARG;
        }
        walls |= dnx[v] != 0 || dny[v] != 0;
    }
    for (int v = 0; v < 8; v++) {
        I.bcx[v] = (signed char)dnx[v];
        I.bcy[v] = (signed char)dny[v];
    }
    I.walls = walls;
    return MLAU_OK;
}

int mlau_batch_set_fixed_dt(mlau_batch *b, int n, double dt)
{
    if (!check_inst(b, n)) return MLAU_ERR_ARG;
    b->h_inst[n].dt_fixed = dt;
    return MLAU_OK;
}

int mlau_batch_run(mlau_batch *b, int max_steps, int steps_per_graph, int *active_left, double *ms)
{
    if (!b || max_steps < 0) { set_error("batch: bad run arguments"); return MLAU_ERR_ARG; }
    int rc = push_table(b);
    if (rc) return rc;
    cudaEvent_t e0, e1;
    MLAU_CUDA(cudaEventCreate(&e0));
    MLAU_CUDA(cudaEventCreate(&e1));
    MLAU_CUDA(cudaEventRecord(e0, b->stream));
    int done = 0;
    while (done < max_steps && b->h_sync->active_left > 0) {
        int k = 1;
        if (steps_per_graph > 0 && max_steps - done >= steps_per_graph) {
            k = steps_per_graph;
            rc = make_graph(b, k);
            if (rc) break;
            cudaError_t e = cudaGraphLaunch(b->gexec, b->stream);
            if (e != cudaSuccess) { set_error("batch: graph launch: %s", cudaGetErrorString(e)); rc = MLAU_ERR_CUDA; break; }
        } else {
            rc = launch_step(b);
            if (rc) break;
            cudaMemcpyAsync(b->h_sync, b->d_sync, sizeof(BSync), cudaMemcpyDeviceToHost, b->stream);
        }
        b->launches += k;
        done += k;
        MLAU_CUDA(cudaStreamSynchronize(b->stream));
        if (b->h_sync->err) break;
    }
    MLAU_CUDA(cudaEventRecord(e1, b->stream));
    MLAU_CUDA(cudaEventSynchronize(e1));
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t;
    const int rc2 = pull_table(b);
    if (active_left) *active_left = b->h_sync->active_left;
    if (b->h_sync->active_left <= 0) b->tiles_dirty = true;
    for (int n = 0; n < b->max_inst; n++)
        if (b->used[n] && !b->h_inst[n].active) b->tiles_dirty = true;
    return rc ? rc : rc2;
}

int mlau_batch_set_tile(mlau_batch *b, int tw, int th)
{
    if (b && b->dim == 1) {
        if (th != 1 || (tw != 64 && tw != 128 && tw != 256)) {
            set_error("batch1d: tile must be 64, 128 or 256 cells by 1");
            return MLAU_ERR_ARG;
        }
    } else if (!b || tw <= 0 || th <= 0 || tw * th != 256 || tw % 16) {
        set_error("batch: tile must be TW x TH = 256 threads with TW a multiple of 16");
        return MLAU_ERR_ARG;
    }
    b->tw = tw;
    b->th = th;
    b->tiles_dirty = true;
    if (b->gexec) { cudaGraphExecDestroy(b->gexec); b->gexec = nullptr; }
    return occupancy(b);
}

int mlau_batch_set_grid(mlau_batch *b, int nblocks)
{
    if (!b || nblocks < 0) { set_error("batch: bad grid size"); return MLAU_ERR_ARG; }
    const unsigned old = b->nblocks;
    b->want_blocks = (unsigned)nblocks;
    b->nblocks = nblocks ? std::min(b->want_blocks, b->max_blocks) : b->max_blocks;
    if (b->nblocks != old && b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    return (int)b->nblocks;
}

int mlau_batch_max_grid(mlau_batch *b) { return b ? (int)b->max_blocks : 0; }

int mlau_batch_autotune(mlau_batch *b, int steps, int *tw_out, int *th_out, double *ms_out)
{
    if (!b || steps <= 0) { set_error("batch: bad autotune arguments"); return MLAU_ERR_ARG; }
    const int cand2[4][2] = {{32, 8}, {64, 4}, {16, 16}, {128, 2}};
    const int cand1[3][2] = {{256, 1}, {128, 1}, {64, 1}};
    const int(*cand)[2] = b->dim == 1 ? cand1 : cand2;
    const int ncand = b->dim == 1 ? 3 : 4;
    double best = 1e300;
    int bw = cand[0][0], bh = cand[0][1];
    for (int k = 0; k < ncand; k++) {
        const int *c = cand[k];
        int rc = mlau_batch_set_tile(b, c[0], c[1]);
        if (rc) return rc;
        double ms = 0;
        int left = 0;
        rc = mlau_batch_run(b, steps, 0, &left, &ms);
        if (rc) return rc;
        if (ms < best) { best = ms; bw = c[0]; bh = c[1]; }
        if (left <= 0) break;
    }
    const int rc = mlau_batch_set_tile(b, bw, bh);
    if (tw_out) *tw_out = bw;
    if (th_out) *th_out = bh;
    if (ms_out) *ms_out = best;
    return rc;
}

int mlau_batch_info(mlau_batch *b, int n, double *t, int *steps, int *active)
{
    if (!check_inst(b, n)) return MLAU_ERR_ARG;
    const BInst &I = b->h_inst[n];
    if (t) *t = I.t;
    if (steps) *steps = I.steps;
    if (active) *active = I.active;
    return MLAU_OK;
}

int mlau_batch_status(mlau_batch *b, int n)
{
    if (!check_inst(b, n)) return MLAU_ERR_ARG;
    if (b->h_inst[n].status) {
        set_error("batch: instance %d retired on a NaN or non-positive density/pressure", n);
        return MLAU_ERR_STATE;
    }
    return MLAU_OK;
}

long long mlau_batch_cells(mlau_batch *b)
{
    if (!b) return 0;
    long long c = 0;
    for (int n = 0; n < b->max_inst; n++)
        if (b->used[n]) c += (long long)b->h_inst[n].nx * b->h_inst[n].ny;
    return c;
}
long long mlau_batch_device_bytes(mlau_batch *b) { return b ? b->bytes : 0; }
long long mlau_batch_launches(mlau_batch *b) { return b ? b->launches : 0; }

}  // extern "C"
