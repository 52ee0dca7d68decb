// Plane schedule of one step of a periodic state held in host arrays (the
// C-ABI drivers in FP32-split mode): which kernels run over which z-planes,
// and in what order, so that the host->device copy of the state overlaps the
// first RK stage and the device->host copy the last one, while every kernel
// reads exactly the values the whole-grid step gives it (the results are the
// same bits).
//
// The plan is demand-driven.  The first stage asks for the update of one
// z-slab after another (from a chosen slab on, cyclically; the bottom slab
// first at the last stage); each request first asks for what the update reads
// (z fluxes and edge EMFs of the neighbouring planes, x / y fluxes of its
// planes), each of those for its own inputs, down to the primitive recovery,
// which asks for the copies of the state planes it reads.  Whatever is not
// done yet is launched over maximal runs of planes.  An update overwrites its
// state planes and their periodic ghost images, so before it runs, every
// primitive recovery that reads one of those planes has run.  The last stage
// asks for the slabs the same way and sends each plane back to the host as
// soon as the update that writes it has run.  Stages in between run whole.
//
// Pure host code (no CUDA): split3d.cu carries the plan out;
// tests/c/slab_plan_check.cpp replays plans against the kernels' read and
// write sets on the CPU.
#pragma once

#include <algorithm>
#include <vector>

namespace mlau {

enum SlabOpKind {
    SP_UPLOAD,    // copy state planes [a, b) host -> device as upload number n
    SP_WAIT,      // the compute stream waits for upload n
    SP_PRIM,      // primitive recovery of planes [a, b) at stage rk
    SP_AUX,       // CT weights and shock sensors of planes [a, b)
    SP_SWEEP_X,   // x reconstruction + flux of planes [a, b)
    SP_SWEEP_Y,   // y reconstruction + flux of planes [a, b)
    SP_SWEEP_Z,   // z reconstruction + flux of tile rows [a, b) along z
    SP_EMF,       // edge EMFs of planes [a, b)
    SP_UPDATE,    // RK combine + CT curl of interior planes [a, b), with images
    SP_DOWNLOAD,  // copy state planes [a, b) device -> host after the updates so far
    SP_STAGE,     // stage rk over the whole grid
};

struct SlabOp {
    int kind, rk, a, b, n;
};

// Read and write sets of the kernels along z (planes 0..nz-1, ghost depth
// oz, periodic).  tz: cells per z-sweep tile (tile t holds cells
// 2 + (tz-1) t .. 2 + (tz-1) t + tz - 1 and yields the faces of all but its
// first cell).
struct SlabGeom {
    int nz, oz, tz;
    int Nz() const { return nz - 2 * oz; }
    // interior source of a plane (the periodic wrap of the ghost planes)
    int wrap(int k) const { return k < oz ? k + Nz() : (k >= nz - oz ? k - Nz() : k); }
    int nseg() const { return std::max(0, (nz - 5 + tz - 2) / (tz - 1)); }
    // planes whose state the primitive recovery of plane k reads: its own
    // cells and the face-B stencil (4 faces) around its source plane
    void prim_reads(int k, std::vector<int> &o) const
    {
        o.push_back(k);
        for (int m = -1; m <= 2; m++) o.push_back(wrap(k) + m);
    }
    // primitive planes the CT weights (planes k-1, k) and the shock sensors
    // (around the source plane) of plane k read
    void aux_reads(int k, std::vector<int> &o) const
    {
        if (k >= 1) o.push_back(k - 1);
        o.push_back(k);
        for (int m = -1; m <= 1; m++) o.push_back(wrap(k) + m);
    }
    // z-sweep tile row t: staged planes [r0, r1) and faces written [f0, f1)
    void seg_reads(int t, int &r0, int &r1) const
    {
        r0 = (tz - 1) * t;
        r1 = std::min(nz, r0 + tz + 4);
    }
    void seg_faces(int t, int &f0, int &f1) const
    {
        f0 = std::max(3, 3 + (tz - 1) * t);
        f1 = std::min(nz - 2, 2 + (tz - 1) * t + tz);
    }
    int seg_of_face(int k) const { return (k - 3) / (tz - 1); }
    // planes of the x / y fluxes the EMFs of plane k read (the z
    // interpolations of the edges along x and y: planes k-3..k+2; the
    // in-plane edge along z: plane k)
    bool emf_has_z(int k) const { return k >= 3 && k < nz - 2; }
    // periodic images an update of interior plane k writes
    void images(int k, std::vector<int> &o) const
    {
        if (k < 2 * oz) o.push_back(k + Nz());
        if (k >= Nz()) o.push_back(k - Nz());
    }
};

class SlabPlan {
public:
    // first / last: the interior slab sizes (in z order, summing to the
    // interior depth) the first and last stages are requested in; chunk:
    // planes per upload; first_start: the slab the first stage asks for
    // first, the others following cyclically (a slab away from the ends
    // needs no periodic source at the far end, so fewer uploads before its
    // update can run)
    SlabPlan(const SlabGeom &g, int nrk, const std::vector<int> &first,
             const std::vector<int> &last, int chunk, int first_start = 0)
        : g_(g), nrk_(nrk), chunk_(std::max(1, chunk))
    {
        build(first, last, first_start);
    }
    // nslab equal slabs in both stages
    SlabPlan(const SlabGeom &g, int nrk, int nslab, int chunk, int first_start = 0)
        : g_(g), nrk_(nrk), chunk_(std::max(1, chunk))
    {
        const int Nz = g.Nz();
        nslab = std::max(1, std::min(nslab, Nz));
        std::vector<int> sz;
        for (int c = 0; c < nslab; c++)
            sz.push_back((int)((long long)Nz * (c + 1) / nslab - (long long)Nz * c / nslab));
        build(sz, sz, first_start);
    }
    std::vector<SlabOp> ops;
    int uploads() const { return nup_; }

private:
    void build(const std::vector<int> &first, const std::vector<int> &last, int first_start)
    {
        const SlabGeom &g = g_;
        const int nz = g.nz, oz = g.oz;
        readers_.assign(nz, {});
        std::vector<int> r;
        for (int k = 0; k < nz; k++) {
            r.clear();
            g.prim_reads(k, r);
            for (int p : r)
                if (p >= 0 && p < nz) readers_[p].push_back(k);
        }
        writer_.assign(nz, -1);
        for (int k = oz; k < nz - oz; k++) {
            writer_[k] = k;
            r.clear();
            g.images(k, r);
            for (int p : r) writer_[p] = k;
        }
        up_.assign(nz, -1);
        for (int rk = 0; rk < nrk_; rk++) {
            const bool is_first = rk == 0, is_last = rk == nrk_ - 1;
            if (!is_first && !is_last) {
                ops.push_back({SP_STAGE, rk, 0, nz, 0});
                continue;
            }
            reset(rk);
            std::vector<char> sent(nz, 0);
            // slab boundaries in z order; whatever the sizes leave out is a
            // last slab of its own
            std::vector<std::pair<int, int>> slabs;
            int a = oz;
            for (int len : is_first ? first : last) {
                const int b = std::min(nz - oz, a + std::max(0, len));
                slabs.push_back({a, b});
                a = b;
            }
            slabs.push_back({a, nz - oz});
            const int n = (int)slabs.size();
            const int c0 = is_first ? ((first_start % n) + n) % n : 0;
            for (int c = 0; c < n; c++) {
                const std::pair<int, int> &sl = slabs[(c0 + c) % n];
                need_update(range(sl.first, sl.second));
                if (is_last) download_final(sent);
            }
        }
    }

    SlabGeom g_;
    int nrk_, chunk_;
    int rk_ = 0, nup_ = 0, waited_ = -1;
    std::vector<std::vector<int>> readers_;  // plane -> primitive recoveries reading its state
    std::vector<int> writer_;                // plane -> interior plane whose update writes it
    std::vector<int> up_;                    // plane -> upload number, -1 not yet asked for
    std::vector<char> q_, a_, x_, y_, z_, e_, u_;

    static std::vector<int> range(int a, int b)
    {
        std::vector<int> v;
        for (int k = a; k < b; k++) v.push_back(k);
        return v;
    }
    // the planes of v inside [0, n) that are not done, sorted, without repeats
    static std::vector<int> todo(std::vector<int> v, const std::vector<char> &done)
    {
        std::vector<int> o;
        for (int k : v)
            if (k >= 0 && k < (int)done.size() && !done[k]) o.push_back(k);
        std::sort(o.begin(), o.end());
        o.erase(std::unique(o.begin(), o.end()), o.end());
        return o;
    }
    // one op per maximal run of consecutive entries of v
    void emit_runs(int kind, const std::vector<int> &v)
    {
        for (size_t s = 0; s < v.size();) {
            size_t e = s + 1;
            while (e < v.size() && v[e] == v[e - 1] + 1) e++;
            ops.push_back({kind, rk_, v[s], v[e - 1] + 1, 0});
            s = e;
        }
    }
    void reset(int rk)
    {
        rk_ = rk;
        const size_t nz = g_.nz;
        q_.assign(nz, 0); a_.assign(nz, 0); x_.assign(nz, 0); y_.assign(nz, 0);
        e_.assign(nz, 0); u_.assign(nz, 0); z_.assign(g_.nseg(), 0);
    }
    // upload number a plane's copy goes out as, the chunk issued on first need
    int upload_of(int p)
    {
        if (up_[p] < 0) {
            const int c0 = p / chunk_ * chunk_, c1 = std::min(g_.nz, c0 + chunk_);
            ops.push_back({SP_UPLOAD, 0, c0, c1, nup_});
            for (int k = c0; k < c1; k++) up_[k] = nup_;
            nup_++;
        }
        return up_[p];
    }
    void wait_upload(int n)
    {
        if (n > waited_) {
            ops.push_back({SP_WAIT, 0, 0, 0, n});
            waited_ = n;  // uploads complete in order on their stream
        }
    }
    // Everything the updates of interior planes v need and has not run yet,
    // then the updates, each kind over maximal runs of planes (the kinds
    // only read earlier kinds, so this order keeps every dependence).
    void need_update(const std::vector<int> &v)
    {
        const std::vector<int> u = todo(v, u_);
        if (u.empty()) return;
        std::vector<int> e, zf, xy, a, q, r;
        for (int k : u)
            for (int m = -1; m <= 2; m++) {
                e.push_back(k + m);
                zf.push_back(k + m);
            }
        e = todo(e, e_);
        for (int k : u) xy.push_back(k);
        for (int k : e) {
            xy.push_back(k);
            if (g_.emf_has_z(k)) {
                for (int m = -3; m <= 2; m++) xy.push_back(k + m);
                zf.push_back(k);
            }
        }
        std::vector<int> segs;
        for (int k : zf)
            if (k >= 3 && k < g_.nz - 2) segs.push_back(g_.seg_of_face(k));
        segs = todo(segs, z_);
        const std::vector<int> x = todo(xy, x_), y = todo(xy, y_);
        a = xy;
        a.insert(a.end(), e.begin(), e.end());
        for (int t : segs) {
            int r0, r1;
            g_.seg_reads(t, r0, r1);
            for (int k = r0; k < r1; k++) a.push_back(k);
        }
        a = todo(a, a_);
        q = xy;
        for (int t : segs) {
            int r0, r1;
            g_.seg_reads(t, r0, r1);
            for (int k = r0; k < r1; k++) q.push_back(k);
        }
        for (int k : a) g_.aux_reads(k, q);
        // every reader of the state planes the updates overwrite runs first
        for (int k : u) {
            r.assign(1, k);
            g_.images(k, r);
            for (int p : r) q.insert(q.end(), readers_[p].begin(), readers_[p].end());
        }
        q = todo(q, q_);
        // primitive recoveries in the order their uploads land, each group
        // after a wait for its last upload
        std::vector<std::pair<int, int>> order;  // (upload needed, plane)
        for (int k : q) {
            int need = -1;
            if (rk_ == 0) {
                r.clear();
                g_.prim_reads(k, r);
                for (int p : r) need = std::max(need, upload_of(p));
            }
            order.push_back({need, k});
        }
        std::sort(order.begin(), order.end());
        for (size_t s = 0; s < order.size();) {
            size_t e2 = s;
            std::vector<int> grp;
            while (e2 < order.size() && order[e2].first == order[s].first) grp.push_back(order[e2++].second);
            wait_upload(order[s].first);
            emit_runs(SP_PRIM, grp);
            s = e2;
        }
        for (int k : q) q_[k] = 1;
        for (int k : a) a_[k] = 1;
        emit_runs(SP_AUX, a);
        for (int k : x) x_[k] = 1;
        emit_runs(SP_SWEEP_X, x);
        for (int k : y) y_[k] = 1;
        emit_runs(SP_SWEEP_Y, y);
        for (int t : segs) z_[t] = 1;
        emit_runs(SP_SWEEP_Z, segs);
        for (int k : e) e_[k] = 1;
        emit_runs(SP_EMF, e);
        if (rk_ == 0) {
            int need = -1;
            for (int k : u) need = std::max(need, upload_of(k));
            wait_upload(need);
        }
        for (int k : u) u_[k] = 1;
        emit_runs(SP_UPDATE, u);
    }
    // send back every plane whose writer has run and that is not sent yet
    void download_final(std::vector<char> &sent)
    {
        std::vector<int> v;
        for (int p = 0; p < g_.nz; p++)
            if (!sent[p] && writer_[p] >= 0 && u_[writer_[p]]) {
                v.push_back(p);
                sent[p] = 1;
            }
        for (size_t s = 0; s < v.size();) {
            size_t e = s + 1;
            while (e < v.size() && v[e] == v[e - 1] + 1) e++;
            ops.push_back({SP_DOWNLOAD, rk_, v[s], v[e - 1] + 1, 0});
            s = e;
        }
    }
};

}  // namespace mlau
