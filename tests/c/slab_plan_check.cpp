// Replays plans of mlau_gb300/csrc/slab_plan.h on the CPU and checks each op
// against the kernels' own read and write sets along z (split3d.cu), stated
// here independently of the planner:
//   prim(k)    reads state planes k and wrap(k)-1 .. wrap(k)+2 (cells, face-B
//              stencil at the periodic source); writes primitives Q(k), and
//              at the first stage U^n(k)
//   aux(k)     reads Q(k-1), Q(k) (CT weights) and Q(wrap(k)-1 .. wrap(k)+1)
//              (shock sensors); writes A(k)
//   x/y sweep  reads Q(k), A(k); writes X(k) / Y(k)
//   z sweep    tile row t: cells c = 2 + (tz-1) t + m, m < tz; each cell
//              2 <= c < nz-2 reads Q, A at c-2 .. c+2; writes the z fluxes of
//              faces c with m >= 1, 3 <= c < nz-2
//   emf(k)     reads A(k), X(k), Y(k); for 3 <= k < nz-2 also X, Y at
//              k-3 .. k+2 and the z flux of face k; writes E(k)
//   update(k)  reads X(k), Y(k), z fluxes and E at k-1 .. k+2, the state of
//              plane k at this stage's version and U^n(k); writes the state
//              of plane k and of its periodic images (version + 1)
// and the copies: an upload makes its planes readable once a wait on it (or
// on a later upload) has been issued on the compute stream; a download takes
// planes at their final version, each plane once.
//
// Usage: slab_plan_check  -> prints "ok <plans checked>" or the first fault.
#include "../../mlau_gb300/csrc/slab_plan.h"

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

using namespace mlau;

namespace {

struct Replay {
    int nz, oz, tz, nrk, Nz;
    std::string err;
    bool fail(const char *what, int k)
    {
        if (err.empty()) err = std::string(what) + " at plane " + std::to_string(k);
        return false;
    }
    int wrap(int k) const { return k < oz ? k + Nz : (k >= nz - oz ? k - Nz : k); }

    bool run(const std::vector<SlabOp> &ops)
    {
        std::vector<int> version(nz, -1), upnum(nz, -1), sent(nz, 0);
        std::vector<char> u0(nz, 0);
        int waited = -1, stage = -1;
        std::vector<char> Q, A, X, Y, Z, E, U;
        auto begin_stage = [&](int rk) {
            Q.assign(nz, 0); A.assign(nz, 0); X.assign(nz, 0); Y.assign(nz, 0);
            Z.assign(nz, 0); E.assign(nz, 0); U.assign(nz, 0);
            stage = rk;
        };
        auto readable = [&](int p, int rk) {
            if (p < 0 || p >= nz) return fail("state read outside the grid", p);
            if (rk == 0 && version[p] == -1) {
                if (upnum[p] < 0 || upnum[p] > waited) return fail("state read before its upload", p);
                version[p] = 0;
            }
            if (version[p] != rk) return fail("state read at the wrong version", p);
            return true;
        };
        auto have = [&](const std::vector<char> &f, int p, const char *what) {
            if (p < 0 || p >= nz || !f[p]) return fail(what, p);
            return true;
        };
        auto produce = [&](std::vector<char> &f, int p, const char *what) {
            if (f[p]) return fail(what, p);
            f[p] = 1;
            return true;
        };
        // scratch no update reads need not be computed (every read above is
        // checked against this stage's own producers); every update must run
        auto finish_check = [&]() {
            for (int k = oz; k < nz - oz; k++)
                if (!U[k]) return fail("stage left an update undone", k);
            return true;
        };
        for (const SlabOp &o : ops) {
            // every launch stays inside the grid (planes) or the z-sweep's
            // tile rows
            const int lim = o.kind == SP_SWEEP_Z ? (nz - 5 + tz - 2) / (tz - 1) : nz;
            if (o.kind != SP_WAIT && (o.a < 0 || o.b > lim || o.a >= o.b))
                return fail("op range outside the grid", o.a);
            if (o.kind == SP_UPLOAD) {
                for (int p = o.a; p < o.b; p++) {
                    if (upnum[p] >= 0) return fail("plane uploaded twice", p);
                    upnum[p] = o.n;
                }
                continue;
            }
            if (o.kind == SP_WAIT) {
                waited = std::max(waited, o.n);
                continue;
            }
            if (o.kind == SP_DOWNLOAD) {
                for (int p = o.a; p < o.b; p++) {
                    if (version[p] != nrk) return fail("plane downloaded before its final update", p);
                    if (sent[p]++) return fail("plane downloaded twice", p);
                }
                continue;
            }
            if (o.rk != stage) {
                if (stage >= 0 && !finish_check()) return false;
                if (o.rk != stage + 1) return fail("stages out of order", o.rk);
                begin_stage(o.rk);
            }
            const int rk = o.rk;
            if (o.kind == SP_STAGE) {
                for (int p = 0; p < nz; p++)
                    if (version[p] != rk) return fail("whole stage on a state at the wrong version", p);
                std::fill(Q.begin(), Q.end(), 1); std::fill(A.begin(), A.end(), 1);
                std::fill(X.begin(), X.end(), 1); std::fill(Y.begin(), Y.end(), 1);
                std::fill(Z.begin(), Z.end(), 1); std::fill(E.begin(), E.end(), 1);
                std::fill(U.begin(), U.end(), 1);
                for (int p = 0; p < nz; p++) version[p] = rk + 1;
                continue;
            }
            if (o.kind == SP_SWEEP_Z) {
                for (int t = o.a; t < o.b; t++)
                    for (int m = 0; m < tz; m++) {
                        const int c = 2 + (tz - 1) * t + m;
                        if (c >= 2 && c < nz - 2)
                            for (int d = -2; d <= 2; d++)
                                if (!have(Q, c + d, "z sweep before a primitive plane") ||
                                    !have(A, c + d, "z sweep before an aux plane"))
                                    return false;
                        if (m >= 1 && c >= 3 && c < nz - 2 && !produce(Z, c, "z face computed twice"))
                            return false;
                    }
                continue;
            }
            for (int k = o.a; k < o.b; k++) {
                switch (o.kind) {
                case SP_PRIM:
                    if (!readable(k, rk)) return false;
                    for (int m = -1; m <= 2; m++)
                        if (!readable(wrap(k) + m, rk)) return false;
                    if (!produce(Q, k, "primitives computed twice")) return false;
                    if (rk == 0) u0[k] = 1;
                    break;
                case SP_AUX:
                    if (k >= 1 && !have(Q, k - 1, "aux before a primitive plane")) return false;
                    if (!have(Q, k, "aux before its primitive plane")) return false;
                    for (int m = -1; m <= 1; m++)
                        if (!have(Q, wrap(k) + m, "aux before a sensor plane")) return false;
                    if (!produce(A, k, "aux computed twice")) return false;
                    break;
                case SP_SWEEP_X:
                case SP_SWEEP_Y:
                    if (!have(Q, k, "sweep before its primitives") || !have(A, k, "sweep before its aux"))
                        return false;
                    if (!produce(o.kind == SP_SWEEP_X ? X : Y, k, "sweep computed twice")) return false;
                    break;
                case SP_EMF:
                    if (!have(A, k, "emf before aux") || !have(X, k, "emf before x flux") ||
                        !have(Y, k, "emf before y flux"))
                        return false;
                    if (k >= 3 && k < nz - 2) {
                        for (int m = -3; m <= 2; m++)
                            if (!have(X, k + m, "emf before x flux plane") ||
                                !have(Y, k + m, "emf before y flux plane"))
                                return false;
                        if (!have(Z, k, "emf before z face")) return false;
                    }
                    if (!produce(E, k, "emf computed twice")) return false;
                    break;
                case SP_UPDATE: {
                    if (k < oz || k >= nz - oz) return fail("update of a ghost plane", k);
                    if (!have(X, k, "update before x flux") || !have(Y, k, "update before y flux"))
                        return false;
                    for (int m = -1; m <= 2; m++)
                        if (!have(Z, k + m, "update before z face") || !have(E, k + m, "update before emf"))
                            return false;
                    if (!u0[k]) return fail("update before U^n", k);
                    if (!readable(k, rk)) return false;
                    if (!produce(U, k, "update computed twice")) return false;
                    std::vector<int> w = {k};
                    if (k < 2 * oz) w.push_back(k + Nz);
                    if (k >= Nz) w.push_back(k - Nz);
                    for (int p : w) {
                        // an upload still in flight would land on the new values
                        if (rk == 0 && (upnum[p] < 0 || upnum[p] > waited))
                            return fail("update writes a plane whose upload may land later", p);
                        version[p] = rk + 1;
                    }
                    break;
                }
                default:
                    return fail("unknown op", o.kind);
                }
            }
        }
        if (!finish_check()) return false;
        if (stage != nrk - 1) return fail("plan ends before the last stage", stage);
        for (int p = 0; p < nz; p++) {
            if (version[p] != nrk) return fail("plane not at its final version", p);
            if (sent[p] != 1) return fail("plane not downloaded", p);
        }
        return true;
    }
};

}  // namespace

int main()
{
    int checked = 0;
    unsigned seed = 12345u;
    const int tzs[] = {16, 5, 32};
    for (int tz : tzs)
        for (int oz = 4; oz <= 5; oz++)
            for (int Nz = oz; Nz <= 300; Nz += (Nz < 48 ? 1 : 37))
                for (int nrk = 1; nrk <= 3; nrk++)
                    for (int nslab : {1, 2, 3, 8, 16})
                        for (int chunk : {1, 7, 16, 64}) {
                            const int nz = Nz + 2 * oz;
                            const SlabGeom g{nz, oz, tz};
                            SlabPlan plan(g, nrk, nslab, chunk, (Nz + nslab + chunk) % (nslab + 1));
                            Replay r{nz, oz, tz, nrk, Nz, ""};
                            if (!r.run(plan.ops)) {
                                printf("FAIL nz=%d oz=%d tz=%d nrk=%d nslab=%d chunk=%d: %s\n", nz, oz,
                                       tz, nrk, nslab, chunk, r.err.c_str());
                                return 1;
                            }
                            checked++;
                            // arbitrary slab sizes (short, long, zero)
                            const int body = std::max(1, Nz / nslab);
                            std::vector<int> rnd, rnd2;
                            for (std::vector<int> *v : {&rnd, &rnd2})
                                for (int a = 0; a < Nz + 8;) {
                                    seed = seed * 1103515245u + 12345u;
                                    const int len = (int)((seed >> 16) % (unsigned)(2 * body + 2));
                                    v->push_back(len);
                                    a += std::max(1, len);
                                }
                            std::vector<int> uni;
                            for (int c = 0; c < nslab; c++) uni.push_back(body);
                            const std::vector<int> *sets[][2] = {{&rnd, &rnd2}, {&uni, &rnd}, {&rnd2, &uni}};
                            for (auto &pr : sets) {
                                SlabPlan p2(g, nrk, *pr[0], *pr[1], chunk, (int)(seed >> 20) % 7);
                                Replay r2{nz, oz, tz, nrk, Nz, ""};
                                if (!r2.run(p2.ops)) {
                                    printf("FAIL (sized slabs) nz=%d oz=%d tz=%d nrk=%d body=%d chunk=%d: %s\n",
                                           nz, oz, tz, nrk, body, chunk, r2.err.c_str());
                                    return 1;
                                }
                                checked++;
                            }
                        }
    printf("ok %d\n", checked);
    return 0;
}
