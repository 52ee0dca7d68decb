// Floating-point operation counter for the CPU oracle.  TEST/MEASUREMENT
// INFRASTRUCTURE ONLY.
//
// Compiles mlau_oracle.c as C++ with `double` replaced by a counting type, so
// every +, -, *, / and sqrt the reference's algorithm performs is tallied,
// split by phase (ORACLE_PHASE hooks): 0 cell B + primitives, 1 CT weights +
// shock sensors, 2 reconstruction, 3 Riemann flux, 4 edge EMF, 5 RK update +
// CT curl.  Division and sqrt count as one operation each; compares, min,
// max, fabs and negation are not counted.  These are the algorithmic FP64
// work figures behind the roofline of each GPU kernel.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <cstdio>

namespace opc {
long long ops[8][4];  // [phase][add/sub, mul, div, sqrt]
int phase = 7;
}

struct OpD {
    double v;
    OpD() = default;
    OpD(double x) : v(x) {}
};
static inline OpD operator+(OpD a, OpD b) { opc::ops[opc::phase][0]++; return OpD(a.v + b.v); }
static inline OpD operator-(OpD a, OpD b) { opc::ops[opc::phase][0]++; return OpD(a.v - b.v); }
static inline OpD operator*(OpD a, OpD b) { opc::ops[opc::phase][1]++; return OpD(a.v * b.v); }
static inline OpD operator/(OpD a, OpD b) { opc::ops[opc::phase][2]++; return OpD(a.v / b.v); }
static inline OpD operator-(OpD a) { return OpD(-a.v); }
static inline OpD operator+(OpD a) { return a; }
static inline OpD &operator+=(OpD &a, OpD b) { a = a + b; return a; }
static inline OpD &operator-=(OpD &a, OpD b) { a = a - b; return a; }
static inline OpD &operator*=(OpD &a, OpD b) { a = a * b; return a; }
static inline OpD &operator/=(OpD &a, OpD b) { a = a / b; return a; }
static inline bool operator<(OpD a, OpD b) { return a.v < b.v; }
static inline bool operator>(OpD a, OpD b) { return a.v > b.v; }
static inline bool operator<=(OpD a, OpD b) { return a.v <= b.v; }
static inline bool operator>=(OpD a, OpD b) { return a.v >= b.v; }
static inline bool operator==(OpD a, OpD b) { return a.v == b.v; }
static inline bool operator!=(OpD a, OpD b) { return a.v != b.v; }
static inline OpD sqrt(OpD a) { opc::ops[opc::phase][3]++; return OpD(std::sqrt(a.v)); }
static inline OpD fabs(OpD a) { return OpD(std::fabs(a.v)); }
static inline bool isfinite(OpD a) { return std::isfinite(a.v); }

#define ORACLE_PHASE(p) (opc::phase = (p))
#define double OpD
#include "mlau_oracle.c"
#undef double

// Counted 3D step on caller-supplied float64 arrays (copied in and out).
extern "C" void opcount_step3d(double **st, double dt, double dx, int nx, int ny, int nz,
                               int off, double gamma, int odr, int flux, int nrk,
                               long long *out32)
{
    long n = (long)nx * ny * nz;
    OpD *a[8];
    for (int v = 0; v < 8; v++) {
        a[v] = (OpD *)malloc(sizeof(OpD) * n);
        for (long s = 0; s < n; s++) a[v][s] = OpD(st[v][s]);
    }
    std::memset(opc::ops, 0, sizeof(opc::ops));
    oracle_fd_ct_3d(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], dt, dx, dx, dx, nx, ny, nz,
                    off, off, off, gamma, odr, flux, nrk);
    std::memcpy(out32, opc::ops, sizeof(opc::ops));
    for (int v = 0; v < 8; v++) {
        for (long s = 0; s < n; s++) st[v][s] = a[v][s].v;
        free(a[v]);
    }
}

extern "C" void opcount_step2d(double **st, double dt, double dx, int nx, int ny, int off,
                               double gamma, int odr, int flux, int nrk, long long *out32)
{
    long n = (long)nx * ny;
    OpD *a[8];
    for (int v = 0; v < 8; v++) {
        a[v] = (OpD *)malloc(sizeof(OpD) * n);
        for (long s = 0; s < n; s++) a[v][s] = OpD(st[v][s]);
    }
    std::memset(opc::ops, 0, sizeof(opc::ops));
    oracle_fd_ct_2d(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], dt, dx, dx, nx, ny, off, off,
                    gamma, odr, flux, nrk);
    std::memcpy(out32, opc::ops, sizeof(opc::ops));
    for (int v = 0; v < 8; v++) {
        for (long s = 0; s < n; s++) st[v][s] = a[v][s].v;
        free(a[v]);
    }
}
