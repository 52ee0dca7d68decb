"""Seeded synthetic initial conditions for the solver's benchmark workloads.

The reference ships no datasets; its problems are analytic.  These generators
produce host arrays in the reference layout (one float64 array per variable,
x fastest, ``off`` ghost cells per side, ghosts filled periodically) for:

* ``riemann_1d``  - a seeded 1D Riemann problem (2048 cells, discontinuity at
  x=0.5; left/right rho,p ~ U[0.1,1], v ~ U[-1,1]^3, By,Bz ~ U[-1,1], shared
  Bx ~ U[0.5,1], gamma=2).
* ``turbulence_2d`` - a periodic [0,1]^2 box: rho=1, p=1/gamma, velocity and
  Az each a sum of 16 random-phase Fourier modes with 0<|k|<=8 and amplitude
  ~|k|^-2; v_rms set, B_rms from plasma beta.
* ``turbulence_3d`` - a periodic [0,1]^3 box: rho=1 with a 1% random-phase
  perturbation (|k|<=6), solenoidal random-phase velocity at a given rms sonic
  Mach, B = B0 + curl A with A at 10% of |B0|, beta=1 w.r.t. |B0|^2.
* ``mrx_2d`` - the reference's magnetic-reconnection problem (Harris sheet,
  2048 x 256 cells, x periodic, y walls), seeded where it seeds from the clock.

Face-centred B is built as the discrete curl of an edge-centred vector
potential with the scheme's own face-to-centre difference (2-point for
order<=2, the (27,-1)/24 stencil for order>=3, reference mhd_fd_ct_3d.c:80-88),
so the scheme's discrete div B vanishes to round-off from the first step.
"""
from __future__ import annotations

import numpy as np

VARS3 = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
VARS1 = ("ro", "mx", "my", "mz", "en", "by", "bz")


def _modes(rng, ndim, nmodes, kmax):
    """Random integer wave vectors with 0 < |k| <= kmax."""
    out = []
    while len(out) < nmodes:
        k = rng.integers(-kmax, kmax + 1, size=ndim)
        kk = float(np.sqrt((k * k).sum()))
        if 0 < kk <= kmax:
            out.append(k)
    return np.array(out, dtype=np.int64)


def _trig(k, ph, axes):
    """cos and sin of 2*pi*k.x + ph on the tensor grid of 1D coordinate
    vectors `axes` = (x, y[, z]), returned with array axes ordered (z, y, x),
    built by angle addition from 1D factors (no full-grid transcendental)."""
    c = s = None
    for kc, ax in zip(k, axes):
        a = 2.0 * np.pi * float(kc) * ax
        ca, sa = np.cos(a), np.sin(a)
        if c is None:
            c, s = ca * np.cos(ph) - sa * np.sin(ph), sa * np.cos(ph) + ca * np.sin(ph)
        else:
            # prepend a new (slower) array axis for this coordinate
            shp = (-1,) + (1,) * c.ndim
            ca, sa = ca.reshape(shp), sa.reshape(shp)
            c, s = ca * c - sa * s, sa * c + ca * s
    return c, s


def _field(rng, axes, nmodes, kmax, slope=-2.0):
    """Sum of random-phase cosine modes, amplitude ~ |k|^slope, on the tensor
    grid of 1D coordinate vectors `axes` (x first)."""
    ks = _modes(rng, len(axes), nmodes, kmax)
    phases = rng.uniform(0.0, 2.0 * np.pi, size=nmodes)
    f = 0.0
    for k, ph in zip(ks, phases):
        c, _ = _trig(k, ph, axes)
        f = f + (float(np.sqrt((k * k).sum())) ** slope) * c
    return f


def _ddx(f, axis, n, odr):
    """Scheme difference of a periodic staggered field along `axis`: value at
    index i uses f[i-1..i+2] (face-to-centre or edge-to-face), divided by 1/n."""
    f1 = f
    f2 = np.roll(f, -1, axis=axis)
    if odr <= 2 or odr > 4:  # 5, 6: MUSCL codes, 2nd-order differences
        d = f2 - f1
    else:
        f0 = np.roll(f, 1, axis=axis)
        f3 = np.roll(f, -2, axis=axis)
        d = (27.0 * (f2 - f1) - (f3 - f0)) / 24.0
    return d * n


def _center(f, axis, odr):
    """Scheme face-to-centre average (calc_bc) of a periodic face field."""
    f1 = f
    f2 = np.roll(f, -1, axis=axis)
    if odr <= 2 or odr > 4:  # 5, 6: MUSCL codes, 2nd-order differences
        return 0.5 * (f1 + f2)
    f0 = np.roll(f, 1, axis=axis)
    f3 = np.roll(f, -2, axis=axis)
    return 0.0625 * (9.0 * (f1 + f2) - (f0 + f3))


def pad_periodic(f, off):
    return np.ascontiguousarray(np.pad(f, off, mode="wrap"))


def turbulence_3d(n=64, mach=1e-2, seed=0, off=4, gamma=5.0 / 3.0, odr=4, ny=None, nz=None,
                  b0=(1.0, 0.5, 0.0), a_frac=0.1, beta=1.0, rho_pert=0.01, nmodes=16):
    """Config-3 workload.  Returns (state dict of padded arrays, meta dict)."""
    nx = n
    ny = ny or n
    nz = nz or n
    rng = np.random.default_rng(seed)
    ic = (np.arange(nx) + 0.5) / nx
    jc = (np.arange(ny) + 0.5) / ny
    kc = (np.arange(nz) + 0.5) / nz
    ifc, jfc, kfc = np.arange(nx) / nx, np.arange(ny) / ny, np.arange(nz) / nz
    B0 = np.array(b0, dtype=np.float64)
    b0abs = float(np.sqrt((B0 * B0).sum()))
    p0 = beta * 0.5 * b0abs ** 2

    # density: 1 + 1% random-phase perturbation with |k|<=6
    dr = _field(rng, (ic, jc, kc), nmodes, 6)
    ro = 1.0 + rho_pert * dr / np.sqrt(np.mean(dr * dr))

    # solenoidal velocity: v = curl(psi), analytic per mode
    cs = np.sqrt(gamma * p0 / 1.0)
    v = [np.zeros((nz, ny, nx)) for _ in range(3)]
    ks = _modes(rng, 3, nmodes, 8)
    for k in ks:
        amp = rng.normal(size=3) * float(np.sqrt((k * k).sum())) ** -2.0
        ph = rng.uniform(0, 2 * np.pi)
        _, sn = _trig(k, ph, (ic, jc, kc))
        sn = -2 * np.pi * sn
        kxp = np.cross(k.astype(np.float64), amp)  # k x psi_k
        for c in range(3):
            v[c] = v[c] + kxp[c] * sn
    vr = np.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    v = [c * (mach * cs / vr) for c in v]

    # vector potential on edges: Ax at (i, j-1/2, k-1/2), Ay at (i-1/2, j, k-1/2),
    # Az at (i-1/2, j-1/2, k); B = B0 + curl A on faces with the scheme difference
    fa = [_field(rng, (ic, jfc, kfc), nmodes, 6),
          _field(rng, (ifc, jc, kfc), nmodes, 6),
          _field(rng, (ifc, jfc, kc), nmodes, 6)]
    # arrays are (z, y, x): axis 2 = x, 1 = y, 0 = z.  Differences land one
    # half-cell over, matching the face the component lives on.
    bx = _ddx(fa[2], 1, ny, odr) - _ddx(fa[1], 0, nz, odr)
    by = _ddx(fa[0], 0, nz, odr) - _ddx(fa[2], 2, nx, odr)
    bz = _ddx(fa[1], 2, nx, odr) - _ddx(fa[0], 1, ny, odr)
    brms = np.sqrt(np.mean(bx ** 2 + by ** 2 + bz ** 2))
    scale = a_frac * b0abs / brms
    bx = B0[0] + bx * scale
    by = B0[1] + by * scale
    bz = B0[2] + bz * scale
    cxc = _center(bx, 2, odr)
    cyc = _center(by, 1, odr)
    czc = _center(bz, 0, odr)
    en = p0 / (gamma - 1.0) + 0.5 * (ro * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
                                     + (cxc ** 2 + cyc ** 2 + czc ** 2))
    st = {"ro": ro, "mx": ro * v[0], "my": ro * v[1], "mz": ro * v[2], "en": en,
          "bx": bx, "by": by, "bz": bz}
    st = {k: pad_periodic(a, off) for k, a in st.items()}
    meta = dict(dx=1.0 / nx, dy=1.0 / ny, dz=1.0 / nz, gamma=gamma, off=off, p0=p0, mach=mach,
                cs=cs, vfast=float(np.sqrt(gamma * p0 + b0abs ** 2)) + mach * cs)
    return st, meta


def turbulence_2d(n=512, seed=0, off=4, gamma=5.0 / 3.0, odr=4, ny=None, vrms=0.5, beta=1.0,
                  nmodes=16, kmax=8):
    """Config-2 workload: 2D periodic box; returns (state, meta)."""
    nx = n
    ny = ny or n
    rng = np.random.default_rng(seed)
    ic = (np.arange(nx) + 0.5) / nx
    jc = (np.arange(ny) + 0.5) / ny
    ifc, jfc = np.arange(nx) / nx, np.arange(ny) / ny
    p0 = 1.0 / gamma
    vx = _field(rng, (ic, jc), nmodes, kmax)
    vy = _field(rng, (ic, jc), nmodes, kmax)
    r = np.sqrt(np.mean(vx ** 2 + vy ** 2))
    vx, vy = vx * (vrms / r), vy * (vrms / r)
    # Az at cell corners (i-1/2, j-1/2)
    az = _field(rng, (ifc, jfc), nmodes, kmax)
    bx = _ddx(az, 0, ny, odr)
    by = -_ddx(az, 1, nx, odr)
    b2 = np.mean(_center(bx, 1, odr) ** 2 + _center(by, 0, odr) ** 2)
    scale = np.sqrt(2.0 * p0 / beta / b2)
    bx, by = bx * scale, by * scale
    bz = np.zeros_like(bx)
    ro = np.ones_like(vx)
    cxc, cyc = _center(bx, 1, odr), _center(by, 0, odr)
    en = p0 / (gamma - 1.0) + 0.5 * (ro * (vx ** 2 + vy ** 2) + (cxc ** 2 + cyc ** 2))
    st = {"ro": ro, "mx": ro * vx, "my": ro * vy, "mz": np.zeros_like(vx), "en": en,
          "bx": bx, "by": by, "bz": bz}
    st = {k: pad_periodic(a, off) for k, a in st.items()}
    meta = dict(dx=1.0 / nx, dy=1.0 / ny, gamma=gamma, off=off, p0=p0,
                vfast=float(np.sqrt(gamma * p0 + 2.0 * p0 / beta)) + vrms)
    return st, meta


MRX_TABLES = ((0,) * 8, (1, 1, -1, 1, 1, 1, -1, 1))  # 2D/MPI/MRX/global.hpp:22-23


def mrx_2d(n=2048, ny=256, seed=0, off=4, gamma=5.0 / 3.0, lx=128.0, lam=1.0, beta=0.2, b0=1.0,
           b1=0.05, dv=0.01, ro0=1.0, ro1=1.0, cfl=0.2):
    """Magnetic reconnection (2D/MPI/MRX/init.hpp:11-76, global.hpp:11-75):
    a Harris current sheet Bx = b0 tanh(y/lam), density (ro0-ro1) sech^2 + ro1
    in pressure balance with lobe beta, the X-point perturbation of amplitude
    b1 on the face fields, and a random Vy of amplitude dv per column damped
    as exp(-y^2/4lam^2).  The reference seeds that noise from the clock; here
    it comes from `seed`.  Every cell, ghosts included, takes the analytic
    value, as the reference's initialiser does.  Periodic in x, walls in y
    (MRX_TABLES); the diffusion coefficients eta0 = nu0 = lam/500."""
    nx_, ny_ = n + 2 * off, ny + 2 * off
    ly = lx * ny / n
    dx, dy = lx / n, ly / ny
    x = (np.arange(nx_) - off + 0.5) * dx - 0.5 * lx
    y = (np.arange(ny_) - off + 0.5) * dy - 0.5 * ly
    xm, ym = x - 0.5 * dx, y - 0.5 * dy
    X, Y = np.meshgrid(x, y)
    XM, YM = np.meshgrid(xm, ym)
    rng = np.random.default_rng(seed)
    dvy = rng.uniform(-dv, dv, nx_)
    ro = (ro0 - ro1) / np.cosh(Y / (lam + 1e-15)) ** 2 + ro1
    vy = dvy[None, :] * np.exp(-(Y * Y) / (4 * lam * lam))
    bxh = b0 * np.tanh(Y / (lam + 1e-15))
    pr = 0.5 * ((1.0 + beta) * b0 * b0 - bxh * bxh)
    bx = bxh - b1 * (Y / lam) * np.exp(-(XM * XM + Y * Y) / (4 * lam * lam))
    by = b1 * (X / lam) * np.exp(-(X * X + YM * YM) / (4 * lam * lam))
    g = np.exp(-(X * X + Y * Y) / (4 * lam * lam))
    bxc = bxh - b1 * (Y / lam) * g
    byc = b1 * (X / lam) * g
    en = pr / (gamma - 1) + 0.5 * (ro * vy * vy + bxc * bxc + byc * byc)
    z = np.zeros_like(ro)
    st = {"ro": ro, "mx": z.copy(), "my": ro * vy, "mz": z.copy(), "en": en, "bx": bx, "by": by,
          "bz": z.copy()}
    st = {k: np.ascontiguousarray(a, dtype=np.float64) for k, a in st.items()}
    vfast = float(np.sqrt((0.5 * gamma * beta * b0 * b0 + b0 * b0) / ro0))
    dr = min(dx, dy)
    return st, dict(dx=dx, dy=dy, gamma=gamma, off=off, vfast=vfast, cfl=cfl, dr=dr,
                    dt=cfl * dr / vfast, eta0=lam / 5e2, nu0=lam / 5e2, tables=MRX_TABLES)


def glibc_draws(seed, count):
    """The C library's srandom(seed) then count draws of random()/RAND_MAX, as
    doubles: the noise the reference's problems draw (RMI inflow,
    2D/MPI/RMI/inj_ro.hpp:34-35), so that a run can reproduce it."""
    import ctypes
    libc = ctypes.CDLL(None)
    libc.srandom.argtypes = [ctypes.c_uint]
    libc.random.restype = ctypes.c_long
    libc.srandom(seed)
    rand_max = 2147483647.0
    return np.array([float(libc.random()) / rand_max for _ in range(count)])


def rmi_2d(n=128, ny=10240, off=4, gamma=5.0 / 3.0, ma_u=100.0, beta=1e5, vref=-0.625, psi=0.1,
           ro_1=1.0, vy_1=-1.0, ro3_over_ro1=10.0, cfl=0.4):
    """Richtmyer-Meshkov instability (2D/MPI/RMI/init.hpp:11-100,
    global.hpp:11-80): a Mach-ma_u fast shock (jump conditions of the
    reference) at y = 0 in the frame moving with vref, a contact of density
    ro_3 = 10 ro_1 at y = 1 + psi cos(2 pi x), x periodic on [0, 1], y on
    [-ly/2, ly/2] with Neumann walls and the upstream inflow injected at the
    upper boundary before each step (`inflow`).  The single-mode interface of
    the reference's default (RANDOM 0)."""
    nx_, ny_ = n + 2 * off, ny + 2 * off
    lx = 1.0
    ly = lx * ny / n
    dx, dy = lx / n, ly / ny
    x = (np.arange(nx_) - off + 0.5) * dx
    y = (np.arange(ny_) - off + 0.5) * dy - 0.5 * ly
    pr_1 = (ro_1 * vy_1 * vy_1) / (gamma * ma_u * ma_u)
    b0_1 = np.sqrt(2.0 * pr_1 / beta)
    bx_1, by_1, bz_1 = b0_1, 0.0, 0.0
    a = 2.0 * (2.0 - gamma) / beta
    b = gamma * ((gamma - 1.0) * ma_u * ma_u + 2.0 / beta + 2.0)
    c = -gamma * (gamma + 1.0) * ma_u * ma_u
    r = (-b + np.sqrt(b * b - 4.0 * a * c)) / (2.0 * a)
    rr = gamma * ma_u * ma_u * (1.0 - 1.0 / r) - (r * r - 1.0) / beta + 1.0
    ro_2, vy_2, bx_2, bz_2, pr_2 = ro_1 * r, vy_1 / r, bx_1 * r, bz_1 * r, pr_1 * rr
    ro_3 = ro_1 * ro3_over_ro1
    dw = 0.5 * dy
    ypos = 1.0 + psi * np.cos(2 * np.pi * x / lx)
    X, Y = np.meshgrid(x, y)
    sf = 0.5 * (1.0 + np.tanh(Y / dw))
    ro = ro_2 + (ro_1 - ro_2) * sf
    vy = vy_2 + (vy_1 - vy_2) * sf - vref
    bx = bx_2 + (bx_1 - bx_2) * sf
    by = np.full_like(ro, by_1)
    bz = bz_2 + (bz_1 - bz_2) * sf
    pr = pr_2 + (pr_1 - pr_2) * sf
    ro = ro + (ro_3 - ro_1) * 0.5 * (1.0 + np.tanh((Y - ypos[None, :]) / dw))
    b2 = bx * bx + by * by + bz * bz
    z = np.zeros_like(ro)
    st = {"ro": ro, "mx": z.copy(), "my": ro * vy, "mz": z.copy(),
          "en": pr / (gamma - 1) + 0.5 * (ro * vy * vy + b2), "bx": bx, "by": by, "bz": bz}
    st = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in st.items()}
    vfast = float(np.sqrt((0.5 * gamma * 2.0 * pr_1 + b0_1 * b0_1) / ro_1))
    inflow = dict(ro3=ro_3, dro3=0.1 * ro_3, vy1=vy_1, bx1=bx_1, by1=by_1, bz1=bz_1, pr1=pr_1,
                  vref=vref)
    # dt: the reference takes it from cflcheck before the loop (the flow at
    # Mach 100 sets it, not vfast)
    return st, dict(dx=dx, dy=dy, gamma=gamma, off=off, vfast=vfast, cfl=cfl, dr=min(dx, dy),
                    tables=RMI_TABLES, inflow=inflow)


RMI_TABLES = ((0,) * 8, (1,) * 8)  # 2D/MPI/RMI/global.hpp:21-22


def riemann_1d(n=2048, seed=0, off=4, gamma=2.0):
    """Config-1 workload: seeded 1D Riemann problem on [0,1]; returns (state, meta)."""
    rng = np.random.default_rng(seed)
    nx = n + 2 * off
    dx = 1.0 / n
    x = (np.arange(nx) - off + 0.5) * dx
    left = x <= 0.5
    rl, rr = rng.uniform(0.1, 1.0, 2)
    pl, pr = rng.uniform(0.1, 1.0, 2)
    vl = rng.uniform(-1, 1, 3)
    vrr = rng.uniform(-1, 1, 3)
    bl = rng.uniform(-1, 1, 2)
    br = rng.uniform(-1, 1, 2)
    bx = float(rng.uniform(0.5, 1.0))
    ro = np.where(left, rl, rr)
    p = np.where(left, pl, pr)
    v = [np.where(left, vl[c], vrr[c]) for c in range(3)]
    by = np.where(left, bl[0], br[0])
    bz = np.where(left, bl[1], br[1])
    en = p / (gamma - 1) + 0.5 * (ro * (v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
                                  + (bx * bx + by * by + bz * bz))
    st = {"ro": ro, "mx": ro * v[0], "my": ro * v[1], "mz": ro * v[2], "en": en, "by": by,
          "bz": bz}
    st = {k: np.ascontiguousarray(a, dtype=np.float64) for k, a in st.items()}
    return st, dict(bx=bx, dx=dx, gamma=gamma, off=off)


def copy_state(s):
    return {k: v.copy() for k, v in s.items()}


def div_b_3d(st, dx, dy, dz, off=4, odr=4, base=None):
    """max |div B| * dx / max|B| over interior cells with the scheme
    difference; with `base`, the change of div B from that state."""
    def d(f, ax, h):
        f1 = f
        f2 = np.roll(f, -1, axis=ax)
        if odr <= 2 or odr > 4:  # 5, 6: MUSCL codes, 2nd-order differences
            return (f2 - f1) / h
        f0, f3 = np.roll(f, 1, axis=ax), np.roll(f, -2, axis=ax)
        return (27.0 * (f2 - f1) - (f3 - f0)) / 24.0 / h
    div = d(st["bx"], 2, dx) + d(st["by"], 1, dy) + d(st["bz"], 0, dz)
    if base is not None:
        div = div - (d(base["bx"], 2, dx) + d(base["by"], 1, dy) + d(base["bz"], 0, dz))
    sl = (slice(off, -off),) * 3
    bmax = max(np.abs(st[k][sl]).max() for k in ("bx", "by", "bz"))
    return float(np.abs(div[sl]).max() * min(dx, dy, dz) / bmax)


def div_b_2d(st, dx, dy, off=4, odr=4, base=None):
    """max |div B| * dx / max|B| over interior cells with the scheme
    difference; with `base`, the change of div B from that state instead
    (a CT update keeps it at round-off when the initial field is not
    discretely solenoidal)."""
    def d(f, ax, h):
        f1 = f
        f2 = np.roll(f, -1, axis=ax)
        if odr <= 2 or odr > 4:  # 5, 6: MUSCL codes, 2nd-order differences
            return (f2 - f1) / h
        f0, f3 = np.roll(f, 1, axis=ax), np.roll(f, -2, axis=ax)
        return (27.0 * (f2 - f1) - (f3 - f0)) / 24.0 / h
    div = d(st["bx"], 1, dx) + d(st["by"], 0, dy)
    if base is not None:
        div = div - (d(base["bx"], 1, dx) + d(base["by"], 0, dy))
    sl = (slice(off, -off),) * 2
    bmax = max(np.abs(st[k][sl]).max() for k in ("bx", "by"))
    return float(np.abs(div[sl]).max() * min(dx, dy) / bmax)
