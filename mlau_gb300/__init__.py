"""GB300-native (sm_103a) MHD step library: Python binding of libmlau_gb300.so.

The compute path is the CUDA library built in-tree by ``mlau_gb300._build``;
this module only binds its C ABI (include/mlau_gb300.h) with ctypes.  There is
no CPU fallback: if the library is missing, loading raises.

Two call styles, as in the C ABI:

* reference-style drivers that update numpy arrays in place, with the
  reference's argument lists: ``mhd_fd_ct_3d``, ``mhd_fd_ct_2d``,
  ``mhd_fd4c_1d`` (each call: host -> GPU, one RK step, GPU -> host);
* ``Sim``, a device-resident simulation handle for the fast path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libmlau_gb300.so")

FLUX = {"mlau": 0, "lhlld": 1, "hlld": 2, "roe": 3}
EIGEN = {"full": 0, "miyoshi": 1}
FP64, FP32_SPLIT, FP32_SPLIT_F64 = 0, 1, 2
OUT_F64, OUT_F32_RANK = 0, 1
BC1D = {"open": 0, "periodic": 1}
VARS = ("ro", "mx", "my", "mz", "en", "bx", "by", "bz")
KERNEL_KINDS = ("prim", "aux", "rec", "flux", "emf", "update", "copy", "cfl",
                "split_sweep", "split_prep", "split_update")


class MlauError(RuntimeError):
    pass


_lib = None


def _bind(lib):
    d, i, vp = C.c_double, C.c_int, C.c_void_p
    pd = C.POINTER(C.c_double)
    lib.mlau_last_error.restype = C.c_char_p
    lib.mlau_clear_error.restype = None
    lib.mlau_sim_create.argtypes = [C.POINTER(vp), i, i, i, i, i, i, i, d, d, d, d, i, i, i, i]
    lib.mlau_sim_destroy.argtypes = [vp]
    lib.mlau_sim_upload.argtypes = [vp, C.POINTER(pd)]
    lib.mlau_sim_download.argtypes = [vp, C.POINTER(pd)]
    lib.mlau_sim_set_bx_1d.argtypes = [vp, d]
    lib.mlau_sim_set_bc_1d.argtypes = [vp, i]
    lib.mlau_sim_set_eigen.argtypes = [vp, i]
    lib.mlau_set_eigen.argtypes = [i, i]
    lib.mlau_sim_set_bc_2d.argtypes = [vp, C.POINTER(i), C.POINTER(i)]
    lib.mlau_sim_set_bc_3d.argtypes = [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
    lib.mlau_sim_step.argtypes = [vp, d, i]
    lib.mlau_sim_resistive_2d.argtypes = [vp, d, d]
    lib.mlau_sim_viscous_2d.argtypes = [vp, d, d]
    lib.mlau_sim_conduction_2d.argtypes = [vp, d, d, C.POINTER(i)]
    lib.mlau_sim_inject_2d.argtypes = [vp] + [d] * 8 + [vp]
    lib.mlau_sim_cfl.argtypes = [vp, d, d, d, d, pd, pd]
    lib.mlau_sim_sync.argtypes = [vp]
    lib.mlau_sim_stream.argtypes = [vp]
    lib.mlau_sim_stream.restype = vp
    lib.mlau_sim_device_ptr.argtypes = [vp, i, C.POINTER(pd)]
    lib.mlau_sim_set_timing.argtypes = [vp, i]
    lib.mlau_sim_timing.argtypes = [vp, i, C.POINTER(C.c_long), pd]
    lib.mlau_sim_device_bytes.argtypes = [vp]
    lib.mlau_sim_device_bytes.restype = C.c_longlong
    lib.mlau_sim_launches_per_step.argtypes = [vp]
    lib.mlau_sim_time_steps.argtypes = [vp, d, i, pd]
    lib.mlau_measure_fma_peaks.argtypes = [pd, pd]
    lib.mlau_pin_host.argtypes = [vp, C.c_longlong]
    lib.mlau_unpin_host.argtypes = [vp]
    lib.mlau_set_device.argtypes = [i]
    lib.mlau_device_pci_bus_id.argtypes = [i, C.c_char_p, i]
    cp = C.c_char_p
    lib.mlau_sim_bkup_save.argtypes = [vp, cp, i, i, d, d, d, i]
    lib.mlau_sim_bkup_load.argtypes = [vp, cp, C.POINTER(i), C.POINTER(i), pd, pd, pd, i]
    lib.mlau_sim_outdat.argtypes = [vp, cp, i, i, i]
    lib.mlau_outdat_meta.argtypes = [cp, i, i, d, d, d, i, i, i]
    pi = C.POINTER(C.c_int)
    lib.mlau_batch_create.argtypes = [C.POINTER(vp), i, pi, pi, i, pd, pd, pd, pi, pd, pd, i]
    lib.mlau_batch_open.argtypes = [C.POINTER(vp), i, C.c_longlong, i, i, i]
    lib.mlau_batch_add.argtypes = [vp, i, i, d, d, d, i, d, d, C.POINTER(pd), pi]
    lib.mlau_batch1d_open.argtypes = [C.POINTER(vp), C.c_longlong, i, i, i]
    lib.mlau_batch1d_add.argtypes = [vp, i, d, d, d, i, i, i, d, d, C.POINTER(pd), pi]
    lib.mlau_batch_remove.argtypes = [vp, i]
    lib.mlau_batch_destroy.argtypes = [vp]
    lib.mlau_batch_upload.argtypes = [vp, i, C.POINTER(pd)]
    lib.mlau_batch_download.argtypes = [vp, i, C.POINTER(pd)]
    lib.mlau_batch_set_fixed_dt.argtypes = [vp, i, d]
    lib.mlau_batch_set_bc.argtypes = [vp, i, C.POINTER(i), C.POINTER(i)]
    lib.mlau_batch_set_tile.argtypes = [vp, i, i]
    lib.mlau_batch_autotune.argtypes = [vp, i, pi, pi, pd]
    lib.mlau_batch_run.argtypes = [vp, i, i, pi, pd]
    lib.mlau_batch_info.argtypes = [vp, i, pd, pi, pi]
    lib.mlau_batch_status.argtypes = [vp, i]
    lib.mlau_batch_set_grid.argtypes = [vp, i]
    lib.mlau_batch_max_grid.argtypes = [vp]
    for f in ("mlau_batch_cells", "mlau_batch_device_bytes", "mlau_batch_launches"):
        getattr(lib, f).argtypes = [vp]
        getattr(lib, f).restype = C.c_longlong
    lib.mlau_set_scheme.argtypes = [i, i, i, i]
    lib.mlau_set_bc_1d.argtypes = [i]
    lib.mlau_set_precision.argtypes = [i, i]
    lib.mlau_release_dropin.restype = None
    lib.mhd_fd_ct_3d.argtypes = [pd] * 8 + [d] * 4 + [i] * 6 + [d] + [i] * 4
    lib.mhd_fd_ct_3d.restype = None
    lib.mhd_fd_ct_2d.argtypes = [pd] * 8 + [d] * 3 + [i] * 4 + [d]
    lib.mhd_fd_ct_2d.restype = None
    lib.mhd_fd4c_1d.argtypes = [pd] * 7 + [d] * 3 + [i, i, d]
    lib.diff_ctfield_e.argtypes = [pd] * 4 + [d] * 4 + [i] * 4 + [d] + [i] * 3
    lib.diff_ctfield_e.restype = None
    lib.ns_viscous_2d.argtypes = [pd] * 5 + [d] * 4 + [i] * 4 + [d] + [i] * 3
    lib.ns_viscous_2d.restype = None
    lib.t_conduction.argtypes = [pd] * 8 + [d] * 4 + [i] * 4 + [d] + [i] * 3
    lib.t_conduction.restype = None
    lib.mhd_fd4c_1d.restype = None
    return lib


def lib():
    """The loaded library; raises MlauError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MlauError(f"{LIB_PATH} is missing: build it with "
                            "`python -c 'import __graft_entry__ as g; g.build()'`")
        _lib = _bind(C.CDLL(LIB_PATH))
    return _lib


def last_error() -> str:
    return lib().mlau_last_error().decode(errors="replace")


def _check(rc):
    if rc != 0:
        raise MlauError(f"mlau error {rc}: {last_error()}")


def _ptr(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise MlauError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _flux(f):
    return FLUX[f] if isinstance(f, str) else int(f)


# --- reference-style drivers --------------------------------------------------
def set_scheme(dim: int, odr: int, flux="lhlld", nrk: int = 3):
    _check(lib().mlau_set_scheme(dim, odr, _flux(flux), nrk))


def set_bc_1d(bc: str):
    _check(lib().mlau_set_bc_1d(BC1D[bc]))


def set_eigen(dim: int, eig: str):
    """Eigen-system of the drop-in drivers where Mach^2 >= 1 ("full" or
    "miyoshi")."""
    _check(lib().mlau_set_eigen(dim, EIGEN[eig]))


def set_precision(dim: int, precision: int):
    _check(lib().mlau_set_precision(dim, precision))


def release_dropin():
    lib().mlau_release_dropin()


def mhd_fd_ct_3d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, dz, nx, ny, nz, xoff, yoff, zoff,
                 gamma, mpi_rank=0, mpi_numx=1, mpi_numy=1, mpi_numz=1):
    """Reference 3D/MPI/OTvortex/mhd_fd_ct_3d.c:99-103 signature; in place."""
    before = _clear()
    lib().mhd_fd_ct_3d(*[_ptr(a) for a in (ro, mx, my, mz, en, bx, by, bz)], dt, dx, dy, dz, nx, ny,
                   nz, xoff, yoff, zoff, gamma, mpi_rank, mpi_numx, mpi_numy, mpi_numz)
    _raise_if_new(before)


def mhd_fd_ct_2d(ro, mx, my, mz, en, bx, by, bz, dt, dx, dy, nx, ny, xoff, yoff, gamma):
    """Reference 2D/SERIAL/OTvortex/mhd_fd_ct_2d.c:91-94 signature; in place."""
    before = _clear()
    lib().mhd_fd_ct_2d(*[_ptr(a) for a in (ro, mx, my, mz, en, bx, by, bz)], dt, dx, dy, nx, ny,
                       xoff, yoff, gamma)
    _raise_if_new(before)


def mhd_fd4c_1d(ro, mx, my, mz, en, by, bz, bx, dt, dx, nx, xoff, gamma):
    """Reference 1D/SERIAL/shock/mhd_fd4c_1d.c:60-63 signature; in place."""
    before = _clear()
    lib().mhd_fd4c_1d(*[_ptr(a) for a in (ro, mx, my, mz, en, by, bz)], bx, dt, dx, nx, xoff,
                      gamma)
    _raise_if_new(before)


def _clear():
    lib().mlau_clear_error()
    return ""


def _raise_if_new(before):
    # The void drivers report failures through mlau_last_error(), which is
    # cleared before each call.
    after = last_error()
    if after and after != before:
        raise MlauError(after)


def measure_fma_peaks():
    """(FP64, FP32) FMA throughput of the current GPU in flop/s."""
    a, b = C.c_double(), C.c_double()
    _check(lib().mlau_measure_fma_peaks(C.byref(a), C.byref(b)))
    return a.value, b.value


def set_device(dev: int):
    _check(lib().mlau_set_device(dev))


def local_cpus(dev: int = 0):
    """The host CPUs attached to a device's PCI root (Linux sysfs), or None
    where that is not known.  Host arrays first touched by a thread on these
    CPUs sit on the device's own memory node, which is what keeps per-step
    host<->device copies at the link's full speed on multi-socket hosts."""
    buf = C.create_string_buffer(64)
    if lib().mlau_device_pci_bus_id(dev, buf, 64) != 0:
        return None
    parts = buf.value.decode().lower().split(":")
    if len(parts) != 3:
        return None
    bus = f"{int(parts[0], 16):04x}:{parts[1]}:{parts[2]}"
    try:
        with open(f"/sys/bus/pci/devices/{bus}/local_cpulist") as fh:
            spec = fh.read().strip()
    except OSError:
        return None
    cpus = set()
    for part in spec.split(","):
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        elif part:
            cpus.add(int(part))
    return cpus or None


def pin(arr: np.ndarray):
    _check(lib().mlau_pin_host(arr.ctypes.data, arr.nbytes))


def unpin(arr: np.ndarray):
    _check(lib().mlau_unpin_host(arr.ctypes.data))


def outdat_meta(dir: str, dim: int, first: bool, tim: float, gamma: float, bx: float = 0.0,
                xoff: int = 4, yoff: int = 4, zoff: int = 4):
    """params.dat / offsets.dat (1D: xoff.dat) and t.dat as the reference's
    output routines write them."""
    _check(lib().mlau_outdat_meta(os.fsencode(dir), dim, int(first), tim, gamma, bx, xoff, yoff,
                                  zoff))


# --- device-resident handle ---------------------------------------------------
class Sim:
    """A simulation resident on the GPU (handle API of include/mlau_gb300.h)."""

    def __init__(self, dim, shape, off=4, dx=1.0, dy=1.0, dz=1.0, gamma=5 / 3, odr=4,
                 flux="mlau", nrk=3, precision=FP64):
        shape = tuple(shape)
        if dim == 3:
            nz, ny, nx = shape
        elif dim == 2:
            (ny, nx), nz = shape, 1
        else:
            (nx,), ny, nz = shape, 1, 1
        self.dim, self.shape, self.off = dim, shape, off
        h = C.c_void_p()
        _check(lib().mlau_sim_create(C.byref(h), dim, nx, ny, nz, off, off if dim >= 2 else 0,
                                     off if dim == 3 else 0, dx, dy, dz, gamma, odr, _flux(flux),
                                     nrk, precision))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            lib().mlau_sim_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _vars(self):
        return VARS if self.dim != 1 else ("ro", "mx", "my", "mz", "en", None, "by", "bz")

    def upload(self, state: dict):
        ptrs = (C.POINTER(C.c_double) * 8)()
        keep = []
        for v, k in enumerate(self._vars()):
            if k is None:
                continue
            a = np.ascontiguousarray(state[k], dtype=np.float64)
            if a.shape != self.shape:
                raise MlauError(f"{k}: shape {a.shape} != {self.shape}")
            keep.append(a)
            ptrs[v] = _ptr(a)
        _check(lib().mlau_sim_upload(self._h, ptrs))
        _check(lib().mlau_sim_sync(self._h))

    def download(self, out: dict | None = None) -> dict:
        out = out if out is not None else {}
        ptrs = (C.POINTER(C.c_double) * 8)()
        for v, k in enumerate(self._vars()):
            if k is None:
                continue
            if k not in out:
                out[k] = np.empty(self.shape, dtype=np.float64)
            ptrs[v] = _ptr(out[k])
        _check(lib().mlau_sim_download(self._h, ptrs))
        return out

    # --- the reference's checkpoint and output files ---
    def bkup_save(self, dir: str, n: int, cnt: int, tim: float, dt: float, trec: float,
                  rank: int = 0):
        _check(lib().mlau_sim_bkup_save(self._h, os.fsencode(dir), n, cnt, tim, dt, trec, rank))

    def bkup_load(self, dir: str, rank: int = 0):
        """(n, cnt, tim, dt, trec) of the loaded checkpoint, or None when the
        directory holds none."""
        n, cnt = C.c_int(), C.c_int()
        tim, dt, trec = C.c_double(), C.c_double(), C.c_double()
        rc = lib().mlau_sim_bkup_load(self._h, os.fsencode(dir), C.byref(n), C.byref(cnt),
                                      C.byref(tim), C.byref(dt), C.byref(trec), rank)
        if rc == 1:
            return None
        _check(rc)
        return n.value, cnt.value, tim.value, dt.value, trec.value

    def outdat(self, dir: str, cnt: int, rank: int = 0, format: int = OUT_F64):
        _check(lib().mlau_sim_outdat(self._h, os.fsencode(dir), cnt, rank, format))

    def set_bx(self, bx: float):
        _check(lib().mlau_sim_set_bx_1d(self._h, bx))

    def set_bc(self, bc: str):
        _check(lib().mlau_sim_set_bc_1d(self._h, BC1D[bc]))

    def set_eigen(self, eig: str):
        """Eigen-system where Mach^2 >= 1: "full" (the drivers') or
        "miyoshi" (mhd_m_reconst)."""
        _check(lib().mlau_sim_set_eigen(self._h, EIGEN[eig]))

    def set_bc3d(self, dnx, dny, dnz):
        """3D boundary tables (8 entries each, order ro mx my mz en bx by bz;
        0 periodic, -1 Dirichlet, +1 Neumann; each axis all zero or all
        nonzero)."""
        t = [(C.c_int * 8)(*[int(v) for v in a]) for a in (dnx, dny, dnz)]
        _check(lib().mlau_sim_set_bc_3d(self._h, *t))

    def set_bc2d(self, dnx, dny):
        """2D boundary tables (8 entries each, order ro mx my mz en bx by bz;
        0 periodic, -1 Dirichlet, +1 Neumann)."""
        tx = (C.c_int * 8)(*[int(v) for v in dnx])
        ty = (C.c_int * 8)(*[int(v) for v in dny])
        _check(lib().mlau_sim_set_bc_2d(self._h, tx, ty))

    def step(self, dt: float, nsteps: int = 1):
        _check(lib().mlau_sim_step(self._h, dt, nsteps))

    def resistive(self, eta0: float, dt: float):
        """Resistive diffusion of B (with the energy) over dt, 2D FP64."""
        _check(lib().mlau_sim_resistive_2d(self._h, eta0, dt))

    def viscous(self, nu0: float, dt: float):
        """Viscosity of the velocity (with the energy) over dt, 2D FP64."""
        _check(lib().mlau_sim_viscous_2d(self._h, nu0, dt))

    def inject(self, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref, noise=None):
        """The RMI inflow at the upper boundary (inj_ro) and the periodic
        exchange that follows it; noise: yoff*nx uniform draws or None."""
        nz = None
        if noise is not None:
            nz = np.ascontiguousarray(noise, dtype=np.float64)
            if nz.size < self.shape[-1] * self.off:
                raise MlauError("noise needs yoff * nx draws")
        _check(lib().mlau_sim_inject_2d(self._h, ro3, dro3, vy1, bx1, by1, bz1, pr1, vref,
                                        None if nz is None else nz.ctypes.data))

    def conduction(self, kk0: float, dt: float) -> int:
        """Anisotropic heat conduction along B over dt, 2D FP64; returns the
        Gauss-Seidel sweep count (MlauError when 2048 sweeps did not
        converge; the energy is then as the reference leaves it)."""
        n = C.c_int(0)
        _check(lib().mlau_sim_conduction_2d(self._h, kk0, dt, C.byref(n)))
        return n.value

    def sync(self):
        _check(lib().mlau_sim_sync(self._h))

    def cfl(self, cfl, dr, vfast, dt_old=0.0):
        dt, vm = C.c_double(), C.c_double()
        _check(lib().mlau_sim_cfl(self._h, cfl, dr, vfast, dt_old, C.byref(dt), C.byref(vm)))
        return dt.value, vm.value

    @property
    def stream(self) -> int:
        return lib().mlau_sim_stream(self._h) or 0

    def device_ptr(self, var: str) -> int:
        p = C.POINTER(C.c_double)()
        _check(lib().mlau_sim_device_ptr(self._h, VARS.index(var), C.byref(p)))
        return C.cast(p, C.c_void_p).value

    def set_timing(self, on: bool):
        _check(lib().mlau_sim_set_timing(self._h, int(on)))

    def timing(self) -> dict:
        out = {}
        for k, name in enumerate(KERNEL_KINDS):
            n, ms = C.c_long(), C.c_double()
            _check(lib().mlau_sim_timing(self._h, k, C.byref(n), C.byref(ms)))
            if n.value:
                out[name] = (n.value, ms.value)
        return out

    def time_steps(self, dt: float, nsteps: int) -> float:
        """Device time (ms) of nsteps steps, CUDA events on the simulation's stream."""
        ms = C.c_double()
        _check(lib().mlau_sim_time_steps(self._h, dt, nsteps, C.byref(ms)))
        return ms.value

    @property
    def device_bytes(self) -> int:
        return int(lib().mlau_sim_device_bytes(self._h))

    @property
    def launches_per_step(self) -> int:
        return int(lib().mlau_sim_launches_per_step(self._h))


VARS_1D = ("ro", "mx", "my", "mz", "en", None, "by", "bz")


class Batch:
    """Batched engine (include/mlau_gb300.h section 5): slots of periodic 2D
    instances with their own size, solver, gamma, CFL dt and end time, or (a
    1D engine) of 1D problems stepped like mhd_fd4c_1d.

    Batch(shapes, ...) fills one slot per shape (FP32-split); Batch.open(...)
    makes an empty 2D engine that admits instances with add(); Batch.open1d()
    an empty 1D engine that admits them with add1d()."""

    def __init__(self, shapes=None, dx=None, dy=None, gamma=None, flux=None, cfl=None,
                 t_end=None, off=4, odr=4, _handle=None, _dim=2):
        self.shapes = {}
        self.dim = _dim
        if _handle is not None:
            self._h = _handle
            return
        n = len(shapes)
        ai = lambda xs: (C.c_int * n)(*[int(x) for x in xs])
        ad = lambda xs: (C.c_double * n)(*[float(x) for x in xs])
        h = C.c_void_p()
        _check(lib().mlau_batch_create(
            C.byref(h), n, ai([s[1] for s in shapes]), ai([s[0] for s in shapes]), off, ad(dx),
            ad(dy), ad(gamma), ai([_flux(f) for f in flux]), ad(cfl), ad(t_end), odr))
        self._h = h
        self.shapes = {k: tuple(s) for k, s in enumerate(shapes)}

    @classmethod
    def open(cls, capacity_cells, max_inst, precision=FP32_SPLIT, off=4, odr=4):
        h = C.c_void_p()
        _check(lib().mlau_batch_open(C.byref(h), precision, int(capacity_cells), max_inst, off,
                                     odr))
        return cls(_handle=h)

    @classmethod
    def open1d(cls, capacity_cells, max_inst, off=4, odr=2):
        h = C.c_void_p()
        _check(lib().mlau_batch1d_open(C.byref(h), int(capacity_cells), max_inst, off, odr))
        return cls(_handle=h, _dim=1)

    @property
    def _vars(self):
        return VARS_1D if self.dim == 1 else VARS

    def _ptrs(self, state, shape):
        keep, ptrs = [], (C.POINTER(C.c_double) * 8)()
        for v, name in enumerate(self._vars):
            if name is None:
                continue
            a = np.ascontiguousarray(state[name], dtype=np.float64)
            if a.shape != shape:
                raise MlauError(f"{name}: shape {a.shape} != {shape}")
            keep.append(a)
            ptrs[v] = _ptr(a)
        return keep, ptrs

    def add1d(self, state, dx, bx, gamma, flux="mlau", nrk=3, bc="open", cfl=0.4, t_end=0.1):
        """Admit a 1D problem (state: ro, mx, my, mz, en, by, bz with ghosts);
        returns its slot, or None when the engine is full."""
        shape = np.shape(state["ro"])
        keep, ptrs = self._ptrs(state, shape)
        slot = C.c_int()
        rc = lib().mlau_batch1d_add(self._h, shape[0], dx, bx, gamma, _flux(flux), nrk,
                                    BC1D[bc] if isinstance(bc, str) else int(bc), cfl, t_end,
                                    ptrs, C.byref(slot))
        if rc == -3:
            return None
        _check(rc)
        self.shapes[slot.value] = tuple(shape)
        return slot.value

    def add(self, state, dx, dy, gamma, flux, cfl, t_end):
        """Admit an instance; returns its slot, or None when the engine is full."""
        shape = state["ro"].shape
        keep = [np.ascontiguousarray(state[v], dtype=np.float64) for v in VARS]
        ptrs = (C.POINTER(C.c_double) * 8)(*[_ptr(a) for a in keep])
        slot = C.c_int()
        rc = lib().mlau_batch_add(self._h, shape[1], shape[0], dx, dy, gamma, _flux(flux), cfl,
                                  t_end, ptrs, C.byref(slot))
        if rc == -3:
            return None
        _check(rc)
        self.shapes[slot.value] = tuple(shape)
        return slot.value

    def remove(self, k):
        _check(lib().mlau_batch_remove(self._h, k))
        self.shapes.pop(k, None)

    def close(self):
        if getattr(self, "_h", None):
            lib().mlau_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, k, state):
        keep, ptrs = self._ptrs(state, self.shapes[k])
        _check(lib().mlau_batch_upload(self._h, k, ptrs))

    def download(self, k):
        out = {v: np.empty(self.shapes[k]) for v in self._vars if v is not None}
        ptrs = (C.POINTER(C.c_double) * 8)()
        for v, name in enumerate(self._vars):
            if name is not None:
                ptrs[v] = _ptr(out[name])
        _check(lib().mlau_batch_download(self._h, k, ptrs))
        return out

    def set_fixed_dt(self, k, dt):
        _check(lib().mlau_batch_set_fixed_dt(self._h, k, dt))

    def set_bc(self, k, dnx, dny):
        """Boundary tables (the problem's dnxs, dnys) of 2D instance k."""
        tab = lambda t: (C.c_int * 8)(*[int(x) for x in t])
        _check(lib().mlau_batch_set_bc(self._h, k, tab(dnx), tab(dny)))

    def set_tile(self, tw, th):
        _check(lib().mlau_batch_set_tile(self._h, tw, th))

    def set_grid(self, nblocks):
        """Blocks of the persistent step kernel (0: all that fit); returns the
        grid actually used."""
        rc = lib().mlau_batch_set_grid(self._h, int(nblocks))
        if rc < 0:
            _check(rc)
        return rc

    @property
    def max_grid(self):
        return int(lib().mlau_batch_max_grid(self._h))

    def autotune(self, steps=2):
        tw, th, ms = C.c_int(), C.c_int(), C.c_double()
        _check(lib().mlau_batch_autotune(self._h, steps, C.byref(tw), C.byref(th), C.byref(ms)))
        return tw.value, th.value, ms.value

    def run(self, max_steps, steps_per_graph=0):
        left, ms = C.c_int(), C.c_double()
        _check(lib().mlau_batch_run(self._h, max_steps, steps_per_graph, C.byref(left),
                                    C.byref(ms)))
        return left.value, ms.value

    def info(self, k):
        t, st, act = C.c_double(), C.c_int(), C.c_int()
        _check(lib().mlau_batch_info(self._h, k, C.byref(t), C.byref(st), C.byref(act)))
        return t.value, st.value, bool(act.value)

    def failed(self, k) -> bool:
        """True when instance k retired on a bad state (NaN, or density or
        pressure not positive)."""
        rc = lib().mlau_batch_status(self._h, k)
        if rc not in (0, -4):
            _check(rc)
        return rc == -4

    @property
    def cells(self):
        return int(lib().mlau_batch_cells(self._h))

    @property
    def device_bytes(self):
        return int(lib().mlau_batch_device_bytes(self._h))

    @property
    def launches(self):
        return int(lib().mlau_batch_launches(self._h))
