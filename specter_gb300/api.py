"""Host-side mirror of SPECTER's fftp / pseudo / boundary module interfaces over the C ABI.

Names, argument order and meaning follow the reference routines (src/fftp/fftp.fpp,
src/pseudo/pseudospec_hd.f90, pseudospec_phd.f90, src/boundary/*.f90); the MPI communicator
argument has no counterpart.  Host arrays use the reference layouts:
  complex spectral / mixed fields: numpy (nx/2+1, ny, nz) C order  == Fortran C(nz, ny, nx/2+1)
  real physical fields:            numpy (nz, ny, nx)     C order  == Fortran R(nx, ny, nz)
in the plan's precision (complex128/float64 for FP64, complex64/float32 for FP32).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import SolverParams, SpecterError, check, load

TABLES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tables")
FP64, FP32 = 0, 1
COMPLEX, REAL = 0, 1
HD, BOUSS, ROTBOUSS = 0, 1, 2


def _pd(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def set_device(device: int) -> None:
    """CUDA device for plans created afterwards on this thread."""
    check(load().specter_set_device(int(device)))


class Plan:
    """fcgram_create_plan (src/fftp/fcgram_mod.f90:49-144) plus the grid / kes setup
    (src/specter.fpp:683-800).  n = (nx, ny, nz) with nz the total z size (physical + Cz)."""

    def __init__(self, n, c=(0, 0, 25), o=(0, 0, 5), lengths=(1.0, 1.0, 1.0), tdir=None, precision=FP64):
        L = load()
        self._L = L
        h = C.c_void_p()
        n3 = (C.c_int * 3)(*n)
        c3 = (C.c_int * 3)(*c)
        o3 = (C.c_int * 3)(*o)
        l3 = (C.c_double * 3)(*lengths)
        check(L.specter_plan_create(n3, c3, o3, l3, (tdir or TABLES).encode(), int(precision), C.byref(h)))
        self.h = h
        info = (C.c_int * 8)()
        check(L.specter_plan_info(h, info))
        self.nx, self.ny, self.nz, self.cz, self.oz, self.nxh, self.ldx, self.precision = list(info)
        self.nzp = self.nz - self.cz
        eng = (C.c_int * 12)()
        check(L.specter_plan_engines(h, eng))
        # per axis: working length, four-step split (L1, L2; 0 = generic engine), Bluestein flag
        self.engines = {ax: dict(L=eng[4 * i], L1=eng[4 * i + 1], L2=eng[4 * i + 2], bluestein=bool(eng[4 * i + 3]))
                        for i, ax in enumerate("xyz")}
        self.lengths = tuple(lengths)
        self.rdtype = np.float64 if self.precision == FP64 else np.float32
        self.cdtype = np.complex128 if self.precision == FP64 else np.complex64
        kx, ky, kz, z = np.zeros(self.nxh), np.zeros(self.ny), np.zeros(self.nz), np.zeros(self.nz)
        d = np.zeros(self.cz * self.oz)
        check(L.specter_plan_arrays(h, _pd(kx), _pd(ky), _pd(kz), _pd(z), _pd(d)))
        self.kx, self.ky, self.kz, self.z = kx, ky, kz, z
        self.dir = d.reshape(self.oz, self.cz).T.copy()

    def close(self):
        if getattr(self, "h", None):
            self._L.specter_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def sshape(self):
        return (self.nxh, self.ny, self.nz)

    @property
    def rshape(self):
        return (self.nz, self.ny, self.nx)

    def field(self, kind=COMPLEX, data=None) -> "Field":
        f = Field(self, kind)
        if data is not None:
            f.upload(data)
        return f

    def synchronize(self):
        check(self._L.specter_plan_synchronize(self.h))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(self._L.specter_plan_stream(self.h, C.byref(s)))
        return s.value or 0

    def timers(self):
        out = (C.c_double * 6)()
        check(self._L.specter_timers(self.h, out))
        return list(out)

    def profile(self, enable=True):
        """Bracket every kernel launch with CUDA events (resets the per-kernel report)."""
        check(self._L.specter_profile(self.h, 1 if enable else 0))

    def profile_report(self):
        """{kernel: (launches, total_ms, algorithmic_bytes)} since profiling was enabled."""
        buf = C.create_string_buffer(1 << 16)
        check(self._L.specter_profile_report(self.h, buf, len(buf)))
        out = {}
        for line in buf.value.decode().splitlines():
            name, n, ms, b = line.split()
            out[name] = (int(n), float(ms), float(b))
        return out

    @property
    def launch_count(self) -> int:
        n = C.c_longlong()
        check(self._L.specter_launch_count(self.h, C.byref(n)))
        return n.value


class Field:
    """Device-resident field handle (complex spectral/mixed or real physical)."""

    def __init__(self, plan: Plan, kind=COMPLEX):
        self.plan = plan
        self.kind = kind
        h = C.c_void_p()
        check(plan._L.specter_field_create(plan.h, kind, C.byref(h)))
        self.h = h
        self._owned = True

    @classmethod
    def _borrow(cls, plan, h, kind=COMPLEX):
        f = cls.__new__(cls)
        f.plan, f.kind, f.h, f._owned = plan, kind, h, False
        return f

    def close(self):
        if getattr(self, "_owned", False) and getattr(self, "h", None):
            self.plan._L.specter_field_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def shape(self):
        return self.plan.sshape if self.kind == COMPLEX else self.plan.rshape

    @property
    def dtype(self):
        return self.plan.cdtype if self.kind == COMPLEX else self.plan.rdtype

    @property
    def nbytes(self) -> int:
        """Bytes of the host array in the reference layout."""
        return int(np.prod(self.shape)) * np.dtype(self.dtype).itemsize

    def upload_ptr(self, host_ptr: int):
        """Asynchronous upload from a host buffer (reference layout) at host_ptr."""
        check(self.plan._L.specter_field_upload(self.h, C.c_void_p(host_ptr)))

    def download_ptr(self, host_ptr: int):
        """Download into a host buffer (reference layout); returns when the data is there."""
        check(self.plan._L.specter_field_download(self.h, C.c_void_p(host_ptr)))

    def upload(self, a):
        a = np.ascontiguousarray(a, dtype=self.dtype)
        if a.shape != self.shape:
            raise ValueError(f"expected shape {self.shape}, got {a.shape}")
        check(self.plan._L.specter_field_upload(self.h, a.ctypes.data_as(C.c_void_p)))
        self.plan.synchronize()
        return self

    def download(self, out=None):
        if out is None:
            out = np.empty(self.shape, self.dtype)
        check(self.plan._L.specter_field_download(self.h, out.ctypes.data_as(C.c_void_p)))
        return out

    def copy_from(self, other: "Field"):
        check(self.plan._L.specter_field_copy(self.h, other.h))
        return self

    def zero(self):
        check(self.plan._L.specter_field_zero(self.h))
        return self


def _L(plan):
    return plan._L


# ---------------------------------------------------------------- fftp (src/fftp/fftp.fpp)
def fftp3d_real_to_complex(plan, inp: Field, out: Field):
    check(_L(plan).specter_fftp3d_real_to_complex(plan.h, inp.h, out.h))


def fftp3d_complex_to_real(plan, inp: Field, out: Field):
    """The input is destroyed, as in the reference (fftp.fpp:812)."""
    check(_L(plan).specter_fftp3d_complex_to_real(plan.h, inp.h, out.h))


def fftp2d_real_to_complex_xy(plan, inp, out):
    check(_L(plan).specter_fftp2d_real_to_complex_xy(plan.h, inp.h, out.h))


def fftp2d_complex_to_real_xy(plan, inp, out):
    check(_L(plan).specter_fftp2d_complex_to_real_xy(plan.h, inp.h, out.h))


def fftp1d_real_to_complex_z(plan, inout):
    check(_L(plan).specter_fftp1d_real_to_complex_z(plan.h, inout.h))


def fftp1d_complex_to_real_z(plan, inout):
    check(_L(plan).specter_fftp1d_complex_to_real_z(plan.h, inout.h))


# ---------------------------------------------------------------- pseudo
def derivk(plan, a, b, dir):
    check(_L(plan).specter_derivk(plan.h, a.h, b.h, dir))


def laplak(plan, a, b):
    check(_L(plan).specter_laplak(plan.h, a.h, b.h))


def curlk(plan, a, b, c, dir):
    check(_L(plan).specter_curlk(plan.h, a.h, b.h, c.h, dir))


def gradre(plan, a, b, c, d, e, f):
    check(_L(plan).specter_gradre(plan.h, a.h, b.h, c.h, d.h, e.h, f.h))


def advect(plan, a, b, c, d, e):
    check(_L(plan).specter_advect(plan.h, a.h, b.h, c.h, d.h, e.h))


def fc_filter(plan, a):
    check(_L(plan).specter_fc_filter(plan.h, a.h))


def _scalar(fn, *args):
    out = C.c_double()
    check(fn(*args, C.byref(out)))
    return out.value


def energy(plan, a, b, c, kin):
    return _scalar(_L(plan).specter_energy, plan.h, a.h, b.h, c.h, kin)


def helicity(plan, a, b, c):
    return _scalar(_L(plan).specter_helicity, plan.h, a.h, b.h, c.h)


def cross(plan, a, b, c, d, e, f, kin):
    return _scalar(_L(plan).specter_cross, plan.h, a.h, b.h, c.h, d.h, e.h, f.h, kin)


def divergence(plan, a, b, c):
    return _scalar(_L(plan).specter_divergence, plan.h, a.h, b.h, c.h)


def variance(plan, a, kin):
    return _scalar(_L(plan).specter_variance, plan.h, a.h, kin)


def product(plan, a, b):
    return _scalar(_L(plan).specter_product, plan.h, a.h, b.h)


# ---------------------------------------------------------------- boundary
def bouncheck_z(plan, a, b=None):
    bot, top = C.c_double(), C.c_double()
    check(_L(plan).specter_bouncheck_z(plan.h, a.h, b.h if b is not None else None, C.byref(bot), C.byref(top)))
    return bot.value, top.value


def bouncheck_z_static(plan, a, b=None):
    """bouncheck_z without allocating: working memory is a fixed device array (see the C header)."""
    bot, top = C.c_double(), C.c_double()
    check(_L(plan).specter_bouncheck_z_static(plan.h, a.h, b.h if b is not None else None, C.byref(bot), C.byref(top)))
    return bot.value, top.value


def sol_project(plan, a, b, c, d, bctarget=1, bczsta=0, bczend=0):
    check(_L(plan).specter_sol_project(plan.h, a.h, b.h, c.h, d.h, bctarget, bczsta, bczend))


def v_imposebc_and_project(plan, vx, vy, vz, pr, rki, ord, v_zsta=(0.0, 0.0), v_zend=(0.0, 0.0)):
    zs = (C.c_double * 2)(*v_zsta)
    ze = (C.c_double * 2)(*v_zend)
    check(_L(plan).specter_v_imposebc_and_project(plan.h, vx.h, vy.h, vz.h, pr.h, rki, ord, zs, ze))


def s_imposebc(plan, th):
    check(_L(plan).specter_s_imposebc(plan.h, th.h))


# ---------------------------------------------------------------- solver (RK loop)
class Solver:
    """The RK loop of src/specter.fpp:1142-1161 with the HD or BOUSS stage body.

    solver HD, BOUSS or ROTBOUSS (rotation rate omega).  fused=True runs the GB300 fused stage
    kernels; fused=False runs the reference's call sequence (gradre, fc_filter, laplak, update, v_imposebc_and_project, ...) on the GPU.
    nl_fp32=True (fused solvers on an FP64 plan) is the precision form: the nonlinear term in FP32,
    everything that carries the state (update, wall round trips, projection, filter) in FP64."""

    def __init__(self, plan: Plan, solver=HD, ord=2, dt=1e-4, nu=1e-3, kappa=0.0, gama=1.0,
                 xmom=1.0, xtemp=1.0, v_zsta=(0.0, 0.0), v_zend=(0.0, 0.0), fused=True, omega=(0.0, 0.0, 0.0),
                 nl_fp32=False):
        self.plan = plan
        p = SolverParams()
        p.solver, p.ord, p.dt, p.nu, p.kappa = solver, ord, dt, nu, kappa
        p.gama, p.xmom, p.xtemp = gama, xmom, xtemp
        p.v_zsta[0], p.v_zsta[1] = v_zsta
        p.v_zend[0], p.v_zend[1] = v_zend
        p.fused = 1 if fused else 0
        p.omega[0], p.omega[1], p.omega[2] = omega
        p.nl_fp32 = 1 if nl_fp32 else 0
        self.params = p
        h = C.c_void_p()
        check(_L(plan).specter_solver_create(plan.h, C.byref(p), C.byref(h)))
        self.h = h
        ptrs = [C.c_void_p() for _ in range(5)]
        check(_L(plan).specter_solver_fields(h, *[C.byref(x) for x in ptrs]))
        vx, vy, vz, th, pr = ptrs
        self.vx, self.vy, self.vz = (Field._borrow(plan, x) for x in (vx, vy, vz))
        self.th = Field._borrow(plan, th) if th.value else None
        self.pr = Field._borrow(plan, pr)

    def close(self):
        if getattr(self, "h", None):
            _L(self.plan).specter_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def state(self):
        return [f for f in (self.vx, self.vy, self.vz, self.th) if f is not None] + [self.pr]

    def step(self, n=1):
        check(_L(self.plan).specter_solver_step(self.h, n))

    def stage(self, o):
        check(_L(self.plan).specter_solver_stage(self.h, o))

    def check(self):
        check(_L(self.plan).specter_solver_check(self.h))

    def autotune(self):
        """Pick the tile-width caps of the plan's kernel families (and, for fused solvers, the
        one- or two-kernel velocity stage) by timing RK steps of this solver (state restored).
        Returns (z, y, x, fused caps, velocity_split)."""
        caps = (C.c_int * 5)()
        check(_L(self.plan).specter_solver_autotune(self.h, caps))
        return tuple(caps)


def table_check(C_=25, d=5, tdir=None):
    """Validates FC-Gram tables A{C}-{d}.dat / Q{d}.dat (default: the packaged ones): returns
    (max |Q^T Q - I|, max |dir|, max row sum of |dir|)."""
    out = (C.c_double * 3)()
    check(load().specter_table_check((tdir or TABLES).encode(), int(C_), int(d), out))
    return tuple(out)


def fields_upload(fields, host_ptrs):
    """Uploads several fields of one plan from host buffers (reference layout) given as
    addresses; copies overlap the layout conversions.  Keep the buffers valid until the plan
    is synchronised."""
    n = len(fields)
    f = (C.c_void_p * n)(*[x.h.value for x in fields])
    h = (C.c_void_p * n)(*host_ptrs)
    check(_L(fields[0].plan).specter_fields_upload(n, f, h))


def fields_download(fields, host_ptrs):
    """Downloads several fields of one plan into host buffers (reference layout); returns when
    the data is in host memory."""
    n = len(fields)
    f = (C.c_void_p * n)(*[x.h.value for x in fields])
    h = (C.c_void_p * n)(*host_ptrs)
    check(_L(fields[0].plan).specter_fields_download(n, f, h))


def device_memory():
    """(free, total) bytes of the current device."""
    f, t = C.c_ulonglong(), C.c_ulonglong()
    check(load().specter_device_memory(C.byref(f), C.byref(t)))
    return f.value, t.value


def solver_memory(s: "Solver") -> int:
    """Device bytes held by a solver (state, RK and fused buffers, its plan's tables and scratch)."""
    b = C.c_ulonglong()
    check(_L(s.plan).specter_solver_memory(s.h, C.byref(b)))
    return b.value


def set_option(plan: Plan, name: str, value: int):
    """Named plan option (specter_plan_set_option): "velocity_split", "tile_cap_z" ..."""
    check(_L(plan).specter_plan_set_option(plan.h, name.encode(), int(value)))


def get_option(plan: Plan, name: str) -> int:
    """Current value of a named plan option (specter_plan_get_option)."""
    v = C.c_int()
    check(_L(plan).specter_plan_get_option(plan.h, name.encode(), C.byref(v)))
    return v.value


def set_tile_caps(plan: Plan, caps):
    """Tile-width caps (z, y, x, fused) of the plan's kernels; entries <= 0 are left unchanged."""
    c = (C.c_int * 4)(*caps)
    check(_L(plan).specter_plan_tile_caps(plan.h, c))


class Graph:
    """nsteps RK steps of several solvers captured as one CUDA graph (specter_graph_create):
    each solver's kernels on its own plan stream, the solvers as parallel branches."""

    def __init__(self, solvers, nsteps=1):
        self.solvers = list(solvers)
        L = load()
        self._L = L
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        check(L.specter_graph_create(arr, len(self.solvers), int(nsteps), C.byref(h)))
        self.h = h
        self.nsteps = nsteps
        n = C.c_longlong()
        check(L.specter_graph_kernels(h, C.byref(n)))
        self.kernels = n.value

    def launch(self):
        check(self._L.specter_graph_launch(self.h))

    def done(self) -> bool:
        """True when every launch so far has finished (non-blocking)."""
        d = C.c_int()
        check(self._L.specter_graph_query(self.h, C.byref(d)))
        return bool(d.value)

    def synchronize(self):
        check(self._L.specter_graph_synchronize(self.h))

    def close(self):
        if getattr(self, "h", None):
            self._L.specter_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Batched ensemble (specter_batch_create): one RK step of several fused FP32 HD solvers,
    each on its own plan, as a few dozen batched launches captured in one CUDA graph; the i-th
    kernel of every solver's step runs as one launch per FFT length class."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        L = load()
        self._L = L
        arr = (C.c_void_p * len(self.solvers))(*[s.h.value for s in self.solvers])
        h = C.c_void_p()
        check(L.specter_batch_create(arr, len(self.solvers), C.byref(h)))
        self.h = h
        n = C.c_longlong()
        check(L.specter_batch_kernels(h, C.byref(n)))
        self.kernels = n.value

    def step(self, n=1):
        check(self._L.specter_batch_step(self.h, int(n)))

    def synchronize(self):
        check(self._L.specter_batch_synchronize(self.h))

    def close(self):
        if getattr(self, "h", None):
            self._L.specter_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = [n for n in dir() if not n.startswith("_")] + ["SpecterError"]
