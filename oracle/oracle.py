"""ORACLE — test infrastructure only.

ctypes wrapper around ``oracle/liboracle.so``, the FP64 CPU restatement of
SPECTER's per-RK-stage hot path (see ``oracle/oracle.h`` for the parity status).
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module.  Arrays use the reference's layouts, as numpy arrays:

* spectral / mixed fields: complex128, shape ``(nx//2+1, ny, nz)`` (C order, so
  z is fastest — the Fortran array ``C(nz, ny, nx/2+1)``),
* physical fields: float64, shape ``(nz, ny, nx)`` (x fastest — ``R(nx, ny, nz)``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

_P = C.POINTER(C.c_double)


class OrcParams(C.Structure):
    _fields_ = [("dt", C.c_double), ("nu", C.c_double), ("kappa", C.c_double),
                ("xmom", C.c_double), ("xtemp", C.c_double),
                ("vxzsta", C.c_double), ("vyzsta", C.c_double),
                ("vxzend", C.c_double), ("vyzend", C.c_double), ("ord", C.c_int)]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(_LIB):
        subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        L.orc_create.restype = C.c_void_p
        L.orc_create.argtypes = [C.c_int] * 5 + [C.c_double] * 3 + [C.c_char_p, C.POINTER(C.c_int)]
        L.orc_destroy.argtypes = [C.c_void_p]
        for name in ("orc_energy", "orc_helicity", "orc_cross", "orc_divergence", "orc_variance", "orc_product"):
            getattr(L, name).restype = C.c_double
        L.orc_sol_project.restype = C.c_int
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


def set_threads(n: int) -> None:
    lib().orc_set_threads(C.c_int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


class Grid:
    """Grid + FC-Gram plan; mirrors fcgram_create_plan + the kes/grid modules."""

    def __init__(self, nx, ny, nz, cz=25, oz=5, Lx=1.0, Ly=1.0, Lz=1.0, tdir=None):
        if tdir is None:
            tdir = os.path.join(os.path.dirname(_HERE), "specter_gb300", "tables")
        err = C.c_int(0)
        h = lib().orc_create(nx, ny, nz, cz, oz, C.c_double(Lx), C.c_double(Ly), C.c_double(Lz),
                             tdir.encode(), C.byref(err))
        if not h:
            raise ValueError(f"orc_create failed (err={err.value})")
        self.h = C.c_void_p(h)
        self.nx, self.ny, self.nz, self.cz, self.oz = nx, ny, nz, cz, oz
        self.nxh = nx // 2 + 1
        self.Lx, self.Ly, self.Lz = Lx, Ly, Lz
        kx = np.zeros(self.nxh); ky = np.zeros(ny); kz = np.zeros(nz); z = np.zeros(nz)
        d = np.zeros(cz * oz)
        lib().orc_grid_info(self.h, _p(kx), _p(ky), _p(kz), _p(z), _p(d))
        self.kx, self.ky, self.kz, self.z = kx, ky, kz, z
        self.dir = d.reshape(oz, cz).T.copy()  # dir[i, j], C x d

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.orc_destroy(self.h)
            self.h = None

    # shapes ------------------------------------------------------------
    @property
    def sshape(self):
        return (self.nxh, self.ny, self.nz)

    @property
    def rshape(self):
        return (self.nz, self.ny, self.nx)

    def czeros(self):
        return np.zeros(self.sshape, np.complex128)

    def rzeros(self):
        return np.zeros(self.rshape, np.float64)

    @staticmethod
    def _c(a):
        return np.ascontiguousarray(a, dtype=np.complex128)

    # fftp ----------------------------------------------------------------
    def fftp3d_real_to_complex(self, r):
        out = self.czeros()
        lib().orc_fftp3d_real_to_complex(self.h, _p(np.ascontiguousarray(r, np.float64)), _p(out))
        return out

    def fftp3d_complex_to_real(self, c):
        cin = self._c(c).copy()
        out = self.rzeros()
        lib().orc_fftp3d_complex_to_real(self.h, _p(cin), _p(out))
        return out

    def fftp2d_real_to_complex_xy(self, r):
        out = self.czeros()
        lib().orc_fftp2d_real_to_complex_xy(self.h, _p(np.ascontiguousarray(r, np.float64)), _p(out))
        return out

    def fftp2d_complex_to_real_xy(self, c):
        out = self.rzeros()
        lib().orc_fftp2d_complex_to_real_xy(self.h, _p(self._c(c)), _p(out))
        return out

    def fftp1d_real_to_complex_z(self, c):
        a = self._c(c).copy()
        lib().orc_fftp1d_real_to_complex_z(self.h, _p(a))
        return a

    def fftp1d_complex_to_real_z(self, c):
        a = self._c(c).copy()
        lib().orc_fftp1d_complex_to_real_z(self.h, _p(a))
        return a

    # pseudo --------------------------------------------------------------
    def derivk(self, a, d):
        b = self.czeros()
        lib().orc_derivk(self.h, _p(self._c(a)), _p(b), C.c_int(d))
        return b

    def laplak(self, a):
        b = self.czeros()
        lib().orc_laplak(self.h, _p(self._c(a)), _p(b))
        return b

    def curlk(self, a, b, d):
        c = self.czeros()
        lib().orc_curlk(self.h, _p(self._c(a)), _p(self._c(b)), _p(c), C.c_int(d))
        return c

    def gradre(self, a, b, c):
        d, e, f = self.czeros(), self.czeros(), self.czeros()
        lib().orc_gradre(self.h, _p(self._c(a)), _p(self._c(b)), _p(self._c(c)), _p(d), _p(e), _p(f))
        return d, e, f

    def advect(self, a, b, c, d):
        e = self.czeros()
        lib().orc_advect(self.h, *[_p(self._c(x)) for x in (a, b, c, d)], _p(e))
        return e

    def fc_filter(self, a):
        b = self._c(a).copy()
        lib().orc_fc_filter(self.h, _p(b))
        return b

    def energy(self, a, b, c, kin):
        return lib().orc_energy(self.h, _p(self._c(a)), _p(self._c(b)), _p(self._c(c)), C.c_int(kin))

    def helicity(self, a, b, c):
        return lib().orc_helicity(self.h, _p(self._c(a)), _p(self._c(b)), _p(self._c(c)))

    def cross(self, a, b, c, d, e, f, kin):
        return lib().orc_cross(self.h, *[_p(self._c(x)) for x in (a, b, c, d, e, f)], C.c_int(kin))

    def divergence(self, a, b, c):
        return lib().orc_divergence(self.h, _p(self._c(a)), _p(self._c(b)), _p(self._c(c)))

    def variance(self, a, kin):
        return lib().orc_variance(self.h, _p(self._c(a)), C.c_int(kin))

    def product(self, a, b):
        return lib().orc_product(self.h, _p(self._c(a)), _p(self._c(b)))

    # boundary -------------------------------------------------------------
    def bouncheck_z(self, a, b=None):
        bot, top = C.c_double(), C.c_double()
        lib().orc_bouncheck_z(self.h, _p(self._c(a)), _p(self._c(b)) if b is not None else None,
                              C.byref(bot), C.byref(top))
        return bot.value, top.value

    def sol_project(self, a, b, c, bctarget=1, bczsta=0, bczend=0):
        a, b, c = (self._c(x).copy() for x in (a, b, c))
        d = self.czeros()
        err = lib().orc_sol_project(self.h, _p(a), _p(b), _p(c), _p(d), bctarget, bczsta, bczend)
        if err:
            raise ValueError(f"sol_project error {err}")
        return a, b, c, d

    def v_imposebc_and_project(self, vx, vy, vz, pr, rki, ord, vzsta=(0.0, 0.0), vzend=(0.0, 0.0)):
        vx, vy, vz, pr = (self._c(x).copy() for x in (vx, vy, vz, pr))
        zs = (C.c_double * 2)(*vzsta)
        ze = (C.c_double * 2)(*vzend)
        lib().orc_v_imposebc_and_project(self.h, _p(vx), _p(vy), _p(vz), _p(pr), rki, ord, zs, ze)
        return vx, vy, vz, pr

    def s_imposebc(self, th):
        th = self._c(th).copy()
        lib().orc_s_imposebc(self.h, _p(th))
        return th

    # stages ---------------------------------------------------------------
    @staticmethod
    def params(dt, nu, ord, kappa=0.0, xmom=1.0, xtemp=1.0, gama=1.0, vzsta=(0.0, 0.0), vzend=(0.0, 0.0)):
        return OrcParams(dt, nu, kappa, xmom * gama, xtemp * gama, vzsta[0], vzsta[1], vzend[0], vzend[1], ord)

    def hd_stage(self, p, o, vx, vy, vz, pr, C1, C2, C3):
        vx, vy, vz, pr = (self._c(x).copy() for x in (vx, vy, vz, pr))
        lib().orc_hd_stage(self.h, C.byref(p), o, _p(vx), _p(vy), _p(vz), _p(pr),
                           _p(self._c(C1)), _p(self._c(C2)), _p(self._c(C3)), None, None, None)
        return vx, vy, vz, pr

    def bouss_stage(self, p, o, vx, vy, vz, th, pr, C1, C2, C3, C7):
        vx, vy, vz, th, pr = (self._c(x).copy() for x in (vx, vy, vz, th, pr))
        lib().orc_bouss_stage(self.h, C.byref(p), o, _p(vx), _p(vy), _p(vz), _p(th), _p(pr),
                              *[_p(self._c(x)) for x in (C1, C2, C3, C7)], None, None, None, None)
        return vx, vy, vz, th, pr

    def rotbouss_stage(self, p, omega, o, vx, vy, vz, th, pr, C1, C2, C3, C7):
        vx, vy, vz, th, pr = (self._c(x).copy() for x in (vx, vy, vz, th, pr))
        om = (C.c_double * 3)(*omega)
        lib().orc_rotbouss_stage(self.h, C.byref(p), om, o, _p(vx), _p(vy), _p(vz), _p(th), _p(pr),
                                 *[_p(self._c(x)) for x in (C1, C2, C3, C7)])
        return vx, vy, vz, th, pr

    def run(self, p, nsteps, vx, vy, vz, pr, th=None, omega=None):
        """RK loop; with omega the ROTBOUSS stage (th required)."""
        vx, vy, vz, pr = (self._c(x).copy() for x in (vx, vy, vz, pr))
        tha = self._c(th).copy() if th is not None else None
        if omega is not None:
            om = (C.c_double * 3)(*omega)
            lib().orc_run_rot(self.h, C.byref(p), om, nsteps, _p(vx), _p(vy), _p(vz), _p(tha), _p(pr))
        else:
            lib().orc_run(self.h, C.byref(p), nsteps, _p(vx), _p(vy), _p(vz),
                          _p(tha) if tha is not None else None, _p(pr))
        return (vx, vy, vz, pr) if th is None else (vx, vy, vz, tha, pr)
