"""ctypes front end of the FP64 CPU oracle (oracle/opaw_oracle.c).

TEST INFRASTRUCTURE ONLY: the oracle the GPU library is compared against.
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
"""
from __future__ import annotations

import ctypes as ct
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_P = ct.c_void_p
_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ct.CDLL(_build.build())
        sig = {
            "orc_create": (ct.c_void_p, [_P]),
            "orc_free": (None, [_P]),
            "orc_fft3d": (None, [ct.c_int, ct.c_int, ct.c_int, _P, ct.c_int]),
            "orc_set_vks": (None, [_P, ct.c_int, _P]),
            "orc_get_vks": (None, [_P, ct.c_int, _P]),
            "orc_set_dij": (None, [_P, ct.c_int, _P]),
            "orc_get_dij": (None, [_P, ct.c_int, _P]),
            "orc_get_rhoij": (None, [_P, ct.c_int, _P]),
            "orc_get_density": (None, [_P, ct.c_int, _P]),
            "orc_get_nhat": (None, [_P, ct.c_int, _P]),
            "orc_get_vh": (None, [_P, ct.c_int, _P]),
            "orc_get_vxc": (None, [_P, ct.c_int, _P]),
            "orc_get_ek": (None, [_P, _P]),
            "orc_get_vk": (None, [_P, _P]),
            "orc_h_phi_batch": (None, [_P, ct.c_int, _P, _P, ct.c_int]),
            "orc_sn_phi_batch": (None, [_P, ct.c_double, _P, _P, ct.c_int]),
            "orc_shs_batch": (None, [_P, ct.c_int, _P, _P, ct.c_int]),
            "orc_proj_batch": (None, [_P, ct.c_int, _P, ct.c_int, _P]),
            "orc_rhoij": (None, [_P, ct.c_int, _P, ct.c_int]),
            "orc_density": (None, [_P, ct.c_int, _P, ct.c_int]),
            "orc_nhat": (None, [_P, ct.c_int]),
            "orc_vxc": (None, [_P, _P, ct.c_size_t]),
            "orc_rconv": (None, [ct.c_int, ct.c_int, ct.c_int, _P, _P, _P]),
            "orc_vh": (None, [_P, _P, _P]),
            "orc_vks": (None, [_P, ct.c_int]),
            "orc_dij": (None, [_P, ct.c_int]),
            "orc_rebuild": (None, [_P, ct.c_int, _P, ct.c_int]),
            "orc_excite": (None, [_P, ct.c_int, ct.c_double, _P, _P, ct.c_int]),
            "orc_dipole": (None, [_P, _P, _P, ct.c_int, ct.c_double, _P, _P, _P]),
            "orc_rk4_prop_shs": (None, [_P, _P, _P, ct.c_int, ct.c_double]),
            "orc_tddft_steps": (None, [_P, _P, _P, ct.c_int, ct.c_int, ct.c_double, ct.c_double, _P]),
            "orc_nthreads": (ct.c_int, []),
            "orc_onsite_xc": (None, [_P, _P, _P]),
        }
        for n, (r, a) in sig.items():
            f = getattr(L, n)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ct.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def fft3d(a, sign):
    """In-place-style unnormalised 3D DFT of a (nz, ny, nx) complex array."""
    b = _c(a, np.complex128).copy()
    nz, ny, nx = b.shape
    lib().orc_fft3d(nx, ny, nz, _p(b), sign)
    return b


def rconv(gin, bk):
    g = _c(gin, np.float64)
    k = _c(bk, np.float64)
    nz, ny, nx = g.shape
    out = np.empty_like(g)
    lib().orc_rconv(nx, ny, nz, _p(g), _p(k), _p(out))
    return out


def vxc(dens):
    d = _c(dens, np.float64)
    out = np.empty_like(d)
    lib().orc_vxc(_p(d), _p(out), d.size)
    return out


def nthreads():
    return int(lib().orc_nthreads())


class Oracle:
    def __init__(self, system):
        # the product's struct mirror describes the same opaw_system layout
        import opaw_tddft_gb300 as pkg

        self.system = system
        s = system
        st, keep = pkg.system_struct(s)
        self._keep = keep
        self._st = st
        self.h = lib().orc_create(ct.byref(st))
        self.nn = s.nx * s.ny * s.nz
        self.ns = int(np.sum(s.ms))
        self.nd = int(np.sum(np.asarray(s.ms, np.int64) ** 2))
        self.nb = (s.scale_vh * s.nx) * (s.scale_vh * s.ny) * (s.scale_vh * s.nz)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def _get(self, fn, set_, n):
        out = np.empty(n)
        fn(self.h, set_, _p(out))
        return out

    def set_vks(self, set_, v):
        a = _c(v, np.float64)
        lib().orc_set_vks(self.h, set_, _p(a))

    def set_dij(self, set_, d):
        a = _c(d, np.float64)
        lib().orc_set_dij(self.h, set_, _p(a))

    def get_vks(self, set_=0):
        return self._get(lib().orc_get_vks, set_, self.nn)

    def get_dij(self, set_=0):
        return self._get(lib().orc_get_dij, set_, self.nd)

    def get_rhoij(self, set_=0):
        return self._get(lib().orc_get_rhoij, set_, self.nd)

    def get_density(self, set_=0):
        return self._get(lib().orc_get_density, set_, self.nn)

    def get_nhat(self, set_=0):
        return self._get(lib().orc_get_nhat, set_, self.nn)

    def get_vh(self, set_=0):
        return self._get(lib().orc_get_vh, set_, self.nn)

    def get_vxc(self, set_=0):
        return self._get(lib().orc_get_vxc, set_, self.nn)

    def ek(self):
        out = np.empty(self.nn)
        lib().orc_get_ek(self.h, _p(out))
        return out

    def vk(self):
        out = np.empty(self.nb)
        lib().orc_get_vk(self.h, _p(out))
        return out

    def _norb(self, a):
        return a.size // self.nn

    def h_phi(self, pin, set_=0):
        a = _c(pin, np.complex128)
        out = np.empty_like(a)
        lib().orc_h_phi_batch(self.h, set_, _p(a), _p(out), self._norb(a))
        return out

    def sn_phi(self, pin, n):
        a = _c(pin, np.complex128)
        out = np.empty_like(a)
        lib().orc_sn_phi_batch(self.h, float(n), _p(a), _p(out), self._norb(a))
        return out

    def shs(self, pin, set_=0):
        a = _c(pin, np.complex128)
        out = np.empty_like(a)
        lib().orc_shs_batch(self.h, set_, _p(a), _p(out), self._norb(a))
        return out

    def proj(self, pin, which):
        a = _c(pin, np.complex128)
        norb = self._norb(a)
        out = np.empty((norb, self.ns), np.complex128)
        lib().orc_proj_batch(self.h, which, _p(a), norb, _p(out))
        return out

    def rhoij(self, psit, set_=0):
        a = _c(psit, np.complex128)
        lib().orc_rhoij(self.h, set_, _p(a), self._norb(a))
        return self.get_rhoij(set_)

    def density(self, psit, set_=0):
        a = _c(psit, np.complex128)
        lib().orc_density(self.h, set_, _p(a), self._norb(a))
        return self.get_density(set_)

    def nhat(self, set_=0):
        lib().orc_nhat(self.h, set_)

    def vks(self, set_=0):
        lib().orc_vks(self.h, set_)

    def dij(self, set_=0):
        lib().orc_dij(self.h, set_)

    def onsite_xc(self, rhoij):
        """The on-site XC term D_xc of the given rho_ij [sum ms^2]."""
        r = _c(rhoij, np.float64)
        out = np.zeros_like(r)
        lib().orc_onsite_xc(self.h, _p(r), _p(out))
        return out

    def rebuild(self, psibar, set_=0):
        a = _c(psibar, np.complex128)
        lib().orc_rebuild(self.h, set_, _p(a), self._norb(a))

    def vh(self, dens):
        d = _c(dens, np.float64)
        out = np.empty_like(d)
        lib().orc_vh(self.h, _p(d), _p(out))
        return out

    def excite(self, psi, ipol, gamma):
        a = _c(psi, np.complex128)
        out = np.empty_like(a)
        lib().orc_excite(self.h, ipol, float(gamma), _p(a), _p(out), self._norb(a))
        return out

    def dipole(self, p, pp, gamma):
        a = _c(p, np.complex128)
        b = _c(pp, np.complex128)
        d0, d1, dd = np.zeros(3), np.zeros(3), np.zeros(3)
        lib().orc_dipole(self.h, _p(a), _p(b), self._norb(a), float(gamma), _p(d0), _p(d1), _p(dd))
        return d0, d1, dd

    def rk4(self, p, pp, dt):
        """rk4_prop_shs on copies of p, pp; returns the propagated pair."""
        a = _c(p, np.complex128).copy()
        b = _c(pp, np.complex128).copy()
        lib().orc_rk4_prop_shs(self.h, _p(a), _p(b), self._norb(a), float(dt))
        return a, b

    def tddft_steps(self, p, pp, nsteps, dt, gamma):
        a = _c(p, np.complex128).copy()
        b = _c(pp, np.complex128).copy()
        out = np.zeros((max(nsteps, 1), 3))
        lib().orc_tddft_steps(self.h, _p(a), _p(b), self._norb(a), nsteps, float(dt), float(gamma), _p(out))
        return a, b, out[:nsteps]
