"""GB300 (sm_103a) OPAW-TDDFT propagation path.

The compute lives in ``libopaw_gb300.so`` (CUDA kernels behind the C ABI of
``include/opaw_gb300.h``).  This module is the Python host side: it loads that
library with ctypes and mirrors the reference's Fortran subroutines
(``h_phi``, ``sn_phi``, ``shs``, ``proj``, ``tddft_rhoij_2``, ``tddft_dens_2``,
``get_nhat``, ``get_pot_tddft_2``, ``get_dij``, ``excite_psi_bar_pert``,
``plot_dip``, ``rk4_prop_shs``) with the same argument meaning.  There is no
CPU fallback: without the built library every call raises.

The directory name is not a valid identifier; the package registers itself
as ``opaw_tddft_gb300`` (see ``__graft_entry__.load_package``).
"""
from __future__ import annotations

import ctypes as ct
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libopaw_gb300.so")

OPAW_OK = 0
OPAW_C128, OPAW_C64, OPAW_C128_DD = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
STATUS = {1: "OPAW_ERR_ARG", 2: "OPAW_ERR_CUDA", 3: "OPAW_ERR_STATE", 4: "OPAW_ERR_BOX",
          5: "OPAW_ERR_NOMEM", 6: "OPAW_ERR_NONFINITE", 7: "OPAW_ERR_NODEV"}


class OpawError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


_I = ct.POINTER(ct.c_int)
_D = ct.POINTER(ct.c_double)


class OpawSystem(ct.Structure):
    """ctypes mirror of `opaw_system`."""

    _fields_ = [
        ("nx", ct.c_int), ("ny", ct.c_int), ("nz", ct.c_int),
        ("dx", ct.c_double), ("dy", ct.c_double), ("dz", ct.c_double),
        ("ekcut", ct.c_double), ("scale_vh", ct.c_int), ("periodic", ct.c_int),
        ("rnel", ct.c_double), ("natom", ct.c_int),
        ("ir_start", _I), ("nrough", _I), ("ms", _I),
        ("p3d", _D), ("p3d1", _D), ("s", _D), ("sinv", _D),
        ("ngrid", _I), ("local_grid", _I), ("nlm", _I),
        ("g3d", _D), ("qijlm", _D), ("vloc", _D), ("ncoret", _D),
        ("dij0", _D), ("eijkl", _D), ("dij_max", ct.c_double),
        ("rad_n", _I), ("rad_r", _D), ("rad_w", _D), ("nphi", _I), ("phi", _D), ("tphi", _D),
        ("coredens", _D), ("tcoredens", _D), ("proj_lmn", _I),
    ]


def system_struct(s):
    """The opaw_system of a host System and the arrays it points to (keep
    them alive as long as the struct is used).  Systems without the radial
    tables of the on-site XC term pass NULL for them."""
    keep = {}

    def I(name, v):
        a = _arr(v, np.int32).reshape(-1)
        keep[name] = a
        return a.ctypes.data_as(_I)

    def D(name, v):
        a = _arr(v, np.float64).reshape(-1)
        keep[name] = a
        return a.ctypes.data_as(_D)

    st = OpawSystem(
        s.nx, s.ny, s.nz, s.dx, s.dy, s.dz, s.ekcut, s.scale_vh, s.periodic, s.rnel, s.natom,
        I("ir_start", s.ir_start), I("nrough", s.nrough), I("ms", s.ms),
        D("p3d", s.p3d), D("p3d1", s.p3d1), D("s", s.s), D("sinv", s.sinv),
        I("ngrid", s.ngrid), I("local_grid", s.local_grid), I("nlm", s.nlm),
        D("g3d", s.g3d), D("qijlm", s.qijlm), D("vloc", s.vloc), D("ncoret", s.ncoret),
        D("dij0", s.dij0), D("eijkl", s.eijkl), s.dij_max,
    )
    rad = getattr(s, "radial", None)
    if rad is not None:
        st.rad_n = I("rad_n", rad["rad_n"])
        st.rad_r = D("rad_r", rad["rad_r"])
        st.rad_w = D("rad_w", rad["rad_w"])
        st.nphi = I("nphi", rad["nphi"])
        st.phi = D("phi", rad["phi"])
        st.tphi = D("tphi", rad["tphi"])
        st.coredens = D("coredens", rad["coredens"])
        st.tcoredens = D("tcoredens", rad["tcoredens"])
        st.proj_lmn = I("proj_lmn", rad["proj_lmn"])
    return st, keep


# every exported symbol of include/opaw_gb300.h with its ctypes signature
_P = ct.c_void_p
SIGNATURES = {
    "opaw_dev_init": (ct.c_int, [ct.POINTER(OpawSystem), ct.POINTER(ct.c_void_p)]),
    "opaw_dev_free": (ct.c_int, [_P]),
    "opaw_last_error": (ct.c_char_p, []),
    "opaw_stream": (ct.c_void_p, [_P]),
    "opaw_kernel_launches": (ct.c_int64, [_P]),
    "opaw_ktime_begin": (ct.c_int, [_P]),
    "opaw_ktime_end": (ct.c_int, [_P, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int), ct.POINTER(ct.c_double)]),
    "opaw_tune_enable": (ct.c_int, [_P, ct.c_int]),
    "opaw_tune_report": (ct.c_int, [_P, ct.c_char_p, ct.c_int64, ct.POINTER(ct.c_int64)]),
    "opaw_sync": (ct.c_int, [_P]),
    "opaw_psi_upload": (ct.c_int, [_P, ct.c_int, _P, ct.c_int]),
    "opaw_psi_download": (ct.c_int, [_P, ct.c_int, _P, ct.c_int]),
    "opaw_psi_device": (ct.c_void_p, [_P, ct.c_int]),
    "opaw_set_vks": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_get_vks": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_set_dij": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_get_dij": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_get_rhoij": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_get_density": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_get_nhat": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_h_apply_dev": (ct.c_int, [_P, ct.c_int, ct.c_int, _P, _P, ct.c_int]),
    "opaw_sn_apply_dev": (ct.c_int, [_P, ct.c_int, ct.c_double, _P, _P, ct.c_int]),
    "opaw_shs_apply_dev": (ct.c_int, [_P, ct.c_int, ct.c_int, _P, _P, ct.c_int]),
    "opaw_proj_dev": (ct.c_int, [_P, ct.c_int, ct.c_int, _P, ct.c_int, _P]),
    "opaw_fft3d_dev": (ct.c_int, [_P, ct.c_int, _P, ct.c_int, ct.c_int]),
    "opaw_gram_dev": (ct.c_int, [_P, ct.c_int, _P, ct.c_int, _P, ct.c_int, _P]),
    "opaw_rotate_dev": (ct.c_int, [_P, ct.c_int, _P, ct.c_int, _P, ct.c_int, _P]),
    "opaw_orthog": (ct.c_int, [_P, ct.c_int, _P]),
    "opaw_herm_eig": (ct.c_int, [ct.c_int, _P, _P, _P]),
    "opaw_h_phi": (ct.c_int, [_P, ct.c_int, ct.c_int, _P, _P, ct.c_int]),
    "opaw_sn_phi": (ct.c_int, [_P, ct.c_int, ct.c_double, _P, _P, ct.c_int]),
    "opaw_shs": (ct.c_int, [_P, ct.c_int, ct.c_int, _P, _P, ct.c_int]),
    "opaw_rhoij": (ct.c_int, [_P, ct.c_int, ct.c_int]),
    "opaw_density": (ct.c_int, [_P, ct.c_int, ct.c_int]),
    "opaw_nhat": (ct.c_int, [_P, ct.c_int]),
    "opaw_vks": (ct.c_int, [_P, ct.c_int]),
    "opaw_dij": (ct.c_int, [_P, ct.c_int]),
    "opaw_rebuild": (ct.c_int, [_P, ct.c_int, ct.c_int]),
    "opaw_vh": (ct.c_int, [_P, _P, _P]),
    "opaw_rconv": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, _P, _P, _P]),
    "opaw_rconv_noalloc": (ct.c_int, [ct.c_int, ct.c_int, ct.c_int, _P, _P, _P, _P]),
    "opaw_vxc_lda": (ct.c_int, [_P, _P, _P, ct.c_int64]),
    "opaw_excite": (ct.c_int, [_P, ct.c_int, ct.c_double]),
    "opaw_dipole": (ct.c_int, [_P, ct.c_double, _P, _P, _P]),
    "opaw_tddft_steps": (ct.c_int, [_P, ct.c_int, ct.c_double, ct.c_double, ct.c_int, _P]),
    "opaw_tddft_steps_dip": (ct.c_int, [_P, ct.c_int, ct.c_double, ct.c_double, ct.c_int, _P, _P, _P]),
    "opaw_tddft_steps_host": (ct.c_int, [_P, _P, _P, ct.c_int, ct.c_int, ct.c_double, ct.c_double,
                                         ct.c_int, _P]),
    "opaw_excite_kicks": (ct.c_int, [_P, ct.c_int, _P, _P]),
    "opaw_kick_download": (ct.c_int, [_P, ct.c_int, _P, ct.c_int]),
    "opaw_tddft_steps_kicks": (ct.c_int, [_P, ct.c_int, ct.c_double, ct.c_int, _P, _P, _P]),
    "opaw_precond_kinetic_dev": (ct.c_int, [_P, ct.c_int, _P, _P, _P, ct.c_int]),
    "opaw_kinetic_energy_dev": (ct.c_int, [_P, ct.c_int, _P, ct.c_int, _P]),
    "opaw_net_create": (ct.c_int, [ct.c_ulonglong, ct.POINTER(ct.c_void_p)]),
    "opaw_net_free": (ct.c_int, [_P]),
    "opaw_net_params": (ct.c_int, [_P, _P]),
    "opaw_net_set_params": (ct.c_int, [_P, _P]),
    "opaw_net_launches": (ct.c_int64, [_P]),
    "opaw_net_forward": (ct.c_int, [_P, ct.c_int, ct.c_int, ct.c_int, ct.c_int, _P, _P]),
    "opaw_net_loss_grad": (ct.c_int, [_P, ct.c_int, ct.c_int, ct.c_int, _P, _P, _P, _P]),
    "opaw_net_add_patches": (ct.c_int, [_P, _P, _P, _P, ct.c_int, _P, _P, ct.c_int, _P, ct.c_int, ct.c_int]),
    "opaw_net_train": (ct.c_int, [_P, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_int, ct.c_double, _P]),
    "opaw_precond_learned_dev": (ct.c_int, [_P, _P, ct.c_int, _P, _P, _P, _P, ct.c_int]),
    "opaw_orthonormalize_dev": (ct.c_int, [_P, ct.c_int, ct.c_int, _P]),
    "opaw_gram_herm_dev": (ct.c_int, [_P, ct.c_int, _P, _P, ct.c_int, _P]),
    "opaw_ensemble_steps": (ct.c_int, [_P, ct.c_int, ct.c_int, ct.c_double, _P, _P, _P]),
}

_lib = None


def lib():
    """The loaded C-ABI library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OpawError(2, f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback exists)")
        L = ct.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status):
    if status != OPAW_OK:
        raise OpawError(status, lib().opaw_last_error().decode())


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ct.c_void_p)


def _arr(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


class Context:
    """One device context: operator tables + resident orbitals of both sets."""

    def __init__(self, system):
        self.system = system
        s = system
        st, self._keep = system_struct(s)
        self._sys = st
        self._norb = [0, 0]
        self.nkick = 1
        h = ct.c_void_p()
        _check(lib().opaw_dev_init(ct.byref(st), ct.byref(h)))
        self.h = h
        self.nn = s.nx * s.ny * s.nz
        self.ns = int(np.sum(s.ms))
        self.nd = int(np.sum(np.asarray(s.ms, np.int64) ** 2))

    def close(self):
        if getattr(self, "h", None):
            lib().opaw_dev_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- plumbing
    @property
    def stream(self) -> int:
        return lib().opaw_stream(self.h) or 0

    @property
    def launches(self) -> int:
        return int(lib().opaw_kernel_launches(self.h))

    def sync(self):
        _check(lib().opaw_sync(self.h))

    def tune_enable(self, on=True):
        """Launch-shape autotuner: True (timing, the default), False (off:
        the defaults) or "frozen" (decided sites kept, no more timing)."""
        mode = 2 if on == "frozen" else (1 if on else 0)
        _check(lib().opaw_tune_enable(self.h, mode))

    def tune_report(self):
        """The autotuner's sites: [{"site", "candidates", "ms", "chosen"}]."""
        import json

        need = ct.c_int64(0)
        _check(lib().opaw_tune_report(self.h, None, 0, ct.byref(need)))
        buf = ct.create_string_buffer(int(need.value))
        _check(lib().opaw_tune_report(self.h, buf, need.value, ct.byref(need)))
        return json.loads(buf.value.decode())

    def ktime_begin(self):
        """Start live event timing of the fused dense pass (opaw_ktime_begin)."""
        _check(lib().opaw_ktime_begin(self.h))

    def ktime_end(self):
        """(device ms summed over launches, launches, algorithmic bytes)."""
        ms, n, b = ct.c_double(), ct.c_int(), ct.c_double()
        _check(lib().opaw_ktime_end(self.h, ct.byref(ms), ct.byref(n), ct.byref(b)))
        return ms.value, n.value, b.value

    # ---- orbitals
    def upload(self, set_, psi):
        a = _arr(psi, np.complex128)
        norb = a.size // self.nn
        _check(lib().opaw_psi_upload(self.h, set_, _ptr(a), norb))
        self._norb[set_] = norb
        if set_ == 1:
            self.nkick = 1

    def download(self, set_, norb):
        out = np.empty((norb,) + self.system.shape_f, np.complex128)
        _check(lib().opaw_psi_download(self.h, set_, _ptr(out), norb))
        return out

    def psi_device(self, set_) -> int:
        return lib().opaw_psi_device(self.h, set_) or 0

    # ---- operator state
    def set_vks(self, set_, v):
        a = _arr(v, np.float64)
        _check(lib().opaw_set_vks(self.h, set_, _ptr(a)))

    def _get(self, fn, set_, n):
        out = np.empty(n, np.float64)
        _check(fn(self.h, set_, _ptr(out)))
        return out

    def get_vks(self, set_=0):
        return self._get(lib().opaw_get_vks, set_, self.nn)

    def set_dij(self, set_, d):
        a = _arr(d, np.float64)
        _check(lib().opaw_set_dij(self.h, set_, _ptr(a)))

    def get_dij(self, set_=0):
        return self._get(lib().opaw_get_dij, set_, self.nd)

    def get_rhoij(self, set_=0):
        return self._get(lib().opaw_get_rhoij, set_, self.nd)

    def get_density(self, set_=0):
        return self._get(lib().opaw_get_density, set_, self.nn)

    def get_nhat(self, set_=0):
        return self._get(lib().opaw_get_nhat, set_, self.nn)

    # ---- per-routine operators on host arrays (h_phi, sn_phi, shs)
    def h_phi(self, pin, set_=0, dtype=OPAW_C128):
        a = _arr(pin, np.complex128)
        out = np.empty_like(a)
        _check(lib().opaw_h_phi(self.h, set_, dtype, _ptr(a), _ptr(out), a.size // self.nn))
        return out

    def sn_phi(self, pin, n, dtype=OPAW_C128):
        a = _arr(pin, np.complex128)
        out = np.empty_like(a)
        _check(lib().opaw_sn_phi(self.h, dtype, float(n), _ptr(a), _ptr(out), a.size // self.nn))
        return out

    def shs(self, pin, set_=0, dtype=OPAW_C128):
        a = _arr(pin, np.complex128)
        out = np.empty_like(a)
        _check(lib().opaw_shs(self.h, set_, dtype, _ptr(a), _ptr(out), a.size // self.nn))
        return out

    # ---- per-routine operators on device pointers (asynchronous)
    def h_apply_dev(self, set_, dtype, pin_ptr, out_ptr, norb):
        _check(lib().opaw_h_apply_dev(self.h, set_, dtype, ct.c_void_p(pin_ptr), ct.c_void_p(out_ptr), norb))

    def shs_apply_dev(self, set_, dtype, pin_ptr, out_ptr, norb):
        _check(lib().opaw_shs_apply_dev(self.h, set_, dtype, ct.c_void_p(pin_ptr), ct.c_void_p(out_ptr), norb))

    def sn_apply_dev(self, dtype, n, pin_ptr, out_ptr, norb):
        _check(lib().opaw_sn_apply_dev(self.h, dtype, float(n), ct.c_void_p(pin_ptr), ct.c_void_p(out_ptr), norb))

    def precond_kinetic_dev(self, dtype, pin_ptr, ekin, out_ptr, norb):
        """Teter-Payne-Allan kinetic preconditioner (opaw_precond_kinetic_dev)."""
        e = _arr(ekin, np.float64)
        _check(lib().opaw_precond_kinetic_dev(self.h, dtype, ct.c_void_p(pin_ptr), _ptr(e), ct.c_void_p(out_ptr),
                                              norb))

    def kinetic_energy_dev(self, dtype, x_ptr, norb):
        out = np.empty(norb)
        _check(lib().opaw_kinetic_energy_dev(self.h, dtype, ct.c_void_p(x_ptr), norb, _ptr(out)))
        return out

    def fft3d_dev(self, dtype, ptr, norb, sign):
        _check(lib().opaw_fft3d_dev(self.h, dtype, ct.c_void_p(ptr), norb, sign))

    def gram_dev(self, dtype, a_ptr, na, b_ptr, nb):
        out = np.empty((nb, na), np.complex128)  # C order [j][i] == column-major G[i + na j]
        _check(lib().opaw_gram_dev(self.h, dtype, ct.c_void_p(a_ptr), na, ct.c_void_p(b_ptr), nb, _ptr(out)))
        return out.T

    def gram_herm_dev(self, dtype, a_ptr, b_ptr, n):
        """dv A^H B for a result known to be Hermitian (upper tiles summed)."""
        out = np.empty((n, n), np.complex128)
        _check(lib().opaw_gram_herm_dev(self.h, dtype, ct.c_void_p(a_ptr), ct.c_void_p(b_ptr), n, _ptr(out)))
        return out.T

    def rotate_dev(self, dtype, a_ptr, na, M, out_ptr):
        Mf = np.asfortranarray(M, dtype=np.complex128)
        _check(lib().opaw_rotate_dev(self.h, dtype, ct.c_void_p(a_ptr), na, Mf.ctypes.data_as(ct.c_void_p),
                                     Mf.shape[1], ct.c_void_p(out_ptr)))

    def orthog(self, set_=0):
        """orthog_phi: canonical orthogonalisation of the resident orbitals."""
        w = np.empty(self.system_norb(set_))
        _check(lib().opaw_orthog(self.h, set_, _ptr(w)))
        return w

    def orthonormalize(self, set_=0, method=0):
        """FP64 orthonormalisation on the device: 0 Cholesky, 1 Loewdin
        (Newton-Schulz); returns max |G - I| before it."""
        off = ct.c_double()
        _check(lib().opaw_orthonormalize_dev(self.h, set_, method, ct.byref(off)))
        return off.value

    def system_norb(self, set_):
        return self._norb[set_]

    def proj_dev(self, which, dtype, pin_ptr, norb):
        out = np.empty((norb, self.ns), np.complex128)
        _check(lib().opaw_proj_dev(self.h, which, dtype, ct.c_void_p(pin_ptr), norb, _ptr(out)))
        return out

    # ---- rebuild chain
    def rhoij(self, set_=0, precision=PREC_FP64):
        _check(lib().opaw_rhoij(self.h, set_, precision))
        return self.get_rhoij(set_)

    def density(self, set_=0, precision=PREC_FP64):
        _check(lib().opaw_density(self.h, set_, precision))
        return self.get_density(set_)

    def nhat(self, set_=0):
        _check(lib().opaw_nhat(self.h, set_))

    def vks(self, set_=0):
        _check(lib().opaw_vks(self.h, set_))

    def dij(self, set_=0):
        _check(lib().opaw_dij(self.h, set_))

    def rebuild(self, set_=0, precision=PREC_FP64):
        _check(lib().opaw_rebuild(self.h, set_, precision))

    def vh(self, dens):
        a = _arr(dens, np.float64)
        out = np.empty_like(a)
        _check(lib().opaw_vh(self.h, _ptr(a), _ptr(out)))
        return out

    def vxc_lda(self, dens):
        a = _arr(dens, np.float64)
        out = np.empty_like(a)
        _check(lib().opaw_vxc_lda(self.h, _ptr(a), _ptr(out), a.size))
        return out

    # ---- kick, dipole, propagation
    def excite(self, ipol, gamma):
        _check(lib().opaw_excite(self.h, ipol, float(gamma)))
        self._norb[1] = self._norb[0]
        self.nkick = 1

    def excite_kicks(self, ipol, gamma):
        """Kicked sets k = psi exp(-i gamma[k] r_ipol[k]) for every (ipol, gamma)
        pair, all propagated against the one unperturbed set."""
        ip = _arr(np.atleast_1d(ipol), np.int32)
        ga = _arr(np.atleast_1d(gamma), np.float64)
        assert ip.size == ga.size
        _check(lib().opaw_excite_kicks(self.h, int(ip.size), _ptr(ip), _ptr(ga)))
        self._norb[1] = self._norb[0]
        self.nkick = int(ip.size)

    def kick_download(self, kick, norb):
        out = np.empty((norb,) + self.system.shape_f, np.complex128)
        _check(lib().opaw_kick_download(self.h, kick, _ptr(out), norb))
        return out

    def tddft_steps_kicks(self, nsteps, dt, precision=PREC_FP64):
        """nsteps steps of every set; returns (dip [nsteps, 3],
        dip_pert [nsteps, nkick, 3], d_dip [nsteps, nkick, 3])."""
        n = max(nsteps, 1)
        K = self.nkick
        dip, dpp, dd = np.zeros((n, 3)), np.zeros((n, K, 3)), np.zeros((n, K, 3))
        _check(lib().opaw_tddft_steps_kicks(self.h, nsteps, float(dt), precision, _ptr(dip), _ptr(dpp), _ptr(dd)))
        return dip[:nsteps], dpp[:nsteps], dd[:nsteps]

    def dipole(self, gamma):
        d0 = np.zeros(3)
        d1 = np.zeros(3)
        dd = np.zeros(3)
        _check(lib().opaw_dipole(self.h, float(gamma), _ptr(d0), _ptr(d1), _ptr(dd)))
        return d0, d1, dd

    def tddft_steps(self, nsteps, dt, gamma, precision=PREC_FP64, want_dipoles=True):
        out = np.zeros((max(nsteps, 1), 3)) if want_dipoles else None
        _check(lib().opaw_tddft_steps(self.h, nsteps, float(dt), float(gamma), precision,
                                      _ptr(out) if want_dipoles else None))
        return out[:nsteps] if want_dipoles else None

    def tddft_steps_dip(self, nsteps, dt, gamma, precision=PREC_FP64):
        """nsteps steps; returns (dip, dip_pert, d_dip), each [nsteps, 3]: the
        values plot_dip writes to dip.dat and d_dip.dat."""
        n = max(nsteps, 1)
        dip, dpp, dd = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        _check(lib().opaw_tddft_steps_dip(self.h, nsteps, float(dt), float(gamma), precision, _ptr(dip),
                                          _ptr(dpp), _ptr(dd)))
        return dip[:nsteps], dpp[:nsteps], dd[:nsteps]

    def tddft_steps_host(self, psi, psi_pert, nsteps, dt, gamma, precision=PREC_FP64):
        """Uploads both orbital sets from host arrays, propagates, downloads
        them back in place; returns d_dip per step."""
        assert psi.dtype == np.complex128 and psi.flags.c_contiguous
        assert psi_pert.dtype == np.complex128 and psi_pert.flags.c_contiguous
        norb = psi.size // self.nn
        out = np.zeros((max(nsteps, 1), 3))
        _check(lib().opaw_tddft_steps_host(self.h, _ptr(psi), _ptr(psi_pert), norb, nsteps, float(dt),
                                           float(gamma), precision, _ptr(out)))
        return out[:nsteps]


def ensemble_steps(contexts, nsteps, dt):
    """opaw_ensemble_steps: nsteps mixed-precision steps of every context (each
    with its kicked sets from excite_kicks) through one replayed CUDA graph.
    Returns per context (dip [nsteps, 3], dip_pert [nsteps, nkick, 3],
    d_dip [nsteps, nkick, 3])."""
    n = len(contexts)
    outs = [(np.zeros((max(nsteps, 1), 3)), np.zeros((max(nsteps, 1), c.nkick, 3)),
             np.zeros((max(nsteps, 1), c.nkick, 3))) for c in contexts]
    H = (ct.c_void_p * n)(*[c.h.value for c in contexts])
    P = [(ct.c_void_p * n)(*[o[j].ctypes.data for o in outs]) for j in range(3)]
    _check(lib().opaw_ensemble_steps(ct.cast(H, ct.c_void_p), n, nsteps, float(dt), ct.cast(P[0], ct.c_void_p),
                                     ct.cast(P[1], ct.c_void_p), ct.cast(P[2], ct.c_void_p)))
    return [(a[:nsteps], b[:nsteps], d[:nsteps]) for a, b, d in outs]


def rconv(gin, bk):
    """gout = 1/N ifft(bk * fft(gin)) on the device (rconv of the reference)."""
    g = _arr(gin, np.float64)
    b = _arr(bk, np.float64)
    assert g.shape == b.shape and g.ndim == 3
    n2, n1, n0 = g.shape
    out = np.empty_like(g)
    _check(lib().opaw_rconv(n0, n1, n2, _ptr(g), _ptr(b), _ptr(out)))
    return out


def herm_eig(H):
    """Eigenvalues (ascending) and eigenvectors of a complex Hermitian matrix
    with the library's host Jacobi solver."""
    A = np.array(H, dtype=np.complex128, order="F", copy=True)
    n = A.shape[0]
    w = np.empty(n)
    V = np.empty((n, n), np.complex128, order="F")
    _check(lib().opaw_herm_eig(n, A.ctypes.data_as(ct.c_void_p), _ptr(w), V.ctypes.data_as(ct.c_void_p)))
    return w, V
