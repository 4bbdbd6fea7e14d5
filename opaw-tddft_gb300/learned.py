"""The learned preconditioner of the ground-state eigensolver (host side of
the opaw_net_* entry points of include/opaw_gb300.h).

A 3-layer 3D convolutional network (3^3 kernels, 16 channels, BF16 weights,
FP32 accumulation; csrc/precond_net.cu) corrects the Teter-Payne-Allan
kinetic preconditioner: for an orbital with residual r and Ritz value eps the
search direction is

    w = K r + |r| N(r / |r|, v_ks - eps).

It is trained on the device on residual -> correction pairs that the plain
solver produces itself (`pairs_from_run`): for a recorded iterate x with
residual r, once the solver has converged to the invariant subspace X*, the
correction that removes x's error is t = X* X*^H x - x; the network learns
the part of c t (c the scalar that best aligns K r with t) that K r misses.
The reference has no counterpart (its SCF, chebyr_m.f90, has no
preconditioner).
"""
from __future__ import annotations

import ctypes as ct

import numpy as np

import opaw_tddft_gb300 as pkg

LAYERS = 3
TAPS = 27
CH = 16
WL = TAPS * CH * CH
PL = WL + CH
NPARAM = LAYERS * PL


class Net:
    """A device network (opaw_net)."""

    def __init__(self, seed=1):
        h = ct.c_void_p()
        pkg._check(pkg.lib().opaw_net_create(seed, ct.byref(h)))
        self.h = h
        self.npatch = 0
        self.P = None

    def close(self):
        if getattr(self, "h", None):
            pkg.lib().opaw_net_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def launches(self):
        return int(pkg.lib().opaw_net_launches(self.h))

    def params(self):
        out = np.empty(NPARAM, np.float32)
        pkg._check(pkg.lib().opaw_net_params(self.h, out.ctypes.data_as(ct.c_void_p)))
        return out

    def set_params(self, w):
        a = np.ascontiguousarray(w, np.float32)
        assert a.size == NPARAM
        pkg._check(pkg.lib().opaw_net_set_params(self.h, a.ctypes.data_as(ct.c_void_p)))

    def forward(self, x_bits):
        """x_bits: uint16 BF16 bits [batch, nz, ny, nx, 16] -> float32 [..., 16]."""
        x = np.ascontiguousarray(x_bits, np.uint16)
        b, nz, ny, nx, c = x.shape
        assert c == CH
        out = np.empty(x.shape, np.float32)
        pkg._check(pkg.lib().opaw_net_forward(self.h, b, nz, ny, nx, x.ctypes.data_as(ct.c_void_p),
                                              out.ctypes.data_as(ct.c_void_p)))
        return out

    def loss_grad(self, x_bits, tgt, margin):
        x = np.ascontiguousarray(x_bits, np.uint16)
        t = np.ascontiguousarray(tgt, np.float32)
        b, P = x.shape[0], x.shape[1]
        loss = ct.c_double()
        g = np.empty(NPARAM, np.float32)
        pkg._check(pkg.lib().opaw_net_loss_grad(self.h, b, P, margin, x.ctypes.data_as(ct.c_void_p),
                                                t.ctypes.data_as(ct.c_void_p), ct.byref(loss),
                                                g.ctypes.data_as(ct.c_void_p)))
        return loss.value, g

    def add_patches(self, ctx, r_ptr, t_ptr, norb, eps, scale, origins, P):
        o = np.ascontiguousarray(origins, np.int32).reshape(-1, 4)
        e = np.ascontiguousarray(eps, np.float64)
        s = np.ascontiguousarray(scale, np.float64)
        if self.P is not None and self.P != P:
            raise ValueError("all patches of a net have one size")
        pkg._check(pkg.lib().opaw_net_add_patches(self.h, ctx.h, ct.c_void_p(r_ptr), ct.c_void_p(t_ptr), norb,
                                                  e.ctypes.data_as(ct.c_void_p), s.ctypes.data_as(ct.c_void_p),
                                                  o.shape[0], o.ctypes.data_as(ct.c_void_p), P, self.npatch))
        self.npatch += o.shape[0]
        self.P = P

    def train(self, nsteps, batch=32, lr=1e-3, margin=3):
        losses = np.empty(max(nsteps, 1))
        pkg._check(pkg.lib().opaw_net_train(self.h, self.npatch, self.P, margin, nsteps, batch, float(lr),
                                            losses.ctypes.data_as(ct.c_void_p)))
        return losses[:nsteps]

    def apply(self, ctx, dtype, r_ptr, eps, ekin, w_ptr, norb):
        e = np.ascontiguousarray(eps, np.float64)
        k = np.ascontiguousarray(ekin, np.float64)
        pkg._check(pkg.lib().opaw_precond_learned_dev(ctx.h, self.h, dtype, ct.c_void_p(r_ptr),
                                                      e.ctypes.data_as(ct.c_void_p), k.ctypes.data_as(ct.c_void_p),
                                                      ct.c_void_p(w_ptr), norb))


def pairs_from_run(ctx, net, snapshots, Xc, P=16, per_orbital=8, seed=0):
    """Adds training patches from a finished plain solve to `net`.
    snapshots: list of (X, R, eps) device tensors / host Ritz values of
    recorded iterations; Xc: the converged orbitals (device, complex128,
    orthonormal with the dv inner product).  Target of orbital x with residual
    r: c t - K r with t = Xc Xc^H x dv - x and c = <K r, t> / <t, t>, all
    scaled by 1 / |r| in the patches.  Patch origins are drawn around the
    orbital's largest residual values (P^3 boxes, periodic wrap)."""
    import torch

    rng = np.random.default_rng(seed)
    dv = ctx.system.dv
    nz, ny, nx = ctx.system.shape_f
    for X, R, eps in snapshots:
        m = X.shape[0]
        ekin = ctx.kinetic_energy_dev(pkg.OPAW_C128, X.data_ptr(), m)
        KR = torch.empty_like(R)
        ctx.precond_kinetic_dev(pkg.OPAW_C128, R.data_ptr(), ekin, KR.data_ptr(), m)
        ctx.sync()
        C = (Xc.conj() @ X.T) * dv            # [nc, m]
        T = (Xc.T @ C).T - X                  # t = Xc Xc^H x - x
        tt = (T.abs() ** 2).sum(dim=1).double()
        c = ((KR.conj() * T).sum(dim=1) / torch.clamp(tt, min=1e-300)).real
        Tg = (c[:, None] * T - KR).contiguous()
        rn = torch.sqrt((R.abs() ** 2).sum(dim=1).double() * dv).cpu().numpy()
        scale = np.where(rn > 0, 1.0 / np.maximum(rn, 1e-300), 0.0)
        # origins weighted by |r|^2 of each orbital
        org = []
        w2 = (R.abs() ** 2).reshape(m, -1)
        for o in range(m):
            p = (w2[o] / w2[o].sum()).double().cpu().numpy()
            idx = rng.choice(p.size, size=per_orbital, p=p / p.sum())
            for g in idx:
                x, y, z = g % nx, (g // nx) % ny, g // (nx * ny)
                org.append((o, (z - P // 2) % nz, (y - P // 2) % ny, (x - P // 2) % nx))
        net.add_patches(ctx, R.data_ptr(), Tg.data_ptr(), m, np.asarray(eps, np.float64), scale, org, P)
        ctx.sync()
