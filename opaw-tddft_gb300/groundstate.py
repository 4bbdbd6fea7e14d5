"""Stationary initial states for the propagation.

A real OPAW-TDDFT run starts from the self-consistent ground state of the
SCF (main.f90:67-96): the occupied orbitals are eigenvectors of
S^-1/2 H[rho] S^-1/2, where rho is their own density, so without a kick the
density does not move and the kicked set carries a small linear response.
The seeded random orbitals of `synthetic` are far from that regime.  This
module produces such a state for a synthetic system, using the device
operators of the library:

* `lowest_states` — Chebyshev-filtered subspace iteration with Rayleigh-Ritz
  (the reference's chebyr_m.f90 filter, orthog_phi.f90 orthogonalisation and
  diag.f90 subspace diagonalisation), for the lowest eigenvectors of
  S^-1/2 H0 S^-1/2 with H0 = T + v_ks0 + sum p~ D0 <p~|;
* `stationary_system` — rebuilds rho, n^, v_ks and D_ij from those orbitals
  and shifts v_loc and D0 so that the rebuilt Hamiltonian is exactly H0: the
  orbitals are then an exact stationary state of the TDDFT Hamiltonian;
* `scf` — the self-consistent ground state of the system as it is (the
  reference's SCF loop, main.f90:67-96): rebuild, DIIS mixing, filtering.

Device memory is handled with torch tensors (plumbing); every operator runs
in libopaw_gb300.so.
"""
from __future__ import annotations

import dataclasses

import numpy as np

import opaw_tddft_gb300 as pkg


def _torch():
    import torch

    return torch


def _shs(ctx, dtype, X, Y):
    norb = X.shape[0]
    ctx.shs_apply_dev(0, dtype, X.data_ptr(), Y.data_ptr(), norb)
    ctx.sync()


def _orthonormalise(ctx, dtype, X, scratch, refill=None):
    """X <- X G^-1/2 (canonical orthogonalisation, orthog_phi.f90).  When the
    block has (numerically) lost rank, the directions whose Gram eigenvalue is
    below 1e-6 of the largest are dropped, as orthog_phi.f90 drops the small
    eigenvalues of its Gram matrix, and `refill(n)` supplies that many fresh
    vectors before the block is orthonormalised again."""
    norb = X.shape[0]
    G = ctx.gram_dev(dtype, X.data_ptr(), norb, X.data_ptr(), norb)
    G = 0.5 * (G + G.conj().T)
    w, V = np.linalg.eigh(G)
    keep = w > 1e-6 * w.max()
    if keep.all():
        ctx.rotate_dev(dtype, X.data_ptr(), norb, V / np.sqrt(w)[None, :], scratch.data_ptr())
        X.copy_(scratch)
        return
    if refill is None or not keep.any():
        raise RuntimeError("subspace lost rank")
    nk = int(keep.sum())
    # the kept directions first, largest Gram eigenvalue (least filtered away) first
    order = np.argsort(-w[keep])
    M = (V[:, keep] / np.sqrt(w[keep])[None, :])[:, order]
    ctx.rotate_dev(dtype, X.data_ptr(), norb, M, scratch.data_ptr())
    X[:nk].copy_(scratch[:nk])
    X[nk:].copy_(refill(norb - nk))
    _orthonormalise(ctx, dtype, X, scratch, None)


def _rayleigh_ritz(ctx, dtype, X, HX, scratch):
    """Subspace diagonalisation (diag.f90): X <- X V, HX <- HX V."""
    norb = X.shape[0]
    Hs = ctx.gram_dev(dtype, X.data_ptr(), norb, HX.data_ptr(), norb)
    Hs = 0.5 * (Hs + Hs.conj().T)
    w, V = np.linalg.eigh(Hs)
    ctx.rotate_dev(dtype, X.data_ptr(), norb, V, scratch.data_ptr())
    X.copy_(scratch)
    ctx.rotate_dev(dtype, HX.data_ptr(), norb, V, scratch.data_ptr())
    HX.copy_(scratch)
    return w


def _residuals(X, HX, w, dv):
    torch = _torch()
    ww = torch.as_tensor(w, device=X.device, dtype=torch.float64).to(X.real.dtype)
    R = HX - X * ww[:, None]
    return torch.sqrt((R.abs() ** 2).sum(dim=1).double() * dv).cpu().numpy()


def lowest_states(ctx, psi0, n_iter=200, degree=24, tol=1e-4, fp64_polish=4, nbuf=None, seed=0, verbose=False):
    """Lowest eigenpairs of S^-1/2 H S^-1/2; see `_lowest_states`.  Every
    torch operation runs on the library's stream (opaw_stream): the device
    entry points read their inputs in that stream's order, so a torch kernel
    queued on another stream could still be writing an input when the
    library's kernels read it."""
    torch = _torch()
    with torch.cuda.stream(torch.cuda.ExternalStream(ctx.stream)):
        out = _lowest_states(ctx, psi0, n_iter, degree, tol, fp64_polish, nbuf, seed, verbose)
        torch.cuda.current_stream().synchronize()
    return out


def _lowest_states(ctx, psi0, n_iter, degree, tol, fp64_polish, nbuf, seed, verbose):
    """Lowest eigenpairs of S^-1/2 H S^-1/2 (set 0's v_ks and D_ij) starting
    from the orbitals psi0 [norb, nn].  FP32 Chebyshev-filtered subspace
    iteration on norb + nbuf vectors (the buffer vectors converge last and are
    dropped) until the largest residual of the wanted ones is below tol, then
    `fp64_polish` FP64 correction / Rayleigh-Ritz sweeps.  Returns
    (eigenvalues, orbitals complex128 [norb, nn], residual norms)."""
    torch = _torch()
    dv = ctx.system.dv
    nn = ctx.nn
    norb = psi0.shape[0]
    if nbuf is None:
        nbuf = max(8, norb // 4)
    nsub = norb + nbuf
    dt32 = pkg.OPAW_C64
    gen = torch.Generator(device="cuda").manual_seed(seed)

    def noise(n):
        return torch.complex(torch.randn(n, nn, device="cuda", generator=gen),
                             torch.randn(n, nn, device="cuda", generator=gen))

    def smooth_noise(n):
        # Gaussian-filtered noise (sigma = 1.5 Bohr), like the seed orbitals:
        # low Ritz values, so the buffer does not push the filter cut up
        s = ctx.system
        z = noise(n).reshape(n, s.nz, s.ny, s.nx)
        kx = 2 * np.pi * np.fft.fftfreq(s.nx, s.dx)
        ky = 2 * np.pi * np.fft.fftfreq(s.ny, s.dy)
        kz = 2 * np.pi * np.fft.fftfreq(s.nz, s.dz)
        k2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
        filt = torch.from_numpy(np.exp(-k2 * 1.5 * 1.5 / 2.0).astype(np.float32)).to("cuda")
        z = torch.fft.ifftn(torch.fft.fftn(z, dim=(1, 2, 3)) * filt, dim=(1, 2, 3))
        return z.reshape(n, nn).to(torch.complex64)

    X = torch.empty((nsub, nn), dtype=torch.complex64, device="cuda")
    X[:norb] = torch.from_numpy(np.ascontiguousarray(psi0, dtype=np.complex64)).to("cuda")
    X[norb:] = smooth_noise(nbuf)
    HX = torch.empty_like(X)
    Y0 = torch.empty_like(X)
    Y1 = torch.empty_like(X)
    S = torch.empty_like(X)
    _orthonormalise(ctx, dt32, X, S)
    # upper spectral bound: power iteration from white noise (all k present)
    v = noise(1)
    hv = torch.empty_like(v)
    lam_max = 0.0
    for _ in range(60):
        v = v / torch.sqrt((v.abs() ** 2).sum())
        _shs(ctx, dt32, v, hv)
        lam_max = float(torch.sqrt((hv.abs() ** 2).sum()))
        v = hv
    # the power iteration approaches the sparse top of the kinetic spectrum
    # from below; the filter must not amplify anything above b, so also take
    # the kinetic maximum (ek.f90) plus the largest potential, with margins
    s_ = ctx.system
    tmax = 0.5 * ((np.pi / s_.dx) ** 2 + (np.pi / s_.dy) ** 2 + (np.pi / s_.dz) ** 2)
    if s_.ekcut > 0:
        tmax = min(tmax, s_.ekcut)
    vmax = float(np.max(ctx.get_vks(0)))
    lam_max = 1.1 * max(lam_max, tmax + max(vmax, 0.0)) + 0.5
    _shs(ctx, dt32, X, HX)
    w = _rayleigh_ritz(ctx, dt32, X, HX, S)
    for it in range(n_iter):
        res = _residuals(X[:norb], HX[:norb], w[:norb], dv)
        if verbose:
            print(f"chebyshev iteration {it}: eig[0]={w[0]:.6f} eig[norb-1]={w[norb - 1]:.6f} max residual {res.max():.3e}")
        if res.max() < tol:
            break
        # scaled Chebyshev filter damping [a, lam_max] (chebyr_m.f90:20-45)
        a = float(w[-1])
        b = max(lam_max, a + 1.0)
        e = 0.5 * (b + a)
        h = 0.5 * (b - a)
        sigma = h / (float(w[0]) - e)
        sigma1 = sigma
        # degree capped so the filter amplifies the lowest Ritz direction at
        # most ~300x over the cut: the filtered block stays well conditioned
        # for single-precision orthonormalisation
        x0 = (e - float(w[0])) / h
        m = degree
        if x0 > 1.0:
            m = int(max(2, min(degree, np.floor(np.arccosh(300.0) / np.arccosh(x0)))))
        _shs(ctx, dt32, X, Y1)
        Y1.sub_(e * X).mul_(sigma1 / h)
        Y0.copy_(X)
        for _k in range(2, m + 1):
            sigma2 = 1.0 / (2.0 / sigma1 - sigma)
            _shs(ctx, dt32, Y1, HX)
            HX.sub_(e * Y1).mul_(2.0 * sigma2 / h).sub_((sigma * sigma2) * Y0)
            Y0, Y1, HX = Y1, HX, Y0
            sigma = sigma2
        X.copy_(Y1)
        if verbose:
            print(f"  filter a={a:.4f} b={b:.4f} m={m} lam_max={lam_max:.3f} |Y| max row {float(torch.sqrt((X.abs() ** 2).sum(dim=1)).max()):.3e}")
        _orthonormalise(ctx, dt32, X, S, refill=smooth_noise)
        _shs(ctx, dt32, X, HX)
        w = _rayleigh_ritz(ctx, dt32, X, HX, S)
    # FP64 polish of the wanted vectors
    X64 = X[:norb].to(torch.complex128)
    H64 = torch.empty_like(X64)
    S64 = torch.empty_like(X64)
    dt64 = pkg.OPAW_C128
    dtg = pkg.OPAW_C128_DD  # Gram matrices and rotations in double-FP32 arithmetic
    _orthonormalise(ctx, dtg, X64, S64)
    _shs(ctx, dt64, X64, H64)
    w = _rayleigh_ritz(ctx, dtg, X64, H64, S64)
    for _ in range(fp64_polish):
        ww = torch.as_tensor(w, device="cuda", dtype=torch.float64)
        R = H64 - X64 * ww[:, None]
        X64.sub_(R / (lam_max - ww[:, None]))
        _orthonormalise(ctx, dtg, X64, S64)
        _shs(ctx, dt64, X64, H64)
        w = _rayleigh_ritz(ctx, dtg, X64, H64, S64)
    res = _residuals(X64, H64, w, dv)
    if not np.all(np.isfinite(res)):
        raise RuntimeError("ground-state iteration produced non-finite orbitals")
    return w, X64.cpu().numpy(), res


def stationary_system(system, psi):
    """Shift v_loc and D0 of `system` so that the Hamiltonian rebuilt from the
    orbitals psi (rho_ij, density, n^, v_H, v_xc, D_ij of tddft_rhoij.f90,
    tddft_dens.f90, nhat.f90, tddft_pot.f90, get_dij.f90) equals
    v_ks = system.vks0 and D = system.dij_init.  Returns a new System."""
    target_v = np.asarray(system.vks0, np.float64)
    target_d = np.asarray(system.dij_init, np.float64)
    s1 = system
    for _ in range(2):  # v_loc first (it changes Dhat), then D0
        ctx = pkg.Context(s1)
        ctx.upload(0, psi)
        ctx.rebuild(0, pkg.PREC_FP64)
        vks = ctx.get_vks(0)
        dij = ctx.get_dij(0)
        ctx.close()
        s1 = dataclasses.replace(s1, vloc=s1.vloc + (target_v - vks), dij0=s1.dij0 + (target_d - dij))
    return s1


def scf(ctx, psi0, max_iter=60, tol_v=1e-7, tol_res=1e-5, beta=0.3, ndiis=6, filter_iter=2, verbose=False,
        filter_tol_frac=0.0):
    """Self-consistent ground state on the device, the loop of main.f90:67-96:
    each iteration rebuilds v_ks and D_ij from the current orbitals
    (ncpaw_make_hamiltonian: rho_ij, density, n^, Hartree, LDA, D_ij, all
    FP64 on the device), mixes the joint vector [v_ks, D_ij] with Pulay/DIIS
    extrapolation of the residuals (diis.f90: residual = rebuilt - input,
    a history of ndiis pairs, linear mixing beta), and runs `filter_iter`
    warm-started Chebyshev filter passes with orthogonalisation and
    Rayleigh-Ritz (chebyr_m.f90, orthog_phi.f90, diag.f90) in that potential.
    With filter_tol_frac > 0 the filter passes of an iteration stop early
    once the largest eigen-residual is below filter_tol_frac x the last
    max |dv_ks| (up to `filter_iter` passes): the subspace then follows the
    potential as closely as the potential has converged.
    Stops when the largest change of v_ks is below tol_v and the largest
    eigen-residual below tol_res.  The orbitals live in set 0 of ctx; the
    input potentials of the first iteration are the ones ctx holds.  Returns
    (eigenvalues, orbitals complex128 [norb, nn], history of
    (max |dv_ks|, max residual))."""
    psi = np.ascontiguousarray(psi0, dtype=np.complex128)
    norb = psi.shape[0]
    nn = ctx.nn
    x_in = np.concatenate([ctx.get_vks(0), ctx.get_dij(0)])
    xs, rs = [], []
    hist = []
    w = res = None
    for it in range(max_iter):
        ctx.upload(0, psi)
        ctx.rebuild(0, pkg.PREC_FP64)
        x_out = np.concatenate([ctx.get_vks(0), ctx.get_dij(0)])
        r = x_out - x_in
        dv = float(np.abs(r[:nn]).max())
        if res is not None:
            hist.append((dv, float(res.max())))
            if verbose:
                print(f"scf iteration {it}: max |dv_ks| {dv:.3e}, max eigen-residual {res.max():.3e}")
            if dv < tol_v and res.max() < tol_res:
                break
        xs.append(x_in)
        rs.append(r)
        xs, rs = xs[-ndiis:], rs[-ndiis:]
        m = len(rs)
        if m == 1:
            x_next = x_in + beta * r
        else:
            B = np.empty((m + 1, m + 1))
            for i in range(m):
                for j in range(m):
                    B[i, j] = float(np.dot(rs[i], rs[j]))
            B[:m, m] = B[m, :m] = 1.0
            B[m, m] = 0.0
            rhs = np.zeros(m + 1)
            rhs[m] = 1.0
            cvec = np.linalg.lstsq(B, rhs, rcond=None)[0][:m]
            x_next = sum(c * (xv + beta * rv) for c, xv, rv in zip(cvec, xs, rs))
        ctx.set_vks(0, x_next[:nn])
        ctx.set_dij(0, x_next[nn:])
        x_in = x_next
        ftol = max(1e-9, filter_tol_frac * dv) if filter_tol_frac > 0 else 0.0
        w, psi, res = lowest_states(ctx, psi, n_iter=filter_iter, tol=ftol, fp64_polish=3 if ftol > 0 else 1,
                                    seed=it, verbose=False)
    else:
        raise RuntimeError(f"SCF did not converge in {max_iter} iterations: last (max |dv|, residual) "
                           f"{hist[-1] if hist else None}")
    return w, psi, hist


def self_consistent_state(system, norb, seed=2025, max_iter=100, tol_v=3e-6, tol_res=1e-5, polish_tol=1e-6,
                          verbose=False):
    """Self-consistent ground state of `system` with `norb` doubly occupied
    orbitals, from its initial potentials (system.vks0, system.dij_init):
    Chebyshev-filtered lowest states in that potential, the SCF loop of
    `scf` (main.f90:67-96), the lowest states polished to `polish_tol` in the
    last rebuilt potential, and `stationary_system` so that the rebuild of the
    returned orbitals reproduces that potential exactly (the shifts are of
    the size of the SCF's last potential change).  Returns (system with the
    self-consistent v_ks and D_ij as vks0 / dij_init, orbitals complex128
    [norb, nn], eigenvalues, max eigen-residual, SCF history)."""
    from . import synthetic

    psi0 = synthetic.orbitals(system, norb, seed=seed).reshape(norb, -1)
    ctx = pkg.Context(system)
    try:
        ctx.set_vks(0, system.vks0)
        ctx.set_dij(0, system.dij_init)
        w, psi, res = lowest_states(ctx, psi0, n_iter=80, tol=1e-3)
        w, psi, hist = scf(ctx, psi, max_iter=max_iter, tol_v=tol_v, tol_res=tol_res, verbose=verbose,
                           filter_iter=16, filter_tol_frac=0.03)
        vks, dij = ctx.get_vks(0), ctx.get_dij(0)
        w, psi, res = lowest_states(ctx, psi, n_iter=80, tol=polish_tol)
    finally:
        ctx.close()
    s1 = stationary_system(dataclasses.replace(system, vks0=vks, dij_init=dij), psi)
    return s1, psi, w, float(res.max()), hist
