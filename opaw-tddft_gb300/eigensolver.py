"""Preconditioned block eigensolver for the ground state (the lowest
eigenpairs of S^-1/2 H S^-1/2 with a fixed Hamiltonian).

The reference finds its ground state with a Chebyshev-filtered subspace
iteration and DIIS-mixed SCF (chebyr_m.f90:1-48, orthog_phi.f90, diag.f90,
main.f90:67-96, restated in `groundstate`); it has no preconditioner.  This
module adds LOBPCG (Knyazev, SIAM J. Sci. Comput. 23, 517 (2001)): per
iteration the Rayleigh-Ritz problem on span[X, W, P] (current vectors,
preconditioned residuals, previous directions), with

* the Teter-Payne-Allan kinetic preconditioner (opaw_precond_kinetic_dev),
  the plain method, or
* in the complex128 phase, that preconditioner's direction K r together
  with the one corrected by the learned 3D-conv network, K r + |r| N
  (opaw_precond_learned_dev, `learned.Net`): both join the basis, so the
  Rayleigh-Ritz step uses the network's direction as far as it helps (or
  the learned direction alone, with K r as the fallback when it stalls).
  In the complex64 phase the augmented basis converges far more slowly
  (measured: 351 instead of 79 complex64 iterations on C26H16), so the
  network is not used there.

Every operator runs in libopaw_gb300.so: S^-1/2 H S^-1/2 (opaw_shs_apply_dev),
the Gram matrices of the Rayleigh-Ritz step (opaw_gram_herm_dev), the subspace
rotations (opaw_rotate_dev) — in the complex128 phase both in double-FP32
arithmetic (OPAW_C128_DD) — the preconditioners and the kinetic energies
they scale with; the small dense eigenproblems (3m x 3m) run on the host in
FP64.  The iteration runs in complex64 until the largest residual is below
`switch_tol` (1e-5: a complex64 iteration costs a fraction of a complex128
one, whose Gram work is FP64), then in complex128 until the judge, the
unpreconditioned eigen-residual max_i |H x_i - eps_i x_i| (dv norm), is
below `tol`.  Converged columns are soft-locked: they stay in X and in the
Rayleigh-Ritz step but add no W or P directions.
"""
from __future__ import annotations

import time

import numpy as np

import opaw_tddft_gb300 as pkg


def _torch():
    import torch

    return torch


class Result:
    def __init__(self):
        self.eigenvalues = None
        self.orbitals = None
        self.residuals = None
        self.iterations = 0
        self.iterations_fp32 = 0
        self.seconds = 0.0
        self.history = []  # (iteration, max residual, seconds)
        self.converged = False
        self.fallback_iteration = None  # learned_mode "replace": where K r took over


def _rr(ctx, dt, S, HS, m, drop=1e-12):
    """Rayleigh-Ritz on span(S): canonical orthogonalisation of the Gram
    matrix (small eigenvalues dropped), the m lowest Ritz pairs.  Returns
    (theta[m], Y [ns, m]) with the Ritz vectors S^T Y."""
    ns = S.shape[0]
    G = ctx.gram_herm_dev(dt, S.data_ptr(), S.data_ptr(), ns)
    Hs = ctx.gram_herm_dev(dt, S.data_ptr(), HS.data_ptr(), ns)
    lg, Vg = np.linalg.eigh(G)
    keep = lg > drop * lg.max()
    B = Vg[:, keep] / np.sqrt(lg[keep])[None, :]
    Hr = B.conj().T @ Hs @ B
    Hr = 0.5 * (Hr + Hr.conj().T)
    th, C = np.linalg.eigh(Hr)
    return th[:m], B @ C[:, :m]


def lobpcg(ctx, X0, net=None, tol=1e-8, switch_tol=1e-5, max_iter=400, record=None, record_every=4,
           verbose=False, learned_mode="augment", lock=True, learned_frac=1.0):
    """Lowest len(X0) eigenpairs of S^-1/2 H S^-1/2 (set 0's v_ks and D_ij)
    from the starting orbitals X0 [m, nn].  net: a trained `learned.Net`
    (None: the plain kinetic preconditioner).  learned_mode: "augment" puts
    both K r and the learned K r + |r| N in the basis; "replace" uses the
    learned direction alone, falling back to K r for the rest of the solve
    when the largest residual has not fallen by 10% over 6 iterations.
    learned_frac: in "augment" mode the learned direction is formed only for
    this fraction of the unconverged columns, those with the largest
    residuals (the Rayleigh-Ritz basis grows by that many vectors).
    lock: columns whose residual is below tol contribute no W or P
    directions (soft locking; they stay in X and in the Rayleigh-Ritz step).
    record: a list that receives (X, R, eps) of every `record_every`-th
    complex128 iteration (device tensors) for training.  Every torch
    operation runs on the library's stream.  Returns a `Result`."""
    if learned_mode not in ("augment", "replace"):
        raise ValueError("learned_mode must be 'augment' or 'replace'")
    torch = _torch()
    with torch.cuda.stream(torch.cuda.ExternalStream(ctx.stream)):
        out = _lobpcg(ctx, X0, net, tol, switch_tol, max_iter, record, record_every, verbose, learned_mode, lock,
                      learned_frac)
        torch.cuda.current_stream().synchronize()
    return out


def _lobpcg(ctx, X0, net, tol, switch_tol, max_iter, record, record_every, verbose, learned_mode, lock,
            learned_frac):
    torch = _torch()
    res = Result()
    dv = ctx.system.dv
    m = X0.shape[0]
    t0 = time.perf_counter()
    phases = [(pkg.OPAW_C64, torch.complex64, max(switch_tol, tol)), (pkg.OPAW_C128, torch.complex128, tol)]
    X = torch.from_numpy(np.ascontiguousarray(X0)).to("cuda")
    it = 0
    w = None
    for dt, tdt, ptol in phases:
        # the complex128 phase's Gram matrices and rotations in double-FP32
        # arithmetic (~1e-14 relative; FP64 runs at 1/64 of the FP32 rate)
        gdt = pkg.OPAW_C128_DD if dt == pkg.OPAW_C128 else dt
        X = X.to(tdt).contiguous()
        nn = X.shape[1]
        # orthonormal start of the phase, its Ritz pairs
        HX = torch.empty_like(X)
        ctx.shs_apply_dev(0, dt, X.data_ptr(), HX.data_ptr(), m)
        S0 = X
        th, Y = _rr(ctx, gdt, S0, HX, m)
        Xn = torch.empty_like(X)
        ctx.rotate_dev(gdt, X.data_ptr(), m, Y, Xn.data_ptr())
        HXn = torch.empty_like(X)
        ctx.rotate_dev(gdt, HX.data_ptr(), m, Y, HXn.data_ptr())
        X, HX, w = Xn, HXn, th
        P = HP = None
        pvalid = None
        hist = []  # largest residual per iteration of the phase
        fallback = False
        fresh = True  # HX is H X itself, not the rotated recurrence
        since = 0
        best = np.inf
        # Gram eigenvalues below drop x the largest are rounding noise of the
        # phase's precision and are left out of the Rayleigh-Ritz basis
        drop = 1e-6 if dt == pkg.OPAW_C64 else 1e-13
        while it < max_iter:
            if not fresh and since >= 8:  # the recurrence HX drifts from H X: refresh it
                ctx.shs_apply_dev(0, dt, X.data_ptr(), HX.data_ptr(), m)
                fresh, since = True, 0
            ww = torch.as_tensor(w, device="cuda", dtype=torch.float64).to(X.real.dtype)
            R = HX - X * ww[:, None]
            rn = torch.sqrt((R.abs() ** 2).sum(dim=1).double() * dv).cpu().numpy()
            res.history.append((it, float(rn.max()), time.perf_counter() - t0))
            if verbose:
                print(f"lobpcg {'fp32' if dt == pkg.OPAW_C64 else 'fp64'} it {it}: max residual {rn.max():.3e}")
            if dt == pkg.OPAW_C64:
                if rn.max() > 10.0 * best:
                    X = Xbest  # complex64 has reached its rounding floor: go on in complex128
                    break
                if rn.max() < best:
                    Xbest = X.clone()
            best = min(best, float(rn.max()))
            if rn.max() < ptol:
                if fresh:
                    break
                # confirm with H X itself (the judge is the true residual)
                ctx.shs_apply_dev(0, dt, X.data_ptr(), HX.data_ptr(), m)
                fresh, since = True, 0
                continue
            if record is not None and dt == pkg.OPAW_C128 and it % record_every == 0:
                record.append((X.clone(), R.clone(), np.array(w, np.float64)))
            hist.append(float(rn.max()))
            if (net is not None and learned_mode == "replace" and not fallback and len(hist) > 6
                    and hist[-1] > 0.9 * hist[-7]):
                fallback = True  # the learned direction stalls: the kinetic one takes over
                res.fallback_iteration = it
            # soft locking: converged columns add no directions
            ia = np.nonzero(rn >= ptol)[0] if lock else np.arange(m)
            ia_t = torch.as_tensor(ia, device="cuda")
            Ra = R if len(ia) == m else R[ia_t].contiguous()
            Xa = X if len(ia) == m else X[ia_t].contiguous()
            wa = np.asarray(w, np.float64)[ia]
            ekin = ctx.kinetic_energy_dev(dt, Xa.data_ptr(), len(ia))
            W = torch.empty_like(Ra)
            ctx.precond_kinetic_dev(dt, Ra.data_ptr(), ekin, W.data_ptr(), len(ia))
            if net is not None and dt == pkg.OPAW_C128 and not fallback:
                # augment: the learned direction joins the kinetic one
                # (span[X, K r, K r + |r| N, P]), so the Rayleigh-Ritz step
                # takes what helps; replace: the learned direction alone
                if learned_mode == "augment" and learned_frac < 1.0:
                    nb = max(1, int(np.ceil(learned_frac * len(ia))))
                    ib = np.argsort(-rn[ia])[:nb]  # the hardest columns
                    ib_t = torch.as_tensor(ib, device="cuda")
                    Rb = Ra[ib_t].contiguous()
                    WL = torch.empty_like(Rb)
                    net.apply(ctx, dt, Rb.data_ptr(), wa[ib], np.asarray(ekin)[ib], WL.data_ptr(), nb)
                else:
                    WL = torch.empty_like(Ra)
                    net.apply(ctx, dt, Ra.data_ptr(), wa, ekin, WL.data_ptr(), len(ia))
                W = torch.cat([W, WL]) if learned_mode == "augment" else WL
            # unit columns: the residual directions shrink with convergence
            # and would otherwise fall under the Gram matrix's drop threshold
            W /= torch.sqrt((W.abs() ** 2).sum(dim=1, keepdim=True) * dv).clamp_min(1e-300).to(W.real.dtype)
            HW = torch.empty_like(W)
            ctx.shs_apply_dev(0, dt, W.data_ptr(), HW.data_ptr(), W.shape[0])
            blocks, hblocks = [X, W], [HX, HW]
            if P is not None:
                ip = ia[pvalid[ia]]
                if len(ip):
                    ip_t = torch.as_tensor(ip, device="cuda")
                    Pa, HPa = P[ip_t], HP[ip_t]
                    pn = torch.sqrt((Pa.abs() ** 2).sum(dim=1, keepdim=True) * dv).clamp_min(1e-300).to(Pa.real.dtype)
                    blocks.append(Pa / pn)
                    hblocks.append(HPa / pn)
            S = torch.cat(blocks)
            HS = torch.cat(hblocks)
            th, Y = _rr(ctx, gdt, S, HS, m, drop)
            ns = S.shape[0]
            Xn = torch.empty_like(X)
            HXn = torch.empty_like(X)
            ctx.rotate_dev(gdt, S.data_ptr(), ns, Y, Xn.data_ptr())
            ctx.rotate_dev(gdt, HS.data_ptr(), ns, Y, HXn.data_ptr())
            # the new directions of the active columns: the part of their Ritz
            # vectors outside span(X)
            Ya = np.ascontiguousarray(Y[m:][:, ia])
            St, HSt = S[m:].contiguous(), HS[m:].contiguous()
            Pn_a = torch.empty_like(Ra)
            HPn_a = torch.empty_like(Ra)
            ctx.rotate_dev(gdt, St.data_ptr(), ns - m, Ya, Pn_a.data_ptr())
            ctx.rotate_dev(gdt, HSt.data_ptr(), ns - m, Ya, HPn_a.data_ptr())
            if len(ia) == m:
                P, HP = Pn_a, HPn_a
            else:
                P = torch.zeros_like(X)
                HP = torch.zeros_like(X)
                P[ia_t] = Pn_a
                HP[ia_t] = HPn_a
            pvalid = np.zeros(m, bool)
            pvalid[ia] = True
            X, HX, w = Xn, HXn, th
            fresh = False
            since += 1
            it += 1
            if dt == pkg.OPAW_C64:
                res.iterations_fp32 = it
        if not np.all(np.isfinite(w)):
            raise RuntimeError("eigensolver produced non-finite Ritz values")
    res.iterations = it
    res.seconds = time.perf_counter() - t0
    res.eigenvalues = np.asarray(w, np.float64)
    res.residuals = rn
    res.converged = bool(rn.max() < tol)
    res.orbitals = X
    return res
