"""The TDDFT driver loop of the reference (`opaw_tddft`, tddft.f90:1-95) over
the device step: start from a checkpoint or a ground state, kick, propagate,
write the dipole files and checkpoints.

  restart (n_restart > 0 and tddft_save/ present, tddft.f90:25-28):
      read the orbitals of both sets (read_phi_bar.f90), continue after the
      step they were saved at; the dipole files continue as plot_dip does
  fresh start (tddft.f90:29-58):
      ground-state orbitals from wf_bar.bin / wf_bar.txt (read_wf.f90) or
      from the caller, the kick e^{-i gamma r_ipol} (tddft_excite.f90)
  loop it = istart .. nt (tddft.f90:67-91):
      rebuild + RK4 + dipole (one device call per block of steps), and a
      checkpoint (tddft_write_to_restart.f90) whenever mod(it, n_restart) = 0

Blocks end at every checkpoint step so that the saved orbitals are those of
that step.  Host-side code: everything on the device goes through the
Context.
"""
from __future__ import annotations

import os

import numpy as np

from . import dipfile, restart, wfio

PREC_FP64 = 0
PREC_MIXED = 1


def orbitals_from_wf(path, norb=None):
    """Ground-state orbitals [norb, nn] (complex128) from a wave-function file;
    norb defaults to the occupied count the file records (ihomo), else all."""
    d = wfio.read_wf(path)
    phi = d["phi"].reshape(d["nstates"], -1)
    if norb is None:
        norb = d.get("ihomo", d["nstates"])
    if norb > phi.shape[0]:
        raise ValueError(f"{norb} orbitals requested, the file holds {phi.shape[0]}")
    return np.ascontiguousarray(phi[:norb].astype(np.complex128))


def opaw_tddft(ctx, nt, dt, gamma, workdir=".", ipol=1, psi0=None, wf_path=None, n_restart=0, block=50,
               precision=PREC_MIXED):
    """Runs steps up to nt of a TDDFT run in `workdir`; returns (it_first,
    d_dip) with d_dip [steps run, 3].  The orbitals come from tddft_save/
    when n_restart > 0 and it exists, else from psi0 or wf_path."""
    if nt < 1 or dt <= 0 or block < 1:
        raise ValueError("nt >= 1, dt > 0 and block >= 1 are required")
    save_dir = os.path.join(workdir, "tddft_save")
    if n_restart > 0 and os.path.isdir(save_dir):
        psi, pp, it_restart = restart.read_restart(save_dir, ctx.nn)
        ctx.upload(0, psi)
        ctx.upload(1, pp)
        norb = psi.shape[0]
        log = dipfile.DipoleLog(dt, workdir, it_restart=it_restart)
        istart = it_restart + 1
    else:
        if psi0 is None:
            if wf_path is None:
                raise ValueError("a fresh run needs psi0 or wf_path")
            psi0 = orbitals_from_wf(wf_path)
        psi0 = np.ascontiguousarray(np.asarray(psi0, dtype=np.complex128).reshape(-1, ctx.nn))
        norb = psi0.shape[0]
        ctx.upload(0, psi0)
        ctx.excite(ipol, gamma)
        log = dipfile.DipoleLog(dt, workdir)
        istart = 1
    out = []
    it = istart
    with log:
        while it <= nt:
            n = min(block, nt - it + 1)
            if n_restart > 0:  # end the block at the next checkpoint step
                n = min(n, n_restart - (it - 1) % n_restart)
            dip, dpp, dd = ctx.tddft_steps_dip(n, dt, gamma, precision)
            log.write_steps(it - 1, dip, dpp, dd)
            out.append(dd)
            it += n
            if n_restart > 0 and (it - 1) % n_restart == 0:
                restart.save(ctx, save_dir, it - 1, norb)
    d = np.concatenate(out) if out else np.zeros((0, 3))
    return istart, d


def run_folder(folder, precision=PREC_MIXED, nt=None, block=50, n_restart=0):
    """The reference's program on one of its input folders (main.f90 with
    `dim_paw.inp`'s `tddft` switch): the set-up chain of the folder's
    datasets and geometry (`pawsetup.from_folder`); for `tddft` -1 or 0 the
    self-consistent ground state, written to wf_bar.bin or wf_bar.txt as
    `flg_bin` says (write_wf.f90); for `tddft` 0 or 1 (1: orbitals read from
    that file) the kick `strength` along `exct_pol` and `nt` steps of `dt`
    (theory 3, TDDFT) in `precision`, with d_dip.dat and dip.dat written in
    the folder (tddft_plot.f90).  Returns a dict of what ran."""
    import opaw_tddft_gb300 as pkg

    from . import groundstate, pawsetup, pawxml

    params = pawxml.read_parameters(os.path.join(folder, "dim_paw.inp"))
    mode = int(params.get("tddft", "-1"))
    if mode not in (-1, 0, 1):
        raise ValueError(f"tddft = {mode}: expected -1, 0 or 1")
    if mode >= 0 and int(params.get("theory", "3")) != 3:
        raise ValueError("only theory 3 (TDDFT with the rebuild of every stage) is on this path")
    s = pawsetup.from_folder(folder)
    norb = int(round(s.rnel / 2))
    binary = params.get("flg_bin", "F").upper().startswith("T")
    wf_path = os.path.join(folder, "wf_bar.bin" if binary else "wf_bar.txt")
    out = {"norb": norb, "grid": (s.nx, s.ny, s.nz)}
    psi = None
    if mode in (-1, 0):
        s, psi, w, res, hist = groundstate.self_consistent_state(s, norb)
        wfio.write_wf(wf_path, psi.reshape(norb, s.nz, s.ny, s.nx), w, s.dx, s.dy, s.dz, norb, binary=binary)
        out.update(eigenvalues=w, scf_iterations=len(hist), max_eigen_residual=res)
        if mode == -1:
            return out
    else:
        psi = orbitals_from_wf(wf_path, norb)
    nt = int(params["nt"]) if nt is None else int(nt)
    dt = pawxml.fortran_float(params["dt"])
    gamma = pawxml.fortran_float(params["strength"])
    ipol = int(params.get("exct_pol", "1"))
    ctx = pkg.Context(s)
    try:
        _, d = opaw_tddft(ctx, nt, dt, gamma, workdir=folder, ipol=ipol, psi0=psi, precision=precision,
                          block=block, n_restart=n_restart)
    finally:
        ctx.close()
    out.update(d_dip=d, nt=nt, dt=dt, gamma=gamma, ipol=ipol)
    return out
