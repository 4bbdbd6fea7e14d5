"""TDDFT restart checkpoints in the reference's `tddft_save/` format.

tddft_write_to_restart.f90:1-66 writes, and read_phi_bar.f90:1-52 reads:

  tddft_save/info              list-directed text: nb nodes it
  tddft_save/phi_bar.bin       Fortran unformatted sequential, one record per
  tddft_save/phi_bar_pert.bin  orbital: complex*16 (nx, ny, nz), x fastest;
                               rank 0's nb orbitals first, then rank 1's, ...

nb is the orbitals per rank and `nodes` the rank count of the run that wrote
the files (the reference refuses to read with another count; here one GPU
holds every orbital, so a file of nodes x nb orbitals is read whole).  `it`
is the step the run had reached.  Host-side numpy code; `save` / `load`
move the resident orbitals of a Context through these files.
"""
from __future__ import annotations

import os
import struct

import numpy as np


def _write_records(path, arrays):
    with open(path, "wb") as f:
        for a in arrays:
            b = np.ascontiguousarray(a, dtype="<c16").tobytes()
            n = struct.pack("<i", len(b))
            f.write(n + b + n)


def _read_records(path, nn, count):
    out = np.empty((count, nn), np.complex128)
    with open(path, "rb") as f:
        for i in range(count):
            h = f.read(4)
            if len(h) < 4:
                raise ValueError(f"{path}: {i} orbital records where {count} were expected")
            (n,) = struct.unpack("<i", h)
            if n != 16 * nn:
                raise ValueError(f"{path}: record {i + 1} holds {n} bytes, a grid of {nn} points needs {16 * nn}")
            out[i] = np.frombuffer(f.read(n), "<c16")
            (m,) = struct.unpack("<i", f.read(4))
            if m != n:
                raise ValueError(f"{path}: corrupt record {i + 1}")
    return out


def write_restart(directory, psi, psi_pert, it, nodes=1):
    """psi, psi_pert: [norb, nz, ny, nx] (or [norb, nn]) complex; norb must be
    a multiple of nodes (nb = norb / nodes orbitals per rank)."""
    psi = np.asarray(psi)
    psi_pert = np.asarray(psi_pert)
    if psi.shape != psi_pert.shape:
        raise ValueError("psi and psi_pert differ in shape")
    norb = psi.shape[0]
    if norb % nodes:
        raise ValueError(f"{norb} orbitals do not split over {nodes} ranks")
    os.makedirs(directory, exist_ok=True)
    with open(os.path.join(directory, "info"), "w") as f:
        f.write(f" {norb // nodes:12d} {nodes:12d} {int(it):12d}\n")
    _write_records(os.path.join(directory, "phi_bar.bin"), psi.reshape(norb, -1))
    _write_records(os.path.join(directory, "phi_bar_pert.bin"), psi_pert.reshape(norb, -1))


def read_restart(directory, nn):
    """Returns (psi, psi_pert, it) with the orbitals as [nodes*nb, nn]."""
    with open(os.path.join(directory, "info")) as f:
        nb, nodes, it = (int(x) for x in f.read().split()[:3])
    count = nb * max(nodes, 1)
    psi = _read_records(os.path.join(directory, "phi_bar.bin"), nn, count)
    pp = _read_records(os.path.join(directory, "phi_bar_pert.bin"), nn, count)
    return psi, pp, it


def save(ctx, directory, it, norb):
    """Checkpoint the resident orbitals of both sets of a Context."""
    write_restart(directory, ctx.download(0, norb).reshape(norb, -1), ctx.download(1, norb).reshape(norb, -1), it)


def load(ctx, directory):
    """Upload a checkpoint into a Context; returns the step it was taken at."""
    psi, pp, it = read_restart(directory, ctx.nn)
    ctx.upload(0, psi)
    ctx.upload(1, pp)
    return it
