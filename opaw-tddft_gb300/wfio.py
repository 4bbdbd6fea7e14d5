"""Wave-function files in the reference's format (wf_bar.bin / wf_bar.txt).

The reference hands ground states to its TDDFT run and to other codes through
these files (write_wf.f90:24-119 writes them, read_wf.f90:130-228 reads them
back for `tddft 1`).  Layout, in order:

  'nx      ' nx / 'ny      ' ny / 'nz      ' nz        (8-character tag + integer)
  'dx      ' dx / 'dy      ' dy / 'dz      ' dz        (tag + real*8)
  'nsp     ' 1 / 'nstates ' n / 'orbmn_wf' 1 / 'ihomo   ' nocc
  'evls    '  then the n eigenvalues (real*8)
  'orbitals'  then per state:  i 1  and the real*8 array (nx, ny, nz), x fastest

The orbital values are real: sign(Re phi) * |phi| (write_wf.f90:54-62).  The
binary form is Fortran unformatted sequential access (a 4-byte record length
before and after every record, default 4-byte integers); the text form is the
same sequence written list-directed.  The reader walks the records by tag, so
it also takes files without the orbmn_wf / ihomo records (the layout
read_wf.f90 itself expects).  Host-side code: numpy only.
"""
from __future__ import annotations

import struct

import numpy as np


def _tag(name: str) -> bytes:
    b = name.encode("ascii")
    if len(b) > 8:
        raise ValueError(f"tag {name!r} longer than 8 characters")
    return b.ljust(8)


def _real_values(phi) -> np.ndarray:
    """sign(Re phi) |phi| for complex orbitals (write_wf.f90:54-62); real
    orbitals pass unchanged."""
    a = np.asarray(phi)
    if np.iscomplexobj(a):
        return np.where(a.real > 0.0, np.abs(a), -np.abs(a))
    return a.astype(np.float64)


def write_wf(path, phi, eig, dx, dy, dz, nocc, binary=True):
    """Writes orbitals phi[nstates, nz, ny, nx] (complex or real) and their
    eigenvalues; binary=False writes the text form (wf_bar.txt)."""
    phi = np.asarray(phi)
    if phi.ndim != 4:
        raise ValueError("phi must be [nstates, nz, ny, nx]")
    ns, nz, ny, nx = phi.shape
    eig = np.asarray(eig, np.float64).reshape(-1)
    if eig.size != ns:
        raise ValueError(f"{eig.size} eigenvalues for {ns} states")
    vals = _real_values(phi).reshape(ns, -1)
    ints = [("nx", nx), ("ny", ny), ("nz", nz)]
    reals = [("dx", dx), ("dy", dy), ("dz", dz)]
    ints2 = [("nsp", 1), ("nstates", ns), ("orbmn_wf", 1), ("ihomo", int(nocc))]
    if binary:
        with open(path, "wb") as f:
            def rec(payload: bytes):
                n = struct.pack("<i", len(payload))
                f.write(n + payload + n)

            for k, v in ints:
                rec(_tag(k) + struct.pack("<i", int(v)))
            for k, v in reals:
                rec(_tag(k) + struct.pack("<d", float(v)))
            for k, v in ints2:
                rec(_tag(k) + struct.pack("<i", int(v)))
            rec(_tag("evls"))
            rec(eig.astype("<f8").tobytes())
            rec(_tag("orbitals"))
            for i in range(ns):
                rec(struct.pack("<ii", i + 1, 1))
                rec(vals[i].astype("<f8").tobytes())
    else:
        with open(path, "w") as f:
            for k, v in ints:
                f.write(f" {k:<8s} {int(v):12d}\n")
            for k, v in reals:
                f.write(f" {k:<8s} {float(v):25.17E}\n")
            for k, v in ints2:
                f.write(f" {k:<8s} {int(v):12d}\n")
            f.write(" evls    \n")
            f.write(_fmt_reals(eig))
            f.write(" orbitals\n")
            for i in range(ns):
                f.write(f" {i + 1:12d} {1:12d}\n")
                f.write(_fmt_reals(vals[i]))


def _fmt_reals(a, per_line=4):
    out = []
    for j in range(0, a.size, per_line):
        out.append(" " + " ".join(f"{v:25.17E}" for v in a[j:j + per_line]) + "\n")
    return "".join(out)


def _records(data: bytes):
    pos = 0
    while pos < len(data):
        (n,) = struct.unpack_from("<i", data, pos)
        payload = data[pos + 4:pos + 4 + n]
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        if m != n:
            raise ValueError(f"corrupt record at byte {pos}: length markers {n} and {m}")
        yield payload
        pos += n + 8


def read_wf(path, binary=None):
    """Reads a wave-function file; returns a dict with the header values,
    'eig' and 'phi' [nstates, nz, ny, nx] (real).  binary=None decides from
    the file's first bytes."""
    with open(path, "rb") as f:
        data = f.read()
    if binary is None:
        binary = len(data) >= 4 and struct.unpack_from("<i", data, 0)[0] in (12, 16)
    if binary:
        return _read_bin(data)
    return _read_txt(data.decode("ascii"))


_INT_TAGS = ("nx", "ny", "nz", "nsp", "nstates", "orbmn_wf", "ihomo")
_REAL_TAGS = ("dx", "dy", "dz")


def _read_bin(data: bytes):
    it = _records(data)
    hdr = {}
    eig = None
    for rec in it:
        tag = rec[:8].decode("ascii").strip()
        if tag in _INT_TAGS:
            hdr[tag] = struct.unpack_from("<i", rec, 8)[0]
        elif tag in _REAL_TAGS:
            hdr[tag] = struct.unpack_from("<d", rec, 8)[0]
        elif tag == "evls":
            eig = np.frombuffer(next(it), "<f8").copy()
        elif tag == "orbitals":
            break
        else:
            raise ValueError(f"unexpected record {rec[:8]!r}")
    nx, ny, nz, ns = hdr["nx"], hdr["ny"], hdr["nz"], hdr["nstates"]
    phi = np.empty((ns, nz, ny, nx))
    for i in range(ns):
        idx = struct.unpack("<ii", next(it))
        if idx[0] != i + 1:
            raise ValueError(f"state record {idx[0]} where {i + 1} was expected")
        v = np.frombuffer(next(it), "<f8")
        if v.size != nx * ny * nz:
            raise ValueError(f"state {i + 1}: {v.size} values for a {nx}x{ny}x{nz} grid")
        phi[i] = v.reshape(nz, ny, nx)
    return dict(hdr, eig=eig, phi=phi)


def _expand(tokens):
    """List-directed input allows r*c repeat counts."""
    for t in tokens:
        if "*" in t:
            r, c = t.split("*", 1)
            for _ in range(int(r)):
                yield c
        else:
            yield t


def _read_txt(text: str):
    toks = iter(list(_expand(text.split())))
    hdr = {}
    eig = None
    while True:
        tag = next(toks)
        if tag in _INT_TAGS:
            hdr[tag] = int(next(toks))
        elif tag in _REAL_TAGS:
            hdr[tag] = float(next(toks).replace("D", "E").replace("d", "e"))
        elif tag == "evls":
            eig = np.array([float(next(toks).replace("D", "E")) for _ in range(hdr["nstates"])])
        elif tag == "orbitals":
            break
        else:
            raise ValueError(f"unexpected token {tag!r}")
    nx, ny, nz, ns = hdr["nx"], hdr["ny"], hdr["nz"], hdr["nstates"]
    phi = np.empty((ns, nz * ny * nx))
    for i in range(ns):
        i_orb = int(next(toks))
        next(toks)  # spin index
        if i_orb != i + 1:
            raise ValueError(f"state {i_orb} where {i + 1} was expected")
        phi[i] = [float(next(toks).replace("D", "E")) for _ in range(nx * ny * nz)]
    return dict(hdr, eig=eig, phi=phi.reshape(ns, nz, ny, nx))
