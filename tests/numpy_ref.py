"""A second, independent restatement of the operators in numpy (pure array
code, numpy's FFT), used to cross-check the C oracle on small cases.
Follows the same reference lines as oracle/opaw_oracle.c."""
import numpy as np


def boxes(s):
    """per atom: (flat grid indices of the box points in box order, projector offset)"""
    out = []
    off = 0
    for a in range(s.natom):
        n0, n1, n2 = s.nrough[a]
        i0 = s.ir_start[a] - 1
        bz, by, bx = np.meshgrid(np.arange(n2), np.arange(n1), np.arange(n0), indexing="ij")
        ix = (i0[0] + bx) % s.nx
        iy = (i0[1] + by) % s.ny
        iz = (i0[2] + bz) % s.nz
        g = (ix + s.nx * (iy + s.ny * iz)).reshape(-1)
        out.append((g, off))
        off += int(s.ms[a]) * n0 * n1 * n2
    return out


def proj(s, psi, which):
    """psi [norb, nn] -> [norb, ns]  (proj.f90:19-23, proj1.f90:19-24)"""
    P = s.p3d1 if which else s.p3d
    cols = []
    for a, (g, off) in enumerate(boxes(s)):
        m = int(s.ms[a])
        Pa = P[off:off + m * g.size].reshape(m, g.size)
        cols.append((psi[:, g] @ Pa.T) * s.dv)
    return np.concatenate(cols, axis=1)


def scatter(s, out, coef, which):
    P = s.p3d1 if which else s.p3d
    col = 0
    for a, (g, off) in enumerate(boxes(s)):
        m = int(s.ms[a])
        Pa = P[off:off + m * g.size].reshape(m, g.size)
        np.add.at(out, (slice(None), g), coef[:, col:col + m] @ Pa)
        col += m


def sn_phi(s, psi, n):
    """snphi.f90:14-48"""
    psi = psi.reshape(psi.shape[0], -1)
    c = proj(s, psi, 1)
    sig = s.sinv if n == -1 else (1.0 + s.s) ** n - 1.0
    out = psi.copy()
    scatter(s, out, c * sig[None, :], 1)
    return out


def ek(s):
    def k(n, d):
        i = np.arange(n)
        kk = i * (2 * np.pi / (n * d))
        return np.where(kk > np.pi / d, kk - 2 * np.pi / d, kk)

    kx, ky, kz = k(s.nx, s.dx), k(s.ny, s.dy), k(s.nz, s.dz)
    e = (kx[None, None, :] ** 2 + ky[None, :, None] ** 2 + kz[:, None, None] ** 2) / 2.0
    if s.ekcut > 0:
        e = np.minimum(e, s.ekcut)
    return e / (s.nx * s.ny * s.nz)


def h_phi(s, psi, vks, dij):
    """hphi.f90:14-65"""
    norb = psi.shape[0]
    p3 = psi.reshape(norb, s.nz, s.ny, s.nx)
    t = np.fft.fftn(p3, axes=(1, 2, 3)) * ek(s)
    t = np.fft.ifftn(t, axes=(1, 2, 3)) * (s.nx * s.ny * s.nz)
    out = t.reshape(norb, -1) + psi.reshape(norb, -1) * vks[None, :]
    c = proj(s, psi.reshape(norb, -1), 0)
    col = 0
    doff = 0
    coef = np.zeros_like(c)
    for a in range(s.natom):
        m = int(s.ms[a])
        D = dij[doff:doff + m * m].reshape(m, m, order="F")
        coef[:, col:col + m] = c[:, col:col + m] @ D.T
        col += m
        doff += m * m
    scatter(s, out, coef, 0)
    return out


def shs(s, psi, vks, dij):
    t = sn_phi(s, psi, -0.5)
    u = h_phi(s, t, vks, dij)
    return sn_phi(s, u, -0.5)
