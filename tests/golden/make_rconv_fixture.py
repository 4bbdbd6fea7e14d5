"""Generates tests/golden/rconv_8x6x3.npz: the reference's own known-answer
check of the r2c Hartree convolution (src/lib/library_rconv_drv.f90:5-95).

Inputs follow its gin_bk_set (:22-50) on an 8x6x3 grid; the expected output
follows its rconv_ana (:52-94): a brute-force O(N^2) DFT, times bk, then the
conjugate-DFT-conjugate inverse divided by N.  Arrays are stored in numpy C
order (z, y, x), i.e. Fortran (x, y, z) with x fastest.
"""
import os

import numpy as np

NX, NY, NZ = 8, 6, 3


def inputs():
    gin = np.zeros((NZ, NY, NX))
    bk = np.zeros((NZ, NY, NX))
    for ix in range(1, NX + 1):
        for iy in range(1, NY + 1):
            for iz in range(1, NZ + 1):
                x, y, z = ix - NX / 2.0, iy - NY / 2.0, iz - NZ / 2.0
                gin[iz - 1, iy - 1, ix - 1] = np.exp(
                    -(x + 0.4) ** 2 * 0.5 - (x - 1.9) * (y - 0.7) * 0.4 + (x - y) * (x - 0.5) * 0.2 - (z + y) ** 2 * 0.4
                )
                x, y, z = ix - 1.0, iy - 1.0, iz - 1.0
                if ix > NX // 2 + 1:
                    x -= NX
                if iy > NY // 2 + 1:
                    y -= NY
                if iz > NZ // 2 + 1:
                    z -= NZ
                bk[iz - 1, iy - 1, ix - 1] = 1.0 / max(x * x + 0.8 * y * y + 0.5 * z * z, 0.1)
    return gin, bk


def fft_ana(g):
    """h(k) = sum_j g(j) exp(-2 pi i k.j / n), written as the brute-force sum."""
    h = np.zeros_like(g, dtype=np.complex128)
    jz, jy, jx = np.meshgrid(np.arange(NZ), np.arange(NY), np.arange(NX), indexing="ij")
    for kz in range(NZ):
        for ky in range(NY):
            for kx in range(NX):
                ph = np.exp(-2j * np.pi * (kx * jx / NX + ky * jy / NY + kz * jz / NZ))
                h[kz, ky, kx] = np.sum(g * ph)
    return h


def expected(gin, bk):
    gk = fft_ana(gin.astype(np.complex128))
    gk = gk * bk
    gk = np.conj(fft_ana(np.conj(gk)))
    return (gk / (NX * NY * NZ)).real


if __name__ == "__main__":
    gin, bk = inputs()
    gana = expected(gin, bk)
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "rconv_8x6x3.npz")
    np.savez(out, gin=gin, bk=bk, gana=gana)
    print(out, float(np.abs(gana).sum()))
