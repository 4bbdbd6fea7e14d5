"""PAW set-up chain: from PAW-XML datasets and a geometry to the operator
tables of `opaw_system` (the `System` of synthetic.py).

This is the host-side chain the reference runs once before the propagation
(prepare_paw / ncpaw_libpaw_prepare), restated step by step:

* per species (readpaw, read_paw.f90:1-67): the radial overlaps of the
  projectors and of phi^2 - phi~^2 inside rcut + rpad_r (read_p_phi,
  :482-539), their per-l orthogonalisation (transform_pphi.f90:1-70,
  :146-190: O^-1/2 on the projectors, O^1/2 on the partial waves, then the
  eigenvectors of O^1/2 (phi^2 - phi~^2) O^1/2), the channel layout (state,
  m) (get_nm, :429-480), the compensation shape functions g_l normalised to
  sum r^(l+2) g_l dr = 1 (get_gl, :112-182; the `sinc` and `bessel` forms), the moments
  Q_ij^LM = n_ij^L G^LM_ij and the diagonal overlap s_ij from the
  orthogonalised waves (calc_qijlm, :695-782), the box size nrough (get_nrcut,
  :229-272) and the natural-cubic-spline transfer matrices from the fine
  grid to the box grid (get_b, :274-345);
* per atom: the box corner (get_irs.f90:18-24), the projectors on the fine
  grid (linear radial interpolation x real Y_lm, p3d.f90:120-215) contracted
  to the box with the transfer matrices (get_p3d_r, p3d.f90:79-118), the grid
  orthonormalisation of the orthogonalised projectors with the overlap
  spectrum s (transform_p3d.f90:1-99), the sphere points r < rcut
  (map_localgrid.f90:4-60) and g_L Y_LM on them (g3d.f90:1-119);
* the libpaw tables the reference takes from `pawtab`: D0 = K_ij +
  <phi_i|v_H(n_Zc)|phi_j> - <phi~_i|v_H(n~_Zc)|phi~_j> (atompaw_dij0,
  libpaw 2_m_paw_atom.F90:362-450) and E_ijkl, the second derivative of the
  on-site Hartree energy E_H[n^1] - E_H[n~^1 + n^] in rho_ij (pawinit,
  libpaw m_paw_init.F90:509-600, eq. A17 of Holzwarth et al., PRB 55, 2005
  (1997)), and the radial tables of the on-site XC term;
* the local potential and the pseudo core density on the grid, band-limited
  to the grid as the reference builds them in reciprocal space (atm2fft of
  libpaw m_atm2fft.F90 for n~_c; the form factors of vloc/vloc_prep.f90 for
  an isolated system's v_loc): n~_c and the short-range part v_loc + Z_val
  erf(r / r_g) / r go through their radial form factors 4 pi int f j0(G r)
  r^2 dr and the structure factor of the atoms on the grid's own G vectors;
  the long-range -Z_val erf(r / r_g) / r, smooth at r_g = 1.2 Bohr, is summed
  in real space without periodic images.

Radial integrals that the reference forms as plain sums f(r_i) dr_i keep that
rule (the overlaps, the moments, the shape-function norm); the libpaw
integrals (D0, E_ijkl) use the cubic-spline antiderivative of f dr/di in the
mesh index, a fourth-order rule like libpaw's Simpson integration.
Partial waves up to l = 1 are supported (nine LM moments)."""
from __future__ import annotations

import math

import numpy as np
from scipy.interpolate import CubicSpline

from . import synthetic

SQ4PI = math.sqrt(4.0 * math.pi)
RPAD = 1.0  # box padding for the spline transfer (0_parameter.f90:15)
RPAD_R = 2.0  # radial overlap range beyond rcut (0_parameter.f90:16)
TOLL_SIJ = 0.01  # floor of 1 + s_ii (0_parameter.f90:20)


# ---------------------------------------------------------------- helpers

def ylm(l, m, x, y, z):
    """Real spherical harmonics of unit vectors in the order of ylm.f90:4-60
    (m = -1 -> y, 0 -> z, 1 -> x for l = 1; xy, yz, 3z^2 - r^2, xz, x^2 - y^2
    for l = 2)."""
    p0 = 0.5 / math.sqrt(math.pi)
    if l == 0:
        return np.full(np.shape(x), p0)
    if l == 1:
        return math.sqrt(3.0) * p0 * {-1: y, 0: z, 1: x}[m]
    if l == 2:
        p2 = math.sqrt(15.0) * p0
        return {-2: p2 * x * y, -1: p2 * y * z, 0: p2 * (2 * z * z - x * x - y * y) / (2 * math.sqrt(3.0)),
                1: p2 * x * z, 2: p2 * (x * x - y * y) / 2.0}[m]
    raise ValueError(f"l = {l} not supported")


def real_gaunt(lmax_wave=1):
    """G[LM, lm_i, lm_j] = integral of Y_LM Y_i Y_j over the sphere for L <=
    2 lmax_wave and waves up to lmax_wave, by Gauss-Legendre x uniform-phi
    quadrature (exact for these degrees).  Equals cg3 of cg.f90:71-134."""
    t, w = np.polynomial.legendre.leggauss(16)
    ph = np.arange(32) * 2.0 * math.pi / 32
    T, P = np.meshgrid(t, ph, indexing="ij")
    W = np.outer(w, np.full(32, 2.0 * math.pi / 32))
    st = np.sqrt(1.0 - T * T)
    X, Y, Z = st * np.cos(P), st * np.sin(P), T
    waves = [(l, m) for l in range(lmax_wave + 1) for m in range(-l, l + 1)]
    Ls = [(L, M) for L in range(2 * lmax_wave + 1) for M in range(-L, L + 1)]
    yw = [ylm(l, m, X, Y, Z) for (l, m) in waves]
    G = np.zeros((len(Ls), len(waves), len(waves)))
    for a, (L, M) in enumerate(Ls):
        yL = ylm(L, M, X, Y, Z) * W
        for i in range(len(waves)):
            for j in range(len(waves)):
                G[a, i, j] = float(np.sum(yL * yw[i] * yw[j]))
    return G, waves


def bracket(r, t):
    """interpolate.f90: the mesh interval r[i] <= t < r[i+1] (0-based i,
    clipped to the mesh) and the linear weights of its two ends."""
    t = np.asarray(t, dtype=np.float64)
    i = np.clip(np.searchsorted(r, t, side="right") - 1, 0, r.size - 2)
    w2 = (t - r[i]) / (r[i + 1] - r[i])
    return i, 1.0 - w2, w2


def upper_count(r, t):
    """Number of mesh points up to and including the upper end of t's interval."""
    i, _, _ = bracket(r, t)
    return int(i) + 2


def cumint(f, dr):
    """Cumulative integral of f dr along the mesh: the cubic-spline
    antiderivative of f dr/di in the mesh index."""
    n = f.shape[-1]
    idx = np.arange(n, dtype=np.float64)
    return CubicSpline(idx, f * dr, axis=-1).antiderivative()(idx)


def hartree_radial(n, r, dr, L):
    """Potential of the L component of a density n(r) (3D units): v(r) =
    4 pi / (2L+1) [r^-(L+1) int_0^r n r'^(L+2) dr' + r^L int_r^R n r'^(1-L) dr']."""
    inner = cumint(n * r ** (L + 2), dr)
    outer_all = cumint(n * r ** (1 - L), dr)
    outer = outer_all[-1] - outer_all
    return 4.0 * math.pi / (2 * L + 1) * (inner / r ** (L + 1) + outer * r ** L)


def _sph_jn(l, x, derivative=False):
    from scipy.special import spherical_jn

    return spherical_jn(l, x, derivative=derivative)


def _bessel_shape(l, rc):
    """atompaw_shapebes: q_1, q_2 = the first two positive zeros of j_l over
    rc, and (a_1, a_2) with sum a_i q_i j_l'(q_i rc) = 0 and sum a_i
    rc^(l+2) j_(l+1)(q_i rc) / q_i = 1 (the moment int_0^rc j_l(q r)
    r^(l+2) dr)."""
    from scipy.optimize import brentq

    roots = []
    x = 1e-3
    f0 = _sph_jn(l, x)
    while len(roots) < 2:
        x1 = x + 0.05
        f1 = _sph_jn(l, x1)
        if f0 * f1 < 0:
            roots.append(brentq(lambda t: _sph_jn(l, t), x, x1, xtol=1e-15))
        x, f0 = x1, f1
    q = np.array(roots) / rc
    A = np.array([[q[i] * _sph_jn(l, q[i] * rc, derivative=True) for i in range(2)],
                  [rc ** (l + 2) * _sph_jn(l + 1, q[i] * rc) / q[i] for i in range(2)]])
    a = np.linalg.solve(A, np.array([0.0, 1.0]))
    return a, q


# ---------------------------------------------------------------- species

class Species:
    """Per-element tables of readpaw (read_paw.f90), transform_pphi and libpaw's
    pawinit for one dataset (they do not depend on the grid)."""

    def __init__(self, d):
        self.d = d
        self.symbol = d["symbol"]
        self.Z, self.zval = float(d["Z"]), float(d["valence"])
        r = np.maximum(d["r"], 1e-8)  # read_rr, read_paw.f90:547
        dr = d["dr"]
        self.r, self.dr = r, dr
        self.rcut = float(d["rpaw"])
        self.rcomp = float(d["rcomp"])
        lst = np.asarray(d["l"], int)
        if lst.max() > 1:
            raise ValueError(f"{self.symbol}: partial waves with l > 1 are not supported")
        self.lstate = lst
        ns = lst.size
        phi, tphi, pt = (np.asarray(d[k], np.float64) for k in ("phi", "tphi", "ptilde"))
        # radial overlaps inside rcut + rpad_r (read_p_phi, read_paw.f90:517-532)
        nri = upper_count(r, self.rcut + RPAD_R)
        w = (r * r * dr)[:nri]
        mat_sp = (pt[:, :nri] * w) @ pt[:, :nri].T
        mat_t = (phi[:, :nri] * w) @ phi[:, :nri].T - (tphi[:, :nri] * w) @ tphi[:, :nri].T
        # per-l orthogonalisation (transform_pphi.f90)
        pt1, phi1, tphi1 = pt.copy(), phi.copy(), tphi.copy()
        for lv in sorted(set(lst.tolist())):
            idx = np.nonzero(lst == lv)[0]
            e, V = np.linalg.eigh(mat_sp[np.ix_(idx, idx)])
            sq = np.sign(e) * np.sqrt(np.abs(e))
            m1 = (V / sq) @ V.T
            m2 = (V * sq) @ V.T
            pt1[idx] = m1 @ pt[idx]
            phi1[idx] = m2.T @ phi[idx]
            tphi1[idx] = m2.T @ tphi[idx]
            e, V = np.linalg.eigh(m2.T @ mat_t[np.ix_(idx, idx)] @ m2)
            pt1[idx] = V.T @ pt1[idx]
            phi1[idx] = V.T @ phi1[idx]
            tphi1[idx] = V.T @ tphi1[idx]
        self.phi, self.tphi, self.pt = phi, tphi, pt
        self.phi1, self.tphi1, self.pt1 = phi1, tphi1, pt1
        # channels (state, m) (get_nm, read_paw.f90:449-475)
        chan = []
        for i, lv in enumerate(lst):
            chan += [(i, lv, m) for m in range(-lv, lv + 1)]
        self.chan = chan
        self.ms = len(chan)
        self.nl = len(set(lst.tolist()))
        self.nL = 2 * self.nl - 1
        self.nlm = self.nL ** 2
        G, waves = real_gaunt(1)
        widx = {wv: k for k, wv in enumerate(waves)}
        self.gaunt = np.zeros((self.nlm, self.ms, self.ms))
        for a in range(self.nlm):
            for p, (_, li, mi) in enumerate(chan):
                for q, (_, lj, mj) in enumerate(chan):
                    self.gaunt[a, p, q] = G[a, widx[(li, mi)], widx[(lj, mj)]]
        self._shape_functions()
        self._moments()

    def _shape_functions(self):
        """get_gl (read_paw.f90:112-182): the `sinc` form (sin(x)/x)^2 r^l,
        x = pi r / rc, and the `bessel` form a_1 j_l(q_1 r) + a_2 j_l(q_2 r)
        (libpaw atompaw_shapebes, 2_m_paw_atom.F90:211-256: q_i rc the first
        two zeros of j_l, a_i from a zero derivative at rc and unit
        moment), each then normalised to sum r^(l+2) g_l dr = 1."""
        d, r, dr = self.d, self.r, self.dr
        kind = d["shape_type"]
        if kind not in ("sinc", "bessel"):
            raise ValueError(f"{self.symbol}: shape function {kind!r} not supported (sinc, bessel)")
        nc = upper_count(r, self.rcomp)
        self.nrcomp = nc
        gl = np.zeros((self.nL, r.size))
        rc = self.rcomp
        for L in range(self.nL):
            if kind == "sinc":
                arg = math.pi * r[1:nc] / rc
                gl[L, 0] = 1.0 if L == 0 else 0.0
                gl[L, 1:nc] = (np.sin(arg) / arg) ** 2 * r[1:nc] ** L
            else:
                a, q = _bessel_shape(L, rc)
                gl[L, :nc] = a[0] * _sph_jn(L, q[0] * r[:nc]) + a[1] * _sph_jn(L, q[1] * r[:nc])
            gl[L] /= np.sum(r[:nc] ** (L + 2) * dr[:nc] * gl[L, :nc])
        self.gl = gl

    def _radial_moment(self, a, b, ta, tb, L):
        f = (a * b - ta * tb) * self.r ** (L + 2) * self.dr
        f[0] = 0.0
        return float(np.sum(f))

    def _moments(self):
        """calc_qijlm (read_paw.f90:695-782): the overlap s_ij from the
        orthogonalised waves (L = 0) and Q_ij^LM from the dataset's waves."""
        ms = self.ms
        sij = np.zeros((ms, ms))
        for p, (i, _, _) in enumerate(self.chan):
            for q, (j, _, _) in enumerate(self.chan):
                n0 = self._radial_moment(self.phi1[i], self.phi1[j], self.tphi1[i], self.tphi1[j], 0)
                sij[p, q] = n0 * self.gaunt[0, p, q] * SQ4PI
        off = sij - np.diag(np.diag(sij))
        if np.abs(off).max() > 1e-6 * SQ4PI:
            raise ValueError(f"{self.symbol}: the orthogonalised overlap s_ij is not diagonal")
        np.fill_diagonal(sij, np.maximum(np.diag(sij), -1.0 + TOLL_SIJ))
        self.sij = sij
        self.qL = np.zeros((self.nL, ms, ms))  # radial moments n_ij^L
        Q = np.zeros((self.nlm, ms, ms))
        for a in range(self.nlm):
            L = int(math.isqrt(a))
            for p, (i, _, _) in enumerate(self.chan):
                for q, (j, _, _) in enumerate(self.chan):
                    n = self._radial_moment(self.phi[i], self.phi[j], self.tphi[i], self.tphi[j], L)
                    self.qL[L, p, q] = n
                    Q[a, p, q] = n * self.gaunt[a, p, q]
        self.qijlm = Q

    def box(self, h):
        """nrough per axis for spacings h (get_nrcut, read_paw.f90:247-250)."""
        nrough = [2 * (math.ceil((self.rcut + RPAD) / hk) + 1) for hk in h]
        return nrough

    def dij0(self):
        """atompaw_dij0 (libpaw 2_m_paw_atom.F90:362-518): K_ij +
        <phi_i|v_H(n_Zc)|phi_j> - <phi~_i|v_H(n~_Zc)|phi~_j> - q_ij int
        v_H(n~_Zc) g_0 r^2 dr for channels of equal (l, m); v_H(n_Zc) = -Z/r
        + v_H[n_c], v_H(n~_Zc) the Bloechl local ionic potential, q_ij the
        L = 0 moment of phi_i phi_j - phi~_i phi~_j and g_0 the shape
        function normalised to int g_0 r^2 dr = 1 (the interaction of the
        compensation charge with v_H(n~_Zc), :475-518)."""
        r, dr, d = self.r, self.dr, self.d
        nc = np.asarray(d["ae_core"]) / SQ4PI
        vzc = -self.Z / r + hartree_radial(nc, r, dr, 0)
        vtzc = np.asarray(d["vloc_blochl"]) / SQ4PI
        nc_ = self.nrcomp
        intvh = cumint(vtzc[:nc_] * self.gl[0, :nc_] * r[:nc_] ** 2, dr[:nc_])[-1]
        ns = self.lstate.size
        M = np.zeros((ns, ns))
        for i in range(ns):
            for j in range(ns):
                f = (self.phi[i] * self.phi[j] * vzc - self.tphi[i] * self.tphi[j] * vtzc) * r * r
                q = cumint((self.phi[i] * self.phi[j] - self.tphi[i] * self.tphi[j]) * r * r, dr)[-1]
                M[i, j] = cumint(f, dr)[-1] - intvh * q
        K = np.asarray(d["kij"])
        D = np.zeros((self.ms, self.ms))
        for p, (i, li, mi) in enumerate(self.chan):
            for q, (j, lj, mj) in enumerate(self.chan):
                if li == lj and mi == mj:
                    D[p, q] = K[i, j] + M[i, j]
        return 0.5 * (D + D.T)

    def eijkl(self):
        """E_ijkl = sum_LM G^LM_ij G^LM_kl [ (n_ij|n_kl)_L - (n~_ij + q_ij^L g_L |
        n~_kl + q_kl^L g_L)_L ] on the augmentation sphere, (a|b)_L the radial
        Coulomb integral of the L components (pawinit, libpaw
        m_paw_init.F90:509-600).  Returned as [i, j, k, l]."""
        r, dr = self.r, self.dr
        npt = upper_count(r, self.rcut)
        rs, drs = r[:npt], dr[:npt]
        ms = self.ms
        pairs = [(p, q) for p in range(ms) for q in range(ms)]
        E = np.zeros((ms, ms, ms, ms))
        for L in range(self.nL):
            gL = self.gl[L, :npt]
            dens_ae, dens_ps = {}, {}
            for (p, q) in pairs:
                i, j = self.chan[p][0], self.chan[q][0]
                if not np.any(self.gaunt[L * L:(L + 1) ** 2, p, q]):
                    continue
                dens_ae[p, q] = self.phi[i, :npt] * self.phi[j, :npt]
                dens_ps[p, q] = self.tphi[i, :npt] * self.tphi[j, :npt] + self.qL[L, p, q] * gL
            keys = list(dens_ae)
            if not keys:
                continue
            # the Coulomb matrix of the pair densities for this L
            pot_ae = {k: hartree_radial(dens_ae[k], rs, drs, L) for k in keys}
            pot_ps = {k: hartree_radial(dens_ps[k], rs, drs, L) for k in keys}
            C = np.zeros((len(keys), len(keys)))
            w = rs * rs
            for a, ka in enumerate(keys):
                for b, kb in enumerate(keys):
                    C[a, b] = cumint((dens_ae[kb] * pot_ae[ka] - dens_ps[kb] * pot_ps[ka]) * w, drs)[-1]
            C = 0.5 * (C + C.T)
            GL = np.array([self.gaunt[L * L:(L + 1) ** 2, p, q] for (p, q) in keys])  # [npair, 2L+1]
            for a, (p, q) in enumerate(keys):
                for b, (s, t) in enumerate(keys):
                    E[p, q, s, t] += C[a, b] * float(GL[a] @ GL[b])
        return E

    def radial_tables(self):
        """On-site XC inputs on the dataset's mesh inside the sphere: u = r R
        for the all-electron and pseudo partial waves, the core densities, and
        weights of the integral of f dr (Simpson in the mesh index x dr/di)."""
        r, dr, d = self.r, self.dr, self.d
        n = upper_count(r, self.rcut)
        if n % 2 == 0:
            n += 1
        w = np.ones(n)
        w[1:-1:2] = 4.0
        w[2:-1:2] = 2.0
        w *= dr[:n] / 3.0
        return dict(r=r[:n], w=w, phi=self.phi[:, :n] * r[:n], tphi=self.tphi[:, :n] * r[:n],
                    core=np.asarray(d["ae_core"][:n]) / SQ4PI, tcore=np.asarray(d["ps_core"][:n]) / SQ4PI,
                    lmn=[(l, m, i) for (i, l, m) in self.chan])


# ---------------------------------------------------------------- system

R_GAUSS = 1.2  # width of the smooth long-range part of v_loc (Bohr)


def _simpson_weights(dr):
    n = dr.size
    w = np.ones(n)
    w[1:-1:2] = 4.0
    w[2:-1:2] = 2.0
    if n % 2 == 0:  # trapezoid on the last interval
        w[-1] = 1.5
        w[-2] = 2.5 if n > 2 else 1.5
    return w * dr / 3.0


def form_factor(f, r, dr, G):
    """4 pi int f(r) j0(G r) r^2 dr on the radial mesh, for an array of |G|."""
    w = _simpson_weights(dr) * f * r * r * 4.0 * math.pi
    G = np.asarray(G, dtype=np.float64)
    out = np.empty(G.size)
    for a in range(0, G.size, 256):
        x = np.outer(G[a:a + 256], r)
        j0 = np.where(x > 1e-12, np.sin(x) / np.where(x > 1e-12, x, 1.0), 1.0)
        out[a:a + 256] = j0 @ w
    return out


def _bandlimited(n, h, terms):
    """Sum over atoms of radial functions, band-limited to the grid: terms is a
    list of (form factor on the grid's |G| [nz, ny, nx], coordinates of the
    atoms that carry it).  Grid points x_i = -L/2 + i h (main.f90:353)."""
    nx, ny, nz = n
    dx, dy, dz = h
    kx = 2 * np.pi * np.fft.fftfreq(nx, dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, dy)
    kz = 2 * np.pi * np.fft.fftfreq(nz, dz)
    x0 = -np.array([nx * dx, ny * dy, nz * dz]) / 2.0
    acc = np.zeros((nz, ny, nx), np.complex128)
    for F, R in terms:
        S = np.zeros((nz, ny, nx), np.complex128)
        for c in R:
            d = x0 - c
            S += (np.exp(1j * kz * d[2])[:, None, None] * np.exp(1j * ky * d[1])[None, :, None]
                  * np.exp(1j * kx * d[0])[None, None, :])
        acc += F * S
    vol = nx * ny * nz * dx * dy * dz
    return (np.fft.ifftn(acc) * (nx * ny * nz / vol)).real


def _gnorm(n, h):
    nx, ny, nz = n
    dx, dy, dz = h
    kx = 2 * np.pi * np.fft.fftfreq(nx, dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, dy)
    kz = 2 * np.pi * np.fft.fftfreq(nz, dz)
    return np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)


def _radial_form_factor_on_grid(f, r, dr, Gn):
    """Form factor of f on every |G| of the grid (through its distinct values)."""
    u, inv = np.unique(np.round(Gn.ravel(), 12), return_inverse=True)
    return form_factor(f, r, dr, u)[inv].reshape(Gn.shape)

def _erf_over_r(r, rg):
    """erf(r / rg) / r, finite at r -> 0."""
    from scipy.special import erf

    r = np.asarray(r, dtype=np.float64)
    small = r < 1e-6 * rg
    rs = np.where(small, 1.0, r)
    return np.where(small, 2.0 / (math.sqrt(math.pi) * rg), erf(rs / rg) / rs)


def _spline_transfer(n_rough, n_fine, h):
    """get_b (read_paw.f90:274-345): b[i, j] = s_i(x_j) dxf / h with s_i the
    natural cubic spline through the unit vector e_i on the box points and
    x_j the fine points spanning the same interval."""
    xx = np.arange(n_rough) * h
    dxf = h * (n_rough - 1) / (n_fine - 1)
    xf = np.arange(n_fine) * dxf
    S = CubicSpline(xx, np.eye(n_rough), bc_type="natural", axis=0)(xf)  # [fine, rough]
    return S.T * (dxf / h), dxf


def _minimage(u, half):
    """minbyabs of p3d.f90:225-241 / g3d.f90: the image of u, u + 2 half,
    u - 2 half with the smallest magnitude (first wins ties)."""
    a, b, c = u, u + 2 * half, u - 2 * half
    out = a.copy()
    out = np.where(np.abs(b) < np.abs(out), b, out)
    out = np.where(np.abs(c) < np.abs(out), c, out)
    return out


def build(datasets, symbols, coords, n, h, ekcut=None, nfovnr=None, finegrid=0.15, periodic=0):
    """Operator tables for atoms `symbols` at `coords` (Bohr) on the grid n =
    (nx, ny, nz) with spacings h = (dx, dy, dz).  `datasets` maps element
    symbols to `pawxml.read_dataset` dicts.  ekcut None takes the
    reference's default cap; nfovnr None follows main.f90:342-344
    (ceil(h / finegrid)).  Returns a synthetic.System with the initial
    potential (v_loc plus the Hartree potential of the atoms' pseudo valence
    densities) in `vks0` and D0 in `dij_init`."""
    nx, ny, nz = n
    dx, dy, dz = (float(v) for v in h)
    coords = np.asarray(coords, dtype=np.float64)
    natom = len(symbols)
    if periodic:
        # the long-range -Z_val erf(r / r_g) / r part of v_loc is summed
        # without images; a periodic box needs its lattice sum
        raise ValueError("the set-up chain builds isolated systems (periodic F)")
    if nfovnr is None:
        nfovnr = max(1, max(math.ceil(hk / finegrid) for hk in (dx, dy, dz)))
    if ekcut is None:
        ekcut = synthetic.reference_ekcut((nx, ny, nz), (dx, dy, dz))
    half = np.array([nx * dx, ny * dy, nz * dz]) / 2.0
    species = {s: Species(datasets[s]) for s in sorted(set(symbols))}
    for s, sp in species.items():
        if np.any(sp.rcut > half):
            raise ValueError(f"{s}: rcut larger than half the box (get_rcut, read_paw.f90:213-226)")
    transfer = {}
    for s, sp in species.items():
        nr = sp.box((dx, dy, dz))
        transfer[s] = [(nr[k],) + _spline_transfer(nr[k], nr[k] * nfovnr, hk)
                       for k, hk in enumerate((dx, dy, dz))]

    dv = dx * dy * dz
    ir_start = np.zeros((natom, 3), np.int32)
    nrough = np.zeros((natom, 3), np.int32)
    ms = np.zeros(natom, np.int32)
    p3d, p3d1, s_all, sinv_all = [], [], [], []
    for a in range(natom):
        sp = species[symbols[a]]
        tr = transfer[symbols[a]]
        ms[a] = sp.ms
        for k in range(3):
            nrk = tr[k][0]
            nrough[a, k] = nrk
            ir_start[a, k] = math.ceil((coords[a, k] + half[k]) / (dx, dy, dz)[k]) - nrk // 2 + 1
            if not periodic and (ir_start[a, k] < 1 or ir_start[a, k] + nrk - 1 > n[k]):
                raise ValueError(f"atom {a}: its box leaves the grid (get_irs.f90:27-36)")
        # fine-grid points of the box (get_xyz, p3d.f90:171-185), x fastest
        fc = []
        for k, hk in enumerate((dx, dy, dz)):
            nrk, B, dxf = tr[k]
            x = -half[k] + (ir_start[a, k] - 1) * hk + np.arange(nrk * nfovnr) * dxf
            fc.append(_minimage(x - coords[a, k], half[k]))
        Zc, Yc, Xc = np.meshgrid(fc[2], fc[1], fc[0], indexing="ij")
        R = np.maximum(np.sqrt(Xc * Xc + Yc * Yc + Zc * Zc), 1e-8)
        ux, uy, uz = Xc / R, Yc / R, Zc / R
        i0, w1, w2 = bracket(sp.r, R)
        P, P1 = [], []
        for (i, l, m) in sp.chan:
            yl = ylm(l, m, ux, uy, uz)
            f = (sp.pt[i][i0] * w1 + sp.pt[i][i0 + 1] * w2) * yl
            f1 = (sp.pt1[i][i0] * w1 + sp.pt1[i][i0 + 1] * w2) * yl
            # get_p3d_r (p3d.f90:79-118): contract fine -> box along x, y, z
            Bx, By, Bz = tr[0][1], tr[1][1], tr[2][1]
            P.append(np.einsum("ia,jb,kc,cba->kji", Bx, By, Bz, f, optimize=True).reshape(-1))
            P1.append(np.einsum("ia,jb,kc,cba->kji", Bx, By, Bz, f1, optimize=True).reshape(-1))
        P, P1 = np.stack(P), np.stack(P1)
        # transform_p3d.f90: grid orthonormalisation and the overlap spectrum
        e, V = np.linalg.eigh((P1 @ P1.T) * dv)
        sq = np.sign(e) * np.sqrt(np.abs(e))
        m1 = (V / sq) @ V.T
        m2 = (V * sq) @ V.T
        P1 = m1 @ P1
        e, V = np.linalg.eigh(m2.T @ sp.sij @ m2)
        P1 = V.T @ P1
        p3d.append(P.reshape(-1))
        p3d1.append(P1.reshape(-1))
        s_all.append(e)
        sinv_all.append(1.0 / (1.0 + e) - 1.0)

    # sphere points and shape functions (map_localgrid.f90, g3d.f90)
    xs = -half[0] + np.arange(nx) * dx
    ys = -half[1] + np.arange(ny) * dy
    zs = -half[2] + np.arange(nz) * dz
    local_grid, g3d, ngrid, qij = [], [], [], []
    vloc = np.zeros((nz, ny, nx))
    vh_atoms = np.zeros((nz, ny, nx))
    for a in range(natom):
        sp = species[symbols[a]]
        X = _minimage(xs - coords[a, 0], half[0])
        Y = _minimage(ys - coords[a, 1], half[1])
        Zz = _minimage(zs - coords[a, 2], half[2])
        R = np.sqrt(Zz[:, None, None] ** 2 + Y[None, :, None] ** 2 + X[None, None, :] ** 2)
        iz, iy, ix = np.nonzero(R < sp.rcut)  # C order == the reference's z, y, x loops
        r = np.maximum(R[iz, iy, ix], 1e-8)
        ux, uy, uz = X[ix] / r, Y[iy] / r, Zz[iz] / r
        i0, w1, w2 = bracket(sp.r, r)
        G = np.zeros((sp.nlm, r.size))
        inside = r <= sp.rcomp
        for lm in range(sp.nlm):
            L = int(math.isqrt(lm))
            M = lm - L * L - L
            rad = np.where(inside, sp.gl[L][i0] * w1 + sp.gl[L][i0 + 1] * w2, 0.0)
            G[lm] = rad * ylm(L, M, ux, uy, uz)
        local_grid.append(np.stack([ix + 1, iy + 1, iz + 1], axis=1).astype(np.int32))
        g3d.append(G.reshape(-1))
        ngrid.append(r.size)
        # Fortran qijlm(lm, i, j) with lm fastest == C [j][i][lm]
        qij.append(np.ascontiguousarray(sp.qijlm.transpose(2, 1, 0)).reshape(-1))
        # the long-range part of v_loc and the initial Hartree potential in
        # real space (direct distances: an isolated system)
        Rd = np.sqrt((zs[:, None, None] - coords[a, 2]) ** 2 + (ys[None, :, None] - coords[a, 1]) ** 2
                     + (xs[None, None, :] - coords[a, 0]) ** 2)
        Rd = np.maximum(Rd, 1e-8)
        vloc += -sp.zval * _erf_over_r(Rd, R_GAUSS)
        nval = np.asarray(sp.d["ps_valence"]) / SQ4PI
        vh = hartree_radial(nval, sp.r, sp.dr, 0)
        qv = 4.0 * math.pi * cumint(nval * sp.r * sp.r, sp.dr)[-1]
        i0, w1, w2 = bracket(sp.r, Rd.ravel())
        v = vh[i0] * w1 + vh[i0 + 1] * w2
        far = Rd.ravel() >= sp.r[-1]
        v[far] = qv / Rd.ravel()[far]
        vh_atoms += v.reshape(Rd.shape)

    # band-limited short-range v_loc and pseudo core density
    Gn = _gnorm((nx, ny, nz), (dx, dy, dz))
    tv, tc = [], []
    for s_, sp in species.items():
        R = coords[[a for a in range(natom) if symbols[a] == s_]]
        r, dr = sp.r, sp.dr
        vshort = np.asarray(sp.d["vloc_blochl"]) / SQ4PI + sp.zval * _erf_over_r(r, R_GAUSS)
        tv.append((_radial_form_factor_on_grid(vshort, r, dr, Gn), R))
        tc.append((_radial_form_factor_on_grid(np.asarray(sp.d["ps_core"]) / SQ4PI, r, dr, Gn), R))
    vloc += _bandlimited((nx, ny, nz), (dx, dy, dz), tv)
    ncoret = _bandlimited((nx, ny, nz), (dx, dy, dz), tc)

    dij0, eij, rad = [], [], {}
    cache = {}
    for s, sp in species.items():
        cache[s] = (sp.dij0(), sp.eijkl(), sp.radial_tables())
    for a in range(natom):
        D, E, _ = cache[symbols[a]]
        dij0.append(D.reshape(-1, order="F"))
        # Fortran order (i fastest): element (i,j,k,l) at i + m*(j + m*(k + m*l))
        eij.append(E.transpose(3, 2, 1, 0).reshape(-1))
    rad_n, rad_r, rad_w, nphi, phi, tphi, core, tcore, lmn = [], [], [], [], [], [], [], [], []
    for a in range(natom):
        t = cache[symbols[a]][2]
        rad_n.append(t["r"].size)
        rad_r.append(t["r"])
        rad_w.append(t["w"])
        nphi.append(t["phi"].shape[0])
        phi.append(t["phi"].reshape(-1))
        tphi.append(t["tphi"].reshape(-1))
        core.append(t["core"])
        tcore.append(t["tcore"])
        lmn.extend(t["lmn"])
    radial = {"rad_n": np.array(rad_n, np.int32), "rad_r": np.concatenate(rad_r), "rad_w": np.concatenate(rad_w),
              "nphi": np.array(nphi, np.int32), "phi": np.concatenate(phi), "tphi": np.concatenate(tphi),
              "coredens": np.concatenate(core), "tcoredens": np.concatenate(tcore),
              "proj_lmn": np.array(lmn, np.int32).reshape(-1)}
    nel = sum(species[s].zval for s in symbols)
    vks0 = (vloc + vh_atoms).reshape(-1)
    sysobj = synthetic.System(
        nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, ekcut=float(ekcut),
        scale_vh=1 if periodic else 2, periodic=int(periodic), rnel=float(nel), natom=natom,
        ir_start=ir_start, nrough=nrough, ms=ms,
        p3d=np.concatenate(p3d), p3d1=np.concatenate(p3d1),
        s=np.concatenate(s_all), sinv=np.concatenate(sinv_all),
        ngrid=np.array(ngrid, np.int32), local_grid=np.concatenate(local_grid),
        nlm=np.array([species[s].nlm for s in symbols], np.int32),
        g3d=np.concatenate(g3d), qijlm=np.concatenate(qij),
        vloc=vloc.reshape(-1).copy(), ncoret=ncoret.reshape(-1).copy(),
        dij0=np.concatenate(dij0), eijkl=np.concatenate(eij),
        vks0=vks0, dij_init=np.concatenate(dij0), coords=coords, radial=radial,
    )
    sysobj.extra["species"] = species
    sysobj.extra["symbols"] = list(symbols)
    return sysobj


def from_bundle(path, **kw):
    """The system of a bundle written by `pawxml.save_bundle` (datasets,
    geometry and `dim_paw.inp` parameters: nx, ny, nz, box_x, box_y, box_z,
    periodic, finegrid, ekcut)."""
    from . import pawxml

    return from_parts(*pawxml.load_bundle(path), **kw)


def from_folder(folder, **kw):
    """The system of one of the reference's input folders (`pawfiles`, the
    datasets it names, `cnt.ini`, `dim_paw.inp`)."""
    from . import pawxml

    return from_parts(*pawxml.read_folder(folder), **kw)


def from_parts(datasets, symbols, coords, params, **kw):
    """`build` with the grid, box, boundary, fine-grid and kinetic-cap
    settings of `dim_paw.inp` (main.f90:326-344)."""
    from . import pawxml

    n = tuple(int(params[k]) for k in ("nx", "ny", "nz"))
    box = [pawxml.fortran_float(params[k]) for k in ("box_x", "box_y", "box_z")]
    h = tuple(b / nk for b, nk in zip(box, n))  # main.f90:326-328
    periodic = 1 if params.get("periodic", "F").upper().startswith("T") else 0
    finegrid = pawxml.fortran_float(params.get("finegrid", "0.15"))
    ek = pawxml.fortran_float(params.get("ekcut", "-1"))
    kw.setdefault("ekcut", ek if ek > 0 else None)
    return build(datasets, symbols, coords, n, h, finegrid=finegrid, periodic=periodic, **kw)
