"""Seeded synthetic OPAW systems with the shapes of the reference's workloads.

The reference has no benchmark inputs or golden outputs; its naphthalene
example needs the JTH PAW datasets and a set-up chain (p3d.f90,
transform_p3d.f90, g3d.f90, libpaw) that is not part of the propagation path.
These generators build every operator table of that path directly, with the
reference's layouts and conventions:

* grid coordinates x_i = -xmax + i*dx with xmax = nx*dx/2 (main.f90:353,
  map_localgrid.f90:100, 0-based here);
* projector boxes of side nrough = 2*(ceil((rc + rpad)/h) + 1), rpad = 1
  (read_paw.f90:250-253, 0_parameter.f90:14), placed at
  ir_start = ceil((x_a + xmax)/dx) - nrough/2 + 1 (get_irs.f90:22-26);
* raw projectors p~ (Gaussian radial x real Y_lm, the ylm.f90 order
  m = -1 -> y, 0 -> z, 1 -> x) and per-atom orthonormalised projectors p1 with
  an overlap spectrum s_i (transform_p3d.f90:53-55);
* compensation-sphere points, shape functions g_LM and Q_ij^LM
  (map_localgrid.f90, g3d.f90, read_paw.f90:695-782);
* D_ij = Q diag(lambda) Q^T with Haar Q and lambda ~ U[-1, 1] Ha.

`hamiltonian_microbench()` is the 96^3 / 128-orbital / 40-atom workload of the
Hamiltonian-apply microbenchmark; `small_system()` are test-sized cases.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SQ3_4PI = math.sqrt(3.0 / (4.0 * math.pi))
Y00 = 1.0 / math.sqrt(4.0 * math.pi)


@dataclass
class System:
    """Host-side operator tables; field names follow `opaw_system` in include/opaw_gb300.h."""

    nx: int
    ny: int
    nz: int
    dx: float
    dy: float
    dz: float
    ekcut: float
    scale_vh: int
    periodic: int
    rnel: float
    natom: int
    ir_start: np.ndarray  # int32 [natom,3], 1-based
    nrough: np.ndarray  # int32 [natom,3]
    ms: np.ndarray  # int32 [natom]
    p3d: np.ndarray  # float64 concatenated per atom [ms][nbox]
    p3d1: np.ndarray
    s: np.ndarray  # float64 [sum ms]
    sinv: np.ndarray
    ngrid: np.ndarray  # int32 [natom]
    local_grid: np.ndarray  # int32 [sum ngrid, 3], 1-based
    nlm: np.ndarray  # int32 [natom]
    g3d: np.ndarray  # float64 per atom [nlm][ngrid]
    qijlm: np.ndarray  # float64 per atom [ms][ms][nlm] (lm fastest)
    vloc: np.ndarray  # float64 [nn]
    ncoret: np.ndarray  # float64 [nn]
    dij0: np.ndarray  # float64 per atom [ms*ms] column-major
    eijkl: np.ndarray  # float64 per atom [ms^4]
    dij_max: float = 500.0
    # not part of opaw_system: initial state for the operators and orbitals
    vks0: np.ndarray | None = None  # [nn] v_ks used by the H-apply microbench
    dij_init: np.ndarray | None = None  # [sum ms^2]
    coords: np.ndarray | None = None  # [natom,3] Bohr
    extra: dict = field(default_factory=dict)
    # radial tables of the on-site XC term (keys of the rad_* / phi / core
    # fields of opaw_system); None leaves D_xc out
    radial: dict | None = None

    @property
    def nn(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def dv(self) -> float:
        return self.dx * self.dy * self.dz

    @property
    def shape_f(self):
        """numpy shape of one orbital in C order (z, y, x) == Fortran (nx, ny, nz)."""
        return (self.nz, self.ny, self.nx)

    def nbox(self, a: int) -> int:
        return int(np.prod(self.nrough[a]))

    def proj_offsets(self):
        off = [0]
        for a in range(self.natom):
            off.append(off[-1] + int(self.ms[a]) * self.nbox(a))
        return off

    def ms_offsets(self):
        return np.concatenate([[0], np.cumsum(self.ms)]).astype(np.int64)

    def mat_offsets(self):
        return np.concatenate([[0], np.cumsum(self.ms.astype(np.int64) ** 2)]).astype(np.int64)


def _coords(n, d):
    xmax = n * d / 2.0
    return -xmax + np.arange(n) * d


def _ylm_p(x, y, z):
    """real l=1 harmonics times r, ylm.f90 order: m=-1 -> y, 0 -> z, 1 -> x."""
    return [SQ3_4PI * y, SQ3_4PI * z, SQ3_4PI * x]


def _ylm_l2_over_r2(x, y, z):
    c1 = 0.5 * math.sqrt(15.0 / math.pi)
    c0 = 0.25 * math.sqrt(5.0 / math.pi)
    c2 = 0.25 * math.sqrt(15.0 / math.pi)
    return [c1 * x * y, c1 * y * z, c0 * (3 * z * z - (x * x + y * y + z * z)), c1 * x * z, c2 * (x * x - y * y)]


def _haar(rng, m):
    q, r = np.linalg.qr(rng.standard_normal((m, m)))
    return q * np.sign(np.diag(r))


def _place_atoms(rng, natom, lo, hi, dmin, max_tries=200000):
    pts = []
    tries = 0
    while len(pts) < natom:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place atoms with the requested spacing")
        c = lo + (hi - lo) * rng.random(3)
        if all(np.linalg.norm(c - p) >= dmin for p in pts):
            pts.append(c)
    return np.array(pts)


def reference_ekcut(n, h, ek_factor=1.0):
    """The kinetic cap ekcut that the reference derives when none is read
    (prepare_libpaw.f90:189-194): getcut.f90:39-41 takes ecut =
    0.5 (2 pi)^2 boxsq (ek_factor - 1e-10), boxsq the smallest reduced |G|^2
    on the faces of the FFT box (bound.f90: indices +-(n_k/2) in integer
    division, metric 1/L_k^2 for an orthorhombic cell at the Gamma point,
    so the minimum sits at a face centre).  ek.f90:42-44 then clips every
    k^2/2 above it, which bounds the spectrum the RK4 step sees."""
    boxsq = min(((nk // 2) / (nk * hk)) ** 2 for nk, hk in zip(n, h))
    return 0.5 * (2.0 * np.pi) ** 2 * boxsq * (ek_factor - 1e-10)


def build_system(
    n=(24, 20, 16),
    h=0.5,
    natom=4,
    seed=7,
    rc=0.8,
    rpad=1.0,
    alphas=(0.5, 0.8),
    ekcut=None,
    periodic=0,
    scale_vh=None,
    norb=4,
    ngauss=None,
    face_margin=None,
    atom_min_dist=2.0,
    coords=None,
    comp_rc=None,
    comp_sigma=0.45,
    species=None,
    onsite_xc=True,
):
    """Builds a synthetic system; `n` is (nx, ny, nz) and h the spacing (all
    axes).  ekcut None takes the reference's default cap (`reference_ekcut`);
    0 leaves the kinetic energy uncapped.  `species` (one entry per atom of
    `coords`, keys of SPECIES) gives each atom its own cutoff and projector
    channels; without it every atom has cutoff rc with one s and three p
    channels per radial width in `alphas`.  onsite_xc adds the radial tables
    of the on-site XC term of D_ij (`radial_tables`)."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = n
    dx = dy = dz = float(h)
    if ekcut is None:
        ekcut = reference_ekcut((nx, ny, nz), (dx, dy, dz))
    xs, ys, zs = _coords(nx, dx), _coords(ny, dy), _coords(nz, dz)
    L = np.array([nx * dx, ny * dy, nz * dz])
    xmax = L / 2.0
    nr = 2 * (math.ceil((rc + rpad) / h) + 1)
    if face_margin is None:
        face_margin = (nr / 2 + 0.5) * h
    if coords is None:
        coords = _place_atoms(rng, natom, -xmax + face_margin, xmax - face_margin, atom_min_dist)
    coords = np.asarray(coords, dtype=np.float64)
    natom = len(coords)

    if species is None:
        kinds = [dict(rc=rc, s_alphas=tuple(alphas), p_alphas=tuple(alphas))] * natom
    else:
        kinds = [SPECIES[k] for k in species]
    # one s channel per s width, three p channels per p width
    ms_of = [len(k["s_alphas"]) + 3 * len(k["p_alphas"]) for k in kinds]
    nr_of = [2 * (math.ceil((k["rc"] + rpad) / h) + 1) for k in kinds]
    ir_start = np.zeros((natom, 3), np.int32)
    nrough = np.array([[v, v, v] for v in nr_of], np.int32).reshape(natom, 3)
    ms = np.array(ms_of, np.int32)
    dv = dx * dy * dz
    p3d, p3d1, s, sinv = [], [], [], []
    for a in range(natom):
        nr = nr_of[a]
        rc_a = kinds[a]["rc"]
        ms_atom = ms_of[a]
        for k in range(3):
            ir_start[a, k] = math.ceil((coords[a, k] + xmax[k]) / h) - nr // 2 + 1
        # box coordinates (box x fastest -> arrays indexed [bz, by, bx])
        i0 = ir_start[a] - 1
        bx = -xmax[0] + (i0[0] + np.arange(nr)) * dx
        by = -xmax[1] + (i0[1] + np.arange(nr)) * dy
        bz = -xmax[2] + (i0[2] + np.arange(nr)) * dz
        Z, Y, X = np.meshgrid(bz, by, bx, indexing="ij")
        X = X - coords[a, 0]
        Y = Y - coords[a, 1]
        Z = Z - coords[a, 2]
        if periodic:
            X = X - L[0] * np.round(X / L[0])
            Y = Y - L[1] * np.round(Y / L[1])
            Z = Z - L[2] * np.round(Z / L[2])
        R2 = X * X + Y * Y + Z * Z
        inside = (R2 < rc_a * rc_a).astype(np.float64)
        chans = []
        for al in kinds[a]["s_alphas"]:
            chans.append(Y00 * np.exp(-R2 / (2 * al * al)) * inside)
        for al in kinds[a]["p_alphas"]:
            g = np.exp(-R2 / (2 * al * al)) * inside
            for comp in _ylm_p(X, Y, Z):
                chans.append(comp * g)
        P = np.stack([c.reshape(-1) for c in chans])  # [ms, nbox]
        P = P / np.sqrt((P * P).sum(axis=1, keepdims=True) * dv)  # unit norm
        O = (P @ P.T) * dv
        w, V = np.linalg.eigh(O)
        Oih = (V * (1.0 / np.sqrt(w))) @ V.T
        P1 = Oih @ P
        sa = rng.uniform(-0.5, 1.0, ms_atom)
        p3d.append(P.reshape(-1))
        p3d1.append(P1.reshape(-1))
        s.append(sa)
        sinv.append(1.0 / (1.0 + sa) - 1.0)

    # compensation spheres, shape functions, Q_ij^LM
    nlm = 9
    Zg, Yg, Xg = np.meshgrid(zs, ys, xs, indexing="ij")
    local_grid, g3d_all, ngrid, qijlm_all = [], [], [], []
    for a in range(natom):
        X = Xg - coords[a, 0]
        Y = Yg - coords[a, 1]
        Z = Zg - coords[a, 2]
        if periodic:
            X = X - L[0] * np.round(X / L[0])
            Y = Y - L[1] * np.round(Y / L[1])
            Z = Z - L[2] * np.round(Z / L[2])
        R2 = X * X + Y * Y + Z * Z
        crc = kinds[a]["rc"] if comp_rc is None else comp_rc
        iz, iy, ix = np.nonzero(R2 < crc * crc)  # C order == reference's z,y,x loop order
        x, y, z = X[iz, iy, ix], Y[iz, iy, ix], Z[iz, iy, ix]
        r2 = x * x + y * y + z * z
        gauss = np.exp(-r2 / (2 * comp_sigma**2))
        norm0 = 1.0 / ((2 * math.pi) ** 1.5 * comp_sigma**3)
        g = [norm0 / Y00 * Y00 * gauss]
        g += [norm0 * c * gauss / comp_sigma for c in _ylm_p(x, y, z)]
        g += [norm0 * c * gauss / comp_sigma**2 for c in _ylm_l2_over_r2(x, y, z)]
        G = np.stack(g)  # [nlm, ngrid]
        g3d_all.append(G.reshape(-1))
        local_grid.append(np.stack([ix + 1, iy + 1, iz + 1], axis=1).astype(np.int32))
        ngrid.append(len(ix))
        m = ms_of[a]
        Q = np.zeros((m, m, nlm))  # [j][i][lm] in C order == Fortran (lm, i, j)
        for lm in range(nlm):
            A = rng.standard_normal((m, m)) * (0.05 if lm == 0 else 0.02)
            Q[:, :, lm] = A + A.T
        qijlm_all.append(Q.reshape(-1))

    nn = nx * ny * nz
    # v_ks: -sum_j d_j exp(-|r-R_j|^2 / (2 w_j^2)) over the atom centres (the
    # microbench's 40 attractive Gaussians sit on the 40 atoms)
    if ngauss is None:
        ngauss = natom
    vks = np.zeros((nz, ny, nx))
    depth = rng.uniform(1.0, 3.0, ngauss)
    width = rng.uniform(0.8, 1.5, ngauss)
    for j in range(ngauss):
        c = coords[j % natom]
        X = Xg - c[0]
        Y = Yg - c[1]
        Z = Zg - c[2]
        vks -= depth[j] * np.exp(-(X * X + Y * Y + Z * Z) / (2 * width[j] ** 2))
    ncoret = np.zeros((nz, ny, nx))
    for a in range(natom):
        X = Xg - coords[a, 0]
        Y = Yg - coords[a, 1]
        Z = Zg - coords[a, 2]
        ncoret += 0.05 * np.exp(-(X * X + Y * Y + Z * Z) / (2 * 0.4**2))

    dij0, eijkl, dinit = [], [], []
    for a in range(natom):
        m = ms_of[a]
        Qh = _haar(rng, m)
        lam = rng.uniform(-1.0, 1.0, m)
        D = (Qh * lam) @ Qh.T
        dinit.append(D.reshape(-1, order="F"))
        dij0.append(D.reshape(-1, order="F"))
        U = rng.standard_normal((3, m, m))
        U = U + U.transpose(0, 2, 1)
        E = 0.01 * np.einsum("pij,pkl->ijkl", U, U)  # E[i,j,k,l], symmetric
        # Fortran order (i fastest): element (i,j,k,l) at i + m*(j + m*(k + m*l))
        eijkl.append(E.transpose(3, 2, 1, 0).reshape(-1))

    radial = radial_tables(kinds, ms_of, seed + 17) if onsite_xc else None
    sysobj = System(
        nx=nx, ny=ny, nz=nz, dx=dx, dy=dy, dz=dz, ekcut=float(ekcut),
        scale_vh=int(scale_vh if scale_vh is not None else (1 if periodic else 2)),
        periodic=int(periodic), rnel=float(2 * norb), natom=natom,
        ir_start=ir_start, nrough=nrough, ms=ms,
        p3d=np.concatenate(p3d), p3d1=np.concatenate(p3d1),
        s=np.concatenate(s), sinv=np.concatenate(sinv),
        ngrid=np.array(ngrid, np.int32),
        local_grid=np.concatenate(local_grid) if local_grid else np.zeros((0, 3), np.int32),
        nlm=np.full(natom, nlm, np.int32),
        g3d=np.concatenate(g3d_all), qijlm=np.concatenate(qijlm_all),
        vloc=vks.reshape(-1).copy(), ncoret=ncoret.reshape(-1),
        dij0=np.concatenate(dij0), eijkl=np.concatenate(eijkl),
        vks0=vks.reshape(-1).copy(), dij_init=np.concatenate(dinit), coords=coords, radial=radial,
    )
    return sysobj


def radial_mesh(rc, n=241, b=5.0):
    """Log-type mesh of the PAW sphere, r_k = rc (e^{b (k+1)/n} - 1) / (e^b - 1),
    k = 0..n-1, and Simpson weights in k times dr/dk (n odd)."""
    k = np.arange(n, dtype=np.float64)
    e = np.exp(b * (k + 1) / n)
    r = rc * (e - 1.0) / (np.exp(b) - 1.0)
    drdk = rc * (b / n) * e / (np.exp(b) - 1.0)
    w = np.ones(n)
    w[1:-1:2] = 4.0
    w[2:-1:2] = 2.0
    w /= 3.0
    return r, w * drdk


def radial_tables(kinds, ms_of, seed):
    """Synthetic one-centre data of every atom with the layout of libpaw's
    pawtab / pawrad: a log mesh of the sphere (radius rc), partial waves per
    channel width (all-electron u(r) = r^(l+1) e^(-r^2/2a^2) (1 + 0.3
    e^(-r^2/2(0.3a)^2)), pseudo u~ without the inner bump, both scaled so
    that int u~^2 dr = 1), a 1s-like core of 2 electrons for carbon-like
    atoms (none for hydrogen-like ones, whose core is zero) and a smooth
    pseudo core, and per projector (l, m, partial-wave index) in the order
    of the projector channels (s channels, then p channels with m = -1, 0, 1
    for y, z, x)."""
    rad_n, rad_r, rad_w, nphi, phi, tphi, core, tcore, lmn = [], [], [], [], [], [], [], [], []
    for kd, m in zip(kinds, ms_of):
        r, w = radial_mesh(kd["rc"])
        waves = [(0, a) for a in kd["s_alphas"]] + [(1, a) for a in kd["p_alphas"]]
        for (l, a) in waves:
            tu = r ** (l + 1) * np.exp(-r * r / (2 * a * a))
            u = tu * (1.0 + 0.3 * np.exp(-r * r / (2 * (0.3 * a) ** 2)))
            nrm = np.sqrt(np.sum(w * tu * tu))
            phi.append(u / nrm)
            tphi.append(tu / nrm)
        ns_ = len(kd["s_alphas"])
        ch = [(0, 0, i) for i in range(ns_)]
        for j in range(len(kd["p_alphas"])):
            ch += [(1, mm, ns_ + j) for mm in (-1, 0, 1)]
        assert len(ch) == m
        lmn.extend(ch)
        rad_n.append(r.size)
        rad_r.append(r)
        rad_w.append(w)
        nphi.append(len(waves))
        nc = 2.0 if kd.get("valence", 4) >= 4 else 0.0
        beta = 20.0
        core.append(nc * (beta / np.pi) ** 1.5 * np.exp(-beta * r * r))
        tcore.append(0.05 * np.exp(-r * r / (2 * 0.4 ** 2)) * (1.0 if nc > 0 else 0.0))
    return {"rad_n": np.array(rad_n, np.int32), "rad_r": np.concatenate(rad_r), "rad_w": np.concatenate(rad_w),
            "nphi": np.array(nphi, np.int32), "phi": np.concatenate(phi), "tphi": np.concatenate(tphi),
            "coredens": np.concatenate(core), "tcoredens": np.concatenate(tcore),
            "proj_lmn": np.array(lmn, np.int32).reshape(-1)}


# Projector channels of the two elements of the polyacenes, with the counts
# and cutoffs of the JTH LDA datasets the reference ships (C: 2 s + 2x3 p
# partial waves, r_c = 1.507 Bohr; H: 2 s + 1x3 p, r_c = 0.995 Bohr) and
# Gaussian radial shapes standing in for the tabulated projectors.
SPECIES = {
    "C": dict(rc=1.507, s_alphas=(0.5, 0.8), p_alphas=(0.5, 0.8), valence=4),
    "H": dict(rc=0.995, s_alphas=(0.4, 0.6), p_alphas=(0.5,), valence=1),
}
ANGSTROM = 1.8897261  # Bohr


def polyacene_geometry(nring, cc=1.40, ch=1.09):
    """Planar linear polyacene C(4n+2)H(2n+4) along x in the z = 0 plane:
    regular hexagons of side cc (Angstrom) sharing their vertical edges, one
    H per carbon with two carbon neighbours, at ch along the ring radius.
    Returns (species list, coordinates in Bohr) centred on the origin."""
    a = cc
    sx = math.sqrt(3.0) * a  # ring-centre spacing
    cpos = []
    centres = [((i - (nring - 1) / 2.0) * sx, 0.0) for i in range(nring)]
    for cxr, cyr in centres:
        for k in range(6):
            th = math.radians(30.0 + 60.0 * k)
            p = (round(cxr + a * math.cos(th), 6), round(cyr + a * math.sin(th), 6))
            if p not in cpos:
                cpos.append(p)
    cpos.sort(key=lambda q: (q[0], q[1]))
    hpos = []
    for (x, y) in cpos:
        nb = sum(1 for (u, v) in cpos if 0.1 < math.hypot(u - x, v - y) < 1.1 * a)
        if nb == 2:  # outer carbon: H along the radius of its own ring
            cxr = min(centres, key=lambda c: math.hypot(c[0] - x, c[1] - y))
            d = (x - cxr[0], y - cxr[1])
            r = math.hypot(*d)
            hpos.append((x + ch * d[0] / r, y + ch * d[1] / r))
    species = ["C"] * len(cpos) + ["H"] * len(hpos)
    xyz = np.array([[x, y, 0.0] for (x, y) in cpos + hpos]) * ANGSTROM
    return species, xyz


def polyacene(nring, n, h, seed=None, **kw):
    """Synthetic OPAW system of the polyacene with `nring` rings on the grid
    n = (nx, ny, nz) at spacing h: the generated geometry, C and H projector
    channels (SPECIES), Gaussian wells of v_ks on every atom, and the
    valence electron count (4 per C, 1 per H; norb = electrons / 2)."""
    species, xyz = polyacene_geometry(nring)
    nel = sum(SPECIES[k]["valence"] for k in species)
    return build_system(n=n, h=h, coords=xyz, species=species, norb=nel // 2,
                        seed=1000 + nring if seed is None else seed, **kw)


# The molecules of the propagation benchmarks: rings, grid, spacing
MOLECULES = {
    "benzene": (1, (40, 40, 28), 0.5),
    "naphthalene": (2, (48, 48, 32), 0.5),
    "anthracene": (3, (64, 48, 32), 0.5),
    "tetracene": (4, (96, 64, 48), 0.45),
}


def molecule(name, **kw):
    """The named polyacene on its benchmark grid (MOLECULES)."""
    nring, n, h = MOLECULES[name]
    return polyacene(nring, n, h, **kw)


def orbitals(sysobj: System, norb: int, seed: int = 11, sigma: float = 1.5, chunk: int = 16):
    """norb orbitals: complex N(0,1) noise, Gaussian-filtered (exp(-k^2 sigma^2/2)
    in k-space), then orthonormalised with the dv inner product (Cholesky QR,
    twice: the same orthonormal basis modified Gram-Schmidt produces, with
    better rounding).  Returns complex128 [norb, nz, ny, nx]."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = sysobj.shape_f
    kx = 2 * np.pi * np.fft.fftfreq(nx, sysobj.dx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, sysobj.dy)
    kz = 2 * np.pi * np.fft.fftfreq(nz, sysobj.dz)
    K2 = kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2
    filt = np.exp(-K2 * sigma * sigma / 2.0)
    psi = np.empty((norb, nz, ny, nx), np.complex128)
    for b0 in range(0, norb, chunk):
        b1 = min(norb, b0 + chunk)
        z = rng.standard_normal((b1 - b0, nz, ny, nx)) + 1j * rng.standard_normal((b1 - b0, nz, ny, nx))
        psi[b0:b1] = np.fft.ifftn(np.fft.fftn(z, axes=(1, 2, 3)) * filt, axes=(1, 2, 3))
    flat = psi.reshape(norb, -1)
    dv = sysobj.dv
    for _ in range(2):
        # rows are orbitals: G = conj(Psi) Psi^T dv = L L^H, so conj(L)^-1 Psi
        # has the identity as its Gram matrix
        G = (flat.conj() @ flat.T) * dv
        Lc = np.linalg.cholesky(G)
        flat[:] = np.linalg.solve(Lc.conj(), flat)
    return psi


def hamiltonian_microbench(norb=128, seed=2024):
    """96^3 grid at h = 0.4 Bohr, 40 atoms x 8 projectors (2 s + 2x3 p,
    Gaussian radial x real Y_lm, cutoff 1.6 Bohr, 16^3 boxes), v_ks = 40
    attractive Gaussians (depth 1-3 Ha, width 0.8-1.5 Bohr), centres >= 2 Bohr
    apart and >= 3.2 Bohr from the faces."""
    return build_system(n=(96, 96, 96), h=0.4, natom=40, seed=seed, rc=1.6, norb=norb,
                        face_margin=3.2, atom_min_dist=2.0)


def small_system(kind="tiny", seed=7, norb=4):
    """Test-sized systems.  'tiny' 24x20x16; 'odd' exercises radices 3,5,7;
    'edge' is periodic with boxes that wrap around the faces; 'spec' uses
    extents with compile-time specialised FFT kernels (32, 48, 64 and the
    64, 96, 128 Hartree box).  All but 'odd' take the reference's kinetic
    cap; 'odd' leaves it off (ekcut 0) so both branches of the kinetic
    factor are exercised."""
    if kind == "tiny":
        return build_system(n=(24, 20, 16), h=0.5, natom=3, seed=seed, rc=0.8, norb=norb)
    if kind == "odd":
        return build_system(n=(30, 28, 20), h=0.5, natom=4, seed=seed, rc=0.8, norb=norb, ekcut=0.0)
    if kind == "edge":
        coords = np.array([[5.9, 0.3, -0.2], [-1.0, -4.8, 3.7], [0.5, 1.5, 0.1]])
        return build_system(n=(24, 20, 16), h=0.5, natom=3, seed=seed, rc=0.8, norb=norb,
                            periodic=1, coords=coords)
    if kind == "spec":
        return build_system(n=(32, 48, 64), h=0.5, natom=4, seed=seed, rc=0.8, norb=norb)
    if kind == "medium":
        return build_system(n=(48, 48, 32), h=0.5, natom=10, seed=seed, rc=1.0, norb=norb)
    raise ValueError(kind)
