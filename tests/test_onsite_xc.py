"""The on-site XC term of D_ij in the oracle (libpaw pawxcm with pawxcdev = 1
and pawdijxcm, LDA, nspden = 1): checked against an independent NumPy
restatement that forms the finite differences of v_xc in 40-digit arithmetic,
against the exact spherical case, against a full angular quadrature of
v_xc(n(r, Omega)) for a weakly non-spherical density (the moment development
is second-order accurate), and as a term of the oracle's D_ij."""
import dataclasses

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")

import oracle as orc
from opaw_tddft_gb300 import synthetic

SQ4PI = np.sqrt(4.0 * np.pi)


def vxc_mp(n):
    """The same potential at one point in 40-digit arithmetic (mpmath)."""
    mp = mpmath.mp
    n = mpmath.mpf(float(n))
    A, a1 = mpmath.mpf(0.031091), mpmath.mpf(0.21370)
    b1, b2, b3, b4 = (mpmath.mpf(v) for v in (7.5957, 3.5876, 1.6382, 0.49294))
    vx = -mpmath.cbrt(3 * n / mp.pi)
    rs = mpmath.cbrt(3 / (4 * mp.pi * n))
    s = mpmath.sqrt(rs)
    Q = 2 * A * (b1 * s + b2 * rs + b3 * rs * s + b4 * rs * rs)
    dQ = 2 * A * (b1 / (2 * s) + b2 + 3 * b3 * s / 2 + 2 * b4 * rs)
    lg = mpmath.log(1 + 1 / Q)
    ec = -2 * A * (1 + a1 * rs) * lg
    dec = -2 * A * a1 * lg + 2 * A * (1 + a1 * rs) * dQ / (Q * Q + Q)
    return vx + ec - rs / 3 * dec


def derivatives_mp(ns, h):
    """(v+ - v-) / 2h and (v+ + v- - 2 v0) / h^2 at the double steps ns +- h,
    formed in 40-digit arithmetic and rounded once."""
    d1, d2 = np.zeros_like(ns), np.zeros_like(ns)
    with mpmath.workdps(40):
        for k in range(ns.size):
            v0, vp, vm = vxc_mp(ns[k]), vxc_mp(ns[k] + h[k]), vxc_mp(ns[k] - h[k])
            hk = mpmath.mpf(float(h[k]))
            d1[k] = float((vp - vm) / (2 * hk))
            d2[k] = float((vp + vm - 2 * v0) / (hk * hk))
    return d1, d2


def vxc_ld(n):
    """Slater exchange + PW92 correlation (unpolarised) in long double."""
    n = np.asarray(n, np.longdouble)
    pi = np.longdouble(np.pi)
    A, a1 = np.longdouble(0.031091), np.longdouble(0.21370)
    b1, b2, b3, b4 = (np.longdouble(v) for v in (7.5957, 3.5876, 1.6382, 0.49294))
    vx = -np.cbrt(3 * n / pi)
    rs = np.cbrt(3 / (4 * pi * n))
    s = np.sqrt(rs)
    Q = 2 * A * (b1 * s + b2 * rs + b3 * rs * s + b4 * rs * rs)
    dQ = 2 * A * (b1 / (2 * s) + b2 + 3 * b3 * s / 2 + 2 * b4 * rs)
    lg = np.log1p(1 / Q)
    ec = -2 * A * (1 + a1 * rs) * lg
    dec = -2 * A * a1 * lg + 2 * A * (1 + a1 * rs) * dQ / (Q * Q + Q)
    return vx + ec - rs / 3 * dec


def ylm(x, y, z):
    """Real Y_lm, l <= 2, index l^2 + l + m (ylm.f90 order)."""
    c0, c1 = np.sqrt(1 / (4 * np.pi)), np.sqrt(3 / (4 * np.pi))
    c2, c20, c22 = np.sqrt(15 / (4 * np.pi)), np.sqrt(5 / (16 * np.pi)), np.sqrt(15 / (16 * np.pi))
    return np.stack([c0 + 0 * x, c1 * y, c1 * z, c1 * x, c2 * x * y, c2 * y * z,
                     c20 * (3 * z * z - 1), c2 * x * z, c22 * (x * x - y * y)])


def sphere(nt=16, nph=32):
    t, wt = np.polynomial.legendre.leggauss(nt)
    ph = 2 * np.pi * np.arange(nph) / nph
    T, P = np.meshgrid(t, ph, indexing="ij")
    st = np.sqrt(1 - T * T)
    Y = ylm((st * np.cos(P)).ravel(), (st * np.sin(P)).ravel(), T.ravel())
    w = (wt[:, None] * np.full(nph, 2 * np.pi / nph)[None]).ravel()
    return Y, w


def gaunt():
    Y, w = sphere()
    return np.einsum("lq,aq,bq,q->lab", Y, Y[:4], Y[:4], w)


def atom_tables(s, a):
    rd = s.radial
    roff = np.concatenate([[0], np.cumsum(rd["rad_n"])])
    poff = np.concatenate([[0], np.cumsum(rd["nphi"] * rd["rad_n"])])
    soff = np.concatenate([[0], np.cumsum(s.ms)])
    nr = rd["rad_n"][a]
    sl = slice(roff[a], roff[a + 1])
    ps = slice(poff[a], poff[a + 1])
    lmn = rd["proj_lmn"].reshape(-1, 3)[soff[a]:soff[a + 1]]
    return dict(r=rd["rad_r"][sl], w=rd["rad_w"][sl], core=rd["coredens"][sl], tcore=rd["tcoredens"][sl],
                phi=rd["phi"][ps].reshape(-1, nr), tphi=rd["tphi"][ps].reshape(-1, nr),
                ang=lmn[:, 0] ** 2 + lmn[:, 0] + lmn[:, 1], wave=lmn[:, 2])


def moments(R, U, core, t):
    """n_L(r) of sum_ij R_ij u_i u_j / r^2 Y_i Y_j + n_c."""
    uu = U[t["wave"]]
    n = np.einsum("ij,lij,ik,jk->lk", R, G[:, t["ang"]][:, :, t["ang"]], uu, uu) / t["r"] ** 2
    n[0] += SQ4PI * core
    return n


G = gaunt()


def dxc_numpy(s, rho):
    """pawxcm (pawxcdev = 1) + pawdijxcm, finite differences in 40 digits."""
    out = np.zeros_like(rho)
    doff = np.concatenate([[0], np.cumsum(np.asarray(s.ms) ** 2)])
    for a in range(s.natom):
        m = s.ms[a]
        t = atom_tables(s, a)
        R = rho[doff[a]:doff[a + 1]].reshape(m, m, order="F")
        Ga = G[:, t["ang"]][:, :, t["ang"]]
        D = np.zeros((m, m))
        for sign, U, core in ((1.0, t["phi"], t["core"]), (-1.0, t["tphi"], t["tcore"])):
            n = moments(R, U, core, t)
            up = np.maximum(0.5 * n[0] / SQ4PI, 1e-14)
            ns = 2 * up
            h = (ns + 1e-4 * ns) - ns  # ns +- h exact in double
            v0 = vxc_ld(ns).astype(np.float64)
            d1, d2 = derivatives_mp(ns, h)
            d1[up <= 1e-14] = 0.0
            d2[up <= 1e-14] = 0.0
            V = d1[None] * n
            V[0] = SQ4PI * v0 + d2 * (n[1:] ** 2).sum(axis=0) / (2 * SQ4PI)
            uu = U[t["wave"]]
            D += sign * np.einsum("lij,lk,ik,jk,k->ij", Ga, V, uu, uu, t["w"])
        out[doff[a]:doff[a + 1]] = D.reshape(-1, order="F")
    return out


def dxc_angular(s, rho):
    """The same term with v_xc evaluated on a full angular grid (no moment
    development): D_ij = int dOmega Y_i Y_j int (v(n) u_i u_j - v(n~) u~_i u~_j) dr."""
    Y, wq = sphere()
    out = np.zeros_like(rho)
    doff = np.concatenate([[0], np.cumsum(np.asarray(s.ms) ** 2)])
    for a in range(s.natom):
        m = s.ms[a]
        t = atom_tables(s, a)
        R = rho[doff[a]:doff[a + 1]].reshape(m, m, order="F")
        D = np.zeros((m, m))
        for sign, U, core in ((1.0, t["phi"], t["core"]), (-1.0, t["tphi"], t["tcore"])):
            n = moments(R, U, core, t)
            nq = np.einsum("lk,lq->kq", n, Y)
            v = vxc_ld(np.maximum(nq, 2e-14)).astype(np.float64)
            Yi = Y[t["ang"]]
            uu = U[t["wave"]]
            D += sign * np.einsum("iq,jq,q,kq,ik,jk,k->ij", Yi, Yi, wq, v, uu, uu, t["w"])
        out[doff[a]:doff[a + 1]] = D.reshape(-1, order="F")
    return out


def random_rhoij(s, seed, scale_sp=1.0, pp=True):
    """Symmetric rho_ij per atom: the s-s block positive, s-p couplings times
    scale_sp, p-p blocks only when pp."""
    rng = np.random.default_rng(seed)
    blocks = []
    for a in range(s.natom):
        m = s.ms[a]
        l = s.radial["proj_lmn"].reshape(-1, 3)[int(np.sum(s.ms[:a])):int(np.sum(s.ms[:a + 1])), 0]
        B = rng.standard_normal((m, m)) * 0.3
        B = B + B.T
        is_s = l == 0
        B[np.ix_(is_s, is_s)] = np.abs(B[np.ix_(is_s, is_s)]) + np.eye(int(is_s.sum()))
        B[np.ix_(is_s, ~is_s)] *= scale_sp
        B[np.ix_(~is_s, is_s)] *= scale_sp
        if not pp:
            B[np.ix_(~is_s, ~is_s)] = 0.0
        blocks.append(B.reshape(-1, order="F"))
    return np.concatenate(blocks)


def small_molecule():
    """A carbon-like and a hydrogen-like atom (the polyacene species: C with
    a core, H without) in a small box."""
    coords = np.array([[-1.2, 0.3, 0.1], [1.4, -0.2, -0.3]])
    return synthetic.build_system(n=(24, 20, 16), h=0.5, coords=coords, species=["C", "H"], seed=3)


@pytest.fixture(scope="module", params=["tiny", "molecule"])
def system(request):
    if request.param == "tiny":
        return synthetic.small_system("tiny", norb=3)
    return small_molecule()


def test_gaunt_coefficients():
    """G^0_ij = delta_ij / sqrt(4 pi); G^L_{00,L'} = delta_LL' / sqrt(4 pi)."""
    assert np.allclose(G[0], np.eye(4) / SQ4PI, atol=1e-15)
    for L in range(1, 4):
        assert np.allclose(G[L, 0], np.eye(4)[L] / SQ4PI, atol=1e-15)
    assert np.allclose(G, G.transpose(0, 2, 1), atol=1e-16)


def test_oracle_matches_numpy(system):
    s = system
    o = orc.Oracle(s)
    rho = random_rhoij(s, 4)
    got = o.onsite_xc(rho)
    ref = dxc_numpy(s, rho)
    assert np.abs(ref).max() > 1e-3
    assert np.abs(got - ref).max() <= 1e-11 * np.abs(ref).max()
    # symmetric in i, j
    doff = np.concatenate([[0], np.cumsum(np.asarray(s.ms) ** 2)])
    for a in range(s.natom):
        m = s.ms[a]
        B = got[doff[a]:doff[a + 1]].reshape(m, m)
        assert np.array_equal(B, B.T)


def test_spherical_density_is_exact(system):
    """With only s-s occupations the density is spherical: the moment
    development is exact, D_ij = delta(lm_i, lm_j) int (v(n) u_i u_j -
    v(n~) u~_i u~_j) dr with n = sum R u u / (4 pi r^2) + n_c."""
    s = system
    o = orc.Oracle(s)
    rho = random_rhoij(s, 5, scale_sp=0.0, pp=False)
    got = o.onsite_xc(rho)
    doff = np.concatenate([[0], np.cumsum(np.asarray(s.ms) ** 2)])
    for a in range(s.natom):
        m = s.ms[a]
        t = atom_tables(s, a)
        R = rho[doff[a]:doff[a + 1]].reshape(m, m, order="F")
        ref = np.zeros((m, m))
        for sign, U, core in ((1.0, t["phi"], t["core"]), (-1.0, t["tphi"], t["tcore"])):
            uu = U[t["wave"]]
            n = np.einsum("ij,ik,jk->k", R, uu, uu) / (4 * np.pi * t["r"] ** 2) + core
            v = vxc_ld(np.maximum(n, 2e-14)).astype(np.float64)
            same = (t["ang"][:, None] == t["ang"][None, :]).astype(np.float64)
            ref += sign * same * np.einsum("k,ik,jk,k->ij", v, uu, uu, t["w"])
        B = got[doff[a]:doff[a + 1]].reshape(m, m, order="F")
        assert np.abs(B - ref).max() <= 1e-9 * np.abs(ref).max(), a


def test_moment_development_is_second_order():
    """Scaling the non-spherical (s-p) part of rho_ij by t, the difference to
    the full angular quadrature falls at least as t^2 (pawxcdev = 1 keeps
    the second-order term of V_0 and the first-order V_L)."""
    s = small_molecule()
    o = orc.Oracle(s)
    errs = []
    for t in (0.1, 0.05, 0.025):
        rho = random_rhoij(s, 6, scale_sp=t, pp=False)
        errs.append(np.abs(o.onsite_xc(rho) - dxc_angular(s, rho)).max())
    assert errs[0] / errs[1] > 3.0 and errs[1] / errs[2] > 3.0, errs


def test_dij_carries_the_term():
    """The oracle's D_ij with the radial tables minus the one without them is
    D_xc of the same rho_ij (the clamp at dij_max is not reached here)."""
    s = small_molecule()
    psi = synthetic.orbitals(s, 3, seed=2).reshape(3, -1)
    s0 = dataclasses.replace(s, radial=None)
    o, o0 = orc.Oracle(s), orc.Oracle(s0)
    for q in (o, o0):
        q.set_vks(0, s.vks0)
        q.set_dij(0, s.dij_init)
        q.rebuild(psi, 0)
    d, d0 = o.get_dij(0), o0.get_dij(0)
    assert np.abs(d).max() < s.dij_max
    dx = o.onsite_xc(o.get_rhoij(0))
    assert np.abs(dx).max() > 1e-3
    assert np.abs((d - d0) - dx).max() <= 1e-12 * np.abs(d).max()
