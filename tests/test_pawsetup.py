"""The PAW set-up chain (pawxml.py, pawsetup.py) on the reference's naphthalene
example: the JTH C and H datasets, cnt.ini and dim_paw.inp of its `naph/`
folder, bundled in tests/golden/jth_naphthalene.npz.  The reference ships no
outputs of its set-up, so the tables are held to the identities each step
must satisfy and to values stated in the datasets themselves."""
import math
import os

import numpy as np
import pytest

from opaw_tddft_gb300 import pawsetup, pawxml

HERE = os.path.dirname(os.path.abspath(__file__))
BUNDLE = os.path.join(HERE, "golden", "jth_naphthalene.npz")
SQ4PI = math.sqrt(4 * math.pi)


@pytest.fixture(scope="module")
def bundle():
    return pawxml.load_bundle(BUNDLE)


@pytest.fixture(scope="module")
def naph():
    return pawsetup.from_bundle(BUNDLE)


def test_bundle_contents(bundle):
    ds, sym, xyz, par = bundle
    assert sorted(ds) == ["C", "H"]
    assert (ds["C"]["Z"], ds["C"]["core"], ds["C"]["valence"]) == (6.0, 2.0, 4.0)
    assert (ds["H"]["Z"], ds["H"]["core"], ds["H"]["valence"]) == (1.0, 0.0, 1.0)
    assert ds["C"]["rpaw"] == pytest.approx(1.5073670273)
    assert list(ds["C"]["l"]) == [0, 0, 1, 1] and list(ds["H"]["l"]) == [0, 0, 1]
    # the log grid r = a (e^(d i) - 1) of the C dataset
    a, d = 9.4548737315239002e-04, 5.6729242389143399e-03
    i = np.arange(ds["C"]["r"].size)
    assert np.allclose(ds["C"]["r"], a * np.expm1(d * i), rtol=1e-12, atol=1e-15)
    assert sym.count("C") == 10 and sym.count("H") == 8 and xyz.shape == (18, 3)
    assert (par["nx"], par["ny"], par["nz"]) == ("56", "52", "32")
    # the datasets' densities: core charge of C is 2, H has none
    for s, nc in (("C", 2.0), ("H", 0.0)):
        r, dr = ds[s]["r"], ds[s]["dr"]
        q = 4 * math.pi * np.sum(ds[s]["ae_core"] / SQ4PI * r * r * dr)
        assert q == pytest.approx(nc, abs=1e-9)


def test_radial_orthogonalisation(naph):
    """transform_pphi: within each l the orthogonalised projectors are
    orthonormal on the radial mesh (inside rcut + rpad_r) and the overlap
    s_ij of the orthogonalised waves is diagonal."""
    for sp in naph.extra["species"].values():
        r, dr = sp.r, sp.dr
        n = pawsetup.upper_count(r, sp.rcut + pawsetup.RPAD_R)
        w = (r * r * dr)[:n]
        for lv in set(sp.lstate.tolist()):
            idx = np.nonzero(sp.lstate == lv)[0]
            P = sp.pt1[idx, :n]
            O = (P * w) @ P.T
            assert np.abs(O - np.eye(idx.size)).max() < 1e-12
            M = (sp.phi1[idx, :n] * w) @ sp.phi1[idx, :n].T - (sp.tphi1[idx, :n] * w) @ sp.tphi1[idx, :n].T
            assert np.abs(M - np.diag(np.diag(M))).max() < 1e-10
        assert np.allclose(sp.sij, np.diag(np.diag(sp.sij)))


def test_gaunt_and_moments(naph):
    G, waves = pawsetup.real_gaunt(1)
    # int Y00 Y_i Y_j = delta_ij / sqrt(4 pi); int Y20 p_z p_z = 2 / sqrt(20 pi)
    assert np.allclose(G[0], np.eye(4) / SQ4PI, atol=1e-14)
    iz = waves.index((1, 0))
    assert G[6, iz, iz] == pytest.approx(2.0 / math.sqrt(20 * math.pi), abs=1e-14)
    # p_x p_y couples only to L = 2, M = -2
    ix, iy = waves.index((1, 1)), waves.index((1, -1))
    nz = [a for a in range(9) if abs(G[a, ix, iy]) > 1e-14]
    assert nz == [4]
    for sp in naph.extra["species"].values():
        # Q^00 sqrt(4 pi) is the norm difference of the partial waves
        for p, (i, l, m) in enumerate(sp.chan):
            f = (sp.phi[i] ** 2 - sp.tphi[i] ** 2) * sp.r ** 2 * sp.dr
            assert sp.qijlm[0, p, p] * SQ4PI == pytest.approx(np.sum(f[1:]), rel=1e-12)
        # shape functions normalised to sum r^(L+2) g_L dr = 1
        nc = sp.nrcomp
        for L in range(sp.nL):
            assert np.sum(sp.r[:nc] ** (L + 2) * sp.dr[:nc] * sp.gl[L, :nc]) == pytest.approx(1.0, abs=1e-13)


def test_grid_tables(naph):
    s = naph
    mo = s.proj_offsets()
    so = s.ms_offsets()
    for a in range(s.natom):
        m, nb = int(s.ms[a]), s.nbox(a)
        P1 = s.p3d1[mo[a]:mo[a + 1]].reshape(m, nb)
        assert np.abs(P1 @ P1.T * s.dv - np.eye(m)).max() < 1e-12
        assert np.all(1.0 + s.s[so[a]:so[a + 1]] > 0)
        assert np.allclose(s.sinv[so[a]:so[a + 1]], 1.0 / (1.0 + s.s[so[a]:so[a + 1]]) - 1.0)
        # boxes inside the grid (non-periodic)
        assert s.ir_start[a].min() >= 1
        assert np.all(s.ir_start[a] + s.nrough[a] - 1 <= [s.nx, s.ny, s.nz])
    # the reference's box rule: 2 (ceil((rcut + 1) / h) + 1) -> 14 for C, 10 for H
    sym = s.extra["symbols"]
    assert all(s.nrough[a, 0] == (14 if sym[a] == "C" else 10) for a in range(s.natom))
    # g_00 integrates to sqrt(4 pi) x 1 / sqrt(4 pi) over its sphere (grid sum, 1%)
    off = 0
    for a in range(s.natom):
        ng = int(s.ngrid[a])
        g = s.g3d[off:off + s.nlm[a] * ng].reshape(s.nlm[a], ng)
        off += s.nlm[a] * ng
        assert g[0].sum() * s.dv / SQ4PI == pytest.approx(1.0, abs=0.02)
    # pseudo core charge: 10 carbons of the dataset's value, none for H
    sp = s.extra["species"]["C"]
    qc = 4 * math.pi * np.sum(sp.d["ps_core"] / SQ4PI * sp.r ** 2 * sp.dr)
    # band-limited on the grid: the G = 0 component carries the charge exactly
    assert s.ncoret.sum() * s.dv == pytest.approx(10 * qc, rel=1e-7)
    # far from the molecule v_loc is the sum of -Z_val / r
    nz_, ny_, nx_ = s.shape_f
    iz, iy, ix = 0, 0, 0
    p = np.array([-s.nx * s.dx / 2, -s.ny * s.dy / 2, -s.nz * s.dz / 2])
    zv = np.array([4.0 if t == "C" else 1.0 for t in sym])
    expect = -np.sum(zv / np.linalg.norm(s.coords - p, axis=1))
    assert s.vloc.reshape(nz_, ny_, nx_)[iz, iy, ix] == pytest.approx(expect, rel=1e-6)
    assert s.rnel == 48.0


def test_dij0_and_eijkl(naph):
    for sp in naph.extra["species"].values():
        D = sp.dij0()
        E = sp.eijkl()
        assert np.abs(D - D.T).max() == 0.0
        for p, (i, l, m) in enumerate(sp.chan):
            for q, (j, l2, m2) in enumerate(sp.chan):
                if (l, m) != (l2, m2):
                    assert D[p, q] == 0.0
        # equal across m of one p shell
        ps = [p for p, c in enumerate(sp.chan) if c[1] == 1 and c[0] == sp.chan[-1][0]]
        assert np.ptp([D[p, p] for p in ps]) < 1e-12
        # Hessian symmetries of the on-site Hartree energy
        assert np.abs(E - E.transpose(1, 0, 2, 3)).max() < 1e-12
        assert np.abs(E - E.transpose(0, 1, 3, 2)).max() < 1e-12
        assert np.abs(E - E.transpose(2, 3, 0, 1)).max() < 1e-12
        # rotational invariance: p_x p_x | p_x p_x equals p_y p_y | p_y p_y
        px = [p for p, c in enumerate(sp.chan) if c[1] == 1 and c[2] == 1]
        py = [p for p, c in enumerate(sp.chan) if c[1] == 1 and c[2] == -1]
        for a, b in zip(px, py):
            assert E[a, a, a, a] == pytest.approx(E[b, b, b, b], rel=1e-12)


def test_eijkl_is_the_hartree_hessian(naph):
    """E_ijkl against the on-site Hartree energy of whole densities:
    1/2 rho E rho = E_H[n1] - E_H[n~1 + n^] with n1, n~1 + n^ assembled per
    LM component from one random symmetric rho and solved once per L."""
    sp = naph.extra["species"]["C"]
    rng = np.random.default_rng(3)
    A = rng.standard_normal((sp.ms, sp.ms))
    rho = A + A.T
    E = sp.eijkl()
    lhs = 0.5 * np.einsum("ij,ijkl,kl->", rho, E, rho)
    r, dr = sp.r, sp.dr
    n = pawsetup.upper_count(r, sp.rcut)
    rs, drs = r[:n], dr[:n]
    tot = 0.0
    for a in range(sp.nlm):
        L = int(math.isqrt(a))
        nae = np.zeros(n)
        nps = np.zeros(n)
        for p, (i, _, _) in enumerate(sp.chan):
            for q, (j, _, _) in enumerate(sp.chan):
                g = sp.gaunt[a, p, q] * rho[p, q]
                if g == 0.0:
                    continue
                nae += g * sp.phi[i, :n] * sp.phi[j, :n]
                nps += g * (sp.tphi[i, :n] * sp.tphi[j, :n] + sp.qL[L, p, q] * sp.gl[L, :n])
        for dens, sgn in ((nae, 1.0), (nps, -1.0)):
            v = pawsetup.hartree_radial(dens, rs, drs, L)
            tot += sgn * 0.5 * pawsetup.cumint(dens * v * rs * rs, drs)[-1]
    assert lhs == pytest.approx(tot, rel=1e-10)


def test_radial_tables(naph):
    """The on-site XC tables: u = r R inside the sphere with Simpson weights;
    the norm difference of each partial wave matches its Q^00 moment."""
    for sp in naph.extra["species"].values():
        t = sp.radial_tables()
        assert t["r"][-1] >= sp.rcut and t["r"].size % 2 == 1
        for i in range(sp.lstate.size):
            dn = np.sum((t["phi"][i] ** 2 - t["tphi"][i] ** 2) * t["w"])
            p = [k for k, c in enumerate(sp.chan) if c[0] == i][0]
            assert dn == pytest.approx(sp.qijlm[0, p, p] * SQ4PI, rel=2e-4, abs=1e-6)


def test_read_dataset_errors(tmp_path):
    bad = tmp_path / "x.xml"
    bad.write_text("<not_paw/>")
    with pytest.raises(ValueError):
        pawxml.read_dataset(str(bad))


def _atom_levels(ds, el):
    """Lowest eigenvalues of one atom (28^3 grid, h = 0.5) after one oracle
    rebuild from the dataset's own bound pseudo waves and occupations."""
    import scipy.sparse.linalg as sla

    import oracle as orc

    d = ds[el]
    n, h = 28, 0.5
    c0 = np.array([0.1, 0.05, 0.02])
    s = pawsetup.build(ds, [el], c0[None, :], (n, n, n), (h, h, h))
    s.rnel = float(d["valence"])
    sp = s.extra["species"][el]
    xs = -n * h / 2 + np.arange(n) * h
    Z, Y, X = np.meshgrid(xs - c0[2], xs - c0[1], xs - c0[0], indexing="ij")
    R = np.maximum(np.sqrt(X * X + Y * Y + Z * Z), 1e-8).ravel()
    i0, w1, w2 = pawsetup.bracket(sp.r, R)
    orbs = []
    for i, (l, f) in enumerate(zip(d["l"], d["f"])):
        if f <= 0:
            continue
        rad = d["tphi"][i][i0] * w1 + d["tphi"][i][i0 + 1] * w2
        for m in range(-l, l + 1):
            yl = pawsetup.ylm(l, m, X.ravel() / R, Y.ravel() / R, Z.ravel() / R)
            orbs.append(np.sqrt(f / 2 / (2 * l + 1)) * rad * yl)
    o = orc.Oracle(s)
    o.set_vks(0, s.vks0)
    o.set_dij(0, s.dij_init)
    o.rebuild(o.sn_phi(np.array(orbs, dtype=np.complex128), 0.5), 0)
    k = 2 * np.pi * np.fft.fftfreq(n, h)
    K2 = (k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2) / 2

    def mv(V):
        V = np.asarray(V).reshape(s.nn, -1)
        return np.stack([o.shs(V[:, j].astype(np.complex128)[None, :], 0)[0].real for j in range(V.shape[1])], 1)

    def pc(V):
        V = np.asarray(V).reshape(s.nn, -1)
        return np.stack([np.fft.ifftn(np.fft.fftn(V[:, j].reshape(n, n, n)) / (K2 + 1.0)).real.ravel()
                         for j in range(V.shape[1])], 1)

    A = sla.LinearOperator((s.nn, s.nn), matvec=mv, matmat=mv, dtype=np.float64)
    M = sla.LinearOperator((s.nn, s.nn), matvec=pc, matmat=pc, dtype=np.float64)
    w, _ = sla.lobpcg(A, np.random.default_rng(0).standard_normal((s.nn, 5)), M=M, largest=False,
                      tol=1e-8, maxiter=500)
    return np.sort(w)


@pytest.mark.parametrize("el", ["C", "H"])
def test_atom_reproduces_dataset_eigenvalues(bundle, el):
    """The whole chain against the dataset's own numbers: one atom on a 28^3
    grid (h = 0.5 Bohr), its density built from the dataset's bound pseudo
    partial waves with the dataset's occupations (spherical: each m of a
    shell gets f / (2l + 1)), one rebuild (n~, n^, v_H, v_xc, D0 + E rho +
    D_xc + Dhat through the oracle), then the lowest eigenvalues of
    S^-1/2 H S^-1/2.  They equal the atomic eigenvalues the dataset states
    (`e` of its bound valence states: C 2s -0.5012, 2p -0.1990; H 1s
    -0.2335 Ha) to the grid's discretisation error."""
    d = bundle[0][el]
    w = _atom_levels(bundle[0], el)
    bound = {int(l): e for l, e, f in zip(d["l"], d["e"], d["f"]) if f > 0}
    assert w[0] == pytest.approx(bound[0], abs=2e-3)
    if 1 in bound:
        assert np.abs(w[1:4] - bound[1]).max() < 3e-3


def test_xml_round_trip_and_folder(bundle, naph, tmp_path):
    """write_dataset / read_dataset return every array bit for bit, and a
    folder laid out like the reference's input folder gives the system of
    the bundle."""
    ds = bundle[0]
    for s, d in ds.items():
        p = tmp_path / f"{s}.xml"
        pawxml.write_dataset(str(p), d)
        e = pawxml.read_dataset(str(p))
        for k in ("r", "dr", "phi", "tphi", "ptilde", "kij", "ae_core", "ps_core", "vloc_blochl", "l", "f", "e"):
            assert np.array_equal(np.asarray(e[k]), np.asarray(d[k])), (s, k)
        assert (e["Z"], e["rpaw"], e["rcomp"], e["shape_type"]) == (d["Z"], d["rpaw"], d["rcomp"], d["shape_type"])
    pawxml.write_folder(str(tmp_path), *bundle)
    f = pawsetup.from_folder(str(tmp_path))
    for k in ("p3d", "p3d1", "s", "qijlm", "g3d", "vloc", "ncoret", "dij0", "eijkl"):
        assert np.array_equal(getattr(f, k), getattr(naph, k)), k


def test_folder_errors(bundle, tmp_path):
    """A geometry atom without a dataset in pawfiles, and a periodic box, are
    refused before any table is built."""
    ds, sym, xyz, par = bundle
    only_c = {"C": ds["C"]}
    pawxml.write_folder(str(tmp_path), only_c, sym, xyz, par)
    with pytest.raises(ValueError, match="no dataset"):
        pawxml.read_folder(str(tmp_path))
    with pytest.raises(ValueError, match="isolated"):
        pawsetup.build(ds, sym, xyz, (56, 52, 32), (0.5, 0.5, 0.5), periodic=1)


def test_bessel_shape_functions(bundle):
    """The `bessel` compensation shapes: zero value and zero slope at r_comp,
    unit moment; and the atom's eigenvalues hardly depend on the shape (PAW
    is exact for any shape on a complete grid): the C levels with Bessel
    shapes stay within 1 mHa of those with the dataset's sinc shapes."""
    ds = dict(bundle[0])
    c = dict(ds["C"], shape_type="bessel")
    sp = pawsetup.Species(c)
    for L in range(sp.nL):
        a, q = pawsetup._bessel_shape(L, sp.rcomp)
        g = lambda r: a[0] * pawsetup._sph_jn(L, q[0] * r) + a[1] * pawsetup._sph_jn(L, q[1] * r)
        assert abs(g(sp.rcomp)) < 1e-12 * abs(g(0.3 * sp.rcomp))
        slope = (g(sp.rcomp * (1 + 1e-6)) - g(sp.rcomp * (1 - 1e-6))) / (2e-6 * sp.rcomp)
        assert abs(slope) < 1e-6 * abs(g(0.3 * sp.rcomp)) / sp.rcomp
        nc = sp.nrcomp
        assert np.sum(sp.r[:nc] ** (L + 2) * sp.dr[:nc] * sp.gl[L, :nc]) == pytest.approx(1.0, abs=1e-13)
    ds["C"] = c
    wb = _atom_levels(ds, "C")
    ws = _atom_levels(bundle[0], "C")
    assert np.abs(wb[:4] - ws[:4]).max() < 1e-3


def test_run_folder_refuses_other_modes(bundle, tmp_path):
    """driver.run_folder checks dim_paw.inp's switches before it builds
    anything: tddft must be -1, 0 or 1, and a propagation needs theory 3
    (the other theories are not on this path)."""
    from opaw_tddft_gb300 import driver

    ds, sym, xyz, par = bundle
    pawxml.write_folder(str(tmp_path), ds, sym, xyz, dict(par, tddft="2"))
    with pytest.raises(ValueError, match="tddft"):
        driver.run_folder(str(tmp_path))
    pawxml.write_folder(str(tmp_path), ds, sym, xyz, dict(par, tddft="0", theory="2"))
    with pytest.raises(ValueError, match="theory 3"):
        driver.run_folder(str(tmp_path))
    assert pawxml.fortran_float("-1d0") == -1.0 and pawxml.fortran_float("1e-3") == 1e-3
