"""GPU tests of the Gram / subspace-rotation row (orthog_phi.f90, diag.f90)
and of the stationary ground states built with it."""
import numpy as np
import pytest

import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import groundstate, synthetic

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def spec():
    s = synthetic.small_system("spec", norb=6)
    c = pkg.Context(s)
    c.set_vks(0, s.vks0)
    c.set_dij(0, s.dij_init)
    yield s, c
    c.close()


def test_gram_and_rotate(spec):
    torch = pytest.importorskip("torch")
    s, c = spec
    rng = np.random.default_rng(2)
    A = rng.standard_normal((6, s.nn)) + 1j * rng.standard_normal((6, s.nn))
    B = rng.standard_normal((5, s.nn)) + 1j * rng.standard_normal((5, s.nn))
    ref = A.conj() @ B.T * s.dv
    for dtype, tdt, tol in [(pkg.OPAW_C128, torch.complex128, 1e-12), (pkg.OPAW_C64, torch.complex64, 1e-5)]:
        a = torch.from_numpy(A).to(tdt).cuda()
        b = torch.from_numpy(B).to(tdt).cuda()
        G = c.gram_dev(dtype, a.data_ptr(), 6, b.data_ptr(), 5)
        assert rel(G, ref) < tol
        M = rng.standard_normal((6, 3)) + 1j * rng.standard_normal((6, 3))
        out = torch.empty((3, s.nn), dtype=tdt, device="cuda")
        c.rotate_dev(dtype, a.data_ptr(), 6, M, out.data_ptr())
        assert rel(out.cpu().numpy(), M.T @ A) < tol


def test_orthog_canonical(spec):
    s, c = spec
    rng = np.random.default_rng(3)
    A = rng.standard_normal((6, s.nn)) + 1j * rng.standard_normal((6, s.nn))
    c.upload(0, A)
    w = c.orthog(0)
    G0 = A.conj() @ A.T * s.dv
    assert np.allclose(w, np.linalg.eigvalsh(G0), rtol=1e-11)
    X = c.download(0, 6).reshape(6, -1)
    assert np.abs(X.conj() @ X.T * s.dv - np.eye(6)).max() < 1e-12
    # same span: the projector onto span(A) reproduces X
    Q, _ = np.linalg.qr(A.T)
    assert np.abs(Q @ (Q.conj().T @ X.T) - X.T).max() < 1e-10 * np.abs(X).max()


def test_stationary_ground_state():
    """Chebyshev subspace iteration + the v_loc / D0 shift give an exact
    stationary state: without a kick the density does not move."""
    s = synthetic.small_system("spec", norb=4)
    c = pkg.Context(s)
    c.set_vks(0, s.vks0)
    c.set_dij(0, s.dij_init)
    w, psi, res = groundstate.lowest_states(c, synthetic.orbitals(s, 4, seed=8).reshape(4, -1), n_iter=80, tol=1e-5)
    c.close()
    assert res.max() < 1e-5, res
    s2 = groundstate.stationary_system(s, psi)
    c = pkg.Context(s2)
    c.upload(0, psi)
    c.rebuild(0, pkg.PREC_FP64)
    assert rel(c.get_vks(0), s.vks0) < 1e-12
    assert rel(c.get_dij(0), s.dij_init) < 1e-11
    rho0 = c.get_density(0)
    c.excite(1, 0.0)
    c.tddft_steps(5, 0.05, 1e-3, pkg.PREC_FP64)
    c.rebuild(0, pkg.PREC_FP64)
    assert rel(c.get_density(0), rho0) < 1e-5
    c.close()


def test_mixed_dipole_on_stationary_state():
    """The mixed-precision signal against FP64 from a stationary ground state
    (the regime of a real run): relative error <= 1e-6 over 20 steps."""
    s = synthetic.small_system("spec", norb=4)
    c = pkg.Context(s)
    c.set_vks(0, s.vks0)
    c.set_dij(0, s.dij_init)
    w, psi, res = groundstate.lowest_states(c, synthetic.orbitals(s, 4, seed=8).reshape(4, -1), n_iter=80, tol=1e-5)
    c.close()
    s2 = groundstate.stationary_system(s, psi)
    c = pkg.Context(s2)
    out = {}
    for prec in (pkg.PREC_FP64, pkg.PREC_MIXED):
        c.upload(0, psi)
        c.excite(1, 1e-3)
        out[prec] = c.tddft_steps(20, 0.05, 1e-3, prec)[:, 0]
    err = np.abs(out[pkg.PREC_MIXED] - out[pkg.PREC_FP64]).max() / np.abs(out[pkg.PREC_FP64]).max()
    assert err < 1e-6, err
    c.close()


def test_scf_self_consistent():
    """The device SCF (main.f90:67-96 loop: rebuild, DIIS mixing, Chebyshev
    filtering) reaches a self-consistent state of the system as it is: the
    Hamiltonian rebuilt from the final orbitals is the one they diagonalise,
    and the density no longer moves under an unkicked propagation."""
    s = synthetic.small_system("tiny", norb=4)
    c = pkg.Context(s)
    c.set_vks(0, s.vks0)
    c.set_dij(0, s.dij_init)
    w, psi, hist = groundstate.scf(c, synthetic.orbitals(s, 4, seed=3).reshape(4, -1), max_iter=80,
                                   tol_v=1e-7, tol_res=1e-5)
    v_in, d_in = c.get_vks(0), c.get_dij(0)
    c.upload(0, psi)
    c.rebuild(0, pkg.PREC_FP64)
    assert np.abs(c.get_vks(0) - v_in).max() < 1e-6
    assert np.all(np.diff(w) >= -1e-12)
    rho0 = c.get_density(0)
    c.excite(1, 0.0)
    c.tddft_steps(5, 0.05, 1e-3, pkg.PREC_FP64)
    c.rebuild(0, pkg.PREC_FP64)
    assert rel(c.get_density(0), rho0) < 1e-4
    c.close()


def test_lowest_states_against_oracle():
    """The device eigensolver's eigenpairs checked with the oracle's operator:
    the Rayleigh-Ritz eigenvalues of S^-1/2 H S^-1/2 (oracle shs) on the
    returned orbitals equal the returned eigenvalues within 1e-6 Ha, and the
    oracle's residuals |shs x_i - w_i x_i| stay at the solver's tolerance."""
    import oracle as orc

    s = synthetic.small_system("spec", norb=4)
    c = pkg.Context(s)
    c.set_vks(0, s.vks0)
    c.set_dij(0, s.dij_init)
    w, psi, res = groundstate.lowest_states(c, synthetic.orbitals(s, 4, seed=8).reshape(4, -1), n_iter=80, tol=1e-5)
    c.close()
    o = orc.Oracle(s)
    o.set_vks(0, s.vks0)
    o.set_dij(0, s.dij_init)
    X = np.asarray(psi).reshape(4, -1)
    HX = np.asarray(o.shs(X)).reshape(4, -1)
    Hs = X.conj() @ HX.T * s.dv
    assert np.abs(Hs - Hs.conj().T).max() < 1e-9 * np.abs(Hs).max()
    ev = np.linalg.eigvalsh(0.5 * (Hs + Hs.conj().T))
    assert np.abs(ev - np.sort(w)).max() < 1e-6, (ev, w)
    r = np.sqrt((np.abs(HX - w[:, None] * X) ** 2).sum(axis=1) * s.dv)
    assert r.max() < 1e-4, r


def test_orthonormalize_on_device(spec):
    """FP64 Cholesky and Loewdin orthonormalisation without a host eigensolve
    (opaw_orthonormalize_dev): Cholesky gives Psi L^-H, Loewdin Psi G^-1/2,
    both with an identity Gram matrix; Loewdin refuses orbitals far from
    orthonormal."""
    s, c = spec
    rng = np.random.default_rng(4)
    Q = synthetic.orbitals(s, 6, seed=9).reshape(6, -1)
    A = Q + 0.02 * (rng.standard_normal(Q.shape) + 1j * rng.standard_normal(Q.shape)) * np.abs(Q).max()
    G = A.conj() @ A.T * s.dv
    w, V = np.linalg.eigh(G)
    lo = (A.T @ (V @ np.diag(w ** -0.5) @ V.conj().T)).T   # Psi G^-1/2
    L = np.linalg.cholesky(G)
    ch = (A.T @ np.linalg.inv(L).conj().T).T                # Psi L^-H
    for method, ref in ((0, ch), (1, lo)):
        c.upload(0, A)
        off = c.orthonormalize(0, method)
        assert abs(off - np.abs(G - np.eye(6)).max()) < 1e-12
        X = c.download(0, 6).reshape(6, -1)
        assert np.abs(X.conj() @ X.T * s.dv - np.eye(6)).max() < 1e-12, method
        assert rel(X, ref) < 1e-11, method
    B = rng.standard_normal((6, s.nn)) + 1j * rng.standard_normal((6, s.nn))
    c.upload(0, B)
    with pytest.raises(pkg.OpawError) as e:
        c.orthonormalize(0, 1)
    assert e.value.status == 1
    c.orthonormalize(0, 0)
    X = c.download(0, 6).reshape(6, -1)
    assert np.abs(X.conj() @ X.T * s.dv - np.eye(6)).max() < 1e-11


def test_gram_hermitian_form(spec):
    """opaw_gram_herm_dev sums only the tiles on and above the diagonal and
    mirrors the rest: it equals the full Gram of A^H A, and the Hermitian
    part of A^H (H A), 40 orbitals (three tiles per side)."""
    torch = pytest.importorskip("torch")
    s, c = spec
    rng = np.random.default_rng(5)
    A = rng.standard_normal((40, s.nn)) + 1j * rng.standard_normal((40, s.nn))
    a = torch.from_numpy(A).cuda()
    ha = torch.empty_like(a)
    c.shs_apply_dev(0, pkg.OPAW_C128, a.data_ptr(), ha.data_ptr(), 40)
    c.sync()
    G = c.gram_dev(pkg.OPAW_C128, a.data_ptr(), 40, a.data_ptr(), 40)
    Gh = c.gram_herm_dev(pkg.OPAW_C128, a.data_ptr(), a.data_ptr(), 40)
    assert rel(Gh, G) < 1e-13 and np.abs(Gh - Gh.conj().T).max() < 1e-13 * np.abs(G).max()
    H = c.gram_dev(pkg.OPAW_C128, a.data_ptr(), 40, ha.data_ptr(), 40)
    Hh = c.gram_herm_dev(pkg.OPAW_C128, a.data_ptr(), ha.data_ptr(), 40)
    assert rel(Hh, 0.5 * (H + H.conj().T)) < 1e-11


def test_double_fp32_gram_and_rotation(spec):
    """OPAW_C128_DD: complex128 Gram matrices and rotations in double-FP32
    arithmetic agree with exact complex128 results to 1e-13 of the largest
    entry (rotations: of the largest output element), Hermitian form too."""
    torch = pytest.importorskip("torch")
    s, c = spec
    rng = np.random.default_rng(11)
    A = rng.standard_normal((37, s.nn)) + 1j * rng.standard_normal((37, s.nn))
    A[3] *= 1e-3  # rows of different scale
    B = rng.standard_normal((21, s.nn)) + 1j * rng.standard_normal((21, s.nn))
    a = torch.from_numpy(A).cuda()
    b = torch.from_numpy(B).cuda()
    ref = A.conj() @ B.T * s.dv
    G = c.gram_dev(pkg.OPAW_C128_DD, a.data_ptr(), 37, b.data_ptr(), 21)
    assert np.abs(G - ref).max() <= 1e-13 * np.abs(ref).max()
    refh = A.conj() @ A.T * s.dv
    Gh = c.gram_herm_dev(pkg.OPAW_C128_DD, a.data_ptr(), a.data_ptr(), 37)
    assert np.abs(Gh - refh).max() <= 1e-13 * np.abs(refh).max()
    assert np.array_equal(Gh, Gh.conj().T) or np.abs(Gh - Gh.conj().T).max() <= 1e-13 * np.abs(refh).max()
    M = rng.standard_normal((37, 19)) + 1j * rng.standard_normal((37, 19))
    out = torch.empty((19, s.nn), dtype=torch.complex128, device="cuda")
    c.rotate_dev(pkg.OPAW_C128_DD, a.data_ptr(), 37, M, out.data_ptr())
    c.sync()
    refr = M.T @ A
    assert np.abs(out.cpu().numpy() - refr).max() <= 1e-13 * np.abs(refr).max()
