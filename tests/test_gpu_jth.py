"""The reference's naphthalene example on the device: the operator tables of
the JTH C and H datasets and cnt.ini's geometry on dim_paw.inp's 56 x 52 x 32
grid (pawsetup.py, tests/golden/jth_naphthalene.npz).  The FP64 rebuild and
one TDDFT step against the oracle on the same tables, then the
self-consistent LDA ground state of the molecule and the mixed-precision
d_dip(t) against FP64 from it."""
import dataclasses
import os

import numpy as np
import pytest

import oracle as orc
import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import groundstate, pawsetup, synthetic

pytestmark = pytest.mark.gpu

BUNDLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "jth_naphthalene.npz")


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.fixture(scope="module")
def naph():
    return pawsetup.from_bundle(BUNDLE)


def test_rebuild_and_step_match_oracle(naph):
    # four orbitals occupied (eight electrons) so that the rebuild's
    # renormalisation keeps the density near the orbitals'
    s = dataclasses.replace(naph, rnel=8.0)
    psi = synthetic.orbitals(s, 4, seed=5).reshape(4, -1)
    o = orc.Oracle(s)
    o.set_vks(0, s.vks0)
    o.set_dij(0, s.dij_init)
    o.rebuild(psi, 0)
    c = pkg.Context(s)
    try:
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        c.upload(0, psi)
        c.rebuild(0, pkg.PREC_FP64)
        assert rel(c.get_dij(0), o.get_dij(0)) < 1e-11
        assert rel(c.get_vks(0), o.get_vks(0)) < 1e-11
        g = 1e-3
        pp = o.excite(psi, 1, g)
        p1, pp1, dref = o.tddft_steps(psi, pp, 1, 0.05, g)
        c.upload(0, psi)
        c.excite(1, g)
        d64 = c.tddft_steps(1, 0.05, g, pkg.PREC_FP64)
        assert rel(c.download(0, 4).reshape(p1.shape), p1) < 1e-10
        assert rel(c.download(1, 4).reshape(pp1.shape), pp1) < 1e-10
        assert np.allclose(d64, dref, rtol=1e-8, atol=1e-9 * np.abs(dref).max())
    finally:
        c.close()


def test_ground_state_and_mixed_series(naph):
    """SCF of naphthalene (24 orbitals), then 40 steps after a gamma = 1e-3
    x kick: mixed against FP64, max_t |d_mixed - d_fp64| / max_t |d_fp64|
    <= 1e-6; the occupied eigenvalues are bound and the HOMO-LUMO order
    holds (the lowest state is the most bound)."""
    s, psi, w, res, hist = groundstate.self_consistent_state(naph, 24)
    assert res < 1e-5
    assert np.all(w < 0) and np.all(np.diff(w) >= -1e-12)
    c = pkg.Context(s)
    try:
        g = 1e-3
        c.upload(0, psi)
        c.excite(1, g)
        d64 = c.tddft_steps(40, 0.05, g, pkg.PREC_FP64)[:, 0]
        c.upload(0, psi)
        c.excite(1, g)
        dmx = c.tddft_steps(40, 0.05, g, pkg.PREC_MIXED)[:, 0]
    finally:
        c.close()
    assert np.abs(d64).max() > 0
    assert np.abs(dmx - d64).max() <= 1e-6 * np.abs(d64).max()


@pytest.mark.parametrize("n", [(26, 22, 16), (52, 24, 20)])
def test_radix_11_and_13_grids(n):
    """Extents with prime factors 11 and 13 (the naphthalene input's ny = 52
    = 4 x 13, its Hartree box 104): one step in FP64 and mixed precision
    against the oracle."""
    s = synthetic.build_system(n=n, h=0.5, natom=3, seed=9, rc=0.8, norb=3)
    psi = synthetic.orbitals(s, 3, seed=2).reshape(3, -1)
    o = orc.Oracle(s)
    g = 1e-3
    pp = o.excite(psi, 1, g)
    p1, pp1, dref = o.tddft_steps(psi, pp, 1, 0.05, g)
    c = pkg.Context(s)
    try:
        c.upload(0, psi)
        c.excite(1, g)
        d64 = c.tddft_steps(1, 0.05, g, pkg.PREC_FP64)
        assert rel(c.download(0, 3).reshape(p1.shape), p1) < 1e-10
        assert rel(c.download(1, 3).reshape(pp1.shape), pp1) < 1e-10
        assert np.allclose(d64, dref, rtol=1e-8, atol=1e-9 * np.abs(dref).max())
        c.upload(0, psi)
        c.excite(1, g)
        c.tddft_steps(1, 0.05, g, pkg.PREC_MIXED)
        assert rel(c.download(0, 3).reshape(p1.shape), p1) < 1e-5
    finally:
        c.close()


def test_run_folder(tmp_path):
    """driver.run_folder on an input folder laid out like the reference's
    (`tddft 0`: ground state, wf_bar.txt, then 12 mixed steps): the dipole
    files and the wave-function file are written, and d_dip.dat holds the
    (it - 1) dt stamps and the dipoles the run returned."""
    from opaw_tddft_gb300 import dipfile, driver, pawxml, wfio

    ds, sym, xyz, par = pawxml.load_bundle(BUNDLE)
    pawxml.write_folder(str(tmp_path), ds, sym, xyz, dict(par, tddft="0", nt="12"))
    out = driver.run_folder(str(tmp_path), precision=driver.PREC_MIXED, block=6)
    assert out["nt"] == 12 and out["d_dip"].shape == (12, 3)
    assert np.all(np.isfinite(out["d_dip"])) and np.abs(out["d_dip"][:, 0]).max() > 0
    wf = wfio.read_wf(str(tmp_path / "wf_bar.txt"))
    assert wf["nstates"] == 24
    rows = dipfile.read_series(str(tmp_path / "d_dip.dat"))
    assert rows.shape[0] == 12
    # time stamps (it - 1) dt and the x component as computed
    assert np.allclose(rows[:, 0], np.arange(12) * out["dt"])
    assert np.allclose(rows[:, 1], out["d_dip"][:, 0], rtol=1e-7, atol=1e-12)
    assert (tmp_path / "dip.dat").exists()
