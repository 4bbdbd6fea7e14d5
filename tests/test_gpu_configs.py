"""GPU parity on the grid shapes of the other two benchmark configurations:
the naphthalene case (48 x 48 x 32 at h = 0.5 Bohr, 18 atoms) and the
tetracene case (96 x 64 x 48 at h = 0.45 Bohr, 30 atoms), seeded synthetic
systems with those shapes and atom counts (projector boxes of the carbon
cutoff), and the generated naphthalene geometry with its carbon and hydrogen
projector sets, a few orbitals each: one TDDFT step in FP64 and mixed
precision against the oracle, and the mixed d_dip against FP64 over several
steps."""
import dataclasses

import numpy as np
import pytest

import oracle as orc
import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

SHAPES = {
    "naphthalene_48x48x32": dict(n=(48, 48, 32), h=0.5, natom=18, rc=1.5, seed=11, face_margin=3.6),
    "tetracene_96x64x48": dict(n=(96, 64, 48), h=0.45, natom=30, rc=1.5, seed=12, face_margin=3.7),
}


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def make_system(name):
    if name in SHAPES:
        return synthetic.build_system(norb=3, **SHAPES[name])
    # a generated polyacene (C atoms: 8 projectors, H atoms: 5, two box sizes),
    # three of its orbitals occupied
    return dataclasses.replace(synthetic.molecule(name), rnel=6.0)


@pytest.fixture(scope="module", params=sorted(SHAPES) + ["naphthalene"])
def case(request):
    s = make_system(request.param)
    psi = synthetic.orbitals(s, 3, seed=21).reshape(3, -1)
    o = orc.Oracle(s)
    c = pkg.Context(s)
    yield request.param, s, psi, o, c
    c.close()


def test_step_matches_oracle(case):
    name, s, psi, o, c = case
    g = 1e-3
    pp = o.excite(psi, 1, g)
    p1, pp1, dref = o.tddft_steps(psi, pp, 1, 0.05, g)
    c.upload(0, psi)
    c.excite(1, g)
    d64 = c.tddft_steps(1, 0.05, g, pkg.PREC_FP64)
    assert rel(c.download(0, 3).reshape(p1.shape), p1) < 1e-10, name
    assert rel(c.download(1, 3).reshape(pp1.shape), pp1) < 1e-10, name
    assert np.allclose(d64, dref, rtol=1e-8, atol=1e-9 * np.abs(dref).max()), name
    c.upload(0, psi)
    c.excite(1, g)
    dmx = c.tddft_steps(1, 0.05, g, pkg.PREC_MIXED)
    q0 = c.download(0, 3).reshape(p1.shape)
    q1 = c.download(1, 3).reshape(pp1.shape)
    assert rel(q0, p1) < 1e-5, name
    assert rel(q1 - q0, pp1 - p1) < 1e-5, name
    assert np.abs(dmx - dref).max() < 1e-6 * np.abs(dref).max(), name


def test_mixed_dipole_series_vs_fp64(case):
    """d_dip(t) over 6 steps, mixed against the FP64 path from the same
    state: max_t |d_mixed - d_fp64| / max_t |d_fp64| (tolerance 1e-6)."""
    name, s, psi, o, c = case
    g = 1e-3
    c.upload(0, psi)
    c.excite(1, g)
    d64 = c.tddft_steps(6, 0.05, g, pkg.PREC_FP64)[:, 0]
    c.upload(0, psi)
    c.excite(1, g)
    dmx = c.tddft_steps(6, 0.05, g, pkg.PREC_MIXED)[:, 0]
    assert np.abs(dmx - d64).max() <= 1e-6 * np.abs(d64).max(), (name, dmx, d64)
