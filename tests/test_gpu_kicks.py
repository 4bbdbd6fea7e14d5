"""Several kicks against one unperturbed set (opaw_excite_kicks /
opaw_tddft_steps_kicks): every kicked set's d_dip(t), dip'(t) and orbitals
equal those of a run with that kick alone (tddft_excite.f90:1-16,
rk4.f90:15-33, tddft_plot.f90:57), in FP64 and in mixed precision, and the
unperturbed dipole equals the single-kick runs' one.  Each kick's arithmetic
is the single-kick arithmetic, so the tolerances are tight: 1e-12 of the
signal in FP64, 1e-9 in mixed precision (the 1e-6 bar of the dipole signal
holds by a wide margin)."""
import numpy as np
import pytest

import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import synthetic

pytestmark = pytest.mark.gpu

KICKS = [(1, 1e-3), (2, 5e-4), (3, 2e-3), (1, 1e-4), (2, 1e-3)]
DT = 0.05


@pytest.fixture(scope="module", params=["tiny", "spec"])
def case(request):
    s = synthetic.small_system(request.param, norb=3)
    psi = synthetic.orbitals(s, 3, seed=31).reshape(3, -1)
    c = pkg.Context(s)
    yield request.param, s, psi, c
    c.close()


@pytest.mark.parametrize("prec,tol", [(pkg.PREC_FP64, 1e-12), (pkg.PREC_MIXED, 1e-9)])
def test_kicks_equal_single_kick_runs(case, prec, tol):
    name, s, psi, c = case
    nsteps = 3
    ipol = [k[0] for k in KICKS]
    gam = [k[1] for k in KICKS]
    c.upload(0, psi)
    c.excite_kicks(ipol, gam)
    dip, dpp, dd = c.tddft_steps_kicks(nsteps, DT, prec)
    p0 = c.download(0, 3)
    kicked = [c.kick_download(k, 3) for k in range(len(KICKS))]
    assert dd.shape == (nsteps, len(KICKS), 3)
    for k, (ip, g) in enumerate(KICKS):
        c.upload(0, psi)
        c.excite(ip, g)
        d1, dp1, ddd1 = c.tddft_steps_dip(nsteps, DT, g, prec)
        scale = np.abs(ddd1).max()
        assert np.abs(dd[:, k] - ddd1).max() <= tol * scale, (name, k, dd[:, k], ddd1)
        assert np.abs(dpp[:, k] - dp1).max() <= tol * np.abs(dp1).max(), (name, k)
        assert np.abs(dip - d1).max() <= tol * np.abs(d1).max(), (name, k)
        q1 = c.download(1, 3)
        q0 = c.download(0, 3)
        # the kicked orbitals relative to their kick-induced difference
        assert np.abs(kicked[k] - q1).max() <= tol * 1e3 * np.abs(q1 - q0).max(), (name, k)
        assert np.abs(p0 - q0).max() <= tol * np.abs(q0).max(), (name, k)


def test_single_kick_entry_points_refuse_several_kicks(case):
    name, s, psi, c = case
    c.upload(0, psi)
    c.excite_kicks([1, 2], [1e-3, 1e-3])
    with pytest.raises(pkg.OpawError) as e:
        c.tddft_steps(1, DT, 1e-3, pkg.PREC_MIXED)
    assert e.value.status == 3
    # uploading a kicked set by hand returns to one kick
    c.upload(1, c.kick_download(1, 3))
    c.tddft_steps(1, DT, 1e-3, pkg.PREC_MIXED)


def test_kick_arguments_are_checked(case):
    name, s, psi, c = case
    c.upload(0, psi)
    for ip, g in [([4], [1e-3]), ([1], [float("nan")]), ([0, 1], [1e-3, 1e-3])]:
        with pytest.raises(pkg.OpawError) as e:
            c.excite_kicks(ip, g)
        assert e.value.status == 1


def test_ensemble_equals_separate_runs():
    """Three molecules-worth of contexts on different grids, each with its own
    kicks, stepped together through the replayed CUDA graph of
    opaw_ensemble_steps: every series equals that context's own
    opaw_tddft_steps_kicks run (7 steps: one plain, three graph replays of two
    steps)."""
    systems = [synthetic.small_system(k, norb=3) for k in ("tiny", "odd", "spec")]
    kicks = [([1, 2], [1e-3, 5e-4]), ([3], [2e-3]), ([1, 2, 3], [1e-3, 1e-3, 1e-4])]
    ctxs, psis = [], []
    for i, s in enumerate(systems):
        psis.append(synthetic.orbitals(s, 3, seed=40 + i).reshape(3, -1))
        ctxs.append(pkg.Context(s))
    nsteps = 7
    try:
        ref = []
        for c, p, (ip, g) in zip(ctxs, psis, kicks):
            c.upload(0, p)
            c.excite_kicks(ip, g)
            ref.append(c.tddft_steps_kicks(nsteps, DT, pkg.PREC_MIXED))
            ref[-1] = ref[-1] + (c.download(0, 3),)
        for c, p, (ip, g) in zip(ctxs, psis, kicks):
            c.upload(0, p)
            c.excite_kicks(ip, g)
        launches0 = [c.launches for c in ctxs]
        got = pkg.ensemble_steps(ctxs, nsteps, DT)
        for i, c in enumerate(ctxs):
            dip, dpp, dd, p0 = ref[i]
            gd, gp, gdd = got[i]
            assert np.abs(gdd - dd).max() <= 1e-12 * np.abs(dd).max(), i
            assert np.abs(gp - dpp).max() <= 1e-12 * np.abs(dpp).max(), i
            assert np.abs(gd - dip).max() <= 1e-12 * np.abs(dip).max(), i
            assert np.abs(c.download(0, 3) - p0).max() <= 1e-12 * np.abs(p0).max(), i
            assert c.launches > launches0[i]
    finally:
        for c in ctxs:
            c.close()
