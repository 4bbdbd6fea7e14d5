"""The launch-shape autotuner (csrc/autotune.cu): its candidates compute
bit-identical results, so a run with the tuner on equals a run with it off
bit for bit, and after a few steps the step's launch sites have picked a
candidate."""
import numpy as np
import pytest

import opaw_tddft_gb300 as pkg
from opaw_tddft_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["spec", "tiny"])
def test_tuned_run_equals_untuned(kind):
    s = synthetic.small_system(kind, norb=4)
    psi = synthetic.orbitals(s, 4, seed=6).reshape(4, -1)
    out = {}
    for on in (True, False):
        c = pkg.Context(s)
        c.tune_enable(on)
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        c.upload(0, psi)
        c.excite(1, 1e-3)
        # single steps (plain launches: every site is timed) then a block
        # that replays the captured graph
        d = [c.tddft_steps(1, 0.05, 1e-3, pkg.PREC_MIXED) for _ in range(12)]
        d.append(c.tddft_steps(10, 0.05, 1e-3, pkg.PREC_MIXED))
        out[on] = (np.concatenate(d), c.download(0, 4), c.download(1, 4), c.tune_report())
        c.close()
    assert np.array_equal(out[True][0], out[False][0])
    assert np.array_equal(out[True][1], out[False][1])
    assert np.array_equal(out[True][2], out[False][2])
    # the sites of the step (launched several times per step) have decided;
    # a set-up pass launched once or twice may still be timing
    rep = out[True][3]
    done = [t for t in rep if t["chosen"] >= 0]
    assert len(done) >= 3, rep
    for site in done:
        assert site["chosen"] < len(site["candidates"]), site
        assert len(site["ms"]) == len(site["candidates"]) and min(site["ms"]) > 0
    assert any(t["site"].startswith("dense pass") for t in done)
    assert any(t["site"].startswith("box terms") for t in done)
    if kind == "spec":  # z = 64 has a compile-time z pass
        # the kinetic z pass has timed its TMA-staged candidate as well (so
        # the bitwise equality above covers it)
        tma = [t for t in done if any("TMA" in x for x in t["candidates"])]
        assert tma and all(len(t["ms"]) == 3 and min(t["ms"]) > 0 for t in tma), rep
    # switched off after the context's set-up: nothing decided since
    assert all(t["chosen"] < 0 for t in out[False][3])


def test_graph_replay_equals_plain_launches():
    """A block of steps replays a captured two-step graph; the same call with
    kernel timing on (which issues every launch one by one) gives
    bit-identical dipoles and orbitals, with an odd step count (the last step
    runs plain after the replays)."""
    s = synthetic.small_system("spec", norb=4)
    psi = synthetic.orbitals(s, 4, seed=8).reshape(4, -1)
    out = []
    for block in (True, False):
        c = pkg.Context(s)
        c.tune_enable(False)
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        c.upload(0, psi)
        c.excite(1, 1e-3)
        if not block:
            c.ktime_begin()
        d = c.tddft_steps(11, 0.05, 1e-3, pkg.PREC_MIXED)
        if not block:
            assert c.ktime_end()[1] > 0  # the dense pass ran as timed plain launches
        out.append((d, c.download(0, 4), c.download(1, 4)))
        c.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)
