"""The driver loop of opaw_tddft (tddft.f90:1-95) on a stand-in context that
records the calls: block sizes, checkpoint steps, the dipole files of a fresh
run and of two restarts, and the start from a wf_bar file."""
import os

import numpy as np
import pytest

from opaw_tddft_gb300 import dipfile, driver, restart, wfio


class FakeContext:
    """Orbitals on the host; a 'step' multiplies both sets by a fixed phase
    and returns dipoles that encode the step number."""

    def __init__(self, nn):
        self.nn = nn
        self.psi = [None, None]
        self.calls = []
        self.step = 0

    def upload(self, set_, psi):
        self.psi[set_] = np.array(psi, dtype=np.complex128).reshape(-1, self.nn)
        self.calls.append(("upload", set_, self.psi[set_].copy()))

    def download(self, set_, norb):
        return self.psi[set_][:norb].copy()

    def excite(self, ipol, gamma):
        r = np.arange(self.nn)
        self.psi[1] = self.psi[0] * np.exp(-1j * gamma * r)[None, :]
        self.calls.append(("excite", ipol, gamma))

    def tddft_steps_dip(self, n, dt, gamma, precision):
        self.calls.append(("steps", n))
        dip, dpp = np.zeros((n, 3)), np.zeros((n, 3))
        for k in range(n):
            self.step += 1
            for s in (0, 1):
                self.psi[s] = self.psi[s] * np.exp(-0.1j)
            dip[k] = [self.step, 0.5 * self.step, 0.0]
            dpp[k] = dip[k] + gamma * np.array([1.0, 2.0, 3.0]) * self.step
        return dip, dpp, (dpp - dip) / gamma


def test_fresh_run_blocks_and_checkpoints(tmp_path):
    c = FakeContext(12)
    psi0 = np.ones((2, 12)) + 0j
    it0, d = driver.opaw_tddft(c, nt=10, dt=0.05, gamma=1e-3, workdir=tmp_path, psi0=psi0, n_restart=4, block=3)
    assert it0 == 1 and d.shape == (10, 3)
    # blocks end at the checkpoint steps 4 and 8
    assert [x[1] for x in c.calls if x[0] == "steps"] == [3, 1, 3, 1, 2]
    assert restart.read_restart(tmp_path / "tddft_save", 12)[2] == 8
    a = dipfile.read_series(tmp_path / "d_dip.dat")
    assert a.shape == (10, 4)
    assert np.allclose(a[:, 0], 0.05 * np.arange(10), atol=1e-12)
    assert np.allclose(a[:, 1:], d, rtol=1e-7)
    assert not (tmp_path / "d_dip_cont.dat").exists()


def test_restart_chain(tmp_path):
    c = FakeContext(12)
    psi0 = np.arange(24).reshape(2, 12) + 1j
    driver.opaw_tddft(c, nt=10, dt=0.05, gamma=1e-3, workdir=tmp_path, psi0=psi0, n_restart=4, block=50)
    saved = restart.read_restart(tmp_path / "tddft_save", 12)
    # a new run resumes from the step-8 checkpoint: steps 9..14
    c2 = FakeContext(12)
    c2.step = 8
    it0, d = driver.opaw_tddft(c2, nt=14, dt=0.05, gamma=1e-3, workdir=tmp_path, n_restart=4, block=50)
    assert it0 == 9 and d.shape == (6, 3)
    assert not any(x[0] == "excite" for x in c2.calls)  # the kicked set comes from the checkpoint
    assert [x[1] for x in c2.calls if x[0] == "steps"] == [4, 2]
    cont = dipfile.read_series(tmp_path / "d_dip_cont.dat")
    assert cont.shape == (14, 4)  # steps 1-8 copied from d_dip.dat, then 9-14
    assert np.allclose(cont[:8], dipfile.read_series(tmp_path / "d_dip.dat")[:8])
    assert np.allclose(cont[8:, 0], 0.05 * np.arange(8, 14), atol=1e-12)
    assert restart.read_restart(tmp_path / "tddft_save", 12)[2] == 12
    # the second run started from the step-8 checkpoint's orbitals of both sets
    ups = [x for x in c2.calls if x[0] == "upload"]
    assert np.array_equal(ups[0][2], saved[0]) and np.array_equal(ups[1][2], saved[1])


def test_start_from_wf_bar(tmp_path):
    rng = np.random.default_rng(1)
    phi = rng.standard_normal((3, 2, 2, 3))
    wfio.write_wf(tmp_path / "wf_bar.bin", phi, [-1.0, -0.5, 0.2], 0.5, 0.5, 0.5, nocc=2)
    c = FakeContext(12)
    driver.opaw_tddft(c, nt=2, dt=0.05, gamma=1e-3, workdir=tmp_path, wf_path=tmp_path / "wf_bar.bin")
    # the occupied orbitals (ihomo = 2) were uploaded and kicked
    assert c.psi[0].shape == (2, 12)
    assert ("excite", 1, 1e-3) in c.calls
    with pytest.raises(ValueError):
        driver.opaw_tddft(FakeContext(12), nt=2, dt=0.05, gamma=1e-3, workdir=tmp_path / "x")


@pytest.mark.gpu
def test_driver_on_device_matches_straight_run(tmp_path):
    """FP64: 4 steps with a checkpoint every 2, then a restarted run to step 6,
    give the d_dip series of one straight 6-step call from the same state."""
    import opaw_tddft_gb300 as pkg
    from opaw_tddft_gb300 import synthetic

    s = synthetic.small_system("tiny", norb=3)
    psi = synthetic.orbitals(s, 3, seed=5).reshape(3, -1)
    c = pkg.Context(s)
    c.upload(0, psi)
    c.excite(1, 1e-3)
    ref = c.tddft_steps(6, 0.05, 1e-3, pkg.PREC_FP64)
    c.close()
    c = pkg.Context(s)
    _, d1 = driver.opaw_tddft(c, nt=4, dt=0.05, gamma=1e-3, workdir=tmp_path, psi0=psi, n_restart=2,
                              precision=pkg.PREC_FP64)
    c.close()
    c = pkg.Context(s)
    it0, d2 = driver.opaw_tddft(c, nt=6, dt=0.05, gamma=1e-3, workdir=tmp_path, n_restart=2,
                                precision=pkg.PREC_FP64)
    c.close()
    assert it0 == 5
    assert np.array_equal(np.concatenate([d1, d2]), ref)
    cont = dipfile.read_series(tmp_path / "d_dip_cont.dat")
    assert cont.shape == (6, 4) and np.allclose(cont[:, 1:], ref, rtol=1e-7)
