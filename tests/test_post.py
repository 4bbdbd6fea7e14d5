"""Host-side companions of the propagation: the reference's wave-function
file format (write_wf.f90 / read_wf.f90) and the absorption-spectrum
post-processing of d_dip(t)."""
import struct

import numpy as np
import pytest

from opaw_tddft_gb300 import spectrum, wfio


def _orbitals(rng, ns=3, nz=4, ny=3, nx=5):
    return rng.standard_normal((ns, nz, ny, nx)) + 1j * rng.standard_normal((ns, nz, ny, nx))


@pytest.mark.parametrize("binary", [True, False])
def test_wf_roundtrip(tmp_path, binary):
    rng = np.random.default_rng(4)
    phi = _orbitals(rng)
    eig = np.array([-0.5, -0.25, 0.125])
    p = tmp_path / ("wf_bar.bin" if binary else "wf_bar.txt")
    wfio.write_wf(p, phi, eig, 0.5, 0.45, 0.4, nocc=2, binary=binary)
    d = wfio.read_wf(p)
    assert (d["nx"], d["ny"], d["nz"], d["nstates"], d["ihomo"], d["nsp"]) == (5, 3, 4, 3, 2, 1)
    assert (d["dx"], d["dy"], d["dz"]) == (0.5, 0.45, 0.4)
    assert np.array_equal(d["eig"], eig)
    # sign(Re phi) |phi| (write_wf.f90:54-62), exact in both forms
    ref = np.where(phi.real > 0, np.abs(phi), -np.abs(phi))
    assert np.array_equal(d["phi"], ref)


def test_wf_binary_records(tmp_path):
    """The byte layout of Fortran unformatted sequential records: 4-byte
    length, payload, 4-byte length; 8-character tags; x fastest."""
    phi = np.arange(2 * 2 * 1 * 3, dtype=float).reshape(2, 2, 1, 3) + 1.0  # [ns, nz, ny, nx]
    p = tmp_path / "wf.bin"
    wfio.write_wf(p, phi, [1.0, 2.0], 1.0, 1.0, 1.0, nocc=1)
    b = p.read_bytes()
    assert b[:4] == struct.pack("<i", 12) and b[4:12] == b"nx      " and b[12:16] == struct.pack("<i", 3)
    assert b[16:20] == struct.pack("<i", 12)
    recs = list(wfio._records(b))
    assert [r[:8] for r in recs[:10]] == [b"nx      ", b"ny      ", b"nz      ", b"dx      ", b"dy      ",
                                        b"dz      ", b"nsp     ", b"nstates ", b"orbmn_wf", b"ihomo   "]
    assert recs[10] == b"evls    " and np.array_equal(np.frombuffer(recs[11], "<f8"), [1.0, 2.0])
    assert recs[12] == b"orbitals" and recs[13] == struct.pack("<ii", 1, 1)
    # state 1, tmp(nx, ny, nz) in Fortran order = x fastest
    assert np.array_equal(np.frombuffer(recs[14], "<f8"), phi[0].reshape(-1))


def test_wf_reader_takes_short_header(tmp_path):
    """Files without the orbmn_wf / ihomo records (the layout read_wf.f90
    reads) are accepted."""
    p = tmp_path / "wf.bin"
    with open(p, "wb") as f:
        def rec(x):
            f.write(struct.pack("<i", len(x)) + x + struct.pack("<i", len(x)))
        for k, v in (("nx", 2), ("ny", 1), ("nz", 1)):
            rec(k.ljust(8).encode() + struct.pack("<i", v))
        for k in ("dx", "dy", "dz"):
            rec(k.ljust(8).encode() + struct.pack("<d", 0.3))
        rec(b"nsp     " + struct.pack("<i", 1))
        rec(b"nstates " + struct.pack("<i", 1))
        rec(b"evls    ")
        rec(struct.pack("<d", -0.1))
        rec(b"orbitals")
        rec(struct.pack("<ii", 1, 1))
        rec(struct.pack("<2d", 0.5, -0.25))
    d = wfio.read_wf(p)
    assert d["nstates"] == 1 and np.array_equal(d["phi"].reshape(-1), [0.5, -0.25])


def test_strength_function_harmonic():
    """A harmonic response d(t) = -(N/w0) sin(w0 t) (N electrons kicked by
    exp(-i gamma x)) gives one positive peak at w0 whose weight approaches N."""
    N, w0, dt = 4.0, 0.35, 0.05
    t = dt * np.arange(1, 40001)
    d = -(N / w0) * np.sin(w0 * t)
    w = np.linspace(0.01, 1.0, 2000)
    S = spectrum.strength_function(d, dt, w, tau=200.0)
    assert abs(spectrum.first_peak(w, S) - w0) < 2e-3
    assert S.min() > -0.05 * S.max()
    assert np.trapezoid(S, w) == pytest.approx(N, rel=0.05)


def test_first_peak_of_two_lines():
    dt = 0.05
    t = dt * np.arange(1, 20001)
    d = -(1.0 / 0.2) * np.sin(0.2 * t) - (3.0 / 0.6) * np.sin(0.6 * t)
    w = np.linspace(0.02, 1.0, 1500)
    S = spectrum.strength_function(d, dt, w, tau=150.0, window="gauss")
    assert abs(spectrum.first_peak(w, S) - 0.2) < 3e-3


def test_restart_roundtrip_and_layout(tmp_path):
    """tddft_save/ as tddft_write_to_restart.f90 writes it: info = nb nodes it,
    one complex*16 record per orbital, rank 0's orbitals first."""
    from opaw_tddft_gb300 import restart

    rng = np.random.default_rng(9)
    psi = _orbitals(rng, ns=4)
    pp = _orbitals(rng, ns=4)
    d = tmp_path / "tddft_save"
    restart.write_restart(d, psi, pp, it=37, nodes=2)
    assert (d / "info").read_text().split() == ["2", "2", "37"]
    b = (d / "phi_bar.bin").read_bytes()
    nn = psi[0].size
    assert struct.unpack_from("<i", b, 0)[0] == 16 * nn and len(b) == 4 * (16 * nn + 8)
    assert np.array_equal(np.frombuffer(b[4:4 + 16 * nn], "<c16"), psi[0].reshape(-1))
    a, c, it = restart.read_restart(d, nn)
    assert it == 37 and np.array_equal(a, psi.reshape(4, -1)) and np.array_equal(c, pp.reshape(4, -1))
    with pytest.raises(ValueError):
        restart.read_restart(d, nn + 1)


@pytest.mark.gpu
def test_restart_through_context(tmp_path):
    """Resident orbitals of both sets -> tddft_save/ -> a fresh context."""
    import opaw_tddft_gb300 as pkg
    from opaw_tddft_gb300 import restart, synthetic

    s = synthetic.small_system("tiny", norb=3)
    psi = synthetic.orbitals(s, 3, seed=5).reshape(3, -1)
    c = pkg.Context(s)
    c.upload(0, psi)
    c.excite(1, 1e-3)
    restart.save(c, tmp_path / "tddft_save", it=12, norb=3)
    pp = c.download(1, 3).reshape(3, -1)
    c.close()
    c2 = pkg.Context(s)
    assert restart.load(c2, tmp_path / "tddft_save") == 12
    assert np.array_equal(c2.download(0, 3).reshape(3, -1), psi)
    assert np.array_equal(c2.download(1, 3).reshape(3, -1), pp)
    c2.close()


def test_fortran_e_format():
    """Ew.d output of format 888 (' ',4e18.8) in tddft_plot.f90."""
    from opaw_tddft_gb300.dipfile import fortran_e, format_d_dip_line

    assert fortran_e(1.5) == "    0.15000000E+01"
    assert fortran_e(-0.0123456789) == "   -0.12345679E-01"
    assert fortran_e(0.0) == "    0.00000000E+00"
    assert fortran_e(9.9999999999) == "    0.10000000E+02"
    assert fortran_e(2.5e-120) == "    0.25000000-119"
    line = format_d_dip_line(0.05, [1.0, -2.0, 3.0e-5])
    assert line == " " + "    0.50000000E-01    0.10000000E+01   -0.20000000E+01    0.30000000E-04\n"


def test_dipole_log_restart_chain(tmp_path):
    """plot_dip's files over a fresh run, a first restart (d_dip_cont.dat
    seeded from d_dip.dat) and a second restart (appended)."""
    from opaw_tddft_gb300.dipfile import DipoleLog, read_series

    rng = np.random.default_rng(3)
    dt = 0.05
    dd, dp, dq = rng.standard_normal((9, 3)), rng.standard_normal((9, 3)), rng.standard_normal((9, 3))
    with DipoleLog(dt, tmp_path) as log:  # fresh run, steps 1-5
        log.write_steps(0, dp[:5], dq[:5], dd[:5])
    a = read_series(tmp_path / "d_dip.dat")
    assert a.shape == (5, 4)
    assert np.allclose(a[:, 0], dt * np.arange(5), atol=1e-12)
    assert np.allclose(a[:, 1:], dd[:5], rtol=1e-7, atol=0)
    b = read_series(tmp_path / "dip.dat")
    assert b.shape == (5, 7) and np.allclose(b[:, 1:4], dp[:5], rtol=1e-15) and np.allclose(b[:, 4:], dq[:5], rtol=1e-15)
    with DipoleLog(dt, tmp_path, it_restart=3) as log:  # restarted from step 3's checkpoint
        with pytest.raises(ValueError):
            log.write(5, dd[4], dp[4], dq[4])
        log.write_steps(3, dp[3:6], dq[3:6], dd[3:6])
    c = read_series(tmp_path / "d_dip_cont.dat")
    assert c.shape == (6, 4)
    assert np.array_equal(c[:3], a[:3])  # copied through the same format
    assert np.allclose(c[3:, 1:], dd[3:6], rtol=1e-7, atol=0)
    e = read_series(tmp_path / "dip_cont.dat")
    assert e.shape == (6, 7)
    assert np.all(np.isnan(e[:3, 4:])) and np.allclose(e[:3, :4], b[:3, :4], rtol=1e-15)  # t, dip only
    assert np.allclose(e[3:, 4:], dq[3:6], rtol=1e-15)
    with DipoleLog(dt, tmp_path, it_restart=6) as log:  # second restart: appended
        log.write_steps(6, dp[6:9], dq[6:9], dd[6:9])
    f = read_series(tmp_path / "d_dip_cont.dat")
    assert f.shape == (9, 4) and np.array_equal(f[:6], c)
    assert np.allclose(f[6:, 0], dt * np.arange(6, 9), atol=1e-12)
    assert read_series(tmp_path / "d_dip.dat").shape == (5, 4)  # untouched


@pytest.mark.gpu
def test_steps_dip_matches_steps(tmp_path):
    """opaw_tddft_steps_dip returns what plot_dip writes: d_dip = (dip_pert -
    dip) / gamma, and the same d_dip as opaw_tddft_steps from the same state."""
    import opaw_tddft_gb300 as pkg
    from opaw_tddft_gb300 import synthetic
    from opaw_tddft_gb300.dipfile import DipoleLog, read_series

    s = synthetic.small_system("tiny", norb=3)
    psi = synthetic.orbitals(s, 3, seed=5).reshape(3, -1)
    gamma = 1e-3
    c = pkg.Context(s)
    for prec in (pkg.PREC_FP64, pkg.PREC_MIXED):
        c.upload(0, psi)
        c.excite(1, gamma)
        dip, dpp, dd = c.tddft_steps_dip(3, 0.05, gamma, prec)
        assert np.allclose(dd, (dpp - dip) / gamma, rtol=1e-6, atol=1e-9 * np.abs(dip).max() / gamma)
        c.upload(0, psi)
        c.excite(1, gamma)
        dd2 = c.tddft_steps(3, 0.05, gamma, prec)
        assert np.array_equal(dd, dd2)
    with DipoleLog(0.05, tmp_path) as log:
        log.write_steps(0, dip, dpp, dd)
    assert np.allclose(read_series(tmp_path / "d_dip.dat")[:, 1:], dd, rtol=1e-7, atol=0)
    c.close()
