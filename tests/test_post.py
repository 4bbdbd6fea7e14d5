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
