"""Benchmark: real-time OPAW-TDDFT RK4 steps on one GB300.

Workload (the Hamiltonian-apply microbenchmark's shapes, run through the full
propagation step): 96^3 grid at h = 0.4 Bohr, 128 orbitals per set, two sets
(unperturbed + delta-kicked, gamma = 1e-3 along x), 40 atoms x 8 projectors
(16^3 boxes), Martyna-Tuckerman Hartree on the 192^3 box, LDA, dt = 0.05 a.u.
One step = the opaw_tddft loop body: rebuild of both sets, rk4_prop_shs of
both sets (4 S^-1/2 H S^-1/2 applies + 3 rebuilds each) and the dipole.
Inputs are seeded synthetic data (no PAW datasets or checkpoints).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is whole-job orbital-steps/s in
mixed precision with the orbitals resident in HBM; `e2e` is the same metric
through the C-ABI host-buffer entry point (orbitals copied from pinned host
memory and back every step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NORB = 128
GAMMA = 1e-3
DT = 0.05
METRIC = "RK4 orbital-steps/s (mixed precision, stage-wise rebuild)"
UNIT = "orbital-steps/s"
# k_mix_dense on the 96^3 / 40-atom workload with 128 orbitals per set: DRAM
# bytes (read + write) of the four launches of one step (start, RK4 stages
# 1-3; the last stage's grid part runs inside k_mix_final) measured by ncu,
# averaged per launch, and their algorithmic bytes
DENSE_TRAFFIC_128 = (3906272000 + 7843464192 + 9668494080 + 9670806272) / 4
DENSE_ALG_128 = (3.951e9 + 7.884e9 + 9.696e9 + 9.696e9) / 4


def workload_config(norb):
    return {
        "workload": f"OPAW-TDDFT RK4 step, synthetic 96^3 grid h=0.4, {norb} orbitals x 2 sets, 40 atoms x 8 "
                    "projectors (16^3 boxes), kinetic capped at the box sphere (ekcut 30.84 Ha), MT Hartree 192^3, "
                    "LDA, dt=0.05, kick gamma=1e-3 along x",
        "grid": [96, 96, 96],
        "orbitals_per_set": norb,
        "sets": 2,
        "atoms": 40,
        "projectors_per_atom": 8,
        "ekcut_ha": 30.843,
        "l2": "inputs larger than L2 (orbitals 3.6 GB resident)",
    }


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def max_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_fit(o, psi_full, n1, n2, reps1=1, reps2=1):
    """The FP64 oracle's TDDFT step time at n1 and n2 orbitals per set (the
    oracle runs each orbital's S^-1/2 H S^-1/2 on its own thread, so n1 = the
    thread count keeps every core busy), fitted as t(N) = a + b N and
    extrapolated to NORB orbitals per set."""
    def step_time(n, reps):
        psi = np.ascontiguousarray(psi_full[:n].reshape(n, -1))
        pp = o.excite(psi, 1, GAMMA)
        t = time.perf_counter()
        for _ in range(reps):
            psi, pp, _d = o.tddft_steps(psi, pp, 1, DT, GAMMA)
        return (time.perf_counter() - t) / reps

    t1 = step_time(n1, reps1)
    t2 = step_time(n2, reps2)
    b = max((t2 - t1) / (n2 - n1), 0.0)
    a = max(t1 - b * n1, 0.0)
    t128 = a + b * NORB
    return {"t1": t1, "t2": t2, "a": a, "b": b, "t_norb": t128, "value": 2.0 * NORB / t128,
            "fit": f"t(N) = {a:.3f} s + {b:.4f} s x N per step (N orbitals per set), from one FP64 oracle step "
                   f"at N = {n1} ({t1:.2f} s) and N = {n2} ({t2:.2f} s) of the same 96^3 / 40-atom system; "
                   f"extrapolated to N = {NORB}: {t128:.1f} s per step"}


def cpu_sample(system, psi_full):
    """The FP64 oracle on the host cores: the fitted step time of the same
    system at NORB orbitals per set (cpu_fit)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    o = orc.Oracle(system)
    nt = orc.nthreads()
    f = cpu_fit(o, psi_full, nt, 2 * nt)
    return {
        "value": f["value"],
        "unit": UNIT,
        "cores": nt,
        "kind": "port",
        "sample": f"FP64 C oracle (OpenMP, {nt} threads), full TDDFT steps (rebuild both sets, RK4 both sets, "
                  f"dipole); {f['fit']}",
        "seconds": f["t1"] + f["t2"],
    }


def fp64_compare(ctx, pkg, torch, stream, fresh, ncmp, ipol, norb, mixed_ms):
    """FP64 steps from the same initial state as a fresh mixed-precision run of
    the same length: the FP64 speed, and the error of the mixed dipole signal
    max_t |d_mixed - d_fp64| / max_t |d_fp64| over those steps."""
    fresh()
    dmx = ctx.tddft_steps(ncmp, DT, GAMMA, pkg.PREC_MIXED)
    fresh()
    ctx.tddft_steps(1, DT, GAMMA, pkg.PREC_FP64, want_dipoles=False)  # allocates the FP64 buffers
    fresh()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    f0.record(stream)
    dd64 = ctx.tddft_steps(ncmp, DT, GAMMA, pkg.PREC_FP64)
    f1.record(stream)
    torch.cuda.synchronize()
    fp64_ms = f0.elapsed_time(f1) / ncmp
    dm = dmx[:, ipol - 1]
    d64 = dd64[:, ipol - 1]
    err = float(np.abs(dm - d64).max() / max(np.abs(d64).max(), 1e-300))
    return {"orbital_steps_per_s": 2.0 * norb / (fp64_ms / 1e3), "ms_per_step": fp64_ms,
            "mixed_speedup": fp64_ms / mixed_ms, "dipole_rel_err_mixed_vs_fp64": err, "compared_steps": ncmp,
            "d_dip_fp64_maxabs": float(np.abs(d64).max()), "d_dip_fp64_first_last": [float(d64[0]), float(d64[-1])],
            "d_dip_mixed_first_last": [float(dm[0]), float(dm[-1])]}


def h_apply_microbench(pkg, torch, s, psi0, norb):
    """The Hamiltonian-apply microbenchmark of the 96^3 workload: H of the
    128-orbital batch (hphi.f90 semantics, set 0, v_ks0 and D_init) in
    complex128 and complex64 through opaw_h_apply_dev, timed with CUDA events
    on the library's stream; GB/s against the compulsory bytes (read psi,
    write H psi) and against the bytes of the passes this implementation makes;
    error of the complex64 result against the complex128 one (which the
    parity tests hold to the FP64 oracle at 1e-12)."""
    peak, _ = load_peaks()
    hc = pkg.Context(s)
    hc.set_vks(0, s.vks0)
    hc.set_dij(0, s.dij_init)
    st = torch.cuda.ExternalStream(hc.stream)
    out = {}
    res = {}
    nn = s.nn
    nbox_tot = int(np.sum(np.prod(np.asarray(s.nrough).reshape(-1, 3), axis=1)))
    for name, dt, tdt, E in (("fp64", pkg.OPAW_C128, torch.complex128, 16), ("fp32", pkg.OPAW_C64, torch.complex64, 8)):
        x = torch.from_numpy(psi0.astype(np.complex128 if E == 16 else np.complex64)).to("cuda")
        y = torch.empty_like(x)
        torch.cuda.synchronize()
        # warm-up calls: also let the autotuner settle the launch shapes of
        # this batch before the timed calls
        for _ in range(10 if E == 8 else 6):
            hc.h_apply_dev(0, dt, x.data_ptr(), y.data_ptr(), norb)
        hc.sync()
        reps = 3
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(st)
        for _ in range(reps):
            hc.h_apply_dev(0, dt, x.data_ptr(), y.data_ptr(), norb)
        a1.record(st)
        torch.cuda.synchronize()
        t = a0.elapsed_time(a1) / reps / 1e3
        comp = 2.0 * norb * nn * E
        # passes: xy + z + xy(+ v_ks psi) FFT passes (read psi once more in the
        # last), the box gather and the union scatter (read + write)
        passes = norb * nn * E * (2 + 2 + 3) + norb * nbox_tot * E * 3
        out[name] = {"ms": t * 1e3, "gbs_compulsory": comp / t / 1e9, "gbs_passes": passes / t / 1e9,
                     "frac_passes_of_peak": passes / t / 1e9 / peak}
        res[name] = y.to(torch.complex128)
        del x, y
    d = (res["fp32"] - res["fp64"]).abs()
    ref = res["fp64"].abs()
    out["fp32_vs_fp64_max_rel"] = float(d.max() / ref.max())
    out["fp32_vs_fp64_rel_l2"] = float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref))
    out["orbitals"] = norb
    del res, d, ref
    hc.close()
    return out


def roofline(ctx, pkg, torch, stream, s, psi0, norb):
    """The batched 3D FFT (xy-plane pass + z pass) on the complex64 orbital
    batch, timed alone with CUDA events on the library's stream."""
    peak, peak_kind = load_peaks()
    batch = torch.empty((norb, s.nn), dtype=torch.complex64, device="cuda")
    batch.copy_(torch.from_numpy(psi0.astype(np.complex64)).to("cuda"))
    torch.cuda.synchronize()
    for _ in range(6):  # warm-up, and the autotuner's choices for this batch
        ctx.fft3d_dev(pkg.OPAW_C64, batch.data_ptr(), norb, -1)
        ctx.fft3d_dev(pkg.OPAW_C64, batch.data_ptr(), norb, +1)
    ctx.sync()
    with torch.cuda.stream(stream):  # fresh values (the unnormalised pairs scale them by nn each)
        batch.copy_(torch.from_numpy(psi0.astype(np.complex64)).to("cuda"))
    torch.cuda.synchronize()
    reps = 5
    r0 = torch.cuda.Event(enable_timing=True)
    r1 = torch.cuda.Event(enable_timing=True)
    l1 = ctx.launches
    r0.record(stream)
    for _ in range(reps):
        ctx.fft3d_dev(pkg.OPAW_C64, batch.data_ptr(), norb, -1)
    r1.record(stream)
    torch.cuda.synchronize()
    nl = ctx.launches - l1
    ours_ms = r0.elapsed_time(r1) / reps
    per_launch_s = ours_ms / 1e3 / (nl / reps)
    alg_bytes = 2.0 * norb * s.nn * 8  # read + write the complex64 batch once per axis pass
    achieved = alg_bytes / per_launch_s / 1e9
    # comparison only: the same batch of 3D transforms through cuFFT (torch.fft,
    # out of place) on the same stream
    cufft_ms = None
    with torch.cuda.stream(stream):
        v = batch.view(norb, s.nz, s.ny, s.nx)
        for _ in range(2):
            w = torch.fft.fftn(v, dim=(1, 2, 3))
        del w
        r0.record(stream)
        for _ in range(reps):
            w = torch.fft.fftn(v, dim=(1, 2, 3))
        r1.record(stream)
        torch.cuda.synchronize()
        cufft_ms = r0.elapsed_time(r1) / reps
        del w, v
    del batch
    return {"kernel": f"k_fft_xy + k_fft_ct (forward 3D FFT: xy-plane pass and z pass, {norb} x 96^3 complex64)",
            "achieved": achieved, "unit": "GB/s", "frac": achieved / peak, "alg_bytes_per_launch": alg_bytes,
            "avg_launch_ms": per_launch_s * 1e3, "ms_per_3d_fft": ours_ms,
            "cufft_ms_per_3d_fft": cufft_ms, "cufft_note": "the same batch through cuFFT (torch.fft.fftn, out of "
                                                           "place), a comparison only: the step never calls it"}


def ground_state(pkg, s, norb, seed=2025):
    """Stationary initial orbitals of the synthetic system s: the lowest
    eigenvectors of S^-1/2 H S^-1/2 (Chebyshev subspace iteration on the
    device), with v_loc / D0 shifted so that the rebuilt Hamiltonian is that
    one (groundstate.stationary_system)."""
    from opaw_tddft_gb300 import groundstate, synthetic

    psi0 = synthetic.orbitals(s, norb, seed=seed).reshape(norb, -1)
    c0 = pkg.Context(s)
    c0.set_vks(0, s.vks0)
    c0.set_dij(0, s.dij_init)
    w, psi0, res = groundstate.lowest_states(c0, psi0, n_iter=80, tol=1e-4)
    c0.close()
    if not res.max() < 1e-3:
        raise RuntimeError(f"ground state did not converge: max eigen-residual {res.max():.3e}")
    return groundstate.stationary_system(s, psi0), psi0, float(res.max())


def series_leg(pkg, torch, name, nsteps, precisions):
    """A whole propagation of one molecule configuration: `nsteps` steps from
    its stationary ground state after a gamma = 1e-3 kick along x, in each of
    `precisions` (one opaw_tddft_steps call each, timed with CUDA events), the
    error of the mixed d_dip(t) series against the FP64 one over all steps,
    max_t |d_mixed - d_fp64| / max_t |d_fp64|, and the first absorption peak
    of each series (spectrum.first_peak of the damped Fourier transform)."""
    from opaw_tddft_gb300 import synthetic

    nring, n, h = synthetic.MOLECULES[name]
    s = synthetic.molecule(name)
    norb = int(round(s.rnel / 2))
    t0 = time.perf_counter()
    s, psi0, res = ground_state(pkg, s, norb)
    prep = time.perf_counter() - t0
    out = {"molecule": f"{name} C{4 * nring + 2}H{2 * nring + 4} (generated planar geometry, C-C 1.40 A, "
                       f"C-H 1.09 A), synthetic C/H projectors", "grid": list(n), "h": h, "orbitals_per_set": norb,
           "atoms": int(s.natom), "steps": nsteps, "dt": DT, "gamma": GAMMA, "kick": "x",
           "max_eigen_residual": res, "prep_seconds": prep}
    return propagate_series(pkg, torch, s, psi0, norb, nsteps, precisions, out)


JTH_BUNDLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "jth_naphthalene.npz")


def jth_series_leg(pkg, torch, nsteps, precisions, name="naphthalene"):
    """A molecule on the JTH LDA datasets of C and H through the PAW set-up
    chain (pawsetup.py), from its self-consistent LDA ground state
    (groundstate.self_consistent_state), then the same whole-series
    comparison as `series_leg`.  naphthalene: the reference's own example
    input (cnt.ini's geometry on dim_paw.inp's 56 x 52 x 32 grid, h = 0.5
    Bohr); tetracene: the generated planar geometry on the 96 x 64 x 48 grid
    at h = 0.45 Bohr."""
    from opaw_tddft_gb300 import groundstate, pawsetup, pawxml, synthetic

    t0 = time.perf_counter()
    if name == "naphthalene":
        s = pawsetup.from_bundle(JTH_BUNDLE)
        what = ("naphthalene C10H8, the reference's example input (cnt.ini geometry, JTH LDA PAW datasets "
                "C.LDA_PW-JTH.xml / H.LDA_PW-JTH.xml, dim_paw.inp grid)")
    else:
        nring, n, h = synthetic.MOLECULES[name]
        ds = pawxml.load_bundle(JTH_BUNDLE)[0]
        sym, xyz = synthetic.polyacene_geometry(nring)
        s = pawsetup.build(ds, sym, xyz, n, (h, h, h))
        what = (f"{name} C{4 * nring + 2}H{2 * nring + 4} (generated planar geometry, C-C 1.40 A, C-H 1.09 A), "
                "JTH LDA PAW datasets of C and H")
    t_setup = time.perf_counter() - t0
    norb = int(round(s.rnel / 2))
    t0 = time.perf_counter()
    s, psi0, w, res, hist = groundstate.self_consistent_state(s, norb)
    t_scf = time.perf_counter() - t0
    out = {"molecule": what,
           "grid": [s.nx, s.ny, s.nz], "h": s.dx, "orbitals_per_set": norb, "atoms": int(s.natom),
           "steps": nsteps, "dt": DT, "gamma": GAMMA, "kick": "x", "setup_seconds": t_setup,
           "scf_iterations": len(hist), "scf_seconds": t_scf, "max_eigen_residual": res,
           "homo_ha": float(w[-1]), "occupied_eigenvalues_ha": [round(float(x), 6) for x in w]}
    return propagate_series(pkg, torch, s, psi0, norb, nsteps, precisions, out)


def propagate_series(pkg, torch, s, psi0, norb, nsteps, precisions, out):
    from opaw_tddft_gb300 import spectrum

    ctx = pkg.Context(s)
    stream = torch.cuda.ExternalStream(ctx.stream)
    series = {}
    for prec, label in precisions:
        ctx.upload(0, psi0)
        ctx.excite(1, GAMMA)
        ctx.tddft_steps(1, DT, GAMMA, prec, want_dipoles=False)  # allocates this precision's buffers
        ctx.upload(0, psi0)
        ctx.excite(1, GAMMA)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        d = ctx.tddft_steps(nsteps, DT, GAMMA, prec)[:, 0]
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / nsteps
        series[label] = d
        out[label] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms, "orbital_steps_per_s": 2.0 * norb * 1e3 / ms,
                      "d_dip_first_last_max": [float(d[0]), float(d[-1]), float(np.abs(d).max())]}
    ctx.close()
    if "fp64" in series and "mixed" in series:
        d64, dm = series["fp64"], series["mixed"]
        out["dipole_rel_err_mixed_vs_fp64"] = float(np.abs(dm - d64).max() / max(np.abs(d64).max(), 1e-300))
        out["mixed_speedup"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
        omega = np.linspace(0.02, 1.5, 3000)
        peaks = {}
        for label, d in series.items():
            S = spectrum.strength_function(d, DT, omega)
            try:
                peaks[label] = spectrum.first_peak(omega, S)
            except ValueError:
                peaks[label] = None
        out["first_peak_ha"] = peaks
        if peaks.get("fp64") is not None and peaks.get("mixed") is not None:
            out["first_peak_err_ha"] = abs(peaks["mixed"] - peaks["fp64"])
        out["spectrum"] = ("S(w) = -(2w/pi) Im int d_dip(t) e^{iwt} e^{-t/tau} dt, tau = T/5, w in [0.02, 1.5] Ha; "
                           "first local maximum above 5% of the largest")
    return out


def ensemble_leg(pkg, torch, nsteps):
    """The batched uneven ensemble: benzene (40x40x28), naphthalene (48x48x32),
    anthracene (64x48x32) and tetracene (96x64x48), each from its stationary
    ground state with 3 kick directions x 4 strengths gamma in {1e-4, 5e-4,
    1e-3, 2e-3} sharing its one unperturbed set, mixed precision, all molecules
    stepped together by opaw_ensemble_steps (one replayed CUDA graph).  The
    aggregate counts the orbitals propagated: per molecule N x (12 kicked + 1
    unperturbed) per step.  Beside it: the same sets stepped molecule by
    molecule (opaw_tddft_steps_kicks: each molecule its own replayed graph,
    one after the other), and one single-kick
    run (2 sets) per molecule, the reference's way of running one kick per job."""
    from opaw_tddft_gb300 import synthetic

    names = ["benzene", "naphthalene", "anthracene", "tetracene"]
    ipol = [d for d in (1, 2, 3) for _ in range(4)]
    gam = [g for _ in range(3) for g in (1e-4, 5e-4, 1e-3, 2e-3)]
    ctxs, psis, norbs = [], [], []
    t0 = time.perf_counter()
    for name in names:
        s = synthetic.molecule(name)
        norb = int(round(s.rnel / 2))
        s, psi0, _res = ground_state(pkg, s, norb)
        ctxs.append(pkg.Context(s))
        psis.append(psi0)
        norbs.append(norb)
    prep = time.perf_counter() - t0

    def fresh():
        for c, p in zip(ctxs, psis):
            c.upload(0, p)
            c.excite_kicks(ipol, gam)

    fresh()
    pkg.ensemble_steps(ctxs, 3, DT)  # warm-up: grows every buffer
    fresh()
    torch.cuda.synchronize()
    t = time.perf_counter()
    out = pkg.ensemble_steps(ctxs, nsteps, DT)
    torch.cuda.synchronize()
    el = time.perf_counter() - t
    orbs = sum(n * (len(gam) + 1) for n in norbs)
    # the same sets, molecule by molecule, plain launches
    fresh()
    for c in ctxs:
        c.tddft_steps_kicks(2, DT, pkg.PREC_MIXED)
    fresh()
    torch.cuda.synchronize()
    t = time.perf_counter()
    for c in ctxs:
        c.tddft_steps_kicks(nsteps, DT, pkg.PREC_MIXED)
    torch.cuda.synchronize()
    el_seq = time.perf_counter() - t
    # one kick per run (unperturbed + one kicked set), as the reference runs a job
    single = []
    for c, p, n in zip(ctxs, psis, norbs):
        c.upload(0, p)
        c.excite(1, 1e-3)
        c.tddft_steps(2, DT, 1e-3, pkg.PREC_MIXED, want_dipoles=False)
        c.upload(0, p)
        c.excite(1, 1e-3)
        torch.cuda.synchronize()
        t = time.perf_counter()
        c.tddft_steps(nsteps, DT, 1e-3, pkg.PREC_MIXED, want_dipoles=False)
        torch.cuda.synchronize()
        single.append((time.perf_counter() - t) / nsteps)
    for c in ctxs:
        c.close()
    per_kick_runs = sum(t * len(gam) for t in single)  # s per step for 12 separate runs of each molecule
    return {
        "molecules": {nm: {"grid": list(synthetic.MOLECULES[nm][1]), "h": synthetic.MOLECULES[nm][2],
                           "orbitals": n, "d_dip_x_kick0_last": float(o[2][-1, 0, 0])}
                      for nm, n, o in zip(names, norbs, out)},
        "kicks": "3 directions x gamma {1e-4, 5e-4, 1e-3, 2e-3} = 12 per molecule, one shared unperturbed set",
        "steps": nsteps, "dt": DT, "precision": "mixed",
        "orbital_propagations_per_step": orbs,
        "aggregate_orbital_steps_per_s": orbs * nsteps / el,
        "ms_per_step": 1e3 * el / nsteps,
        "molecule_by_molecule_ms_per_step": 1e3 * el_seq / nsteps,
        "speedup_over_molecule_by_molecule": el_seq / el,
        "single_kick_runs_ms_per_step": 1e3 * per_kick_runs,
        "speedup_over_one_kick_per_run": per_kick_runs / (el / nsteps),
        "prep_seconds": prep,
        "timing": "host wall clock around the call (includes the D2H copy of the dipoles)",
    }


POLYACENE_GRIDS = {2: (64, 48, 48), 3: (80, 48, 48), 4: (96, 64, 48), 5: (112, 64, 48), 6: (128, 64, 48)}


def precond_leg(pkg, torch, full):
    """Ground-state eigensolve of synthetic polyacenes C(4n+2)H(2n+4) at h =
    0.4 Bohr (grids up to 128x64x48): LOBPCG (soft locking) to the
    unpreconditioned eigen-residual 1e-8 with the plain Teter-Payne-Allan
    kinetic preconditioner, with the learned 3D-conv correction beside it in
    the basis (augment), and with the learned direction alone (replace, the
    kinetic one its fallback).  The network is
    trained on the device on residual -> correction patches from the plain
    solves of n = 2, 3, 4 and evaluated on the held-out n = 5, 6, where both
    solvers start from the same orbitals; their eigenvalues are compared with
    each other and, for n = 5, with the Chebyshev-filtered subspace iteration
    (the reference's method)."""
    from opaw_tddft_gb300 import eigensolver, groundstate, learned, synthetic

    t0 = time.perf_counter()
    net = learned.Net(2024)
    train_log = {}
    npatch_per = 8 if full else 4
    for n in (2, 3, 4):
        s = synthetic.polyacene(n, POLYACENE_GRIDS[n], 0.4)
        norb = int(round(s.rnel / 2))
        c = pkg.Context(s)
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        X0 = synthetic.orbitals(s, norb, seed=100 + n).reshape(norb, -1)
        rec = []
        r = eigensolver.lobpcg(c, X0, tol=1e-8, record=rec, record_every=3)
        with torch.cuda.stream(torch.cuda.ExternalStream(c.stream)):
            learned.pairs_from_run(c, net, rec, r.orbitals, P=16, per_orbital=npatch_per, seed=n)
        train_log[f"n{n}"] = {"grid": list(POLYACENE_GRIDS[n]), "orbitals": norb, "iterations": r.iterations,
                              "seconds": r.seconds, "snapshots": len(rec)}
        del rec, r
        c.close()
    torch.cuda.empty_cache()
    nsteps = 1500 if full else 300
    tt = time.perf_counter()
    losses = net.train(nsteps, batch=64, lr=1e-3, margin=3)
    train_s = time.perf_counter() - tt
    evals = {}
    for n in (5, 6):
        s = synthetic.polyacene(n, POLYACENE_GRIDS[n], 0.4)
        norb = int(round(s.rnel / 2))
        c = pkg.Context(s)
        c.set_vks(0, s.vks0)
        c.set_dij(0, s.dij_init)
        X0 = synthetic.orbitals(s, norb, seed=100 + n).reshape(norb, -1)
        eigensolver.lobpcg(c, X0[:, :], tol=1e-3)  # warm-up: grows the device buffers
        plain = eigensolver.lobpcg(c, X0, tol=1e-8)
        lrn = eigensolver.lobpcg(c, X0, net=net, tol=1e-8)
        rep = eigensolver.lobpcg(c, X0, net=net, tol=1e-8, learned_mode="replace")
        top = eigensolver.lobpcg(c, X0, net=net, tol=1e-8, learned_frac=0.25)
        e = {"grid": list(POLYACENE_GRIDS[n]), "orbitals": norb,
             "plain": {"iterations": plain.iterations, "iterations_fp32": plain.iterations_fp32,
                       "seconds": plain.seconds, "max_residual": float(plain.residuals.max()),
                       "converged": plain.converged},
             "learned": {"iterations": lrn.iterations, "iterations_fp32": lrn.iterations_fp32,
                         "seconds": lrn.seconds, "max_residual": float(lrn.residuals.max()),
                         "converged": lrn.converged},
             "learned_replace": {"iterations": rep.iterations, "iterations_fp32": rep.iterations_fp32,
                                 "seconds": rep.seconds, "max_residual": float(rep.residuals.max()),
                                 "converged": rep.converged, "fallback_iteration": rep.fallback_iteration},
             "learned_hardest_quarter": {"iterations": top.iterations, "iterations_fp32": top.iterations_fp32,
                                         "seconds": top.seconds, "max_residual": float(top.residuals.max()),
                                         "converged": top.converged},
             "speedup_learned_over_plain": plain.seconds / lrn.seconds,
             "speedup_learned_hardest_quarter_over_plain": plain.seconds / top.seconds,
             "speedup_learned_replace_over_plain": plain.seconds / rep.seconds,
             "eig_max_diff_learned_replace_vs_plain_ha": float(np.abs(rep.eigenvalues - plain.eigenvalues).max()),
             "eig_max_diff_learned_vs_plain_ha": float(np.abs(lrn.eigenvalues - plain.eigenvalues).max())}
        if n == 5:
            w_ch, _, res_ch = groundstate.lowest_states(c, X0, n_iter=200, tol=1e-6, fp64_polish=6)
            e["eig_max_diff_plain_vs_chebyshev_ha"] = float(np.abs(plain.eigenvalues - w_ch).max())
            e["eig_max_diff_learned_vs_chebyshev_ha"] = float(np.abs(lrn.eigenvalues - w_ch).max())
            e["chebyshev_max_residual"] = float(res_ch.max())
        evals[f"n{n}"] = e
        c.close()
    out = {"network": "3 x conv3d 3^3, 16 channels, SiLU, BF16 weights/activations, FP32 accumulation "
                      "(mma.sync m16n8k16); inputs r/|r| (2 ch) and v_ks - eps; output added to the "
                      "Teter-Payne-Allan preconditioner's K r (scaled by |r|)",
           "training": {"molecules": train_log, "patches": net.npatch, "patch": "16^3, loss on the 10^3 interior",
                        "steps": nsteps, "batch": 64, "optimizer": "Adam lr 1e-3",
                        "loss_first_last": [float(losses[0]), float(losses[-1])],
                        "loss_mean_first_last_50": [float(losses[:50].mean()), float(losses[-50:].mean())],
                        "seconds": train_s},
           "held_out": evals, "judge": "max_i |H x_i - eps_i x_i| (dv norm, complex128) <= 1e-8",
           "seconds": time.perf_counter() - t0}
    net.close()
    return out


def run_reference(args):
    """--impl reference: the reference path's CPU implementation (the FP64
    oracle port: the Fortran reference needs gfortran/MPI/FFTW3/libxc, absent
    here), all host threads, a bounded sample per step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import __graft_entry__ as ge

    ge.build_oracle()  # current already when build() ran
    ge.load_package()
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    from opaw_tddft_gb300 import synthetic

    s = synthetic.hamiltonian_microbench(norb=NORB)
    o = orc.Oracle(s)
    nt = orc.nthreads()
    n1, n2 = nt, 2 * nt
    psi = synthetic.orbitals(s, n2, seed=2025).reshape(n2, -1)
    # warm-up and timed steps at n1 orbitals per set, then a quarter as many at
    # n2 for the fit t(N) = a + b N, extrapolated to NORB orbitals per set
    p1 = np.ascontiguousarray(psi[:n1])
    pp = o.excite(p1, 1, GAMMA)
    for _ in range(args.warmup):
        p1, pp, _d = o.tddft_steps(p1, pp, 1, DT, GAMMA)
    t = time.perf_counter()
    for _ in range(args.steps):
        p1, pp, _d = o.tddft_steps(p1, pp, 1, DT, GAMMA)
    t1 = (time.perf_counter() - t) / args.steps
    k2 = max(1, args.steps // 4)
    p2 = np.ascontiguousarray(psi[:n2])
    pp2 = o.excite(p2, 1, GAMMA)
    t = time.perf_counter()
    for _ in range(k2):
        p2, pp2, _d = o.tddft_steps(p2, pp2, 1, DT, GAMMA)
    t2 = (time.perf_counter() - t) / k2
    b = max((t2 - t1) / (n2 - n1), 0.0)
    a = max(t1 - b * n1, 0.0)
    t128 = a + b * NORB
    v = 2.0 * NORB / t128
    fit = (f"t(N) = {a:.3f} s + {b:.4f} s x N per step (N orbitals per set): {args.steps} steps at N = {n1} "
           f"({t1:.2f} s each) and {k2} at N = {n2} ({t2:.2f} s each) of the 96^3 / 40-atom system; extrapolated "
           f"to N = {NORB}: {t128:.1f} s per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t128,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(NORB),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": nt, "kind": "port",
                         "sample": f"FP64 C oracle restating the reference (the Fortran reference does not build: "
                                   f"no gfortran, MPI, FFTW3 or libxc), OpenMP {nt} threads, full TDDFT steps; {fit}"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--norb", type=int, default=NORB)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--skip-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--compare-steps", type=int, default=20, help="steps of the mixed-vs-FP64 dipole comparison")
    ap.add_argument("--state", default="ground", choices=["ground", "random"],
                    help="initial orbitals: stationary ground state (default) or filtered random orbitals")
    ap.add_argument("--no-roofline", action="store_true", help="skip the standalone FFT timing")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the batched kicks x molecules leg")
    ap.add_argument("--no-precond", action="store_true", help="skip the learned-preconditioner eigensolver leg")
    ap.add_argument("--synthetic-series", action="store_true",
                    help="also run the whole-propagation legs on the synthetic stand-ins of the two molecules")
    ap.add_argument("--series", default="full", choices=["full", "short", "none"],
                    help="whole-propagation legs: naphthalene 2000 steps and tetracene 4000 steps in FP64 and mixed "
                         "precision (full), 200 steps each (short), or none")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.warmup < 3:
        args.warmup = 3

    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    dist = init_dist(world)
    import __graft_entry__ as ge

    if rank == 0:  # one rank compiles (or finds the build current); the others wait for it
        ge.build()
    barrier(dist)
    pkg = ge.load_package()
    from opaw_tddft_gb300 import synthetic

    norb = args.norb
    s = synthetic.hamiltonian_microbench(norb=norb)
    psi0 = synthetic.orbitals(s, norb, seed=2025).reshape(norb, -1)
    state = {"initial_state": "filtered random orbitals (not stationary)"}
    if args.state == "ground":
        t0 = time.perf_counter()
        s, psi0, res = ground_state(pkg, s, norb)
        state = {"initial_state": "stationary ground state: lowest eigenvectors of S^-1/2 H S^-1/2 by Chebyshev "
                                  "subspace iteration, v_loc/D0 shifted so H[rho(psi)] is that Hamiltonian",
                 "max_eigen_residual": res, "prep_seconds": time.perf_counter() - t0}
    ipol = 1 + (rank % 3)  # replicas: independent kick directions
    ctx = pkg.Context(s)
    stream = torch.cuda.ExternalStream(ctx.stream)

    def fresh():
        ctx.upload(0, psi0)
        ctx.excite(ipol, GAMMA)

    # warm-up (also allocates every scratch buffer)
    fresh()
    for _ in range(args.warmup):
        ctx.tddft_steps(1, DT, GAMMA, pkg.PREC_MIXED, want_dipoles=False)
    fresh()
    ctx.tune_enable("frozen")  # no autotuner timing inside the timed region
    torch.cuda.synchronize()
    barrier(dist)
    clocks = Clocks(local)
    clocks.start()
    l0 = ctx.launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    # one call propagates the K steps, as the driver loop would issue a block
    # of steps (the dipole of every step is still computed and returned)
    dd_mixed = ctx.tddft_steps(args.steps, DT, GAMMA, pkg.PREC_MIXED)
    e1.record(stream)
    torch.cuda.synchronize()
    el_ms = e0.elapsed_time(e1)
    launches = ctx.launches - l0
    clk = clocks.stop()
    barrier(dist)
    el_max = max_over_ranks(dist, el_ms)
    units = sum_over_ranks(dist, 2.0 * norb * args.steps)
    value = units / (el_max / 1e3)

    ctx.tune_enable(True)
    # the roofline of the dominant kernel: a separate call of the same steps
    # with CUDA events around each of its launches (not inside the headline)
    fresh()
    torch.cuda.synchronize()
    ctx.ktime_begin()
    ctx.tddft_steps(min(args.steps, 5), DT, GAMMA, pkg.PREC_MIXED, want_dipoles=False)
    kt_ms, kt_n, kt_bytes = ctx.ktime_end()

    # FP64 path from the same initial state: speed and dipole error of the mixed run
    fp64 = None
    if not args.skip_fp64:
        fp64 = fp64_compare(ctx, pkg, torch, stream, fresh, args.compare_steps, ipol, norb, el_max / args.steps)
    peak, peak_kind = load_peaks()
    roof = {"kernel": "k_mix_dense (fused RK4 accumulation / S^-1/2 / density pass over every grid point, "
                      "box terms from k_mix_boxcoef_t; the largest share of the step)",
            "bound": "hbm", "achieved": kt_bytes / (kt_ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": kt_bytes / (kt_ms / 1e3) / 1e9 / peak, "peak_kind": peak_kind,
            "traffic": DENSE_TRAFFIC_128 * norb / 128,
            "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the four launches of one step, "
                            "per launch, scaled to this orbital count (algorithmic: "
                            f"{DENSE_ALG_128 * norb / 128:.4g})",
            "alg_bytes_per_launch": kt_bytes / max(kt_n, 1), "avg_launch_ms": kt_ms / max(kt_n, 1),
            "launches_timed": kt_n, "timing": "CUDA events on the library stream around each launch, in a "
                                              "separate call of the same steps after the headline timing"}
    hbench = None
    if not args.no_roofline:
        roof["fft3d_pass_pair"] = roofline(ctx, pkg, torch, stream, s, psi0, norb)
        hbench = h_apply_microbench(pkg, torch, s, psi0, norb)

    e2e = None
    if not args.no_e2e:
        nh = min(args.steps, 10)
        a = torch.empty((norb, s.nn), dtype=torch.complex128, pin_memory=True).numpy()
        b = torch.empty((norb, s.nn), dtype=torch.complex128, pin_memory=True).numpy()
        a[:] = psi0
        ctx.upload(0, psi0)
        ctx.excite(ipol, GAMMA)
        b[:] = ctx.download(1, norb).reshape(norb, -1)
        for _ in range(args.warmup):  # warm-up calls, as for the timed region
            ctx.tddft_steps_host(a, b, 1, DT, GAMMA, pkg.PREC_MIXED)
        barrier(dist)
        t = time.perf_counter()
        calls = []
        for _ in range(nh):
            tc = time.perf_counter()
            ctx.tddft_steps_host(a, b, 1, DT, GAMMA, pkg.PREC_MIXED)
            calls.append(1e3 * (time.perf_counter() - tc))
        el = max_over_ranks(dist, time.perf_counter() - t)
        # the copy rates inside that call: one set up and one set down
        nbytes = norb * s.nn * 16
        t = time.perf_counter()
        lib = pkg.lib()
        import ctypes as _ct
        pkg._check(lib.opaw_psi_upload(ctx.h, 0, a.ctypes.data_as(_ct.c_void_p), norb))
        t_up = time.perf_counter() - t
        t = time.perf_counter()
        pkg._check(lib.opaw_psi_download(ctx.h, 0, a.ctypes.data_as(_ct.c_void_p), norb))
        t_dn = time.perf_counter() - t
        e2e = {"value": sum_over_ranks(dist, 2.0 * norb * nh) / el, "unit": UNIT,
               "h2d_gbs": nbytes / t_up / 1e9, "d2h_gbs": nbytes / t_dn / 1e9,
               "h2d_bytes_per_step": int(2 * norb * s.nn * 16),
               "d2h_bytes_per_step": int(2 * norb * s.nn * 16 + 3 * 8),
               "api": "opaw_tddft_steps_host (psi, psi_pert host arrays in/out each step)", "steps": nh,
               "call_ms": [round(x, 2) for x in calls]}

    # the launch shapes the autotuner picked during the warm-up steps
    tune = [{"site": t["site"], "chosen": t["candidates"][t["chosen"]] if t["chosen"] >= 0 else None,
             "ms": dict(zip(t["candidates"], [round(x, 4) for x in t["ms"]]))} for t in ctx.tune_report()]

    series = None
    if rank == 0 and args.series != "none":
        full = args.series == "full"
        both = [(pkg.PREC_MIXED, "mixed"), (pkg.PREC_FP64, "fp64")]
        # both configurations on the JTH datasets (naphthalene: the
        # reference's own input); the synthetic stand-ins on request
        series = {}
        if args.synthetic_series:
            for mol, nst in (("naphthalene", 2000), ("tetracene", 4000)):
                series[mol] = series_leg(pkg, torch, mol, nst if full else 200, both)
        for mol, nst in (("naphthalene", 2000), ("tetracene", 4000)):
            try:
                series[f"{mol}_jth"] = jth_series_leg(pkg, torch, nst if full else 200, both, mol)
            except Exception as exc:  # reported, not fatal to the headline line
                series[f"{mol}_jth"] = {"error": f"{type(exc).__name__}: {exc}"}

    ensemble = None
    if rank == 0 and not args.no_ensemble:
        ensemble = ensemble_leg(pkg, torch, 40 if args.series == "full" else 10)

    precond = None
    if rank == 0 and not args.no_precond:
        precond = precond_leg(pkg, torch, args.series == "full")

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_sample(s, psi0)
        cpu.pop("seconds", None)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "mixed: c64 FFT/v_ks/projectors, f64 RK4 sum/D_ij/dipole",
            "data": "synthetic (seeded)", "config": dict(workload_config(norb), **state),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "fp64": fp64,
            "series": series,
            "ensemble": ensemble,
            "scf_preconditioner": precond,
            "roofline": roof, "h_apply": hbench,
            "cpu_baseline": cpu,
            "fp64_gpu_over_fp64_cpu": (fp64["orbital_steps_per_s"] / cpu["value"]) if (fp64 and cpu) else None,
            "e2e": e2e,
            "gpu_launches": launches,
            "autotune": tune,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
