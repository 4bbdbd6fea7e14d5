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
CPU_SAMPLE_NORB = 2


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


def cpu_sample(system, psi_full):
    """The FP64 oracle on the host cores: one full TDDFT step of the same
    system with CPU_SAMPLE_NORB orbitals per set."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc

    o = orc.Oracle(system)
    psi = np.ascontiguousarray(psi_full[:CPU_SAMPLE_NORB].reshape(CPU_SAMPLE_NORB, -1))
    pp = o.excite(psi, 1, GAMMA)
    t = time.perf_counter()
    o.tddft_steps(psi, pp, 1, DT, GAMMA)
    dt = time.perf_counter() - t
    return {
        "value": 2 * CPU_SAMPLE_NORB / dt,
        "unit": UNIT,
        "cores": orc.nthreads(),
        "kind": "port",
        "sample": f"one full TDDFT step (rebuild both sets, RK4 both sets, dipole) of the same 96^3 / 40-atom "
                  f"system with {CPU_SAMPLE_NORB} orbitals per set instead of {NORB}; FP64 C oracle, OpenMP; "
                  f"{dt:.1f} s",
        "seconds": dt,
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
    for _ in range(2):
        ctx.fft3d_dev(pkg.OPAW_C64, batch.data_ptr(), norb, -1)
        ctx.fft3d_dev(pkg.OPAW_C64, batch.data_ptr(), norb, +1)
    ctx.sync()
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
    per_launch_s = r0.elapsed_time(r1) / 1e3 / nl
    alg_bytes = 2.0 * norb * s.nn * 8  # read + write the complex64 batch once per axis pass
    achieved = alg_bytes / per_launch_s / 1e9
    del batch
    return {"kernel": f"k_fft_xy + k_fft_ct (forward 3D FFT: xy-plane pass and z pass, {norb} x 96^3 complex64)",
            "achieved": achieved, "unit": "GB/s", "frac": achieved / peak, "alg_bytes_per_launch": alg_bytes,
            "avg_launch_ms": per_launch_s * 1e3}


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
    psi = synthetic.orbitals(s, CPU_SAMPLE_NORB, seed=2025).reshape(CPU_SAMPLE_NORB, -1)
    o = orc.Oracle(s)
    pp = o.excite(psi, 1, GAMMA)
    for _ in range(args.warmup):
        psi, pp, _d = o.tddft_steps(psi, pp, 1, DT, GAMMA)
    t = time.perf_counter()
    for _ in range(args.steps):
        psi, pp, _d = o.tddft_steps(psi, pp, 1, DT, GAMMA)
    el = time.perf_counter() - t
    v = 2 * CPU_SAMPLE_NORB * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(NORB),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": orc.nthreads(), "kind": "port",
                         "sample": f"each step: one full TDDFT step of the 96^3 / 40-atom system with "
                                   f"{CPU_SAMPLE_NORB} orbitals per set (of {NORB}); FP64 C oracle restating "
                                   "the reference (the Fortran reference does not build: no gfortran, MPI, "
                                   "FFTW3 or libxc)"},
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
        from opaw_tddft_gb300 import groundstate

        t0 = time.perf_counter()
        c0 = pkg.Context(s)
        c0.set_vks(0, s.vks0)
        c0.set_dij(0, s.dij_init)
        w, psi0, res = groundstate.lowest_states(c0, psi0, n_iter=80, tol=1e-4)
        c0.close()
        if not res.max() < 1e-3:
            raise RuntimeError(f"ground state did not converge: max eigen-residual {res.max():.3e}")
        s = groundstate.stationary_system(s, psi0)
        state = {"initial_state": "stationary ground state: lowest eigenvectors of S^-1/2 H S^-1/2 by Chebyshev "
                                  "subspace iteration, v_loc/D0 shifted so H[rho(psi)] is that Hamiltonian",
                 "max_eigen_residual": float(res.max()), "prep_seconds": time.perf_counter() - t0}
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
    torch.cuda.synchronize()
    barrier(dist)
    clocks = Clocks(local)
    clocks.start()
    l0 = ctx.launches
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ctx.ktime_begin()  # CUDA events around every launch of the dominant kernel
    e0.record(stream)
    # one call propagates the K steps, as the driver loop would issue a block
    # of steps (the dipole of every step is still computed and returned)
    dd_mixed = ctx.tddft_steps(args.steps, DT, GAMMA, pkg.PREC_MIXED)
    e1.record(stream)
    torch.cuda.synchronize()
    el_ms = e0.elapsed_time(e1)
    kt_ms, kt_n, kt_bytes = ctx.ktime_end()
    launches = ctx.launches - l0
    clk = clocks.stop()
    barrier(dist)
    el_max = max_over_ranks(dist, el_ms)
    units = sum_over_ranks(dist, 2.0 * norb * args.steps)
    value = units / (el_max / 1e3)

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
            "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the four launches of one step at "
                            "128 orbitals, per launch (algorithmic: "
                            f"{DENSE_ALG_128 * norb / 128:.4g}; profiles/dram_traffic_k_mix_dense_96cube_128orb.md)",
            "alg_bytes_per_launch": kt_bytes / max(kt_n, 1), "avg_launch_ms": kt_ms / max(kt_n, 1),
            "launches_timed": kt_n, "timing": "CUDA events on the library stream around each launch, "
                                              "inside the timed region"}
    hbench = None
    if not args.no_roofline:
        roof["fft3d_pass_pair"] = roofline(ctx, pkg, torch, stream, s, psi0, norb)
        hbench = h_apply_microbench(pkg, torch, s, psi0, norb)

    e2e = None
    if not args.no_e2e:
        nh = min(args.steps, 5)
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
            "roofline": roof, "h_apply": hbench,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
