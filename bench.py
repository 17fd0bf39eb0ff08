#!/usr/bin/env python
"""Benchmark of the GB300 force path on the large rigid-water workload.

A step is one constant-energy MD step on the GPU (mdgpu_md_run): half drift
of centres of mass and quaternions, site co-ordinates, the force evaluation
-- link-cell real-space forces (force_calc) plus the reciprocal-space Ewald
sum (ewald), the work the reference's step hands to them -- molecular forces
and torques, two half kicks and the second half drift.  Workload: rigid
4-site TIP4P-like water, 32,768 molecules = 131,072 sites in a 99.34 Å cubic
box at 1.0 g/cm^3, Ewald alpha 0.3 /Å, cutoff 9 Å, k-cutoff for 1e-5 accuracy
(69,876 k-vectors); seeded lattice positions, uniform random orientations and
300 K Maxwell-Boltzmann momenta, dt = 1 fs (synthetic: there is no dataset).

Default arm (--impl gb300):
  value      MD steps/s of the FP32-mixed form, state resident in HBM,
             per-step CUDA events on the launching stream (L2 flushed between
             steps);
  fp64       the same for the plain FP64 GPU form, and their ratio;
  force_eval the force evaluation alone in both forms; accuracy of the mixed
             forces against the FP64 ones on the same configuration;
  nve        constant-energy runs (10^4 mixed steps, 300 FP64 steps by
             default): steps/s, ns/day, drift of the conserved quantity;
  e2e        MD steps/s through the public C API with the dynamic state in
             pinned host memory: every step uploads it (mdgpu_md_set_state),
             runs one step (mdgpu_md_run) and downloads it with the step's
             energies (mdgpu_md_get_state);
  e2e_force_call  force evaluations/s through the drop-in force call
             (mdgpu_forces), as a host-side integrator would make it: the H2D
             copy of the site co-ordinates and the D2H copy of forces,
             energies and stress inside every call;
  roofline   the dominant kernel's algorithmic FLOP/s (reference op counts)
             against the bound of the pipe it runs on: the measured bf16
             tensor peak (MEASURED_PEAKS.json, sustained) for the tensor-core
             reciprocal-space kernels, with the MMA work they issue beside
             it; the FP32 FMA peak measured on this GPU for the pair kernel;
  cpu_baseline  the reference algorithm's C restatement (oracle/port),
             -O2 -ffast-math, on all host cores: one full force evaluation
             timed whole (the reference's integrator is under 1% of its step
             at this size); cpu_baseline_1core the same on one core.
--impl reference: the CPU restatement alone (the reference is serial C with no
GPU code) on all host cores, on this workload, each step one full force
evaluation timed whole (nothing extrapolated).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "MD steps/s: FP32-mixed vs FP64 GPU forces at <=1e-5 rel RMS force err"
WORKLOAD = ("rigid 4-site water (TIP4P-like), 32768 molecules / 131072 sites, cubic box 99.34 A "
            "at 1.0 g/cm^3, LJ O-O + Ewald alpha=0.3/A, rc=9 A, kc=2.0358/A (1e-5), lazy link cells")
# Algorithmic work per unit (reference op counts; a sqrt/exp/divide is 1 flop,
# an FMA 2): k-space per (site, k): lz combination 6 + structure-factor adds 2
# (src/ewald.c:124-141,528-533) in the structure-factor pass, force 9
# (src/ewald.c:557-566) in the force pass; real space per evaluated pair:
# mk_r_sqr 11 + kernel (LJ + erfc) 45 + mk_forces 9 (src/force.c:700-743,
# src/kernel.c:188-211).
FLOPS_SFAC_PER_SITE_K = 8
FLOPS_FORCE_PER_SITE_K = 9
FLOPS_PAIR_LJ_ERFC = 65
STEP_PS = 0.001                      # 1 fs


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks():
    """The machine's measured HBM and bf16 tensor peaks (MEASURED_PEAKS.json at
    the repository root), or the stated fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return {"hbm_gbs": float(m["hbm_gbs"]), "bf16": float(m["bf16_tflops"]),
                "bf16_sustained": float(m["bf16_tflops_sustained"]), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16": 1900.0, "bf16_sustained": 1700.0, "source": "fallback"}


def tc_item_counts(sysm):
    """Counts of the tensor-core items (runs of up to 64 l values per (h,k)
    column of the k-list), largest first, padded with empty items to a
    multiple of 128 -- as the library builds them."""
    import math
    h = np.asarray(sysm.h, np.float64).reshape(9)
    kc = sysm.control.k_cutoff
    hmax = int(math.floor(kc / (2 * math.pi) * h[0]))
    kmax = int(math.floor(kc / (2 * math.pi) * math.sqrt(h[1] ** 2 + h[4] ** 2)))
    lmax = int(math.floor(kc / (2 * math.pi) * math.sqrt(h[2] ** 2 + h[5] ** 2 + h[8] ** 2)))
    hi = (2 * math.pi * np.linalg.inv(h.reshape(3, 3))).reshape(9)
    counts = []
    for hh in range(hmax + 1):
        for k in range(0 if hh == 0 else -kmax, kmax + 1):
            kx, ky, kzt = hh * hi[0] + k * hi[3], hh * hi[1] + k * hi[4], hh * hi[2] + k * hi[5]
            ls = np.arange(1 if hh == 0 and k == 0 else -lmax, lmax + 1)
            n = int(np.count_nonzero((kzt + ls * hi[8]) ** 2 + kx * kx + ky * ky < kc * kc))
            while n > 0:
                counts.append(min(n, 64))
                n -= 64
    counts = sorted(counts, reverse=True)
    return counts + [0] * (-len(counts) % 128)


def tc_mma_flops(sysm, nq):
    """Tensor-core work the two reciprocal-space kernels issue per launch
    (bf16 MMA flops, the split-operand term products and the padding of
    items to 16-column multiples included), from the k-list columns exactly
    as the library builds them (tc_item_counts): 128 items per
    structure-factor tile, 32 per force tile."""
    counts = tc_item_counts(sysm)
    np32 = (nq + 31) // 32 * 32
    # per 128-item tile and 16 sites: Ar and Ai times [Zr | Zi], six term products, N = 128
    sfac = (len(counts) // 128) * (np32 // 16) * 12 * 2 * 128 * 128 * 16
    force = ((nq + 127) // 128) * sum(12 * ((counts[t] + 15) // 16) * 2 * 128 * 128 * 16
                                      for t in range(0, len(counts), 32))
    return {"sfac": float(sfac), "kforce": float(force)}


def make_workload(seed=7):
    from moldy_gb300 import system as S
    return S.water(nside=32, seed=seed, alpha=0.3, cutoff=9.0)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while running."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[3:]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(sysm, threads=None, fast=True):
    """One full force evaluation of the reference algorithm on the host: its
    C restatement (bit-exact with the reference; -O2 -ffast-math, the
    reference's release flags) running force_calc and then ewald over every
    k-vector, each timed whole.  Returns (seconds, details)."""
    from oracle import port
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    r = port.force_calc(sysm, nthreads=threads, fast=fast)
    t_rs = time.perf_counter() - t0
    t0 = time.perf_counter()
    e = port.ewald(sysm, nthreads=threads, fast=fast)
    t_ew = time.perf_counter() - t0
    details = {"t_real_s": t_rs, "t_ewald_s": t_ew, "nkvec": e.info.nkvec, "pairs": int(r.info.npairs),
               "threads": threads}
    return t_rs + t_ew, details


def bench_config(world):
    """The workload description both arms print (the same dict)."""
    return {"workload": WORKLOAD, "nsites": 131072, "nkvec": 69876,
            "parallelism": f"{world} independent replicas" if world > 1 else "one replica"}


REFERENCE_STEP = ("one force evaluation (force_calc + ewald over all 69,876 k-vectors) of the reference "
                  "algorithm on the host; the reference's integrator, under 1% of its step at this size, "
                  "is not timed")


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    sysm = make_workload()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_baseline(sysm, threads)
    times, det = [], None
    t_all = time.perf_counter()
    for _ in range(args.steps):
        t, det = cpu_baseline(sysm, threads)
        times.append(t)
    wall = time.perf_counter() - t_all
    sec = sum(times) / len(times)
    sample = (f"each step one full force evaluation, timed whole: force_calc ({det['pairs']} pairs) and "
              f"ewald over all {det['nkvec']} k-vectors; C restatement of the reference, -O2 -ffast-math, "
              f"{threads} threads")
    line = {"metric": METRIC, "value": 1.0 / sec, "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded lattice water, uniform random orientations)",
            "config": bench_config(world),
            "step": REFERENCE_STEP,
            "impl": "reference",
            "cpu_baseline": {"value": 1.0 / sec, "unit": "steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": 1.0 / sec, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "ms_per_step_each": [1e3 * t for t in times],
            "wall_s": wall}
    print(json.dumps(line), flush=True)


def reduce_max(x, dist=None, device="cpu"):
    """The maximum of x over the ranks of the default process group (x itself
    without one): the slowest replica's time, which the job's rate uses."""
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def traffic_from_profiles():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except Exception:
            return {}
    return {}


def run_gpu(args):
    import torch
    from moldy_gb300 import _lib
    from moldy_gb300.dynamics import (MolecularDynamics, drift_per_ns, ns_per_day, species_dynamics,
                                      thermal_state)
    from moldy_gb300.forcefield import ForceField
    from moldy_gb300.system import CONV_E
    import ctypes as C

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    sysA = make_workload(seed=7)
    sysB = make_workload(seed=8)          # a second configuration for the force-only steps
    n = sysA.nsites
    dyn = species_dynamics(sysA, STEP_PS)
    state0 = thermal_state(sysA, dyn, 300.0, seed=9)
    # a dedicated (non-default) stream: the library launches on it and the
    # CUDA events below are recorded on it
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ff = ForceField(sysA, precision="mixed", device=local)
    ff.set_stream(stream.cuda_stream)
    d_site = [torch.from_numpy(np.ascontiguousarray(s.site)).to(dev) for s in (sysA, sysB)]
    d_force = torch.empty((3, n), dtype=torch.float64, device=dev)
    d_pe = torch.zeros(2, dtype=torch.float64, device=dev)
    d_st = torch.zeros(9, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def force_step(i):
        ff.forces_device(d_site[i % 2].data_ptr(), d_force.data_ptr(), d_pe.data_ptr(), d_st.data_ptr())

    def barrier():
        if dist is not None:
            dist.barrier()

    def timed(fn, nsteps):
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(nsteps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(nsteps)]
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(nsteps):
            flush.zero_()                      # L2 flush between timed steps
            starts[i].record(stream)
            fn(i)
            ends[i].record(stream)
        torch.cuda.synchronize()
        barrier()
        wall = time.perf_counter() - t0
        ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        return sum(ms) / nsteps, wall

    def max_over_ranks(x):
        return reduce_max(x, dist, dev)

    # ---- the headline: MD steps on the GPU, mixed form ----------------------
    md = MolecularDynamics(ff, dyn, state0)
    md_step = lambda i: md.run(1)          # noqa: E731
    for i in range(args.warmup):
        md_step(i)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    launches0 = ff.info()["launches"]
    sampler.start()
    time.sleep(0.3)
    ms_mixed, wall_mixed = timed(md_step, args.steps)
    clocks = sampler.stop()
    launches_timed = ff.info()["launches"] - launches0
    ms_mixed = max_over_ranks(ms_mixed)

    # ---- FP64 form of the same MD step -----------------------------------------
    ff.set_precision("fp64")
    md_step(0)
    ms_fp64, _ = timed(md_step, max(1, args.fp64_steps))
    ms_fp64 = max_over_ranks(ms_fp64)
    ff.set_precision("mixed")

    # ---- force evaluation alone: accuracy, phases -------------------------------
    force_step(0)
    torch.cuda.synchronize()
    f_mixed, pe_mixed = d_force.clone(), d_pe.clone()
    ms_force_mixed, _ = timed(force_step, args.steps)
    ff.set_phase_timing(True)
    phases = None
    for i in range(3):
        flush.zero_()
        force_step(i)
        ph = ff.phase_times()
        phases = ph if phases is None else {k: min(phases[k], ph[k]) for k in ph}
    ff.set_phase_timing(False)
    ff.set_precision("fp64")
    ms_force_fp64, _ = timed(force_step, max(1, args.fp64_steps))
    force_step(0)
    torch.cuda.synchronize()
    f64, pe64 = d_force.clone(), d_pe.clone()
    ferr = float(torch.sqrt(((f_mixed - f64) ** 2).sum() / (f64 ** 2).sum()).item())
    e_err = float((pe_mixed.sum() - pe64.sum()).abs().item() / pe64.sum().abs().item())
    ff.set_precision("mixed")

    # ---- NVE runs: steps/s, ns/day and energy drift ------------------------------
    nve = {}
    for prec, nsteps in (("mixed", args.nve_steps), ("fp64", args.nve_fp64_steps)):
        if nsteps <= 0:
            continue
        ff.set_precision(prec)
        run = MolecularDynamics(ff, dyn, state0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        en = run.run(nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) * 1e-3 / nsteps
        H = en.sum(1)
        ke = float(np.mean(en[:, 2] + en[:, 3]))
        half = en[nsteps // 2:]
        nve[prec] = {"steps": nsteps, "step_fs": STEP_PS * 1e3, "steps_per_s": 1.0 / sec,
                     "ns_per_day": ns_per_day(1.0 / sec, STEP_PS),
                     "drift_kjmol_per_ns_per_mol": drift_per_ns(en, STEP_PS, sysA.nmols) * CONV_E,
                     "drift_second_half_kjmol_per_ns_per_mol": drift_per_ns(half, STEP_PS, sysA.nmols) * CONV_E,
                     "H_first_last_kjmol_per_mol": [float(H[0]) * CONV_E / sysA.nmols,
                                                    float(H[-1]) * CONV_E / sysA.nmols],
                     "ke_mean_kjmol_per_mol": ke * CONV_E / sysA.nmols,
                     "timing": "one CUDA-event interval around the whole run (no L2 flush)"}
    ff.set_precision("mixed")

    # ---- end to end through the C ABI, pinned host buffers -------------------
    h_site = [torch.from_numpy(np.ascontiguousarray(s.site)).pin_memory() for s in (sysA, sysB)]
    h_force = torch.empty((3, n), dtype=torch.float64).pin_memory()
    cm = np.ascontiguousarray(sysA.c_of_m)
    L = _lib.load()
    hh = np.ascontiguousarray(sysA.h, np.float64).reshape(9)
    pe_h = np.zeros(2)
    st_h = np.zeros(9)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ff.set_stream(0)  # the context's own stream for the host-buffer calls

    def e2e_step(i):
        st = L.mdgpu_forces(ff.ctx, dp(hh), C.cast(h_site[i % 2].data_ptr(), C.POINTER(C.c_double)),
                            dp(cm), C.cast(h_force.data_ptr(), C.POINTER(C.c_double)), dp(pe_h), dp(st_h))
        if st != 0:
            raise RuntimeError(L.mdgpu_last_error(ff.ctx).decode())

    for i in range(args.warmup):
        e2e_step(i)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        e2e_step(i)
    barrier()
    force_call_s = max_over_ranks((time.perf_counter() - t0) / args.steps)

    # the MD step through the public C API with the dynamic state in pinned
    # host memory: upload the state, one step, download the state and the
    # step's energies -- every step
    md_h = MolecularDynamics(ff, dyn, state0)
    nq = md_h.nq
    h_cm = torch.from_numpy(np.ascontiguousarray(state0.c_of_m, np.float64)).pin_memory()
    h_mom = torch.from_numpy(np.ascontiguousarray(state0.mom, np.float64)).pin_memory()
    h_q = torch.from_numpy(np.ascontiguousarray(state0.quat, np.float64).reshape(-1)).pin_memory()
    h_am = torch.from_numpy(np.ascontiguousarray(state0.amom, np.float64).reshape(-1)).pin_memory()
    h_en = torch.zeros(4, dtype=torch.float64).pin_memory()
    pt = lambda t: C.cast(t.data_ptr(), C.POINTER(C.c_double))  # noqa: E731

    def md_e2e_step(i):
        for st in (L.mdgpu_md_set_state(ff.ctx, pt(h_cm), pt(h_mom), pt(h_q), pt(h_am)),
                   L.mdgpu_md_run(ff.ctx, 1, pt(h_en)),
                   L.mdgpu_md_get_state(ff.ctx, pt(h_cm), pt(h_mom), pt(h_q), pt(h_am))):
            if st != 0:
                raise RuntimeError(L.mdgpu_last_error(ff.ctx).decode())

    for i in range(args.warmup):
        md_e2e_step(i)
    barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        md_e2e_step(i)
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    state_bytes = 8 * (6 * sysA.nmols + 8 * nq)
    info = ff.info()

    # ---- roofline of the dominant kernel ---------------------------------------
    tf32 = C.c_double()
    tf64 = C.c_double()
    L.mdgpu_fma_peak(local, 0, C.byref(tf32))
    L.mdgpu_fma_peak(local, 1, C.byref(tf64))
    nk = info["nkvec"]
    # the k-space passes run over the charged sites only (units processed per launch)
    n_q = int(np.count_nonzero(sysA.chg()))
    work = {"kforce": FLOPS_FORCE_PER_SITE_K * n_q * nk, "sfac": FLOPS_SFAC_PER_SITE_K * n_q * nk,
            "pairs": FLOPS_PAIR_LJ_ERFC * info["npairs"]}
    dom = max(work, key=lambda k: phases.get(k, 0.0))
    achieved = work[dom] / (phases[dom] * 1e-3) / 1e12
    traffic = traffic_from_profiles().get(dom)
    kernel_names = {"kforce": "k_force_tc", "sfac": "k_sfac_tc", "pairs": "k_pairs_col<LJ,erfc>"}
    peaks = measured_peaks()
    mma = tc_mma_flops(sysA, n_q)
    if dom in mma:
        # tensor-core kernels: the bound is the bf16 tensor pipe (sustained,
        # as the kernel runs inside a long step); achieved counts the
        # reference's own FP32 operations, the MMA work they expand to (three
        # bf16 terms per operand, six term products, complex arithmetic as
        # real products, padded columns) is reported beside it
        peak, unit, bound = peaks["bf16_sustained"], "TFLOP/s", "tensor"
        peak_source = (f"{peaks['source']} cuBLAS bf16 GEMM throughput, sustained "
                       f"(MEASURED_PEAKS.json bf16_tflops_sustained)")
        mma_rate = mma[dom] / (phases[dom] * 1e-3) / 1e12
        mma_line = {"flops_per_launch": mma[dom], "tflops": mma_rate, "frac": mma_rate / peak,
                    "expansion": mma[dom] / work[dom]}
    else:
        peak, unit, bound = tf32.value, "TFLOP/s", "fp32"
        peak_source = "measured FP32 FMA throughput on this GPU (mdgpu_fma_peak)"
        mma_line = None

    cpu = cpu1 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        log("timing the CPU baseline (reference algorithm restated in C) ...")
        sec, det = cpu_baseline(sysA)
        cpu = {"value": 1.0 / sec, "unit": "steps/s", "cores": det["threads"], "kind": "port",
               "sample": (f"one full force evaluation, timed whole: force_calc ({det['pairs']} pairs, "
                          f"{det['t_real_s']:.2f} s) + ewald over all {det['nkvec']} k-vectors "
                          f"({det['t_ewald_s']:.2f} s); -O2 -ffast-math, {det['threads']} threads; the "
                          f"reference's integrator (under 1% of its step) not timed")}
        if args.cpu_1core:
            sec1, det1 = cpu_baseline(sysA, threads=1)
            cpu1 = {"value": 1.0 / sec1, "unit": "steps/s", "cores": 1, "kind": "port",
                    "sample": (f"one full force evaluation on one core, timed whole: force_calc "
                               f"{det1['t_real_s']:.2f} s + ewald {det1['t_ewald_s']:.2f} s")}

    value = world * 1e3 / ms_mixed
    line = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (f64 accumulation; f64 integrator)",
        "data": "synthetic (seeded lattice water, uniform random orientations, 300 K Maxwell-Boltzmann)",
        "config": bench_config(world),
        "step": ("one constant-energy MD step on the GPU (half drift, sites, forces, molecular "
                 "forces/torques, kicks, half drift), dt = 1 fs"),
        "timing": {"l2": "flushed between timed steps (256 MiB write)", "events": "per-step CUDA events "
                   "on the launching stream, summed"},
        "workload_stats": {"nsites": n, "nkvec": nk, "pairs_last_evaluation": info["npairs"]},
        "fp64": {"value": world * 1e3 / ms_fp64, "unit": "steps/s", "ms_per_step": ms_fp64,
                 "steps": max(1, args.fp64_steps)},
        "mixed_over_fp64": ms_fp64 / ms_mixed,
        "force_eval": {"ms_mixed": ms_force_mixed, "ms_fp64": ms_force_fp64,
                       "mixed_over_fp64": ms_force_fp64 / ms_force_mixed},
        "accuracy": {"force_rel_rms_mixed_vs_fp64": ferr, "energy_rel_mixed_vs_fp64": e_err},
        "nve": nve,
        "e2e": {"value": world / e2e_s, "unit": "steps/s", "h2d_bytes_per_step": state_bytes,
                "d2h_bytes_per_step": state_bytes + 4 * 8,
                "path": "mdgpu_md_set_state + mdgpu_md_run(1) + mdgpu_md_get_state on pinned host "
                        "arrays each step (centres of mass, momenta, quaternions, angular momenta)"},
        "e2e_force_call": {"value": world / force_call_s, "unit": "force evaluations/s",
                           "h2d_bytes_per_step": 3 * n * 8, "d2h_bytes_per_step": 3 * n * 8 + 11 * 8 + 512,
                           "path": "mdgpu_forces (the drop-in force call of a host integrator) on pinned "
                                   "host arrays each step"},
        "gpu_launches": int(launches_timed),
        "phases_ms": phases,
        "roofline": {"kernel": kernel_names[dom], "bound": bound, "achieved": achieved,
                     "work": ({"kforce": f"{FLOPS_FORCE_PER_SITE_K} flops per (charged site, k): "
                                         f"{n_q} sites x {nk} k",
                               "sfac": f"{FLOPS_SFAC_PER_SITE_K} flops per (charged site, k): "
                                       f"{n_q} sites x {nk} k",
                               "pairs": f"{FLOPS_PAIR_LJ_ERFC} flops per evaluated pair"}[dom]),
                     "peak": peak, "unit": unit, "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_source, "mma": mma_line,
                     "fp32_fma_peak": tf32.value, "fp64_fma_peak": tf64.value},
        "cpu_baseline": cpu,
        "cpu_baseline_1core": cpu1,
        "clocks": clocks,
        "wall_s_mixed_timed": wall_mixed,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ff.close()
    if dist is not None:
        dist.destroy_process_group()


def run_adjoint(args):
    """Force-matching gradients on the adjoint workload: rigid water, 4096
    molecules (16,384 sites), a batch of seeded frames; epsilon, sigma and
    q_H scaled by seeded factors in [0.9, 1.1] (q_M = -2 q_H); reference
    forces at the original parameters.  Times the loss + gradient over the
    batch (torch autograd over the C ABI) in both forms and checks the
    gradient with respect to (epsilon, sigma, q_H, alpha) against central
    finite differences of the FP64 C restatement on all host cores."""
    import torch
    from moldy_gb300 import system as S
    from moldy_gb300.fitting import FitProblem, ForceMatchLoss, water_frames, water_tables
    from moldy_gb300.forcefield import ForceField
    from oracle import port
    import dataclasses

    base = S.water(nside=16, seed=21)
    frames = water_frames(base, args.adjoint_frames, seed=22)
    theta0 = np.array([0.6485, 3.154, 0.52, base.control.alpha])
    theta = theta0 * np.append(np.random.default_rng(23).uniform(0.9, 1.1, 3), 1.0)
    threads = os.cpu_count() or 1

    def sys_at(t, fr):
        pot, _ = water_tables(*[torch.tensor(v, dtype=torch.float64) for v in t[:3]], base)
        qid = np.zeros(base.max_id)
        qid[2], qid[3] = t[2] / S.CONV_Q, -2 * t[2] / S.CONV_Q
        return dataclasses.replace(fr, potpar=pot.numpy(), site_charge=qid,
                                   control=dataclasses.replace(base.control, alpha=float(t[3])))

    def port_forces(sysm):
        return port.force_calc(sysm, nthreads=threads, fast=False).force + \
            port.ewald(sysm, nthreads=threads, fast=False).force

    t0 = time.perf_counter()
    f_refs = [port_forces(sys_at(theta0, fr)) for fr in frames]
    w = 1.0 / (len(frames) * f_refs[0].size)

    def oracle_loss(t):
        return sum(w * float(np.sum((port_forces(sys_at(t, fr)) - f) ** 2)) for fr, f in zip(frames, f_refs))

    fd = np.zeros(4)
    for k in range(4):
        h = 1e-5 * theta[k]
        tp, tm = theta.copy(), theta.copy()
        tp[k] += h
        tm[k] -= h
        fd[k] = (oracle_loss(tp) - oracle_loss(tm)) / (2 * h)
    t_fd = time.perf_counter() - t0
    out = {"metric": "force-matching loss gradient, water 16,384 sites", "unit": "s per batch",
           "frames": len(frames), "theta": theta.tolist(), "fd_grad": fd.tolist(),
           "fd": f"central, step 1e-5 relative, FP64 C restatement on {threads} threads ({t_fd:.0f} s)"}
    for prec in ("mixed", "fp64"):
        ff = ForceField(sys_at(theta, frames[0]), precision=prec)
        pb = FitProblem(ff, [f.site for f in frames], [f.c_of_m for f in frames], f_refs, w)
        res = None
        for rep in range(2):   # the first pass uploads tables and builds the k-list
            t = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in theta]
            pot, chg = water_tables(t[0], t[1], t[2], base)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            L = ForceMatchLoss.apply(pot, chg, t[3], pb)
            t2 = time.perf_counter()
            L.backward()
            torch.cuda.synchronize()
            t3 = time.perf_counter()
            g = np.array([float(x.grad) for x in t])
            res = {"loss": L.item(), "grad": g.tolist(), "rel_err_vs_fd": (np.abs(g - fd) / np.abs(fd)).tolist(),
                   "s_forward": t2 - t1, "s_backward": t3 - t2,
                   "ms_per_frame_loss_and_grad": 1e3 * (t3 - t1) / len(frames)}
        out[prec] = res
        ff.close()
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--fp64-steps", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-1core", type=int, default=1,
                    help="also time one full force evaluation on one host core (0: skip)")
    ap.add_argument("--nve-steps", type=int, default=10000,
                    help="mixed-form constant-energy run for ns/day and drift (0: skip)")
    ap.add_argument("--nve-fp64-steps", type=int, default=300,
                    help="FP64-form constant-energy run (0: skip)")
    ap.add_argument("--adjoint", action="store_true",
                    help="run the force-matching gradient workload instead (prints its own JSON line)")
    ap.add_argument("--adjoint-frames", type=int, default=64)
    ap.add_argument("--profile-case", choices=["mixed", "fp64"],
                    help="run three untimed evaluations of the workload and exit (for ncu captures)")
    ap.add_argument("--profile-nside", type=int, default=32,
                    help="molecules per cell edge of the profile case (32: the benchmark workload; "
                         "16: 16,384 sites, for captures of many passes)")
    args = ap.parse_args()
    if args.profile_case:
        from moldy_gb300.forcefield import ForceField
        from moldy_gb300 import system as S
        sysm = make_workload() if args.profile_nside == 32 else S.water(nside=args.profile_nside, seed=7,
                                                                           alpha=0.3, cutoff=9.0)
        ff = ForceField(sysm, precision=args.profile_case)
        for _ in range(3):
            _, pe, _ = ff.forces()
        log("profile case done", pe)
        return
    if args.adjoint:
        run_adjoint(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
