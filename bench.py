"""Benchmark of the D2Q9 collide-stream step on GB300.

Workload (the configuration the headline metric is quoted on): lid-driven
cavity, 1024 x 1024, MRT (the reference's rate set), lid u = 0.1 as a
half-way moving wall, half-way bounce-back on the other walls, Re = 1000
(nu = u L / Re with L = NY, src/main.cu:66), rho = 1 and u = 0 initially.

  value     MLUPS of the fused step kernel, FP32 storage, inputs resident in
            HBM; every timed step is preceded by an L2 flush (a 256 MB write,
            then a 256 MB read of a second buffer) -- the 1024^2 lattice,
            38 MB per population set, would otherwise stay in the 129 MB L2.
  e2e       the same metric through the C-ABI with host buffers: fields
            uploaded from pinned host memory, 1000 LBM steps by one
            lbmx_step_sums call that reduces the FP64 mass/momentum sums in
            every step's kernel and copies each step's sums to pinned host
            memory without stalling the GPU (the reference copies its moment
            averages back with a blocking copy every step,
            macroscopics.cuh:177), final density and velocity read back.
  variants  FP16 / BF16 offset storage on the same workload, each with the
            relative L2 velocity error against the FP64 oracle after 200
            steps.
  hbm_bound the same kernel on an 8192 x 8192 cavity (2.4 GB per population
            set, far above L2) for the roofline fraction without a flush.
  ensemble  the batched-ensemble workload: 512 lid-driven cavities of
            uneven sizes and Reynolds numbers in one persistent launch per
            step (CUDA graphs, autotuned tile shape), aggregate MLUPS for
            FP16-offset and FP32 storage and the per-instance L2 velocity
            error against the FP64 oracle of one instance per side class.
  adjoint   the discrete adjoint on the Brinkman channel (4096 x 1024,
            5000 steps, checkpoint every 250): forward and backward times,
            the gradients of the outlet mass flux, and a bounded check
            against FP64 central differences of the oracle.
  validation  the Taylor-Green vortex (256^2, 2000 steps) against its
            analytic decay, and the IBM cylinder channel (2048 x 512, Re 100)
            run 200k steps from rest in FP32 and FP16 offset storage: MLUPS,
            mean C_D, C_L amplitude and Strouhal number of the shedding state
            from every step's drag and lift.
  cpu_baseline  the FP64 CPU oracle (OpenMP, all host cores) on the same
            workload, 200 steps.

`--impl reference` times the CPU implementation of the reference step (the
oracle port; the reference itself has no CPU path) on this workload.
Under torchrun each rank advances its own lattice replica (the path needs no
collective on one lattice per GPU); value is the sum over ranks with the
maximum per-rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(REPO, "cuda-lbm_gb300"), os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

def metric_name(n, storage=0):
    """The metric of a lid-driven cavity run on n x n nodes (the default run:
    1024 x 1024, FP32 storage)."""
    return "MLUPS (D2Q9 lid-driven cavity %dx%d MRT, %s storage)" % (n, n, ("FP32", "FP16-offset", "BF16-offset")[storage])
BYTES_PER_LU = {0: 72, 1: 36, 2: 36}
STORAGE_NAME = {0: "f32", 1: "f16_offset", 2: "bf16_offset"}


def cavity_case(n, storage=0):
    import cases as C
    nu = 0.1 * n / 1000.0
    return C.cavity_moving_wall(n, n, op=C.MRT, nu=nu, u_lid=0.1)


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            return json.load(fh), "measured"
    return {"hbm_gbs": 6800.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


class L2Flush:
    """Evicts the lattice from L2 between timed steps: a 256 MB write (twice
    the 129 MB L2), then a 256 MB read of a second buffer, so L2 holds only
    clean, unrelated lines when the step starts (the step then pays neither
    for its own data being cached nor for writing back the flush's)."""

    def __init__(self, torch):
        self.w = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
        self.r = torch.ones(64 << 20, dtype=torch.float32, device="cuda")
        self.acc = torch.zeros(1, dtype=torch.float32, device="cuda")

    def __call__(self):
        self.w.zero_()
        self.acc.add_(self.r.sum())


def time_steps(L, torch, stream, steps, warmup, flush):
    """Per-step CUDA-event time (ms) of `steps` single LBM steps, each after an L2 flush."""
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            if flush is not None:
                flush()
            L.step(1, flags=0)
        stream.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for s, e in evs:
            if flush is not None:
                flush()
            s.record(stream)
            L.step(1, flags=0)
            e.record(stream)
        stream.synchronize()
    return np.array([s.elapsed_time(e) for s, e in evs])


def max_over_ranks(value, dist, device):
    """The slowest rank's per-step time (every rank runs its own replica)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_mlups(nodes_per_rank, ms_per_step, world):
    """Whole-job throughput: all ranks' lattice updates over the slowest rank's time."""
    return world * nodes_per_rank / (ms_per_step * 1e-3) / 1e6


def l2_error(u, uref):
    return float(np.sqrt(((u - uref) ** 2).sum() / (uref ** 2).sum()))


def run_cpu_oracle(n, steps, threads):
    import cases as C
    o = C.make_oracle(cavity_case(n))
    o.step(1)
    t0 = time.perf_counter()
    o.step(steps - 1)
    dt = time.perf_counter() - t0
    _, u, _ = o.moments()
    return u, (n * n * (steps - 1)) / dt / 1e6, dt


STEADY_RESIDUAL = 1e-5  # relative L2 change of u over 1000 steps; FP32's own floor is 6-7e-6


def bench_steady(args, torch, stream, device):
    """The cavity run to steady state in FP32, FP16 and BF16 offset storage.

    Steady means a relative L2 change of the velocity field over the last
    1000 steps of at most STEADY_RESIDUAL (1e-5): an FP32 run settles at a
    floor of 6-7e-6 set by its own rounding and stays there (checked out to
    3M steps at 256^2 and 1024^2).  At 1024^2 the FP32 run goes 1000 steps at
    a time until it is steady (at most args.steady_max_steps); the 16-bit
    forms then run the same number of steps and report their relative L2
    velocity error against FP32 and their own residual; MLUPS counts the
    stepping only.  At 256^2 all three forms run to the step count of the
    committed FP64 oracle field (tests/golden/steady_cavity256_mrt.npz, made
    by tests/golden/make_steady_cavity.py and steady to 1e-6) and report
    their error against it."""
    import lbmx

    def lattice(n, storage):
        c = cavity_case(n)
        L = lbmx.Lattice(n, n, op=c["op"], omega=c["omega"], S=c["S"], storage=storage, wall_u=c["wall_u"],
                         device=device, stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.ones((n, n), np.float32), np.zeros((2, n, n), np.float32))
        return L

    def run(n, storage, max_steps, until_steady):
        L = lattice(n, storage)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ms, steps, res, u = 0.0, 0, None, None
        while steps < max_steps:
            k = min(1000, max_steps - steps)
            e0.record(stream)
            L.step(k)
            e1.record(stream)
            _, un, _ = L.moments()
            ms += e0.elapsed_time(e1)
            steps += k
            if u is not None and k == 1000:
                res = l2_error(un, u)
            u = un
            if until_steady and res is not None and res <= STEADY_RESIDUAL:
                break
        return u, res, steps, n * n * steps / (ms * 1e-3) / 1e6

    n = args.size
    out = {"criterion": "relative L2 change of u over the last 1000 steps <= %g" % STEADY_RESIDUAL}
    u32, res32, steps, m32 = run(n, 0, args.steady_max_steps, True)
    big = {"workload": "lid-driven cavity %dx%d MRT, lid 0.1, Re 1000, from rest to steady state" % (n, n),
           "steps": steps, "steady": bool(res32 is not None and res32 <= STEADY_RESIDUAL),
           "f32": {"residual_last_1000_steps": res32, "MLUPS_sustained": round(m32, 1)}}
    for storage in (1, 2):
        u, res, _, m = run(n, storage, steps, False)
        big[STORAGE_NAME[storage]] = {"l2_u_err_vs_f32": l2_error(u, u32), "residual_last_1000_steps": res,
                                      "MLUPS_sustained": round(m, 1)}
    out["cavity%d" % n] = big
    g = np.load(os.path.join(REPO, "tests", "golden", "steady_cavity256_mrt.npz"))
    meta = json.loads(str(g["meta"]))
    sub = meta["subsample"]
    small = {"workload": "lid-driven cavity 256x256 MRT, lid 0.1, Re 1000, %d steps from rest, against the FP64 "
                         "oracle's field of the same step (residual %.1e)"
                         % (meta["steps"], meta["residual_last_1000_steps"]), "steps": meta["steps"]}
    for storage in (0, 1, 2):
        u, res, _, _ = run(256, storage, meta["steps"], False)
        small[STORAGE_NAME[storage]] = {"l2_u_err_vs_fp64": l2_error(u[:, ::sub, ::sub], g["u"]),
                                        "residual_last_1000_steps": res}
    out["fp64_256"] = small
    return out


def bench_ensemble(args, torch, stream, device, hbm):
    """Batched ensemble: `args.ens_count` lid-driven cavities (sides uniform in
    {64, ..., 768}, Re log-uniform in [100, 5000], seed 0), D2Q9 MRT, advanced
    by one persistent launch per step replayed from CUDA graphs, tile shape
    from the autotuner.  Aggregate MLUPS for FP16-offset and FP32 storage,
    and the relative L2 velocity error against the FP64 oracle of the first
    instance of every side class, 23 in all (a lattice's result does not
    depend on the batch it runs in: the batched kernel is bit-identical to
    stepping it alone)."""
    import cases as C
    import lbmx
    ens = C.ensemble(count=args.ens_count)
    nodes = sum(s * s for s, _, _ in ens)

    def build(storage, members):
        Ls = []
        for side, _, nu in members:
            c = C.ensemble_cavity(side, nu)
            L = lbmx.Lattice(side, side, op=c["op"], omega=c["omega"], S=c["S"], storage=storage,
                             wall_u=c["wall_u"], device=device, stream=stream.cuda_stream)
            L.set_flags(c["flags"])
            L.init(np.ones((side, side), np.float32), np.zeros((2, side, side), np.float32))
            Ls.append(L)
        return Ls

    out = {"workload": "%d lid-driven cavities, sides uniform in {64,96,...,768}, Re log-uniform [100,5000], "
                       "seed 0, D2Q9 MRT, lid 0.1" % len(ens), "nodes": int(nodes)}
    for storage in (1, 0):
        Ls = build(storage, ens)
        B = lbmx.Batch(Ls)
        cfg = B.autotune(trial_steps=4)
        B.step(max(args.warmup, 3) * 2, flags=0)
        B.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        B.step(args.ens_steps, flags=0)
        e1.record(stream)
        B.step(1, flags=lbmx.STEP_STORE_MOMENTS)
        B.synchronize()
        ms = e0.elapsed_time(e1) / args.ens_steps
        bad = 0
        for L in Ls:
            r, _, _ = L.moments()
            bad += int(not np.isfinite(r).all())
        a = BYTES_PER_LU[storage] * nodes / (ms * 1e-3) / 1e9
        out[STORAGE_NAME[storage]] = {"MLUPS": round(nodes / (ms * 1e-3) / 1e6, 1), "ms_per_step": round(ms, 4),
                                      "achieved_GBs": round(a, 1), "frac": round(a / hbm, 4),
                                      "autotuned": cfg, "nonfinite_instances": bad,
                                      "timed_steps": args.ens_steps}
        B.close()
        del Ls, B
    out["f16_speedup_vs_f32"] = round(out["f16_offset"]["MLUPS"] / out["f32"]["MLUPS"], 3)
    # per-instance error against the FP64 oracle: the first instance of
    # every side class in the ensemble (64, 96, ..., 768)
    sample = []
    for side in sorted({e[0] for e in ens}):
        sample.append(min(i for i in range(len(ens)) if ens[i][0] == side))
    members = [ens[i] for i in sample]
    Ls = build(1, members)
    B = lbmx.Batch(Ls)
    B.step(args.ens_err_steps)
    errs = []
    for (side, re, nu), L in zip(members, Ls):
        o = C.make_oracle(C.ensemble_cavity(side, nu))
        o.step(args.ens_err_steps)
        _, uo, _ = o.moments()
        _, ul, _ = L.moments()
        errs.append({"instance": sample[len(errs)], "side": side, "Re": round(re, 1),
                     "l2_u_err_vs_fp64": l2_error(ul, uo)})
    out["l2_err_sample"] = {"storage": "f16_offset", "steps": args.ens_err_steps,
                            "sample": "the first instance of every side class", "instances": errs,
                            "max": max(e["l2_u_err_vs_fp64"] for e in errs)}
    return out


def bench_validation(args, torch, stream, device):
    """The two remaining configurations as validation lines.

    Taylor-Green vortex: 256 x 256, fully periodic, BGK, nu 0.01, u0 0.04,
    2000 steps, velocity amplitude against exp(-2 nu k^2 t) (the lattice,
    4.7 MB, stays in L2).  Flow past a cylinder: the shedding run of
    bench_cylinder_shedding, then the drag sensitivity of the same
    configuration."""
    import cases as C
    import lbmx

    def lattice(c, storage=0):
        L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                         storage=storage, u_bc=c["u_bc"], device=device, stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32))
        if c["markers"] is not None:
            L.set_markers(c["markers"])
        return L

    def timed(L, steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.step(steps)
        e1.record(stream)
        stream.synchronize()
        return e0.elapsed_time(e1)

    out = {}
    n, nu, u0, T = 256, 0.01, 0.04, 2000
    c = C.taylor_green(n, n, op=C.BGK, nu=nu, u0=u0)
    L = lattice(c)
    ms = timed(L, T)
    _, u, _ = L.moments()
    u_init = np.asarray(c["u"], np.float64)
    amp = float((u * u_init).sum() / (u_init * u_init).sum())
    k = 2 * np.pi / n
    exact = float(np.exp(-2 * nu * k * k * T))
    out["taylor_green"] = {"workload": "Taylor-Green 256x256 BGK nu 0.01 u0 0.04, %d steps, L2-resident" % T,
                           "amplitude": amp, "analytic": exact, "rel_err": abs(amp - exact) / exact,
                           "MLUPS": round(n * n * T / (ms * 1e-3) / 1e6, 1)}
    del L
    out["cylinder_shedding"] = bench_cylinder_shedding(args, torch, stream, device, lattice)
    out["drag_sensitivity"] = bench_drag_sensitivity(args, torch, stream, device)
    return out


def spectral_peak(x):
    """Frequency (cycles per step) of the largest spectral peak of x, from a
    Hann-windowed FFT refined by a parabola through the log magnitudes of
    the peak bin and its neighbours (the lowest bins, the mean's leakage,
    are skipped)."""
    x = np.asarray(x, np.float64) - np.mean(x)
    F = np.abs(np.fft.rfft(x * np.hanning(len(x))))
    k = int(np.argmax(F[4:-1])) + 4
    a, b, c = np.log(F[k - 1:k + 2] + 1e-300)
    d = 0.5 * (a - c) / (a - 2 * b + c) if a - 2 * b + c != 0 else 0.0
    return (k + d) / len(x)


def shedding_stats(series, q, D, U):
    """Force coefficients of the last half of a {drag, lift} series: mean
    C_D; the C_L amplitude as sqrt(2) x its RMS about the mean; the Strouhal
    number f D / U from the lift's spectral peak; the drag's own dominant
    period and RMS (on this channel, the quarter-wave acoustic mode between
    the velocity inlet and the pressure outlet, 4 L / c_s = 14,190 steps for
    L = 2048, rather than twice the shedding frequency); and how much the
    lift RMS changed between the third and last quarters."""
    T = series.shape[0]
    cd = series[:, 0] / q
    cl = series[:, 1] / q
    hd, hl = cd[T // 2:], cl[T // 2:]
    f_l = spectral_peak(hl)
    f_d = spectral_peak(hd)
    r3, r4 = float(np.std(cl[T // 2: 3 * T // 4])), float(np.std(cl[3 * T // 4:]))
    return {"C_D_mean": float(hd.mean()), "C_D_rms": float(hd.std()), "C_D_period_steps": round(1.0 / f_d, 1),
            "C_L_amplitude": float(np.sqrt(2) * hl.std()), "C_L_mean": float(hl.mean()),
            "strouhal": float(f_l * D / U), "shedding_period_steps": round(1.0 / f_l, 1),
            "C_L_rms_change_q3_to_q4": (r4 - r3) / r3 if r3 > 0 else None}


def bench_cylinder_shedding(args, torch, stream, device, lattice):
    """Flow past a cylinder (the C4 configuration): 2048 x 512, Zou-He
    parabolic inlet (peak U = 0.05), Zou-He pressure outlet, bounce-back walls,
    cylinder D = 64 at (256, 256) (half a node above the channel's centre
    line) as 256 IBM markers (multi-direct forcing, 4-point Peskin kernel), Re
    100 on D and U, BGK, from rest for `args.cyl_steps` steps in FP32 and FP16
    offset storage.  Every step's drag and lift are recorded by the IBM kernel
    itself (lbmx_step_forces into pinned host memory); C_D, C_L = force / (1/2
    rho U^2 D) with rho = 1; Strouhal = f D / U.  MLUPS over the whole run."""
    import cases as C

    nx, ny, D, U, T = 2048, 512, 64, 0.05, args.cyl_steps
    markers = C.cylinder_markers(256, 256, D / 2, 256)
    q = 0.5 * 1.0 * U * U * D
    res = {}
    for storage in (0, 1):
        c = C.channel(nx, ny, op=C.BGK, nu=U * D / 100.0, u_in=U, inlet="parabolic", outlet="zouhe_p",
                      markers=markers)
        L = lattice(c, storage)
        series = torch.zeros(2 * T, dtype=torch.float64).pin_memory()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.step_forces(T, out=series)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1)
        sr = series.numpy().reshape(T, 2).copy()
        st = shedding_stats(sr, q, D, U)
        st["MLUPS"] = round(nx * ny * T / (ms * 1e-3) / 1e6, 1)
        st["us_per_step"] = round(ms * 1e3 / T, 2)
        st["finite"] = bool(np.isfinite(sr).all())
        res[STORAGE_NAME[storage]] = st
        del L

    def rel(k):
        a, b = res["f16_offset"][k], res["f32"][k]
        return None if a is None or b is None or b == 0 else abs(a - b) / abs(b)

    res["f16_vs_f32"] = {"C_D_mean_rel_diff": rel("C_D_mean"), "C_L_amplitude_rel_diff": rel("C_L_amplitude"),
                         "strouhal_rel_diff": rel("strouhal")}
    res["strouhal_convention"] = "f D / U with U the peak inlet velocity (the Reynolds number's velocity)"
    res["workload"] = ("cylinder 2048x512, D 64 at (256,256), 256 IBM markers, BGK, Re 100 on D and the peak inlet "
                       "velocity 0.05, Zou-He parabolic inlet, Zou-He pressure outlet, %d steps from rest; statistics "
                       "over the last half" % T)
    res["steps"] = T
    return res


def bench_drag_sensitivity(args, torch, stream, device):
    """d(mean drag)/d(inlet velocity) of the cylinder configuration by the
    tangent-linear model (lbmx_tangent_*), over steps T/2+1..T from rest.
    Checked two ways: against a central difference (h = 1% of the inlet
    velocity) of the engine's own FP32 drag series at full size, and on a
    112 x 44 channel (cylinder D 12, 36 markers, 400 steps) against central
    differences of the FP64 oracle."""
    import cases as C
    import lbmx

    nx, ny, D, U, T = 2048, 512, 64, 0.05, args.sens_steps
    half = T // 2
    mk = C.cylinder_markers(256, 256, D / 2, 256)

    def case(u):
        return C.channel(nx, ny, op=C.BGK, nu=U * D / 100.0, u_in=u, inlet="parabolic", outlet="zouhe_p", markers=mk)

    c = case(U)
    t = lbmx.Tangent(nx, ny, lbmx.TANGENT_U_BC, op=c["op"], omega=c["omega"], S=c["S"], flags=c["flags"], u_bc=U,
                     device=device, stream=stream.cuda_stream)
    t.set_state(np.ones((ny, nx), np.float32), np.zeros((2, ny, nx), np.float32))
    t.set_markers(mk)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s = t.run(T)
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1)
    del t
    deriv = float(s[half:, 2].mean())

    def engine_mean_drag(u):
        L = lbmx.Lattice(nx, ny, op=c["op"], omega=c["omega"], S=c["S"], u_bc=u, device=device,
                         stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.ones((ny, nx), np.float32), np.zeros((2, ny, nx), np.float32))
        L.set_markers(mk)
        L.step(half)
        return float(L.step_forces(T - half)[:, 0].mean())

    h = 0.01 * U
    fd = (engine_mean_drag(U + h) - engine_mean_drag(U - h)) / (2 * h)

    # bounded FP64 check
    import oracle as O
    mk_s = C.cylinder_markers(30.3, 21.7, 6.0, 36)
    cs = C.channel(112, 44, op=C.BGK, nu=0.04, u_in=0.05, inlet="parabolic", outlet="zouhe_p", markers=mk_s)
    ts = lbmx.Tangent(112, 44, lbmx.TANGENT_U_BC, op=cs["op"], omega=cs["omega"], S=cs["S"], flags=cs["flags"],
                      u_bc=0.05, device=device, stream=stream.cuda_stream)
    ts.set_state(np.ones((44, 112), np.float32), np.zeros((2, 44, 112), np.float32))
    ts.set_markers(mk_s)
    ss = ts.run(400)
    del ts

    def oracle_mean_drag(u):
        o = O.Oracle(112, 44, op=cs["op"], omega=cs["omega"], S=cs["S"], u_bc=u, precision="f64")
        o.set_flags(cs["flags"])
        o.init(cs["rho"], cs["u"])
        o.set_markers(mk_s)
        d = []
        for k in range(400):
            o.step(1)
            if k >= 200:
                d.append(-o.markers()[2][0].sum())
        return float(np.mean(d))

    hs = 1e-4
    fd64 = (oracle_mean_drag(0.05 + hs) - oracle_mean_drag(0.05 - hs)) / (2 * hs)
    d_small = float(ss[200:, 2].mean())
    return {"workload": "cylinder 2048x512 as above, BGK, %d steps from rest; J = mean drag over steps %d..%d"
                        % (T, half + 1, T),
            "parameter": "inlet peak velocity u_in = 0.05",
            "method": "tangent-linear (forward mode) through the engine's per-node code and IBM rounds",
            "mean_drag": float(s[half:, 0].mean()), "d_mean_drag_d_u_in": deriv,
            "d_mean_lift_d_u_in": float(s[half:, 3].mean()),
            "engine_fp32_central_fd_h_1pct": fd, "rel_diff_vs_engine_fd": abs(deriv - fd) / abs(fd),
            "tangent_ms": round(ms, 2), "tangent_MLUPS": round(nx * ny * T / (ms * 1e-3) / 1e6, 1),
            "fp64_check": {"workload": "channel 112x44, cylinder D 12 at (30.3, 21.7), 36 markers, 400 steps, "
                                       "J = mean drag over steps 201..400, FP64 oracle central difference h = 1e-4",
                           "tangent": d_small, "fp64_fd": fd64, "rel_err": abs(d_small - fd64) / abs(fd64)}}


def bench_adjoint(args, torch, stream, device):
    """Adjoint of the outlet mass flux (time average over the run) of the
    body-force Brinkman channel: 4096 x 1024, periodic x, half-way bounce-back
    walls, nu 0.02, F_x = 8 nu u_max / ny^2 for u_max 0.05, per-node solid
    fraction gamma in [0, 1] (splitmix64 normal noise, Gaussian blur sigma 16,
    min-max), 5000 steps with a checkpoint every 250, FP32.  CM<NoAdapter>:
    CM<OptimalAdapter> diverges on this flow (the adapter's rate runs away
    once the drag has damped |u| to ~1e-5; the FP64 oracle's run goes
    non-finite near step 110), which the line records.  A bounded check runs
    the same flow at 256 x 64 for 400 steps against FP64 central differences
    of the oracle."""
    import cases as C
    import lbmx
    nx, ny, T, K = args.adj_nx, args.adj_ny, args.adj_steps, args.adj_every

    def build(op, nx_, ny_, every, sigma):
        c = C.channel_brinkman(nx_, ny_, op=op, nu=0.02, u_max=0.05, sigma=sigma, gamma_scale=1.0, seed=0)
        fx = float(c["force"][0].flat[0])
        a = lbmx.Adjoint(nx_, ny_, op=op, omega=c["omega"], S=c["S"], periodic=c["periodic"], flags=c["flags"],
                         checkpoint_every=every, body_force=(fx, 0.0), device=device, stream=stream.cuda_stream)
        a.set_state(np.ones((ny_, nx_), np.float32), np.zeros((2, ny_, nx_), np.float32))
        a.set_gamma(c["gamma"])
        return c, a

    def flux_weights(nx_, ny_, steps):
        w = np.zeros((3, ny_, nx_), np.float32)
        w[1, :, nx_ - 1] = 1.0 / steps
        return w

    c, a = build(C.CM, nx, ny, K, 16.0)
    a.set_objective(flux_weights(nx, ny, T), 1)
    e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    e[0].record(stream)
    J = a.forward(T)
    e[1].record(stream)
    g_gamma, (g_om, g_fx, g_fy) = a.backward()
    e[2].record(stream)
    stream.synchronize()
    fwd_ms, bwd_ms = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
    out = {"workload": "Brinkman channel %dx%d, D2Q9 CM, periodic x, half-way walls, nu 0.02, u_max 0.05, "
                       "gamma in [0,1] (sigma 16), outlet mass flux averaged over %d steps" % (nx, ny, T),
           "steps": T, "checkpoint_every": K, "J": J, "forward_s": round(fwd_ms / 1e3, 3),
           "backward_s": round(bwd_ms / 1e3, 3),
           "backward_MLUPS": round(nx * ny * T / (bwd_ms * 1e-3) / 1e6, 1),
           "dJ_domega": g_om, "dJ_dFx": g_fx, "dJ_dFy": g_fy,
           "dJ_dgamma": {"l2": float(np.sqrt((g_gamma.astype(np.float64) ** 2).sum())),
                         "min": float(g_gamma.min()), "max": float(g_gamma.max()),
                         "finite": bool(np.isfinite(g_gamma).all())},
           "device_memory_GB": round((9 * nx * ny * 4 * ((T + K - 1) // K + K + 1 + 5)) / 1e9, 2)}
    del a
    c_opt, a_opt = build(C.CM_OPT, nx, ny, K, 16.0)
    a_opt.set_objective(flux_weights(nx, ny, T), 1)
    J_opt = a_opt.forward(T)
    out["cm_opt"] = {"J": J_opt if np.isfinite(J_opt) else None, "finite": bool(np.isfinite(J_opt))}
    del a_opt
    # bounded FP64 central-difference check
    import oracle as O
    snx, sny, sT = 256, 64, 400
    cs, a = build(C.CM, snx, sny, 50, 4.0)
    w = flux_weights(snx, sny, sT)
    a.set_objective(w, 1)
    a.forward(sT)
    gg, (gw, gfx, _) = a.backward()
    om, fx = cs["omega"], float(cs["force"][0].flat[0])
    gam = cs["gamma"].astype(np.float64)

    def J64(gamma, omega, force_x):
        o = O.Oracle(snx, sny, op=C.CM, omega=omega, S=C.S_for(C.CM, omega), periodic=(True, False),
                     precision="f64", threads=os.cpu_count() or 1)
        o.set_flags(cs["flags"])
        o.set_gamma(gamma)
        F = np.zeros((2, sny, snx))
        F[0] = force_x
        o.init(np.ones((sny, snx)), np.zeros((2, sny, snx)), F)
        acc = 0.0
        for _ in range(sT):
            o.step(1)
            r, u, _ = o.moments()
            acc += float((w[1] * r * u[0]).sum())
        return acc

    d = C.brinkman_field(snx, sny, sigma=3.0, seed=7).astype(np.float64) - 0.5
    fd_om = (J64(gam, om + 1e-4, fx) - J64(gam, om - 1e-4, fx)) / 2e-4
    fd_fx = (J64(gam, om, fx * (1 + 1e-3)) - J64(gam, om, fx * (1 - 1e-3))) / (2e-3 * fx)
    fd_g = (J64(gam + 1e-6 * d, om, fx) - J64(gam - 1e-6 * d, om, fx)) / 2e-6
    ad_g = float((gg.astype(np.float64) * d).sum())
    rel = lambda x, y: abs(x - y) / max(abs(y), 1e-300)
    out["fd_check"] = {"workload": "same flow, %dx%d, %d steps" % (snx, sny, sT), "reference": "FP64 oracle",
                       "rel_err_omega": rel(gw, fd_om), "rel_err_Fx": rel(gfx, fd_fx),
                       "rel_err_gamma_direction": rel(ad_g, fd_g)}
    return out


def bench_config(n, world):
    """The config dict of the headline workload, shared by both arms."""
    return {"workload": "lid-driven cavity %dx%d, D2Q9 MRT, lid 0.1 half-way moving wall, Re 1000" % (n, n),
            "nodes": n * n,
            "l2": "GPU arm: flushed before every timed step (256 MB write, then 256 MB read of a second buffer); "
                  "CPU arm: FP64 populations (%d MB) stream from DRAM" % (2 * 9 * 8 * n * n // 2 ** 20),
            "parallelism": "replica per GPU" if world > 1 else "single GPU"}


def bench_reference_gpu(args, torch, stream, device):
    """The reference's own CUDA step on this GPU, beside lbmx on the same
    configuration: the 1024^2 MRT lid-driven cavity with the reference's
    regularized walls and lid (nu 0.1024, Re 1000) and the 256^2 BGK
    Taylor-Green vortex, both run back to back (no L2 flush), CUDA events
    over 1000 steps after 50 warm-up steps on each side.  The reference
    binaries are built by oracle/ref_build.sh timers (from the recipe's copy
    of the reference sources) and run the call sequence of its main loop
    (src/main.cu:96-114)."""
    import cases as C
    import lbmx

    out = {}
    cfgs = {"cavity1024_mrt": C.cavity_regularized(1024, 1024, op=C.MRT, nu=0.1024, u_lid=0.1,
                                                   quirks=C.QUIRKS_REFERENCE),
            "tg256_bgk": C.taylor_green(256, 256, op=C.BGK, nu=0.01, u0=0.04, quirks=C.QUIRKS_REFERENCE)}
    for name, c in cfgs.items():
        exe = os.path.join(REPO, "oracle", "_ref", "bin", "time_" + name)
        if not os.path.exists(exe):
            out[name] = {"unavailable": "reference timer binary not built (oracle/ref_build.sh timers)"}
            continue
        r = subprocess.run([exe, "50", "1000"], capture_output=True, text=True, timeout=300)
        if r.returncode != 0:
            out[name] = {"unavailable": "reference timer exited %d: %s" % (r.returncode, r.stderr.strip()[-200:])}
            continue
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith('{"nx"')]
        if not lines:
            out[name] = {"unavailable": "reference timer printed no timing line"}
            continue
        ref = json.loads(lines[-1])
        L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                         quirks=c["quirks"], u_bc=c["u_bc"], device=device, stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32))
        L.step(50, 0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        L.step(1000, 0)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / 1000
        del L
        nodes = c["nx"] * c["ny"]
        out[name] = {"reference_ms_per_step": ref["ms_per_step"], "reference_MLUPS": ref["mlups"],
                     "lbmx_ms_per_step": round(ms, 5), "lbmx_MLUPS": round(nodes / (ms * 1e3), 1),
                     "lbmx_over_reference": round(ref["ms_per_step"] / ms, 1)}
    out["how"] = ("back-to-back steps, CUDA events over 1000 steps after 50 warm-up steps; the reference binaries "
                  "run its LBM<2> main-loop call sequence on the default stream; lbmx with the reference's quirks on")
    return out


def bench_reference(args, rank, world):
    """CPU implementation of the reference step (the oracle port), all host threads."""
    if rank != 0:
        return
    import cases as C
    cores = os.cpu_count() or 1
    n = args.size
    c = cavity_case(n)
    o = C.make_oracle(c)
    per_step = args.ref_lbm_steps
    for _ in range(args.warmup):
        o.step(per_step)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.step(per_step)
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    mlups = n * n * per_step / t / 1e6
    line = {
        "impl": "reference", "metric": metric_name(n), "value": round(mlups, 2), "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 4),
        "lbm_steps_per_bench_step": per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(n, world),
        "cpu_baseline": {"value": round(mlups, 2), "unit": "MLUPS", "cores": cores, "kind": "port",
                         "sample": "%d bench steps x %d LBM steps of the %dx%d cavity" % (args.steps, per_step, n, n)},
        "e2e": {"value": round(mlups, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


PROFILE_CASES = ("batch_f16", "batch_f32", "cm_opt", "edge", "ibm", "adjoint", "tangent")


def run_profile_case(args, torch, stream, device):
    """A small workload of one kernel family, for ncu captures: `args.warmup`
    untimed steps, then `args.steps` steps (no timing, no L2 flush).  Every
    case holds more than the 129 MB L2 and a few GB at most.
      batch_f16 / batch_f32  batch_step_kernel: 64 cavities of the ensemble
                             (sides 64..768), MRT, fixed tile configuration
      cm_opt                 opt_prepass_kernel + step_kernel: Poiseuille
                             channel 4096 x 1024, CM<OptimalAdapter>
      edge                   edge_prepass_kernel + step_kernel: Zou-He inlet /
                             zero-gradient outlet channel 4096 x 1024, BGK
      ibm                    ibm_step_kernel + step_kernel: the cylinder
                             2048 x 512, 256 markers
      adjoint                adjoint kernels: Brinkman channel 2048 x 1024, CM,
                             checkpoint every 4, forward then backward
      tangent                tangent kernels: the cylinder 2048 x 512"""
    import cases as C
    import lbmx
    case, W, K = args.profile, args.warmup, args.steps

    def single(c, storage=0):
        L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], periodic=c["periodic"],
                         storage=storage, u_bc=c["u_bc"], wall_u=c["wall_u"], device=device,
                         stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.asarray(c["rho"], np.float32), np.asarray(c["u"], np.float32),
               None if c["force"] is None else np.asarray(c["force"], np.float32))
        if c["markers"] is not None:
            L.set_markers(c["markers"])
        return L

    if case.startswith("batch"):
        storage = 1 if case == "batch_f16" else 0
        Ls = []
        for side, _, nu in C.ensemble(count=64):
            c = C.ensemble_cavity(side, nu)
            Ls.append(single(c, storage))
        B = lbmx.Batch(Ls)
        B.set_config(tile_w=128, tile_h=8 if storage else 4, ctas_per_sm=3, chunk=8, graph_steps=0)
        B.step(W, flags=0)
        B.step(K, flags=0)
        B.synchronize()
        B.close()
    elif case in ("cm_opt", "edge", "ibm"):
        if case == "cm_opt":
            c = C.poiseuille(4096, 1024, op=C.CM_OPT, nu=0.02)
        elif case == "edge":
            c = C.channel(4096, 1024, op=C.BGK, nu=0.04, u_in=0.05, inlet="zouhe", outlet="zg")
        else:
            c = C.channel(2048, 512, op=C.BGK, nu=0.032, u_in=0.05, inlet="parabolic", outlet="zouhe_p",
                          markers=C.cylinder_markers(256, 256, 32, 256))
        L = single(c)
        L.step(W, 0)
        L.step(K, 0)
        L.synchronize()
    elif case == "adjoint":
        nx, ny = 2048, 1024
        ca = C.channel_brinkman(nx, ny, op=C.CM, sigma=16.0)
        w = np.zeros((3, ny, nx), np.float32)
        w[1, :, -1] = 1.0
        a = lbmx.Adjoint(nx, ny, op=C.CM, omega=ca["omega"], S=ca["S"], periodic=(True, False), flags=ca["flags"],
                         checkpoint_every=4, body_force=(float(ca["force"][0].flat[0]), 0.0), device=device,
                         stream=stream.cuda_stream)
        a.set_state(np.ones((ny, nx), np.float32), np.zeros((2, ny, nx), np.float32))
        a.set_gamma(ca["gamma"])
        a.set_objective(w, 1)
        a.forward(W + K)
        a.backward()
        a.close()
    elif case == "tangent":
        mk = C.cylinder_markers(256, 256, 32, 256)
        c = C.channel(2048, 512, op=C.BGK, nu=0.032, u_in=0.05, inlet="parabolic", outlet="zouhe_p", markers=mk)
        t = lbmx.Tangent(2048, 512, lbmx.TANGENT_U_BC, op=c["op"], omega=c["omega"], S=c["S"], flags=c["flags"],
                         u_bc=0.05, device=device, stream=stream.cuda_stream)
        t.set_state(np.ones((512, 2048), np.float32), np.zeros((2, 512, 2048), np.float32))
        t.set_markers(mk)
        t.run(W + K)
    torch.cuda.synchronize()
    print(json.dumps({"profile_case": case, "warmup": W, "steps": K, "ok": True}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="lbmx", choices=["lbmx", "reference"])
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--hbm-size", type=int, default=8192)
    ap.add_argument("--err-steps", type=int, default=200)
    ap.add_argument("--ref-lbm-steps", type=int, default=5)
    ap.add_argument("--ens-count", type=int, default=512)
    ap.add_argument("--ens-steps", type=int, default=64)
    ap.add_argument("--ens-err-steps", type=int, default=1000)
    ap.add_argument("--cyl-steps", type=int, default=200000, help="steps of the cylinder shedding run")
    ap.add_argument("--sens-steps", type=int, default=2000, help="steps of the drag-sensitivity run")
    ap.add_argument("--steady-max-steps", type=int, default=1500000, help="cap of the 1024^2 run to steady state")
    ap.add_argument("--adj-nx", type=int, default=4096)
    ap.add_argument("--adj-ny", type=int, default=1024)
    ap.add_argument("--adj-steps", type=int, default=5000)
    ap.add_argument("--adj-every", type=int, default=250)
    ap.add_argument("--quick", action="store_true", help="main number only (profiling runs)")
    ap.add_argument("--profile", choices=PROFILE_CASES, help="run one small kernel workload for an ncu capture")
    ap.add_argument("--storage", default="f32", choices=["f32", "f16_offset", "bf16_offset"],
                    help="storage of the main lattice with --quick (profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        bench_reference(args, rank, world)
        return

    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import cases as C
    import lbmx

    stream = torch.cuda.Stream()
    if args.profile:
        run_profile_case(args, torch, stream, local)
        return
    n = args.size
    nodes = n * n
    peaks, peak_kind = measured_peaks()
    hbm = float(peaks["hbm_gbs"])
    flush = L2Flush(torch)

    def lattice(storage, size=n):
        c = cavity_case(size)
        L = lbmx.Lattice(c["nx"], c["ny"], op=c["op"], omega=c["omega"], S=c["S"], storage=storage,
                         wall_u=c["wall_u"], device=local, stream=stream.cuda_stream)
        L.set_flags(c["flags"])
        L.init(np.ones((c["ny"], c["nx"]), np.float32), np.zeros((2, c["ny"], c["nx"]), np.float32))
        return L

    # ---- headline: FP32, L2 flushed before every timed step
    main_storage = {v: k for k, v in STORAGE_NAME.items()}[args.storage] if args.quick else 0
    L = lattice(main_storage)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    with ClockSampler(local) as clk:
        t = time_steps(L, torch, stream, args.steps, args.warmup, flush)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    ms = max_over_ranks(float(t.mean()), dist, "cuda")
    mlups = aggregate_mlups(nodes, ms, world)
    achieved = BYTES_PER_LU[main_storage] * nodes / (float(t.mean()) * 1e-3) / 1e9
    line = {
        "metric": metric_name(n, main_storage), "value": round(mlups, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(n, world), "storage": STORAGE_NAME[main_storage],
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": None,
                     "algorithmic_bytes_per_lu": BYTES_PER_LU[main_storage], "peak_kind": peak_kind + " burst (hbm_gbs)"},
        "gpu_launches": int(args.steps),
        "clocks": clk.summary(),
    }
    prof = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(prof):
        with open(prof) as fh:
            tr = json.load(fh)
        if str(n) in tr:
            t_n = tr[str(n)]
            line["roofline"]["traffic"] = t_n["dram_read_bytes_per_launch"] + t_n["dram_write_bytes_per_launch"]
            line["roofline"]["traffic_source"] = t_n["source"]

    if rank == 0 and not args.quick:
        # ---- e2e through the C-ABI with pinned host buffers
        c = cavity_case(n)
        h_rho = torch.ones((n, n), dtype=torch.float32).pin_memory()
        h_u = torch.zeros((2, n, n), dtype=torch.float32).pin_memory()
        h_flags = torch.from_numpy(c["flags"]).pin_memory()
        out_rho = torch.empty((n, n), dtype=torch.float32).pin_memory()
        out_u = torch.empty((2, n, n), dtype=torch.float32).pin_memory()
        Le = lbmx.Lattice(n, n, op=c["op"], omega=c["omega"], S=c["S"], wall_u=c["wall_u"], device=local,
                          stream=stream.cuda_stream)
        # one upload and boundary setup per 1000 steps (the reference's cavity
        # runs 100k steps per setup)
        K = max(args.steps, 1000)
        # the FP64 mass/momentum sums of every step, read back into pinned
        # host memory without stalling the GPU (the reference reads its
        # averages back with a blocking copy every step)
        sums_ring = torch.zeros((K, 3), dtype=torch.float64).pin_memory()
        for rep in range(2):  # first pass warms up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Le.set_flags(h_flags)
            Le.init(h_rho, h_u)
            Le._check(Le.lib.lbmx_step_sums(Le.h, K, lbmx.STEP_STORE_MOMENTS, sums_ring.data_ptr()))
            Le._check(Le.lib.lbmx_moments(Le.h, out_rho.data_ptr(), out_u.data_ptr(), None))
            e2e_t = time.perf_counter() - t0
        mass = sums_ring[:, 0].numpy()
        line["e2e"] = {"value": round(nodes * K / e2e_t / 1e6, 1), "unit": "MLUPS",
                       "h2d_bytes_per_step": int(round(13 * nodes / K)),
                       "d2h_bytes_per_step": int(round(24 + 12 * nodes / K)),
                       "lbm_steps": K, "seconds": round(e2e_t, 4),
                       "per_step_readback": "FP64 sums {rho, rho ux, rho uy} of every step (lbmx_step_sums)",
                       "mass_drift": float(abs(mass[-1] - mass[0]) / mass[0])}
        del Le

        # ---- FP64 oracle: L2 error reference and CPU baseline
        cores = os.cpu_count() or 1
        u64, cpu_mlups, cpu_dt = run_cpu_oracle(n, args.err_steps, cores)
        line["cpu_baseline"] = {"value": round(cpu_mlups, 2), "unit": "MLUPS", "cores": cores, "kind": "port",
                                "sample": "%d steps of the %dx%d cavity, FP64 oracle, OpenMP" % (args.err_steps, n, n)}

        # ---- storage variants with the L2 error against FP64
        variants = {}
        for storage in (0, 1, 2):
            Lv = lattice(storage)
            tv = time_steps(Lv, torch, stream, args.steps, args.warmup, flush)
            Lw = lattice(storage)
            Lw.step(args.err_steps)
            _, uv, _ = Lw.moments()
            mv = nodes / (float(tv.mean()) * 1e-3) / 1e6
            av = BYTES_PER_LU[storage] * nodes / (float(tv.mean()) * 1e-3) / 1e9
            variants[STORAGE_NAME[storage]] = {
                "MLUPS": round(mv, 1), "ms_per_step": round(float(tv.mean()), 5),
                "achieved_GBs": round(av, 1), "frac": round(av / hbm, 4),
                "l2_u_err_vs_fp64": l2_error(uv, u64), "err_steps": args.err_steps}
            del Lv, Lw
        variants["f16_speedup_vs_f32"] = round(variants["f16_offset"]["MLUPS"] / variants["f32"]["MLUPS"], 3)
        line["variants"] = variants
        # ---- the same cavity run towards steady state
        line["steady_state"] = bench_steady(args, torch, stream, local)

        # ---- HBM-bound size, no flush needed
        hn = args.hbm_size
        Lh = lattice(0, hn)
        th = time_steps(Lh, torch, stream, max(10, args.steps // 5), args.warmup, None)
        del Lh
        Lh16 = lattice(1, hn)
        th16 = time_steps(Lh16, torch, stream, max(10, args.steps // 5), args.warmup, None)
        del Lh16
        a32 = 72 * hn * hn / (float(th.mean()) * 1e-3) / 1e9
        a16 = 36 * hn * hn / (float(th16.mean()) * 1e-3) / 1e9
        line["hbm_bound"] = {
            "workload": "lid-driven cavity %dx%d MRT" % (hn, hn),
            "f32": {"MLUPS": round(hn * hn / (float(th.mean()) * 1e-3) / 1e6, 1), "achieved_GBs": round(a32, 1),
                    "frac": round(a32 / hbm, 4)},
            "f16_offset": {"MLUPS": round(hn * hn / (float(th16.mean()) * 1e-3) / 1e6, 1),
                           "achieved_GBs": round(a16, 1), "frac": round(a16 / hbm, 4)},
        }
        # ---- batched ensemble (many lattices, one persistent launch per step)
        line["ensemble"] = bench_ensemble(args, torch, stream, local, hbm)
        # ---- adjoint of the Brinkman channel
        line["adjoint"] = bench_adjoint(args, torch, stream, local)
        # ---- Taylor-Green decay and the IBM cylinder
        line["validation"] = bench_validation(args, torch, stream, local)
        # ---- the reference's own GPU step on this GPU, beside lbmx
        try:
            line["reference_gpu"] = bench_reference_gpu(args, torch, stream, local)
        except Exception as exc:  # a measurement of the reference: never fails the bench
            line["reference_gpu"] = {"unavailable": "%s: %s" % (type(exc).__name__, exc)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
