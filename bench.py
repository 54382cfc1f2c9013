#!/usr/bin/env python
"""Benchmark: even-odd Wilson Dslash GB/s at 32^3x64 (FP64), one JSON line.

Workload (the plain-FP64 GPU configuration): 32^3x64 lattice, seeded
synthetic SU(3) links exp(i*0.5*H) (seed 2), unit-norm Gaussian source
(seed 2).  One step = one even-odd hopping application D_eo over the Vh =
1,048,576 even sites, on fields resident in HBM.  GB/s counts the compulsory
bytes of one application: 8 links x 144 B + spinor in 192 B + spinor out
192 B = 1536 B per output site (FP64).  The inputs (1.2 GB of links, 201 MB
per spinor parity) are larger than L2 (129 MB), so no flush is needed.

`e2e` measures the same metric through the reference-facing host-buffer
entry point (wd_host_dslash_offd = DslashoffdNew): every step copies the
source parity the term reads from pinned host memory to the device, applies
the hopping term on the reference's site-major layout, and returns the
computed parity (the other parity of the destination is zeroed on the host),
in overlapped time-slab chunks.

Beside the headline line: the other storage formats (double-float, FP32,
FP16), DslashNew, CG solves per arithmetic at 32^3x64 (mass 0.05 and 0.01)
and 48^3x96 (mass 0.01), the reference's own 8^3x16 case, batched solves
(24 right-hand sides; 16 lattices of uneven volume), a continuous-batching
serving run, and the CPU baseline.

Multi-GPU: replicas only (the reference's domain decomposition is replaced by
one lattice per GPU); value = sum over ranks of per-rank work / max time.

--impl reference times the reference's CPU implementation of the same
application (the oracle's C restatement on all host cores; the reference's
own AVX2 sources do not build on an Arm host such as a GB300 node's Grace
CPU).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "ipcc2021-final_gb300"))

DIMS = (32, 32, 32, 64)
SEED = 2
EPS = 0.5
MASS = 0.05
BYTES_PER_SITE_F64 = 8 * 144 + 192 + 192   # links + spinor in + spinor out
# compulsory bytes per output site of one D_eo in each storage format:
# f64 / df64: 18-real links 144 B, spinor 192 B; f32: 12-real links 48 B,
# spinor 96 B; f16: 12-real links 24 B, spinor 48 B + 4 B scale
BYTES_PER_SITE = {"f64": 1536, "df64": 1536, "f32": 8 * 48 + 96 + 96, "f16": 8 * 24 + 52 + 52}
FLOPS_PER_SITE = 1320
METRIC = "Dslash GB/s at 32^3x64 (even-odd D_eo, FP64, compulsory bytes)"


def workload_config(dims, prec: str = "f64") -> dict:
    """The `config` of the benchmark line, the same dict in both arms."""
    V = int(np.prod(dims))
    links, spinor = 4 * V * 9 * 16, V // 2 * 12 * 16
    return {"workload": f"even-odd Dslash D_eo, {'x'.join(map(str, dims))}, seed 2, {prec.upper()} "
                        f"(repeated applications)",
            "lattice": list(dims), "sites": V, "precision": prec,
            "l2": f"inputs larger than L2, no flush ({links / 1e9:.2f} GB links + {spinor / 1e6:.0f} MB "
                  f"spinor per parity; L2 129 MB)"}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm() -> tuple[float, str]:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per D_eo launch
# at 32^3x64, from one ncu capture of each kernel at 24^3x48 scaled by the
# number of output sites (traffic per site is constant across volumes for
# these kernels); not measured by this run.
TRAFFIC_PER_LAUNCH = {"f64": 1.595e9, "df64": 1.592e9, "f32": 5.660e8, "f16": 2.706e8}
TRAFFIC_SOURCE = ("ncu capture at 24^3x48 of the same kernel (dram__bytes_read.sum + dram__bytes_write.sum), "
                  "scaled to 32^3x64 by output sites; a recorded constant, not measured in this run")


def cpu_baseline_port(gauge, src, dims, seconds: float = 12.0) -> dict:
    """The oracle's C restatement of DslashoffdNew on all host cores, full lattice,
    repeated until about `seconds` of CPU work."""
    sys.path.insert(0, str(REPO / "oracle"))
    from oracle import Oracle

    orc = Oracle()
    cores = orc.threads(os.cpu_count() or 1)
    vh = int(np.prod(dims)) // 2
    t0 = time.perf_counter()
    reps = 0
    while True:
        orc.dslash_offd(src, gauge, dims, 0, 0)
        reps += 1
        if time.perf_counter() - t0 > seconds or reps >= 50:
            break
    dt = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    orc.dslash_full(src, gauge, dims, MASS, 0)
    full_ms = (time.perf_counter() - t0) * 1e3
    return {"value": BYTES_PER_SITE_F64 * vh / dt / 1e9, "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{reps} DslashoffdNew applications at {'x'.join(map(str, dims))} (full workload), "
                      f"{dt * 1e3:.1f} ms each, C restatement with OpenMP over sites",
            "dslash_new_ms": full_ms}


def dslash_variants(wd, ctx, lat, src, stream, steps: int, vh: int, peak: float) -> dict:
    """D_eo in the other storage formats on the same lattice (CUDA events)."""
    import torch

    out = {}
    for name, prec in (("df64", wd.DF64), ("f32", wd.F32), ("f16", wd.F16)):
        fi, fo = lat.field(src, prec=prec), lat.field(prec=prec)
        for _ in range(5):
            lat.dslash_eo(fi, fo, 0, 0, prec)
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            lat.dslash_eo(fi, fo, 0, 0, prec)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / steps
        gbs = BYTES_PER_SITE[name] * vh / (ms * 1e-3) / 1e9
        out[name] = {"ms": ms, "gbs": gbs, "frac_of_hbm": gbs / peak, "bytes_per_site": BYTES_PER_SITE[name],
                     "gflops": FLOPS_PER_SITE * vh / (ms * 1e-3) / 1e9}
        fi.close()
        fo.close()
    out["note"] = ("df64: FP64-class results (<=1e-13 rel. L2 vs the FP64 oracle) from float pairs on the "
                   "FP32 pipe; f32/f16: the mixed solvers' inner operators (12-real links)")
    return out


def small_config_bench(wd, ctx, with_cpu: bool) -> dict:
    """The reference's own CPU-runnable case: 8^3x16, seed 1, mass 0.1, CG to
    1e-10 (max 1000 iterations).  On the GPU: the even-odd CG (relative true
    residual) and the reference's CG recurrences (WD_SOLVER_CGNR_REF, absolute
    stop on the normal residual), both from a zero initial guess.  With
    with_cpu, the oracle's C restatement of the reference's CGinvert and
    DslashoffdNew on ONE host thread (the reference runs one rank per core) on
    the same inputs -- a baseline, not part of the GPU path."""
    dims, mass = (8, 8, 8, 16), 0.1
    gauge, src = wd.gen_gauge(dims, 1, EPS), wd.gen_source(dims, 1)
    lat = ctx.lattice(dims, gauge)
    b, x = lat.field(src), lat.field()
    out = {"workload": "8x8x8x16 (8192 sites), seed 1, mass 0.1, CG to 1e-10, max 1000 iterations"}
    for name, kind in (("gpu_cg_eo_f64", wd.CG_EO), ("gpu_cgnr_ref_f64", wd.CGNR_REF)):
        p = wd.solver_params(kind=kind, mass=mass, tol=1e-10, max_iter=1000)
        x.zero()
        lat.solve(b, x, p)  # warm-up
        x.zero()
        st = lat.solve(b, x, p)
        out[name] = {"seconds": st.seconds, "iterations": st.iterations, "true_residual": st.true_residual}
    fi, fo = lat.field(src), lat.field()
    n = 200
    lat.dslash_offd(fi, fo, 0, 0)
    ctx.sync()
    t0 = time.perf_counter()
    for _ in range(n):
        lat.dslash_offd(fi, fo, 0, 0)
    ctx.sync()
    out["gpu_dslashoffd_ms"] = (time.perf_counter() - t0) / n * 1e3
    for f in (b, x, fi, fo):
        f.close()
    lat.close()
    if with_cpu:
        sys.path.insert(0, str(REPO / "oracle"))
        from oracle import Oracle

        orc = Oracle()
        all_threads = orc.threads(os.cpu_count() or 1)
        orc.threads(1)
        t0 = time.perf_counter()
        _, it, rsd = orc.cg_ref(src, gauge, dims, mass, 1000, 1e-10, np.zeros_like(src))
        cg_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        for _ in range(100):
            orc.dslash_offd(src, gauge, dims, 0, 0)
        ds_ms = (time.perf_counter() - t0) / 100 * 1e3
        orc.threads(all_threads)
        out["cpu_oracle_1_thread"] = {"cginvert_seconds": cg_s, "cginvert_iterations": it,
                                      "dslashoffd_ms": ds_ms, "cores": 1, "kind": "port"}
    return out


SOLVER_PLANS = ("f64", "df64", "mixed_f32", "mixed_f16", "mixed_f16_df64")


class OracleSolution:
    """The oracle's solution of one solver workload, computed on the host cores
    before the GPU solves and outside every timed region: even-odd CG driven
    to a normal residual of 1e-14 (FP64 true residual ~1e-13)."""

    def __init__(self, gauge, src, dims, mass: float):
        sys.path.insert(0, str(REPO / "oracle"))
        from oracle import Oracle

        self.orc = Oracle()
        self.cores = self.orc.threads(os.cpu_count() or 1)
        self.gauge, self.src, self.dims, self.mass = gauge, src, dims, mass
        t0 = time.perf_counter()
        self.x, self.iterations, self.true_residual = self.orc.cg_eo(src, gauge, dims, mass, tol=1e-14)
        self.seconds = time.perf_counter() - t0

    def assess(self, sol) -> dict:
        """Error of a GPU solution against this one, and its FP64 true residual
        recomputed by the oracle."""
        r = self.src - self.orc.dslash_full(sol, self.gauge, self.dims, self.mass, 0)
        return {"err_vs_oracle": float(np.linalg.norm(sol - self.x) / np.linalg.norm(self.x)),
                "true_residual_oracle": float(np.linalg.norm(r) / np.linalg.norm(self.src))}

    def summary(self) -> dict:
        return {"solver": "even-odd CG on the host cores, normal residual 1e-14", "cores": self.cores,
                "iterations": self.iterations, "seconds": self.seconds, "true_residual": self.true_residual}


def solver_bench(wd, ctx, lat, src, mass: float, tol: float = 1e-10, plans=SOLVER_PLANS,
                 profile: bool = False, oracle_sol: OracleSolution | None = None) -> dict:
    """Solves per arithmetic on the resident lattice (the median of three timed
    solves after a warm-up): solves/s, iterations, FP64 true residual, the
    relative difference to the FP64 solution and, given the oracle's solution,
    the error against it and the true residual the oracle recomputes.
    profile=True brackets each timed solve with cudaProfilerStart/Stop (for
    `ncu --profile-from-start off`)."""
    import torch

    b = lat.field(src)
    out = {}
    ref = None
    table = {"f64": (wd.F64, wd.F64), "df64": (wd.DF64, wd.F64), "mixed_f32": (wd.F32, wd.F64),
             "mixed_f16": (wd.F16, wd.F64), "mixed_f16_df64": (wd.F16, wd.DF64)}
    for name in plans:
        prec, rel = table[name]
        x = lat.field()
        p = wd.solver_params(kind=wd.CG_EO, mass=mass, tol=tol, max_iter=5000, prec=prec, prec_reliable=rel)
        lat.solve(b, x, p)            # warm-up (derived link copies, allocator)
        times = []
        for rep in range(1 if profile else 3):  # the median of three timed solves
            x.zero()
            ctx.sync()
            if profile:
                torch.cuda.profiler.start()
            st = lat.solve(b, x, p)
            if profile:
                torch.cuda.profiler.stop()
            times.append(st.seconds)
        secs = float(np.median(times))
        sol = x.download()
        if ref is None:
            ref = sol
        out[name] = {"solves_per_s": 1.0 / secs, "seconds": secs, "seconds_each": times, "iterations": st.iterations,
                     "reliable_updates": st.reliable_updates, "true_residual": st.true_residual,
                     "rel_diff_vs_f64": float(np.linalg.norm(sol - ref) / np.linalg.norm(ref))}
        if oracle_sol is not None:
            out[name].update(oracle_sol.assess(sol))
        x.close()
    if "f64" in out:
        for name in out:
            if name != "f64":
                out[name]["speedup_vs_f64"] = out["f64"]["seconds"] / out[name]["seconds"]
    if oracle_sol is not None:
        out["oracle"] = oracle_sol.summary()
    return out


def batch_bench(wd, ctx, profile: bool = False) -> dict:
    """Batched solves against the same systems solved one at a time.
    (a) one 24^3x48 lattice (seed 3, mass 0.05): 12 point sources (unit delta at
        site 0 for each spin/colour) + 12 Gaussian sources;
    (b) 16 lattices, L in {8,12,16,24} (four each), T = 2L, independent seeds,
        masses uniform in [0.05, 0.2], one Gaussian source each.
    All to FP64 true residual 1e-10 with the mixed FP32 solver.  profile=True
    brackets each timed batched solve with cudaProfilerStart/Stop."""
    import torch

    def run(systems, params, timed=False):
        for _, _, x, _ in systems:
            x.zero()
        ctx.sync()
        if profile and timed:
            torch.cuda.profiler.start()
        stats = ctx.solve_batch(systems, params)
        if profile and timed:
            torch.cuda.profiler.stop()
        assert all(st.converged and st.true_residual <= 1e-10 for st in stats)
        return stats[0].seconds, stats   # the solve; the FP64 check of each result follows it

    def solo(systems, prec, rel):
        total, worst = 0.0, 0.0
        for lat, b, x, m in systems:
            x.zero()
            st = lat.solve(b, x, wd.solver_params(kind=wd.CG_EO, mass=m, tol=1e-10, max_iter=5000, prec=prec,
                                                  prec_reliable=rel))
            worst = max(worst, st.true_residual)
            total += st.seconds
        return total, worst

    out = {}
    dims = (24, 24, 24, 48)
    V = int(np.prod(dims))
    lat = ctx.lattice(dims, wd.gen_gauge(dims, 3, EPS))
    srcs = []
    for s_ in range(4):
        for c in range(3):
            b = np.zeros(V * 12, np.complex128)
            b[s_ * 3 + c] = 1.0
            srcs.append(b)
    srcs += [wd.gen_source(dims, 1000 + k) for k in range(12)]
    systems = [(lat, lat.field(b), lat.field(), 0.05) for b in srcs]
    res = {}
    for name, prec, rel in (("f32_inner_f64_reliable", wd.F32, wd.F64), ("f32_inner_df64_reliable", wd.F32, wd.DF64),
                            ("f16_inner_df64_reliable", wd.F16, wd.DF64)):
        p = wd.solver_params(kind=wd.CG_EO, tol=1e-10, max_iter=5000, prec=prec, prec_reliable=rel)
        run(systems, p)  # warm-up
        dt, stats = run(systems, p, timed=True)
        res[name] = {"seconds": dt, "solves_per_s": len(systems) / dt,
                     "max_iterations": max(st.iterations for st in stats),
                     "max_true_residual": max(st.true_residual for st in stats)}
    for name, prec, rel in (("solo_mixed_f32", wd.F32, wd.F64), ("solo_f64", wd.F64, wd.F64)):
        dt, worst = solo(systems, prec, rel)
        res[name] = {"seconds": dt, "solves_per_s": len(systems) / dt, "max_true_residual": worst}
    res["speedup_batched_vs_solo_f64"] = res["solo_f64"]["seconds"] / res["f32_inner_f64_reliable"]["seconds"]
    res["speedup_batched_vs_solo_mixed"] = res["solo_mixed_f32"]["seconds"] / res["f32_inner_f64_reliable"]["seconds"]
    out["multi_rhs_24c48_24_sources"] = res
    for _, b, x, _ in systems:
        b.close()
        x.close()
    lat.close()

    rng = np.random.default_rng(4)
    systems, lats = [], []
    for i, L in enumerate([8, 12, 16, 24] * 4):
        d = (L, L, L, 2 * L)
        la = ctx.lattice(d, wd.gen_gauge(d, 200 + i, EPS))
        lats.append(la)
        systems.append((la, la.field(wd.gen_source(d, 300 + i)), la.field(), float(rng.uniform(0.05, 0.2))))
    res = {}
    for name, prec, rel in (("batched", wd.F32, wd.F64), ("batched_df64_reliable", wd.F32, wd.DF64),
                            ("batched_f16_inner_df64_reliable", wd.F16, wd.DF64)):
        p = wd.solver_params(kind=wd.CG_EO, tol=1e-10, max_iter=5000, prec=prec, prec_reliable=rel)
        run(systems, p)
        dt, stats = run(systems, p, timed=True)
        res[name] = {"seconds": dt, "solves_per_s": len(systems) / dt,
                     "iterations": [st.iterations for st in stats],
                     "max_true_residual": max(st.true_residual for st in stats)}
    for name, prec, rel in (("solo_mixed_f32", wd.F32, wd.F64), ("solo_mixed_f32_df64_reliable", wd.F32, wd.DF64),
                            ("solo_f64", wd.F64, wd.F64)):
        dt, worst = solo(systems, prec, rel)
        res[name] = {"seconds": dt, "solves_per_s": len(systems) / dt, "max_true_residual": worst}
    res["speedup_batched_vs_solo_f64"] = res["solo_f64"]["seconds"] / res["batched"]["seconds"]
    res["speedup_batched_vs_solo_mixed"] = res["solo_mixed_f32"]["seconds"] / res["batched"]["seconds"]
    res["speedup_batched_vs_solo_mixed_df64_reliable"] = (res["solo_mixed_f32_df64_reliable"]["seconds"]
                                                          / res["batched_df64_reliable"]["seconds"])
    out["16_lattices_L8_to_24"] = res
    return out


SERVE_SIZES = [((8, 8, 8, 16), 0.4), ((16, 16, 16, 32), 0.3), ((24, 24, 24, 48), 0.2), ((32, 32, 32, 64), 0.1)]


def serve_workload(n: int, seed: int = 7):
    """n requests: lattice size from the configured mix, one of the two resident
    gauge fields of that size, mass U[0.02, 0.2], tol from {1e-8, 1e-10},
    1-12 seeded Gaussian sources."""
    rng = np.random.default_rng(seed)
    probs = [p for _, p in SERVE_SIZES]
    reqs = []
    for i in range(n):
        c = int(rng.choice(len(SERVE_SIZES), p=probs))
        reqs.append({"size": c, "gauge": 2 * c + int(rng.integers(2)), "mass": float(rng.uniform(0.02, 0.2)),
                     "tol": float(rng.choice([1e-8, 1e-10])), "nsrc": int(rng.integers(1, 13)),
                     "seeds": [int(v) for v in rng.integers(1, 2**62, size=13)]})
    return reqs


def serve_run(wd, ctx, reqs, rate: float, prec: int, budget: float = 150e9, seed: int = 11) -> dict:
    """Poisson arrivals at `rate` requests/s into a server; returns latency
    percentiles and throughput.  Latency = completion - arrival."""
    import time as _t
    sv = wd.Server(ctx, prec=prec, prec_reliable=wd.DF64, hbm_budget_bytes=budget)
    gids = []
    for c, (dims, _) in enumerate(SERVE_SIZES):
        for k in range(2):
            gids.append(sv.add_lattice(dims, wd.gen_gauge(dims, 500 + 2 * c + k, EPS)))
    arrivals = np.cumsum(np.random.default_rng(seed).exponential(1.0 / rate, size=len(reqs)))
    t0 = _t.perf_counter()
    pending, lat, solves, worst = {}, [], 0, 0.0
    i = 0
    while i < len(reqs) or pending:
        now = _t.perf_counter() - t0
        while i < len(reqs) and arrivals[i] <= now:
            r = reqs[i]
            rid = sv.submit(gids[r["gauge"]], r["nsrc"], r["mass"], r["tol"], seeds=r["seeds"][:r["nsrc"]])
            pending[rid] = (arrivals[i], r)
            i += 1
        q, active, _ = sv.status()
        if active or q:
            sv.step()
        elif i < len(reqs):
            _t.sleep(max(0.0, arrivals[i] - (_t.perf_counter() - t0)))
            continue
        done_now = _t.perf_counter() - t0
        for rid in list(pending):
            done, _, stats, _ = sv.poll(rid)
            if done:
                arr, r = pending.pop(rid)
                lat.append(done_now - arr)
                solves += r["nsrc"]
                worst = max(worst, max(st.residual / r["tol"] for st in stats))
                assert all(st.converged for st in stats)
    wall = _t.perf_counter() - t0
    sv.close()
    lat = np.array(lat)
    return {"rate_req_per_s": rate, "requests": len(reqs), "solves": solves, "wall_s": wall,
            "solves_per_s": solves / wall, "requests_per_s": len(reqs) / wall,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "max_residual_over_tol": worst,
            # served below 90 % of the offered rate: the server is the bottleneck
            "saturated": bool(len(reqs) / wall < 0.9 * rate)}


def serve_bench(wd, ctx, n: int, rates_mixed, rates_f64, n_f64: int | None = None) -> dict:
    """The same request stream (its first n_f64 requests for the FP64 server)
    at each arrival rate."""
    reqs = serve_workload(n)
    reqs64 = reqs[:n_f64] if n_f64 else reqs
    out = {"workload": f"{n} Poisson-arrival requests ({len(reqs64)} for plain FP64), sizes "
                       "{8^3x16:.4, 16^3x32:.3, 24^3x48:.2, 32^3x64:.1}, mass U[0.02,0.2], tol {1e-8,1e-10}, "
                       "1-12 sources, 8 resident gauge fields, 150 GB budget",
           "mixed_batched": [serve_run(wd, ctx, reqs, r, wd.F16) for r in rates_mixed],
           "plain_f64": [serve_run(wd, ctx, reqs64, r, wd.F64) for r in rates_f64],
           "mixed_batched_solver": "FP16 inner (per-site scale, 12-real links), double-float reliable updates"}
    sat = {k: max((r["solves_per_s"] for r in out[k] if r["saturated"]), default=None)
           for k in ("mixed_batched", "plain_f64")}
    out["saturated_solves_per_s"] = sat
    if sat["mixed_batched"] and sat["plain_f64"]:
        out["saturated_ratio_mixed_vs_f64"] = sat["mixed_batched"] / sat["plain_f64"]
    return out


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: replicas run independent lattices, and the
    job is done when the last one is."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput of `world` replicas: all ranks' units over the max time."""
    return world * units_per_rank / seconds_max


def run_reference(args) -> None:
    """The reference's CPU implementation of the path on the host cores, on
    the same workload: only the oracle's host library is loaded (its copy of
    the seeded generator gives the GPU arm's input bytes)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    from oracle import Oracle

    orc = Oracle()
    gauge = orc.gen_gauge(DIMS, SEED, EPS)
    src = orc.gen_source(DIMS, SEED)
    cores = orc.threads(os.cpu_count() or 1)
    vh = int(np.prod(DIMS)) // 2
    orc.dslash_offd(src, gauge, DIMS, 0, 0)  # warm-up (page in, thread pool)
    # bounded sample: at most `steps` applications or ~60 s
    t0 = time.perf_counter()
    n = 0
    while n < args.steps and (time.perf_counter() - t0) < 60.0:
        orc.dslash_offd(src, gauge, DIMS, 0, 0)
        n += 1
    dt = (time.perf_counter() - t0) / n
    v = BYTES_PER_SITE_F64 * vh / dt / 1e9
    why_port = ("; the reference's AVX2 sources do not build on this Arm host"
                if platform.machine().lower() in ("aarch64", "arm64") else "")
    line = {"metric": METRIC, "value": v, "unit": "GB/s", "n_gpus": world, "steps": n, "warmup": args.warmup,
            "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded SU(3) links eps=0.5, unit Gaussian source)",
            "config": workload_config(DIMS),
            "parallelism": f"host threads x{cores}",
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "GB/s", "cores": cores, "kind": "port",
                             "sample": f"{n} DslashoffdNew applications at 32x32x32x64 (C restatement of the "
                                       f"reference, OpenMP over sites{why_port})"},
            "e2e": {"value": v, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import wilson_gb300 as wd

    prec = {"f64": wd.F64, "df64": wd.DF64, "f32": wd.F32, "f16": wd.F16}[args.prec]
    bps = BYTES_PER_SITE[args.prec]
    dims = tuple(args.dims)
    gauge = wd.gen_gauge(dims, SEED, EPS)
    src = wd.gen_source(dims, SEED)
    vh = int(np.prod(dims)) // 2
    ctx = wd.Context(local)
    lat = ctx.lattice(dims, gauge)
    fin, fout = lat.field(src, prec=prec), lat.field(prec=prec)
    stream = torch.cuda.ExternalStream(ctx.stream, device=torch.device("cuda", local))

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        lat.dslash_eo(fin, fout, 0, 0, prec)
    ctx.sync()

    clocks = ClockSampler(local)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    clocks.start()
    time.sleep(0.3)
    launches0 = ctx.launches
    e0.record(stream)
    for _ in range(args.steps):
        lat.dslash_eo(fin, fout, 0, 0, prec)
    e1.record(stream)
    e1.synchronize()
    launches = ctx.launches - launches0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    t_max = max_over_ranks(ms, world)
    value = replica_throughput(bps * vh, t_max * 1e-3, world) / 1e9

    # e2e through the reference-facing entry point, pinned host buffers
    e2e = None
    if not args.no_e2e:
        h_src = torch.from_numpy(src).pin_memory().numpy()
        h_dst = torch.empty(src.size, dtype=torch.complex128).pin_memory().numpy()
        host_gauge = [torch.from_numpy(g).pin_memory().numpy() for g in gauge]
        ctx.host_dslash_offd(dims, host_gauge, h_src, 0, 0)  # first call uploads the links
        n_e2e = max(3, min(args.steps, 20))
        # the C call's arguments, built once (a C/C++ caller passes them as they are)
        c_dims, c_gauge, c_src, c_dst = wd._dims(dims), wd._gauge_ptrs(host_gauge), wd._ptr(h_src), wd._ptr(h_dst)
        barrier()
        t0 = time.perf_counter()
        per_call = []
        for _ in range(n_e2e):
            tc = time.perf_counter()
            ctx.check(wd.lib.wd_host_dslash_offd(ctx.handle, c_dims, c_gauge, c_src, c_dst, 0, 0))
            per_call.append(time.perf_counter() - tc)
        e2e_s = max_over_ranks((time.perf_counter() - t0) / n_e2e, world)
        # DslashNew (full M) through its host-buffer entry point, same buffers
        ctx.check(wd.lib.wd_host_dslash_full(ctx.handle, wd._dims(dims), wd._gauge_ptrs(host_gauge),
                                             wd._ptr(h_src), wd._ptr(h_dst), MASS, 0))
        t1 = time.perf_counter()
        for _ in range(n_e2e):
            ctx.check(wd.lib.wd_host_dslash_full(ctx.handle, c_dims, c_gauge, c_src, c_dst, MASS, 0))
        full_ms = (time.perf_counter() - t1) / n_e2e * 1e3
        e2e = {"value": replica_throughput(BYTES_PER_SITE_F64 * vh, e2e_s, world) / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": int(src.nbytes // 2), "d2h_bytes_per_step": int(src.nbytes // 2),
               "steps": n_e2e, "ms_per_step": e2e_s * 1e3, "dslash_new_host_ms": full_ms,
               "ms_per_call_min_median_max": [round(1e3 * min(per_call), 4),
                                              round(1e3 * float(np.median(per_call)), 4),
                                              round(1e3 * max(per_call), 4)],
               "path": "wd_host_dslash_offd (DslashoffdNew): the source parity it reads goes up and the "
                       "computed parity comes back in up to 16 time-slab chunks overlapped with compute on "
                       "two streams, the kernel working on the reference's site-major layout in the staging "
                       "buffers; the other parity of dest is zeroed on the host meanwhile; pinned host "
                       "buffers, links resident"}

    if rank == 0:
        peak, peak_src = measured_peak_hbm()
        fp64_peak, fp32_peak = ctx.fma_peak()
        achieved = bps * vh / (ms * 1e-3) / 1e9
        gflops = FLOPS_PER_SITE * vh / (ms * 1e-3) / 1e9
        traffic = TRAFFIC_PER_LAUNCH[args.prec] if dims == DIMS else None
        line = {
            "metric": METRIC if args.prec == "f64" else METRIC.replace("FP64", args.prec.upper()), "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": args.prec,
            "data": "synthetic (seeded SU(3) links eps=0.5, unit Gaussian source)",
            "config": workload_config(dims, args.prec),
            "parallelism": f"replicas x{world}",
            "gflops": gflops * world,
            "effective_gbs_quda_style": 2880 * vh / (ms * 1e-3) / 1e9,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "traffic_source": TRAFFIC_SOURCE,
                         "peak_source": peak_src,
                         "note": "FP64 kernels are bounded by the FP64 pipe on GB300; see compute"},
            "compute": {"bound": "fp64" if args.prec == "f64" else "fp32",
                        "achieved_tflops": gflops / 1e3,
                        "fp64_peak_tflops": fp64_peak, "fp32_peak_tflops": fp32_peak,
                        "fp64_frac": gflops / 1e3 / fp64_peak if args.prec == "f64" else None,
                        "peak_source": "measured live (wd_diag_fma_peak)"},
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
        }
        if args.prec == "f64":
            line["dslash_other_storage"] = dslash_variants(wd, ctx, lat, src, stream, min(args.steps, 300), vh, peak)
            # the full operator (DslashNew: diagonal + both hopping halves), resident fields
            n_full = max(3, min(args.steps, 100))
            lat.dslash_full(fin, fout, MASS, 0)
            ctx.sync()
            e0.record(stream)
            for _ in range(n_full):
                lat.dslash_full(fin, fout, MASS, 0)
            e1.record(stream)
            e1.synchronize()
            line["dslash_new_ms"] = e0.elapsed_time(e1) / n_full
        with_oracle = not args.no_cpu_baseline
        if not args.no_solver:
            osol = OracleSolution(gauge, src, dims, MASS) if with_oracle else None
            line["solver"] = {"workload": f"even-odd CG to true residual 1e-10, {'x'.join(map(str, dims))}, "
                                          f"mass {MASS}, seed 2",
                              **solver_bench(wd, ctx, lat, src, MASS, plans=args.solver_plans,
                                             profile=args.profile_solves, oracle_sol=osol)}
            del osol
        if not args.no_solver_mixed:
            # the mixed-precision configuration: mass 0.01 on 32^3x64 and on 48^3x96
            for key, sd in (("solver_mixed", tuple(args.solver_dims)), ("solver_mixed_large", (48, 48, 48, 96))):
                if key == "solver_mixed_large" and args.no_solver_large:
                    continue
                sgauge = gauge if sd == dims else wd.gen_gauge(sd, SEED, EPS)
                ssrc = src if sd == dims else wd.gen_source(sd, SEED)
                osol = OracleSolution(sgauge, ssrc, sd, args.solver_mass) if with_oracle else None
                slat = ctx.lattice(sd, sgauge)
                line[key] = {"workload": f"even-odd CG to true residual 1e-10, {'x'.join(map(str, sd))}, "
                                         f"mass {args.solver_mass}, seed 2",
                             **solver_bench(wd, ctx, slat, ssrc, args.solver_mass,
                                            plans=args.solver_plans, profile=args.profile_solves, oracle_sol=osol)}
                slat.close()
                del osol, sgauge, ssrc
        if not args.no_solver:
            line["small_config"] = small_config_bench(wd, ctx, not args.no_cpu_baseline)
        if not args.no_batch:
            line["batch"] = batch_bench(wd, ctx, profile=args.profile_batch)
        if args.serve_requests > 0:
            line["serving"] = serve_bench(wd, ctx, args.serve_requests, args.serve_rates, args.serve_rates_f64,
                                          args.serve_requests_f64)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline_port(gauge, src, dims)
        # launch shapes the tuner chose for every kernel and size run above
        # (half_volume: half-lattice sites, or a batch's system-sites rounded up to a power of 2)
        line["autotune"] = [{"kernel": k, "half_volume": v, "variant": var, "ms": ms}
                            for _, k, v, var, ms in wd.tune_report()]
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--prec", choices=["f64", "df64", "f32", "f16"], default="f64",
                    help="storage/arithmetic of the timed kernel (e2e always uses the FP64 drop-in path)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-solver", action="store_true", help="skip the CG solves/s measurements")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-solve measurements")
    ap.add_argument("--solver-plans", nargs="*", choices=SOLVER_PLANS, default=list(SOLVER_PLANS))
    ap.add_argument("--profile-solves", action="store_true",
                    help="bracket each timed solve with cudaProfilerStart/Stop (ncu --profile-from-start off)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="bracket each timed batched solve with cudaProfilerStart/Stop")
    ap.add_argument("--solver-dims", type=int, nargs=4, default=[32, 32, 32, 64],
                    help="lattice of the second solver measurement (mixed-precision configuration; 48 48 48 96 also)")
    ap.add_argument("--solver-mass", type=float, default=0.01)
    ap.add_argument("--no-solver-mixed", action="store_true", help="skip the mass-0.01 solver measurements")
    ap.add_argument("--no-solver-large", action="store_true", help="skip the 48^3x96 solver measurement")
    ap.add_argument("--serve-requests", type=int, default=2000,
                    help="requests per serving run (the configured workload: 2000; 0 skips serving)")
    ap.add_argument("--serve-requests-f64", type=int, default=300,
                    help="requests for the plain FP64 server (the first ones of the same stream)")
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[16.0, 48.0],
                    help="arrival rates (requests/s) for the batched mixed-precision server: one below "
                         "saturation, one above it")
    ap.add_argument("--serve-rates-f64", type=float, nargs="*", default=[12.0],
                    help="arrival rates (requests/s) for the plain FP64 server (above its saturation)")
    ap.add_argument("--dims", type=int, nargs=4, default=list(DIMS),
                    help="lattice extents (default 32 32 32 64, the benchmark configuration)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
