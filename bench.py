"""Benchmark: solves/s of the MoM hot path (fill + LU + far field) on GB300.

Workload (default): PEC sphere, level-4 icosphere (5120 triangles, N = 7680
RWG), radius 1 m, seeded tangential jitter +-3% of the edge length, 450 MHz,
x-polarised plane wave incident along -z, bistatic far field (sigma_VV,
sigma_HH) at R = 10 m on 181 theta x 2 phi cuts. One step = one full solve:
  fill Z -> plane-wave RHS -> LU + solve (mixed: complex64 LU + FP64
  refinement against the FP64 Z) -> current lumping -> far-field sigma.
Synthetic inputs (seeded mesh); the working set (Z: 0.94 GB c128 + 0.47 GB c64)
is far larger than L2, so no extra flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
                  [--impl ours|reference]

`--impl reference` times FRICO's CPU path on the host cores: the oracle
(a restatement of FRICO's fill / lumping / fields with OpenMP) plus LAPACK
zgetrf/zgetrs through scipy, each step a bounded sample (fill on a slice of
the columns, scaled to the full matrix; full LU + solve; full fields).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

FREQ = 450e6
R_FAR = 10.0
WORKLOAD = "sphere_L4_N7680_450MHz_planewave_bistatic181x2"
METRIC = "solves/s (fill+LU+far-field)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--level", type=int, default=4, help="icosphere level (4: N=7680)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the FP64 GPU drop-in run (its solves/s and the mixed-vs-FP64 accuracy)")
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed steps of the FP64 GPU drop-in")
    ap.add_argument("--gemm-engine", default="auto", choices=["auto", "simt", "tc", "tc_f16"],
                    help="auto/tc: 3xTF32 operands; tc_f16: 3xFP16 block columns of the unpivoted LU")
    ap.add_argument("--pivoting", default="auto", choices=["auto", "partial", "none"])
    ap.add_argument("--workload", default="sphere", choices=["sphere", "strip", "sphere64", "sweep", "adjoint"],
                    help="sphere: one solve per step (headline); sphere64: level-5 sphere, 64 incidences, "
                         "181 x 361 bistatic grid; sweep: bowtie frequency sweep per step; "
                         "adjoint: bowtie gradients per step")
    ap.add_argument("--validate", type=int, default=0,
                    help="adjoint: check this many seeded random directions by central differences")
    ap.add_argument("--sweep-n", type=int, default=3000, choices=[500, 1500, 3000])
    ap.add_argument("--sweep-freqs", type=int, default=256)
    ap.add_argument("--lanes", type=int, default=0, help="sweep lanes (0: chosen by the library)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile
            fd, name = tempfile.mkstemp(prefix="frico_clocks_", suffix=".csv")
            os.close(fd)
            self.path = Path(name)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        try:
            self.path.unlink()
        except OSError:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


# DRAM traffic (ncu: dram__bytes_read.sum + dram__bytes_write.sum) per launch of the complex64
# LU's narrow (k_gemm_tf32x3) and trailing-update (k_gemm_pair_tf32x3) GEMMs, averaged over
# the 116 update launches of one L4-sphere solve; the capture and its command are summarised
# in profiles/launch_list_sphere_L4_mixed.md.
GEMM_TRAFFIC_BYTES_PER_LAUNCH = {("k_gemm_pair_tf32x3 + k_gemm_tf32x3", 4): 177.3e6}


def gemm_traffic_per_launch(level: int, precision: str, kernel: str):
    """Measured DRAM bytes per update launch for the configuration the capture was
    made on (the L4 sphere, mixed precision); None for any other."""
    if precision != "mixed":
        return None
    return GEMM_TRAFFIC_BYTES_PER_LAUNCH.get((kernel, level))


# ------------------------------------------------------------------ CPU paths
def cpu_sample(mesh, steps: int, warmup: int, Zfull=None):
    """FRICO's CPU path on a bounded sample; returns (sec/solve list, cores, sample desc)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    from frico_gb300 import meshes
    o = Oracle(mesh)
    n = o.n
    cols = max(64, n // 16)
    if Zfull is None:
        Zfull = o.compute_matrix(FREQ)
    V = o.rhs_plane_wave(FREQ, 0.0, 0.0, 1.0, 0.0)
    T, P, _ = meshes.bistatic_cuts(R_FAR)
    times = []
    for s in range(warmup + steps):
        c0 = (s * cols) % max(1, n - cols)
        t0 = time.perf_counter()
        o.compute_matrix_cols(FREQ, c0, c0 + cols)
        t_fill = (time.perf_counter() - t0) * (n / cols)
        t1 = time.perf_counter()
        V = o.rhs_plane_wave(FREQ, 0.0, 0.0, 1.0, 0.0)
        I = o.solve(Zfull, V)
        o.lump(FREQ, I)
        o.rcs(R_FAR, T, P)
        t_rest = time.perf_counter() - t1
        if s >= warmup:
            times.append(t_fill + t_rest)
    sample = (f"per step: fill of {cols}/{n} columns (scaled x{n / cols:.1f}), full zgetrf+zgetrs (N={n}), "
              f"lumping, 362-point far field")
    return times, os.cpu_count(), sample


def cpu_sample_sweep(mesh, freqs, pws, feed_tags, pts):
    """FRICO's CPU path for the bowtie sweep on a bounded sample of frequencies: per
    frequency the fill of n/16 columns (scaled), zgetrf + zgetrs with the 4 right-hand
    sides, port values, and per right-hand side the lumping and the 8-point field."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    o = Oracle(mesh)
    tags = list(feed_tags)
    signs = o.reorient(tags)
    n = o.n
    cols = max(64, n // 16)
    Z = o.compute_matrix(freqs[0])   # zgetrf's time does not depend on the frequency
    times = []
    for k, f in enumerate(freqs):
        c0 = (k * cols) % max(1, n - cols)
        t0 = time.perf_counter()
        o.compute_matrix_cols(f, c0, c0 + cols)
        t_fill = (time.perf_counter() - t0) * (n / cols)
        t1 = time.perf_counter()
        V = np.stack([o.rhs_delta_gap(f, tags, 1.0, signs)] +
                     [o.rhs_plane_wave(f, pw.theta, pw.phi, pw.Etheta, pw.Ephi) for pw in pws], axis=1)
        I = o.solve(Z, V)
        o.port_values(I[:, 0], o.rwg(), tags, 1.0, signs)
        for c in range(I.shape[1]):
            o.lump(f, I[:, c])
            o.eval_fields(pts)
        times.append(t_fill + time.perf_counter() - t1)
    sample = (f"{len(freqs)} frequencies of the band: fill of {cols}/{n} columns (scaled x{n / cols:.1f}), "
              f"zgetrf+zgetrs with 4 RHS, port values, lumping and 8-point fields per RHS")
    return times, os.cpu_count(), sample


def cpu_sample_sphere64(mesh, f0, pws, T, P):
    """FRICO's CPU path for the 64-incidence L5 step on a bounded sample: fill of n/64
    columns (scaled), zgetrf + zgetrs of an n/4 system with the 64 right-hand sides
    (scaled by (n / (n/4))^3 = 64), and lumping + fields of 8 of the 64 currents at
    1024 of the points (scaled by 8 and by the point count)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    from frico_gb300 import meshes
    o = Oracle(mesh)
    n = o.n
    cols = max(64, n // 64)
    t0 = time.perf_counter()
    o.compute_matrix_cols(f0, 0, cols)
    t_fill = (time.perf_counter() - t0) * (n / cols)
    m = n // 4
    rng = np.random.default_rng(7)
    A = (rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))) + 4.0 * np.sqrt(m) * np.eye(m)
    B = rng.standard_normal((m, len(pws))) + 0j
    t1 = time.perf_counter()
    o.solve(A, B)
    t_lu = (time.perf_counter() - t1) * (n / m) ** 3
    cur = o.rhs_plane_wave(f0, pws[0].theta, pws[0].phi, pws[0].Etheta, pws[0].Ephi)   # any current vector
    idx = np.random.default_rng(5).choice(T.size, 1024, replace=False)
    pts = meshes.sph2rect(R_FAR, T[idx], P[idx])
    t2 = time.perf_counter()
    for _ in range(8):
        o.lump(f0, cur)
        o.eval_fields(pts)
    t_fields = (time.perf_counter() - t2) * (len(pws) / 8) * (T.size / 1024)
    sample = (f"fill of {cols}/{n} columns (scaled x{n / cols:.0f}); zgetrf+zgetrs of a {m} x {m} system with "
              f"{len(pws)} RHS (scaled x{(n / m) ** 3:.0f}); lumping + fields of 8 currents at 1024 of the "
              f"{T.size} points (scaled x{len(pws) / 8 * T.size / 1024:.0f})")
    return t_fill + t_lu + t_fields, os.cpu_count(), sample


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from frico_gb300 import meshes
    mesh = meshes.icosphere(args.level)
    times, cores, sample = cpu_sample(mesh, args.steps, args.warmup)
    t = sum(times)
    value = len(times) / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * t / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded icosphere)", "config": {"workload": WORKLOAD, "precision": "fp64 (LAPACK)"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FP64_NOMINAL_TFLOPS = 1.25   # GB300 FP64 (vector and tensor), nominal; a DFMA loop on one GB300 measured 1.255


def stage_rooflines(stage, steps, n, nt, npts, iters, green_evals, precision, hbm, bf16, f16=False):
    """Per-stage achieved rate against its bound, with the work counts of the
    stage table: fill = Green evaluations x 105 flops (FP64) and Z bytes
    written; LU = 8/3 N^3 (mixed: 3 split products on the tensor cores, FP16
    at the dense bf16 rate or TF32 at half of it); refinement = 16 N^2 bytes of
    FP64 Z per residual; fields = Nobs Nt (30 + 90) flops (FP64)."""
    per = {k: v / steps / 1000.0 for k, v in stage.items()}   # seconds per step
    out = {}
    # the mixed path's fill and fields run in double-float on the FP32 pipe: their FP64-accurate work
    # is reported as an FP64-equivalent rate, with no fraction of the FP64 pipe's peak
    dfl = precision == "mixed"
    if per["fill_ms"] > 0:
        zb = (16.0 + (8.0 if precision == "mixed" else 0.0)) * n * n
        fl = 105.0 * green_evals
        rate = fl / per["fill_ms"] / 1e12
        out["fill"] = ({"fp64_equiv_tflops": rate, "pipe": "double-float on the FP32 pipe"} if dfl else
                       {"fp64_tflops": rate, "fp64_frac_of_nominal": rate / FP64_NOMINAL_TFLOPS})
        out["fill"].update({"z_write_gbs": zb / per["fill_ms"] / 1e9, "hbm_frac": zb / per["fill_ms"] / 1e9 / hbm})
    if per["factor_ms"] > 0:
        t = (8.0 / 3.0) * n ** 3 / per["factor_ms"] / 1e12
        mixed_peak = bf16 if f16 else bf16 / 2.0
        out["lu"] = {"algorithmic_tflops": t,
                     "frac": t * (3.0 if precision == "mixed" else 1.0) / (mixed_peak if precision == "mixed"
                                                                            else FP64_NOMINAL_TFLOPS),
                     "peak": ("FP16 = measured bf16 (3xFP16 does 3 products)" if f16 else
                              "TF32 = measured bf16 / 2 (3xTF32 does 3 products)") if precision == "mixed"
                     else "FP64 nominal"}
    if per["refine_ms"] > 0 and iters and iters[-1] > 0:
        gbs = 16.0 * n * n * iters[-1] / per["refine_ms"] / 1e9
        out["refine"] = {"residual_gbs_equiv": gbs, "hbm_frac": gbs / hbm, "iters": iters[-1],
                         "note": "whole refinement stage (residuals + triangular solves) against the residuals' Z reads"}
    if per["fields_ms"] > 0:
        rate = npts * nt * 120.0 / per["fields_ms"] / 1e12
        out["fields"] = ({"fp64_equiv_tflops": rate, "pipe": "double-float on the FP32 pipe"} if dfl else
                         {"fp64_tflops": rate, "fp64_frac_of_nominal": rate / FP64_NOMINAL_TFLOPS})
    return out


# ------------------------------------------------------------------ GPU path
def run_ours(args):
    ws, rank, local = dist_env()
    from frico_gb300.replicas import ReplicaGroup
    dist = ReplicaGroup(ws, rank)   # independent replicas: barrier + max of times only
    import ctypes as C
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import _abi, meshes
    from frico_gb300.solver import PlaneWave, Simulation

    mesh = meshes.icosphere(args.level)
    T, P, _ = meshes.bistatic_cuts(R_FAR)
    sim = Simulation(mesh, precision=args.precision, device=local, profile_kernels=False,
                     gemm_engine=args.gemm_engine, pivoting=args.pivoting)
    lib = sim.lib
    n = sim.n
    pw = PlaneWave(0.0, 0.0, 1.0, 0.0)
    stream = C.c_void_p()
    lib.frico_gpu_get_stream(sim.ctx, C.byref(stream))
    import torch
    torch.cuda.set_device(local)
    ext = torch.cuda.ExternalStream(stream.value, device=local)

    def step():
        sim.compute_matrix(FREQ)
        sim.set_nrhs(1)
        sim.update_rhs(FREQ, pw)
        sim.solve(download=False)
        return sim.rcs_points(R_FAR, T, P)

    for _ in range(args.warmup):
        step()
    s0 = sim.stats()
    clocks = ClockSampler(local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    stage = {k: 0.0 for k in ("fill_ms", "rhs_ms", "factor_ms", "solve_ms", "refine_ms", "fields_ms")}
    iters = []
    for _ in range(args.steps):
        sig = step()
        st = sim.stats()
        for k in stage:
            stage[k] += st[k]
        iters.append(st["refine_iters"])
    e1.record(ext)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    dist.barrier()
    clk = clocks.stop()
    s1 = sim.stats()
    ms_max = dist.max(ms)
    value = ws * args.steps / (ms_max / 1000.0)

    # -- end to end through the C-ABI with host buffers (mesh in, currents + sigma out)
    fs = sim.fs
    I_host = np.empty((n, 1), np.complex128, order="F")
    th = np.ascontiguousarray(T)
    ph = np.ascontiguousarray(P)
    sig_host = np.empty((T.shape[0], 2))
    info = C.c_int32(0)
    h2d = fs.vertices.nbytes + fs.triangles.nbytes + fs.rwg.nbytes + 3 * 8 * T.shape[0]
    d2h = I_host.nbytes + 3 * 16 * T.shape[0]

    def e2e_step():
        sim._call("frico_gpu_set_mesh", fs.vertices.shape[0], _abi.ptr(fs.vertices), fs.triangles.shape[0],
                  _abi.ptr(fs.triangles), n, _abi.ptr(fs.rwg))
        sim._call("frico_gpu_fill", FREQ, None, n)
        sim._call("frico_gpu_set_nrhs", 1)
        sim._call("frico_gpu_rhs_plane_wave", FREQ, 0, 0.0, 0.0, _abi.C128(1.0, 0.0), _abi.C128(0.0, 0.0))
        sim._call("frico_gpu_solve", _abi.ptr(I_host), n, C.byref(info))
        sim._call("frico_gpu_rcs_points", 0, R_FAR, T.shape[0], _abi.ptr(th), _abi.ptr(ph), _abi.ptr(sig_host))

    e2e_step()
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = ws * args.steps / e2e_s

    # -- roofline of the LU's GEMMs (the O(N^3) kernel), timed live with CUDA events on
    #    the library's stream around every launch, in two extra profiled steps after the
    #    timed region (profiling runs the factorisation eagerly instead of as a graph)
    sim.set_options(profile_kernels=1)
    p0 = sim.stats()
    for _ in range(2):
        step()
    p1 = sim.stats()
    sim.set_options(profile_kernels=0)
    gl = p1["gemm_launches"] - p0["gemm_launches"]
    gms = p1["gemm_ms"] - p0["gemm_ms"]
    gfl = p1["gemm_flops"] - p0["gemm_flops"]
    gby = p1["gemm_bytes"] - p0["gemm_bytes"]
    hbm, bf16, peak_src = measured_peaks()
    sec = gms / 1000.0 if gms > 0 else float("inf")
    tc = args.precision == "mixed" and args.gemm_engine != "simt"
    # the unpivoted LU's block columns run 3xFP16 when asked for; everything else 3xTF32
    f16 = tc and args.gemm_engine == "tc_f16" and s1["pivoting_used"] == 2
    # trailing updates on SM pairs, the narrow update of the next block column on single SMs
    kernel = (("tc::k_gemm_pair_f16x3 + tc::k_gemm_f16x3" if f16 else "tc::k_gemm_pair_tf32x3 + tc::k_gemm_tf32x3")
              if tc else "k_gemm_update<float>")
    # tensor work of the split path: 3 real GEMMs of (2m x 2k)(2k x n) = 3 x algorithmic complex flops;
    # FP16 dense peak = the measured dense bf16 peak, TF32 = half of it
    tflops_alg = gfl / sec / 1e12
    tensor_ach = 3.0 * tflops_alg if tc else tflops_alg
    tensor_peak = (bf16 if f16 else bf16 / 2.0) if tc else bf16
    gbs = gby / sec / 1e9
    frac_t, frac_m = tensor_ach / tensor_peak, gbs / hbm
    if tc and frac_t >= frac_m:
        roof = {"bound": "tensor", "achieved": tensor_ach, "peak": tensor_peak, "unit": "TFLOP/s", "frac": frac_t}
    else:
        roof = {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": frac_m}
    roof.update({"traffic": gemm_traffic_per_launch(args.level, args.precision, kernel.replace("tc::", ""))
                 if tc else None,
                 "traffic_unit": "bytes per launch (ncu, DRAM read + write)",
                 "algorithmic_bytes_per_launch": gby / max(1, gl),
                 "kernel": kernel if args.precision == "mixed" else "k_gemm_update<double>",
                 "launches_per_step": gl / 2, "avg_launch_us": 1000.0 * gms / max(1, gl),
                 "algorithmic_tflops_complex": tflops_alg, "hbm_gbs_algorithmic": gbs,
                 "hbm_frac": frac_m, "tensor_frac": frac_t if tc else None,
                 "note": f"peaks: hbm {hbm} GB/s, dense bf16 {bf16} TF/s ({peak_src}); "
                         + ("FP16 = bf16" if f16 else "TF32 = bf16/2")})

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": "synthetic (seeded icosphere L%d)" % args.level,
            "config": {"workload": WORKLOAD.replace("L4_N7680", f"L{args.level}_N{n}"), "n": n, "ntri": sim.nt,
                       "precision": args.precision, "rhs": 1, "far_field_points": int(T.shape[0]),
                       "l2": "working set > L2 (Z 0.94 GB)", "replicas": ws},
            "stages_ms_per_step": {k: v / args.steps for k, v in stage.items()},
            "stages_roofline": stage_rooflines(stage, args.steps, n, sim.nt, int(T.shape[0]), iters,
                                               s1["green_evals"], args.precision, hbm, bf16, f16),
            "refine_iters": iters[-1] if iters else 0,
            "pivoting_used": {1: "partial", 2: "none"}.get(s1["pivoting_used"], "?"),
            "gpu_launches": int(s1["kernel_launches"] - s0["kernel_launches"]),
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "roofline": roof, "clocks": clk}
    if rank == 0 and args.precision == "mixed" and not args.no_accuracy:
        # the metric's reference point, the plain FP64 GPU drop-in on the same workload in the
        # same run: one untimed step (which also gives the accuracy reference), then
        # `fp64_steps` timed steps with CUDA events on its stream
        ref = Simulation(mesh, precision="fp64", device=local)
        rstream = C.c_void_p()
        lib.frico_gpu_get_stream(ref.ctx, C.byref(rstream))
        rext = torch.cuda.ExternalStream(rstream.value, device=local)

        def step64():
            ref.compute_matrix(FREQ)
            ref.set_nrhs(1)
            ref.update_rhs(FREQ, pw)
            ref.solve(download=False)
            return ref.rcs_points(R_FAR, T, P)

        step64()
        I_64 = ref.solve()[:, 0]      # factors kept: the solve is repeated, not refactored
        sig_64 = ref.rcs_points(R_FAR, T, P)
        E_64, _ = ref.eval_fields(meshes.sph2rect(R_FAR, T, P))
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(rext)
        for _ in range(args.fp64_steps):
            step64()
        f1.record(rext)
        torch.cuda.synchronize()
        fp64_value = args.fp64_steps / (f0.elapsed_time(f1) / 1000.0)
        ref.close()
        line["fp64_gpu_value"] = fp64_value
        line["fp64_gpu_steps"] = args.fp64_steps
        line["mixed_over_fp64"] = value / fp64_value
        sim.compute_matrix(FREQ)
        sim.set_nrhs(1)
        sim.update_rhs(FREQ, pw)
        I_mx = sim.solve()[:, 0]
        sig_mx = sim.rcs_points(R_FAR, T, P)
        E_mx, _ = sim.eval_fields(meshes.sph2rect(R_FAR, T, P))
        line["accuracy_vs_fp64_gpu"] = {
            "currents_rel_l2": float(np.linalg.norm(I_mx - I_64) / np.linalg.norm(I_64)),
            "far_field_E_rel_l2": float(np.linalg.norm(E_mx - E_64) / np.linalg.norm(E_64)),
            "sigma_rel_max": float(np.max(np.abs(sig_mx - sig_64)) / np.max(np.abs(sig_64))),
            "bound": 1e-6}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        Zfull = sim.compute_matrix(FREQ, download=True)
        times, cores, sample = cpu_sample(mesh, 1, 0, Zfull)
        line["cpu_baseline"] = {"value": 1.0 / times[0], "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": sample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
    dist.close()


# ------------------------------------------------------------------ sweep workload
def run_sweep(args):
    """Bowtie sweep: N ~ 500/1500/3000, 256 frequencies in [200, 800] MHz, 4 right-hand
    sides per frequency (delta-gap feed + plane waves (0,0,theta), (45,0,theta),
    (90,90,phi)), port values and E at 8 far-field points per RHS. One step = the
    whole sweep through frico_gpu_sweep (host inputs, host outputs), so the
    step time is also the end-to-end time."""
    ws, rank, local = dist_env()
    from frico_gb300.replicas import ReplicaGroup, shard
    dist = ReplicaGroup(ws, rank)
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import meshes
    from frico_gb300.solver import DeltaGap, PlaneWave, Simulation
    import torch
    torch.cuda.set_device(local)
    mesh = meshes.bowtie_preset(args.sweep_n)
    all_freqs = meshes.sweep_frequencies(200e6, 800e6, args.sweep_freqs)
    freqs = np.array(shard(list(all_freqs), rank, ws))   # weak scaling: each replica its own frequencies
    d = np.pi / 180
    pws = (PlaneWave(0.0, 0.0, 1.0, 0.0), PlaneWave(45 * d, 0.0, 1.0, 0.0), PlaneWave(90 * d, 90 * d, 0.0, 1.0))
    feed = DeltaGap((meshes.FEED_TAG,), 1.0)
    pts = meshes.sph2rect(10.0, np.linspace(0, 180, 8) * d, np.zeros(8))
    sim = Simulation(mesh, precision=args.precision, device=local, gemm_engine=args.gemm_engine,
                     pivoting=args.pivoting)
    for _ in range(args.warmup):
        out = sim.sweep(freqs, feed, pws, pts, lanes=args.lanes)
    clocks = ClockSampler(local)
    dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    reps = []
    for _ in range(args.steps):
        out = sim.sweep(freqs, feed, pws, pts, lanes=args.lanes)
        reps.append(out["report"])
    torch.cuda.synchronize()
    sec = dist.max(time.perf_counter() - t0)
    dist.barrier()
    clk = clocks.stop()
    nsys = len(all_freqs) * args.steps
    value = nsys / sec
    r = reps[-1]
    nf = max(1, len(freqs))
    n = sim.n
    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": f"synthetic (seeded bowtie N={n})",
            "config": {"workload": f"bowtie_sweep_N{n}_{len(all_freqs)}freq_4rhs", "n": n, "ntri": sim.nt,
                       "precision": args.precision, "frequencies": int(len(all_freqs)), "rhs_per_frequency": 4,
                       "far_field_points_per_rhs": 8, "lanes": r["lanes"], "autotuned": bool(r["autotuned"]),
                       "solve_unit": "one frequency system (fill + LU + 4 RHS + port + fields)",
                       "l2": "per-lane Z %.0f MB; lanes' Z together %s L2" % (
                           16 * n * n / 1e6, ">" if 16 * n * n * r["lanes"] > 129e6 else "<"),
                       "replicas": ws},
            "stages_ms_per_frequency": {k: r[k] / nf for k in ("fill_ms", "rhs_ms", "factor_ms", "solve_ms",
                                                                "refine_ms", "fields_ms")},
            "max_refine_iters": r["max_refine_iters"], "partial_pivot_fallbacks": r["partial_pivot_fallbacks"],
            "fp64_fallbacks": r["fp64_fallbacks"], "fp64_direct": r["fp64_direct"],
            "gpu_launches": int(sum(x["kernel_launches"] for x in reps)),
            "e2e": {"value": value, "unit": "solves/s",
                    "h2d_bytes_per_step": int(freqs.nbytes + pts.nbytes + 6 * 8 * 3),
                    "d2h_bytes_per_step": int(nf * (4 * 8 * 3 * 16 + 88))},
            "clocks": clk}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cf = list(all_freqs[:: max(1, len(all_freqs) // 4)])[:4]
        ctimes, cores, csample = cpu_sample_sweep(mesh, cf, pws, feed.interfaces, pts)
        line["cpu_baseline"] = {"value": len(ctimes) / sum(ctimes), "unit": "solves/s", "cores": cores,
                                "kind": "port", "sample": csample}
    if rank == 0:
        print(json.dumps(line), flush=True)
    sim.close()
    dist.close()


# ------------------------------------------------------------------ adjoint workload
def run_adjoint(args):
    """Bowtie N ~ 3000 at 500 MHz: gradients of Re Zin, Im Zin and |E(0, 0, 10 m)|^2
    with respect to every vertex coordinate, the flare angle and the frequency.
    One step = frico_gpu_adjoint (fill, LU, solve, transposed solve, reverse pass
    over the fill) + the flare chain rule. --validate K compares K seeded random
    directions with central differences (step 1e-6 wavelength) of the forward
    path, outside the timed region."""
    ws, rank, local = dist_env()
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import meshes
    from frico_gb300.solver import DeltaGap, Simulation
    import torch
    torch.cuda.set_device(local)
    nx, ny = meshes.BOWTIE_PRESETS[args.sweep_n]
    mesh = meshes.bowtie(nx, ny)
    f0 = 500e6
    feed = DeltaGap((meshes.FEED_TAG,), 1.0)
    P = np.array([0.0, 0.0, 10.0])
    tang = meshes.bowtie_flare_tangent(nx, ny)
    sim = Simulation(mesh, precision=args.precision, device=local)

    def step():
        out = sim.adjoint(f0, feed, P)
        G = np.stack([out["grad_zin_re"], out["grad_zin_im"], out["grad_e2"]])
        return out, G, np.einsum("kvc,vc->k", G, tang)

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out, G, dflare = step()
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    clk = clocks.stop()
    # one forward solve, the unit a finite-difference gradient would repeat 2 (3 nv + 2) times
    fwd = Simulation(mesh, precision=args.precision, device=local)
    fwd.run_context(f0, feed)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(3):
        fwd.run_context(f0, feed)
        fwd.port_values(feed)
        fwd.eval_fields(P[None, :])
    torch.cuda.synchronize()
    t_fwd = (time.perf_counter() - t1) / 3
    fwd.close()
    line = {"metric": "adjoint gradient evaluations/s", "value": args.steps / sec, "unit": "evals/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * sec / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128" if args.precision == "mixed" else "c128", "data": f"synthetic (seeded bowtie N={sim.n})",
            "config": {"workload": f"bowtie_adjoint_N{sim.n}_500MHz", "n": sim.n, "nv": int(mesh.nv),
                       "parameters": 3 * int(mesh.nv) + 2, "objectives": ["Re Zin", "Im Zin", "|E(0,0,10)|^2"],
                       "precision": args.precision},
            "zin": [out["zin"].real, out["zin"].imag], "e2": out["e2"],
            "d_dflare": list(map(float, dflare)),
            "d_df": [out["dzin_df"].real, out["dzin_df"].imag, out["de2_df"]],
            "forward_solve_ms": 1000 * t_fwd,
            "finite_difference_equivalent_ms": 1000 * t_fwd * 2 * (3 * mesh.nv + 2),
            "e2e": {"value": args.steps / sec, "unit": "evals/s", "h2d_bytes_per_step": 8 * 3,
                    "d2h_bytes_per_step": 3 * 8 * 3 * int(mesh.nv)},
            "clocks": clk}
    if args.validate:
        C0 = 1.0 / np.sqrt(1.256637061435917e-06 * 8.8541878188e-12)
        h = 1e-6 * C0 / f0
        rng = np.random.default_rng(20260104)

        def J(verts):
            m = meshes.bowtie(nx, ny)
            m.vertices = verts
            s2 = Simulation(m, precision="fp64", device=local)
            s2.run_context(f0, feed)
            z = s2.port_values(feed)["impedance"]
            E, _ = s2.eval_fields(P[None, :])
            s2.close()
            return np.array([z.real, z.imag, float(np.sum(np.abs(E) ** 2))])

        errs = []
        scale = np.linalg.norm(G.reshape(3, -1), axis=1)
        for _ in range(args.validate):
            d = rng.standard_normal(mesh.vertices.shape)
            d /= np.linalg.norm(d)
            fd = (J(mesh.vertices + h * d) - J(mesh.vertices - h * d)) / (2 * h)
            errs.append(np.abs(np.einsum("kvc,vc->k", G, d) - fd) / scale)
        line["validation"] = {"directions": args.validate, "step_m": h,
                              "max_err_over_grad_norm": list(map(float, np.max(errs, axis=0)))}
    print(json.dumps(line), flush=True)
    sim.close()


# ------------------------------------------------------------------ strip dipole (CPU-runnable case)
def run_strip(args):
    """Strip dipole N = 119 at 300 MHz (1 V delta gap): Zin and E on the 1-degree
    theta x phi grid (181 x 360 = 65 160 points at R = 10 m). Launch-latency bound
    at this size; reported, not optimised."""
    ws, rank, local = dist_env()
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import meshes
    from frico_gb300.solver import DeltaGap, Simulation
    import torch
    torch.cuda.set_device(local)
    mesh = meshes.strip_dipole()
    f0 = 300e6
    dg = DeltaGap((meshes.FEED_TAG,), 1.0)
    _, _, pts = meshes.far_field_grid(R_FAR, 1.0)
    sim = Simulation(mesh, precision=args.precision, device=local)

    def step():
        sim.run_context(f0, dg)
        pv = sim.port_values(dg)
        E, _ = sim.eval_fields(pts)
        return pv["impedance"], E

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        zin, E = step()
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    clk = clocks.stop()
    line = {"metric": METRIC, "value": args.steps / sec, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128" if args.precision == "fp64" else "c64+c128",
            "data": "synthetic (strip dipole 60 x 1)",
            "config": {"workload": "strip_N119_300MHz_deltagap_farfield181x360", "n": sim.n,
                       "precision": args.precision, "far_field_points": int(pts.shape[0])},
            "zin": [zin.real, zin.imag],
            "e2e": {"value": args.steps / sec, "unit": "solves/s", "h2d_bytes_per_step": int(pts.nbytes),
                    "d2h_bytes_per_step": int(2 * E.nbytes)},
            "clocks": clk}
    print(json.dumps(line), flush=True)
    sim.close()


# ------------------------------------------------------------------ many-incidence workload
def run_sphere64(args):
    """Sphere level 5 (N = 30 720) at 900 MHz, 64 plane waves theta_i = i 180/63 deg,
    phi = 0, polarisation alternating theta / phi, sigma_VV and sigma_HH of every
    incidence on the 181 x 361 (theta x phi) grid at R = 10 m (65 341 points).
    One step = fill + one 64-RHS solve + the multi-column field pass, timed on
    the host clock around device-synchronised calls."""
    ws, rank, local = dist_env()
    import frico_gb300
    frico_gb300.build()
    from frico_gb300 import meshes
    from frico_gb300.solver import PlaneWave, Simulation
    import torch
    torch.cuda.set_device(local)
    level = args.level if args.level != 4 else 5
    mesh = meshes.icosphere(level)
    f0 = 900e6 if level == 5 else 450e6
    nrhs = 64
    th_in = np.arange(nrhs) * np.pi / (nrhs - 1)
    pws = [PlaneWave(float(t), 0.0, 1.0 if i % 2 == 0 else 0.0, 0.0 if i % 2 == 0 else 1.0)
           for i, t in enumerate(th_in)]
    th = np.radians(np.arange(181.0))
    ph = np.radians(np.arange(361.0))
    T, Pg = np.meshgrid(th, ph, indexing="ij")
    T, Pg = T.ravel(), Pg.ravel()
    sim = Simulation(mesh, precision=args.precision, device=local, gemm_engine=args.gemm_engine,
                     pivoting=args.pivoting)
    stage = {k: 0.0 for k in ("fill_ms", "factor_ms", "refine_ms", "solve_ms", "fields_ms")}

    def step():
        sim.compute_matrix(f0)
        sim.set_nrhs(nrhs)
        for c, pw in enumerate(pws):
            sim.update_rhs(f0, pw, c)
        sim.solve(download=False)
        st = sim.stats()
        sig = sim.rcs_points_multi(R_FAR, T, Pg)
        st2 = sim.stats()
        return sig, st, st2

    for _ in range(args.warmup):
        step()
    clocks = ClockSampler(local)
    torch.cuda.synchronize()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sig, st, st2 = step()
        for k in ("fill_ms", "factor_ms", "refine_ms", "solve_ms"):
            stage[k] += st[k]
        stage["fields_ms"] += st2["fields_ms"]
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    clk = clocks.stop()
    n = sim.n
    line = {"metric": METRIC, "value": args.steps / sec, "unit": "solves/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sec / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c64+c128" if args.precision == "mixed" else "c128",
            "data": f"synthetic (seeded icosphere L{level})",
            "config": {"workload": f"sphere_L{level}_N{n}_{f0 / 1e6:.0f}MHz_64planewaves_bistatic181x361",
                       "n": n, "ntri": sim.nt, "precision": args.precision, "rhs": nrhs,
                       "far_field_points": int(T.shape[0]), "z_bytes": 16 * n * n},
            "stages_ms_per_step": {k: v / args.steps for k, v in stage.items()},
            "refine_iters": st["refine_iters"], "precision_used": st["precision_used"],
            "sigma_checksum": float(np.sum(sig)),
            "e2e": {"value": args.steps / sec, "unit": "solves/s", "h2d_bytes_per_step": int(16 * T.shape[0]),
                    "d2h_bytes_per_step": int(sig.nbytes)},
            "clocks": clk}
    if args.precision == "mixed" and not args.no_accuracy:
        # the field pass's engine (tensor-core GEMMs for many columns on the mixed path) against the
        # direct double-float kernels on 2000 seeded points of the grid, every incidence
        idx = np.random.default_rng(5).choice(T.size, 2000, replace=False)
        sim.set_options(fields_engine=1)
        sig_d = sim.rcs_points_multi(R_FAR, T[idx], Pg[idx])
        sim.set_options(fields_engine=0)
        sig_s = sig[:, idx]
        line["fields_vs_direct"] = {
            "sigma_rel_max": float(max(np.abs(sig_s[c] - sig_d[c]).max() / np.abs(sig_d[c]).max()
                                       for c in range(nrhs))),
            "points": 2000, "engine": "tensor-core GEMM (auto)", "bound": 1e-6}
    if not args.no_cpu_baseline:
        csec, cores, csample = cpu_sample_sphere64(mesh, f0, pws, T, Pg)
        line["cpu_baseline"] = {"value": 1.0 / csec, "unit": "solves/s", "cores": cores, "kind": "port",
                                "sample": csample}
    print(json.dumps(line), flush=True)
    sim.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "sphere64":
        run_sphere64(args)
    elif args.workload == "strip":
        run_strip(args)
    elif args.workload == "sweep":
        run_sweep(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
