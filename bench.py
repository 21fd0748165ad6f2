#!/usr/bin/env python
"""Benchmark: log-evidence + gradient evaluations per second on one GB300.

Workload (the K = 1e6 configuration): K = 1,000,000 visibilities, a 100 x 100
image grid at 0.04" with a 2.4" circular mask (M = 9,504 image pixels),
S = 1,500 Delaunay source pixels (3 barycentric weights per image pixel).
w_tilde (M x M, float64) is precomputed once and shared by every evaluation,
as in the reference (numba.py:814).  One step = one lens-model evaluation:
logE (numba.py:761-857) and its adjoint (dlogE/dlambda, dlogE/dweights), with
the regularisation coefficient cycling through lambda in {1e-3, 1e-1, 1e1, 1e3}.

Inputs are synthetic with the configuration's shapes and distributions (the
reference's dataset is not public); w_tilde alone (722 MB) exceeds L2
(129 MB), so no explicit L2 flush is needed between steps.

`--impl reference` times the reference's algorithm on the host cores: the
NumPy restatement of numba.py (the oracle) for logE plus the closed-form
adjoint, on the same shapes (w_tilde is built from a visibility sample, since
its values do not change the per-evaluation cost).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "python-autojax_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

LAMBDAS = (1e-3, 1e-1, 1e1, 1e3)
METRIC = "logE+grad evals/s (mixed precision; K=1e6, M=9504, S=1500)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--config", default="cfg3")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the cpu_baseline leg")
    ap.add_argument("--skip-wtilde", action="store_true", help="omit the w_tilde kernel measurement")
    ap.add_argument("--stages", action="store_true", help="also time the pipeline stages separately")
    ap.add_argument("--skip-batch", action="store_true", help="omit the batched many-model measurement")
    ap.add_argument("--skip-roofline", action="store_true", help="omit the standalone roofline group (for ncu)")
    ap.add_argument("--batch", type=int, default=64, help="lens models in the batched measurement")
    ap.add_argument("--only", choices=("roofline", "wtilde"), help="run one kernel measurement alone (for ncu)")
    ap.add_argument("--tile-policy", help="fixed tile policy 'update,inverse' instead of tuning (for ncu)")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers


class Dist:
    def __init__(self, gpus: int):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            backend = "nccl"
            import torch

            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
            else:
                backend = "gloo"
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg is not None:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if self.pg is None:
            return x
        import torch

        dev = torch.device("cuda", self.local) if torch.cuda.is_available() else torch.device("cpu")
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg is not None:
            self.pg.destroy_process_group()


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        self.path = Path(tempfile.gettempdir()) / f"aj_bench_clocks_{os.getpid()}.csv"
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the timed region starts once the sampler is producing lines
        t_end = time.time() + 3.0
        while time.time() < t_end and self.path.stat().st_size == 0:
            time.sleep(0.01)

    def stop(self, t0: float | None = None, t1: float | None = None) -> dict:
        """Summarise the samples taken between host times t0 and t1 (the timed region); if none
        fell inside it, the nearest ones (the result says which)."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.05)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                ts = time.mktime(time.strptime(parts[0].split(".")[0], "%Y/%m/%d %H:%M:%S"))
                ts += float("0." + parts[0].split(".")[1]) if "." in parts[0] else 0.0
                rows.append((ts, float(parts[2]), float(parts[3]),
                             {n for n, v in zip(names, parts[6:10]) if v.lower() in ("active", "1", "0x1")}))
            except (ValueError, IndexError):
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        inside = [r for r in rows if t0 is not None and t1 is not None and t0 <= r[0] <= t1]
        where = "timed region"
        if not inside:
            mid = 0.5 * (t0 + t1) if t0 is not None and t1 is not None else rows[-1][0]
            inside = sorted(rows, key=lambda r: abs(r[0] - mid))[:3]
            where = "nearest to the timed region (none fell inside it)"
        reasons = sorted(set().union(*(r[3] for r in inside)))
        return {"sm_mhz": float(np.median([r[1] for r in inside])), "sm_max_mhz": max(r[2] for r in inside),
                "reasons": reasons, "samples": len(inside), "sampled": where}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


_DATASETS: dict = {}


def dataset(name: str):
    from autojax_gb300 import synthetic

    if name not in _DATASETS:
        _DATASETS[name] = synthetic.make_dataset(name)
    return _DATASETS[name]


def models(d: dict, n: int = len(LAMBDAS)):
    """The per-step lens models: the dataset's mapping and mesh with the lambda schedule."""
    return [(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["neighbors"],
             d["neighbors_sizes"], float(np.sqrt(lam))) for lam in LAMBDAS[:n]]


# --------------------------------------------------------------- GPU arm


def fma_peak_tflops(precision: int) -> float:
    """FMA issue rate of this GPU (a register-only probe kernel of the library)."""
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks = sms * 8
    iters = 20000 if precision == _lib.AJ_MIXED else 400
    out = torch.empty(blocks * 256, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    lib.aj_probe_fma(precision, blocks, 10, out.data_ptr(), st.cuda_stream)
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        _lib.check(lib.aj_probe_fma(precision, blocks, iters, out.data_ptr(), st.cuda_stream), "aj_probe_fma")
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        best = max(best, 2.0 * 128 * iters * blocks * 256 / (ms * 1e-3) / 1e12)
    return best


def time_region(fn, steps: int, dist: Dist, name: str = "region") -> float:
    """Max over ranks of the CUDA-event time of `steps` calls of fn (barrier + synchronize on both sides).

    The region is an NVTX range ``bench:<name>`` so a profiler can keep only its launches.
    """
    import torch

    dist.barrier()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push(f"bench:{name}")
    e0.record(st)
    for i in range(steps):
        fn(i)
    e1.record(st)
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    dist.barrier()
    return dist.max(e0.elapsed_time(e1) / 1e3)


# DRAM bytes (read + write) of one aj_spd_inverse_mixed call at S = 1,500, summed
# over its launches in a warm-cache ncu capture of one call (9.9 MB read,
# 108.3 MB written): the group's working set, the double-float S x S planes and
# the tensor-core product's digit planes (74 MB together), stays in L2.
ROOFLINE_TRAFFIC_BYTES = 118.2e6


def roofline(A, dist: Dist, tune_policy: bool = True):
    """Roofline of the dominant kernel group of the mixed path: the double-float
    factorisation chain (Cholesky panel, trailing updates, triangular inverse,
    L^-T L^-1), run standalone through aj_spd_inverse_mixed on the S x S matrix
    A and timed with CUDA events on the launching stream.

    Algorithmic work: S^3 float64-class flops (S^3/3 each for the factor, the
    inverse factor and L^-T L^-1).  Peak: the measured float32 FMA rate over the
    11.4 float32 instructions one double-float multiply-add takes (2 flops).
    The float64 path's aj_spd_inverse does the same work on the FP64 pipe.
    """
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    dev = A.device
    S = A.shape[0]
    Ainv = torch.empty((S, S), dtype=torch.float64, device=dev)
    ld = torch.empty(1, dtype=torch.float64, device=dev)
    info = torch.zeros(2, dtype=torch.int32, device=dev)
    stc = torch.cuda.current_stream().cuda_stream
    ws_m = torch.empty(lib.aj_spd_inverse_mixed_workspace_size(S), dtype=torch.uint8, device=dev)
    ws_f = torch.empty(lib.aj_spd_inverse_workspace_size(S), dtype=torch.uint8, device=dev)

    def inv_mixed(i):
        _lib.check(lib.aj_spd_inverse_mixed(A.data_ptr(), S, Ainv.data_ptr(), ld.data_ptr(), ws_m.data_ptr(),
                                            ws_m.numel(), info.data_ptr(), stc), "aj_spd_inverse_mixed")

    def inv_fp64(i):
        _lib.check(lib.aj_spd_inverse(A.data_ptr(), S, Ainv.data_ptr(), ld.data_ptr(), ws_f.data_ptr(), ws_f.numel(),
                                      info.data_ptr(), stc), "aj_spd_inverse")

    for i in range(3):
        inv_mixed(i)
        inv_fp64(i)
    torch.cuda.synchronize()
    if int(info[0]) != 0:
        raise RuntimeError(f"roofline matrix not positive definite (info {info.tolist()})")
    # the group alone shares the GPU differently from a whole evaluation (no H factorisation, no
    # gathers beside it): time it with the tile policy tuned for this call, then restore the
    # evaluation's
    from autojax_gb300 import tune

    saved = tune.get_tile_policy()
    policy = tune.tune_tile_policy(lambda: inv_mixed(0), reps=3)["policy"] if tune_policy else saved
    reps = 5
    try:
        t_inv_mixed = time_region(inv_mixed, reps, dist, "roofline_mixed") / reps
    finally:
        tune.set_tile_policy(*saved)
    t_inv_fp64 = time_region(inv_fp64, reps, dist, "roofline_fp64") / reps

    # the same float64 work through the vendor's solver (torch.linalg: cuSOLVER/MAGMA), for scale
    def inv_vendor(i):
        L, _ = torch.linalg.cholesky_ex(A)
        torch.cholesky_inverse(L)

    try:
        inv_vendor(0)
        t_inv_vendor = time_region(inv_vendor, reps, dist, "roofline_fp64_vendor") / reps
    except RuntimeError:  # torch's linear-algebra library may be unavailable (e.g. under a profiler)
        t_inv_vendor = None
    fp64_peak = fma_peak_tflops(_lib.AJ_FP64)
    fp32_peak = fma_peak_tflops(_lib.AJ_MIXED)
    df_peak = fp32_peak / 11.4
    inv_flops = float(S) ** 3
    achieved = inv_flops / t_inv_mixed / 1e12
    roof = {
        "kernel": "double-float Cholesky + triangular inverse of A, then L^-T L^-1 on the tensor cores "
                  "(aj_spd_inverse_mixed: dfchol_panel, dfsyrk_update, df_trtri_step, digit_syrk)",
        "bound": "fp32 (double-float)",
        "achieved": achieved,
        "peak": df_peak,
        "unit": "TFLOP/s (float64-class)",
        "frac": achieved / df_peak,
        "peak_source": "measured in this run: aj_probe_fma float32 FMA rate / 11.4 float32 instructions "
                       "per double-float multiply-add",
        "traffic": ROOFLINE_TRAFFIC_BYTES,
        "S": S,
        "tile_policy": list(policy),
        "ms": 1e3 * t_inv_mixed,
        "fp64_same_work_ms": 1e3 * t_inv_fp64,
        "fp64_same_work_frac_of_fp64_peak": inv_flops / t_inv_fp64 / 1e12 / fp64_peak,
        "fp64_vendor_same_work_ms": 1e3 * t_inv_vendor if t_inv_vendor else None,
        "fp64_vendor_note": "torch.linalg.cholesky_ex + torch.cholesky_inverse in float64 on the same A "
                            "(the vendor solver, not this library): a reference point for the float64 path",
    }
    # the same launch against the measured peaks (neither bounds a float32-pipe group)
    mp = measured_peaks()
    roof["frac_vs_measured_peaks"] = {
        "bf16_tflops_sustained": (achieved / mp["bf16_tflops_sustained"]) if mp.get("bf16_tflops_sustained") else None,
        "hbm_gbs": (ROOFLINE_TRAFFIC_BYTES / t_inv_mixed / 1e9 / mp["hbm_gbs"]) if mp.get("hbm_gbs") else None,
        "note": "achieved float64-class TFLOP/s over the sustained bf16 tensor peak, and the group's DRAM "
                "traffic per call over the timed duration against the copy bandwidth (MEASURED_PEAKS.json)",
    }
    return roof, fp64_peak, fp32_peak


def roofline_only(args, dist: Dist) -> dict:
    """The roofline group alone on a synthetic SPD matrix of the workload's S (the
    kernels' work does not depend on the values): a small-memory run for ncu."""
    import torch

    torch.cuda.set_device(dist.local)
    if args.tile_policy:
        from autojax_gb300 import tune

        tune.set_tile_policy(*(int(v) for v in args.tile_policy.split(",")))
    S = 1500
    rng = np.random.default_rng(3)
    X = rng.standard_normal((S, S))
    A = torch.from_numpy(X @ X.T / S + np.eye(S)).cuda()
    roof, fp64_peak, fp32_peak = roofline(A, dist, tune_policy=False)
    return {"roofline": roof, "peaks": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak}}


def gpu_arm(args, dist: Dist) -> dict:
    import torch

    import autojax_gb300 as aj
    from autojax_gb300 import _lib
    from autojax_gb300.inversion import LogEvidence

    torch.cuda.set_device(dist.local)
    lib = _lib.load()
    d = dataset(args.config)
    M, K, S = d["M"], d["K"], d["S"]
    dev = torch.device("cuda", dist.local)
    # shared w_tilde (float64), built on the device from the compact table and expanded
    noise_real = torch.from_numpy(d["noise_map_real"]).to(dev)
    uv = torch.from_numpy(d["uv_wavelengths"]).to(dev)
    w_compact = aj.w_compact_curvature_interferometer_from(d["grid_size"], noise_real, uv, d["pixel_scale"])
    native = torch.from_numpy(d["native_index_for_slim_index"]).to(dev)
    w_tilde = aj.w_tilde_via_compact_from(w_compact, native)
    torch.cuda.synchronize()
    B, P = d["pix_indexes_for_sub_slim_index"].shape[1], d["neighbors"].shape[1]
    common = dict(S=S, B=B, P=P, with_grad=True, device=dev)
    ev = {prec: LogEvidence(d["dirty_image"], d["data"], d["noise_map"], w_tilde, precision=prec, **common)
          for prec in ("mixed", "fp64")}
    mods = models(d)
    for e in ev.values():
        e.set_model(*mods[0][:4], coefficient=mods[0][4])
    # tile shapes of the double-float factorisation, chosen by timing this evaluation
    from autojax_gb300 import tune

    if args.tile_policy:
        tune.set_tile_policy(*(int(v) for v in args.tile_policy.split(",")))
        tuned = {"policy": tune.get_tile_policy(), "ms": None, "ms_default": None, "candidates_timed": 0}
    else:
        # timed as graph replays when the bench replays graphs (a graph keeps its capture's policy)
        em = ev["mixed"]
        tuned = (tune.tune_tile_policy(em.launch) if args.no_graph
                 else tune.tune_tile_policy(em.step, prepare=em.capture))
    for e in ev.values():
        if not args.no_graph:
            e.capture()
    coefs = [torch.full((1,), m[4], dtype=torch.float64, device=dev) for m in mods]

    def stepper(e):
        def f(i):
            e.coefficient.copy_(coefs[i % len(coefs)])
            e.step()
        return f

    # accuracy of the mixed path against the float64 path over the lambda schedule
    rel = []
    mixed_vals = {"logE": [], "s": []}
    for c in coefs:
        vals = {}
        for prec, e in ev.items():
            e.coefficient.copy_(c)
            e.step()
            torch.cuda.synchronize()
            e.check()
            vals[prec] = e.out.cpu().numpy().copy()
        rel.append(abs(vals["mixed"][0] - vals["fp64"][0]) / abs(vals["fp64"][0]))
        mixed_vals["logE"].append(float(vals["mixed"][0]))
        mixed_vals["s"].append(ev["mixed"].reconstruction.cpu().numpy().copy())

    for e in ev.values():
        f = stepper(e)
        for i in range(args.warmup):
            f(i)
    torch.cuda.synchronize()

    clk = ClockSampler(dist.local)
    clk.start()
    c0 = time.time()
    t_mixed = time_region(stepper(ev["mixed"]), args.steps, dist, "timed_mixed")
    clocks = clk.stop(c0, time.time())
    t_fp64 = time_region(stepper(ev["fp64"]), args.steps, dist, "timed_fp64")
    ev["mixed"].check()

    # end to end through the public evaluator: host NumPy inputs -> pinned H2D -> evaluation -> D2H
    e = ev["mixed"]
    for i in range(args.warmup):
        e.evaluate_host(*mods[i % len(mods)])
    dist.barrier()
    t0 = time.perf_counter()
    for i in range(args.steps):
        e.evaluate_host(*mods[i % len(mods)])
    t_e2e = dist.max(time.perf_counter() - t0)

    # roofline of the dominant kernel group, timed standalone on this workload's A = F + H
    A = torch.from_numpy(aj.constant_regularization_matrix_from(1.0, d["neighbors"], d["neighbors_sizes"])).to(dev)
    F = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(
        w_tilde, torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).to(dev),
        torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev), S)
    A = (A + F).contiguous()
    if args.skip_roofline:
        roof, fp64_peak, fp32_peak = None, fma_peak_tflops(_lib.AJ_FP64), fma_peak_tflops(_lib.AJ_MIXED)
    else:
        roof, fp64_peak, fp32_peak = roofline(A, dist, tune_policy=not args.tile_policy)
    del F

    result = {
        "metric": METRIC,
        "value": args.steps * dist.world / t_mixed,
        "unit": "evals/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * t_mixed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "df32 (double-float) + f64",
        "data": "synthetic (seeded; shapes and distributions of the K=1e6 configuration)",
        "config": {
            "workload": f"{args.config}: K={K} visibilities, M={M} image pixels (100x100 at 0.04\", r=2.4\"), "
                        f"S={S} Delaunay source pixels, B={B}; w_tilde precomputed (float64, resident)",
            "lambdas": list(LAMBDAS),
            "l2": "inputs larger than L2 (w_tilde 722 MB float64 re-read every step)",
            "graph": not args.no_graph,
            "parallelism": f"replicas x{dist.world}",
            "tile_policy": {"min_64_tiles (update, L^-1)": list(tuned["policy"]),
                            "tuned_ms": tuned["ms"], "default_ms": tuned["ms_default"],
                            "candidates_timed": tuned["candidates_timed"]},
        },
        "fp64_path": {"value": args.steps * dist.world / t_fp64, "ms_per_step": 1e3 * t_fp64 / args.steps,
                      # five S^3/6 multiply-add passes (Cholesky of A and H, L^-1 of both, L^-T L^-1)
                      "fp64_pipe_floor_ms": 1e3 * 5 * S**3 / 6 * 2 / (fp64_peak * 1e12),
                      "mixed_over_fp64_pipe_floor": (5 * S**3 / 6 * 2 / (fp64_peak * 1e12)) / (t_mixed / args.steps)},
        "mixed_over_fp64": t_fp64 / t_mixed,
        "max_rel_dlogE_mixed_vs_fp64": max(rel),
        "e2e": {"value": args.steps * dist.world / t_e2e, "unit": "evals/s", "h2d_bytes_per_step": e.h2d_bytes(),
                "d2h_bytes_per_step": e.d2h_bytes()},
        "gpu_launches": (ev["mixed"].launches_per_eval or 0) * args.steps,
        "roofline": roof,
        "peaks": {"fp64_tflops": fp64_peak, "fp32_tflops": fp32_peak,
                  "hbm_gbs": measured_peaks().get("hbm_gbs"), "bf16_tflops": measured_peaks().get("bf16_tflops")},
        "clocks": clocks,
    }
    if not args.skip_wtilde:
        result["w_tilde"] = wtilde_bench(d, dev, fp32_peak)
    if dist.rank == 0 and dist.world == 1 and not args.skip_cpu:
        # the checker, after every timed region
        result["err_vs_oracle"] = oracle_errors(d, w_tilde, mixed_vals, result.get("w_tilde"))
    result.get("w_tilde", {}).pop("sample", None)
    if args.stages:
        result["stages_ms"] = stage_times(d, w_tilde, dev, dist)
    if not args.skip_batch:
        del ev, A, w_tilde, w_compact
        torch.cuda.empty_cache()
        result["batched"] = batched_bench(args, dev, dist)
    return result


def batched_bench(args, dev, dist: Dist) -> dict:
    """Many lens models against one dataset (the batched configuration).

    K = 500,000 visibilities, a 100 x 100 grid at 0.04" with a 2.0" mask
    (~8,000 image pixels), ``--batch`` lens models with S uniform in
    [500, 2000], Einstein radius uniform in [0.6", 1.2"] and lambda
    log-uniform in [1e-3, 1e3]; mixed precision with gradients.  One step is
    one replay of the captured batch graph (every model evaluated once);
    ``sequential`` replays the models' own single-evaluation graphs one after
    another on the same inputs.
    """
    import torch

    import autojax_gb300 as aj
    from autojax_gb300 import synthetic
    from autojax_gb300.inversion import Dataset, LogEvidenceBatch

    d = dataset("cfg5")
    noise_real = torch.from_numpy(d["noise_map_real"]).to(dev)
    uv = torch.from_numpy(d["uv_wavelengths"]).to(dev)
    w_compact = aj.w_compact_curvature_interferometer_from(d["grid_size"], noise_real, uv, d["pixel_scale"])
    w_tilde = aj.w_tilde_via_compact_from(w_compact, torch.from_numpy(d["native_index_for_slim_index"]).to(dev))
    ds = Dataset(d["dirty_image"], d["data"], d["noise_map"], w_tilde, precision="mixed", device=dev)
    lm = synthetic.lens_models(d, args.batch, seed=55 + dist.rank)
    P = max(m["neighbors"].shape[1] for m in lm)
    batch = LogEvidenceBatch(ds, [m["S"] for m in lm], B=3, P=P)
    for i, m in enumerate(lm):
        batch.set_model(i, m["pix_indexes_for_sub_slim_index"], m["pix_weights_for_sub_slim_index"], m["neighbors"],
                        m["neighbors_sizes"], m["coefficient"])
    # the tile policy for throughput: many evaluations in flight favour the bigger tiles that the
    # latency-bound single evaluation avoids (results do not depend on the policy)
    from autojax_gb300 import tune

    single_policy = tune.get_tile_policy()
    batch.capture()
    if args.tile_policy:
        tuned = {"policy": single_policy, "candidates_timed": 0}
    else:
        tuned = tune.tune_tile_policy(batch.step, prepare=batch.capture, reps=2, rounds=1)
    for _ in range(max(2, args.warmup)):
        batch.step()
    torch.cuda.synchronize()
    batch.check()
    steps = 5
    t = time_region(lambda i: batch.step(), steps, dist, "timed_batch")
    batch.check()
    # one graph at a time, each captured with the single evaluation's policy
    tune.set_tile_policy(*single_policy)
    for e in batch.evals:
        e.capture()
    for e in batch.evals:
        e.step()
    t_seq = time_region(lambda i: [e.step() for e in batch.evals], 1, dist, "timed_batch_sequential")
    for e in batch.evals:
        e.release_graph()
    n = batch.n
    Ss = [m["S"] for m in lm]
    return {
        "workload": f"cfg5: K={d['K']} visibilities, M={d['M']} image pixels (100x100 at 0.04\", r=2.0\"); "
                    f"{n} lens models, S uniform in [500, 2000] (drawn {min(Ss)}..{max(Ss)}), Einstein radius "
                    f"uniform in [0.6, 1.2]\", lambda log-uniform in [1e-3, 1e3]; mixed precision with gradients",
        "value": steps * n * dist.world / t,
        "unit": "evals/s",
        "ms_per_batch": 1e3 * t / steps,
        "sequential_value": n * dist.world / t_seq,
        "batched_over_sequential": t_seq / (t / steps),
        "launches_per_batch": batch.launches_per_batch,
        "graph": True,
        "tile_policy": {"batch": list(tuned["policy"]), "sequential": list(single_policy),
                        "candidates_timed": tuned["candidates_timed"]},
    }


def wtilde_bench(d, dev, fp32_peak, Ks: int = 65536) -> dict:
    """Direct w_tilde build (numba.py:156-207) on the workload's M with a visibility sample.

    The mixed build cuts the float64 panel into 7 exact 7-bit digits and sums the 28 digit pairs
    of levels 0..6 on the bf16 tensor cores: 2 x 28 digit multiply-adds (112 bf16 flops) per unique
    (pixel pair, visibility) term of the computed tiles.  Reported against the measured bf16 peak,
    and under the fixed convention of 20 float32 flops a term (phase, cos, Kahan accumulate)
    against the measured float32 FMA rate, the unit the w_tilde target is stated in.
    """
    import torch

    from autojax_gb300 import _lib

    lib = _lib.load()
    Ks = min(Ks, d["K"])
    g = torch.from_numpy(d["grid_radians_slim"]).to(dev)
    uv = torch.from_numpy(d["uv_wavelengths"][:Ks].copy()).to(dev)
    n = torch.from_numpy(d["noise_map_real"][:Ks].copy()).to(dev)
    M = g.shape[0]
    W = torch.empty((M, M), dtype=torch.float64, device=dev)
    planes = torch.empty((2, M, M), dtype=torch.float32, device=dev)
    pc = _lib.AJ_MIXED
    ws = torch.empty(lib.aj_w_tilde_curvature_workspace_size(Ks, M, pc), dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream()

    def call():
        _lib.check(lib.aj_w_tilde_curvature(n.data_ptr(), uv.data_ptr(), g.data_ptr(), Ks, M, W.data_ptr(),
                                            planes.data_ptr(), ws.data_ptr(), ws.numel(), pc, st.cuda_stream),
                   "aj_w_tilde_curvature")

    call()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    call()
    e1.record(st)
    e1.synchronize()
    sec = e0.elapsed_time(e1) / 1e3
    terms = M * (M + 1) / 2 * Ks
    Mp = (M + 127) // 128 * 128
    tile_terms = (Mp // 128) * (Mp // 128 + 1) * 128 * 64 * Ks  # the computed tiles' (pair, visibility) terms
    bf16_tflops = tile_terms * 112 / sec / 1e12
    mp = measured_peaks()
    rng = np.random.default_rng(17)
    rows = np.repeat(np.array([0, M // 3, M // 2, M - 1]), 64)
    cols = rng.integers(0, M, rows.size)
    cols[::64] = rows[::64]
    Wh = W.cpu().numpy()
    return {"precision": "mixed: float64 panel cut into 7 exact 7-bit digits, digit products on the bf16 tensor "
                         "cores (tcgen05), folded into double-float",
            "K_sample": Ks, "M": M, "seconds": sec, "terms_per_s": terms / sec,
            "fp32_convention_frac": terms / sec * 20 / 1e12 / fp32_peak,
            "fp32_convention_note": "unique terms x 20 float32 flops a term over the measured float32 FMA rate",
            "tensor_tflops": bf16_tflops,
            "bf16_tensor_frac": bf16_tflops / mp["bf16_tflops"] if mp.get("bf16_tflops") else None,
            "tensor_note": "112 bf16 flops (2 rows x 28 digit pairs) per term of the computed 128 x 64 tiles, "
                           "over MEASURED_PEAKS.json's bf16 burst peak",
            "sample": {"rows": rows, "cols": cols, "values": Wh[rows, cols],
                       "noise": d["noise_map_real"][:Ks].copy(), "uv": d["uv_wavelengths"][:Ks].copy()}}


def stage_times(d, w_tilde, dev, dist) -> dict:
    import torch

    import autojax_gb300 as aj

    idx = torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).to(dev)
    w = torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev)
    S = d["S"]
    out = {}
    for name, fn in (
        ("curvature_sparse_f64", lambda i: aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(w_tilde, idx, w, S)),
        ("regularization", lambda i: aj.constant_regularization_matrix_from(1.0, torch.from_numpy(d["neighbors"]).to(dev),
                                                                            torch.from_numpy(d["neighbors_sizes"]).to(dev))),
    ):
        fn(0)
        out[name] = 1e3 * time_region(fn, 3, dist) / 3
    return out


# -------------------------------------------------------------- CPU legs


def cpu_eval_setup(d: dict):
    """w_tilde for the host legs at the workload's full K: the offset table by the oracle's
    separable host product (seconds on host cores), expanded as numba.py:238-255 does."""
    from oracle import numpy_port as ref

    wc = ref.w_compact_separable(d["grid_size"], d["noise_map_real"], d["uv_wavelengths"], d["pixel_scale"])
    return ref.w_tilde_via_compact_from(wc, d["native_index_for_slim_index"])


def cpu_time(d: dict, W, evals: int) -> tuple[float, int]:
    from oracle import adjoint

    mods = models(d)
    t0 = time.perf_counter()
    for i in range(evals):
        idx, w, nb, nsz, c = mods[i % len(mods)]
        adjoint.log_evidence_and_grad(d["dirty_image"], d["data"], d["noise_map"], W, idx, w, nb, nsz, coefficient=c)
    return time.perf_counter() - t0, evals


def cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(d: dict, W, budget_s: float = 20.0) -> dict:
    sec1, _ = cpu_time(d, W, 1)
    n = max(1, min(20, int(budget_s / max(sec1, 1e-3))))
    sec, n = cpu_time(d, W, n)
    return {"value": n / sec, "unit": "evals/s", "cores": cores(), "kind": "port",
            "sample": f"{n} logE+grad evaluations of the workload (NumPy port of numba.py logE + closed-form "
                      "adjoint; w_tilde at the workload's full K, as the GPU arm uses)"}


def reference_module():
    """The reference's own numba.py from baseline/_ref (placed by baseline/stage_reference.py),
    or None.  Without numba on the host its functions run un-jitted through a pass-through shim
    (jit returns the function, prange is range), i.e. as the reference's NumPy source."""
    import types

    ref_dir = ROOT / "baseline" / "_ref"
    if not (ref_dir / "autojax" / "numba.py").exists():
        return None, "baseline/_ref not staged"
    try:
        import numba  # noqa: F401

        how = "Numba JIT"
    except ImportError:
        shim = types.ModuleType("numba")

        def jit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        shim.jit = shim.njit = jit
        shim.prange = range
        sys.modules["numba"] = shim
        how = "numba absent: the reference's Numba source executed as NumPy, not JIT"
    if str(ref_dir) not in sys.path:
        sys.path.insert(0, str(ref_dir))
    from autojax import numba as ref_numba

    return ref_numba, how


def reference_time(mod, d: dict, W, evals: int) -> tuple[float, int]:
    """The reference's log_likelihood_function_via_w_tilde_from (numba.py:761-857), unmodified:
    logE only (the reference has no gradient) with its hard-coded coefficient 1.0."""
    args = (d["dirty_image"], d["data"], d["noise_map"], W, d["pix_indexes_for_sub_slim_index"],
            d["pix_weights_for_sub_slim_index"], d["neighbors"], d["neighbors_sizes"])
    t0 = time.perf_counter()
    for _ in range(evals):
        mod.log_likelihood_function_via_w_tilde_from(*args)
    return time.perf_counter() - t0, evals


def oracle_errors(d: dict, w_tilde_dev, lm: dict, wt: dict | None) -> dict:
    """Errors of the mixed path against the oracle (the checker) on the workload: logE and s at
    every lambda of the schedule and F, all given the GPU's float64 w_tilde; w_tilde from the
    mixed direct build on its visibility sample against the oracle's sums on sampled entries."""
    import torch

    import autojax_gb300 as aj
    from oracle import numpy_port as ref

    W = w_tilde_dev.cpu().numpy()
    T = ref.mapping_matrix_from(d["pix_indexes_for_sub_slim_index"], d["pix_weights_for_sub_slim_index"], d["S"])
    F_ref = ref.curvature_matrix_via_w_tilde_from(W, T)
    D_ref = ref.data_vector_from(T, d["dirty_image"])
    dev = w_tilde_dev.device
    F = aj.curvature_matrix_via_w_wilde_sparse_mapping_matrix_from(
        w_tilde_dev, torch.from_numpy(d["pix_indexes_for_sub_slim_index"]).to(dev),
        torch.from_numpy(d["pix_weights_for_sub_slim_index"]).to(dev), d["S"], precision="mixed").cpu().numpy()
    out = {"F": {"max_abs_err_over_max_abs": float(np.abs(F - F_ref).max() / np.abs(F_ref).max())},
           "logE": [], "s": []}
    for lam, logE_mixed, s_mixed in zip(LAMBDAS, lm["logE"], lm["s"]):
        H = ref.constant_regularization_matrix_from(float(np.sqrt(lam)), d["neighbors"], d["neighbors_sizes"])
        r_logE = ref._evidence(d["noise_map"], d["data"], F_ref, H, D_ref)
        A = F_ref + H
        s_ref = np.linalg.solve(A, D_ref)
        ev = np.linalg.eigvalsh(A)
        out["logE"].append({"lambda": lam, "rel_err": abs(logE_mixed - r_logE) / abs(r_logE), "oracle": r_logE})
        out["s"].append({"lambda": lam, "rel_err": float(np.linalg.norm(s_mixed - s_ref) / np.linalg.norm(s_ref)),
                         "cond_A": float(ev[-1] / ev[0])})
    if wt is not None and "sample" in wt:
        smp = wt.pop("sample")
        rows, cols = smp["rows"], smp["cols"]
        exp = ref.w_tilde_entries(smp["noise"], smp["uv"], d["grid_radians_slim"], rows, cols)
        scale = float(np.abs(exp[rows == cols]).max())
        out["w_tilde"] = {"max_abs_err_over_scale": float(np.abs(smp["values"] - exp).max() / scale),
                          "entries": int(rows.size), "K_sample": int(smp["uv"].shape[0]),
                          "scale": "largest diagonal entry"}
    out["checker"] = "oracle/numpy_port.py (NumPy/LAPACK restatement of numba.py), same inputs"
    return out


def reference_arm(args, dist: Dist) -> dict:
    d = dataset(args.config)
    W = cpu_eval_setup(d)
    mod, how = reference_module()
    # the port's logE + gradient beside the reference's own logE
    sec_p, n_p = cpu_time(d, W, max(1, min(args.steps, 5)))
    port = {"value": n_p / sec_p, "unit": "logE+grad evals/s", "kind": "port",
            "sample": f"{n_p} evaluations: numba.py logE restated in NumPy + the closed-form adjoint"}
    if mod is not None:
        for _ in range(max(0, min(args.warmup, 1))):
            reference_time(mod, d, W, 1)
        sec, n = reference_time(mod, d, W, args.steps)
        kind, what = "reference", (f"{n} calls of the reference's own log_likelihood_function_via_w_tilde_from "
                                   f"(numba.py:761-857, logE only: the reference has no gradient; {how})")
    else:
        for _ in range(max(0, min(args.warmup, 1))):
            cpu_time(d, W, 1)
        sec, n = cpu_time(d, W, args.steps)
        kind, what = "port", (f"{n} logE+grad evaluations of the NumPy port ({how}); numba.py logE restated in "
                              "NumPy + the closed-form adjoint")
    v = n / sec
    return {
        "metric": METRIC,
        "impl": "reference",
        "value": v,
        "unit": "evals/s",
        "n_gpus": dist.world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * sec / n,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded; shapes and distributions of the K=1e6 configuration)",
        "config": {"workload": f"{args.config}: K={d['K']}, M={d['M']}, S={d['S']}; w_tilde at the full K "
                               "(float64, precomputed as in numba.py:814)",
                   "lambdas": list(LAMBDAS), "same_config": True},
        "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores(), "kind": kind, "sample": what},
        "port_logE_grad": port,
        "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    dist = Dist(args.gpus)
    try:
        if args.impl == "reference":
            if dist.rank != 0:
                return
            print(json.dumps(reference_arm(args, dist)), flush=True)
            return
        if args.only == "roofline":
            res = roofline_only(args, dist)
        elif args.only == "wtilde":
            import torch

            torch.cuda.set_device(dist.local)
            res = {"w_tilde": wtilde_bench(dataset(args.config), torch.device("cuda", dist.local),
                                           fma_peak_tflops(1))}
            res["w_tilde"].pop("sample", None)
        else:
            res = gpu_arm(args, dist)
        if dist.rank == 0 and dist.world == 1 and not args.skip_cpu and not args.only:
            d = dataset(args.config)
            res["cpu_baseline"] = cpu_baseline(d, cpu_eval_setup(d))
        if dist.rank == 0:
            print(json.dumps(res), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
