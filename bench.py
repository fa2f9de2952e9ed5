"""Benchmark: -2lnL + gradient evaluations per second at nside 16, lmax 47.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--path mixed|fp64] [--batch B] [--no-cpu-baseline]

A step is one batched evaluation of B C_l vectors (lognormal 10% per-l
perturbations of C_l = 1e3 2pi/(l(l+1))) on one seeded synthetic map, returning
-2lnL and d(-2lnL)/dC_l for each vector.  ``value`` is evaluations/s with
inputs resident in HBM (device-pointer entry point); ``e2e`` is the same
through the host-pointer C ABI from pinned buffers, copies included.
Multi-GPU: one process per GPU, each with its own batch (replicas: batch
elements are independent), max-over-ranks time, value summed over ranks.

``--impl reference`` times the reference algorithm on the host cores: the
oracle restatement of clToCMatrix + Likelihood (dpptrf/dpptri) + calculate,
plus the FP64 adjoint gradient, at the same configuration.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "nside16_lmax47_b256"
METRIC = "lnL+grad evals/sec at nside16 lmax47, batched mixed vs plain FP64 GPU, |delta|<=1e-3"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-compare-batch", type=int, default=None,
                    help="elements the plain FP64 path evaluates for the mixed/FP64 ratio and the error bars "
                         "(default: the whole batch)")
    ap.add_argument("--workload", default=WORKLOAD, help="named workload in cosmopp_gb300.workload.WORKLOADS")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default launch shapes (or the tuning file's) instead of autotuning")
    ap.add_argument("--hmc-iters", type=int, default=12, help="batched-HMC iterations reported beside the line "
                                                              "(64 chains x 20 leapfrog steps of 0.05); 0 = skip")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device=None):
    """The largest of every rank's x: the job's time is its slowest rank's (all ranks call it)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(batch_per_rank, world, ms_per_step):
    """Evaluations/s of the whole job: every rank evaluates its own batch each step (replicas)."""
    return batch_per_rank * world / (ms_per_step / 1000.0)


def rank_batch_seed(rank):
    """Seed of a rank's C_l batch: each replica evaluates different vectors."""
    return 7 + rank


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def make_inputs(wl, cg):
    """Seeded data map d = L z, L from the FP64 covariance built by the library (input generation)."""
    from cosmopp_gb300 import workload as W
    ctx = cg.Context(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
                     noise_sigma=wl.sigma, max_batch=1, precision="fp64")
    c = ctx.build_cmatrix(wl.cl_fid)
    ctx.close()
    full = W.packed_to_full(c, wl.n) + wl.sigma ** 2 * np.eye(wl.n)
    return W.draw_data(full, wl.z)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def cpu_baseline(wl, d, seconds_budget=20.0):
    """The reference algorithm (oracle restatement, O(lmax^2) Legendre restarts as the
    reference does) on this host's cores, for a bounded sample of the batch."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    nest = O.ring2nest(wl.nside, wl.ring_kept)
    xyz = O.unit_vectors(wl.nside, nest, "NEST")
    t0 = time.perf_counter()
    done = 0
    while True:
        O.evaluate(wl.cl_batch[done % len(wl.cl_batch)], xyz, wl.fwhm_deg, wl.sigma ** 2, d, grad=True, restart=True)
        done += 1
        if time.perf_counter() - t0 > seconds_budget or done >= 4:
            break
    el = time.perf_counter() - t0
    return {"value": done / el, "unit": "evals/s", "cores": cores, "kind": "port",
            "sample": "%d evaluation(s) of the %d-vector batch (clToCMatrix with per-l Legendre restarts + "
                      "dpptrf/dpptri Likelihood + calculate + FP64 adjoint), %.1f s" % (done, len(wl.cl_batch), el)}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    # the workload module is pure numpy: importing it does not load the product library
    from cosmopp_gb300 import workload as W
    from oracle import oracle as O
    wl = W.make(args.workload, batch=args.batch)
    # data map from the oracle's own FP64 covariance (no GPU on this arm)
    O.build()
    nest = O.ring2nest(wl.nside, wl.ring_kept)
    xyz = O.unit_vectors(wl.nside, nest, "NEST")
    c = O.cl_to_cmatrix(wl.cl_fid, xyz, wl.fwhm_deg)
    d = W.draw_data(W.packed_to_full(c, wl.n) + wl.sigma ** 2 * np.eye(wl.n), wl.z)
    cores = os.cpu_count() or 1
    O.set_threads(cores)
    for k in range(args.warmup):
        O.evaluate(wl.cl_batch[k % len(wl.cl_batch)], xyz, wl.fwhm_deg, wl.sigma ** 2, d, grad=True, restart=True)
    t0 = time.perf_counter()
    for k in range(args.steps):
        O.evaluate(wl.cl_batch[k % len(wl.cl_batch)], xyz, wl.fwhm_deg, wl.sigma ** 2, d, grad=True, restart=True)
    el = time.perf_counter() - t0
    v = args.steps / el
    out = {"metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": args.workload, "nside": wl.nside, "lmax": wl.lmax, "n_pixels": wl.n,
                      "sample": "one C_l vector per step"},
           "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                            "sample": "%d steps x 1 evaluation (clToCMatrix with per-l Legendre restarts, "
                                      "dpptrf/dpptri, calculate, FP64 adjoint)" % args.steps},
           "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    import cosmopp_gb300 as cg
    from cosmopp_gb300 import workload as W
    wl = W.make(args.workload, batch=args.batch, batch_seed=rank_batch_seed(rank))
    B = len(wl.cl_batch)
    d = make_inputs(wl, cg)
    path = args.path
    ctx = cg.Context(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept, scheme="RING",
                     noise_sigma=wl.sigma, max_batch=B, precision=path, device=local,
                     cl_ref=wl.cl_fid if path == "mixed" else None, recenter="fixed")
    L1 = wl.lmax + 1
    tuning = None
    if path == "mixed":
        # launch shapes: the tuning file's entry for this device and shape, else an autotune run
        # (one coordinate pass, CUDA-event timed) appended to the file
        tune_file = os.environ.get("COSMOPP_GB300_TUNE_FILE") or os.path.join(ROOT, "cosmopp_gb300", "_lib",
                                                                               "tune.txt")
        t0 = time.perf_counter()
        found = ctx.tune_load(tune_file)
        tune_ms = None if (found or args.no_autotune) else ctx.autotune(B, tune_file)
        tuning = {"knobs": ctx.tuning(),
                  "source": "tuning file" if found else ("defaults" if args.no_autotune else "autotuned in this run"),
                  "file": os.path.relpath(tune_file, ROOT), "autotune_ms_per_call": tune_ms,
                  "seconds": round(time.perf_counter() - t0, 2)}
    plan = ctx.memory_plan()
    plan180 = cg.plan_memory(180 * 10 ** 9, lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside,
                             good_pixels=wl.ring_kept, scheme="RING", noise_sigma=wl.sigma, max_batch=B,
                             precision=path)
    admission = {"bytes_fixed_gb": round(plan["bytes_fixed"] / 1e9, 3),
                 "bytes_per_element_gb": round(plan["bytes_per_element"] / 1e9, 4),
                 "free_gb_at_create": round(plan["bytes_budget"] / 1e9, 1), "chunk": plan["chunk"],
                 "batch_total_gb": round((plan["bytes_fixed"] + B * plan["bytes_per_element"]) / 1e9, 2),
                 "max_batch_in_180gb": plan180["max_batch_fit"]}
    dev = torch.device("cuda", local)
    # a few distinct batches, cycled so that no two consecutive steps see the same inputs
    nb = 4
    cls = torch.tensor(np.stack([W.lognormal_batch(wl.cl_fid, B, 100 + 17 * rank + k) for k in range(nb)]),
                       dtype=torch.float64, device=dev)
    dd = torch.tensor(d, dtype=torch.float64, device=dev)
    m2 = torch.empty(B, dtype=torch.float64, device=dev)
    chi2 = torch.empty_like(m2)
    ld = torch.empty_like(m2)
    grad = torch.empty(B, L1, dtype=torch.float64, device=dev)
    st = torch.empty(B, dtype=torch.int32, device=dev)
    # an explicit stream: the library launches there and the events bracket exactly that work
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0

    def step(k):
        ctx.loglike_device(B, cls[k % nb].data_ptr(), dd.data_ptr(), 0, m2.data_ptr(), chi2.data_ptr(),
                           ld.data_ptr(), grad.data_ptr(), st.data_ptr(), sp)

    for k in range(max(3, args.warmup)):
        step(k)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = ctx.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for k in range(args.steps):
        step(k)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = (ctx.launch_count() - launches0) // args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms, world, dev)
    value = job_throughput(B, world, ms)
    assert int(st.sum().item()) == 0, "non-OK element status in the timed batch"

    # end to end through the host-pointer C ABI from pinned buffers
    cl_h = torch.empty(nb, B, L1, dtype=torch.float64).pin_memory()
    cl_h.copy_(cls.cpu())
    d_h = torch.empty(wl.n, dtype=torch.float64).pin_memory()
    d_h.copy_(dd.cpu())
    outs = [torch.empty(B, dtype=torch.float64).pin_memory() for _ in range(3)]
    g_h = torch.empty(B, L1, dtype=torch.float64).pin_memory()
    st_h = torch.empty(B, dtype=torch.int32).pin_memory()
    L = cg.library()
    import ctypes

    def e2e_step(k):
        rc = L.cg_loglike(ctx.handle, B, ctypes.cast(cl_h[k % nb].data_ptr(), cg._dp),
                          ctypes.cast(d_h.data_ptr(), cg._dp), 0, ctypes.cast(outs[0].data_ptr(), cg._dp),
                          ctypes.cast(outs[1].data_ptr(), cg._dp), ctypes.cast(outs[2].data_ptr(), cg._dp),
                          ctypes.cast(g_h.data_ptr(), cg._dp), ctypes.cast(st_h.data_ptr(), cg._ip))
        assert rc == 0
    for k in range(2):
        e2e_step(k)
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    e2e_ms = (time.perf_counter() - t0) * 1000.0 / args.steps
    e2e_ms = max_over_ranks(e2e_ms, world, dev)
    h2d = B * L1 * 8 + wl.n * 8
    d2h = B * (3 * 8 + L1 * 8 + 4)

    # per-stage times (profiled pass after the timed region) and the roofline of the top stage; the
    # profiled pass runs the launches in sequence (knob overlap = 0), so that each stage is its own
    # kernels' time (the timed region runs trtri's rows beside the Cholesky where the knob is set)
    ov = ctx.tune_get("overlap") if path == "mixed" else 0
    if ov:
        ctx.tune_set("overlap", 0)
    ctx.set_profiling(True)
    stages = {}
    nprof = 3
    for k in range(nprof):
        step(k)
        for nm, v in ctx.stage_times().items():
            stages[nm] = stages.get(nm, 0.0) + v / nprof
    ctx.set_profiling(False)
    if ov:
        ctx.tune_set("overlap", ov)
    torch.cuda.synchronize()
    peaks, peak_kind = load_peaks()
    tf32 = None
    if path == "mixed":
        # the tensor-core peak of the factorisation kernels' own MMA form, measured now, with the clocks
        pc = ClockSampler(local)
        pc.start()
        rates = [ctx.probe_tf32_rate(1 << 16, 10)[0] for _ in range(4)]
        f32 = [ctx.probe_fp32_rate(1 << 14, 10)[0] for _ in range(4)]
        tf32 = {"tflops": max(rates), "fp32_fma2_tflops": max(f32), "clocks": pc.stop(),
                "form": "tcgen05.mma kind::tf32 M128 N128 K8, A in tensor memory, B in shared memory, one issuing "
                        "thread per SM (cg_probe_tf32_rate); FP32: packed fma.rn.f32x2 chains (cg_probe_fp32_rate)"}
    n, N = wl.n, ((wl.n + 127) // 128) * 128  # the library pads to an even number of 64-tiles
    pairs = n * (n + 1) // 2
    roof_build = None
    if path == "mixed":
        # The dominant kernel: the tensor-core Cholesky (chol_tc_update + chol_tc_panel).  Algorithmic
        # work n^3/3 flops per evaluation.  Its peak: the TF32 rate of its own MMA form, measured live
        # by the library's probe at this run's clocks, divided by the three MMAs per product of the
        # FP32-accurate 3xTF32 split.  (The bf16-derived figure, measured bf16 sustained / 6, is
        # reported beside it; it assumes TF32 = bf16 / 2 at the power-capped bf16 clock.)
        peak3 = tf32["tflops"] / 3.0
        chol_flops = B * n ** 3 / 3.0
        roof = {"kernel": "tensor-core Cholesky (chol_tc_update + chol_tc_panel, 3xTF32 tcgen05)",
                "bound": "tensor", "achieved": chol_flops / (stages["cholesky"] * 1e-3) / 1e12, "peak": peak3,
                "unit": "TFLOP/s", "algorithmic_flops": chol_flops,
                "peak_note": "measured TF32 rate of the kernel's MMA form / 3 (three MMAs per FP32-accurate "
                             "product); bf16-derived alternative %.1f" % (peaks["bf16_tflops_sustained"] / 6.0),
                # ncu dram__bytes_read + dram__bytes_write of one batch-32 Cholesky, x B / 32 (traffic grows
                # with the batch): the 20 update launches measured (4.146 GB), the 19 panel launches from one
                # launch's bytes per block times the block count (0.849 GB); profiles/tc_kernels_nside16_b32.md
                "traffic": 4.995e9 * B / 32.0 if args.workload == WORKLOAD else None,
                "traffic_unit": "bytes per step (whole Cholesky stage)"}
        roof["frac"] = roof["achieved"] / roof["peak"]
        # the forward contraction A_b = I + sum_l eps_bl Ubar_l: reads the FP32 table once
        # (tiles x 4096 x lpad x 4 B) and writes A (B x tiles x 4096 x 4 B)
        nt = N // 64
        tiled = nt * (nt + 1) // 2 * 4096
        lpad = ((L1 + 15) // 16) * 16
        build_bytes = tiled * lpad * 4 + B * tiled * 4
        fwd_tc = bool(tuning and tuning["knobs"].get("fwd") == 1)
        if fwd_tc:
            roof_build = {"kernel": "build stage: A_b = I + sum_l eps_bl Ubar_l, FP32 out (contract_fwd_tc, tcgen05 "
                                    "3xTF32)", "bound": "hbm",
                          "achieved": build_bytes / (stages["build"] * 1e-3) / 1e9, "peak": peaks["hbm_gbs"],
                          "unit": "GB/s", "algorithmic_bytes": build_bytes}
        else:
            # the FP32 contraction does 2 lp flops per entry and element (20 flops per byte moved, above the
            # FP32 pipe's ridge of ~12): its roofline is the FP32 pipe, measured live by the FMA probe
            build_flops = 2.0 * B * tiled * lpad
            roof_build = {"kernel": "build stage: A_b = I + sum_l eps_bl Ubar_l, FP32 out (contract_fwd, packed "
                                    "FP32 FMA)", "bound": "fp32",
                          "achieved": build_flops / (stages["build"] * 1e-3) / 1e12, "peak": tf32["fp32_fma2_tflops"],
                          "unit": "TFLOP/s", "algorithmic_flops": build_flops,
                          "hbm_gbs": build_bytes / (stages["build"] * 1e-3) / 1e9,
                          "hbm_frac": build_bytes / (stages["build"] * 1e-3) / 1e9 / peaks["hbm_gbs"]}
        roof_build["frac"] = roof_build["achieved"] / roof_build["peak"]
    else:
        roof = {"kernel": "FP64 tiled Cholesky", "bound": "fp64", "achieved": B * n ** 3 / 3.0 /
                (stages["cholesky"] * 1e-3) / 1e12, "peak": 1.20, "unit": "TFLOP/s", "traffic": None}
        roof["frac"] = roof["achieved"] / roof["peak"]

    out = {"metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
           "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64" if path == "mixed" else "f64", "data": "synthetic",
           "config": {"workload": args.workload, "path": path, "nside": wl.nside, "lmax": wl.lmax, "n_pixels": wl.n,
                      "batch_per_gpu": B, "fwhm_arcmin": wl.meta["fwhm_arcmin"], "noise_sigma": wl.sigma,
                      "mask_keep": wl.meta["keep"], "reference_point": "fiducial C_l, factorised at set-up",
                      "l2": "per-step working set %.1f GB > 129 MB L2" % (B * 3 * (N * N / 2) * 4 / 1e9),
                      "parallelism": "replicas x%d" % world},
           "clocks": clk, "gpu_launches": int(launches),
           "e2e": {"value": job_throughput(B, world, e2e_ms), "unit": "evals/s", "ms_per_step": e2e_ms,
                   "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "stages_ms": {k: round(v, 4) for k, v in stages.items() if k != "end"},
           "stages_note": "mean of 3 profiled calls with the launches in sequence (overlap = 0); the timed "
                          "calls run trtri's rows beside the Cholesky",
           "roofline": roof, "admission": admission}
    if tuning:
        out["config"]["tuning"] = tuning
    if tf32:
        out["tf32_probe"] = tf32
    if roof_build:
        out["roofline_build"] = roof_build
    out["roofline"]["peak_source"] = peak_kind
    nfp = B if args.fp64_compare_batch is None else min(args.fp64_compare_batch, B)
    if rank == 0 and path == "mixed" and nfp > 0:
        # The plain FP64 GPU path on the same inputs (itself pinned to the reference to <= 1e-6): the
        # mixed/FP64 throughput ratio, the FP64 stage split (build vs Cholesky), and the error of every
        # element's -2lnL and of every gradient component of the timed batch against it.
        Bf = nfp
        c64 = cg.Context(lmax=wl.lmax, fwhm_deg=wl.fwhm_deg, nside=wl.nside, good_pixels=wl.ring_kept,
                         scheme="RING", noise_sigma=wl.sigma, max_batch=Bf, precision="fp64", device=local)
        clsf = cls[0, :Bf].contiguous()
        m64 = torch.empty(Bf, dtype=torch.float64, device=dev)
        g64 = torch.empty(Bf, L1, dtype=torch.float64, device=dev)
        t64 = torch.empty(Bf, L1, dtype=torch.float64, device=dev)
        zero = torch.zeros_like(dd)
        nw = min(Bf, 8)
        c64.loglike_device(nw, clsf.data_ptr(), dd.data_ptr(), 0, m64.data_ptr(), None, None, g64.data_ptr(),
                           None, sp)
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        c64.set_profiling(True)
        f0.record(stream)
        c64.loglike_device(Bf, clsf.data_ptr(), dd.data_ptr(), 0, m64.data_ptr(), None, None, g64.data_ptr(),
                           None, sp)
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1)
        st64 = c64.stage_times()
        c64.set_profiling(False)
        # the trace term T_l = tr(C^-1 dC/dC_l) of each element (the gradient of a zero map): the
        # size of the two terms whose difference is the gradient, the scale of its absolute floor
        mz = torch.empty(Bf, dtype=torch.float64, device=dev)
        c64.loglike_device(Bf, clsf.data_ptr(), zero.data_ptr(), 0, mz.data_ptr(), None, None, t64.data_ptr(),
                           None, sp)
        step(0)
        torch.cuda.synchronize()
        dm = (m2[:Bf] - m64).abs()
        dg = (grad[:Bf, 2:] - g64[:, 2:]).abs()
        rel = dg / g64[:, 2:].abs()
        over_T = dg / t64[:, 2:]
        out["plain_fp64_gpu"] = {
            "value": Bf / (ms64 / 1000.0), "unit": "evals/s", "batch": Bf,
            "mixed_over_fp64": value / world / (Bf / (ms64 / 1000.0)),
            "stages_ms": {k: round(v, 3) for k, v in st64.items() if k != "end"},
            "max_abs_delta_m2lnl": dm.max().item(), "elements_compared": Bf,
            "grad_max_rel_delta": rel.max().item(), "grad_p99_rel_delta": torch.quantile(rel.flatten(), 0.99).item(),
            "grad_max_delta_over_trace": over_T.max().item(),
            "grad_components": int(dg.numel())}
        # the per-component bar of the tests: |dg_l| <= 1e-4 max(|g_l|, s_l), s_l = T_l sqrt(2 / (2l + 1))
        # the smallest standard deviation g_l can have over data realisations
        ell = torch.arange(2, L1, dtype=torch.float64, device=dev)
        s_l = t64[:, 2:] * torch.sqrt(2.0 / (2 * ell + 1))
        bound = 1e-4 * torch.maximum(g64[:, 2:].abs(), s_l)
        out["plain_fp64_gpu"]["grad_worst_error_over_bar"] = (dg / bound).max().item()
        out["plain_fp64_gpu"]["grad_components_within_bar"] = int((dg <= bound).sum().item())
        # the BF16 table variant on the same batch: its measured error (the table rounded to BF16)
        ctx.tune_set("table_bf16", 1)
        step(0)
        torch.cuda.synchronize()
        out["bf16_table"] = {"max_abs_delta_m2lnl": (m2[:Bf] - m64).abs().max().item(),
                             "grad_max_delta_over_max_grad": ((grad[:Bf, 2:] - g64[:, 2:]).abs().max(dim=1).values /
                                                              g64[:, 2:].abs().max(dim=1).values).max().item(),
                             "elements_compared": Bf, "note": "the whitened Legendre table rounded to BF16; "
                             "measured for the record, not the benchmarked path"}
        ctx.tune_set("table_bf16", 0)
        c64.close()
    if rank == 0 and path == "mixed" and args.workload == WORKLOAD and nfp > 0:
        # The plain FP64 workload: 100 lognormal C_l vectors at nside 16 (the same sky, beam, mask and
        # map as the fixture tests/golden/config2_nside16.npz, which holds the reference's own -2lnL of
        # each), through the FP64 path with its stage split, against the reference's values.
        g2 = np.load(os.path.join(ROOT, "tests", "golden", "config2_nside16.npz"))
        n100 = len(g2["cls"])
        c2 = cg.Context(lmax=int(g2["lmax"]), fwhm_deg=float(g2["fwhm_deg"]), nside=int(g2["nside"]),
                        good_pixels=g2["nest_good"], scheme="NEST", noise_sigma=float(g2["sigma"]),
                        max_batch=n100, precision="fp64", device=local)
        cl2 = torch.tensor(g2["cls"], dtype=torch.float64, device=dev)
        d2 = torch.tensor(g2["d"], dtype=torch.float64, device=dev)
        m2b = torch.empty(n100, dtype=torch.float64, device=dev)
        c2.loglike_device(4, cl2.data_ptr(), d2.data_ptr(), 0, m2b.data_ptr(), None, None, None, None, sp)
        torch.cuda.synchronize()
        c2.set_profiling(True)
        q0 = torch.cuda.Event(enable_timing=True)
        q1 = torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        c2.loglike_device(n100, cl2.data_ptr(), d2.data_ptr(), 0, m2b.data_ptr(), None, None, None, None, sp)
        q1.record(stream)
        torch.cuda.synchronize()
        st2 = c2.stage_times()
        c2.set_profiling(False)
        c2.close()
        got = m2b.cpu().numpy()
        out["plain_fp64_100"] = {"workload": "nside16_lmax47 (100 lognormal C_l vectors, likelihood only)",
                                 "evals_per_s": n100 / (q0.elapsed_time(q1) / 1000.0),
                                 "stages_ms": {k: round(v, 3) for k, v in st2.items() if k not in ("end", "adjoint")},
                                 "max_abs_delta_vs_reference": float(np.abs(got - g2["m2lnl"]).max()),
                                 "max_abs_delta_vs_extended_precision": float(np.abs(got - g2["m2lnl_ext"]).max()),
                                 "reference_own_max_abs_delta_vs_extended": float(np.abs(g2["m2lnl"] -
                                                                                         g2["m2lnl_ext"]).max())}
    if rank == 0 and path == "mixed" and args.hmc_iters > 0:
        # gradient + HMC: 64 chains on ln C_l (l = 2..lmax), 20 leapfrog steps of 0.05, unit masses,
        # starts at the fiducial +-10% (seeded); every leapfrog step is one batched evaluation
        from cosmopp_gb300 import diagnostics
        nch = min(64, B)
        rng = np.random.default_rng(11)
        x0 = np.log(wl.cl_fid[2:])[None, :] + np.log1p(rng.uniform(-0.1, 0.1, (nch, wl.lmax - 1)))
        # the same batched evaluation at the chains' batch size, device-timed: what the sampler's
        # host loop (leapfrog arithmetic, copies, one synchronising call per step) costs on top of it
        c64b = cls[0, :nch].contiguous()
        for _ in range(3):
            ctx.loglike_device(nch, c64b.data_ptr(), dd.data_ptr(), 0, m2.data_ptr(), None, None, grad.data_ptr(),
                               None, sp)
        h0 = torch.cuda.Event(enable_timing=True)
        h1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        h0.record(stream)
        for _ in range(20):
            ctx.loglike_device(nch, c64b.data_ptr(), dd.data_ptr(), 0, m2.data_ptr(), None, None, grad.data_ptr(),
                               None, sp)
        h1.record(stream)
        torch.cuda.synchronize()
        bare = 20 * nch / (h0.elapsed_time(h1) / 1000.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        chain, acc = ctx.hmc(d, x0, wl.cl_fid, niter=args.hmc_iters, nleap=20, tau=0.05, seed=3)
        hmc_s = time.perf_counter() - t0
        ess = diagnostics.ess(chain[1:, :, 1:])
        nev = nch * (1 + 20 * args.hmc_iters)
        out["hmc"] = {"chains": nch, "leapfrog_steps": 20, "step_size": 0.05, "iterations": args.hmc_iters,
                      "evals_per_s": nev / hmc_s, "bare_batch_evals_per_s": bare,
                      "host_share": 1.0 - (nev / hmc_s) / bare, "accept_rate": float(acc.mean()),
                      "ess_min": float(ess.min()), "ess_median": float(np.median(ess)),
                      "ess_per_s_min": float(ess.min() / hmc_s), "wall_s": hmc_s,
                      "reference_point": "fiducial, fixed"}
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(wl, d)
    ctx.close()
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
