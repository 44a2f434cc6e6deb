"""Benchmark: SCC-DFTB energy + force evaluations per second on one GB300.

Workload (default): (H2O)1024 cluster, 3072 atoms, 6144 orbitals, 8192 electrons, seeded synthetic
SK tables, Fermi kT = 1e-3 Ha, Broyden mixing 0.2, SCC tolerance 1e-7 e. One step = one full
evaluation from the neutral reference charges: geometry (H0/S, Cholesky), SCC to convergence,
energies and gradients.

  value : steps/s with the geometry already in HBM (device pointers through the C-ABI).
  e2e   : the same through the public Python API with host buffers (coordinates in, energy,
          eigenvalues, fillings, charges and gradients out), copies inside the timed region.
  --impl reference : the CPU oracle (numpy/OpenBLAS dsygvd, all host cores) on a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (n_mol, radius_A, seed)
    "h2o1024": (1024, 30.0, 1024),
    "h2o512": (512, 23.8, 512),
    "h2o128": (128, 20.0, 128),
    "h2o32": (32, 10.0, 1),
}
KT, SCC_TOL, MIX = 1e-3, 1e-7, 0.2
# the headline metric: energy+force evaluations per second of the mixed form (the plain FP64 rate and
# the mixed-vs-FP64 errors are reported beside it); --precision fp64 times the plain form instead
METRIC = "E+F evals/s, mixed vs FP64 on 1 GB300 at |dE|<=1e-6 Ha/atom"


# the large spd system: anatase TiO2 sphere, 1,700 Ti + 3,400 O (Ti spd 9 + O sp 4 = 28,900 orbitals)
TIO2_NTI = 1700


def _workload(name):
    from dftbplus_gb300 import synth
    if name == "tio2":
        coords, species = synth.anatase_cluster(TIO2_NTI)
        return synth.anatase_model(), coords, species
    n_mol, radius, seed = CONFIGS[name]
    coords, species = synth.water_cluster(n_mol, radius, seed)
    return synth.water_model(), coords, species


BATCH_NMOL, BATCH_SEED = 4096, 4096


def batch_sizes(nmol=BATCH_NMOL, seed=BATCH_SEED):
    """Waters per molecule of the batched set: n seeded uniform in [2, 48]."""
    return np.random.default_rng(seed).integers(2, 49, nmol)


def batch_molecule(i, n):
    """Molecule i of the batched set: (H2O)n in a sphere of radius 10 (n/32)^(1/3) A, seed 10000 + i."""
    from dftbplus_gb300 import synth
    return synth.water_cluster(int(n), 10.0 * (n / 32.0) ** (1.0 / 3.0), 10000 + i)


def _batch_workload(nmol=BATCH_NMOL, seed=BATCH_SEED):
    """4,096 independent (H2O)n clusters, n seeded uniform in [2, 48], sphere radius 10 (n/32)^(1/3) A."""
    from dftbplus_gb300 import synth
    mols = [batch_molecule(i, n) for i, n in enumerate(batch_sizes(nmol, seed))]
    return synth.water_model(), mols


def _oracle_molecule(args):
    """One molecule through the CPU oracle (SCC to 1e-7 e + gradients); runs in a worker process."""
    from oracle import dftb_oracle as O
    from dftbplus_gb300 import synth
    coords, species = args
    sys_ = O.System(synth.water_model(), coords, species)
    ref = O.run_scc(sys_, kt=KT, scc_tol=SCC_TOL)
    O.gradients(sys_, ref)
    return ref.n_iter


def cpu_batch_rate(mols, budget_s=20.0):
    """Molecules/s of the CPU oracle over all host cores (one single-threaded process per core) on a
    sample of the batch, stopping after about budget_s seconds."""
    import multiprocessing as mp
    ncpu = os.cpu_count() or 1
    names = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")
    saved = {v: os.environ.get(v) for v in names}
    for v in names:
        os.environ[v] = "1"          # inherited by the workers as they start
    ctx = mp.get_context("spawn")
    done, t0 = 0, time.perf_counter()
    pool = ctx.Pool(ncpu)
    for v, old in saved.items():     # the parent keeps its own BLAS threading
        if old is None:
            os.environ.pop(v, None)
        else:
            os.environ[v] = old
    with pool:
        pool.map(_oracle_molecule, mols[:ncpu])          # worker start-up outside the timing
        t0 = time.perf_counter()
        i = 0
        while time.perf_counter() - t0 < budget_s and i < len(mols):
            chunk = mols[i:i + 4 * ncpu]
            pool.map(_oracle_molecule, chunk)
            done += len(chunk)
            i += len(chunk)
    t = time.perf_counter() - t0
    return {"value": done / t, "unit": "molecules/s", "cores": ncpu, "kind": "port",
            "sample": f"{done} molecules of the batch (first after warm-up), SCC to 1e-7 e + gradients, "
                      f"one single-threaded oracle process per core"}


def _dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


class ClockSampler:
    def __init__(self, out_path, device=0):
        self.path = out_path
        self.proc = None
        self.device = device

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def gemm_peak(dtype_name="float64"):
    """Library GEMM rate on this GPU (cuBLAS via torch, 8192^3, best of 5, TF32 off), TFLOP/s."""
    import torch
    torch.backends.cuda.matmul.allow_tf32 = False
    dt = getattr(torch, dtype_name)
    n = 8192
    a = torch.randn(n, n, dtype=dt, device="cuda")
    b = torch.randn(n, n, dtype=dt, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    torch.cuda.empty_cache()
    return 2.0 * n ** 3 / best / 1e12


BF16_PEAK_FALLBACK = 1700.0
HBM_PEAK_FALLBACK = 6800.0
BF16_PEAK_SOURCE = "measured sustained cuBLAS bf16 GEMM (MEASURED_PEAKS.json bf16_tflops_sustained)"
HBM_PEAK_SOURCE = "measured copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
N_SM = 152


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def bf16_peak():
    """Dense BF16 tensor peak of this GPU pool (TFLOP/s): the measured sustained figure (the GEMMs run
    inside a seconds-long step), else the fallback of an earlier GB300 measurement."""
    global BF16_PEAK_SOURCE
    try:
        v = float(_measured_peaks()["bf16_tflops_sustained"])
        BF16_PEAK_SOURCE = "of measured: sustained cuBLAS bf16 GEMM (MEASURED_PEAKS.json bf16_tflops_sustained)"
        return v
    except (KeyError, ValueError, TypeError):
        BF16_PEAK_SOURCE = "of fallback: 1.7 PFLOP/s sustained bf16 of an earlier GB300 measurement"
        return BF16_PEAK_FALLBACK


def hbm_peak():
    """HBM copy bandwidth of this GPU pool (GB/s): measured, else the fallback of an earlier GB300."""
    global HBM_PEAK_SOURCE
    try:
        v = float(_measured_peaks()["hbm_gbs"])
        HBM_PEAK_SOURCE = "of measured: copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
        return v
    except (KeyError, ValueError, TypeError):
        HBM_PEAK_SOURCE = "of fallback: 6.8 TB/s of an earlier GB300 measurement"
        return HBM_PEAK_FALLBACK


def traffic_per_launch(kernel, workload):
    """DRAM bytes per launch of a kernel from the committed ncu summary (profiles/traffic.json:
    dram__bytes_read.sum + dram__bytes_write.sum of one capture, scaled to the workload there)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            return json.load(f)[workload][kernel]
    except (OSError, KeyError, ValueError):
        return None


def kernel_classes(prof, steps, sm_mhz, dgemm_tflops, sgemm_tflops, workload):
    """Per-step time and achieved rate of every timed kernel class of the evaluation, with the peak
    its rate is held against: HBM-streaming kernels against the measured copy bandwidth, CUDA-core
    FP32/FP64 work against SMs x lanes x clock (and the cuBLAS rate measured in the same run),
    tensor-core products against the measured bf16 peak."""
    f = (sm_mhz or 2070.0) * 1e6
    fp32_cc = N_SM * 128 * 2 * f / 1e12          # FP32 FMA lanes per SM: 128
    fp64_cc = N_SM * 2 * 2 * f / 1e12            # FP64 FMA per SM per clock: 2
    hbm = hbm_peak()
    bf16 = bf16_peak()
    spec = {
        "k_sytrd_panel": ("sytrd_panel_resident_kernel<double> (one-stage tridiagonalisation panels, FP64, "
                          "trailing tiles held per panel: symmetric matrix-vector products 2 m^2 FLOPs per column)",
                          "fp64", "TFLOP/s", 1e-12, fp64_cc,
                          f"FP64 {N_SM} SMs x 2 FMA x 2 x {f / 1e6:.0f} MHz (cuBLAS DGEMM measured here: "
                          f"{dgemm_tflops:.2f} TFLOP/s)"),
        "k_sytrd_panel32": ("sytrd_panel_resident_kernel<float> (one-stage tridiagonalisation panels, FP32, "
                            "trailing tiles held per panel: symmetric matrix-vector products 2 m^2 FLOPs per column)",
                            "fp32", "TFLOP/s", 1e-12, fp32_cc,
                            f"FP32 CUDA cores {N_SM} SMs x 128 lanes x 2 x {f / 1e6:.0f} MHz (cuBLAS SGEMM measured "
                            f"here: {sgemm_tflops:.1f} TFLOP/s)"),
        "k_panel_qr": ("panel_qr_kernel (two-stage band reduction, panel QR)", "hbm", "GB/s", 1e-9, hbm,
                       HBM_PEAK_SOURCE),
        "k_back_q2": ("q2_apply_kernel (bulge-chasing reflectors applied to the eigenvectors, FP32)", "fp32",
                      "TFLOP/s", 1e-12, fp32_cc, f"FP32 CUDA cores {N_SM} SMs x 128 lanes x 2 x {f / 1e6:.0f} MHz"),
        "k_chase": ("sb2st_kernel (bulge chasing, band -> tridiagonal)", "latency", "tasks/s", 1.0, None,
                    "latency-bound chain of Householder tasks (no throughput peak)"),
        "gemm_fp64": ("dgemm_kernel<double> (FP64 FMA GEMM launches)", "fp64", "TFLOP/s", 1e-12, fp64_cc,
                      f"FP64 {N_SM} SMs x 2 FMA x 2 x {f / 1e6:.0f} MHz (cuBLAS DGEMM measured here: "
                      f"{dgemm_tflops:.2f} TFLOP/s)"),
        "gemm_fp32": ("dgemm_kernel<float>, sgemm128_kernel, tc_gemm_kernel (FP32-class GEMM launches)", "fp32",
                      "TFLOP/s", 1e-12, fp32_cc, f"FP32 CUDA cores {N_SM} SMs x 128 lanes x 2 x {f / 1e6:.0f} MHz "
                      f"(cuBLAS SGEMM measured here: {sgemm_tflops:.1f} TFLOP/s)"),
        "gemm_tc_fp64": ("dg_gemm_kernel (FP64 products as 36 exact BF16 digit products on tcgen05)", "tensor",
                         "TFLOP/s", 36e-12, bf16, BF16_PEAK_SOURCE),
    }
    out = {}
    for key, (name, bound, unit, scale, peak, src) in spec.items():
        v = prof.get(key)
        if not v or v["ms"] <= 0:
            continue
        ms = v["ms"] / max(steps, 1)
        launches = v["calls"] / max(steps, 1)
        rate = v["flops"] * scale / (v["ms"] / 1e3)
        tr = traffic_per_launch(name.split(" ")[0], workload)
        out[key] = {"kernel": name, "bound": bound, "ms_per_step": ms, "launches_per_step": launches,
                    "achieved": rate, "unit": unit, "peak": peak, "frac": (rate / peak) if peak else None,
                    "peak_source": src, "traffic": tr,
                    "work_per_launch": v["flops"] / max(v["calls"], 1)}
    return out


def _cpu_threads():
    ncpu = os.cpu_count() or 1
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ.setdefault(v, str(ncpu))
    return ncpu


def cpu_full_evaluations(name, budget_s, max_evals):
    """Complete CPU evaluations of the oracle on all host cores: H0/S, SCC from the neutral charges
    to 1e-7 e with Broyden mixing, energies and gradients, one evaluation after another until
    max_evals are done or the next one would pass budget_s. At least one is timed. A warm-up
    evaluation of (H2O)32 (untimed) starts the BLAS threads first. Returns (seconds per evaluation
    list, SCC iterations of the last one)."""
    from oracle import dftb_oracle as O
    model, coords, species = _workload(name)
    wm, wc, ws = _workload("h2o32")
    O.gradients(O.System(wm, wc, ws), O.run_scc(O.System(wm, wc, ws), kt=KT, scc_tol=SCC_TOL))
    times, n_iter = [], 0
    t_start = time.perf_counter()
    while len(times) < max_evals:
        t0 = time.perf_counter()
        sys_ = O.System(model, coords, species)
        ref = O.run_scc(sys_, kt=KT, scc_tol=SCC_TOL, mixer=O.BroydenMixer(alpha=MIX))
        O.gradients(sys_, ref, kt=KT)
        times.append(time.perf_counter() - t0)
        n_iter = ref.n_iter
        if time.perf_counter() - t_start + times[-1] > budget_s:
            break
    return times, n_iter


def cpu_eval_sample(name):
    """Bounded CPU sample (about 10-30 s at (H2O)1024 on 16 cores) of one complete oracle evaluation:
    H0/S build, one SCC iteration (potentials, H, LAPACK dsygvd, Fermi filling, density matrix,
    Mulliken, Broyden step) and the gradients, each timed; the evaluation is H0/S + n_iter SCC
    iterations + gradients. Returns (seconds per evaluation, sample description)."""
    from oracle import dftb_oracle as O
    model, coords, species = _workload(name)
    sys_ = O.System(model, coords, species)
    t0 = time.perf_counter()
    H0S = O.build_h0_s(sys_)
    t_h0s = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref1 = O.run_scc(sys_, kt=KT, scc_tol=SCC_TOL, max_iter=1, H0S=H0S, mixer=O.BroydenMixer(alpha=MIX))
    t_it = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.gradients(sys_, ref1, kt=KT)
    t_grad = time.perf_counter() - t0
    n_iter = REF_SCC_ITERS[name]
    total = t_h0s + n_iter * t_it + t_grad
    return total, (f"one complete oracle evaluation of {name} assembled from timed parts: H0/S build "
                   f"{t_h0s:.1f} s, one SCC iteration {t_it:.1f} s (LAPACK dsygvd via OpenBLAS) x {n_iter} "
                   f"iterations, gradients {t_grad:.1f} s")


REF_BUDGET_S = 300.0    # wall-clock budget of the reference arm's timed evaluations


def run_reference(args):
    rank, world, _ = _dist_env()
    if rank != 0:
        return
    if args.config == "batch4096":
        _, mols = _batch_workload()
        rates = []
        for i in range(args.warmup + args.steps):
            r = cpu_batch_rate(mols[(i * 64) % len(mols):], budget_s=10.0)
            if i >= args.warmup:
                rates.append(r)
        v = float(np.median([r["value"] for r in rates]))
        cpu = dict(rates[-1], value=v)
        line = {"impl": "reference", "metric": BATCH_METRIC, "value": v, "unit": "molecules/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": BATCH_NMOL / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded water clusters, analytic SK tables)",
                "config": {"workload": "batch4096", "molecules": BATCH_NMOL, "kT": KT, "scc_tol": SCC_TOL},
                "cpu_baseline": cpu,
                "e2e": {"value": v, "unit": "molecules/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    ncpu = _cpu_threads()
    times, n_iter = cpu_full_evaluations(args.config, REF_BUDGET_S, max(1, args.steps))
    t_eval = float(np.mean(times))
    value = 1.0 / t_eval
    sample = (f"{len(times)} complete evaluation(s) of {args.config} timed one after another ({args.steps} "
              f"requested; the {REF_BUDGET_S:.0f} s budget bounds the run): H0/S, SCC from the neutral "
              f"charges to 1e-7 e ({n_iter} iterations, LAPACK dsygvd via OpenBLAS on {ncpu} threads), "
              f"energies and gradients, after one untimed (H2O)32 warm-up evaluation")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "evals/s", "n_gpus": world,
            "steps": len(times), "steps_requested": args.steps, "warmup": args.warmup,
            "ms_per_step": t_eval * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded water cluster, analytic SK tables)",
            "config": {"workload": args.config, "orbitals": _norb(args.config), "kT": KT, "scc_tol": SCC_TOL},
            "cpu_baseline": {"value": value, "unit": "evals/s", "cores": ncpu, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# SCC iterations of each workload from the neutral start (same count on the GPU and the oracle;
# the GPU bench asserts it)
REF_SCC_ITERS = {"h2o1024": 14, "h2o512": 14, "h2o128": 14, "h2o32": 13}


def batch_measure(dev, precisions=("mixed", "fp64"), steps=1, warmup=1, seq_sample=48, world=1, rank=0):
    """Batched workload: per precision form molecules/s (device-resident coordinates), the
    host-buffer public-API rate, the one-molecule-at-a-time rate of the single-system path on a sample,
    and the algorithmic FP64 FLOP rate of the FP64 form. With world > 1 every rank solves its
    cost-balanced share of the molecules (no collective on the data path); times are the maximum over
    ranks and rates count all molecules."""
    import torch
    from dftbplus_gb300 import binding
    from dftbplus_gb300.shard import shard_by_cost
    model, all_mols = _batch_workload()
    n_total = len(all_mols)
    share = shard_by_cost([6 * (len(m[1]) // 3) for m in all_mols], world)[rank] if world > 1 else None
    mols = [all_mols[i] for i in share] if share is not None else all_mols
    nmol = len(mols)

    def tmax(t):
        if world == 1:
            return t
        tt = torch.tensor([t], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        return float(tt.item())

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
    off = np.zeros(nmol + 1, dtype=np.int32)
    off[1:] = np.cumsum([len(m[1]) for m in mols])
    xyz_h = np.ascontiguousarray(np.concatenate([m[0].T for m in mols]), dtype=np.float64)
    sp = np.concatenate([m[1] for m in mols]).astype(np.int32)
    xyz_d = torch.tensor(xyz_h, device="cuda")
    ctx = binding.Context(dev)
    ctx.set_model(model)
    out = {}
    for name in precisions:
        prec = binding.PREC_MIXED if name == "mixed" else binding.PREC_FP64
        opts = binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=MIX, precision=prec)

        def step():
            ctx.batch_set_geometries_dev(off, xyz_d.data_ptr(), sp)
            r = ctx.batch_scc(opts)
            ctx.batch_gradients()
            return r
        for _ in range(warmup):
            step()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = ctx.kernel_launches()
        e0.record()
        for _ in range(steps):
            r = step()
        e1.record()
        barrier()
        t = tmax(e0.elapsed_time(e1) / 1e3 / steps)
        nit = r["n_iter"].astype(np.float64)
        out[name] = {"value": n_total / t, "unit": "molecules/s", "latency_s": t, "converged": int(r["converged"].sum()),
                     "scc_iterations_mean": float(nit.mean()), "scc_iterations_max": int(nit.max()),
                     "gpu_launches_per_step": (ctx.kernel_launches() - l0) // steps}
        if name == "fp64":
            n = np.diff(off).astype(np.float64) * 2.0          # 6 orbitals per water = 2 per atom
            k = np.diff(off).astype(np.float64) * 4.0 / 3.0    # 4 occupied levels per water
            flops = float(np.sum(nit * (16.0 / 3.0 * n ** 3 + n ** 2 * k) + n ** 3 / 3.0))
            out[name]["algorithmic_flops"] = flops
    # public API with host buffers, first form
    first = precisions[0]
    prec = binding.PREC_MIXED if first == "mixed" else binding.PREC_FP64
    opts = binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=MIX, precision=prec)
    cl, sl = [m[0] for m in mols], [m[1] for m in mols]
    barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        ctx.batch_set_geometries(cl, sl)
        ctx.batch_scc(opts)
        ctx.batch_gradients()
    barrier()
    t_e2e = tmax((time.perf_counter() - t0) / steps)
    e2e = {"value": n_total / t_e2e, "unit": "molecules/s", "h2d_bytes_per_step": int(xyz_h.nbytes + sp.nbytes + off.nbytes),
           "d2h_bytes_per_step": int(nmol * 96 + 8 * off[-1] + 3 * 8 * off[-1])}
    if rank != 0:
        ctx.close()
        return out, e2e, None, all_mols
    # the single-system path, one molecule at a time, on an even sample
    idx = list(range(0, nmol, max(1, nmol // seq_sample)))[:seq_sample]
    c2 = binding.Context(dev)
    c2.set_model(model)
    o64 = binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=MIX)
    c2.set_geometry(*mols[idx[0]]); c2.scc(o64); c2.gradients()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in idx:
        c2.set_geometry(*mols[i])
        c2.scc(o64)
        c2.gradients()
    torch.cuda.synchronize()
    seq = {"value": len(idx) / (time.perf_counter() - t0), "unit": "molecules/s",
           "sample": f"{len(idx)} molecules spread over the batch, single-system FP64 path, one call sequence each"}
    ctx.close()
    c2.close()
    return out, e2e, seq, all_mols


BATCH_METRIC = "batched molecules/s (4,096 ragged (H2O)n, n in [2, 48], SCC to 1e-7 e + gradients)"


def _batch_summary(out, e2e, seq, cpu, fp64_peak):
    b = {"mixed": out["mixed"]["value"], "fp64": out["fp64"]["value"], "unit": "molecules/s",
         "latency_s": {k: v["latency_s"] for k, v in out.items()},
         "sequential": seq, "batched_vs_sequential": out["mixed"]["value"] / seq["value"],
         "fp64_batched_vs_sequential": out["fp64"]["value"] / seq["value"], "e2e": e2e, "forms": out}
    f = out["fp64"].get("algorithmic_flops")
    if f and fp64_peak:
        ach = f / out["fp64"]["latency_s"] / 1e12
        b["roofline_fp64"] = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s",
                              "frac": ach / fp64_peak,
                              "algorithm": "per molecule and SCC iteration (16/3) n^3 + n^2 k, n^3/3 per geometry"}
    if cpu:
        b["cpu_baseline"] = cpu
    return b


def run_batch(args):
    """Headline line of the batched workload (--config batch4096)."""
    import torch
    rank, world, local = _dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    from dftbplus_gb300 import build
    build.build()
    dev = torch.cuda.current_device()
    clock_file = os.path.join(tempfile.gettempdir(), f"clocks_{os.getpid()}.csv")
    with ClockSampler(clock_file, dev) as clk:
        out, e2e, seq, mols = batch_measure(dev, ("mixed", "fp64") if args.precision == "mixed" else ("fp64",),
                                            steps=args.steps, warmup=args.warmup, world=world, rank=rank)
    if rank != 0:
        return
    cpu = None if args.no_cpu_baseline else cpu_batch_rate(mols)
    peak = gemm_peak("float64")
    main = out[args.precision]
    line = {"metric": BATCH_METRIC, "precision": args.precision, "value": main["value"], "unit": "molecules/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": main["latency_s"] * 1e3, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32+f64" if args.precision == "mixed" else "f64",
            "data": "synthetic (seeded water clusters, analytic SK tables)",
            "config": {"workload": "batch4096", "molecules": BATCH_NMOL, "kT": KT, "scc_tol": SCC_TOL,
                       "l2": "inputs per step re-uploaded; per-molecule working sets L2-resident by design",
                       "parallelism": f"molecules sharded by cost over {world} GPU(s), no collective"},
            "e2e": e2e, "gpu_launches": int(main["gpu_launches_per_step"] * args.steps),
            "clocks": clk.summary(), "cpu_baseline": cpu}
    line.update({k: v for k, v in _batch_summary(out, e2e, seq, cpu, peak).items()
                 if k not in ("e2e", "cpu_baseline")} if "fp64" in out and "mixed" in out else {})
    if "roofline_fp64" in line:
        line["roofline"] = dict(line["roofline_fp64"], kernel="batch_iter_kernel<double> (whole SCC iterations)",
                                traffic=None)
    print(json.dumps(line))


def _norb(name):
    if name == "tio2":
        return 9 * TIO2_NTI + 4 * 2 * TIO2_NTI
    return CONFIGS[name][0] * 6


def run_gpu(args):
    import torch
    rank, world, local = _dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(local)
    dev = torch.cuda.current_device()
    from dftbplus_gb300 import binding, build
    build.build()
    model, coords, species = _workload(args.config)
    N = len(species)
    ctx = binding.Context(dev)
    ctx.set_model(model)
    mixed = args.precision == "mixed"
    prec = binding.PREC_MIXED if mixed else binding.PREC_FP64
    opts = binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=MIX, precision=prec)
    opts64 = binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=MIX, precision=binding.PREC_FP64)
    xyz = torch.tensor(np.ascontiguousarray(coords.T), dtype=torch.float64, device="cuda")
    grad = torch.empty(3 * N, dtype=torch.float64, device="cuda")

    def step_dev(o=None):
        ctx.set_geometry_dev(xyz.data_ptr(), species)
        r = ctx.scc_lite(o or opts)
        ctx.gradients_dev(grad.data_ptr())
        return r

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    info = None
    for _ in range(args.warmup):
        info = step_dev()
    if info is not None:
        assert info["converged"], "SCC did not converge"
    launches0 = ctx.kernel_launches()
    ctx.profile(True)
    clock_file = os.path.join(tempfile.gettempdir(), f"clocks_{os.getpid()}.csv")
    barrier()
    with ClockSampler(clock_file, dev) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e0.record()
        for _ in range(args.steps):
            info = step_dev()
        e1.record()
        barrier()
        wall = time.perf_counter() - t0
    ctx.profile(False)
    prof = ctx.profile_read()
    launches = ctx.kernel_launches() - launches0
    # host time per SCC iteration kind of the last timed evaluation (FP32 eigensolve, FP64 eigensolve,
    # perturbative update)
    hist = ctx.scc_history()
    kinds = {binding.PREC_MIXED: "fp32_eigensolve", binding.PREC_FP64: "fp64_eigensolve",
             binding.ITER_PERTURB: "perturbative"}
    by_kind = {}
    for pk, ms in zip(hist["precision"].tolist(), hist["ms"].tolist()):
        d = by_kind.setdefault(kinds.get(pk, str(pk)), {"iterations": 0, "ms": 0.0})
        d["iterations"] += 1
        d["ms"] = round(d["ms"] + ms, 1)
    assert info["converged"], "SCC did not converge"
    n_iter = info["n_iter"]
    t_dev = e0.elapsed_time(e1) / 1e3
    if world > 1:
        tt = torch.tensor([t_dev], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(tt.item())
    value = world * args.steps / t_dev

    e_main = info["energies"]["EMermin"]
    g_main = grad.cpu().numpy().copy()

    # the plain FP64 form on the same geometry: rate and the accuracy of the main form against it
    fp64 = None
    if mixed:
        barrier()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record()
        r64 = step_dev(opts64)
        e5.record()
        barrier()
        t64 = e4.elapsed_time(e5) / 1e3
        g64 = grad.cpu().numpy()
        fp64 = {"value": 1.0 / t64, "ms_per_step": t64 * 1e3, "scc_iterations": r64["n_iter"],
                "mixed_vs_fp64": (args.steps / t_dev) / (1.0 / t64),
                "accuracy_vs_fp64": {"dE_per_atom": abs(e_main - r64["energies"]["EMermin"]) / N,
                                     "max_dF": float(np.max(np.abs(g_main - g64)))}}

    # e2e through the public API with host buffers (the first context is released first: at the
    # large configuration two contexts would not fit the device together)
    ctx.close()
    calc = binding.DftbGpu(model, coords, species, kT=KT, scc_tol=SCC_TOL, mixing=MIX, device=dev, precision=prec)
    calc.get_energy(); calc.get_gradients()
    barrier()
    e2 = torch.cuda.Event(enable_timing=True); e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    for _ in range(args.steps):
        calc.set_geometry(coords)
        calc.get_energy()
        calc.get_gradients()
    e3.record()
    barrier()
    t_e2e = e2.elapsed_time(e3) / 1e3
    if world > 1:
        tt = torch.tensor([t_e2e], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(tt.item())
    n = calc.ctx.norb
    h2d = 3 * N * 8 + N * 4
    d2h = 8 * 8 + 2 * n * 8 + N * 8 + 3 * N * 8
    calc.close()

    if rank != 0:
        return
    # per-kernel classes of the evaluation; the roofline is the one that takes the most time
    dgemm_tf = gemm_peak("float64")
    sgemm_tf = gemm_peak("float32")
    clocks = clk.summary()
    kc = kernel_classes(prof, args.steps, clocks.get("sm_mhz"), dgemm_tf, sgemm_tf, args.config)
    dom = max(kc, key=lambda k: kc[k]["ms_per_step"]) if kc else None
    cpu = None
    if not args.no_cpu_baseline:
        ncpu = _cpu_threads()
        t_eval, sample = cpu_eval_sample(args.config)
        cpu = {"value": 1.0 / t_eval, "unit": "evals/s", "cores": ncpu, "kind": "port", "sample": sample}
    # the batched workload (second half of the headline metric), measured on the same GPU
    batched = None
    if not args.no_batch and world == 1:
        bout, be2e, bseq, bmols = batch_measure(dev)
        bcpu = None if args.no_cpu_baseline else cpu_batch_rate(bmols)
        batched = _batch_summary(bout, be2e, bseq, bcpu, dgemm_tf)
    phases = {k: round(v["ms"] / max(args.steps, 1), 2) for k, v in prof.items()}
    roof = None
    if dom is not None:
        d = kc[dom]
        roof = {"bound": d["bound"], "kernel": d["kernel"], "achieved": d["achieved"], "peak": d["peak"],
                "unit": d["unit"], "frac": d["frac"], "peak_source": d["peak_source"], "traffic": d["traffic"],
                "ms_per_step": d["ms_per_step"], "share_of_step": d["ms_per_step"] / (t_dev / args.steps * 1e3)}

    expected_iters = REF_SCC_ITERS.get(args.config)
    line = {"metric": METRIC, "precision": args.precision, "value": value, "unit": "evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if mixed else "f64",
            "data": "synthetic (seeded water cluster, analytic SK tables)",
            "config": {"workload": args.config, "atoms": N, "orbitals": n, "kT": KT, "scc_tol": SCC_TOL,
                       "scc_iterations": n_iter, "l2": "working set (n^2 FP64 matrices) larger than L2",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": world * args.steps / t_e2e, "unit": "evals/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "roofline": roof,
            "kernel_classes": kc,
            "fp64": fp64,
            "batched": batched,
            "cpu_baseline": cpu, "gpu_launches": int(launches), "clocks": clocks,
            "phases_ms_per_step": phases, "scc_iterations_by_kind": by_kind, "wall_s": wall,
            "energy": info["energies"]["EMermin"]}
    n_iter64 = fp64["scc_iterations"] if fp64 else n_iter   # the recorded count is the FP64 cycle's
    if expected_iters is not None and expected_iters != n_iter64:
        line["note"] = f"FP64 SCC iterations {n_iter64} differ from the recorded {expected_iters}"
    print(json.dumps(line))


def run_per_iteration(args):
    """For a configuration whose plain FP64 evaluation is too long to time whole (the TiO2 sphere:
    about 110 s per FP64 SCC iteration): each form in its own context, the geometry set-up, two FP64
    SCC iterations (the first also forms L^-1 and the reduced H0), the mixed form's first iteration
    (FP32 eigensolve plus the same one-time products) and one later iteration of each kind (FP32
    eigensolve, FP64-class eigensolve, perturbative update) and the gradients of both forms, each
    timed; then both forms to convergence on smaller spheres of the
    same model (40 and 100 Ti) for their iteration counts and energy agreement. One JSON line; the
    evaluation-time model it prints (set-up + counts x per-iteration costs + gradients) is labelled
    as such."""
    from dftbplus_gb300 import binding, synth
    rank, _, _ = _dist_env()
    if rank != 0:
        return
    mix = args.mix_alpha

    def run(ctx, **kw):
        t0 = time.perf_counter()
        r = ctx.scc(binding.default_opts(kT=KT, scc_tol=SCC_TOL, mix_alpha=mix, **kw))
        t_scc = time.perf_counter() - t0
        t0 = time.perf_counter()
        ctx.gradients()
        t_grad = time.perf_counter() - t0
        h = ctx.scc_history()
        return r, {"scc_s": t_scc, "grad_s": t_grad, "kinds": h["precision"].tolist(),
                   "iter_s": [round(x / 1e3, 3) for x in h["ms"].tolist()]}

    model, c, s = _workload(args.config)

    def fresh():
        # each form in its own context, so that each pays its own one-time set-up (Cholesky at
        # set_geometry; L^-1 and the reduced H0 in the first SCC iteration)
        cx = binding.Context(0)
        cx.set_model(model)
        t0 = time.perf_counter()
        cx.set_geometry(c, s)
        return cx, time.perf_counter() - t0

    ctx, t_geom = fresh()
    _, fp64 = run(ctx, precision=binding.PREC_FP64, max_iter=2)
    norb = ctx.norb
    ctx.close()
    ctx, t_geom_mixed = fresh()
    # FP32 eigensolve (the first one also forms L^-1 and the reduced H0), then (switch tolerance above
    # any error) FP64-class, perturbative, perturbative, FP64-class
    _, mixed = run(ctx, precision=binding.PREC_MIXED, max_iter=5, mixed_switch_tol=1e3)
    # a later FP32 eigensolve (switch tolerance below any error; the last allowed iteration is FP64-class)
    _, mixed2 = run(ctx, precision=binding.PREC_MIXED, max_iter=2, mixed_switch_tol=1e-30)
    ctx.close()
    kinds = {binding.PREC_MIXED: "fp32", binding.PREC_FP64: "fp64_class", binding.ITER_PERTURB: "perturbative"}
    per = {"fp32_first": mixed["iter_s"][0]}
    for k, t in list(zip(mixed2["kinds"], mixed2["iter_s"])) + list(zip(mixed["kinds"][1:], mixed["iter_s"][1:])):
        per.setdefault(kinds[k], t)
    t_fp64_iter = fp64["iter_s"][-1]
    counts = []
    if args.config == "tio2":
        for nti in (40, 100):
            cc, ss = synth.anatase_cluster(nti)
            cx = binding.Context(0)
            cx.set_model(model)
            cx.set_geometry(cc, ss)
            row = {"ti": nti, "orbitals": cx.norb}
            for name, prec in (("fp64", binding.PREC_FP64), ("mixed", binding.PREC_MIXED)):
                r, info = run(cx, precision=prec, max_iter=150)
                kk = info["kinds"]
                row[name] = {"converged": bool(r["converged"]), "iterations": len(kk),
                             "by_kind": {kinds[k]: kk.count(k) for k in sorted(set(kk))},
                             "EMermin": r["energies"]["EMermin"]}
            row["dE_per_atom"] = abs(row["fp64"]["EMermin"] - row["mixed"]["EMermin"]) / len(ss)
            counts.append(row)
            cx.close()
    model_eval = None
    conv = [r for r in counts if r["fp64"]["converged"] and r["mixed"]["converged"]]
    if conv:
        big = conv[-1]
        n64 = big["fp64"]["iterations"]
        bk = big["mixed"]["by_kind"]
        t64 = t_geom + fp64["iter_s"][0] + (n64 - 1) * t_fp64_iter + fp64["grad_s"]
        tmx = (t_geom_mixed + per["fp32_first"] + (bk.get("fp32", 0) - 1) * per["fp32"]
               + bk.get("fp64_class", 0) * per["fp64_class"] + bk.get("perturbative", 0) * per["perturbative"]
               + mixed["grad_s"])
        model_eval = {"basis": f"iteration counts of the converged {big['ti']}-Ti sphere x per-iteration costs "
                               f"measured at full size (a model, not a timed evaluation)",
                      "fp64_s": t64, "mixed_s": tmx, "mixed_vs_fp64": t64 / tmx}
    line = {"mode": "per-iteration", "config": {"workload": args.config, "orbitals": norb, "kT": KT,
                                                "scc_tol": SCC_TOL, "mix_alpha": mix},
            "fp64": {"set_geometry_s": t_geom, "iteration_s": fp64["iter_s"], "gradients_s": fp64["grad_s"]},
            "mixed": {"set_geometry_s": t_geom_mixed, "iteration_s": per, "gradients_s": mixed["grad_s"]},
            "fp64_iteration_vs_mixed_fp32_iteration": t_fp64_iter / per["fp32"],
            "convergence": counts, "evaluation_model": model_eval}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="h2o1024", choices=sorted(CONFIGS) + ["batch4096", "tio2"])
    ap.add_argument("--no-batch", action="store_true", help="leave the batched workload out of the default line")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--per-iteration", action="store_true",
                    help="time one iteration of each kind instead of whole evaluations (large configurations)")
    ap.add_argument("--mix-alpha", type=float, default=0.1, help="Broyden mixing of --per-iteration")
    args = ap.parse_args()
    if args.per_iteration:
        run_per_iteration(args)
    elif args.impl == "reference":
        run_reference(args)
    elif args.config == "batch4096":
        run_batch(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
