"""Benchmark: determinant-CI sigma builds per second at CAS(16e,16o), one GB300 per rank.

One step = one sigma = H C build over the full CAS(16e,16o) Ms=0 determinant space
(12870 x 12870 = 165,636,900 determinants, FP64 vectors of 1.32 GB, larger than L2, so no
L2 flush is needed between steps), seeded synthetic integrals (naux = 64) and a seeded C.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

value     sigma builds/s of the FP64 path with C and sigma resident in HBM (whole job: N ranks
          run independent replicas, weak scaling).
e2e       the same through the public host-buffer API: CISigmaBuilder.Hamiltonian(numpy C,
          numpy sigma) from pinned host memory, H2D + build + D2H inside the timed region.
roofline  the dominant kernel (opposite-spin k_opposite): algorithmic FLOPs per launch
          2 N1a N1b (ma mb)^2 over its CUDA-event duration, against the measured FP64 peak.
--impl reference times the reference algorithm's CPU implementation (the oracle port of the
          Harrison-Zarrabian sigma, all host threads, BLAS from numpy's OpenBLAS) on a bounded
          sample of the same build.
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

from forte2_gb300.synthetic import cas_dims, hz_flops, make_integrals, random_ci_vector, sparse_flops  # noqa: E402

NORB, NEL = 16, 16
ISEED, CSEED = 3000, 114
FP64_DGEMM_TFLOPS = 1.098  # torch.matmul FP64 8192^3 (cuBLAS DGEMM) on this GB300 pool, for context
FP32_PEAK_TFLOPS = 69.70  # measured torch.matmul FP32 (no TF32) 8192^3
METRIC = "CAS(16,16) sigma-builds/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--norb", type=int, default=NORB)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="sigma mode: keep the default kernel variants")
    ap.add_argument("--instances", type=int, default=64, help="batched mode: number of instances")
    ap.add_argument("--requests", type=int, default=10000, help="serve mode: number of requests")
    ap.add_argument("--rate", type=float, default=200.0, help="serve mode: mean arrivals per second")
    ap.add_argument("--unbatched-requests", type=int, default=0,
                    help="serve mode: also serve the first N requests one at a time with a fresh plain "
                         "solver each (the unbatched plain path) and, for comparison, batched")
    ap.add_argument("--mode", default="sigma", choices=["sigma", "davidson", "batched", "serve", "rdm", "blocked"],
                    help="sigma: sigma-builds/s (default); davidson: time to solution, FP64 vs mixed")
    ap.add_argument("--nroot", type=int, default=1)
    ap.add_argument("--e-tol", type=float, default=1e-10)
    ap.add_argument("--precisions", default="fp64,mixed", help="davidson mode: which solves to run")
    ap.add_argument("--maxiter", type=int, default=400, help="davidson mode: iteration limit")
    ap.add_argument("--basis-per-root", type=int, default=0, help="davidson mode: subspace vectors per root "
                                                                  "(0: the reference's default, FP64)")
    ap.add_argument("--collapse-per-root", type=int, default=0)
    ap.add_argument("--no-davidson", action="store_true",
                    help="sigma mode: skip the Davidson time-to-solution runs of the default line")
    return ap.parse_args()


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, max clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for name, val in zip(names, r[5:9]):
                if val.strip() == "Active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_fma_peak(reps=3):
    """FP64 FMA issue rate of this GPU from the library's own probe (k_probe_dfma: 16 independent
    DFMA chains per thread, 8 blocks of 256 threads per SM), timed with CUDA events on the
    launching stream after one warm-up launch; the best of `reps` launches (burst), in TFLOP/s."""
    import torch

    from forte2_gb300._lib import check, lib, stream_handle

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks, threads, iters = 8 * sms, 256, 1 << 14
    out = torch.empty(blocks, dtype=torch.float64, device="cuda")
    st = torch.cuda.current_stream()
    check(lib().f2g_probe_dfma(blocks, threads, iters, out.data_ptr(), stream_handle()))
    best = 0.0
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        check(lib().f2g_probe_dfma(blocks, threads, iters, out.data_ptr(), stream_handle()))
        e1.record(st)
        torch.cuda.synchronize()
        best = max(best, 32.0 * blocks * threads * iters / (e0.elapsed_time(e1) / 1e3) / 1e12)
    assert bool(torch.isfinite(out).all())
    return best


def _measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def fp64_nominal_peak(sm_mhz):
    """GB300's FP64 rate, 4 FLOP (2 DFMA) per clock per SM, at the median SM clock sampled during
    the run (1.26 TFLOP/s at 2070 MHz; the nominal 1.25 TFLOP/s). The library's own issue-rate
    probe is reported beside it: it stays below what the opposite-spin kernel itself sustains, so it
    cannot serve as the ceiling."""
    import torch

    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    return 4.0 * sms * (sm_mhz or 2070.0) * 1e6 / 1e12


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count()


def cpu_baseline(norb, budget_s, na, nb, ints, c):
    """Reference algorithm (HZ, BLAS K-blocks, 1 GiB) on all host cores, bounded sample: the first
    fraction f of every term's K-block chunks; rate = f / time. Returns (builds/s, sample text)."""
    from oracle.port import PortCI, build_port, open_blas

    build_port()
    cores = cpu_cores()
    os.environ["ORACLE_THREADS"] = str(cores)
    blas = open_blas(threads=cores)
    p = PortCI(norb, na, nb)
    p.set_hamiltonian(ints.E, ints.H, ints.V)
    # Two timed samples f0 < f1 of every term's K-block chunks. Time is linear in f with a fixed
    # per-call part O (vector fills and transposes): t = O + f T, so one full build takes O + T.
    f0 = 0.002
    p.set_fraction(f0)
    t = time.perf_counter()
    p.sigma(c)
    t0 = time.perf_counter() - t
    f1 = min(1.0, max(4 * f0, f0 * budget_s / max(t0, 1e-3)))
    p.set_fraction(f1)
    t = time.perf_counter()
    p.sigma(c)
    t1 = time.perf_counter() - t
    T = max((t1 - t0) / (f1 - f0), 1e-9)
    O = max(t0 - f0 * T, 0.0)
    full = O + T
    sample = (f"two samples of one CAS({2 * na}e,{norb}o) FP64 HZ sigma build: the first {f0:.4f} and {f1:.4f} of "
              f"every term's 1 GiB K-block chunks ({t0:.1f} s, {t1:.1f} s); full build = fixed {O:.2f} s + "
              f"{T:.1f} s linear part; OpenBLAS {'numpy-bundled' if blas else 'absent: plain loops'}, {cores} threads")
    return 1.0 / full, sample, cores


def dist_setup(n_gpus):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        return rank, world, local, dist
    torch.cuda.set_device(0)
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(x, dist):
    """Largest value over the ranks (the job's time is its slowest replica's)."""
    if dist is None:
        return x
    import torch

    device = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank, t_local, dist):
    """Whole-job rate of independent replicas: all ranks' units over the slowest rank's time."""
    world = dist.get_world_size() if dist is not None else 1
    return world * units_per_rank / max_over_ranks(t_local, dist)


def opposite_traffic(norb, na, nb):
    """DRAM bytes of one FP64 opposite-spin launch, scaled from the ncu capture at norb 15, na 7,
    nb 8 (dram__bytes_read + dram__bytes_write = 4.71 + 0.33 GB) by the gathered C elements
    N0a * na * N1b * ma * mb (the kernel's reads; the traffic grows with them)."""
    from math import comb

    def gathered(n, a, b):
        return comb(n, a) * a * comb(n, b - 1) * (n - a + 1) * (n - b + 1)

    return 5.04e9 * gathered(norb, na, nb) / gathered(15, 7, 8)


def run_gb300(a):
    import torch

    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    rank, world, local, dist = dist_setup(a.gpus)
    na, nb, n0a, n0b, ndet = cas_dims(a.norb, a.norb, 0)
    ints = make_integrals(a.norb, ISEED)
    strings = CIStrings(na, nb, 0, [[0] * a.norb], [], [])
    sb = CISigmaBuilder(strings, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    c_host = random_ci_vector(ndet, CSEED)
    C = torch.as_tensor(c_host, device="cuda")
    S = torch.empty_like(C)
    stream = torch.cuda.current_stream()
    tuned = None
    if not a.no_autotune:
        # kernel variants with identical results, timed on this workload (forte2_gb300.autotune)
        from forte2_gb300.autotune import autotune_sigma

        tuned = {p: autotune_sigma(sb, a.norb, na, nb, p, reps=1) for p in (("fp64",) if a.no_mixed else ("fp64", "fp32"))}
    for _ in range(a.warmup):
        sb.Hamiltonian(C, S)
    torch.cuda.synchronize()
    sb.reset_build_times()
    clocks = Clocks(local)
    clocks.start()
    fp64_peak = fp64_fma_peak()  # roofline denominator, measured under the same clock sampling
    barrier(dist)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(a.steps):
        sb.Hamiltonian(C, S)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clk = clocks.stop()
    peak64 = fp64_nominal_peak(clk.get("sm_mhz"))
    t_local = ev0.elapsed_time(ev1) / 1e3
    t = max_over_ranks(t_local, dist)
    value = replica_rate(a.steps, t_local, dist)
    # per-term averages over warmup + timed builds (CUDA events around each phase)
    tot, t_ab, t_aa, t_bb = sb.avg_build_time()
    f_sp = sparse_flops(a.norb, na, nb)
    f_hz = hz_flops(a.norb, na, nb)
    achieved = f_sp["ab"] / t_ab / 1e12
    # e2e through the public host-buffer API, pinned host memory
    pin_c = torch.empty(ndet, dtype=torch.float64).pin_memory()
    pin_s = torch.empty(ndet, dtype=torch.float64).pin_memory()
    pin_c.numpy()[:] = c_host
    hc, hs = pin_c.numpy(), pin_s.numpy()
    sb.Hamiltonian(hc, hs)
    barrier(dist)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        sb.Hamiltonian(hc, hs)
    e2e_t = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = world * a.steps / e2e_t
    check = float(np.linalg.norm(hs))
    # mixed mode (FP32 sigma) throughput, same workload
    mixed = None
    mixed_terms = None
    tc_roof = None
    if not a.no_mixed:
        sb.set_precision("fp32")
        for _ in range(2):
            sb.Hamiltonian(C, S)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.steps):
            sb.Hamiltonian(C, S)
        e1.record(stream)
        torch.cuda.synchronize()
        mixed = world * a.steps / max_over_ranks(e0.elapsed_time(e1) / 1e3, dist)
        mt = sb.avg_build_time()
        mixed_terms = {"total": 1e3 * mt[0], "aabb": 1e3 * mt[1], "aaaa_h1a_h0": 1e3 * mt[2], "bbbb_h1b": 1e3 * mt[3]}
        if sb.set_tensor_cores(True):
            # k_opposite_tc: 3 split-FP16 products of M = 128, N = 256, K padded to 16, per tile of
            # 128 beta strings, per alpha string; against the measured dense BF16/FP16 GEMM peak
            from math import comb

            kp = (na * (a.norb - na + 1) + 15) // 16 * 16
            tiles = comb(a.norb, na) * ((comb(a.norb, nb) + 127) // 128)
            tc_flop = 3 * 2 * 128 * 256 * kp * tiles
            bf16 = _measured_peaks().get("bf16_tflops", 1900.0)
            tc_roof = {"bound": "tensor", "kernel": "k_opposite_tc (FP32 opposite-spin sigma, split FP16)",
                       "flop_per_launch": tc_flop, "launch_ms": mt[1] * 1e3,
                       "achieved": tc_flop / mt[1] / 1e12, "peak": bf16, "unit": "TFLOP/s",
                       "frac": tc_flop / mt[1] / 1e12 / bf16,
                       "peak_source": "MEASURED_PEAKS.json bf16_tflops (dense FP16 runs at the BF16 rate)"}
        sb.set_precision("fp64")
    davidson = None
    serving = None
    if rank == 0 and world == 1 and not a.no_davidson and a.norb == NORB:
        davidson = davidson_acceptance()
        serving = serving_sample()
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        v, sample, cores = cpu_baseline(a.norb, a.cpu_seconds, na, nb, ints, c_host)
        cpu = {"value": v, "unit": "sigma-builds/s", "cores": cores, "kind": "port", "sample": sample}
    if rank == 0:
        line = {
            "metric": METRIC if a.norb == NORB else f"CAS({a.norb},{a.norb}) sigma-builds/s",
            "value": value, "unit": "sigma-builds/s", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": 1e3 * t / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded integrals, naux=4n; seeded C)",
            "config": {"workload": f"CAS({a.norb}e,{a.norb}o) Ms=0 FP64 sigma build, {ndet} determinants",
                       "ndet": ndet, "norb": a.norb, "na": na, "nb": nb, "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1.32 GB vectors), no flush"},
            "e2e": {"value": e2e, "unit": "sigma-builds/s", "h2d_bytes_per_step": 8 * ndet,
                    "d2h_bytes_per_step": 8 * ndet},
            "gpu_launches": 5 * a.steps,
            "roofline": {"bound": "compute", "pipe": "fp64", "kernel": "k_opposite (opposite-spin sigma)",
                         "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                         "frac": achieved / peak64, "traffic": opposite_traffic(a.norb, na, nb),
                         "traffic_source": "dram read+write per gathered C element of the ncu capture at "
                                           "CAS(15e,15o) (profiles/k_opposite_fp64_cas15.md: 5.04 GB for "
                                           "2.09e10 elements), times this launch's gathered elements",
                         "peak_source": "FP64 rate 4 FLOP/clk/SM x SMs x median SM clock sampled in this run "
                                        "(no FP64 entry in MEASURED_PEAKS.json)",
                         "probe_tflops": fp64_peak, "frac_of_probe": achieved / fp64_peak,
                         "probe_source": "the library's DFMA issue-rate probe (k_probe_dfma, 16 chains per thread, "
                                         "best of 3 launches, CUDA events), measured in this run",
                         "fp64_dgemm_tflops": FP64_DGEMM_TFLOPS, "frac_of_dgemm": achieved / FP64_DGEMM_TFLOPS,
                         "flops_per_launch": f_sp["ab"], "launch_ms": 1e3 * t_ab,
                         # the reference's dense HZ product counts n^2 x n^2 blocks whose D rows are
                         # mostly zero; the kernel skips exactly those (same sigma to 1e-12)
                         "dense_hz_flops_per_launch": f_hz["ab"],
                         "dense_hz_equivalent_tflops": f_hz["ab"] / t_ab / 1e12,
                         "algorithmic_bytes": 24 * ndet,
                         "traffic_over_algorithmic": opposite_traffic(a.norb, na, nb) / (24 * ndet)},
            "terms_ms": {"total": 1e3 * tot, "aabb": 1e3 * t_ab, "aaaa_h1a_h0": 1e3 * t_aa, "bbbb_h1b": 1e3 * t_bb},
            "same_spin": same_spin_rates(a.norb, na, nb, ndet, t_aa, t_bb),
            "hz_dense_flops": f_hz, "sparse_flops": f_sp,
            "autotune": None if tuned is None else {p: {"choice": r["choice"], "ms": r["ms"], "default_ms": r["default_ms"]}
                                                    for p, r in tuned.items()},
            "davidson": davidson,
            "serving": serving,
            "mixed_fp32_sigma_builds_per_s": mixed,
            "tensor_core_roofline": tc_roof,
            "mixed_fp32_terms_ms": mixed_terms,
            "clocks": clk,
            "cpu_baseline": cpu,
            "sigma_norm": check,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def cpu_full_build(norb, na, nb, ints, c):
    """One complete reference-algorithm sigma build (HZ, every K-block chunk) on all host cores,
    after one small warm-up sample (thread pools, first-touch pages). Returns (seconds, cores)."""
    from oracle.port import PortCI, build_port, open_blas

    build_port()
    cores = cpu_cores()
    os.environ["ORACLE_THREADS"] = str(cores)
    open_blas(threads=cores)
    p = PortCI(norb, na, nb)
    p.set_hamiltonian(ints.E, ints.H, ints.V)
    p.set_fraction(0.001)
    p.sigma(c)
    p.set_fraction(1.0)
    t = time.perf_counter()
    p.sigma(c)
    return time.perf_counter() - t, cores


GPU_FP64_FIXTURE = os.path.join(ROOT, "tests", "golden", "davidson_gpu_fp64_cas16.json")


def davidson_acceptance():
    """Time to solution of the metric's Davidson part, run in the default line:

    * CAS(16e,16o), 1 root, mixed precision, e_tol 1e-10: wall time and |E_mixed - E_FP64| against
      the converged plain FP64 GPU solve of the same integrals (a committed GPU fixture: the CPU
      oracle would need about a day here; FP64 parity is pinned at smaller sizes), and the FP64 /
      mixed time ratio against that fixture's measured FP64 times;
    * CAS(14e,14o), 3 roots, both precisions measured here (plain FP64 with the reference's
      subspace), their energy differences and time ratio.
    """
    out = {}
    m16 = casci_time_to_solution(16, 1, "mixed", 1e-10, 2000, ISEED)
    out["cas16_1root_mixed"] = m16
    if os.path.exists(GPU_FP64_FIXTURE):
        with open(GPU_FP64_FIXTURE) as f:
            fx = json.load(f)
        out["cas16_fp64_fixture"] = {k: fx[k] for k in ("energies", "runs", "command") if k in fx}
        out["cas16_abs_dE_mixed_vs_fp64"] = [abs(x - y) for x, y in zip(m16["energies"], fx["energies"])]
        out["cas16_fp64_over_mixed_time"] = {name: r["seconds_total"] / m16["seconds_total"]
                                             for name, r in fx["runs"].items()}
    r14 = {prec: casci_time_to_solution(14, 3, prec, 1e-10, 1000, 1014) for prec in ("fp64", "mixed")}
    out["cas14_3roots"] = r14
    out["cas14_abs_dE_mixed_vs_fp64"] = [abs(x - y) for x, y in zip(r14["mixed"]["energies"], r14["fp64"]["energies"])]
    out["cas14_fp64_over_mixed_time"] = r14["fp64"]["seconds_total"] / r14["mixed"]["seconds_total"]
    return out


def run_reference(a):
    """Reference arm: the reference's HZ algorithm on the host cores (oracle port), rank 0 only.

    The timed step is ONE complete sigma build (value = 1 / its time). The two-sample model of the
    GPU arm's cpu_baseline is run beside it and its prediction and error are reported. A complete
    build that the model puts above 240 s is not run; the model's rate is reported instead."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    na, nb, n0a, n0b, ndet = cas_dims(a.norb, a.norb, 0)
    ints = make_integrals(a.norb, ISEED)
    c = random_ci_vector(ndet, CSEED)
    model_rate, model_sample, cores = cpu_baseline(a.norb, min(a.cpu_seconds, 10.0), na, nb, ints, c)
    model_s = 1.0 / model_rate
    full_s = None
    if model_s <= 240.0:
        full_s, cores = cpu_full_build(a.norb, na, nb, ints, c)
    value = 1.0 / full_s if full_s else model_rate
    sample = (f"one complete CAS({2 * na}e,{a.norb}o) FP64 HZ sigma build ({full_s:.1f} s) on {cores} threads, "
              f"after a 0.1% warm-up sample" if full_s else
              f"model only (a complete build is predicted to take {model_s:.0f} s): " + model_sample)
    print(json.dumps({
        "impl": "reference", "metric": METRIC if a.norb == NORB else f"CAS({a.norb},{a.norb}) sigma-builds/s",
        "value": value, "unit": "sigma-builds/s", "n_gpus": world, "steps": 1 if full_s else 0,
        "requested_steps": a.steps, "warmup": 1, "ms_per_step": 1e3 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded integrals, naux=4n; seeded C)",
        "config": {"workload": f"CAS({a.norb}e,{a.norb}o) Ms=0 FP64 sigma build, {ndet} determinants", "ndet": ndet},
        "cpu_baseline": {"value": value, "unit": "sigma-builds/s", "cores": cores, "kind": "port", "sample": sample},
        "measured_full_build_s": full_s,
        "model": {"full_build_s": model_s, "sample": model_sample,
                  "rel_error_vs_measured": (model_s - full_s) / full_s if full_s else None},
        "e2e": {"value": value, "unit": "sigma-builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }), flush=True)


def casci_time_to_solution(norb, nroot, prec, e_tol, maxiter, iseed, basis_per_root=None, collapse_per_root=None):
    """One CASCI(n e, n o) Ms=0 singlet solve on the GPU, wall time from the solver's creation to
    its energies on the host (strings, CSF set-up, guess, Davidson-Liu)."""
    import torch

    from forte2_gb300.ci import CASCISolver
    from forte2_gb300.params import CIParams, DavidsonLiuParams

    na, nb, _, _, _ = cas_dims(norb, norb, 0)
    ints = make_integrals(norb, iseed)
    dl = DavidsonLiuParams(e_tol=e_tol, maxiter=maxiter)
    if basis_per_root:
        dl = DavidsonLiuParams(e_tol=e_tol, maxiter=maxiter, basis_per_root=basis_per_root,
                               collapse_per_root=collapse_per_root)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sol = CASCISolver(norb=norb, na=na, nb=nb, multiplicity=1, nroot=nroot, E=ints.E, H=ints.H, V=ints.V,
                      ci_params=CIParams(precision=prec), davidson_liu_params=dl).run()
    torch.cuda.synchronize()
    r = {"seconds_total": time.perf_counter() - t0, "seconds_davidson": sol.timings["davidson"],
         "seconds_setup": sol.timings.get("startup", 0.0) + sol.timings.get("setup", 0.0),
         "converged": bool(sol.converged), "phases": sol.phases, "energies": [float(e) for e in sol.evals],
         "ncsf": sol.basis_size, "subspace": [sol.eigensolver.basis_per_root, sol.eigensolver.collapse_per_root],
         "iterations": sum(p[1] for p in sol.phases if not p[0].endswith("check"))}
    r["seconds_per_iteration"] = r["seconds_davidson"] / max(1, r["iterations"])
    del sol
    torch.cuda.empty_cache()
    return r


def serving_sample(n_requests=1000, rate=200.0):
    """The metric's latency part in the default line: a 1,000-request Poisson stream of the serving
    workload's distribution ((6e,6o)-(16e,16o) weighted 1/Ndet, 200 requests/s, seed 5), served by
    continuous batching in both precisions; p50/p99 from arrival to result and solves/s. The
    10,000-request stream runs with --mode serve."""
    from forte2_gb300.serve import default_prewarm, poisson_stream, serve

    out = {"workload": f"{n_requests} requests, Poisson {rate}/s, (6e,6o)-(16e,16o) weight 1/Ndet, multiplicity "
                       "1/3, 1-3 roots, e_tol 1e-10 (the full 10,000-request stream: --mode serve)"}
    for prec in ("fp64", "mixed"):
        stats, _, _ = serve(poisson_stream(n_requests, rate=rate), precision=prec, prewarm=default_prewarm())
        out[prec] = {k: stats[k] for k in ("solves_per_s", "p50_latency_s", "p99_latency_s", "mean_latency_s",
                                            "wall_s", "max_inflight", "sizes")}
    return out


def same_spin_rates(norb, na, nb, ndet, t_aa, t_bb):
    """The FP64 same-spin terms: FP64 rate of their string-Hamiltonian products, and HBM rate of
    their algorithmic bytes (24 B per determinant per term pass: read C, read and write sigma; the
    beta term also transposes C and sigma, two more passes)."""
    from math import comb

    peak = _measured_peaks().get("hbm_gbs") or 6801.7
    out = {"hbm_peak_gbs": peak, "bound": "fp64 pipe (the products), the passes are HBM"}
    for spin, k, t in (("alpha_h1a_h0", na, t_aa), ("beta_h1b", nb, t_bb)):
        nnz = 1 + k * (norb - k) + comb(k, 2) * comb(norb - k, 2)
        flops = 2 * ndet * (nnz - 1)
        b = 24 * ndet
        out[spin] = {"ms": 1e3 * t, "flops": flops, "tflops": flops / t / 1e12, "algorithmic_bytes": b,
                     "achieved_gbs": b / t / 1e9, "frac_of_hbm": b / t / 1e9 / peak}
    return out


def run_davidson(a):
    """Davidson-Liu CASCI time to solution on one GPU: plain FP64 and mixed (FP32 iterations then
    FP64 refinement), same seeded integrals; energies of the mixed run against the FP64 run."""
    import torch

    torch.cuda.set_device(0)
    na, nb, _, _, ndet = cas_dims(a.norb, a.norb, 0)
    out = {"metric": f"CAS({a.norb},{a.norb}) Davidson time to solution", "unit": "s", "higher_is_better": False,
           "config": {"workload": f"CAS({a.norb}e,{a.norb}o) Ms=0 singlet, {a.nroot} root(s), e_tol {a.e_tol}, "
                                  f"r_tol 1e-6", "ndet": ndet,
                      "subspace": "reference default" if not a.basis_per_root else
                                  f"{a.basis_per_root}/{a.collapse_per_root} per root"}}
    res = {}
    for prec in a.precisions.split(","):
        res[prec] = casci_time_to_solution(a.norb, a.nroot, prec, a.e_tol, a.maxiter,
                                           ISEED if a.norb == NORB else 1000 + a.norb,
                                           a.basis_per_root, a.collapse_per_root)
        print(json.dumps({"partial": prec, **res[prec]}), flush=True)  # each precision as soon as it is done
    out.update(res)
    if "fp64" in res and "mixed" in res:
        out["mixed_vs_fp64_abs_dE"] = [abs(x - y) for x, y in zip(res["mixed"]["energies"], res["fp64"]["energies"])]
        out["speedup_mixed_over_fp64_davidson"] = res["fp64"]["seconds_davidson"] / res["mixed"]["seconds_davidson"]
    out["csf_transforms"] = csf_transform_roofline(a.norb)
    print(json.dumps(out), flush=True)


def csf_transform_roofline(norb):
    """The FP64 CSF <-> determinant transforms of one singlet vector at CAS(n e, n o), timed alone
    with CUDA events, against HBM: algorithmic bytes B_csf = 8 (ncsf + ndet) + 12 ncoupling (the two
    vectors once, every coupling's coefficient and determinant address once) per transform."""
    import torch

    from forte2_gb300.ci_helpers import CISpinAdapter, CIStrings

    na, nb, _, _, ndet = cas_dims(norb, norb, 0)
    s = CIStrings(na, nb, 0, [[0] * norb], [], [])
    sa = CISpinAdapter(0, 0, norb)
    sa.prepare_couplings(s.make_determinants())
    csf = torch.from_numpy(random_ci_vector(sa.ncsf, 5)).cuda()
    det = torch.empty(ndet, dtype=torch.float64, device="cuda")
    back = torch.empty_like(csf)
    st = torch.cuda.current_stream()
    peak = _measured_peaks().get("hbm_gbs") or 6801.7
    out = {"ncsf": sa.ncsf, "ndet": ndet, "ncoupling": sa.ncoupling,
           "bytes_per_transform": 8 * (sa.ncsf + ndet) + 12 * sa.ncoupling, "hbm_peak_gbs": peak}
    for name, f in (("csf_to_det", lambda: sa.csf_C_to_det_C(csf, det)), ("det_to_csf", lambda: sa.det_C_to_csf_C(det, back))):
        f()
        f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(5):
            f()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / 5
        gbs = out["bytes_per_transform"] / (ms * 1e-3) / 1e9
        out[name] = {"ms": ms, "achieved_gbs": gbs, "frac_of_hbm": gbs / peak}
    del sa, s
    torch.cuda.empty_cache()
    return out


def rdm_cpu_baseline(norb, na, nb, c, budget_s):
    """The oracle's spin-free 1- and 2-RDM of one vector on all host cores, bounded sample: the
    first fraction f of every hole-string loop; t = O + f T, one full set = O + T."""
    from oracle.port import PortCI, build_port

    build_port()
    cores = cpu_cores()
    os.environ["ORACLE_THREADS"] = str(cores)
    p = PortCI(norb, na, nb)

    def timed(f):
        p.set_fraction(f)
        t = time.perf_counter()
        p.rdm("sf_1rdm", c, c)
        p.rdm("sf_2rdm", c, c)
        return time.perf_counter() - t

    f0 = 0.001
    t0 = timed(f0)
    f1 = min(1.0, max(4 * f0, f0 * budget_s / max(t0, 1e-3)))
    t1 = timed(f1)
    T = max((t1 - t0) / (f1 - f0), 1e-9)
    O = max(t0 - f0 * T, 0.0)
    sample = (f"two samples of one CAS({na + nb}e,{norb}o) sf_1rdm + sf_2rdm: the first {f0:.4f} and {f1:.4f} of "
              f"every hole-string loop ({t0:.1f} s, {t1:.1f} s); full set = fixed {O:.2f} s + {T:.1f} s linear part; "
              f"{cores} threads")
    return 1.0 / (O + T), sample, cores


def run_rdm(a):
    """Spin-free 1- and 2-RDM of one CI vector (the CI driver's make_sf_1rdm + make_sf_2rdm,
    ci.py:655-699) at CAS(n e, n o), FP64, vector resident in HBM; e2e through the host-array API."""
    import torch

    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings

    torch.cuda.set_device(0)
    n = a.norb
    na, nb, N0a, N0b, ndet = cas_dims(n, n, 0)
    ints = make_integrals(n, ISEED if n == NORB else 1000 + n)
    strings = CIStrings(na, nb, 0, [[0] * n], [], [])
    sb = CISigmaBuilder(strings, ints.E, ints.H, ints.V, 0)
    c_host = random_ci_vector(ndet, CSEED)
    c = torch.from_numpy(c_host).cuda()
    st = torch.cuda.current_stream()

    def step():
        sb.sf_1rdm(c, c)
        sb.sf_2rdm(c, c)

    for _ in range(a.warmup):
        step()
    torch.cuda.synchronize()
    clocks = Clocks()
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(a.steps):
        step()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.steps
    # dominant kernel: the mixed-spin 2-RDM (k_rdm_ab + its mirror), timed alone
    ab_ms = []
    for _ in range(3):
        x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        x0.record(st)
        sb.ab_2rdm(c, c)
        x1.record(st)
        torch.cuda.synchronize()
        ab_ms.append(x0.elapsed_time(x1))
    fp64_peak = fp64_fma_peak()
    clk = clocks.stop()
    # algorithmic FP64 work of k_rdm_ab with bra = ket: alpha pair entries with u <= x times all
    # beta pair entries, one multiply-add each
    from math import comb

    alpha_sym = n * comb(n - 1, na - 1) + n * (n - 1) // 2 * comb(n - 2, na - 1)
    beta_all = comb(n, nb - 1) * (n - nb + 1) ** 2
    ab_flop = 2.0 * alpha_sym * beta_all
    ab_s = statistics.median(ab_ms) / 1e3
    # end to end through the host-array API (numpy in, numpy out)
    t = time.perf_counter()
    for _ in range(a.steps):
        sb.sf_1rdm(c_host, c_host)
        sb.sf_2rdm(c_host, c_host)
    torch.cuda.synchronize()
    e2e_s = (time.perf_counter() - t) / a.steps
    out = {"metric": f"CAS({n},{n}) spin-free 1+2-RDM sets/s", "value": 1e3 / ms, "unit": "RDM sets/s",
           "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"CAS({n}e,{n}o) Ms=0, sf_1rdm + sf_2rdm of one seeded normalised vector "
                                  f"(bra = ket), {ndet} determinants, vector {ndet * 8 / 2**30:.2f} GiB > L2"},
           "e2e": {"value": 1.0 / e2e_s, "unit": "RDM sets/s", "h2d_bytes_per_step": 2 * ndet * 8,
                   "d2h_bytes_per_step": (n * n + n ** 4) * 8},
           "roofline": {"bound": "compute", "pipe": "fp64", "kernel": "k_rdm_ab (mixed-spin 2-RDM, with its mirror)",
                        "achieved": ab_flop / ab_s / 1e12,
                        "peak": fp64_nominal_peak(clk.get("sm_mhz")), "unit": "TFLOP/s",
                        "frac": ab_flop / ab_s / 1e12 / fp64_nominal_peak(clk.get("sm_mhz")),
                        "flop_per_launch": ab_flop, "ms": ab_s * 1e3, "traffic": None,
                        "peak_source": "FP64 rate 4 FLOP/clk/SM x SMs x median SM clock sampled in this run",
                        "probe_tflops": fp64_peak, "fp64_dgemm_tflops": FP64_DGEMM_TFLOPS},
           "clocks": clk,
           # per set: k_rdm_hole<1> x2, k_transpose x2, k_rdm_ab, its mirror, k_rdm_hole<2> x2, k_rdm_sf2
           "gpu_launches": 9 * a.steps}
    # three-body RDMs (make_sf_3rdm / make_sf_3cumulant) at CAS(14e,14o): one warm call, one timed
    n3 = min(n, 14)
    na3, nb3, _, _, ndet3 = cas_dims(n3, n3, 0)
    s3 = CIStrings(na3, nb3, 0, [[0] * n3], [], [])
    ints3 = make_integrals(n3, 1000 + n3)
    sb3 = CISigmaBuilder(s3, ints3.E, ints3.H, ints3.V, 0)
    c3 = torch.from_numpy(random_ci_vector(ndet3, CSEED)).cuda()
    sb3.sf_3rdm(c3, c3)
    three = {}
    for kind in ("aab_3rdm", "aaa_3rdm", "sf_3rdm", "sf_3cumulant"):
        x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        x0.record(st)
        getattr(sb3, kind)(c3, c3)
        x1.record(st)
        torch.cuda.synchronize()
        three[kind + "_ms"] = x0.elapsed_time(x1)
    out["three_body"] = {"workload": f"CAS({n3}e,{n3}o), one seeded vector (bra = ket), {ndet3} determinants",
                         **three}
    del sb3, s3
    if not a.no_cpu_baseline:
        v, sample, cores = rdm_cpu_baseline(n, na, nb, c_host, a.cpu_seconds)
        out["cpu_baseline"] = {"value": v, "unit": "RDM sets/s", "cores": cores, "kind": "port", "sample": sample}
    print(json.dumps(out), flush=True)


def run_batched(a):
    """64 independent CASCI instances, (8e,8o)-(12e,12o), multiplicities 1/3, 1-4 roots, solved
    concurrently by the step scheduler, against a loop of plain single solves."""
    import torch

    from forte2_gb300.batch import batched_instances, solve_batched, solve_loop

    torch.cuda.set_device(0)
    inst = batched_instances(a.instances)
    solve_batched(inst[:4])  # warm-up: library load, kernel attributes, allocator
    out = {"metric": "batched CASCI instances/s", "unit": "instances/s", "higher_is_better": True,
           "config": {"workload": f"{len(inst)} CASCI instances, (8e,8o)-(12e,12o), Ms=0, multiplicity 1/3, "
                                  "1-4 roots, e_tol 1e-10", "sizes": {n: sum(1 for x in inst if x['norb'] == n)
                                                                      for n in (8, 10, 12)}}}
    for prec in a.precisions.split(","):
        res_b, t_b, rounds = solve_batched(inst, prec)
        st = {}
        res_o, t_o, _ = solve_batched(inst, prec, one_launch=True, stats=st)
        res_l, t_l = solve_loop(inst, prec)
        dev = max(max(abs(x - y) for x, y in zip(res_b[i].evals, res_l[i].evals)) for i in range(len(inst)))
        dev_o = max(max(abs(x - y) for x, y in zip(res_o[i].evals, res_l[i].evals)) for i in range(len(inst)))
        out[prec] = {"batched_s": t_b, "loop_s": t_l, "instances_per_s": len(inst) / t_b,
                     "loop_instances_per_s": len(inst) / t_l, "speedup": t_l / t_b, "rounds": rounds,
                     "all_converged": all(res_b[i].converged for i in range(len(inst))),
                     "max_abs_dE_batched_vs_loop": dev,
                     # every instance's iterations in collective graph launches (one while loop per
                     # solve inside one graph), set-up on the instances' own streams
                     "one_launch": {"s": t_o, "instances_per_s": len(inst) / t_o, "speedup": t_l / t_o,
                                    "all_converged": all(res_o[i].converged for i in range(len(inst))),
                                    "max_abs_dE_vs_loop": dev_o, **st}}
    print(json.dumps(out), flush=True)


def run_serve(a):
    """Poisson stream of CASCI solves (6e,6o)-(16e,16o) weighted 1/Ndet, continuous batching under
    an HBM budget; p50/p99 latency from arrival to result, and solves/s."""
    import torch

    from forte2_gb300.serve import default_prewarm, poisson_stream, serve

    torch.cuda.set_device(0)
    reqs = poisson_stream(a.requests, rate=a.rate)
    serve(poisson_stream(20, rate=1000.0, seed=99, sizes=(6, 8)))  # warm-up: library load, allocator
    out = {"metric": "solve-stream p50/p99 latency", "unit": "s", "higher_is_better": False,
           "config": {"workload": f"{len(reqs)} requests, Poisson {a.rate}/s, (6e,6o)-(16e,16o) weight 1/Ndet, "
                                  "multiplicity 1/3, 1-3 roots, e_tol 1e-10"}}
    out["config"]["prewarm"] = "idle solvers created before the stream: 16 per (6e,6o), 6 per (8e,8o), 2 per " \
                               "(10e,10o) shape (multiplicity 1/3 x 1-3 roots)"
    for prec in a.precisions.split(","):
        stats, _, _ = serve(reqs, precision=prec, prewarm=default_prewarm())
        out[prec] = stats
    if a.unbatched_requests:
        # the same arrivals served by the unbatched plain path (one solve at a time, new solver per
        # request, FP64) against continuous batching
        sub = reqs[: a.unbatched_requests]
        plain, _, _ = serve(sub, precision="fp64", max_inflight=1, pool=False)
        batched, _, _ = serve(sub, precision="fp64", prewarm=default_prewarm())
        keys = ("wall_s", "solves_per_s", "p50_latency_s", "p99_latency_s", "mean_latency_s", "sizes")
        out["unbatched_vs_batched_fp64"] = {"requests": len(sub), "unbatched": {k: plain[k] for k in keys},
                                            "batched": {k: batched[k] for k in keys}}
    print(json.dumps(out), flush=True)


def run_blocked(a):
    """FP64 sigma of a point-group-blocked space: CAS(n e, n o) with the orbitals spread over the
    eight irreps of D2h (n/8 per irrep), totally symmetric state, point-group-symmetric seeded
    integrals. Timed with CUDA events through the blocked path (vectors of the space in HBM): the
    irrep-aware opposite-spin kernel, and the C1 kernels on the embedding for comparison."""
    import torch

    from forte2_gb300.ci_helpers import CISigmaBuilder, CIStrings
    from forte2_gb300.synthetic import symmetrize_integrals

    torch.cuda.set_device(0)
    n = a.norb
    na, nb = n // 2, n // 2
    orbsym = [[p % 8 for p in range(n)]]
    ints = symmetrize_integrals(make_integrals(n, ISEED if n == NORB else 1000 + n), orbsym[0])
    strings = CIStrings(na, nb, 0, orbsym, [], [])
    sb = CISigmaBuilder(strings, ints.E, ints.H, ints.V, 0)
    sb.set_algorithm("hz")
    c = torch.from_numpy(random_ci_vector(strings.ndet, CSEED)).cuda()
    out = torch.empty_like(c)
    st = torch.cuda.current_stream()

    def timed(k):
        for _ in range(a.warmup):
            sb.Hamiltonian(c, out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(k):
            sb.Hamiltonian(c, out)
        e1.record(st)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    clocks = Clocks()
    clocks.start()
    ms_sym = timed(a.steps)
    s_sym = out.clone()
    sb.set_variant("irrep_blocks", 0)
    ms_c1 = timed(max(1, a.steps // 2))
    sb.set_variant("irrep_blocks", 1)
    clk = clocks.stop()
    rel = (torch.linalg.norm(s_sym - out) / torch.linalg.norm(out)).item()
    res = {"metric": f"CAS({n},{n}) D2h-blocked FP64 sigma-builds/s", "value": 1e3 / ms_sym, "unit": "sigma-builds/s",
           "n_gpus": 1, "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms_sym, "higher_is_better": True,
           "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"CAS({n}e,{n}o), orbitals over the 8 irreps of D2h, A1 state, "
                                  f"{strings.ndet} determinants of the space (C1 space {strings.nfull}), "
                                  "symmetric seeded integrals"},
           "c1_embedding_ms": ms_c1, "speedup_over_c1_embedding": ms_c1 / ms_sym,
           "rel_diff_vs_c1_embedding": rel, "clocks": clk}
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    args = parse()
    if args.mode in ("batched", "serve"):
        # many streams in flight: let them use more hardware queues (read when CUDA starts)
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    if args.mode == "batched":
        run_batched(args)
    elif args.mode == "serve":
        run_serve(args)
    elif args.mode == "davidson":
        run_davidson(args)
    elif args.mode == "rdm":
        run_rdm(args)
    elif args.mode == "blocked":
        run_blocked(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)
