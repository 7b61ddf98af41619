#!/usr/bin/env python
"""DF-CCSD(T) time-to-solution on a seeded (H2O)8 cluster, one GB300.

Workload: (H2O)8 on a 2x2x2 lattice (seed 0), stand-in cc-pVDZ / cc-pVDZ-RI
shell structure: 192 basis functions, 32 active occupied (8 frozen core), 152
virtual, 672 fitting functions.  One "step" is one full solve: CCSD from the
learned guess (MP2 guess with ``--guess mp2`` or ``--form fp64``) to
convergence (residual rms < 1e-8 and |dE| < 1e-8 Eh) followed by (T).  The
form measured is the mixed one (split-BF16, then exact-slice tensor-core
contractions, an FP64-accurate finish, FP64 update and energies, split-BF16
(T)); ``--form fp64`` measures the plain FP64 form.

JSON line (rank 0): ``value`` = device time-to-solution in seconds with the
integrals resident in HBM (CUDA events on the library's stream, mean over
``--steps``); ``fp64_form`` / ``fp64_time_to_solution_s`` / ``ratio_vs_fp64``
= the plain FP64 form on the same context, timed once (the metric's
comparator), with ``dE_ccsd``, ``dE_t``, ``dE_total``, ``max_dT1`` and
``max_dT2`` of the measured form against it (|dE_total| <= 1e-6 Eh is
required; a violation exits non-zero after the line); ``e2e`` = the same
solve through the C ABI from pinned host buffers (context creation,
host->device upload of the three-index factors, learned guess, solve, (T),
device->host read of T1/T2), host wall clock, mean over ``--steps``;
``roofline`` for the dominant kernel class; ``cpu_baseline`` = the CPU
restatement of Fermi's algorithm (the oracle) timed on a bounded sample of
the same workload on this host and scaled to a full solve with the FP64
form's measured iteration count; ``iterations_mlp`` / ``iterations_mp2`` and
the T2 guess errors compare the learned guess with the MP2 guess.

``--impl reference`` times that CPU restatement alone (Fermi.jl itself cannot
run here: no Julia, no libcint, no basis files) and prints its line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fermi.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "DF-CCSD(T) time-to-solution (H2O)8/cc-pVDZ: mixed+learned vs FP64 GPU @1µEh"
E_CONV = 1e-8
MAX_RMS = 1e-8
DE_BUDGET = 1e-6            # |dE_total| of the mixed form against the FP64 form
# Iterations of the plain FP64 form on (H2O)8 seed 0 at these criteria from the
# MP2 guess, measured on the GPU (the CPU restatement follows the same
# iteration sequence).  The default run measures the count again in its FP64
# arm and scales the one-iteration CPU sample by that; the reference arm,
# which has no GPU, uses this value.
FP64_ITERATIONS = 17
FP64_PEAK_TFLOPS = 1.05     # measured DMMA / DFMA peak of this GB300 pool (own probe)
# MEASURED_PEAKS.json values of this pool, used when the file is not present
PEAKS_FALLBACK = {"hbm_gbs": 6778.3, "bf16_tflops": 1908.9, "bf16_tflops_sustained": 1714.6}
# DRAM traffic per algorithmic flop of the DMMA kernel, from one ncu capture of
# its largest launch (the o^3 v^3 ring contraction at (H2O)8, M = N = K = 4864:
# dram__bytes_read + dram__bytes_write = 7.114e9 + 0.186e9 B for 2 * 4864^3 flop)
DMMA_DRAM_BYTES_PER_FLOP = (7.114e9 + 0.186e9) / (2.0 * 4864.0 ** 3)
# the same for the exact-slice kernel per executed BF16 flop, from one ncu
# capture (dram__bytes_read.sum + dram__bytes_write.sum, one pass) of all 541
# gemm_oz_kernel launches of one (H2O)8 mixed solve: 359.8e9 + 78.6e9 B for
# 541 launches of 8.989e11 executed flop on average
OZ_DRAM_BYTES_PER_FLOP = (359.8e9 + 78.6e9) / (541 * 8.989e11)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--guess", default="auto", choices=["auto", "mp2", "mlp"],
                    help="auto: the learned guess for the mixed form when its trained parameters exist")
    ap.add_argument("--waters", type=int, default=8)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the plain FP64 form (the metric's comparator and the error budget)")
    ap.add_argument("--switch-rms", type=float, default=None,
                    help="mixed form: rms at which it leaves the split-BF16 phase (default: the library's)")
    ap.add_argument("--part", default="cc", choices=["cc", "rhf-fock"],
                    help="rhf-fock: time the DF-RHF Fock build and the RHF iterations instead (own JSON line)")
    ap.add_argument("--profile-case", default=None,
                    choices=["ccsd-fp64-iter", "ccsd-mixed-iter", "ccsd-exact-iter", "triples-mixed",
                             "triples-fp64", "solve-mixed"],
                    help="run one piece of the workload once (for ncu captures) and print its timing, no JSON line")
    return ap.parse_args()


def profile_case(args, inp):
    """One piece of the workload, for kernel profiling: one FP64, one
    split-BF16 or one exact-slice CCSD iteration from the MP2 guess; the mixed
    (T) on the amplitudes after two mixed iterations; the whole FP64 (T) on the
    amplitudes after one FP64 iteration; or one whole mixed solve from the
    learned guess, (T) included."""
    from fermicc import Options, RCCSD, RCCSDpT
    from fermicc.rccsd import Context
    Options.reset()
    ctx = Context(inp)
    t0 = time.perf_counter()
    if args.profile_case == "solve-mixed":
        from fermicc.mlp import DEFAULT_PARAMS, MLPGuess
        Options.set("cc_gpu_precision", "mixed")
        Options.set("pt_gpu_precision", "mixed")
        Options.set("cc_e_conv", E_CONV)
        Options.set("cc_max_rms", MAX_RMS)
        MLPGuess(0, DEFAULT_PARAMS).guess(ctx)
        r = RCCSD.compute(inp, context=ctx)
        pt = RCCSDpT.compute(r, inp)
        print(json.dumps({"case": args.profile_case, "wall_s": time.perf_counter() - t0, "e_total": pt.energy,
                          "kinds": [l["precision"] for l in r.iterations],
                          "rms": [l["rms"] for l in r.iterations], "dE": [l["dE"] for l in r.iterations],
                          "seconds": [l["seconds"] for l in r.iterations]}))
    elif args.profile_case == "triples-fp64":
        Options.set("cc_max_iter", 1)
        r = RCCSD.compute(inp, context=ctx)
        t0 = time.perf_counter()
        pt = RCCSDpT.compute(r, inp)
        print(json.dumps({"case": args.profile_case, "triples_s": time.perf_counter() - t0, "e_t": pt.correction}))
    elif args.profile_case.startswith("ccsd"):
        Options.set("cc_gpu_precision", "fp64" if "fp64" in args.profile_case else "mixed")
        Options.set("cc_max_iter", 1)
        if "exact" in args.profile_case:
            # one split-BF16 iteration, then (switch threshold above any rms)
            # one exact-slice iteration
            Options.set("cc_gpu_switch_rms", 10.0)
            Options.set("cc_max_iter", 2)
        r = RCCSD.compute(inp, context=ctx)
        print(json.dumps({"case": args.profile_case, "iteration_s": r.iterations[-1]["seconds"],
                          "kinds": [l["precision"] for l in r.iterations]}))
    else:
        Options.set("cc_gpu_precision", "mixed")
        Options.set("cc_max_iter", 2)
        r = RCCSD.compute(inp, context=ctx)
        Options.set("pt_gpu_precision", "mixed")
        t0 = time.perf_counter()
        pt = RCCSDpT.compute(r, inp)
        print(json.dumps({"case": args.profile_case, "triples_s": time.perf_counter() - t0, "e_t": pt.correction}))
    ctx.close()


def rhf_fock_part(args):
    """DF-RHF on the same cluster: the Fock build (build_fock!, RHFHelper.jl:88-93)
    through the C ABI from host matrices, in the density form and the
    occupied-orbital form, against the restated build on the host cores; then
    the whole RHF (RHFa.jl:67-203 iterations) with the device build against
    the restated iterations on the host."""
    import numpy as np
    from fermicc import DFFock, Options, RHF, _lib
    from fermicc.inputs import molecule, scf
    from fermicc.rhf import _guess
    from oracle import rhf as orhf          # the host-cores leg and the check only
    p = scf.df_ao_problem(molecule.waters(args.waters, args.seed))
    naux, nbf, _ = p.b.shape
    lib = _lib.load()
    Options.reset()
    f = DFFock(nbf, naux, b=p.b)
    C, Lam = _guess(p.S, p.H, "gwh")
    Co = C[:, :p.ndocc]
    D = Co @ Co.T
    prof = (ctypes.c_double * 24)()

    def timed(fn, k):
        for _ in range(args.warmup):
            fn()
        lib.fcc_prof_read(prof, 6)
        lib.fcc_prof_enable(1)
        t0 = time.perf_counter()
        for _ in range(k):
            fn()
        t = (time.perf_counter() - t0) / k
        lib.fcc_prof_enable(0)
        lib.fcc_prof_read(prof, 6)
        return t, prof[1] / k, prof[2] / k          # wall s, DMMA ms, DMMA flop per build

    k = max(args.steps, 5)
    l0 = lib.fcc_stat_launches()
    t_d, ms_d, fl_d = timed(lambda: f.build(p.H, D), k)
    launches_d = (lib.fcc_stat_launches() - l0) // (k + args.warmup)
    t_o, ms_o, fl_o = timed(lambda: f.build_occ(p.H, Co), k)
    F_dev, _ = f.build(p.H, D)
    t0 = time.perf_counter()
    F_ref = orhf.build_fock_df(p.H, D, p.b)
    t_cpu = time.perf_counter() - t0
    err = float(np.abs(F_dev - F_ref).max())
    t0 = time.perf_counter()
    r = RHF.compute(p.H, p.S, p.ndocc, p.e_nuc, f)
    t_rhf = time.perf_counter() - t0
    t0 = time.perf_counter()
    o = orhf.rhf(p.H, p.S, p.ndocc, p.e_nuc, lambda H, D_: orhf.build_fock_df(H, D_, p.b), C, Lam)
    t_rhf_cpu = time.perf_counter() - t0
    f.close()
    ach = fl_d / (ms_d * 1e9) if ms_d else None
    out = {"metric": f"DF-RHF Fock build time (H2O){args.waters}", "value": t_d * 1e3, "unit": "ms",
           "higher_is_better": False, "n_gpus": 1, "steps": k, "warmup": args.warmup, "dtype": "f64",
           "data": "synthetic (seeded water cluster, stand-in basis)",
           "config": {"workload": f"(H2O){args.waters} seed {args.seed} DF-RHF", "nbf": nbf, "naux": naux,
                      "ndocc": p.ndocc, "l2": "b resident, 8 naux nbf^2 bytes"},
           "e2e_note": "value and occ_form_ms are host wall time per call through the C ABI (H, D / Co in, "
                       "F and the energy out)",
           "occ_form_ms": t_o * 1e3, "max_abs_dF_vs_oracle": err, "gpu_launches": launches_d,
           "roofline": {"bound": "tensor", "kernel": "contract_f64_kernel (DMMA FP64), density form",
                        "achieved": ach, "peak": FP64_PEAK_TFLOPS, "unit": "TFLOP/s",
                        "frac": ach / FP64_PEAK_TFLOPS if ach else None,
                        "dmma_ms_per_build": ms_d, "dmma_flop_per_build": fl_d,
                        "occ_form_dmma_ms": ms_o, "occ_form_dmma_flop": fl_o},
           "cpu_baseline": {"value": t_cpu * 1e3, "unit": "ms", "kind": "port", "cores": os.cpu_count(),
                            "sample": "one restated build_fock! (numpy einsum, all host threads)"},
           "rhf": {"device_fock_s": t_rhf, "iterations": r.iterations, "energy": r.energy,
                   "host_oracle_s": t_rhf_cpu, "host_iterations": o.iterations,
                   "dE_vs_host": r.energy - o.energy}}
    print(json.dumps(out), flush=True)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    """MEASURED_PEAKS.json of this pool (HBM copy GB/s, cuBLAS BF16 TFLOP/s)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return {k: float(d[k]) for k in PEAKS_FALLBACK}, "MEASURED_PEAKS.json"
    except (OSError, KeyError, ValueError):
        return dict(PEAKS_FALLBACK), "MEASURED_PEAKS.json values of this pool (file absent at run time)"


def algorithmic_flops(o, v, Q):
    """Leading-order flops of one CCSD iteration and of (T)."""
    f_it = 2 * o**2 * v**4 + 2 * Q * v**4 + 12 * o**3 * v**3
    f_t = 2 * o * (o + 1) * (o + 2) * v**3 * (v + o)
    return f_it, f_t


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    def __init__(self, device=0):
        # nvidia-smi -i takes physical indices, which CUDA_VISIBLE_DEVICES
        # remaps; the UUID names the device this process uses
        self.samples, self.proc = [], None
        try:
            import torch
            self.index = "GPU-" + str(torch.cuda.get_device_properties(device).uuid)
        except Exception:
            self.index = str(device)

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        num = lambda x: x.replace(".", "", 1).isdigit()
        sm = sorted(float(s[1]) for s in self.samples if len(s) > 2 and num(s[1]))
        mx = max((float(s[2]) for s in self.samples if len(s) > 2 and num(s[2])), default=None)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 5 + k and s[5 + k] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def cpu_sample(inp, ntrip=8, iterations=FP64_ITERATIONS):
    """The CPU restatement of Fermi's algorithm on a bounded sample of the
    workload: one full CCSD iteration (RCCSDHelper.jl update_amp at the MP2
    guess), scaled by `iterations` (the FP64 form's count), and `ntrip` (T)
    triplets spread over the i >= j >= k list, scaled to all triplets."""
    import numpy as np
    from oracle import rccsd as R
    from oracle import triples as T
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    t0 = time.perf_counter()
    R.update_amp(T1, T2, I, D1, D2, lambda a, b: R.ladder_df(a, b, inp.Bvv))
    t_it = time.perf_counter() - t0
    trip = T.triplet_list(inp.o)
    pick = trip[:: max(1, len(trip) // ntrip)][:ntrip]
    t0 = time.perf_counter()
    T.triples_ijk(T1, T2, I["OVVV"], I["OOOV"], I["OVOV"], inp.eps_o, inp.eps_v, triplets=pick)
    t_t = (time.perf_counter() - t0) / len(pick) * len(trip)
    value = iterations * t_it + t_t
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"value": value, "unit": "s", "cores": cores, "kind": "port",
            "sample": (f"1 CCSD iteration ({t_it:.1f} s, scaled x{iterations}, the FP64 form's iteration count) + "
                       f"{len(pick)} of {len(trip)} (T) triplets ({t_t:.1f} s scaled); numpy/BLAS restatement of "
                       f"RCCSDHelper.jl + ijk.jl")}


def run_reference(args, inp):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    vals = []
    for it in range(args.warmup + args.steps):
        cb = cpu_sample(inp)
        if it >= args.warmup:
            vals.append(cb["value"])
    value = sum(vals) / len(vals)
    cb["value"] = value
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": value * 1e3, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded water cluster)",
           "config": {"workload": f"(H2O){args.waters} seed {args.seed} DF-RCCSD(T)", "o": inp.o, "v": inp.v,
                      "naux": inp.naux, "e_conv": E_CONV, "max_rms": MAX_RMS},
           "cpu_baseline": cb, "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.part == "rhf-fock":
        if rank == 0 and args.impl == "ours":
            rhf_fock_part(args)
        return
    from fermicc.inputs import scf
    inp = scf.water_inputs(args.waters, seed=args.seed)
    if args.impl == "reference":
        run_reference(args, inp)
        return
    if args.profile_case:
        profile_case(args, inp)
        return
    import numpy as np
    import torch
    from fermicc import Options, RCCSD, RCCSDpT, _lib
    from fermicc.rccsd import Context

    if world > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    lib = _lib.load()
    peaks, peaks_src = measured_peaks()

    def set_form(form):
        Options.reset()
        Options.set("cc_gpu_device", local)
        Options.set("cc_gpu_precision", form)
        Options.set("pt_gpu_precision", form)
        Options.set("cc_e_conv", E_CONV)
        Options.set("cc_max_rms", MAX_RMS)
        Options.set("cc_max_iter", 100)
        if args.switch_rms is not None:
            Options.set("cc_gpu_switch_rms", args.switch_rms)

    set_form(args.form)
    from fermicc.mlp import DEFAULT_PARAMS, MLPGuess
    guess = args.guess
    if guess == "auto":
        guess = "mlp" if (args.form == "mixed" and os.path.exists(DEFAULT_PARAMS)) else "mp2"
    model = MLPGuess(local, DEFAULT_PARAMS) if guess == "mlp" else None

    ctx = Context(inp, device=local)
    stream = torch.cuda.ExternalStream(lib.fcc_stream(ctx.h))

    def solve(use_model=True):
        if model is not None and use_model:
            model.guess(ctx)          # T1 = 0, T2 = MP2 + learned correction, on the device
        else:
            ctx.lib.fcc_set_guess(ctx.h, None, None)
        ccsd = RCCSD.compute(inp, context=ctx)
        pt = RCCSDpT.compute(ccsd, inp)
        return ccsd, pt

    for _ in range(args.warmup):
        solve()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = lib.fcc_stat_launches()
    times, results = [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ccsd, pt = solve()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            results.append((ccsd, pt))
    torch.cuda.synchronize()
    launches = (lib.fcc_stat_launches() - launches0) // max(1, args.steps)
    t_step = sum(times) / len(times)
    from fermicc.replicas import max_over_ranks
    t_step = max_over_ranks(t_step, world, device="cuda")
    ccsd, pt = results[-1]
    T1m, T2m = ccsd.T1, ccsd.T2

    # one more (untimed) step with per-launch CUDA events on the library's
    # stream, for the per-kernel-class breakdown and the roofline
    prof = (ctypes.c_double * 24)()
    lib.fcc_prof_read(prof, 6)       # clear
    lib.fcc_prof_enable(1)
    solve()
    torch.cuda.synchronize()
    lib.fcc_prof_enable(0)
    lib.fcc_prof_read(prof, 6)

    # the learned guess against the MP2 guess in the same form: iterations and
    # the guess's distance from the converged amplitudes (untimed)
    guess_info = None
    if model is not None and rank == 0:
        it_mlp = len(ccsd.iterations)
        model.guess(ctx)
        T1g, T2g = ctx.amplitudes()
        ctx.lib.fcc_set_guess(ctx.h, None, None)
        T1p, T2p = ctx.amplitudes()
        c_mp2, _ = solve(use_model=False)
        guess_info = {"iterations_mlp": it_mlp, "iterations_mp2": len(c_mp2.iterations),
                      "t2_rms_error_mlp": float(np.sqrt(np.mean((T2g - T2m) ** 2))),
                      "t2_rms_error_mp2": float(np.sqrt(np.mean((T2p - T2m) ** 2)))}

    # the comparator of the metric: the plain FP64 form on the same context,
    # from the MP2 guess, CUDA events on the same stream; its energies and
    # amplitudes give the mixed form's error budget
    fp64 = None
    if not args.no_fp64 and rank == 0 and args.form != "fp64":
        set_form("fp64")
        e0 = torch.cuda.Event(enable_timing=True)
        em = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        ctx.lib.fcc_set_guess(ctx.h, None, None)
        e0.record(stream)
        c64 = RCCSD.compute(inp, context=ctx)
        em.record(stream)
        p64 = RCCSDpT.compute(c64, inp)
        e1.record(stream)
        e1.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3
        fp64 = {"time_to_solution_s": t64, "ccsd_s": e0.elapsed_time(em) / 1e3, "triples_s": em.elapsed_time(e1) / 1e3,
                "iterations": len(c64.iterations), "e_ccsd": c64.energy, "e_t": p64.correction, "e_total": p64.energy,
                "converged": c64.converged}
        set_form(args.form)
    it_kinds = [l["precision"] for l in ccsd.iterations]
    f_it, f_t = algorithmic_flops(inp.o, inp.v, inp.naux)
    # per-class kernel timing over the profiled step (CUDA events on the
    # library's stream): launches, ms, algorithmic work, longest launch
    cls = {0: "contract_f64_kernel (DMMA FP64)", 1: "gemm_bf16_tc_kernel + gemm_t3_kernel (tcgen05 split-BF16)",
           2: "pack kernels (split + gather)", 5: "gemm_oz_kernel (tcgen05 exact-slice BF16)"}
    bf = peaks["bf16_tflops_sustained"]
    pk = {0: (FP64_PEAK_TFLOPS, "TFLOP/s"), 1: (bf, "TFLOP/s"), 2: (peaks["hbm_gbs"], "GB/s"), 5: (bf, "TFLOP/s")}
    kern = {}
    for c, name in cls.items():
        n, ms, work = prof[4 * c], prof[4 * c + 1], prof[4 * c + 2]
        if n == 0 or ms == 0:
            continue
        scale = 1e9 if c != 2 else 1e6          # flop/ms -> TFLOP/s ; bytes/ms -> GB/s
        ach = work / ms / scale
        kern[name] = {"launches": int(n), "ms": ms, "achieved": ach, "unit": pk[c][1],
                      "frac": ach / pk[c][0], "ms_per_launch": ms / n}
    if prof[16] > 0:   # (T) energy kernels: launches, ms, (a >= b >= c) evaluated
        kern["triples energy kernels (sub-cube permutation sums)"] = {
            "launches": int(prof[16]), "ms": prof[17], "ms_per_launch": prof[17] / prof[16],
            "abc_per_s": prof[18] / prof[17] * 1e3 if prof[17] else None}
    dom = max(((c, prof[4 * c + 1]) for c in cls), key=lambda x: x[1])[0]
    n, ms, work = prof[4 * dom], prof[4 * dom + 1], prof[4 * dom + 2]
    ach = work / ms / (1e9 if dom != 2 else 1e6) if ms else None
    traffic = None
    if dom == 0 and n:
        traffic = DMMA_DRAM_BYTES_PER_FLOP * work / n
    elif dom == 5 and n:
        traffic = OZ_DRAM_BYTES_PER_FLOP * work / n
    roof = {"bound": "hbm" if dom == 2 else "tensor", "kernel": cls[dom], "achieved": ach,
            "peak": pk[dom][0], "unit": pk[dom][1], "frac": (ach / pk[dom][0]) if ach else None,
            "traffic": traffic,
            "traffic_note": ("bytes per average launch: ncu-measured DRAM bytes per executed flop (all launches of "
                             "one solve for the exact-slice kernel, the largest launch for the DMMA kernel) times "
                             "the average launch's flops" if traffic is not None else None),
            "launches": int(n), "work_per_launch": (work / n) if n else None,
            "peak_source": ("own measurement (DMMA probe; MEASURED_PEAKS.json has no FP64 figure)" if dom == 0
                            else peaks_src + (" (sustained BF16)" if dom != 2 else " (HBM copy)")),
            "note": ("achieved = sum of executed BF16 flops (tensor kernels; 2*M*N*K per product for FP64) over "
                     "the launches / sum of launch times, CUDA events on the library's stream")}

    e2e = None
    if not args.no_e2e and rank == 0:
        hB = [np.asfortranarray(x) for x in (inp.Boo, inp.Bov, inp.Bvv)]
        pinned = []
        for x in hB:
            t = torch.empty(x.size, dtype=torch.float64, pin_memory=True).numpy()
            t[:] = x.ravel(order="F")
            pinned.append(t)
        h2d = sum(x.nbytes for x in pinned) + 8 * (inp.o + inp.v)
        d2h = 8 * (inp.o * inp.v + inp.o**2 * inp.v**2)
        T1 = torch.empty(inp.o * inp.v, dtype=torch.float64, pin_memory=True).numpy()
        T2 = torch.empty(inp.o**2 * inp.v**2, dtype=torch.float64, pin_memory=True).numpy()
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        eo = np.ascontiguousarray(inp.eps_o)
        ev = np.ascontiguousarray(inp.eps_v)
        pp = np.fromfile(DEFAULT_PARAMS, dtype=np.float32) if model is not None else None
        walls, energy = [], None
        for _ in range(args.steps):
            # create + host->device upload + learned guess + solve + (T) + T1/T2 download, all through the C ABI
            t0 = time.perf_counter()
            h = ctypes.c_void_p()
            assert lib.fcc_create(ctypes.byref(h), inp.o, inp.v, inp.naux, local) == 0
            assert lib.fcc_upload_df(h, dp(pinned[0]), dp(pinned[1]), dp(pinned[2]), dp(eo), dp(ev), inp.e_ref) == 0
            opts = _lib.FccOpts()
            lib.fcc_default_opts(ctypes.byref(opts))
            opts.precision = 1 if args.form == "mixed" else 0
            opts.e_conv, opts.max_rms, opts.max_iter = E_CONV, MAX_RMS, 100
            if pp is not None:
                mh = ctypes.c_void_p()
                assert lib.fcc_mlp_create(ctypes.byref(mh), local) == 0
                assert lib.fcc_mlp_set_params(mh, pp.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), pp.size) == 0
                assert lib.fcc_mlp_guess(h, mh) == 0
                lib.fcc_mlp_destroy(mh)
            res = _lib.FccCCSDResult()
            rc = lib.fcc_ccsd_run(h, ctypes.byref(opts), None, 0, ctypes.byref(res))
            assert rc == 0, rc
            et = ctypes.c_double()
            assert lib.fcc_triples(h, opts.precision, ctypes.byref(et)) == 0
            assert lib.fcc_get_amps(h, dp(T1), dp(T2)) == 0
            lib.fcc_destroy(h)
            walls.append(time.perf_counter() - t0)
            energy = res.energy + et.value
        e2e = {"value": sum(walls) / len(walls), "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "steps": len(walls), "min": min(walls), "max": max(walls), "energy": energy}

    cpu = None
    if not args.no_cpu and rank == 0 and world == 1:
        cpu = cpu_sample(inp, iterations=fp64["iterations"] if fp64 else FP64_ITERATIONS)

    if rank == 0:
        out = {"metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False, "scaling": "weak",
               "vs_baseline": None, "dtype": "bf16x3+f64" if args.form == "mixed" else "f64",
               "data": "synthetic (seeded water cluster, stand-in basis)",
               "config": {"workload": f"(H2O){args.waters} seed {args.seed} DF-RCCSD(T)", "form": args.form,
                          "mixed_finish": Options.get("cc_gpu_finish") if args.form == "mixed" else None,
                          "switch_rms": Options.get("cc_gpu_switch_rms") if args.form == "mixed" else None,
                          "o": inp.o, "v": inp.v, "naux": inp.naux, "e_conv": E_CONV, "max_rms": MAX_RMS,
                          "parallelism": "replicas" if world > 1 else "single GPU",
                          "l2": "working set > L2 (T2 189 MB, factors 160 MB)"},
               "e_ccsd": ccsd.energy, "e_t": pt.correction, "e_total": pt.energy,
               "iterations": len(ccsd.iterations), "iteration_kinds": it_kinds, "guess": guess,
               "kernels": kern, "algorithmic_flops": {"ccsd_iteration": f_it, "triples": f_t},
               "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
               "clocks": clk.summary()}
        if guess_info:
            out.update(guess_info)
        if fp64:
            out["fp64_form"] = fp64
            out["fp64_time_to_solution_s"] = fp64["time_to_solution_s"]
            out["ratio_vs_fp64"] = fp64["time_to_solution_s"] / t_step
            out["dE_ccsd"] = ccsd.energy - fp64["e_ccsd"]
            out["dE_t"] = pt.correction - fp64["e_t"]
            out["dE_total"] = pt.energy - fp64["e_total"]
            T1f, T2f = ctx.amplitudes()
            out["max_dT1"] = float(np.abs(T1m - T1f).max())
            out["max_dT2"] = float(np.abs(T2m - T2f).max())
            out["error_budget_ok"] = bool(abs(out["dE_total"]) <= DE_BUDGET and fp64["converged"])
        print(json.dumps(out), flush=True)
        if fp64 and not out["error_budget_ok"]:
            print(f"error budget violated: |dE_total| = {abs(out['dE_total']):.3e} > {DE_BUDGET:.0e}",
                  file=sys.stderr, flush=True)
            sys.exit(1)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
