"""Train the learned T2 initialiser on the GPU and evaluate it.

Training data: converged T2 of the plain FP64 GPU DF-CCSD (residual and
energy change below 1e-8) on seeded water clusters (fermicc.inputs.molecule:
(H2O)4 on a 2x2x1 lattice, seeds 0..n4-1, and (H2O)6 on 2x3x1, seeds
0..n6-1).  The samples are every `stride`-th of the elements the guess
corrects (|t_MP2| >= 3e-4), each 16 features -> the target correction to the
MP2 amplitude.  The network is trained with Adam (lr 1e-3, batch 65536) by
the library's own forward, backward and Adam kernels (BF16 tensor-core
products, FP32 masters) and saved as raw FP32 parameters.

Evaluation: held-out seeds (1000 + k) of (H2O)4, (H2O)6 and (H2O)8; from the MP2
guess and from the learned guess, in the mixed form and in the plain FP64
form, to a 1e-8 residual with the energy converged to 1e-10; reports the
iterations, the converged energies and the guess errors.

The host inputs (integrals, DF-RHF, the three-index factors) of every
geometry are made by a pool of worker processes started with "spawn" (they
inherit no CUDA state), two BLAS threads each, while the GPU solves the
previous ones.

    python -m fermicc.train_guess --n4 512 --n6 128 --steps 3000 --out params.f32
    python -m fermicc.train_guess --eval-only --eval6 48 --eval8 16 --fp64-eval6 48 --fp64-eval8 4 --out eval
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import time

import numpy as np

GUESS_THRESH = 3e-4   # the guess corrects |t_MP2| >= this (fcc_mlp_guess)
_THREAD_VARS = ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS")


def _make_inputs(case):
    from .inputs import scf
    waters, seed = case
    t0 = time.time()
    inp = scf.water_inputs(waters, seed=seed)
    return waters, seed, inp, time.time() - t0


def input_stream(cases, workers):
    """(waters, seed, inputs, host seconds) in the order of `cases`, made by
    spawned workers with two BLAS threads each."""
    saved = {k: os.environ.get(k) for k in _THREAD_VARS}
    for k in _THREAD_VARS:
        os.environ[k] = "2"
    try:
        pool = mp.get_context("spawn").Pool(max(1, workers))
    finally:
        for k, val in saved.items():
            if val is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = val
    try:
        yield from pool.imap(_make_inputs, cases)
    finally:
        pool.terminate()
        pool.join()


def solve(inp, guess_model=None, precision="fp64", max_rms=1e-8, e_conv=1e-8, lam=None, thresh=None):
    from . import Options, RCCSD
    from .rccsd import Context
    Options.reset()
    Options.set("cc_gpu_precision", precision)
    Options.set("cc_max_rms", max_rms)
    Options.set("cc_e_conv", e_conv)
    Options.set("cc_max_iter", 100)
    ctx = Context(inp)
    if guess_model is not None:
        guess_model.guess(ctx, lam, thresh)
        T1g, T2g = ctx.amplitudes()
        r = RCCSD.compute(inp, T1g, T2g, context=ctx)
    else:
        r = RCCSD.compute(inp, context=ctx)
    return r, ctx


def build_training_set(model, cases, strides, workers=8, log=print, every=32):
    """Converged FP64 amplitudes of every (waters, seed) case -> samples."""
    t0 = time.time()
    done, host_s, gpu_s = {}, 0.0, 0.0
    for q, (waters, sd, inp, th) in enumerate(input_stream(cases, workers)):
        t1 = time.time()
        r, ctx = solve(inp)
        if r.converged:
            model.collect(ctx, strides[waters], GUESS_THRESH)
            done[waters] = done.get(waters, 0) + 1
        else:
            log(f"(H2O){waters} seed {sd} did not converge; skipped")
        ctx.close()
        host_s += th
        gpu_s += time.time() - t1
        if (q + 1) % every == 0 or q + 1 == len(cases):
            log(json.dumps({"geometries": q + 1, "collected": done, "samples": model.num_samples(),
                            "wall_s": time.time() - t0, "solve_s": gpu_s, "host_inputs_s": host_s}), flush=True)


def evaluate(model, cases, precision, workers=8, log=print, lam=None, thresh=None):
    """Per held-out geometry: iterations from the MP2 and from the learned
    guess (same criteria), the converged energies and the T2 guess errors
    (lam, thresh: a scaled correction applied where |t_MP2| >= thresh)."""
    out = []
    for waters, sd, inp, _ in input_stream(cases, workers):
        ref, ctx = solve(inp, precision=precision, e_conv=1e-10)
        T2c = ref.T2
        ctx.lib.fcc_set_guess(ctx.h, None, None)
        _, T2mp2 = ctx.amplitudes()
        model.guess(ctx, lam, thresh)
        _, T2mlp = ctx.amplitudes()
        err_mp2 = float(np.sqrt(np.mean((T2mp2 - T2c) ** 2)))
        err_mlp = float(np.sqrt(np.mean((T2mlp - T2c) ** 2)))
        ctx.close()
        lrn, ctx2 = solve(inp, guess_model=model, precision=precision, e_conv=1e-10, lam=lam, thresh=thresh)
        ctx2.close()
        row = dict(precision=precision, waters=waters, seed=sd, iters_mp2=len(ref.iterations),
                   iters_mlp=len(lrn.iterations), time_mp2=sum(l["seconds"] for l in ref.iterations),
                   time_mlp=sum(l["seconds"] for l in lrn.iterations), e_mp2=ref.energy, e_mlp=lrn.energy,
                   de=abs(ref.energy - lrn.energy), converged=bool(ref.converged and lrn.converged),
                   guess_rms_err_mp2=err_mp2, guess_rms_err_mlp=err_mlp)
        log(json.dumps(row), flush=True)
        out.append(row)
    return out


def summarise(rows):
    s = {}
    for w in sorted({r["waters"] for r in rows}):
        rr = [r for r in rows if r["waters"] == w]
        s[f"h2o{w}"] = {k: float(np.mean([r[k] for r in rr]))
                        for k in ("iters_mp2", "iters_mlp", "time_mp2", "time_mlp", "guess_rms_err_mp2",
                                  "guess_rms_err_mlp")}
        s[f"h2o{w}"]["max_de"] = float(max(r["de"] for r in rr))
        s[f"h2o{w}"]["cases"] = len(rr)
        s[f"h2o{w}"]["fewer_iterations"] = int(sum(r["iters_mlp"] < r["iters_mp2"] for r in rr))
        s[f"h2o{w}"]["more_iterations"] = int(sum(r["iters_mlp"] > r["iters_mp2"] for r in rr))
    return s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n4", type=int, default=512)
    ap.add_argument("--n6", type=int, default=128)
    ap.add_argument("--stride4", type=int, default=4)
    ap.add_argument("--stride6", type=int, default=16)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--out", default="mlp_t2_guess.f32")
    ap.add_argument("--eval4", type=int, default=0, help="held-out (H2O)4 seeds, mixed form")
    ap.add_argument("--fp64-eval4", type=int, default=0, help="held-out (H2O)4 seeds, FP64 form")
    ap.add_argument("--eval6", type=int, default=4, help="held-out (H2O)6 seeds, mixed form")
    ap.add_argument("--eval8", type=int, default=2, help="held-out (H2O)8 seeds, mixed form")
    ap.add_argument("--fp64-eval6", type=int, default=0, help="held-out (H2O)6 seeds, FP64 form")
    ap.add_argument("--fp64-eval8", type=int, default=0, help="held-out (H2O)8 seeds, FP64 form")
    ap.add_argument("--eval-only", action="store_true",
                    help="evaluate the packaged network (fermicc/data) or --params instead of training one")
    ap.add_argument("--params", default=None)
    ap.add_argument("--lam", type=float, default=None, help="scale of the learned correction (default 1)")
    ap.add_argument("--thresh", type=float, default=None, help="apply it where |t_MP2| >= this (default 3e-4)")
    a = ap.parse_args()
    from .mlp import DEFAULT_PARAMS, MLPGuess
    if a.eval_only:
        model = MLPGuess(0, a.params or DEFAULT_PARAMS)
    else:
        model = MLPGuess(0)
        cases = [(4, sd) for sd in range(a.n4)] + [(6, sd) for sd in range(a.n6)]
        build_training_set(model, cases, {4: a.stride4, 6: a.stride6}, a.workers)
        t = time.time()
        loss = model.train(a.steps, a.batch, a.lr, seed=1)
        print(json.dumps({"trained_steps": a.steps, "seconds": time.time() - t, "loss_first": float(loss[0]),
                          "loss_last50": float(np.mean(loss[-50:]))}), flush=True)
        model.save(a.out)
        np.savetxt(a.out + ".loss.txt", loss)
    report = {}
    for prec, n4, n6, n8 in (("mixed", a.eval4, a.eval6, a.eval8), ("fp64", a.fp64_eval4, a.fp64_eval6, a.fp64_eval8)):
        cases = ([(4, 1000 + k) for k in range(n4)] + [(6, 1000 + k) for k in range(n6)] +
                 [(8, 1000 + k) for k in range(n8)])
        if not cases:
            continue
        rows = evaluate(model, cases, prec, a.workers, lam=a.lam, thresh=a.thresh)
        report[prec] = {"summary": summarise(rows), "rows": rows}
        print(json.dumps({prec: report[prec]["summary"]}), flush=True)
    if report:
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        with open(a.out + ".eval.json", "w") as f:
            json.dump(report, f, indent=1)


if __name__ == "__main__":
    main()
