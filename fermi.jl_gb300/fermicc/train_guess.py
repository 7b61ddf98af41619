"""Train the learned T2 initialiser on the GPU and evaluate it.

Training data: converged T2 of the plain FP64 GPU DF-CCSD (residual 1e-8) on
seeded water clusters (fermicc.inputs.molecule: (H2O)4 on a 2x2x1 lattice and
(H2O)6 on 2x3x1).  Every `stride`-th amplitude of each solution becomes a
sample (16 features -> target correction to the MP2 amplitude).  The network
is trained with Adam (lr 1e-3, batch 65536) by the library's own forward,
backward and Adam kernels, and saved as raw FP32 parameters.

Evaluation: held-out seeds, FP64 CCSD from the MP2 guess and from the learned
guess; reports iterations to convergence, the converged energies and the
guess errors.

    python -m fermicc.train_guess --n4 128 --n6 16 --steps 3000 --out params.f32
    python -m fermicc.train_guess --eval-only --eval6 32 --eval8 4 --out eval
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import Options, RCCSD
from .inputs import scf
from .mlp import MLPGuess
from .rccsd import Context


def solve(inp, guess_model=None, precision="fp64", max_rms=1e-8, e_conv=1e-8):
    Options.reset()
    Options.set("cc_gpu_precision", precision)
    Options.set("cc_max_rms", max_rms)
    Options.set("cc_e_conv", e_conv)
    Options.set("cc_max_iter", 100)
    ctx = Context(inp)
    if guess_model is not None:
        guess_model.guess(ctx)
        T1g, T2g = ctx.amplitudes()
        r = RCCSD.compute(inp, T1g, T2g, context=ctx)
    else:
        r = RCCSD.compute(inp, context=ctx)
    return r, ctx


def build_training_set(model, n4, n6, seed0=0, stride4=8, stride6=32, log=print):
    t0 = time.time()
    for waters, count, stride in ((4, n4, stride4), (6, n6, stride6)):
        for sd in range(seed0, seed0 + count):
            inp = scf.water_inputs(waters, seed=sd)
            r, ctx = solve(inp)
            if not r.converged:
                log(f"(H2O){waters} seed {sd} did not converge; skipped")
                continue
            model.collect(ctx, stride)
            ctx.close()
        log(f"(H2O){waters}: {count} seeds collected ({time.time() - t0:.1f} s)")


def evaluate(model, cases, log=print, precision="fp64"):
    """Per held-out geometry: iterations from the MP2 and from the learned
    guess (same criteria), the converged energies and the T2 guess errors."""
    out = []
    for waters, sd in cases:
        inp = scf.water_inputs(waters, seed=sd)
        ref, ctx = solve(inp, precision=precision)
        T1c, T2c = ref.T1, ref.T2
        # guess quality: MP2 vs learned
        ctx.lib.fcc_set_guess(ctx.h, None, None)
        _, T2mp2 = ctx.amplitudes()
        model.guess(ctx)
        _, T2mlp = ctx.amplitudes()
        err_mp2 = float(np.sqrt(np.mean((T2mp2 - T2c) ** 2)))
        err_mlp = float(np.sqrt(np.mean((T2mlp - T2c) ** 2)))
        ctx.close()
        lrn, ctx2 = solve(inp, guess_model=model, precision=precision)
        ctx2.close()
        row = dict(waters=waters, seed=sd, iters_mp2=len(ref.iterations), iters_mlp=len(lrn.iterations),
                   e_mp2=ref.energy, e_mlp=lrn.energy, de=abs(ref.energy - lrn.energy),
                   guess_rms_err_mp2=err_mp2, guess_rms_err_mlp=err_mlp)
        log(json.dumps(row))
        out.append(row)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n4", type=int, default=128)
    ap.add_argument("--n6", type=int, default=16)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--out", default="mlp_t2_guess.f32")
    ap.add_argument("--eval6", type=int, default=4)
    ap.add_argument("--eval8", type=int, default=2)
    ap.add_argument("--eval-only", action="store_true",
                    help="evaluate the packaged network (fermicc/data) instead of training one")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    a = ap.parse_args()
    cases = [(6, 1000 + k) for k in range(a.eval6)] + [(8, 1000 + k) for k in range(a.eval8)]
    if a.eval_only:
        from .mlp import DEFAULT_PARAMS
        rows = evaluate(MLPGuess(0, DEFAULT_PARAMS), cases, precision=a.precision)
        summary = {k: float(np.mean([r[k] for r in rows])) for k in ("iters_mp2", "iters_mlp", "de",
                                                                      "guess_rms_err_mp2", "guess_rms_err_mlp")}
        summary["max_de"] = float(max(r["de"] for r in rows))
        summary["cases"] = len(rows)
        print(json.dumps({"summary": summary}), flush=True)
        with open(a.out + ".eval.json", "w") as f:
            json.dump({"precision": a.precision, "rows": rows, "summary": summary}, f, indent=1)
        return
    model = MLPGuess(0)
    build_training_set(model, a.n4, a.n6)
    t = time.time()
    loss = model.train(a.steps, a.batch, a.lr, seed=1)
    print(f"trained {a.steps} steps in {time.time() - t:.1f} s; loss {loss[0]:.4e} -> "
          f"{np.mean(loss[-50:]):.4e}", flush=True)
    model.save(a.out)
    np.savetxt(a.out + ".loss.txt", loss)
    rows = evaluate(model, cases)
    with open(a.out + ".eval.json", "w") as f:
        json.dump(rows, f, indent=1)


if __name__ == "__main__":
    main()
