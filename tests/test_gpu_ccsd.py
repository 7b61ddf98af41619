"""GPU parity of the CCSD path against the CPU oracle, through the C ABI."""
import numpy as np
import pytest

from conftest import inputs
from oracle import rccsd as R

pytestmark = pytest.mark.gpu


def _oracle_blocks(inp):
    return inp.conv if inp.Bvv is None else R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)


def _gpu_run(inp, guess=None, **opt):
    from fermicc import Options, RCCSD
    Options.reset()
    for k, v in opt.items():
        Options.set(k, v)
    if guess is None:
        return RCCSD.compute(inp)
    return RCCSD.compute(inp, guess[0], guess[1])


def _oracle_run(inp, guess=None, **opt):
    I = _oracle_blocks(inp)
    o = R.CCOptions(**opt)
    g1, g2 = (None, None) if guess is None else guess
    return R.rccsd(I, inp.eps_o, inp.eps_v, inp.e_ref, o, T1guess=g1, T2guess=g2, Bvv=inp.Bvv)


def _random_guess(inp, seed=0):
    I = _oracle_blocks(inp)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    rng = np.random.default_rng(seed)
    T1 = T1 + 0.02 * rng.standard_normal(T1.shape)
    T2 = T2 + 0.01 * rng.standard_normal(T2.shape)
    return T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


@pytest.mark.parametrize("case", ["conv1", "df1", "df2"])
def test_one_jacobi_step_matches_reference_terms(case):
    # one update from arbitrary amplitudes: GPU T1-dressed residual vs the
    # restated term-by-term equations (RCCSDHelper.jl:57-192, 304-349)
    inp = {"conv1": lambda: inputs(1, df=False), "df1": lambda: inputs(1), "df2": lambda: inputs(2)}[case]()
    g = _random_guess(inp)
    gpu = _gpu_run(inp, g, cc_max_iter=1, cc_diis=False)
    I = _oracle_blocks(inp)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    ladder = (lambda a, b: R.ladder_df(a, b, inp.Bvv)) if inp.Bvv is not None else \
        (lambda a, b: R.ladder_conv(a, b, I["VVVV"]))
    n1, n2 = R.update_amp(g[0], g[1], I, D1, D2, ladder)
    assert np.abs(gpu.T1 - n1).max() < 1e-11
    assert np.abs(gpu.T2 - n2).max() < 1e-11
    assert abs(gpu.correlation - R.cc_update_energy(n1, n2, I["OVOV"])) < 1e-11


@pytest.mark.parametrize("case", ["conv1", "df2"])
def test_converged_ccsd_matches_oracle(case):
    inp = inputs(1, df=False) if case == "conv1" else inputs(2)
    opt = dict(cc_e_conv=1e-10, cc_max_rms=1e-8)
    gpu = _gpu_run(inp, **opt)
    ref = _oracle_run(inp, **opt)
    assert gpu.converged and ref.converged
    assert abs(gpu.guessenergy - ref.guessenergy) < 1e-11
    assert abs(gpu.correlation - ref.correlation) < 1e-9
    assert abs(gpu.energy - ref.energy) < 1e-9
    assert abs(len(gpu.iterations) - len(ref.iterations)) <= 1
    # the iteration table tracks the reference's (DIIS dots in FP32 differ only in round-off)
    for a, b in zip(gpu.iterations[:6], ref.iterations[:6]):
        assert abs(a["energy"] - b["energy"]) < 1e-7
        assert a["diis"] == b["diis"]
    assert np.abs(gpu.T2 - ref.T2).max() < 1e-7


@pytest.mark.parametrize("opt", [dict(cc_diis=False), dict(cc_damp_ratio=0.3), dict(diis_prec="double"),
                                 dict(cc_ndiis=5, cc_diis_relax=2, diis_start=2)])
def test_option_paths_follow_oracle(opt):
    inp = inputs(2)
    full = dict(cc_max_iter=7, cc_e_conv=1e-12, cc_max_rms=1e-12, **opt)
    gpu = _gpu_run(inp, **full)
    ref = _oracle_run(inp, **full)
    assert len(gpu.iterations) == len(ref.iterations) == 7
    for a, b in zip(gpu.iterations, ref.iterations):
        assert abs(a["energy"] - b["energy"]) < 1e-8
        assert abs(a["rms"] - b["rms"]) < 1e-8 * max(1.0, b["rms"])


def test_max_iter_is_a_soft_stop():
    inp = inputs(2)
    gpu = _gpu_run(inp, cc_max_iter=2)
    assert not gpu.converged and len(gpu.iterations) == 2 and np.isfinite(gpu.energy)


def test_four_iterations_water_tetramer():
    inp = inputs(4)
    opt = dict(cc_max_iter=4, cc_e_conv=1e-12, cc_max_rms=1e-12)
    gpu = _gpu_run(inp, **opt)
    ref = _oracle_run(inp, **opt)
    for a, b in zip(gpu.iterations, ref.iterations):
        assert abs(a["energy"] - b["energy"]) < 1e-9


def test_errors_surface_as_status_codes():
    from fermicc import FermiException, Options, RCCSD
    from fermicc.rccsd import Context
    inp = inputs(1)
    ctx = Context(inp)
    with pytest.raises(FermiException, match="out of order"):
        ctx.triples(0)
    bad = np.full((inp.o, inp.v), np.nan)
    with pytest.raises(FermiException, match="non-finite"):
        ctx.set_guess(bad, np.zeros((inp.o, inp.o, inp.v, inp.v)))
    Options.reset()
    Options.set("cc_ndiis", 0)
    with pytest.raises(FermiException, match="invalid argument"):
        RCCSD.compute(inp, context=ctx)
    Options.reset()
    ctx.close()


@pytest.mark.parametrize("n,finish", [(2, "exact"), (4, "exact"), (2, "fp64"), (4, "fp64")])
def test_mixed_form_reaches_the_fp64_fixed_point(n, finish):
    # split-BF16 iterations until rms < 1e-5, exact-slice BF16 iterations
    # until the criteria hold, then the finish (exact-slice products at 9
    # weight groups, or FP64 DMMA): same converged energy as the FP64 form
    inp = inputs(n)
    opt = dict(cc_e_conv=1e-9, cc_max_rms=1e-8)
    e64 = _gpu_run(inp, **opt)
    mix = _gpu_run(inp, cc_gpu_precision="mixed", cc_gpu_finish=finish, **opt)
    assert mix.converged
    last = 3 if finish == "exact" else 0
    precs = [l["precision"] for l in mix.iterations]
    assert precs[0] == 1 and precs[-1] == last       # started split-BF16, ended on the finish
    assert precs == sorted(precs, key=lambda p: (1, 2, last).index(p))   # phases 1 -> 2 -> finish
    assert 2 in precs
    # the exact-slice residual is accurate enough that the finish meets the
    # criteria within a step or two of entering it: the FP64 finish (~25
    # exact-slice steps each) is entered only once the criteria hold ten
    # times over, the exact-slice finish as soon as they hold
    assert precs.count(last) <= (2 if finish == "fp64" else 4), precs
    assert abs(mix.correlation - e64.correlation) < 1e-7
    assert np.abs(mix.T2 - e64.T2).max() < 1e-6


@pytest.mark.parametrize("n", [2, 4])
def test_exact_finish_is_the_fp64_fixed_point(n):
    # the 9-group exact-slice residual (the mixed form's finish) at the FP64
    # form's tightly converged amplitudes: one Jacobi step from them moves
    # them no more than the FP64 residual's own step does, to 1e-11, so the
    # two residuals share the fixed point
    inp = inputs(n)
    star = _gpu_run(inp, cc_e_conv=1e-13, cc_max_rms=1e-12, cc_max_iter=200)
    assert star.converged
    g = (star.T1, star.T2)
    s64 = _gpu_run(inp, g, cc_max_iter=1, cc_diis=False)
    s9 = _gpu_run(inp, g, cc_max_iter=1, cc_diis=False, cc_gpu_precision="exact")
    assert [l["precision"] for l in s9.iterations] == [3]
    assert np.abs(s64.T2 - star.T2).max() < 1e-11
    assert np.abs(s9.T2 - s64.T2).max() < 1e-11
    assert np.abs(s9.T1 - s64.T1).max() < 1e-11
    assert abs(s9.correlation - s64.correlation) < 1e-11
    # and whole runs that end on the exact-slice finish land on the FP64
    # solution within the distance their convergence criteria allow
    opt = dict(cc_e_conv=1e-12, cc_max_rms=1e-11, cc_max_iter=100)
    for prec in ("mixed", "exact"):
        r = _gpu_run(inp, cc_gpu_precision=prec, cc_gpu_finish="exact", **opt)
        assert r.converged and r.iterations[-1]["precision"] == 3
        assert np.abs(r.T2 - star.T2).max() < 1e-8
        assert abs(r.correlation - star.correlation) < 1e-9
