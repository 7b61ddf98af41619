"""GPU parity at the workload sizes of the benchmark configurations.

* seeded (H2O)4 (o = 16 active, v = 76, naux = 336): the plain FP64 DF-CCSD
  converged to a 1e-8 residual, then (T), against the CPU restatement of
  RCCSDa.jl:92-244 / RCCSDHelper.jl:304-349 and ijk.jl:20-149;
* seeded (H2O)8 (o = 32, v = 152, naux = 672, the headline size): one FP64
  Jacobi step from the MP2 guess against the restated update_amp!, the same
  step with every contraction from exact-slice products at 9 weight groups,
  and single-triplet (T) contributions against the restated ijk.jl loop body.

Tolerances: 1e-9 Eh on converged energies, 1e-11 on amplitudes after one
step, 1e-12 Eh on single-triplet energies.
"""
import ctypes

import numpy as np
import pytest

from conftest import inputs
from oracle import rccsd as R
from oracle import triples as T

pytestmark = pytest.mark.gpu


def _run(inp, **opt):
    from fermicc import Options, RCCSD
    Options.reset()
    for k, v in opt.items():
        Options.set(k, v)
    return RCCSD.compute(inp)


def test_tetramer_fp64_ccsd_t_matches_oracle():
    inp = inputs(4, seed=0)
    opt = dict(cc_e_conv=1e-10, cc_max_rms=1e-8)
    gpu = _run(inp, **opt)
    from fermicc import RCCSDpT
    pt = RCCSDpT.compute(gpu, inp)
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    ref = R.rccsd(I, inp.eps_o, inp.eps_v, inp.e_ref, R.CCOptions(**opt), Bvv=inp.Bvv)
    assert gpu.converged and ref.converged
    assert abs(gpu.correlation - ref.correlation) < 1e-9
    assert abs(len(gpu.iterations) - len(ref.iterations)) <= 1
    # (T) of the oracle on the oracle's own amplitudes: the whole chain
    et = T.triples_ijk(ref.T1, ref.T2, I["OVVV"], I["OOOV"], I["OVOV"], inp.eps_o, inp.eps_v)
    assert abs(pt.correction - et) < 1e-9
    assert abs(pt.energy - (ref.energy + et)) < 2e-9


@pytest.fixture(scope="module")
def octamer_step():
    """One FP64 Jacobi step at (H2O)8 on the GPU and in the oracle."""
    inp = inputs(8, seed=0)
    gpu = _run(inp, cc_max_iter=1, cc_diis=False)
    I = R.df_blocks(inp.Boo, inp.Bov, inp.Bvv)
    D1, D2 = R.denominators(inp.eps_o, inp.eps_v)
    T1, T2 = R.mp2_guess(I, D1, D2)
    n1, n2 = R.update_amp(T1, T2, I, D1, D2, lambda a, b: R.ladder_df(a, b, inp.Bvv))
    return inp, I, gpu, n1, n2


def test_octamer_one_fp64_step_matches_reference_update(octamer_step):
    inp, I, gpu, n1, n2 = octamer_step
    assert np.abs(gpu.T1 - n1).max() < 1e-11
    assert np.abs(gpu.T2 - n2).max() < 1e-11
    assert abs(gpu.correlation - R.cc_update_energy(n1, n2, I["OVOV"])) < 1e-11


def test_octamer_one_exact_slice_step_is_fp64_accurate(octamer_step):
    # every contraction from exact-slice BF16 products at 9 weight groups: the
    # finish of the mixed form evaluates this residual
    inp, I, _, n1, n2 = octamer_step
    ex = _run(inp, cc_max_iter=1, cc_diis=False, cc_gpu_precision="exact")
    assert [l["precision"] for l in ex.iterations] == [3]
    assert np.abs(ex.T1 - n1).max() < 1e-11
    assert np.abs(ex.T2 - n2).max() < 1e-11
    assert abs(ex.correlation - R.cc_update_energy(n1, n2, I["OVOV"])) < 1e-11


def test_octamer_single_triplets_match_oracle(octamer_step):
    from fermicc import _lib
    inp, I, gpu, _, _ = octamer_step
    lib = _lib.load()
    trip = [(0, 0, 0), (5, 5, 2), (9, 4, 4), (17, 11, 3), (23, 23, 23), (31, 0, 0), (31, 30, 29), (31, 31, 12)]
    flat = (ctypes.c_int32 * (3 * len(trip)))(*[x for t in trip for x in t])
    out = (ctypes.c_double * len(trip))()
    assert lib.fcc_test_triples_subset(gpu.context.h, flat, len(trip), out) == 0
    for q, t in enumerate(trip):
        ref = T.triples_ijk(gpu.T1, gpu.T2, I["OVVV"], I["OOOV"], I["OVOV"], inp.eps_o, inp.eps_v, triplets=[t])
        assert abs(out[q] - ref) < 1e-12, (t, out[q], ref)
    assert out[0] == 0.0 and out[4] == 0.0          # i = j = k carries weight 0


def test_single_triplets_sum_to_the_full_correction():
    from fermicc import Options, RCCSDpT, _lib
    inp = inputs(2)
    gpu = _run(inp, cc_e_conv=1e-10, cc_max_rms=1e-9)
    Options.reset()
    et = RCCSDpT.compute(gpu, inp).correction
    trip = T.triplet_list(inp.o)
    flat = (ctypes.c_int32 * (3 * len(trip)))(*[x for t in trip for x in t])
    out = (ctypes.c_double * len(trip))()
    assert _lib.load().fcc_test_triples_subset(gpu.context.h, flat, len(trip), out) == 0
    assert abs(sum(out) - et) < 1e-13
