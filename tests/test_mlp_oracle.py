"""CPU checks of the MLP oracle and the parameter layout (no GPU)."""
import numpy as np

from oracle import mlp as OM


def test_parameter_count_matches_library():
    from fermicc import _lib
    import os
    if not os.path.exists(_lib.LIB_PATH):
        import __graft_entry__
        __graft_entry__.build()
    assert _lib.load().fcc_mlp_num_params() == OM.NPARAM == 18849


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-9 + 2**-12, -3.14159265], dtype=np.float32)
    r = OM.bf16_round(x)
    assert r[0] == 1.0
    assert r[1] == 1.0              # exactly half an ulp above 1: ties to even
    assert r[2] == 1.0              # below half an ulp
    assert abs(r[3] - (-3.140625)) < 1e-12


def test_oracle_gradient_by_finite_differences():
    rng = np.random.default_rng(0)
    p = np.zeros(OM.NPARAM)
    p[: OM.NTRAIN] = 0.2 * rng.standard_normal(OM.NTRAIN)
    p[OM.OFF_SD:] = 1.0
    X = rng.standard_normal((13, OM.NF))
    y = rng.standard_normal(13)
    # finite differences on the FP32-master parameters (w3, biases) that are
    # not BF16-rounded in the forward pass
    _, g = OM.loss_and_grad(p, X, y)
    for idx in (OM.OFF_B1 + 3, OM.OFF_B2 + 7, OM.OFF_W3 + 5, OM.OFF_B3):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (OM.loss_and_grad(pp, X, y)[0] - OM.loss_and_grad(pm, X, y)[0]) / (2 * h)
        assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(fd))
