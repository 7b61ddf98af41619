"""Options and method dispatch of the host mirror (no GPU needed)."""
import pytest

from fermicc import FermiException, Options, get_pt_alg, get_rccsd_alg
from fermicc.rccsd import CudaPT, RCCSDcuda


def setup_function():
    Options.reset()


def test_defaults_and_coercion():
    assert Options.get("cc_max_iter") == 50
    Options.set("CC_MAX_ITER", "12")
    assert Options.get("cc_max_iter") == 12
    Options.set("cc_diis", "false")
    assert Options.get("cc_diis") is False
    Options.set("cc_gpu_precision", "MIXED")
    assert Options.get("cc_gpu_precision") == "mixed"


def test_unknown_key_and_bad_type():
    with pytest.raises(FermiException):
        Options.set("no_such_option", 1)
    with pytest.raises(FermiException):
        Options.set("cc_max_iter", "many")
    with pytest.raises(FermiException):
        Options.set("cc_max_iter", 1.5)


def test_algorithm_selection():
    assert isinstance(get_rccsd_alg(), RCCSDcuda)
    assert isinstance(get_pt_alg(), CudaPT)
    Options.set("cc_alg", 1)
    with pytest.raises(FermiException):
        get_rccsd_alg()
    with pytest.raises(FermiException):
        get_pt_alg(3)
