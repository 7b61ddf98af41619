"""Checkpoint files of the amplitudes: layout, round trip and restart."""
import struct

import numpy as np
import pytest

from conftest import inputs

pytestmark = pytest.mark.gpu


def _header(raw):
    magic = raw[:8]
    version, o, v, naux = struct.unpack("<4i", raw[8:24])
    ecc, eref = struct.unpack("<2d", raw[24:40])
    iters, conv = struct.unpack("<2i", raw[40:48])
    return magic, version, o, v, naux, ecc, eref, iters, conv


def test_checkpoint_layout_and_restart(tmp_path):
    from fermicc import Options, RCCSD
    from fermicc.options import FermiException
    from fermicc.rccsd import Context
    inp = inputs(2)
    crit = dict(cc_max_rms=1e-9, cc_e_conv=1e-10)

    Options.reset()
    for k, v in crit.items():
        Options.set(k, v)
    full = RCCSD.compute(inp)
    assert full.converged

    # four iterations, checkpointed every second one and at the end
    path = tmp_path / "amps.fcc"
    Options.set("cc_max_iter", 4)
    Options.set("cc_gpu_checkpoint", str(path))
    Options.set("cc_gpu_checkpoint_every", 2)
    part = RCCSD.compute(inp)
    assert not part.converged and len(part.iterations) == 4
    raw = path.read_bytes()
    magic, version, o, v, naux, ecc, eref, iters, conv = _header(raw)
    assert magic == b"FCCCKPT1" and version == 1
    assert (o, v, naux) == (inp.o, inp.v, inp.naux)
    assert iters == 4 and conv == 0
    assert ecc == pytest.approx(part.correlation, abs=1e-14)
    assert len(raw) == 64 + 8 * (o * v + o * o * v * v)
    T1 = np.frombuffer(raw, dtype="<f8", count=o * v, offset=64).reshape((o, v), order="F")
    T2 = np.frombuffer(raw, dtype="<f8", offset=64 + 8 * o * v).reshape((o, o, v, v), order="F")
    assert np.array_equal(T1, part.T1) and np.array_equal(T2, part.T2)

    # restart from the file in a fresh context: same converged energy
    Options.reset()
    for k, val in crit.items():
        Options.set(k, val)
    ctx = Context(inp)
    ctx.load_checkpoint(path)
    res = RCCSD.compute(inp, context=ctx)
    assert res.converged
    assert abs(res.energy - full.energy) < 1e-9
    assert len(res.iterations) < len(full.iterations)

    # a file that is not a checkpoint, or of another size, is refused
    bad = tmp_path / "bad.fcc"
    bad.write_bytes(b"not a checkpoint" * 8)
    with pytest.raises(FermiException, match="not a checkpoint"):
        ctx.load_checkpoint(bad)
    other = inputs(1)
    octx = Context(other)
    with pytest.raises(FermiException, match="dimensions"):
        octx.load_checkpoint(path)
    octx.close()
    ctx.close()
    Options.reset()
