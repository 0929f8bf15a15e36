"""Host-side guards of the adjoint entry points, without a GPU: the C ABI
cannot see buffer sizes, so the Python mirror checks the pick gradients and
the output against the taped batch, and the autograd wrapper refuses to run
a backward whose tape a later call on the same engine has replaced."""
import types

import numpy as np
import pytest


def fake_engine(shape=(2, 5), nxx=8, nzz=6):
    from seisfat2d_gb300.engine import Engine
    e = Engine.__new__(Engine)  # no context: only the host-side checks run
    e.nxx, e.nzz = nxx, nzz
    e.tape_generation = 0
    e.tape_shape = None
    e._tape_changed(shape)
    return e


def test_adjoint_arguments_checked_against_the_taped_batch():
    e = fake_engine()
    e._check_adjoint_args(np.zeros((2, 5)), None, "batch_adjoint")
    e._check_adjoint_args(np.zeros(10), np.zeros((8, 6)), "batch_adjoint")
    with pytest.raises(ValueError, match="12 values for a taped batch of 2 shots x 5 receivers"):
        e._check_adjoint_args(np.zeros((3, 4)), None, "batch_adjoint")
    with pytest.raises(ValueError, match="expected"):
        e._check_adjoint_args(np.zeros((2, 5)), np.zeros((6, 8)), "misfit_gradient")


def test_tape_generation_advances_with_every_replacement():
    e = fake_engine()
    g0 = e.tape_generation
    e._tape_changed((1, 5))
    assert e.tape_generation == g0 + 1 and e.tape_shape == (1, 5)
    e._tape_changed()
    assert e.tape_shape is None


def test_autograd_backward_raises_on_a_replaced_tape():
    torch = pytest.importorskip("torch")
    from seisfat2d_gb300.autograd import EikonalPicks
    e = fake_engine()
    ctx = types.SimpleNamespace(engine=e, generation=e.tape_generation, shape=(8, 6), device="cpu")
    e._tape_changed((1, 5))  # a later forward on the same engine
    with pytest.raises(RuntimeError, match="tape belongs to a later call"):
        EikonalPicks.backward(ctx, torch.zeros(2, 5))
