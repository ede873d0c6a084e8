"""Sequence design: the bounded-variable map, the optimiser loop, the CRLB
(interface of the reference's optim/_design.py, tests/optim/test_design.py)."""

import numpy as np
import pytest
import torch

from torchsim_gb300.design import Bounded, SequenceDesign, crlb


def test_bounded_start_round_trips_and_stays_inside():
    start = torch.tensor([10.0, 35.0, 69.0])
    design = SequenceDesign(lambda flip: (flip ** 2).sum(), flip=Bounded(start, 5.0, 70.0))
    torch.testing.assert_close(design.values()["flip"], start, rtol=1e-5, atol=1e-4)
    result = design.minimize(iterations=300, learning_rate=0.2)
    flip = result.parameters["flip"]
    assert torch.all(flip >= 5.0) and torch.all(flip <= 70.0)
    # The cost pushes every flip to its lower limit.
    assert float(flip.max()) < 5.5
    assert result.loss.shape == (300,)
    assert float(result.loss[-1]) < float(result.loss[0])


def test_per_element_limits_and_free_parameters():
    lower = torch.tensor([0.0, 10.0])
    upper = torch.tensor([1.0, 20.0])
    target = torch.tensor([3.0, -2.0])
    design = SequenceDesign(
        lambda a, b: ((a - 0.25) ** 2).sum() + ((b - target) ** 2).sum(),
        a=Bounded(torch.tensor([0.5, 15.0]), lower, upper), b=torch.zeros(2))
    result = design.minimize(iterations=400, learning_rate=0.1)
    a = result.parameters["a"]
    assert 0.2 < float(a[0]) < 0.3
    assert 10.0 <= float(a[1]) < 10.5
    torch.testing.assert_close(result.parameters["b"], target, atol=1e-2, rtol=0)


def test_callback_stops_early_and_argument_errors():
    design = SequenceDesign(lambda x: (x ** 2).sum(), x=torch.ones(3))
    seen = []
    result = design.minimize(iterations=50, callback=lambda step, values, loss: seen.append(step) or step == 4)
    assert seen == [0, 1, 2, 3, 4] and result.loss.shape == (5,)
    with pytest.raises(ValueError):
        SequenceDesign(lambda: torch.zeros(()))
    with pytest.raises(ValueError):
        SequenceDesign(lambda x: x.sum(), x=Bounded(torch.ones(2), 2.0, 1.0))
    with pytest.raises(ValueError):
        SequenceDesign(lambda x: x, x=torch.ones(2))()
    with pytest.raises(ValueError):
        design.minimize(iterations=0)


def test_crlb_matches_the_inverse_fisher():
    rng = np.random.default_rng(3)
    jac = rng.standard_normal((5, 3, 40)) + 1j * rng.standard_normal((5, 3, 40))
    got = crlb(torch.from_numpy(jac), noise_variance=0.5).numpy()
    for v in range(5):
        rows = np.concatenate([jac[v].real, jac[v].imag], axis=1)
        want = 0.5 * np.diag(np.linalg.inv(rows @ rows.T))
        np.testing.assert_allclose(got[v], want, rtol=1e-10)
    singular = torch.zeros((2, 2, 8), dtype=torch.float64)
    singular[0] = torch.from_numpy(rng.standard_normal((2, 8)))
    bound = crlb(singular, singular="infinite")
    assert torch.isfinite(bound[0]).all() and torch.isinf(bound[1]).all()
    with pytest.raises(torch.linalg.LinAlgError):
        crlb(singular)
    with pytest.raises(ValueError):
        crlb(torch.zeros(4))


def test_design_layer_matches_the_reference(golden):
    """The reference's own crlb and SequenceDesign loop on a pure-torch cost
    (tests/golden/design_loop.npz, made by tests/golden/make_golden.py from
    optim/_design.py): the bounds of real and complex Jacobians, the infinite
    answer of a singular one, and 25 Adam steps over two bounded vectors
    (one with per-element limits) -- every step's loss and the final values."""
    import numpy as np

    d = golden("design_loop")
    for name in ("real", "complex"):
        got = crlb(torch.from_numpy(d[name]), noise_variance=0.5).numpy()
        np.testing.assert_allclose(got, d[f"crlb_{name}"], rtol=1e-5)
    got = crlb(torch.from_numpy(d["singular"]), singular="infinite").numpy()
    want = d["crlb_singular"]
    assert np.array_equal(np.isinf(got), np.isinf(want))
    finite = np.isfinite(want)
    np.testing.assert_allclose(got[finite], want[finite], rtol=1e-5)

    target = torch.from_numpy(d["target"])

    def cost(flip, tr):
        return ((torch.sin(torch.deg2rad(flip)) - target) ** 2).sum() + 1e-3 * (tr - 9.0).square().sum()

    design = SequenceDesign(cost, flip=Bounded(torch.from_numpy(d["flip0"]), 5.0,
                                               torch.from_numpy(d["upper"])),
                            tr=Bounded(torch.from_numpy(d["tr0"]), 8.0, 15.0))
    result = design.minimize(iterations=25, learning_rate=0.05)
    np.testing.assert_allclose(result.loss.numpy(), d["loss"], rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(result.parameters["flip"].numpy(), d["flip"], rtol=1e-5)
    np.testing.assert_allclose(result.parameters["tr"].numpy(), d["tr"], rtol=1e-5)
