"""make_differentiable (monte_carlo.py:389-418), ported from the reference's
tests/test_gradients.py with torch autograd in place of TensorFlow's tape: the
result of ``run_event`` follows the integrand's autograd graph, so gradients
flow through the integral to the integrand's parameters."""

import numpy as np
import pytest
import torch

from vegasflow_gb300 import PlainFlow, VegasFlow, VegasFlowPlus

pytestmark = pytest.mark.gpu


def generate_integrand(variable):
    """An integrand that depends on an input variable (test_gradients.py:13-20)."""

    def example_integrand(x):
        return torch.sum(x, dim=1) * variable

    return example_integrand


def generate_differentiable_function(iclass, integrand, dims=3, n_calls=int(1e5), i_kwargs=None):
    """test_gradients.py:23-42, without the tf.function compilation."""
    i_kwargs = dict(i_kwargs or {})
    i_kwargs.setdefault("seed", 13)
    inst = iclass(dims, n_calls, verbose=False, **i_kwargs)
    inst.compile(integrand)
    _ = inst.run_integration(2)  # train
    runner = inst.make_differentiable()

    def some_complicated_function(x):
        integration_result, *_ = runner()
        return x * integration_result

    return some_complicated_function


def wrapper_test(iclass, x_point=5.0, alpha=10, integrator_kwargs=None):
    """test_gradients.py:45-71."""
    z = torch.tensor(1.0, dtype=torch.float64, device="cuda")
    fun = generate_differentiable_function(iclass, generate_integrand(z), i_kwargs=integrator_kwargs)
    x0 = torch.tensor(x_point, dtype=torch.float64, device="cuda", requires_grad=True)
    (grad_1,) = torch.autograd.grad(fun(x0).sum(), x0)
    z.mul_(alpha)  # change the variable the integrand reads
    (grad_2,) = torch.autograd.grad(fun(x0).sum(), x0)
    np.testing.assert_allclose((grad_1 * alpha).item(), grad_2.item(), rtol=1e-2)


@pytest.mark.parametrize("algorithm", [VegasFlowPlus, VegasFlow, PlainFlow])
def test_gradient(algorithm):
    wrapper_test(algorithm)


def test_gradient_VegasflowPlus_adaptive():
    wrapper_test(VegasFlowPlus, integrator_kwargs={"adaptive": True})


@pytest.mark.parametrize("algorithm", [VegasFlowPlus, VegasFlow, PlainFlow])
def test_gradient_through_the_integral(algorithm):
    """d/dz of the integral of z * sum_d x_d is the integral of sum_d x_d
    (= n_dim / 2 on the unit cube) on the same events."""
    z = torch.tensor(2.0, dtype=torch.float64, device="cuda", requires_grad=True)
    inst = algorithm(3, 200_000, verbose=False, seed=21)
    inst.compile(generate_integrand(z))
    inst.run_integration(2)
    runner = inst.make_differentiable()
    res = runner()[0].sum()
    (dz,) = torch.autograd.grad(res, z)
    np.testing.assert_allclose(dz.item(), res.item() / 2.0, rtol=1e-12)
    assert abs(dz.item() - 1.5) < 0.01
    # each call draws new events
    res_b = runner()[0].sum()
    assert res_b.item() != res.item()


def test_device_integrand_results_carry_no_graph():
    from vegasflow_gb300 import integrands

    inst = VegasFlow(3, 10_000, verbose=False, seed=1)
    inst.compile(integrands.symgauss())
    runner = inst.make_differentiable()
    out = runner()
    assert not out[0].requires_grad
