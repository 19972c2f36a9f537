"""CPU: the autograd wrapper's host table of per-image parameters is reused
only while the parameter tensors are the same objects, unwritten since."""
import torch

from millipyde_gb300 import autograd as A


def test_table_reused_while_unchanged_and_rebuilt_after_writes():
    theta = torch.tensor([10.0, -20.0], dtype=torch.float64)
    sigma = torch.tensor(1.5)
    slots = [(0, 0), (1, 0)]
    p1 = A._param_table(2, 2, slots, [theta, sigma])
    assert p1[:, 0, 0].tolist() == [10.0, -20.0] and p1[:, 1, 0].tolist() == [1.5, 1.5]
    assert A._param_table(2, 2, slots, [theta, sigma]) is p1
    with torch.no_grad():
        theta.mul_(2)
    p2 = A._param_table(2, 2, slots, [theta, sigma])
    assert p2 is not p1 and p2[:, 0, 0].tolist() == [20.0, -40.0]
    # a new tensor object with other values is never mistaken for the old one
    p3 = A._param_table(2, 2, slots, [torch.tensor([1.0, 2.0], dtype=torch.float64), sigma])
    assert p3[:, 0, 0].tolist() == [1.0, 2.0]


def test_host_parameters_match_by_value():
    """Python floats become a new CPU tensor on every call (adjust_gamma's
    implicit gain among them): equal values reuse the table, other values
    do not."""
    gamma = torch.tensor([0.8, 1.2], dtype=torch.float64)
    slots = [(0, 0), (0, 1)]
    p1 = A._param_table(2, 1, slots, [gamma, torch.tensor(1.0, dtype=torch.float64)])
    assert A._param_table(2, 1, slots, [gamma, torch.tensor(1.0, dtype=torch.float64)]) is p1
    p2 = A._param_table(2, 1, slots, [gamma, torch.tensor(0.5, dtype=torch.float64)])
    assert p2 is not p1 and p2[:, 0, 1].tolist() == [0.5, 0.5]
    assert p1[:, 0, 1].tolist() == [1.0, 1.0]
