"""The trainer's row-chunked linear layer on the CPU: the same values and derivatives as
torch.nn.Linear (first order for the forces, second order for the force-matching loss),
on row counts that are and are not multiples of the chunk, and below the chunking size."""
import pytest
import torch

from pyxtal_ff_gb300.train import RowChunkedLinear


@pytest.mark.parametrize("n", [100, 2048, 3001])
def test_row_chunked_linear_matches_linear_to_second_order(n):
    torch.manual_seed(n)
    lin = RowChunkedLinear(30, 17).double()
    ref = torch.nn.Linear(30, 17).double()
    ref.load_state_dict(lin.state_dict())
    x0 = torch.randn(n, 30, dtype=torch.float64)

    def run(m):
        x = x0.clone().requires_grad_(True)
        e = torch.tanh(m(x)).sum()
        g, = torch.autograd.grad(e, x, create_graph=True)
        (g ** 2).sum().backward()
        return e.detach(), g.detach(), m.weight.grad.clone(), m.bias.grad.clone()

    for a, b in zip(run(lin), run(ref)):
        assert torch.allclose(a, b, rtol=1e-12, atol=1e-12)


def test_row_chunked_linear_keeps_linear_parameters():
    lin = RowChunkedLinear(5, 3)
    assert isinstance(lin, torch.nn.Linear) and set(lin.state_dict()) == {"weight", "bias"}
