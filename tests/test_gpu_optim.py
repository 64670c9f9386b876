"""FusedAdam (one ernn_adam_step launch per parameter group) against
torch.optim.Adam, and its device step counter under CUDA-graph replay.
GPU only.  Tolerance: FP32 state; the update of each element matches
torch's to rounding, 1e-5 relative after 25 steps."""
import pytest
import torch

from ernn_gb300.optim import FusedAdam

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _params(seed, sizes=(6, 1000, 262144)):
    g = torch.Generator(device=DEV).manual_seed(seed)
    return [torch.randn(n, device=DEV, generator=g).requires_grad_(True) for n in sizes]


@pytest.mark.parametrize("wd", [0.0, 0.01])
def test_matches_torch_adam(wd):
    a, b = _params(0), _params(0)
    fa = FusedAdam(a, lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=wd)
    ta = torch.optim.Adam(b, lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=wd)
    g = torch.Generator(device=DEV).manual_seed(1)
    for _ in range(25):
        for p, q in zip(a, b):
            gr = torch.randn(p.shape, device=DEV, generator=g) * 1e-3
            p.grad = gr.clone()
            q.grad = gr.clone()
        fa.step()
        ta.step()
    for p, q in zip(a, b):
        err = ((p - q).abs().max() / q.abs().max()).item()
        assert err <= 1e-5, err
    assert int(fa.step_count()) == 25


def test_graph_replay_advances_the_step_count():
    a, b = _params(2, (6, 70)), _params(2, (6, 70))
    for p, q in zip(a, b):
        p.grad = torch.full_like(p, 0.3)
        q.grad = torch.full_like(q, 0.3)
    fa, fb = FusedAdam(a, lr=0.05), FusedAdam(b, lr=0.05)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        fa.step()  # builds the launch table
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        fa.step()
    for _ in range(4):
        graph.replay()
    for _ in range(5):
        fb.step()
    torch.cuda.synchronize()
    assert int(fa.step_count()) == 5 and int(fb.step_count()) == 5
    for p, q in zip(a, b):
        assert torch.equal(p, q)


def test_rejects_bad_parameters():
    p = torch.zeros(4, device=DEV, dtype=torch.float64, requires_grad=True)
    p.grad = torch.zeros_like(p)
    with pytest.raises(ValueError):
        FusedAdam([p]).step()
    with pytest.raises(ValueError):
        FusedAdam([torch.zeros(3, device=DEV, requires_grad=True)], betas=(1.0, 0.9))
