"""torch.ops.sad from the C++ operator library: argument checks with the reference's
messages (backends/pytorch/torch_ext/cuda/sad_bindings.cu), the caller's stream, and the
autograd path through SADRenderFunction on those operators."""
import numpy as np
import pytest
import torch

import cases

pytestmark = pytest.mark.gpu


def t32(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def test_argument_errors(cuda):
    from sad_gb300 import ops
    w, h, n = 16, 12, 20
    _, sites = cases.scene(w, h, n, 3)
    c0, c1 = ops.init_candidates(w, h, n, 1)
    s = torch.from_numpy(sites).cuda()
    with pytest.raises(RuntimeError, match="cand0 must be int32"):
        ops.render_sad(c0.float(), c1, s, 1.0 / w ** 2, w, h)
    with pytest.raises(RuntimeError, match=r"sites must be \[N,10\]"):
        ops.render_sad(c0, c1, s[:, :9].contiguous(), 1.0 / w ** 2, w, h)
    with pytest.raises(RuntimeError, match="cand0 size must match width\\*height"):
        ops.render_sad(c0, c1, s, 1.0 / w ** 2, w + 1, h)
    with pytest.raises(RuntimeError, match=r"grad_output must be \[H,W,3\]"):
        ops.render_sad_backward(c0, c1, s, torch.zeros((h, w), device="cuda"), 1.0 / w ** 2, w, h)
    with pytest.raises(RuntimeError, match="pairs must be non-empty"):
        ops.radix_sort_pairs(torch.zeros((0, 2), dtype=torch.int32, device="cuda"), 16)
    with pytest.raises(RuntimeError):  # no CPU kernel is registered, as in the reference
        ops.render_sad(c0.cpu(), c1.cpu(), s.cpu(), 1.0 / w ** 2, w, h)


def test_ops_follow_current_stream_and_graph_capture(cuda, orc):
    from sad_gb300 import ops
    w, h, n = 64, 48, 300
    _, sites = cases.scene(w, h, n, 4)
    c0, c1 = cases.random_field(w, h, n, 4)
    d0, d1, s = t32(c0), t32(c1), torch.from_numpy(sites).cuda()
    want = ops.render_sad(d0, d1, s, 1.0 / w ** 2, w, h)
    g = torch.cuda.CUDAGraph()
    stream = torch.cuda.Stream()
    stream.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(stream):
        ops.render_sad(d0, d1, s, 1.0 / w ** 2, w, h)  # warm-up on the capture stream
        with torch.cuda.graph(g, stream=stream):
            out = ops.render_sad(d0, d1, s, 1.0 / w ** 2, w, h)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(out, want)


def test_autograd_matches_backward_op(cuda):
    from sad_gb300 import SADRenderFunction, ops
    w, h, n = 48, 40, 200
    _, sites = cases.scene(w, h, n, 5)
    c0, c1 = cases.random_field(w, h, n, 5)
    d0, d1 = t32(c0), t32(c1)
    s = torch.from_numpy(sites).cuda().requires_grad_(True)
    out = SADRenderFunction.apply(s, d0, d1, 1.0 / w ** 2, w, h)
    go = torch.randn_like(out)
    out.backward(go)
    want = ops.render_sad_backward(d0, d1, s.detach(), go, 1.0 / w ** 2, w, h)
    # float atomics: the summation order may differ between the two runs
    torch.testing.assert_close(s.grad, want, rtol=1e-5, atol=1e-6)
