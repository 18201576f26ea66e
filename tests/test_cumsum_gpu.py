"""The optional libtorch binding: differentiable float32 cumsum along the last
dimension, forward = row scan, backward = reverse row scan of the upstream
gradient (a C++ torch::autograd::Function over the C ABI)."""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ext(cuda, built_lib):
    import ppcumsum

    return ppcumsum.load()


def test_forward_matches_fp64(ext, cuda):
    g = cuda.Generator(device="cuda").manual_seed(1)
    x = cuda.randn(257, 3001, device="cuda", generator=g)
    y = ext.cumsum(x)
    ref = cuda.cumsum(x.double(), dim=-1)
    bound = (64 + 4) * np.finfo(np.float32).eps * cuda.cumsum(x.double().abs(), dim=-1)
    assert bool(((y.double() - ref).abs() <= bound + 1e-30).all())


def test_backward_against_central_differences(ext, cuda):
    """FP64 central finite differences (eps = 1e-3) of L(x) = sum(w * cumsum(x))
    on a 64 x 256 input."""
    g = cuda.Generator(device="cuda").manual_seed(2)
    x = cuda.randn(64, 256, device="cuda", generator=g).requires_grad_(True)
    w = cuda.randn(64, 256, device="cuda", generator=g)
    (ext.cumsum(x) * w).sum().backward()
    grad = x.grad.double().cpu().numpy()
    xd = x.detach().double().cpu().numpy()
    wd = w.double().cpu().numpy()
    eps = 1e-3
    fd = np.empty_like(xd)
    for i in range(xd.shape[0]):  # L decomposes over rows
        row, wr = xd[i], wd[i]
        for j in range(xd.shape[1]):
            p, m = row.copy(), row.copy()
            p[j] += eps
            m[j] -= eps
            fd[i, j] = (np.dot(wr, np.cumsum(p)) - np.dot(wr, np.cumsum(m))) / (2 * eps)
    scale = np.cumsum(np.abs(wd[:, ::-1]), axis=1)[:, ::-1]
    assert np.all(np.abs(grad - fd) <= 1e-5 * scale + 1e-6)


def test_backward_full_tensor_against_suffix_sums(ext, cuda):
    """4096 x 8192 input, upstream gradient N(0,1): the gradient equals the
    FP64 suffix sums of the upstream gradient."""
    g = cuda.Generator(device="cuda").manual_seed(3)
    x = cuda.randn(4096, 8192, device="cuda", generator=g).requires_grad_(True)
    up = cuda.randn(4096, 8192, device="cuda", generator=g)
    y = ext.cumsum(x)
    y.backward(up)
    ref = cuda.flip(cuda.cumsum(cuda.flip(up.double(), [1]), dim=1), [1])
    absref = cuda.flip(cuda.cumsum(cuda.flip(up.double().abs(), [1]), dim=1), [1])
    err = (x.grad.double() - ref).abs()
    assert bool((err <= (64 + 4) * np.finfo(np.float32).eps * absref + 1e-30).all())
    fwd = cuda.cumsum(x.detach().double(), dim=1)
    assert float(((y.double() - fwd).abs() / (cuda.cumsum(x.detach().double().abs(), dim=1) + 1e-30)).max()) < 1e-5


def test_views_and_batches(ext, cuda):
    g = cuda.Generator(device="cuda").manual_seed(4)
    x = cuda.randn(3, 5, 1001, device="cuda", generator=g)
    v = x[:, 1:, 1:]  # non-contiguous, offset view
    np.testing.assert_allclose(ext.cumsum(v).cpu().numpy(), cuda.cumsum(v, dim=-1).cpu().numpy(), rtol=1e-5,
                               atol=1e-4)


def test_backward_of_long_rows_takes_the_reverse_look_back_kernel(ext, cuda):
    """Few rows longer than 65,536 elements are not split one warp per row:
    forward and backward run on the segmented decoupled look-back kernel
    (the backward in reverse), with tiles crossing row boundaries."""
    g = cuda.Generator(device="cuda").manual_seed(6)
    x = cuda.randn(3, 300001, device="cuda", generator=g).requires_grad_(True)
    up = cuda.randn(3, 300001, device="cuda", generator=g)
    y = ext.cumsum(x)
    y.backward(up)
    ref = cuda.flip(cuda.cumsum(cuda.flip(up.double(), [1]), dim=1), [1])
    absref = cuda.flip(cuda.cumsum(cuda.flip(up.double().abs(), [1]), dim=1), [1])
    err = (x.grad.double() - ref).abs()
    assert bool((err <= (64 + 64) * np.finfo(np.float32).eps * absref + 1e-30).all())
    fwd = cuda.cumsum(x.detach().double(), dim=1)
    absfwd = cuda.cumsum(x.detach().double().abs(), dim=1)
    assert bool(((y.detach().double() - fwd).abs() <= (64 + 64) * np.finfo(np.float32).eps * absfwd + 1e-30).all())
