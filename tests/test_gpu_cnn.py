"""GPU: the learned estimator's BF16 tensor-core kernels against a PyTorch FP32
reference of the same network (BF16 rounding applied at the same points)."""

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from hermespy_gb300.learned import CnnChannelEstimator

pytestmark = pytest.mark.gpu
H, W = 14, 600


def bf(x):
    return x.to(torch.bfloat16).to(torch.float32)


def planes(z):
    """(B, 16, H, W) complex -> (B, 32, H, W) real, channel 2 p + (re, im)."""

    return torch.stack([z.real, z.imag], dim=2).reshape(z.shape[0], 32, z.shape[2], z.shape[3])


def unplanes(x):
    x = x.reshape(x.shape[0], 16, 2, x.shape[2], x.shape[3])
    return torch.complex(x[:, :, 0], x[:, :, 1])


def reference(model, params, ls):
    wt, bias = model.split(params)
    w = [bf(torch.from_numpy(np.ascontiguousarray(wt[l])).cuda()).reshape(32, 3, 3, 32).permute(0, 3, 1, 2)
         .contiguous() for l in range(6)]
    b = torch.from_numpy(bias).cuda()
    x = planes(ls)
    s = torch.sqrt(torch.mean(x.reshape(x.shape[0], -1) ** 2, dim=1) * 2)[:, None, None, None]  # RMS of |LS|
    acts = [bf(x / s)]
    for l in range(5):
        acts.append(bf(torch.relu(F.conv2d(acts[-1], w[l], padding=1) + b[l][None, :, None, None])))
    z = F.conv2d(acts[-1], w[5], padding=1) + b[5][None, :, None, None]
    return x + s * z, acts, w, s


def _inputs(B, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    truth = torch.randn((B, 16, H, W), dtype=torch.complex64, device="cuda", generator=g)
    noise = 0.3 * torch.randn((B, 16, H, W), dtype=torch.complex64, device="cuda", generator=g)
    return (truth + noise).contiguous(), truth.contiguous()


def test_forward_matches_reference():
    model = CnnChannelEstimator(H, W, max_batch=2, seed=3)
    # a non-trivial last layer, so the refinement is not close to the identity
    p = model.params()
    p[5 * 32 * 288: 6 * 32 * 288] *= 50.0
    p[6 * 32 * 288:] = np.random.default_rng(1).normal(0, 0.1, 6 * 32).astype(np.float32)
    model = CnnChannelEstimator(H, W, max_batch=2, params=p)
    ls, _ = _inputs(3, 5)  # three drops: two chunks of the refine loop
    ref, _, _, _ = reference(model, p, ls)
    out = model.refine(ls.clone())
    torch.cuda.synchronize()
    delta = planes(out) - planes(ls)
    rdelta = ref - planes(ls)
    rel = float(torch.sqrt(torch.sum((delta - rdelta) ** 2) / torch.sum(rdelta ** 2)))
    assert rel < 5e-3, rel


def test_gradients_match_reference():
    model = CnnChannelEstimator(H, W, max_batch=2, seed=4)
    p = model.params()
    p[5 * 32 * 288: 6 * 32 * 288] *= 30.0
    model = CnnChannelEstimator(H, W, max_batch=2, params=p)
    ls, truth = _inputs(2, 6)
    model.train_step(ls, truth, 0.0)
    torch.cuda.synchronize()
    gk = model.grads()
    gw, gb = model.split(gk)
    out, acts, w, sc = reference(model, p, ls)
    g = bf((out - planes(truth)) / sc)
    for l in range(5, -1, -1):
        dw = torch.nn.grad.conv2d_weight(acts[l], w[l].shape, g, padding=1)  # [out][in][ky][kx]
        dw = dw.permute(0, 2, 3, 1).reshape(32, 9, 32).cpu().numpy()
        db = g.sum(dim=(0, 2, 3)).cpu().numpy()
        rel_w = np.sqrt(np.sum((gw[l] - dw) ** 2) / np.sum(dw ** 2))
        rel_b = np.sqrt(np.sum((gb[l] - db) ** 2) / np.sum(db ** 2))
        assert rel_w < 2e-2, (l, rel_w)
        assert rel_b < 2e-2, (l, rel_b)
        if l > 0:
            gin = torch.nn.grad.conv2d_input(acts[l].shape, w[l], g, padding=1)
            g = bf(gin * (acts[l] > 0))


def test_adam_first_step():
    """First Adam step: m_hat = g, v_hat = g^2, so every parameter moves by
    -lr g / (|g| + 1e-8), about -lr sign(g)."""

    model = CnnChannelEstimator(H, W, max_batch=2, seed=9)
    p0 = model.params()
    ls, truth = _inputs(2, 10)
    lr = 1e-3
    model.train_step(ls, truth, lr)
    torch.cuda.synchronize()
    g = model.grads() / (2 * H * W * 32)  # the step averages the gradient sums
    p1 = model.params()
    big = np.abs(g) > 1e-6
    assert big.sum() > 0.05 * g.size
    assert np.allclose(p1[big], p0[big] - lr * g[big] / (np.abs(g[big]) + 1e-8), atol=2e-7)


def _smooth(B, seed):
    """Random smooth channel-like field: a few complex exponentials along the columns,
    slowly rotating over the words, plus LS-like noise."""

    rng = np.random.default_rng(seed)
    c = np.arange(W)[None, :]
    h = np.arange(H)[:, None]
    truth = np.zeros((B, 16, H, W), dtype=np.complex64)
    for b in range(B):
        for p in range(16):
            for _ in range(4):
                f, nu = rng.uniform(0, 0.02), rng.uniform(-0.05, 0.05)
                a = (rng.normal() + 1j * rng.normal()) / 2
                truth[b, p] += (a * np.exp(2j * np.pi * (f * c + nu * h))).astype(np.complex64)
    noise = (rng.normal(size=truth.shape) + 1j * rng.normal(size=truth.shape)).astype(np.complex64) * 0.5
    return torch.from_numpy(truth + noise).cuda(), torch.from_numpy(truth).cuda()


def test_training_denoises_smooth_field():
    model = CnnChannelEstimator(H, W, max_batch=2, seed=7)
    ls, truth = _smooth(2, 8)
    losses = [float(model.train_step(ls, truth, 3e-3).item()) for _ in range(80)]
    assert np.all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.9 * np.mean(losses[:5]), (losses[:5], losses[-5:])
    assert np.all(np.isfinite(model.params()))
