"""CPU reference of the learned preconditioner's network (TEST
INFRASTRUCTURE ONLY: the gradient and forward checks of the GPU kernels
import it; the product never does).

The network has no counterpart in the reference code base: it is the
library's learned preconditioner for the reference's solve (a 3-level 3-D
U-Net, 16/32/64 channels).  This module restates it in float64 PyTorch on the CPU with
autograd supplying the gradients, and emulates the GPU's BF16 storage
(weights and every stored activation rounded to BF16, nearest-even), so
that the only differences left are FP32 accumulation order and the BF16
rounding of activation gradients in the GPU's backward data pass.

Parameter layout (one flat float array, as libvdr's vdr_net_get_params):
for each layer its weights then its biases, each layer start rounded up to
a multiple of 8 floats.  3x3x3 weights are [tap][c_out][c_in] with tap =
(dz+1)*9 + (dy+1)*3 + (dx+1); the head is 16 weights and one bias.
Activations are on the node grid (x fastest); level l+1 halves each
extent, rounding up; pooling averages the children that exist; upsampling
is nearest.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.nn.functional as F

# (c_in skip, c_in upsampled, c_out, level) -- e0a e0b e1a e1b bta btb d1a
# d1b d0a d0b head
LAYERS = [(16, 0, 16, 0), (16, 0, 16, 0), (16, 0, 32, 1), (32, 0, 32, 1),
          (32, 0, 64, 2), (64, 0, 64, 2), (32, 64, 32, 1), (32, 0, 32, 1),
          (16, 32, 16, 0), (16, 0, 16, 0), (16, 0, 1, 0)]
HEAD = 10


def layout():
    """Offsets (weights, biases) of every layer and the total size."""
    off = 0
    out = []
    for i, (c1, c2, co, _) in enumerate(LAYERS):
        wsize = 16 if i == HEAD else 27 * co * (c1 + c2)
        wo = off
        off += wsize
        bo = off
        off += co
        off = (off + 7) & ~7
        out.append((wo, bo, wsize))
    return out, off


def bf16(t: torch.Tensor) -> torch.Tensor:
    return t.to(torch.bfloat16).to(torch.float64)


def dims(W, H, D):
    d = [(W, H, D)]
    for _ in range(2):
        w, h, z = d[-1]
        d.append(((w + 1) // 2, (h + 1) // 2, (z + 1) // 2))
    return d


def pool(x, fine, coarse):
    """x [C, D, H, W] -> [C, Dc, Hc, Wc]: mean of the existing children."""
    W, H, D = fine
    Wc, Hc, Dc = coarse
    pad = (0, 2 * Wc - W, 0, 2 * Hc - H, 0, 2 * Dc - D)
    xs = F.pad(x, pad)
    ones = F.pad(torch.ones((1, D, H, W), dtype=x.dtype), pad)
    C = x.shape[0]
    s = xs.reshape(C, Dc, 2, Hc, 2, Wc, 2).sum(dim=(2, 4, 6))
    n = ones.reshape(1, Dc, 2, Hc, 2, Wc, 2).sum(dim=(2, 4, 6))
    return s / n


def up(x, fine):
    W, H, D = fine
    y = x.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)
    y = y.repeat_interleave(2, dim=3)
    return y[:, :D, :H, :W]


def conv_weight(theta, lay, i):
    c1, c2, co, _ = LAYERS[i]
    wo, bo, ws = lay[i]
    w = theta[wo:wo + ws].reshape(27, co, c1 + c2)       # [tap][co][ci]
    w = w.permute(1, 2, 0).reshape(co, c1 + c2, 3, 3, 3)  # [co][ci][kz][ky][kx]
    return bf16(w), theta[bo:bo + co]


def forward(theta: torch.Tensor, rhat, feat, W, H, D, keep=None):
    """Head output c (length N) of the network for the normalised residual
    rhat (N) and features feat (N x 4); theta float64, requires_grad as the
    caller wishes.  `keep`, if a list, receives the stored activations."""
    lay, _ = layout()
    d = dims(W, H, D)
    N = W * H * D
    x = torch.zeros((16, D, H, W), dtype=torch.float64)
    x[0] = bf16(torch.as_tensor(rhat, dtype=torch.float64)).reshape(D, H, W)
    f = torch.as_tensor(feat, dtype=torch.float64).reshape(D, H, W, 4)
    for k in range(4):
        x[1 + k] = bf16(f[..., k])

    def conv(i, inp):
        w, b = conv_weight(theta, lay, i)
        y = F.conv3d(inp.unsqueeze(0), w, b, padding=1).squeeze(0)
        y = bf16(torch.relu(y))
        if keep is not None:
            keep.append(y)
        return y

    a0 = conv(0, x)
    s0 = conv(1, a0)
    p0 = bf16(pool(s0, d[0], d[1]))
    a1 = conv(2, p0)
    s1 = conv(3, a1)
    p1 = bf16(pool(s1, d[1], d[2]))
    a2 = conv(4, p1)
    b2 = conv(5, a2)
    a3 = conv(6, torch.cat([s1, up(b2, d[1])], dim=0))
    u1 = conv(7, a3)
    a4 = conv(8, torch.cat([s0, up(u1, d[0])], dim=0))
    u0 = conv(9, a4)
    wo, bo, _ = lay[HEAD]
    c = (theta[wo:wo + 16].reshape(16, 1, 1, 1) * u0).sum(dim=0) + theta[bo]
    return c.reshape(N)


def loss_and_grad(params, rhat, feat, target, mask, W, H, D):
    """Relative loss sum_free (c - t)^2 / sum_free t^2 and its gradient
    with respect to every parameter, in float64."""
    theta = torch.tensor(np.asarray(params, dtype=np.float64), requires_grad=True)
    c = forward(theta, rhat, feat, W, H, D)
    t = torch.as_tensor(target, dtype=torch.float64)
    free = torch.as_tensor(np.asarray(mask) == 0)
    d = torch.where(free, c - t, torch.zeros_like(c))
    tf = torch.where(free, t, torch.zeros_like(t))
    loss = (d * d).sum() / (tf * tf).sum()
    loss.backward()
    return (float(loss.detach()), theta.grad.numpy().copy(),
            c.detach().numpy().copy())
