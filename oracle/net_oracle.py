"""FP32 CPU reference of the learned-guess network (test infrastructure).

A torch (CPU) restatement of the network in bluebottle-3.0_gb300/csrc/bbpp_net.cu:
the same parameter layout (per layer W[27][cout][cin] then bias; head w[16],
b[1]), the same padding (periodic x/y, zero z), pooling, upsampling,
concatenation and loss, and BF16 rounding at the points where the GPU stores
BF16 (inputs, weights, layer outputs, pooled values).  The reference has no
network; this is the floating-point reference the GPU kernels are checked
against.
"""
import numpy as np
import torch
import torch.nn.functional as F

LAYERS = [(16, 16), (16, 32), (32, 64), (96, 32), (48, 16)]


def bf16(t):
    return t.to(torch.bfloat16).to(torch.float32)


def bf16_bits(a):
    """float32 numpy -> uint16 BF16 bits (round to nearest even)."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bits_f32(b):
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def conv3(x, w, b=None, relu=False, px=True, py=True, pz=False, round_out=True):
    """x [N][C][z][y][x]; periodic or zero padding per axis; BF16 weights."""
    pad_x = (1, 1)
    x = F.pad(x, pad_x + (0, 0, 0, 0), mode="circular" if px else "constant")
    x = F.pad(x, (0, 0, 1, 1, 0, 0), mode="circular" if py else "constant")
    x = F.pad(x, (0, 0, 0, 0, 1, 1), mode="circular" if pz else "constant")
    y = F.conv3d(x, bf16(w), bias=b)
    if relu:
        y = F.relu(y)
    return bf16(y) if round_out else y


def pool(x):
    return bf16(F.avg_pool3d(x, 2))


def up(x):
    return F.interpolate(x, scale_factor=2, mode="nearest")


def loss_and_grad(params, r, prev, target, mask, h2):
    """Loss and its gradient with respect to the flat parameter vector; r is
    the residual of the warm start prev, target the correction p* - prev."""
    w = torch.tensor(np.asarray(params, dtype=np.float32), requires_grad=True)
    L = loss_torch(w, r, prev, target, mask, h2)
    L.backward()
    return float(L.detach()), w.grad.numpy().copy()


def loss_torch(w, rhs, prev, target, mask, h2):
    """Loss of the network with parameters w (torch tensor, differentiable)."""
    off = 0
    layers = []
    for cin, cout in LAYERS:
        n = 27 * cin * cout
        W = w[off:off + n].reshape(3, 3, 3, cout, cin).permute(3, 4, 0, 1, 2)
        off += n
        b = w[off:off + cout]
        off += cout
        layers.append((W, b))
    hw = w[off:off + 16]
    hb = w[off + 16:off + 17]
    rhs = torch.as_tensor(rhs)
    prev = None if prev is None else torch.as_tensor(prev)
    target = torch.as_tensor(target)
    n = rhs.shape[0]
    fluid = torch.ones(rhs.shape[1:], dtype=torch.bool) if mask is None else torch.as_tensor(mask) == 0
    sc = []
    for b in range(n):
        sb = torch.sqrt((rhs[b][fluid].double() ** 2).mean())
        sp = torch.sqrt((prev[b][fluid].double() ** 2).mean()) if prev is not None else torch.tensor(0.0)
        sc.append((float(1.0 / sb) if sb > 0 else 1.0, float(1.0 / sp) if sp > 0 else 1.0))
    sc = torch.tensor(np.array(sc, dtype=np.float32))
    m = (~fluid).float()
    r = torch.where(fluid, rhs * sc[:, 0].view(-1, 1, 1, 1), torch.zeros(()))
    p = torch.where(fluid, prev * sc[:, 1].view(-1, 1, 1, 1), torch.zeros(())) if prev is not None else torch.zeros_like(r)
    x0 = torch.zeros((n, 16) + tuple(rhs.shape[1:]))
    x0[:, 0] = r
    x0[:, 1] = p
    x0[:, 2] = m
    x0 = bf16(x0)
    (w1, b1), (w2, b2), (w3, b3), (w4, b4), (w5, b5) = layers
    e1 = conv3(x0, w1, b1, relu=True)
    p1 = pool(e1)
    e2 = conv3(p1, w2, b2, relu=True)
    p2 = pool(e2)
    e3 = conv3(p2, w3, b3, relu=True)
    cat2 = torch.cat([up(e3), e2], dim=1)
    d2 = conv3(cat2, w4, b4, relu=True)
    cat1 = torch.cat([up(d2), e1], dim=1)
    d1 = conv3(cat1, w5, b5, relu=True)
    out = torch.einsum("nczyx,c->nzyx", d1, hw) + hb
    d = (out - target * (sc[:, 0] / h2).view(-1, 1, 1, 1))[:, fluid]
    return (d * d).sum() / d.numel()
