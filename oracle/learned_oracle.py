"""CPU oracle of the learned initial guess's network (test infrastructure only).

The same net as the library's learned.cu, in torch on the CPU: a 3-level
U-Net of 3x3x3 convolutions (zero padding, ReLU) with 16/32/64 channels,
2x2x2 average pooling, nearest 2x up-sampling and channel concatenation
(up-sampled first, then the encoder's output of the level), and a 1x1x1
convolution to one channel; trained on the residual-norm loss
|A d - r|^2 / |r|^2 with A the 7-point window operator (neighbours outside the
window are zero), or against a recorded converged correction t on the
supervised loss |d - t|^2 / |t|^2 or the energy norm (d - t)'A(d - t) / t'At.  The library stores weights and activations in BF16 and
accumulates in FP32; the oracle rounds the same quantities to BF16 and
computes everything else in FP32, so outputs and gradients agree to the BF16
rounding of the intermediate tensors.

Parameter vector layout (the library's): for each 3x3x3 layer, in execution
order e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b, W[co][tap][ci]
(tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[co]; then the 1x1x1 weights w[ci]
and bias b.  The first layer's input has one channel; the library stores it as
16 channels of which 15 are zero, so only W[:, :, 0] of layer 0 acts.
"""
import numpy as np

CI = (16, 16, 16, 32, 32, 64, 96, 32, 48, 16)
CO = (16, 16, 32, 32, 64, 64, 32, 32, 16, 16)
C1 = 16
NPARAMS = sum(co * 27 * ci + co for ci, co in zip(CI, CO)) + C1 + 1


def bf16(t):
    import torch
    return t.to(torch.bfloat16).to(torch.float32)


def ste(a):
    """BF16 storage of an activation (rounding seen as identity by the gradient)."""
    return a + (bf16(a) - a).detach()


def unpack(p):
    """Parameter vector -> list of (W (co, ci, 3, 3, 3), b) and (w_last, b_last) as torch tensors."""
    import torch
    p = torch.as_tensor(np.asarray(p, np.float32))
    convs = []
    o = 0
    for ci, co in zip(CI, CO):
        W = p[o:o + co * 27 * ci].reshape(co, 27, ci)        # [co][tap][ci]
        W = W.permute(0, 2, 1).reshape(co, ci, 3, 3, 3)      # (co, ci, kz, ky, kx)
        o += co * 27 * ci
        b = p[o:o + co]
        o += co
        convs.append((W, b))
    return convs, p[o:o + C1], p[o + C1]


def forward(p, x, requires_grad=False):
    """x: (D, H, W) input (extents multiples of 4).  Returns output (D, H, W) and the leaf tensors."""
    import torch
    import torch.nn.functional as F
    convs, wl, bl = unpack(p)
    leaves = []
    for W, b in convs:
        W.requires_grad_(requires_grad)
        b.requires_grad_(requires_grad)
        leaves += [W, b]
    wl.requires_grad_(requires_grad)
    bl.requires_grad_(requires_grad)
    leaves += [wl, bl]

    def conv(a, l):
        W, b = convs[l]
        Wq = bf16(W)
        if l == 0:
            Wq = Wq[:, :1]
        return ste(F.relu(F.conv3d(a, Wq, b, padding=1)))

    def up(a):
        return a.repeat_interleave(2, 2).repeat_interleave(2, 3).repeat_interleave(2, 4)

    a0 = bf16(torch.as_tensor(np.asarray(x, np.float32)))[None, None]   # (1, 1, D, H, W)
    s1 = conv(conv(a0, 0), 1)
    p1 = ste(F.avg_pool3d(s1, 2))
    s2 = conv(conv(p1, 2), 3)
    p2 = ste(F.avg_pool3d(s2, 2))
    b3 = conv(conv(p2, 4), 5)
    x2 = conv(conv(torch.cat([up(b3), s2], 1), 6), 7)
    x1 = conv(conv(torch.cat([up(x2), s1], 1), 8), 9)
    out = (x1[0] * wl[:, None, None, None]).sum(0) + bl
    return out, leaves


def apply_a(coef, d):
    """Window operator: coef (7, D, H, W) planes xp, xm, yp, ym, zp, zm, diag."""
    import torch
    import torch.nn.functional as F
    c = torch.as_tensor(np.asarray(coef, np.float32))
    q = F.pad(d, (1, 1, 1, 1, 1, 1))
    return (c[6] * d - c[0] * q[1:-1, 1:-1, 2:] - c[1] * q[1:-1, 1:-1, :-2] - c[2] * q[1:-1, 2:, 1:-1]
            - c[3] * q[1:-1, :-2, 1:-1] - c[4] * q[2:, 1:-1, 1:-1] - c[5] * q[:-2, 1:-1, 1:-1])


def loss_and_grad(p, rhs, coef, target=None, kind=0):
    """A training loss and its gradient with respect to the parameter vector:
    kind 0 the residual norm |A d - r|^2/|r|^2, 1 supervised |d - t|^2/|t|^2,
    2 energy norm (d - t)'A(d - t)/t'At against the target t."""
    import torch
    out, leaves = forward(p, rhs, requires_grad=True)
    r = torch.as_tensor(np.asarray(rhs, np.float32))
    if kind == 0:
        loss = ((apply_a(coef, out) - r) ** 2).sum() / (r ** 2).sum()
    else:
        t = torch.as_tensor(np.asarray(target, np.float32))
        e = out - t
        if kind == 1:
            loss = (e ** 2).sum() / (t ** 2).sum()
        else:
            loss = (e * apply_a(coef, e)).sum() / (t * apply_a(coef, t)).sum()
    loss.backward()
    g = []
    for l, (ci, co) in enumerate(zip(CI, CO)):
        W, b = leaves[2 * l], leaves[2 * l + 1]
        g.append(W.grad.reshape(co, ci, 27).permute(0, 2, 1).reshape(-1))   # back to [co][tap][ci]
        g.append(b.grad)
    g.append(leaves[-2].grad)
    g.append(leaves[-1].grad.reshape(1))
    return float(loss.detach()), out.detach().numpy(), torch.cat(g).numpy()


def param_slices():
    """(name, slice) of each layer's weights and biases in the parameter vector."""
    names = ("e1a", "e1b", "e2a", "e2b", "e3a", "e3b", "d2a", "d2b", "d1a", "d1b")
    out = []
    o = 0
    for n, ci, co in zip(names, CI, CO):
        out.append((n + ".w", slice(o, o + co * 27 * ci)))
        o += co * 27 * ci
        out.append((n + ".b", slice(o, o + co)))
        o += co
    out.append(("last.w", slice(o, o + C1)))
    out.append(("last.b", slice(o + C1, o + C1 + 1)))
    return out
