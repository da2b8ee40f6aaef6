"""CPU oracle of the learned initial guess's network (test infrastructure only).

The same net as the library's learned.cu, in torch on the CPU: four 3x3x3
convolutions of 16 channels (dilations 1, 2, 4, 8, zero padding, ReLU) and a
1x1x1 convolution to one channel, mean-squared-error loss.  The library stores
weights and activations in BF16 and accumulates in FP32; the oracle rounds the
same quantities to BF16 and computes everything else in FP32, so outputs and
gradients agree to the BF16 rounding of the intermediate tensors.

Parameter vector layout (the library's): for each 3x3x3 layer W[co][tap][ci]
(tap = (dz+1)*9 + (dy+1)*3 + (dx+1)) then b[co]; then the 1x1x1 weights w[ci]
and bias b.  The first layer's input has one channel; the library stores it as
16 channels of which 15 are zero, so only W[:, :, 0] of layer 0 acts.
"""
import numpy as np

C = 16
LAYERS = 4
DIL = (1, 2, 4, 8)
WCONV = C * 27 * C
NPARAMS = LAYERS * (WCONV + C) + C + 1


def bf16(t):
    import torch
    return t.to(torch.bfloat16).to(torch.float32)


def unpack(p):
    """Parameter vector -> list of (W (co, ci, 3, 3, 3), b) and (w_last, b_last) as torch tensors."""
    import torch
    p = torch.as_tensor(np.asarray(p, np.float32))
    convs = []
    o = 0
    for _ in range(LAYERS):
        W = p[o:o + WCONV].reshape(C, 27, C)               # [co][tap][ci]
        W = W.permute(0, 2, 1).reshape(C, C, 3, 3, 3)      # (co, ci, kz, ky, kx)
        o += WCONV
        b = p[o:o + C]
        o += C
        convs.append((W, b))
    return convs, p[o:o + C], p[o + C]


def forward(p, x, requires_grad=False):
    """x: (D, H, W) input.  Returns output (D, H, W) and the leaf tensors."""
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
    a = bf16(torch.as_tensor(np.asarray(x, np.float32)))[None, None]   # (1, 1, D, H, W)
    for l, (W, b) in enumerate(convs):
        Wq = bf16(W)
        if l == 0:
            Wq = Wq[:, :1]
        a = F.conv3d(a, Wq, b, padding=DIL[l], dilation=DIL[l])
        a = F.relu(a)
        # activations are stored in BF16 (rounding seen as identity by the gradient)
        a = a + (bf16(a) - a).detach()
    out = (a[0] * wl[:, None, None, None]).sum(0) + bl
    return out, leaves


def loss_and_grad(p, x, t):
    """MSE loss and its gradient with respect to the parameter vector."""
    import torch
    out, leaves = forward(p, x, requires_grad=True)
    tt = torch.as_tensor(np.asarray(t, np.float32))
    loss = ((out - tt) ** 2).mean()
    loss.backward()
    g = []
    for l in range(LAYERS):
        W, b = leaves[2 * l], leaves[2 * l + 1]
        g.append(W.grad.reshape(C, C, 27).permute(0, 2, 1).reshape(-1))   # back to [co][tap][ci]
        g.append(b.grad)
    g.append(leaves[-2].grad)
    g.append(leaves[-1].grad.reshape(1))
    return float(loss), out.detach().numpy(), torch.cat(g).numpy()
