"""PyTorch FP32 reference of the proposal network (test infrastructure): the forward pass and the
gradients of the loss by autograd on the CPU, with the device path's bf16 rounding points
emulated (weights, activations and the pre-activation gradients rounded to bf16, sums in FP32),
so that the CUDA kernels are compared at FP32 accumulation-order level.

Layout of the parameters (rlf_cnn_param_count floats): per convolution W[32][9 cin] with
k = (3 ky + kx) cin + ci, then b[32]; the head's W[4][512] (feature (4 y + x) 32 + c), then b[4].
"""
import numpy as np
import torch
import torch.nn.functional as F

CIN = (4, 32, 32, 32)


def param_blocks():
    blocks, off = [], 0
    for cin in CIN:
        blocks.append(("w", off, (32, 9 * cin)))
        off += 32 * 9 * cin
        blocks.append(("b", off, (32,)))
        off += 32
    blocks.append(("hw", off, (4, 512)))
    off += 4 * 512
    blocks.append(("hb", off, (4,)))
    off += 4
    return blocks, off


def bf16(x):
    return x.to(torch.bfloat16).to(torch.float32)


def bf16_bits_to_f32(bits):
    return (np.asarray(bits, np.uint32) << 16).view(np.float32)


def f32_to_bf16_bits(x):
    """round to nearest even bf16, as bit patterns"""
    return torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)


def init_params(rng, scale=1.0):
    blocks, n = param_blocks()
    p = np.zeros(n, np.float32)
    for kind, off, shape in blocks:
        size = int(np.prod(shape))
        if kind in ("w", "hw"):
            fan_in = shape[1]
            p[off:off + size] = rng.standard_normal(size) * scale * np.sqrt(2.0 / fan_in)
        else:
            p[off:off + size] = rng.standard_normal(size) * 0.05
    return p


def forward_backward(params, images_bits, targets):
    """images_bits: [n][64][64][4] uint16 bf16 patterns; targets [n][3].  Returns (out [n][4],
    loss, grads in the parameter layout)."""
    blocks, n_par = param_blocks()
    P = torch.tensor(params, dtype=torch.float32, requires_grad=True)
    x = torch.from_numpy(bf16_bits_to_f32(images_bits)).permute(0, 3, 1, 2).contiguous()  # NCHW
    rnd = lambda g: bf16(g)
    k = 0
    for l, cin in enumerate(CIN):
        _, wo, ws = blocks[2 * l]
        _, bo, _ = blocks[2 * l + 1]
        w = P[wo:wo + ws[0] * ws[1]].reshape(32, 3, 3, cin).permute(0, 3, 1, 2)
        w = w + (bf16(w.detach()) - w.detach())  # bf16 values, gradient of the FP32 master weights
        pre = F.conv2d(x, w, P[bo:bo + 32], stride=2, padding=1)
        pre.register_hook(rnd)
        y = torch.relu(pre)
        x = y + (bf16(y.detach()) - y.detach())
    feat = x.permute(0, 2, 3, 1).reshape(x.shape[0], 512)
    _, hwo, _ = blocks[-2]
    _, hbo, _ = blocks[-1]
    out = feat @ P[hwo:hwo + 2048].reshape(4, 512).T + P[hbo:hbo + 4]
    t = torch.from_numpy(np.asarray(targets, np.float32))
    ls = torch.clamp(out[:, 3], -5.0, 0.5)
    iv = torch.exp(-2.0 * ls)
    r2 = (out[:, 0] - t[:, 0]) ** 2 + (out[:, 1] - t[:, 1]) ** 2
    d3 = out[:, 2] - t[:, 2]
    loss = torch.mean(0.5 * r2 * iv + 2.0 * ls + 0.5 * d3 * d3)
    loss.backward()
    return out.detach().numpy(), float(loss.detach()), P.grad.numpy().copy()
