"""torch-CPU restatement of the U-Net of libpps (the oracle of its gradients).

Same layers, order and parameter layout as pps_unet.cu: per layer W[27][cin][cout]
(tap = kz*9 + ky*3 + kx) then b[cout]; convolutions are zero-padded 3x3x3
cross-correlations, pooling is a 2x average, up-sampling is 2x nearest, and the skip
concatenations put the up-sampled tensor first."""
import numpy as np
import torch
import torch.nn.functional as F


def layer_specs(c1, c2, c3):
    return [(1, c1, True), (c1, c1, True), (c1, c2, True), (c2, c2, True), (c2, c3, True), (c3, c3, True),
            (c3 + c2, c2, True), (c2, c2, True), (c2 + c1, c1, True), (c1, c1, True), (c1, 1, False)]


def unflatten(params, channels, dtype=torch.float64, bf16_weights=False):
    out, off = [], 0
    for cin, cout, _ in layer_specs(*channels):
        n = 27 * cin * cout
        W = torch.tensor(np.asarray(params[off:off + n], np.float32).reshape(27, cin, cout))
        if bf16_weights:
            W = W.to(torch.bfloat16).to(torch.float32)
        off += n
        b = torch.tensor(np.asarray(params[off:off + cout], np.float32))
        off += cout
        w = W.reshape(3, 3, 3, cin, cout).permute(4, 3, 0, 1, 2).contiguous().to(dtype).requires_grad_(True)
        out.append((w, b.to(dtype).requires_grad_(True)))
    return out


def flatten_grads(layers):
    g = []
    for w, b in layers:
        cout, cin = w.shape[0], w.shape[1]
        g.append(w.grad.permute(2, 3, 4, 1, 0).reshape(27 * cin * cout).detach().numpy())
        g.append(b.grad.detach().numpy())
    return np.concatenate(g)


def forward(layers, x):
    """x: (nz, ny, nx) tensor -> output (nz, ny, nx)."""
    def conv(i, t, relu=True):
        w, b = layers[i]
        y = F.conv3d(t, w, b, padding=1)
        return F.relu(y) if relu else y
    t = x[None, None]
    e1 = conv(1, conv(0, t))
    e2 = conv(3, conv(2, F.avg_pool3d(e1, 2)))
    e3 = conv(5, conv(4, F.avg_pool3d(e2, 2)))
    d2 = conv(7, conv(6, torch.cat([F.interpolate(e3, scale_factor=2, mode="nearest"), e2], dim=1)))
    d1 = conv(9, conv(8, torch.cat([F.interpolate(d2, scale_factor=2, mode="nearest"), e1], dim=1)))
    return conv(10, d1, relu=False)[0, 0]


def loss_and_grads(params, channels, x, target, bf16_weights=True):
    layers = unflatten(params, channels, bf16_weights=bf16_weights)
    out = forward(layers, torch.tensor(x, dtype=torch.float64))
    loss = torch.mean((out - torch.tensor(target, dtype=torch.float64)) ** 2)
    loss.backward()
    return float(loss.detach()), flatten_grads(layers), out.detach().numpy()
