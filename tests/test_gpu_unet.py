"""The learned preconditioner's kernels (no reference counterpart), checked against
CPU restatements: the U-Net's forward output and its parameter gradients against
torch-CPU autograd in float64 (tests/unet_reference.py; the GPU network runs BF16
activations and weights, hence the tolerances), the 2x grid transfers against
numpy, and a short GPU training run that must lower the loss."""
import numpy as np
import pytest

import parallelpoissonsolver_gb300 as pps

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def test_unet_forward_and_gradients_match_cpu_autograd(gpu):
    import unet_reference as R
    ch = (16, 32, 64)
    net = pps.UNet(ch, seed=7)
    params = net.get_params()
    rng = np.random.default_rng(1)
    shape = (8, 12, 16)
    x = rng.standard_normal(shape).astype(np.float32)
    t = rng.standard_normal(shape).astype(np.float32)
    xd, td, od = dev(x), dev(t), dev(np.zeros(shape))
    net.forward(shape, xd.data_ptr(), od.data_ptr(), normalize=False)
    torch.cuda.synchronize()
    loss_ref, g_ref, out_ref = R.loss_and_grads(params, ch, x, t)
    out = od.cpu().numpy()
    assert np.linalg.norm(out - out_ref) <= 0.03 * np.linalg.norm(out_ref)
    loss, g = net.gradients(shape, xd.data_ptr(), td.data_ptr())
    assert abs(loss - loss_ref) <= 0.02 * loss_ref
    cos = float(np.dot(g, g_ref) / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    assert cos > 0.995, cos
    assert np.linalg.norm(g - g_ref) <= 0.06 * np.linalg.norm(g_ref)
    # per layer, the biggest tensors agree too
    off = 0
    for cin, cout, _ in R.layer_specs(*ch):
        n = 27 * cin * cout + cout
        a, b = g[off:off + n], g_ref[off:off + n]
        assert np.linalg.norm(a - b) <= 0.1 * np.linalg.norm(b) + 1e-6
        off += n
    net.close()


def test_unet_training_lowers_the_loss(gpu):
    net = pps.UNet((16, 32, 64), seed=3)
    shape = (16, 16, 16)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(shape).astype(np.float32)
    t = np.roll(x, 1, axis=2) * 0.5                      # a learnable linear map
    xd, td = dev(x), dev(t)
    losses = [net.train_step(shape, xd.data_ptr(), td.data_ptr(), 3e-3) for _ in range(60)]
    assert losses[-1] < 0.3 * losses[0], (losses[0], losses[-1])
    p = net.get_params()
    net2 = pps.UNet((16, 32, 64), seed=99)
    net2.set_params(p)
    assert np.array_equal(net2.get_params(), p)
    net.close()
    net2.close()


def np_restrict(fine, nc):
    w = np.array([0.25, 0.5, 0.25])
    fz, fy, fx = fine.shape
    pad = np.zeros((fz + 1, fy + 1, fx + 1))
    pad[:fz, :fy, :fx] = fine
    out = np.zeros(nc)
    for a in range(3):
        for b in range(3):
            for c in range(3):
                out += w[a] * w[b] * w[c] * pad[a:a + 2 * nc[0]:2, b:b + 2 * nc[1]:2, c:c + 2 * nc[2]:2]
    return out


def test_grid_transfers(gpu):
    rng = np.random.default_rng(9)
    nc = (5, 6, 7)
    fine = rng.standard_normal((2 * nc[0], 2 * nc[1], 2 * nc[2]))
    fd, cd = dev(fine), dev(np.zeros(nc))
    pps.restrict2(nc, fd.data_ptr(), cd.data_ptr())
    got = cd.cpu().numpy()
    assert np.allclose(got, np_restrict(fine, nc), rtol=1e-5, atol=1e-6)
    # prolongation is the transpose of restriction up to a factor 8: <R f, c> = <f, P c>/8
    coarse = rng.standard_normal(nc)
    cd2, fd2 = dev(coarse), dev(np.zeros(fine.shape))
    pps.prolong2(nc, cd2.data_ptr(), fd2.data_ptr())
    pf = fd2.cpu().numpy()
    assert abs(np.sum(np_restrict(fine, nc) * coarse) - np.sum(fine * pf) / 8) < 1e-4 * np.sum(np.abs(fine * pf))
    # prolongating a trilinear function reproduces it away from the far boundary
    z, y, x = np.meshgrid(*[np.arange(1, n + 1) * 2.0 for n in nc], indexing="ij")
    lin = z + 2 * y - x
    cd3, fd3 = dev(lin), dev(np.zeros(fine.shape))
    pps.prolong2(nc, cd3.data_ptr(), fd3.data_ptr())
    pf3 = fd3.cpu().numpy()
    Z, Y, X = np.meshgrid(*[np.arange(1, 2 * n + 1) * 1.0 for n in nc], indexing="ij")
    ref = Z + 2 * Y - X
    inner = (slice(1, -1),) * 3
    assert np.allclose(pf3[inner], ref[inner], atol=1e-4)
