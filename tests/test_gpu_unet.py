"""The U-Net's tensor-core kernels (tcgen05 implicit-GEMM convolutions, pooling, upsampling,
concatenation, loss, Adam) against torch's CPU conv3d / autograd in FP32 on small shapes: the
forward pass, every parameter gradient of the backward pass, and a training run that fits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    return t


def bf(t, x):
    """round to BF16 (what the device stores) and back to FP32"""
    return x.to(t.bfloat16).to(t.float32)


def torch_unet(t, net, params, x, nx, ny, nz, bf16_acts=True):
    """The same network in torch (FP32, CPU): weights / inputs rounded to BF16 like the device,
    activations rounded to BF16 after each layer. Returns the output [B][V][16] and the weight
    tensors (leaves for autograd)."""
    F = t.nn.functional
    L, c = net.levels, net.base
    ch = [c << l for l in range(L)]
    shapes = net.layer_shapes()
    W, Bs, o = [], [], 0
    for (co, taps, ci) in shapes:
        w = t.tensor(params[o:o + co * taps * ci]).reshape(co, taps, ci)
        o += co * taps * ci
        b = t.tensor(params[o:o + co])
        o += co
        k = 3 if taps == 27 else 1
        wt = bf(t, w).permute(0, 2, 1).reshape(co, ci, k, k, k).contiguous().requires_grad_(True)
        bt = b.clone().requires_grad_(True)
        W.append(wt)
        Bs.append(bt)
    B = x.shape[0]

    def rnd(v):
        # BF16 rounding in the forward value, identity in the backward pass
        return v + (bf(t, v.detach()) - v.detach()) if bf16_acts else v

    h = rnd(t.tensor(x).reshape(B, nz, ny, nx, 16).permute(0, 4, 1, 2, 3))
    li = 0

    def conv(h, relu=True):
        nonlocal li
        w, b = W[li], Bs[li]
        li += 1
        y = F.conv3d(h, w, b, padding=w.shape[-1] // 2)
        return rnd(F.relu(y) if relu else y)

    skips = []
    for l in range(L):
        if l > 0:
            h = rnd(F.avg_pool3d(skips[-1], 2))
        h = conv(h)
        h = conv(h)
        skips.append(h)
    h = skips[-1]
    for l in range(L - 2, -1, -1):
        up = F.interpolate(h, scale_factor=2, mode="nearest")
        h = t.cat([skips[l], up], dim=1)
        h = conv(h)
        h = conv(h)
    w, b = W[li], Bs[li]
    y = F.conv3d(h, w, b)
    return y.permute(0, 2, 3, 4, 1).reshape(B, nx * ny * nz, 16), W, Bs


@pytest.mark.parametrize("levels,base,shape,batch", [(1, 16, (16, 8, 4), 1), (2, 16, (16, 8, 4), 2),
                                                     (4, 16, (32, 16, 8), 2), (3, 32, (32, 24, 8), 1)])
def test_unet_forward_and_gradients_match_torch(torch, levels, base, shape, batch):
    from panslbm2_gb300.surrogate import UNet
    t = torch
    nx, ny, nz = shape
    net = UNet(nx, ny, nz, levels, base, max_batch=batch)
    try:
        rng = np.random.default_rng(levels * 7 + base)
        params = net.get_params()
        params[:] = params + 0.01 * rng.standard_normal(params.size).astype(np.float32)   # non-zero biases too
        net.set_params(params)
        x = rng.standard_normal((batch, nx * ny * nz, 16)).astype(np.float32)
        y = net.forward(x)
        yt, W, Bs = torch_unet(t, net, params, x, nx, ny, nz)
        ref = yt.detach().numpy()
        err = np.max(np.abs(y - ref)) / np.max(np.abs(ref))
        assert err < 2e-2, "forward: max |GPU - torch| / max |torch| = %.3e" % err
        # backward of L = sum(dy * y)
        dy = rng.standard_normal(y.shape).astype(np.float32)
        g = net.backward(dy)
        (yt * t.tensor(dy)).sum().backward()
        o = 0
        worst = 0.0
        for (co, taps, ci), w, b in zip(net.layer_shapes(), W, Bs):
            gw = g[o:o + co * taps * ci].reshape(co, taps, ci)
            o += co * taps * ci
            gb = g[o:o + co]
            o += co
            k = w.shape[-1]
            tw = w.grad.reshape(co, ci, k ** 3).permute(0, 2, 1).numpy()
            ew = np.linalg.norm(gw - tw) / max(np.linalg.norm(tw), 1e-30)
            eb = np.linalg.norm(gb - b.grad.numpy()) / max(np.linalg.norm(b.grad.numpy()), 1e-30)
            cw = float(np.sum(gw * tw) / max(np.linalg.norm(gw) * np.linalg.norm(tw), 1e-30))
            worst = max(worst, ew, eb)
            # the device rounds every gradient tensor to BF16 (8-bit mantissa); the error grows
            # along the backward chain (about 14 roundings deep at the first encoder layer of
            # the 4-level network) and where a weight gradient sums few voxels (the 4 x 2 x 1
            # bottom level): measured up to 11 % there, below 5 % elsewhere. A layout or indexing
            # error gives O(1) errors and cosines far from 1.
            assert ew < 0.2 and eb < 0.2 and cw > 0.98, ((co, taps, ci), ew, eb, cw)
    finally:
        net.close()


def test_unet_trains_on_a_smooth_map(torch):
    """fit targets that are smooth functions of the design: under the cosine learning-rate decay the
    last epoch's loss is below 15% of the first's (60 epochs measured 13.6% on GB300; this runs 120)"""
    from panslbm2_gb300.surrogate import UNet
    nx, ny, nz = 32, 16, 8
    net = UNet(nx, ny, nz, 3, 16, max_batch=2)
    try:
        rng = np.random.default_rng(5)
        n = nx * ny * nz
        ns = 8
        net.reserve(ns, 3)
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        feat = np.stack([i.ravel() / nx, j.ravel() / ny, k.ravel() / nz], 1).astype(np.float32)
        net.set_static(feat)
        from scipy.ndimage import gaussian_filter
        for s in range(ns):
            d = rng.random((nz, ny, nx))
            sm = gaussian_filter(d, 1.5, mode="nearest")
            tg = np.stack([sm.ravel(), (sm ** 2).ravel() * 3.0, sm.ravel() * feat[:, 0]])
            net.add_sample(s, d.ravel(), tg)
        loss = net.train(ns, 120, batch=2, lr=2e-3, seed=1)
        assert np.all(np.isfinite(loss))
        assert loss[-1] < 0.15 * loss[0], loss
        assert loss[-1] < loss[len(loss) // 2], loss
        pred = net.predict(rng.random(n))
        assert pred.shape == (3, n) and np.all(np.isfinite(pred))
    finally:
        net.close()
