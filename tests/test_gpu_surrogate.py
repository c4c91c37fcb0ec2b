"""Surrogate network kernels against the float64 oracle (gradient check), and
a short training run whose loss must fall."""
import numpy as np
import pytest
import torch

import nn_oracle as NO
from biomedisa_gb300 import surrogate as S

pytestmark = pytest.mark.gpu


def _bf(a, dev):
    return torch.from_numpy(np.asarray(a, np.float32)).to(dev).to(torch.bfloat16)


def _np(t):
    return t.float().cpu().numpy().astype(np.float64)


def _conv(cin, cout, dil, rng, dev):
    w = NO.bf16_round(rng.standard_normal((27, cout, cin)) * 0.2)
    b = rng.standard_normal(cout) * 0.1
    wt = torch.from_numpy(w.astype(np.float32)).to(dev)
    c = S.Conv(cin, cout, dil, wt, torch.from_numpy(b.astype(np.float32)).to(dev), wt.to(torch.bfloat16),
               torch.zeros_like(wt), torch.zeros(cout, device=dev))
    return c, w, b


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("cin,cout,dil,shape", [
    (16, 16, 1, (2, 7, 9, 11)), (16, 16, 3, (1, 5, 6, 70)), (16, 16, 8, (2, 9, 4, 129)), (16, 32, 1, (2, 7, 9, 11)),
    (32, 32, 2, (2, 7, 9, 11)), (32, 16, 4, (2, 7, 9, 11)), (32, 32, 1, (2, 7, 9, 11))])
def test_conv_forward_dgrad_wgrad(cin, cout, dil, shape, cuda):
    """16 -> 16 runs the dedicated C = 16 kernel (rows of 64 voxels: W = 70 and
    129 leave partial chunks); the others the generic kernel."""
    rng = np.random.default_rng(cin * 7 + cout + dil)
    x = NO.bf16_round(rng.standard_normal(shape + (cin,)))
    c, w, b = _conv(cin, cout, dil, rng, cuda)
    xt = _bf(x, cuda)
    # forward (fp32 output: only accumulation order differs)
    y = S.conv_fwd(xt, c, shape, relu=False, out_f32=True)
    exp = NO.conv_fwd(x, w, b, dil)
    assert np.max(np.abs(_np(y) - exp)) <= 1e-4 * max(1.0, np.abs(exp).max())
    # forward bf16 with residual + relu
    res = NO.bf16_round(rng.standard_normal(shape + (cout,)))
    yb = S.conv_fwd(xt, c, shape, relu=True, residual=_bf(res, cuda))
    expb = NO.bf16_round(np.maximum(exp + res, 0))
    assert np.max(np.abs(_np(yb) - expb) / (np.abs(expb) + 1e-2)) <= 2 ** -7
    # data gradient through the flipped weights
    dy = NO.bf16_round(rng.standard_normal(shape + (cout,)))
    dx = S.conv_dgrad(_bf(dy, cuda), c, shape)
    assert _rel(_np(dx), NO.conv_dgrad(dy, w, dil)) < 1e-2
    # weight and bias gradients (fp32)
    c.gw.zero_()
    c.gb.zero_()
    S.conv_wgrad(xt, _bf(dy, cuda), c, shape)
    assert _rel(c.gw.cpu().numpy().astype(np.float64), NO.conv_wgrad(x, dy, dil)) < 1e-5
    assert _rel(c.gb.cpu().numpy().astype(np.float64), dy.reshape(-1, cout).sum(0)) < 1e-5


@pytest.mark.parametrize("dil,shape", [(1, (1, 3, 4, 300)), (2, (2, 5, 3, 257)), (8, (1, 4, 6, 128)),
                                       (4, (3, 2, 2, 1)), (1, (2, 4, 70, 130)), (2, (2, 40, 20, 200))])
@pytest.mark.parametrize("streams", [1, 2, 4])
def test_conv16_tensor_core_rows(dil, shape, streams, cuda):
    """The 16 -> 16 convolution on the tcgen05 tensor cores (si_nn_conv16_tc)
    in tiles of 128 voxels of an x-row (partial last tiles, rows shorter than
    a tile, columns of 70 rows that wrap the accumulator rings of 32, 16 or 8
    positions per stream and the 10-slot row ring, several columns per CTA):
    forward with bias,
    residual and ReLU, and the data gradient, against the float64 oracle and
    the mma.sync path; with 1, 2 and 4 interleaved column streams per CTA."""
    from biomedisa_gb300 import _native as nat
    nat.call("si_nn_conv16_tc_set_streams", streams)
    try:
        _conv16_tc_case(dil, shape, cuda)
    finally:
        nat.call("si_nn_conv16_tc_set_streams", 1)


def _conv16_tc_case(dil, shape, cuda):
    rng = np.random.default_rng(dil * 31 + shape[-1])
    x = NO.bf16_round(rng.standard_normal(shape + (16,)))
    c, w, b = _conv(16, 16, dil, rng, cuda)
    xt = _bf(x, cuda)
    y = S.conv_fwd(xt, c, shape, relu=False, out_f32=True, tensor_core=True)
    exp = NO.conv_fwd(x, w, b, dil)
    assert np.max(np.abs(_np(y) - exp)) <= 1e-4 * max(1.0, np.abs(exp).max())
    res = NO.bf16_round(rng.standard_normal(shape + (16,)))
    yb = S.conv_fwd(xt, c, shape, relu=True, residual=_bf(res, cuda), tensor_core=True)
    expb = NO.bf16_round(np.maximum(exp + res, 0))
    assert np.max(np.abs(_np(yb) - expb) / (np.abs(expb) + 1e-2)) <= 2 ** -7
    dy = NO.bf16_round(rng.standard_normal(shape + (16,)))
    dx = S.conv_dgrad(_bf(dy, cuda), c, shape, tensor_core=True)
    assert _rel(_np(dx), NO.conv_dgrad(dy, w, dil)) < 1e-2
    # the mma.sync path gives the same fp32 sums up to accumulation order
    ym = S.conv_fwd(xt, c, shape, relu=False, out_f32=True)
    assert np.max(np.abs(_np(ym) - _np(y))) <= 1e-5 * max(1.0, np.abs(exp).max())
    _umma_ok()


def _umma_ok():
    import ctypes
    from biomedisa_gb300 import _native as nat
    st = ctypes.c_int(0)
    nat.call("si_nn_umma_status", ctypes.byref(st), torch.cuda.current_stream().cuda_stream)


def test_conv16_tensor_core_wait_runs_out(cuda):
    """With the wait limit at 0 spins the tensor-core convolution's waits give
    up at once: the kernel lets its copies and MMAs complete, frees its tensor
    memory, and the status reports it; with the default limit restored the
    same convolution is correct on the same context."""
    import ctypes
    from biomedisa_gb300 import _native as nat
    rng = np.random.default_rng(4)
    shape = (1, 3, 3, 200)
    x = NO.bf16_round(rng.standard_normal(shape + (16,)))
    c, w, b = _conv(16, 16, 1, rng, cuda)
    xt = _bf(x, cuda)
    stream = torch.cuda.current_stream().cuda_stream
    nat.call("si_set_wait_limit", 0)
    try:
        S.conv_fwd(xt, c, shape, relu=False, out_f32=True, tensor_core=True)
        st = ctypes.c_int(0)
        rc = nat.lib().si_nn_umma_status(ctypes.byref(st), ctypes.c_void_p(stream))
        assert rc == 2 and st.value == 1
    finally:
        nat.call("si_set_wait_limit", -1)
    y = S.conv_fwd(xt, c, shape, relu=False, out_f32=True, tensor_core=True)
    exp = NO.conv_fwd(x, w, b, 1)
    assert np.max(np.abs(_np(y) - exp)) <= 1e-4 * max(1.0, np.abs(exp).max())
    _umma_ok()


@pytest.mark.parametrize("channels", [16, 32])
def test_network_gradient_check(channels, cuda):
    """Whole network (stem, 2 residual blocks, head): loss, logits and every
    layer's weight/bias gradient against the oracle."""
    rng = np.random.default_rng(5)
    net = S.SurrogateNet(channels=channels, dilations=(1, 2), seed=3)
    for c in net.convs:  # bf16-exact master weights so both sides start equal
        c.w.copy_(c.wb.float())
    shape = (1, 8, 10, 9)
    x = NO.bf16_round(rng.uniform(0, 1, shape + (16,)) * (rng.random(shape + (16,)) < 0.5))
    nol = 3
    p = rng.dirichlet(np.ones(nol), size=shape)
    wgt = (rng.random(shape) < 0.9).astype(np.float64)
    logits = net.forward(_bf(x, cuda), keep=True)
    loss, dl = net.loss_and_grad(logits, torch.from_numpy(p.astype(np.float32)).to(cuda),
                                 torch.from_numpy(wgt.astype(np.float32)).to(cuda), nol)
    net.zero_grad()
    net.backward(dl)
    ws = [c.w.cpu().numpy().astype(np.float64) for c in net.convs]
    bs = [c.b.cpu().numpy().astype(np.float64) for c in net.convs]
    e_loss, e_logits, dws, dbs = NO.network_grads(x, ws, bs, list(net.dilations), p, wgt, nol)
    assert abs(float(loss) - e_loss) <= 1e-3 * abs(e_loss) + 1e-6
    assert _rel(_np(logits), e_logits) < 1e-2
    for k, c in enumerate(net.convs):
        assert _rel(c.gw.cpu().numpy().astype(np.float64), dws[k]) < 3e-2, f"layer {k} dW"
        assert _rel(c.gb.cpu().numpy().astype(np.float64), dbs[k]) < 3e-2, f"layer {k} db"


def test_training_is_deterministic(cuda):
    """The 16-channel weight and bias gradients reduce in a fixed order, so two
    training runs from the same seed end with identical weights."""
    rng = np.random.default_rng(2)
    x = torch.from_numpy(rng.uniform(0, 1, (2, 12, 12, 70, 16)).astype(np.float32)).to(cuda).to(torch.bfloat16)
    p = torch.from_numpy(rng.dirichlet(np.ones(3), size=(2, 12, 12, 70)).astype(np.float32)).to(cuda)
    ws = []
    for _ in range(2):
        net = S.SurrogateNet(seed=4)
        for _ in range(3):
            logits = net.forward(x, keep=True)
            _, dl = net.loss_and_grad(logits, p, None, 3)
            net.zero_grad()
            net.backward(dl)
            net.adamw(lr=1e-3)
        ws.append(torch.cat([c.w.flatten() for c in net.convs] + [c.b for c in net.convs]))
    assert torch.equal(ws[0], ws[1])


def test_training_reduces_loss(cuda):
    """AdamW on a fixed batch: the loss falls below 60 % of its start in 60 steps."""
    rng = np.random.default_rng(8)
    net = S.SurrogateNet(channels=16, dilations=(1, 2), seed=1)
    shape = (2, 16, 16, 16)
    x = rng.uniform(0, 1, shape + (16,))
    x[..., 4:] = 0
    lab = (x[..., 0] > 0.5).astype(np.int64)
    nol = 2
    p = np.eye(nol)[lab]
    xt = _bf(x, cuda)
    pt = torch.from_numpy(p.astype(np.float32)).to(cuda)
    losses = []
    for _ in range(60):
        logits = net.forward(xt, keep=True)
        loss, dl = net.loss_and_grad(logits, pt, None, nol)
        net.zero_grad()
        net.backward(dl)
        net.adamw(lr=5e-3)
        losses.append(float(loss))
    assert losses[-1] < 0.6 * losses[0], losses


def _job(img, lab, dev):
    from biomedisa_gb300.interpolation import DeviceJob, _IMG_DTYPES, _LAB_DTYPES, upload
    ti, tl = upload(img, lab, device=dev)
    job = DeviceJob(ti, _IMG_DTYPES[img.dtype], tl, _LAB_DTYPES[lab.dtype])
    assert job.analyze() is None
    job.prepare()
    return job


def test_features_and_slot_map(cuda):
    """Feature channels against a NumPy restatement; the slot map comes from
    the seed records (every labelled-slice voxel of a plain volume)."""
    from biomedisa_gb300 import synthetic as syn
    img, lab, _ = syn.plain_volume(seed=2, shape=(40, 36, 44), z_every=7, semi=(6, 14))
    job = _job(img, lab, cuda)
    cp = job.cplan
    sm = S.slot_map_of(job).cpu().numpy()
    f = S.features(job, -3, 2, -1, (cp.Zc + 4, cp.Yc - 3, cp.Xc)).float().cpu().numpy()[0]
    work = job.work.view(cp.Zc, cp.Yc, cp.Xc).cpu().numpy()
    zs = sorted(s for a, s in cp.slice_list.tolist() if a == 0)
    tab = S.slice_table(cp.Zc, zs)
    exp = np.zeros_like(f)
    exp[..., 1] = 1.0
    ys, xs = slice(2, 2 + f.shape[1]), slice(0, cp.Xc - 1)
    for zt in range(f.shape[0]):
        z = zt - 3
        if not 0 <= z < cp.Zc:
            continue
        exp[zt, :, 1:, 0] = work[z, ys, xs] / 255.0
        exp[zt, :, 1:, 1] = np.clip(tab[z, 0] / 16.0, -1, 1)
        exp[zt, :, 1:, 2] = sm[z, ys, xs] >= 0
        lo, hi, w = int(tab[z, 1]), int(tab[z, 2]), float(tab[z, 3])
        slo = sm[lo, ys, xs] if lo >= 0 else np.full((f.shape[1], cp.Xc - 1), -1)
        shi = sm[hi, ys, xs] if hi >= 0 else np.full((f.shape[1], cp.Xc - 1), -1)
        for k in range(13):
            exp[zt, :, 1:, 3 + k] = np.float32(w) * (slo == k) + np.float32(1 - w) * (shi == k)
    assert np.max(np.abs(f - NO.bf16_round(exp))) == 0.0
    # seeds: every voxel of a labelled z-slice inside the volume (the crop
    # of this small volume spans the one-voxel padding frame too)
    for z in zs:
        assert (sm[z, 1:-1, 1:-1] >= 0).all() and (sm[z, 0] == -1).all() and (sm[z, :, -1] == -1).all()
    assert (sm[[z for z in range(cp.Zc) if z not in zs]] == -1).all()


def test_slab_inference_matches_single_pass(cuda):
    """z-slabs with a receptive-radius halo reproduce one pass over the crop bit for bit."""
    from biomedisa_gb300 import synthetic as syn
    img, lab, _ = syn.plain_volume(seed=4, shape=(70, 40, 48), z_every=9, semi=(8, 16))
    job = _job(img, lab, cuda)
    net = S.SurrogateNet(channels=16, dilations=(1, 2, 4, 8), seed=2)
    whole = S.predict(net, job, slab=job.cplan.Zc)
    for slab in (5, 17, 33):
        part = S.predict(net, job, slab=slab)
        assert torch.equal(part, whole), slab
    assert torch.allclose(whole.sum(0), torch.ones_like(whole[0]), atol=1e-5)


def test_hybrid_gain_over_untrained(cuda):
    """What the network gains: after a short training run on walked volumes
    (32 samples, 1000 steps) the hybrid walks fewer than all of the seeds of a
    held-out 256^3 volume and still agrees with the plain walk (per-label
    Dice >= 0.99), while an untrained network is unsure everywhere and saves
    nothing. (The benchmark's network, trained longer, walks far fewer.)"""
    from biomedisa_gb300 import synthetic as syn
    from biomedisa_gb300.interpolation import DeviceJob, _IMG_DTYPES, _LAB_DTYPES, normalize_host_dtypes, upload
    img, lab, _ = syn.large_volume(seed=5, shape=(256, 256, 256), z_every=12)
    d, l = normalize_host_dtypes(img, lab)
    ti, tl = upload(d, l, device=cuda)
    dev_in = (ti, _IMG_DTYPES[d.dtype], tl, _LAB_DTYPES[l.dtype])
    job = DeviceJob(*dev_in)
    assert job.analyze() is None
    job.prepare()
    job.walk()
    plain = job.post()["regular"]
    present = sorted(int(v) for v in np.unique(lab[::12]))
    untrained = S.SurrogateNet(seed=1)
    res0, st0 = S.hybrid_interpolation(None, None, untrained, device_inputs=dev_in)
    assert st0["frac_seeds_walked"] > 0.95
    assert min(S.label_dice(res0["regular"], plain, present).values()) > 0.999
    net = S.SurrogateNet(seed=1)
    S.train(net, S.training_set(32, mix=0.8, seed=3), 1000, seed=3)
    # this briefly trained network is confidently wrong on parts of the small
    # label 1 (31.6 k voxels): the 0.99 gate needs a wide margin around the
    # uncertain voxels (measured: threshold 0.97 / grow 2 / radius 16 walks 59 %
    # at Dice 0.976; 0.99 / 4 / 24 walks 86 % at 0.993)
    res, st = S.hybrid_interpolation(None, None, net, device_inputs=dev_in, threshold=0.99, grow=4, radius=24)
    dice = S.label_dice(res["regular"], plain, present)
    print("hybrid", st["frac_seeds_walked"], st["frac_uncertain"], dice)
    assert st["frac_seeds_walked"] < 0.90
    assert st["walker_steps"] < 0.90 * job.total_steps()
    assert min(dice.values()) >= 0.99


def test_smooth_f32_matches_oracle(cuda):
    """si_smooth_f32 (smoothing of the hybrid's float probability maps) equals
    the oracle's smoothing of the same maps bit for bit."""
    import oracle as O
    from biomedisa_gb300 import _native as nat
    rng = np.random.default_rng(9)
    maps = rng.random((3, 19, 23, 37)).astype(np.float32)
    maps[:, 5:9] *= 4.0
    t = torch.from_numpy(maps.copy()).to(cuda)
    from biomedisa_gb300.interpolation import smooth_buffers, smooth_check
    tmp0, tmp1 = smooth_buffers(19, 23, 37, cuda)
    for iters in (1, 4):
        t.copy_(torch.from_numpy(maps))
        nat.call("si_smooth_f32", t.data_ptr(), tmp0.data_ptr(), tmp1.data_ptr(), 3, 19, 23, 37, iters, 0,
                 torch.cuda.current_stream().cuda_stream)
        smooth_check()
        assert np.array_equal(t.cpu().numpy(), O.smooth(maps, iters, "f32")), iters


def test_hybrid_smooth_and_keys(cuda):
    """The hybrid with smoothing returns regular and smooth label volumes of
    the input shape; an untrained network walks every seed, so on every voxel
    a walk reached its regular result equals the plain walk's."""
    from biomedisa_gb300 import smart_interpolation
    from biomedisa_gb300.synthetic import plain_volume
    img, lab, _ = plain_volume(seed=3, shape=(40, 44, 48), z_every=6, semi=(7, 14))
    net = S.SurrogateNet(seed=2)
    res, st = S.hybrid_interpolation(img, lab, net, nbrw=3, sorw=100, smooth=3)
    plain = smart_interpolation(img, lab, nbrw=3, sorw=100, return_hits=True)
    assert set(res) >= {"regular", "smooth"} and res["smooth"].shape == img.shape
    assert st["frac_seeds_walked"] == 1.0
    reached = plain["hits"].sum(0) > 0
    assert reached.mean() > 0.5
    assert np.array_equal(res["regular"].cpu().numpy()[reached], plain["regular"][reached])


def test_network_tensor_core_matches_mma(cuda):
    """SurrogateNet(tensor_core=True) runs its 16 -> 16 layers on tcgen05: its
    logits and weight gradients match the mma.sync network's."""
    rng = np.random.default_rng(12)
    shape = (1, 10, 12, 140)
    x = torch.from_numpy(rng.uniform(0, 1, shape + (16,)).astype(np.float32)).to(cuda).to(torch.bfloat16)
    p = torch.from_numpy(rng.dirichlet(np.ones(3), size=shape).astype(np.float32)).to(cuda)
    out = []
    for tc in (False, True):
        net = S.SurrogateNet(seed=6, tensor_core=tc)
        logits = net.forward(x, keep=True)
        _, dl = net.loss_and_grad(logits, p, None, 3)
        net.zero_grad()
        net.backward(dl)
        out.append((_np(logits), [c.gw.cpu().numpy().astype(np.float64) for c in net.convs]))
    assert _rel(out[1][0], out[0][0]) < 1e-2
    for k in range(len(out[0][1])):
        assert _rel(out[1][1][k], out[0][1][k]) < 3e-2, k
    _umma_ok()
