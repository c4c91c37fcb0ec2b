"""Learned surrogate for smart interpolation.

A residual 3-D convolutional network predicts, for every voxel, the
probabilities of the label slots the random walk would give it. Its 16 input
channels are the normalised intensity, the signed distance to the nearest
labelled z-slice, a seed mask and one channel per label slot (1 on that
slot's seed voxels; at most 13 slots). It is trained on hit-probability maps
that this package's own walk produces (p_l = hits_l / sum hits), with every
layer's forward and backward pass, the loss and AdamW running as hand-written
CUDA kernels of libsmartinterp.so (bf16 activations and weights, fp32
accumulation on the tensor cores). The hybrid interpolation walks only the
seeds near voxels the network is unsure about and keeps the network's labels
elsewhere; the full plain walk stays the yardstick of its labels.

Network: stem conv 16 -> C, B residual blocks [conv C->C (dilation d), ReLU,
conv C->C (d), + skip, ReLU], head conv C -> 16 (logits, fp32). 3x3x3 kernels,
"same" padding. Default C = 16, dilations (1, 2, 4, 8): receptive field
+-32 voxels, 70 k parameters, 138 kFLOP per voxel.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as nat

BF16 = torch.bfloat16
IN_CH = 16
OUT_CH = 16
MAX_SLOTS = 13  # one-hot slot channels of the input


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _p(t):
    return None if t is None else t.data_ptr()


@dataclass
class Conv:
    cin: int
    cout: int
    dil: int
    w: torch.Tensor        # fp32 master [27][cout][cin]
    b: torch.Tensor        # fp32 [cout]
    wb: torch.Tensor       # bf16 working copy
    gw: torch.Tensor       # fp32 grads
    gb: torch.Tensor
    mw: torch.Tensor = None
    vw: torch.Tensor = None
    mb: torch.Tensor = None
    vb: torch.Tensor = None
    wf: torch.Tensor = None  # bf16 flipped copy for the data gradient


def umma_check():
    """Raises when a tensor-core convolution's bounded wait gave up since the
    last check (synchronises the current stream)."""
    import ctypes

    st = ctypes.c_int(0)
    nat.call("si_nn_umma_status", ctypes.byref(st), _stream())


def _tensor_core_ok(conv: Conv, tensor_core: bool) -> bool:
    return tensor_core and conv.cin == 16 and conv.cout == 16 and conv.dil <= 8


def conv_fwd(x, conv: Conv, shape, relu, residual=None, out_f32=False, tensor_core=False):
    """y = relu?(conv(x) + b + residual). tensor_core: the 16 -> 16 layers on
    the tcgen05 kernel (si_nn_conv16_tc) instead of mma.sync."""
    N, D, H, W = shape
    y = torch.empty((N, D, H, W, conv.cout), dtype=torch.float32 if out_f32 else BF16, device=x.device)
    if _tensor_core_ok(conv, tensor_core):
        nat.call("si_nn_conv16_tc", _p(x), _p(conv.wb), _p(conv.b), _p(residual), _p(y), N, D, H, W, conv.dil,
                 int(relu), int(out_f32), _stream())
    else:
        nat.call("si_nn_conv3d_fwd", _p(x), _p(conv.wb), _p(conv.b), _p(residual), _p(y), N, D, H, W, conv.cin,
                 conv.cout, conv.dil, int(relu), int(out_f32), _stream())
    return y


def conv_dgrad(dy, conv: Conv, shape, residual=None, tensor_core=False):
    """dX = conv(dY, W flipped) (+ residual added in the epilogue)."""
    N, D, H, W = shape
    if conv.wf is None:
        conv.wf = torch.empty_like(conv.wb)
    nat.call("si_nn_flip_weights", _p(conv.wb), _p(conv.wf), conv.cout, conv.cin, _stream())
    dx = torch.empty((N, D, H, W, conv.cin), dtype=BF16, device=dy.device)
    if _tensor_core_ok(conv, tensor_core):
        nat.call("si_nn_conv16_tc", _p(dy), _p(conv.wf), None, _p(residual), _p(dx), N, D, H, W, conv.dil, 0, 0,
                 _stream())
    else:
        nat.call("si_nn_conv3d_fwd", _p(dy), _p(conv.wf), None, _p(residual), _p(dx), N, D, H, W, conv.cout,
                 conv.cin, conv.dil, 0, 0, _stream())
    return dx


_PARTIALS: dict = {}


def _partials(shape, cin, cout, device):
    """Cached scratch for the deterministic 16-channel weight gradient."""
    import ctypes

    need = ctypes.c_uint64(0)
    nat.call("si_nn_wgrad_partial_bytes", *shape, cin, cout, ctypes.byref(need))
    key = str(device)
    buf = _PARTIALS.get(key)
    if buf is None or buf.numel() * 4 < need.value:
        buf = torch.empty((int(need.value) + 3) // 4, dtype=torch.float32, device=device)
        _PARTIALS[key] = buf
    return buf


def conv_wgrad(x, dy, conv: Conv, shape, deterministic=True):
    """Adds the weight and bias gradients of one convolution to conv.gw /
    conv.gb; 16 -> 16 convolutions reduce in a fixed order (deterministic)."""
    N, D, H, W = shape
    part, nbytes = None, 0
    if deterministic and conv.cin == 16 and conv.cout == 16:
        buf = _partials(shape, conv.cin, conv.cout, x.device)
        part, nbytes = buf.data_ptr(), buf.numel() * 4
    nat.call("si_nn_conv3d_wgrad", _p(x), _p(dy), _p(conv.gw), _p(conv.gb), N, D, H, W, conv.cin, conv.cout,
             conv.dil, part, nbytes, _stream())


def relu_bwd(g, y, add=None):
    nat.call("si_nn_relu_bwd", _p(g), _p(y), _p(add), g.numel(), _stream())


class SurrogateNet:
    """The network; parameters live on the current CUDA device."""

    def __init__(self, channels=16, dilations=(1, 2, 4, 8), seed=0, device=None, tensor_core=True):
        if channels not in (16, 32):
            raise ValueError("channels must be 16 or 32")
        self.device = torch.device(device) if device else torch.device("cuda", torch.cuda.current_device())
        self.channels, self.dilations = channels, tuple(dilations)
        # 16 -> 16 layers (forward and data gradient) on the tcgen05 kernel;
        # False: on mma.sync
        self.tensor_core = bool(tensor_core)
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.convs = [self._make(IN_CH, channels, 1, g)]
        for d in self.dilations:
            self.convs.append(self._make(channels, channels, d, g))
            self.convs.append(self._make(channels, channels, d, g))
        self.convs.append(self._make(channels, OUT_CH, 1, g, scale=0.1))
        self.step_count = 0

    def _make(self, cin, cout, dil, g, scale=1.0):
        std = scale * math.sqrt(2.0 / (27 * cin))
        w = (torch.randn((27, cout, cin), generator=g) * std).to(self.device)
        b = torch.zeros(cout, device=self.device)
        c = Conv(cin, cout, dil, w, b, w.to(BF16), torch.zeros_like(w), torch.zeros_like(b))
        c.mw, c.vw, c.mb, c.vb = (torch.zeros_like(w), torch.zeros_like(w), torch.zeros_like(b), torch.zeros_like(b))
        return c

    @property
    def radius(self) -> int:
        """Receptive-field radius in voxels (stem 1, 2 d per block, head 1)."""
        return 2 + 2 * sum(self.dilations)

    @property
    def flops_per_voxel(self) -> int:
        return sum(2 * 27 * c.cin * c.cout for c in self.convs)

    @property
    def n_params(self) -> int:
        return sum(c.w.numel() + c.b.numel() for c in self.convs)

    # ---- forward / backward -------------------------------------------------
    def forward(self, x, keep=False):
        """x: bf16 [N, D, H, W, 16] -> fp32 logits [N, D, H, W, 16]."""
        shape = tuple(x.shape[:4])
        acts = [x]
        tc = self.tensor_core
        a = conv_fwd(x, self.convs[0], shape, relu=True, tensor_core=tc)
        acts.append(a)
        for i in range(len(self.dilations)):
            c1, c2 = self.convs[1 + 2 * i], self.convs[2 + 2 * i]
            t = conv_fwd(a, c1, shape, relu=True, tensor_core=tc)
            a = conv_fwd(t, c2, shape, relu=True, residual=a, tensor_core=tc)
            acts += [t, a]
        logits = conv_fwd(a, self.convs[-1], shape, relu=False, out_f32=True, tensor_core=tc)
        if keep:
            self._acts, self._shape = acts, shape
        return logits

    def backward(self, dlogits):
        """Accumulates parameter gradients from bf16 dlogits (after forward(keep=True))."""
        acts, shape = self._acts, self._shape
        head = self.convs[-1]
        conv_wgrad(acts[-1], dlogits, head, shape)
        tc = self.tensor_core
        da = conv_dgrad(dlogits, head, shape, tensor_core=tc)
        for i in reversed(range(len(self.dilations))):
            c1, c2 = self.convs[1 + 2 * i], self.convs[2 + 2 * i]
            a_in, t, a_out = acts[1 + 2 * i], acts[2 + 2 * i], acts[3 + 2 * i]
            relu_bwd(da, a_out)                 # g = dL/d(pre-activation of the block output)
            conv_wgrad(t, da, c2, shape)
            dt = conv_dgrad(da, c2, shape, tensor_core=tc)
            relu_bwd(dt, t)
            conv_wgrad(a_in, dt, c1, shape)
            da = conv_dgrad(dt, c1, shape, residual=da, tensor_core=tc)  # conv1^T(dt) + g through the skip
        relu_bwd(da, acts[1])
        conv_wgrad(acts[0], da, self.convs[0], shape)
        self._acts = None

    def zero_grad(self):
        for c in self.convs:
            c.gw.zero_()
            c.gb.zero_()

    def adamw(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, wd=1e-4):
        self.step_count += 1
        for c in self.convs:
            nat.call("si_nn_adamw", _p(c.w), _p(c.gw), _p(c.mw), _p(c.vw), _p(c.wb), c.w.numel(), lr, beta1, beta2,
                     eps, wd, self.step_count, _stream())
            nat.call("si_nn_adamw", _p(c.b), _p(c.gb), _p(c.mb), _p(c.vb), None, c.b.numel(), lr, beta1, beta2,
                     eps, 0.0, self.step_count, _stream())

    def loss_and_grad(self, logits, target, weight, nol, extra_scale=1.0, denom=None):
        """Soft-target cross entropy, summed over voxels (times their weight)
        and divided by `denom` (default: the sum of the weights, which costs a
        device synchronisation); returns (loss tensor, bf16 dlogits scaled by
        extra_scale / denom)."""
        V = logits.numel() // OUT_CH
        dl = torch.empty(logits.shape, dtype=BF16, device=logits.device)
        loss = torch.zeros(1, dtype=torch.float32, device=logits.device)
        if denom is None:
            denom = float(weight.sum()) if weight is not None else float(V)
        denom = max(float(denom), 1.0)
        nat.call("si_nn_xent", _p(logits), _p(target), _p(weight), V, OUT_CH, nol, float(extra_scale) / denom, _p(dl),
                 _p(loss), _stream())
        return loss / denom, dl

    # ---- persistence --------------------------------------------------------
    _MOMENTS = ("mw", "vw", "mb", "vb")

    def state_dict(self):
        """Checkpoint: fp32 weights and biases, the AdamW moments and the step
        count (AdamW's bias correction), so training can resume where it
        stopped."""
        sd = {"channels": self.channels, "dilations": list(self.dilations), "step": self.step_count,
              "w": [c.w.cpu() for c in self.convs], "b": [c.b.cpu() for c in self.convs]}
        for m in self._MOMENTS:
            sd[m] = [getattr(c, m).cpu() for c in self.convs]
        return sd

    def load_state_dict(self, sd):
        """Loads a checkpoint. One without moments (weights only) restarts the
        optimiser: zero moments and step count 0, so AdamW's bias correction
        starts afresh too. A checkpoint with only some of the moments is
        refused."""
        have = [m for m in self._MOMENTS if m in sd]
        if have and len(have) != len(self._MOMENTS):
            raise ValueError(f"checkpoint holds only some AdamW moments ({', '.join(have)})")
        if len(sd["w"]) != len(self.convs):
            raise ValueError("checkpoint of a different network depth")
        for i, (c, w, b) in enumerate(zip(self.convs, sd["w"], sd["b"])):
            if tuple(w.shape) != tuple(c.w.shape) or tuple(b.shape) != tuple(c.b.shape):
                raise ValueError("checkpoint of a different network shape")
            c.w.copy_(w.to(self.device))
            c.b.copy_(b.to(self.device))
            c.wb.copy_(c.w.to(BF16))
            for m in self._MOMENTS:
                getattr(c, m).copy_(sd[m][i].to(self.device) if m in sd else torch.zeros_like(getattr(c, m)))
        self.step_count = int(sd.get("step", 0)) if have else 0


# ---------------------------------------------------------------------------
# Features and targets of one prepared job (DeviceJob after walk()).
# ---------------------------------------------------------------------------
def slice_distance(Zc: int, zs) -> np.ndarray:
    """Signed distance of every crop z to the nearest labelled z-slice."""
    z = np.arange(Zc)[:, None]
    zs = np.asarray(sorted(zs))
    if zs.size == 0:
        return np.full(Zc, 16.0, np.float32)
    d = z - zs[None, :]
    k = np.abs(d).argmin(1)
    return d[np.arange(Zc), k].astype(np.float32)


def slice_table(Zc: int, zs) -> np.ndarray:
    """float32 [Zc, 4] = (signed distance to the nearest labelled z-slice,
    labelled z-slice below or at z, labelled z-slice above z, weight of the
    one below); -1 marks a missing neighbour (its weight is then 0 or 1)."""
    zs = np.asarray(sorted(set(int(v) for v in zs)), np.int64)
    out = np.zeros((Zc, 4), np.float32)
    out[:, 0] = slice_distance(Zc, zs)
    for z in range(Zc):
        k = np.searchsorted(zs, z, side="right")
        lo = int(zs[k - 1]) if k > 0 else -1
        hi = int(zs[k]) if k < zs.size else -1
        if lo == z:
            hi = -1
        if lo >= 0 and hi >= 0:
            w = (hi - z) / (hi - lo)
        else:
            w = 1.0 if lo >= 0 else 0.0
        out[z] = (out[z, 0], lo, hi, w)
    return out


def slot_map_of(job) -> torch.Tensor:
    """int16 crop volume: the label slot of every seed voxel, -1 elsewhere
    (built from the job's seed records, so only/ignore and all-axis slices
    are those of the walk)."""
    from .interpolation import SEED_RECORD_BYTES

    cp = job.cplan
    full = torch.full((cp.voxels,), -1, dtype=torch.int16, device=job.dev)
    n = int(job.n_seeds.item())
    if n:
        rec = job.seeds[: n * SEED_RECORD_BYTES].view(torch.int32).view(n, 4)
        pos = rec[:, 0].to(torch.int64) & 0xFFFFFFFF
        full[pos] = (rec[:, 3] & 0xFF).to(torch.int16)
    return full.view(cp.Zc, cp.Yc, cp.Xc)


def features(job, z0=0, y0=0, x0=0, dims=None, slot_map=None) -> torch.Tensor:
    """bf16 [1, Dt, Ht, Wt, 16] features of a box of the job's crop (zero
    outside the crop)."""
    cp = job.cplan
    if job.work_is_float:
        raise ValueError("the surrogate takes uint8 volumes")
    Dt, Ht, Wt = dims if dims else (cp.Zc, cp.Yc, cp.Xc)
    if slot_map is None:
        slot_map = slot_map_of(job)
    zt = torch.from_numpy(slice_table(cp.Zc, [s for a, s in cp.slice_list.tolist() if a == 0])).to(job.dev)
    out = torch.empty((1, Dt, Ht, Wt, IN_CH), dtype=BF16, device=job.dev)
    nat.call("si_nn_features", _p(job.work), _p(slot_map), _p(zt), cp.Zc, cp.Yc, cp.Xc, z0, y0, x0, Dt, Ht, Wt,
             _p(out), _stream())
    return out


def hit_targets(job) -> tuple[torch.Tensor, torch.Tensor]:
    """Per-voxel label probabilities p_l = hits_l / sum_l hits over the crop
    ([Zc, Yc, Xc, nol] fp32) and a weight map (1 inside, 0 on the crop border).
    Voxels without hits take label slot 0 (the argmax rule of the walk)."""
    h = job.hits.to(torch.float32)  # [nol, Z, Y, X]
    s = h.sum(0, keepdim=True)
    p = torch.where(s > 0, h / s.clamp(min=1.0), torch.zeros_like(h))
    p[0] = torch.where(s[0] > 0, p[0], torch.ones_like(p[0]))
    w = torch.ones(h.shape[1:], dtype=torch.float32, device=h.device)
    w[0], w[-1], w[:, 0], w[:, -1], w[:, :, 0], w[:, :, -1] = 0, 0, 0, 0, 0, 0
    return p.permute(1, 2, 3, 0).contiguous(), w


# ---------------------------------------------------------------------------
# Inference in z-slabs
# ---------------------------------------------------------------------------
def predict(net: SurrogateNet, job, slab=None, slab_voxels=1 << 28) -> torch.Tensor:
    """Label-slot probabilities of the whole crop, [nol, Zc, Yc, Xc] fp32.

    The crop is processed in z-slabs over the full (Yc, Xc) planes, each with
    a halo of the network's receptive radius (cut at the crop faces), so the
    result equals one pass over the whole crop."""
    cp = job.cplan
    nol = job.lplan.nol
    if nol > MAX_SLOTS:
        raise ValueError(f"the surrogate handles at most {MAX_SLOTS} label slots")
    sm = slot_map_of(job)
    r = net.radius
    plane = cp.Yc * cp.Xc
    if slab is None:
        slab = max(8, slab_voxels // plane - 2 * r)
    probs = torch.empty((nol, cp.Zc, cp.Yc, cp.Xc), dtype=torch.float32, device=job.dev)
    for zs in range(0, cp.Zc, slab):
        ze = min(cp.Zc, zs + slab)
        a, b = max(0, zs - r), min(cp.Zc, ze + r)
        feats = features(job, a, 0, 0, (b - a, cp.Yc, cp.Xc), sm)
        logits = net.forward(feats)
        del feats
        nat.call("si_nn_probs", _p(logits), b - a, cp.Yc, cp.Xc, zs - a, ze - a, nol, _p(probs), cp.Zc, zs,
                 _stream())
        del logits
    umma_check()
    return probs


# ---------------------------------------------------------------------------
# Training on walk-generated targets
# ---------------------------------------------------------------------------
@dataclass
class Sample:
    feats: torch.Tensor   # bf16 [1, Zc, Yc, Xc, 16]
    target: torch.Tensor  # fp32 [Zc, Yc, Xc, nol]
    weight: torch.Tensor  # fp32 [Zc, Yc, Xc]
    nol: int


def make_sample(img, lab, nbrw=10, sorw=4000, rng_seed=None):
    """Walks one volume with the plain method and returns its features and
    hit-probability targets (None if the volume has no labelled slices)."""
    from .interpolation import DEFAULT_RNG_SEED, DeviceJob, _IMG_DTYPES, _LAB_DTYPES, normalize_host_dtypes, upload

    d, l = normalize_host_dtypes(np.asarray(img), np.asarray(lab))
    ti, tl = upload(d, l)
    job = DeviceJob(ti, _IMG_DTYPES[d.dtype], tl, _LAB_DTYPES[l.dtype], nbrw=nbrw, sorw=sorw,
                    rng_seed=DEFAULT_RNG_SEED if rng_seed is None else rng_seed)
    if d.dtype != np.uint8 or job.analyze() is not None:
        return None
    job.prepare()
    job.walk()
    p, w = hit_targets(job)
    return Sample(features(job), p, w, job.lplan.nol)


def training_set(n, shape=(96, 96, 96), nbrw=10, sorw=4000, seed=0, mix=0.5):
    """n training samples: procedural volumes (synthetic.procedural_volume)
    and, for a fraction `mix`, volumes in the style of the large workload
    (synthetic.large_volume: 6 phases, noise 12, labels every 12th z-slice)."""
    from .synthetic import large_volume, procedural_volume

    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        if rng.random() < mix:
            img, lab, _ = large_volume(seed=int(rng.integers(1 << 30)), shape=shape, z_every=int(rng.integers(8, 15)))
            lab = lab.astype(np.int32)
        else:
            img, lab, _ = procedural_volume(rng, shape)
        smp = make_sample(img, lab, nbrw, sorw)
        if smp is not None and smp.nol <= MAX_SLOTS and min(smp.target.shape[:3]) >= 48:
            out.append(smp)
    return out


def _slot_permutation(rng, nol):
    """Random placement of a sample's label slots 1..nol-1 among the slot
    channels 1..MAX_SLOTS-1: (feature channel order, target channel of each
    slot). Slot 0 keeps channel 0: it is the walk's answer for voxels that no
    walk reaches, a rule the network can only learn if it can tell slot 0."""
    perm = np.concatenate([[0], 1 + rng.permutation(MAX_SLOTS - 1)])
    src = np.arange(IN_CH)
    for k in range(MAX_SLOTS):
        src[3 + perm[k]] = 3 + k
    return src, perm[:nol]


def train(net: SurrogateNet, samples, steps, batch=4, patch=96, lr=2e-3, seed=0, log_every=0, permute=True,
          warmup=200):
    """AdamW on random windows (patch^3, clipped to the smallest sample) with
    a linear learning-rate warmup over `warmup` steps and cosine decay. With `permute`, each window's label slots are
    moved to random slot channels (inputs and targets alike), so that the
    network learns the same rule for every slot; the loss then runs over all
    MAX_SLOTS channels. Returns the loss per step."""
    rng = np.random.default_rng(seed)
    patch = min([patch] + [min(smp.target.shape[:3]) for smp in samples])
    losses = []
    for step in range(steps):
        picks = [samples[int(rng.integers(len(samples)))] for _ in range(batch)]
        feats, tgts = [], []
        for smp in picks:
            Z, Y, X = smp.target.shape[:3]
            z, y, x = (int(rng.integers(0, d - patch + 1)) for d in (Z, Y, X))
            f = smp.feats[:, z:z + patch, y:y + patch, x:x + patch]
            t = smp.target[z:z + patch, y:y + patch, x:x + patch]
            w = smp.weight[z:z + patch, y:y + patch, x:x + patch].contiguous()
            if permute:
                src, dst = _slot_permutation(rng, smp.nol)
                f = f[..., torch.from_numpy(src).to(f.device)]
                t13 = torch.zeros(t.shape[:3] + (MAX_SLOTS,), dtype=t.dtype, device=t.device)
                t13[..., torch.from_numpy(dst).to(t.device)] = t
                tgts.append((t13, w, MAX_SLOTS))
            else:
                tgts.append((t.contiguous(), w, smp.nol))
            feats.append(f)
        xb = torch.cat(feats).contiguous()
        logits = net.forward(xb, keep=True)
        dls, tot = [], torch.zeros(1, dtype=torch.float32, device=xb.device)
        for k, (t, w, nol) in enumerate(tgts):
            loss, dl = net.loss_and_grad(logits[k:k + 1].contiguous(), t, w, nol, extra_scale=1.0 / batch,
                                         denom=patch ** 3)
            dls.append(dl)
            tot += loss / batch
        net.zero_grad()
        net.backward(torch.cat(dls).contiguous())
        ramp = min(1.0, (step + 1) / warmup) if warmup else 1.0
        net.adamw(lr=lr * ramp * 0.5 * (1 + math.cos(math.pi * step / max(steps, 1))))
        losses.append(tot)
        if log_every and step % log_every == 0:
            print(f"step {step}: loss {float(tot):.4f}", flush=True)
    umma_check()
    return [float(v) for v in losses]


def agreement(net: SurrogateNet, smp: Sample) -> dict:
    """Surrogate vs walk on one sample: voxel agreement of the argmax, mean
    cross entropy to the hit fractions and the hit fractions' own entropy."""
    logits = net.forward(smp.feats)[0, ..., : smp.nol]
    logq = torch.log_softmax(logits, -1)
    p, w = smp.target, smp.weight
    ws = w.sum().clamp(min=1)
    xent = float((-(p * logq).sum(-1) * w).sum() / ws)
    ent = float((-(p * torch.log(p.clamp(min=1e-12))).sum(-1) * w).sum() / ws)
    agree = float(((logits.argmax(-1) == p.argmax(-1)).float() * w).sum() / ws)
    return {"agree": agree, "xent": xent, "entropy": ent}


def save(net: SurrogateNet, path):
    torch.save(net.state_dict(), path)


def load(path, device=None) -> SurrogateNet:
    sd = torch.load(path, map_location="cpu")
    net = SurrogateNet(channels=sd["channels"], dilations=tuple(sd["dilations"]), device=device)
    net.load_state_dict(sd)
    return net


# ---------------------------------------------------------------------------
# Hybrid interpolation
# ---------------------------------------------------------------------------
def seeds_near(job, mask: torch.Tensor, radius: int, coarse: int = 8) -> torch.Tensor:
    """Boolean per seed record: the seed lies within about `radius` voxels
    (Chebyshev distance, rounded up to whole cells of `coarse`^3 voxels) of a
    voxel set in `mask` ([Zc, Yc, Xc] bool)."""
    import torch.nn.functional as Fnn

    from .interpolation import SEED_RECORD_BYTES

    cp = job.cplan
    u = Fnn.max_pool3d(mask[None, None].to(torch.float16), coarse, stride=coarse, ceil_mode=True)
    r = max(1, int(math.ceil(radius / coarse)))
    near = Fnn.max_pool3d(u, 2 * r + 1, stride=1, padding=r)[0, 0] > 0
    n = int(job.n_seeds.item())
    rec = job.seeds[: n * SEED_RECORD_BYTES].view(torch.int32).view(n, 4)
    pos = rec[:, 0].to(torch.int64) & 0xFFFFFFFF
    plane = cp.Yc * cp.Xc
    return near[pos // plane // coarse, (pos // cp.Xc) % cp.Yc // coarse, pos % cp.Xc // coarse]


def hybrid_interpolation(img, lab, net: SurrogateNet, nbrw=10, sorw=4000, smooth=0, threshold=0.97, radius=16,
                         coarse=4, grow=2, rng_seed=None, device_inputs=None, keep_maps=False, smooth_update="f32"):
    """Surrogate probabilities everywhere; the plain walk only from the seeds
    within about `radius` voxels of a voxel whose largest probability is below
    `threshold`, grown by `grow` voxels (the uncertain voxels; the seed
    search dilates them on a grid of `coarse`^3 cells); on the uncertain
    voxels that some walk reached, the walk's hit fractions replace the
    surrogate's probabilities. Labels are the argmax of the combined maps
    (and of their smoothed copy when smooth > 0), remapped like the plain
    method's. Returns (dict of device label volumes, stats)."""
    from . import interpolation as I
    from .interpolation import (DEFAULT_RNG_SEED, DeviceJob, SEED_RECORD_BYTES, _IMG_DTYPES, _LAB_DTYPES,
                                normalize_host_dtypes, upload, walk_sorted)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if device_inputs is None:
        d, l = normalize_host_dtypes(np.asarray(img), np.asarray(lab))
        if d.dtype != np.uint8:
            raise ValueError("the surrogate takes uint8 volumes")
        ti, tl = upload(d, l)
        icode, lcode = _IMG_DTYPES[d.dtype], _LAB_DTYPES[l.dtype]
    else:
        ti, icode, tl, lcode = device_inputs
    job = DeviceJob(ti, icode, tl, lcode, nbrw=nbrw, sorw=sorw, smooth=smooth,
                    rng_seed=DEFAULT_RNG_SEED if rng_seed is None else rng_seed)
    msg = job.analyze()
    if msg:
        raise ValueError(msg)
    job.prepare()
    cp, nol = job.cplan, job.lplan.nol
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    probs = predict(net, job)
    unsure = probs.amax(0) < threshold
    if grow > 0:
        import torch.nn.functional as Fnn

        unsure = Fnn.max_pool3d(unsure[None, None].to(torch.float16), 2 * grow + 1, stride=1,
                                padding=grow)[0, 0] > 0
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    keep = seeds_near(job, unsure, radius, coarse)
    n_seeds = int(job.n_seeds.item())
    rec = job.seeds[: n_seeds * SEED_RECORD_BYTES].view(torch.int32).view(n_seeds, 4)
    kept = rec[keep].contiguous()
    n_keep = int(kept.shape[0])
    hits = torch.zeros((nol, cp.Zc, cp.Yc, cp.Xc), dtype=torch.int32, device=job.dev)
    sweeps = 0
    ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    ev[0].record()
    if n_keep:
        cnt = torch.tensor([n_keep], dtype=torch.int32, device=job.dev)
        sweeps = walk_sorted(job.packed, False, cp.Zc, cp.Yc, cp.Xc, kept.view(torch.uint8).reshape(-1), cnt, n_keep,
                             nbrw, sorw, job.rng_seed, hits, nol)
    ev[1].record()
    del kept
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    # combined maps: hit fractions on uncertain voxels that some walk reached
    hs = hits.sum(0, dtype=torch.int32)
    use = unsure & (hs > 0)
    inv = 1.0 / hs.clamp(min=1).to(torch.float32)
    for k in range(nol):
        probs[k] = torch.where(use, hits[k].to(torch.float32) * inv, probs[k])
    del hits, hs, inv
    res = {}
    res["regular"], _ = job._labels_from(probs, True, False)
    if smooth:
        tmp0, tmp1 = I.smooth_buffers(cp.Zc, cp.Yc, cp.Xc, job.dev)
        nat.call("si_smooth_f32", _p(probs), _p(tmp0), _p(tmp1), nol, cp.Zc, cp.Yc, cp.Xc, smooth,
                 I.SMOOTH_UPDATES[smooth_update], _stream())
        I.smooth_check()
        res["smooth"], _ = job._labels_from(probs, True, False)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    stats = {"seconds_prepare": t1 - t0, "seconds_surrogate": t2 - t1, "seconds_walk": t3 - t2,
             "seconds_post": t4 - t3, "seconds_total": t4 - t0, "frac_uncertain": float(unsure.float().mean()),
             "frac_walked_voxels": float(use.float().mean()), "seeds_walked": n_keep, "seeds_total": n_seeds,
             "frac_seeds_walked": n_keep / max(n_seeds, 1), "walker_steps": n_keep * nbrw * sorw,
             "sweeps": sweeps, "nol": nol, "walk_ms_events": ev[0].elapsed_time(ev[1])}
    if keep_maps:
        res["use"] = use
    return res, stats


def label_dice(a: torch.Tensor, b: torch.Tensor, labels):
    """Per-label Dice of two label volumes (device tensors)."""
    out = {}
    for lv in labels:
        ma, mb = a == int(lv), b == int(lv)
        den = int(ma.sum()) + int(mb.sum())
        out[int(lv)] = 1.0 if den == 0 else 2.0 * int((ma & mb).sum()) / den
    return out
