"""Learned reconstruction: the U-Net of tvk_paint_learned, its training on
frame pairs the plain renderer makes, and its evaluation.

Every computation runs in libtvk.so's kernels (the tvk_cnn_* C ABI: tensor-core
3x3 convolutions forward / backward-data / backward-weights, pooling,
upsampling, the pixel-shuffle head, MSE and Adam).  PyTorch only holds device
buffers and orders the calls on its current stream.

The network (also fixed in the C ABI, include/tvk.h): input = the reduced frame
(half resolution, half sample rate) as RGBA + 12 zero channels; a 4-level
U-Net; the head's 16 channels are RGBA x 2x2 sub-pixels added to the bilinear
upscale of the reduced frame, so a zero head reproduces the reference's
progressive low-resolution frame exactly.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from pathlib import Path

import numpy as np

from . import _native as N
from ._native import check, lib

# name, c1, c2, cout, LeakyReLU slope (-1: none); the order of tvk_learned_create
ARCH = [("e0a", 16, 0, 32, 0.1), ("e0b", 32, 0, 32, 0.1), ("e1a", 32, 0, 48, 0.1),
        ("e1b", 48, 0, 48, 0.1), ("e2a", 48, 0, 64, 0.1), ("e2b", 64, 0, 64, 0.1),
        ("b", 64, 0, 64, 0.1), ("d2", 64, 64, 64, 0.1), ("d1", 64, 48, 48, 0.1),
        ("d0", 48, 32, 32, 0.1), ("head", 32, 0, 16, -1.0)]
WEIGHTS = Path(__file__).resolve().parent / "weights" / "recon_unet.npz"


def param_count():
    return sum(9 * cout * (c1 + c2) + cout for _, c1, c2, cout, _ in ARCH)


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


class UNet:
    """Weights, Adam state and the forward/backward passes over torch buffers."""

    def __init__(self, torch, params=None, seed=0):
        self.torch = torch
        rng = np.random.default_rng(seed)
        self.layers = {}
        for name, c1, c2, cout, slope in ARCH:
            cin = c1 + c2
            if params is not None:
                w, b = params[name]
            else:
                lim = math.sqrt(6.0 / (9 * cin))
                w = rng.uniform(-lim, lim, size=(9, cout, cin)).astype(np.float32)
                b = np.zeros(cout, dtype=np.float32)
                if name == "head":  # start at the bilinear upscale
                    w[:] = 0
            dev = "cuda"
            L = {"c1": c1, "c2": c2, "cout": cout, "cin": cin, "slope": slope,
                 "w": torch.tensor(np.asarray(w, np.float32), device=dev),
                 "b": torch.tensor(np.asarray(b, np.float32), device=dev)}
            for k in ("w", "b"):
                L["m" + k] = torch.zeros_like(L[k])
                L["v" + k] = torch.zeros_like(L[k])
                L["d" + k] = torch.zeros_like(L[k])
            L["wf"] = torch.empty((9, cout, cin), dtype=torch.bfloat16, device=dev)
            L["wb"] = torch.empty((9, cin, cout), dtype=torch.bfloat16, device=dev)
            self.layers[name] = L
        self.t = 0
        self.refresh()

    # ---- plumbing
    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def refresh(self):
        for L in self.layers.values():
            check(lib().tvk_cnn_weights_bf16(_p(L["w"]), L["cout"], L["cin"], _p(L["wf"]),
                                             _p(L["wb"]), self.stream()))

    def params(self):
        return {n: (L["w"].cpu().numpy(), L["b"].cpu().numpy()) for n, L in self.layers.items()}

    def flat(self):
        return np.concatenate([np.concatenate([L["w"].cpu().numpy().reshape(-1),
                                               L["b"].cpu().numpy()])
                               for L in (self.layers[n] for n, *_ in ARCH)]).astype(np.float32)

    def save(self, path=WEIGHTS, **meta):
        path = Path(path)
        path.parent.mkdir(parents=True, exist_ok=True)
        arrays = {}
        for n, (w, b) in self.params().items():
            arrays[n + "_w"], arrays[n + "_b"] = w, b
        np.savez_compressed(path, **arrays, meta=np.array(repr(meta)))

    @staticmethod
    def load_params(path=WEIGHTS):
        d = np.load(path)
        return {n: (d[n + "_w"], d[n + "_b"]) for n, *_ in ARCH}

    # ---- kernels
    def _conv(self, name, x1, x2, n, h, w, y_bf16=None, y_f32=None, up=None):
        """up = (h1, w1): x1 is the coarser level's output, read through the
        convolution's clamped 2x upsampling."""
        L = self.layers[name]
        a = N.CnnConv(x1=_p(x1), x2=_p(x2), c1=L["c1"], c2=L["c2"], n=n, h=h, w=w,
                      weights=_p(L["wf"]), bias=_p(L["b"]), cout=L["cout"], slope=L["slope"],
                      y_bf16=_p(y_bf16), y_f32=_p(y_f32), y2_f32=None, split=L["cout"],
                      accumulate=0, upsample1=1 if up else 0, h1=up[0] if up else 0,
                      w1=up[1] if up else 0)
        check(lib().tvk_cnn_conv3x3(C.byref(a), self.stream()))

    def _new(self, n, h, w, c, dtype=None):
        t = self.torch
        return t.empty((n, h, w, c), dtype=dtype or t.bfloat16, device="cuda")

    def forward(self, x16, base):
        """x16: BF16 [n][h][w][16]; base: FP32 [n][2h][2w][4] -> FP32 output."""
        n, h, w, _ = x16.shape
        S = {"x": x16}

        def conv(name, a, b, hh, ww, up=None):
            y = self._new(n, hh, ww, self.layers[name]["cout"])
            self._conv(name, S[a], S[b] if b else None, n, hh, ww, y_bf16=y, up=up)
            S[name] = y

        def pool(src, dst, hh, ww):
            c = S[src].shape[3]
            S[dst] = self._new(n, hh // 2, ww // 2, c)
            check(lib().tvk_cnn_avgpool2(_p(S[src]), n, hh, ww, c, _p(S[dst]), self.stream()))

        conv("e0a", "x", None, h, w)
        conv("e0b", "e0a", None, h, w)
        pool("e0b", "p0", h, w)
        conv("e1a", "p0", None, h // 2, w // 2)
        conv("e1b", "e1a", None, h // 2, w // 2)
        pool("e1b", "p1", h // 2, w // 2)
        conv("e2a", "p1", None, h // 4, w // 4)
        conv("e2b", "e2a", None, h // 4, w // 4)
        pool("e2b", "p2", h // 4, w // 4)
        conv("b", "p2", None, h // 8, w // 8)
        # decoder layers read the coarser level upsampled on the fly
        conv("d2", "b", "e2b", h // 4, w // 4, up=(h // 8, w // 8))
        conv("d1", "d2", "e1b", h // 2, w // 2, up=(h // 4, w // 4))
        conv("d0", "d1", "e0b", h, w, up=(h // 2, w // 2))
        hd = self._new(n, h, w, 16, self.torch.float32)
        self._conv("head", S["d0"], None, n, h, w, y_f32=hd)
        S["head"] = hd
        out = self.torch.empty_like(base)
        check(lib().tvk_cnn_head(_p(hd), _p(base), n, h, w, _p(out), self.stream()))
        self.S, self.shape = S, (n, h, w)
        return out

    def _back(self, name, dy, inputs, hh, ww, need_dx=True):
        """Weight gradients of layer `name` and the FP32 gradients of its inputs."""
        t = self.torch
        L = self.layers[name]
        n = self.shape[0]
        S = self.S
        g = self._new(n, hh, ww, L["cout"])
        y = S[name] if name != "head" else None
        check(lib().tvk_cnn_act_grad(_p(dy), _p(y), L["slope"], _p(g), dy.numel(), self.stream()))
        x1 = S[inputs[0]]
        x2 = S[inputs[1]] if len(inputs) > 1 else None
        wg = N.CnnWgrad(x1=_p(x1), x2=_p(x2), c1=L["c1"], c2=L["c2"], gy=_p(g), n=n, h=hh, w=ww,
                        cout=L["cout"], dw=_p(L["dw"]), db=_p(L["db"]))
        check(lib().tvk_cnn_conv3x3_wgrad(C.byref(wg), self.stream()))
        if not need_dx:
            return []
        dx1 = t.empty((n, hh, ww, L["c1"]), dtype=t.float32, device="cuda")
        dx2 = t.empty((n, hh, ww, L["c2"]), dtype=t.float32, device="cuda") if L["c2"] else None
        a = N.CnnConv(x1=_p(g), x2=None, c1=L["cout"], c2=0, n=n, h=hh, w=ww,
                      weights=_p(L["wb"]), bias=None, cout=L["cin"], slope=-1.0, y_bf16=None,
                      y_f32=_p(dx1), y2_f32=_p(dx2), split=L["c1"] if L["c2"] else L["cin"],
                      accumulate=0)
        check(lib().tvk_cnn_conv3x3(C.byref(a), self.stream()))
        return [dx1] + ([dx2] if dx2 is not None else [])

    def backward(self, dout):
        t = self.torch
        n, h, w = self.shape
        st = self.stream()
        if h % 8 or w % 8:
            raise ValueError("training sizes must be multiples of 8")
        S = self.S
        # the decoders' upsampled inputs, which the weight gradients read
        for src, dst, hh, ww in (("b", "u2", h // 8, w // 8), ("d2", "u1", h // 4, w // 4),
                                 ("d1", "u0", h // 2, w // 2)):
            c = S[src].shape[3]
            S[dst] = t.empty((n, 2 * hh, 2 * ww, c), dtype=t.bfloat16, device="cuda")
            check(lib().tvk_cnn_upsample2(_p(S[src]), n, hh, ww, c, _p(S[dst]), st))
        dh = t.empty((n, h, w, 16), dtype=t.float32, device="cuda")
        check(lib().tvk_cnn_head_backward(_p(dout), n, h, w, _p(dh), st))

        def upb(d, hh, ww, c):
            o = t.empty((n, hh // 2, ww // 2, c), dtype=t.float32, device="cuda")
            check(lib().tvk_cnn_upsample2_backward(_p(d), n, hh // 2, ww // 2, c, _p(o), st))
            return o

        def poolb(d, target, hh, ww, c):
            check(lib().tvk_cnn_avgpool2_backward(_p(d), n, hh, ww, c, _p(target), 1, st))

        (dd0,) = self._back("head", dh, ["d0"], h, w)
        du0, ds0 = self._back("d0", dd0, ["u0", "e0b"], h, w)
        du1, ds1 = self._back("d1", upb(du0, h, w, 48), ["u1", "e1b"], h // 2, w // 2)
        du2, ds2 = self._back("d2", upb(du1, h // 2, w // 2, 64), ["u2", "e2b"], h // 4, w // 4)
        (dp2,) = self._back("b", upb(du2, h // 4, w // 4, 64), ["p2"], h // 8, w // 8)
        poolb(dp2, ds2, h // 4, w // 4, 64)
        (da2,) = self._back("e2b", ds2, ["e2a"], h // 4, w // 4)
        (dp1,) = self._back("e2a", da2, ["p1"], h // 4, w // 4)
        poolb(dp1, ds1, h // 2, w // 2, 48)
        (da1,) = self._back("e1b", ds1, ["e1a"], h // 2, w // 2)
        (dp0,) = self._back("e1a", da1, ["p0"], h // 2, w // 2)
        poolb(dp0, ds0, h, w, 32)
        (da0,) = self._back("e0b", ds0, ["e0a"], h, w)
        self._back("e0a", da0, ["x"], h, w, need_dx=False)

    def zero_grad(self):
        for L in self.layers.values():
            L["dw"].zero_()
            L["db"].zero_()

    def step(self, lr, b1=0.9, b2=0.999, eps=1e-8):
        self.t += 1
        for L in self.layers.values():
            for k in ("w", "b"):
                check(lib().tvk_cnn_adam(_p(L[k]), _p(L["d" + k]), _p(L["m" + k]),
                                         _p(L["v" + k]), L[k].numel(), lr, b1, b2, eps, self.t,
                                         self.stream()))
        self.refresh()

    def loss(self, out, target, with_grad=True):
        t = self.torch
        acc = t.zeros(1, dtype=t.float32, device="cuda")
        dout = t.empty_like(out) if with_grad else None
        check(lib().tvk_cnn_mse(_p(out), _p(target), out.numel(), _p(dout), _p(acc),
                                self.stream()))
        return acc, dout


def prepare_input(torch, low, depth=None):
    """Reduced RGBA frame [h][w][4] and its first-hit depth [h][w] (FP32,
    device) -> BF16 input [1][hp][wp][16]."""
    h, w = low.shape[0], low.shape[1]
    hp, wp = (h + 7) // 8 * 8, (w + 7) // 8 * 8
    x = torch.empty((1, hp, wp, 16), dtype=torch.bfloat16, device="cuda")
    check(lib().tvk_cnn_prepare_input(_p(low), _p(depth) if depth is not None else None, h, w,
                                      hp, wp, _p(x),
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return x


# ------------------------------------------------------------------ data


def random_bands_tf(rng, n=4096):
    """A perturbed version of the two-band TF: 1 to 3 opaque bands with random
    centres, widths, colours and opacities; alpha 0 elsewhere."""
    i = np.arange(n, dtype=np.float64)
    t = np.zeros((n, 4), dtype=np.float32)
    for _ in range(int(rng.integers(1, 4))):
        centre = rng.uniform(0.2, 0.85) * n
        half = rng.uniform(0.01, 0.04) * n
        ramp = rng.uniform(0.3, 1.0) * half
        a = np.clip((half - np.abs(i - centre)) / ramp, 0.0, 1.0) * rng.uniform(0.5, 0.95)
        m = a > t[:, 3]
        col = rng.uniform(0.15, 1.0, 3)
        t[m, 0], t[m, 1], t[m, 2] = col
        t[:, 3] = np.maximum(t[:, 3], a)
    return t


TRAIN_VOLUMES = [  # (size, seed): 8 seeded volumes of 256^3 .. 1024^3, 12-bit in u16
    (256, 11), (384, 12), (512, 13), (512, 14), (640, 15), (768, 16), (896, 17), (1024, 18)]


def make_training_volume(torch, size, seed):
    from .renderer import Volume, generate_volume_device
    from .workloads import PLAIN_LARGE_LIT as W
    rng = np.random.default_rng(seed)
    dims = (size, size, size)
    scale = size / 1024.0
    blobs = np.zeros((256, 7), dtype=np.float32)
    for a in range(3):
        blobs[:, a] = rng.uniform(0, size, 256)
    blobs[:, 3] = rng.uniform(16 * scale, 80 * scale, 256)
    blobs[:, 4] = rng.uniform(512, 3584, 256)
    raw = torch.empty(size ** 3 * 2, dtype=torch.uint8, device="cuda")
    generate_volume_device(raw.data_ptr(), dims, np.uint16, blobs, W.noise_amp,
                           W.noise_octaves, W.noise_cell * scale, seed, 0, W.vmax)
    torch.cuda.synchronize()
    vol = Volume(raw.data_ptr(), brick_size=W.brick_size, overlap=W.overlap, dims=dims,
                 dtype=np.uint16)
    del raw
    return vol


def random_camera(rng):
    r = rng.uniform(1.1, 2.4)
    az = rng.uniform(0, 2 * math.pi)
    el = rng.uniform(-math.radians(70), math.radians(70))
    eye = (r * math.cos(el) * math.sin(az), r * math.sin(el), r * math.cos(el) * math.cos(az))
    at = tuple(rng.uniform(-0.15, 0.15, 3))
    return eye, at


def configure_lit(r, vol, tf, width=1920, height=1080, srm=1.5):
    from .workloads import PLAIN_LARGE_LIT as W
    r.RegisterDataset(vol)
    r.Set1DTransFloat(tf)
    r.SetRendermode(0)
    r.SetUseLighting(True)
    r.SetLightModel(W.light_model, 0.2, 0.6, 0.2, 32.0)
    r.SetSampleRateModifier(srm)
    r.Resize(width, height)


def render_pair(torch, r, eye, at=(0, 0, 0)):
    """(reduced RGBA [540][960][4], its first-hit depth [540][960], bilinear
    upscale [1080][1920][4], plain [1080][1920][4])."""
    r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at)
    r.SetReducedQuality(True, True)
    check(lib().tvk_set_depth_output(r.handle, 1))
    r.Paint()
    rw, rh = r.GetRenderSize()
    W, H = r._w, r._h_px
    low = torch.empty((rh, rw, 4), dtype=torch.float32, device="cuda")
    depth = torch.empty((rh, rw), dtype=torch.float32, device="cuda")
    base = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    full = torch.empty((H, W, 4), dtype=torch.float32, device="cuda")
    check(lib().tvk_copy_image_device(r.handle, 1, _p(low), low.numel() * 4))
    check(lib().tvk_copy_depth_device(r.handle, _p(depth), depth.numel() * 4))
    check(lib().tvk_copy_image_device(r.handle, 0, _p(base), base.numel() * 4))
    check(lib().tvk_set_depth_output(r.handle, 0))
    r.SetReducedQuality(False, False)
    r.Paint()
    check(lib().tvk_copy_image_device(r.handle, 0, _p(full), full.numel() * 4))
    torch.cuda.current_stream().wait_stream(torch.cuda.ExternalStream(r.GetStream()))
    torch.cuda.synchronize()
    return low, depth, base, full


def psnr(mse):
    return 10.0 * math.log10(1.0 / max(mse, 1e-12))


def train(torch, steps=4000, crops=8, crop=128, lr=1e-3, seed=7, log=print, net=None,
          volumes=None, pair_every=1, time_budget_s=None, warmup=300, spike=4.0):
    """Trains on crops of fresh (reduced, plain) frame pairs; returns the net and a
    log.  Learning rate: linear warm-up, then cosine decay.  A step whose loss
    is not finite or exceeds `spike` x the median of the last 64 losses is not
    applied (one unusual pair must not wreck the weights)."""
    from .renderer import Renderer
    rng = np.random.default_rng(seed)
    vols = volumes or [make_training_volume(torch, s, sd) for s, sd in TRAIN_VOLUMES]
    r = Renderer()
    net = net or UNet(torch, seed=seed)
    hist = []
    hist_losses = []
    skipped = 0
    cur = 0.0
    t0 = time.perf_counter()
    pair = None
    for it in range(steps):
        if pair is None or it % pair_every == 0:
            vol = vols[int(rng.integers(0, len(vols)))]
            configure_lit(r, vol, random_bands_tf(rng))
            eye, at = random_camera(rng)
            low, depth, base, full = render_pair(torch, r, eye, at)
            x = prepare_input(torch, low, depth)
            pair = (x, base, full)
        x, base, full = pair
        ys = rng.integers(0, (low.shape[0] - crop) // 2 + 1, crops) * 2
        xs = rng.integers(0, (low.shape[1] - crop) // 2 + 1, crops) * 2
        xb = torch.stack([x[0, y:y + crop, xx:xx + crop] for y, xx in zip(ys, xs)]).contiguous()
        bb = torch.stack([base[2 * y:2 * (y + crop), 2 * xx:2 * (xx + crop)]
                          for y, xx in zip(ys, xs)]).contiguous()
        tb = torch.stack([full[2 * y:2 * (y + crop), 2 * xx:2 * (xx + crop)]
                          for y, xx in zip(ys, xs)]).contiguous()
        net.zero_grad()
        out = net.forward(xb, bb)
        loss, dout = net.loss(out, tb)
        lv = float(loss.item())
        recent = hist_losses[-64:]
        if not math.isfinite(lv) or (len(recent) >= 16 and lv > spike * float(np.median(recent))):
            skipped += 1
        else:
            hist_losses.append(lv)
            net.backward(dout)
            cur = lr * min(1.0, (it + 1) / warmup) * 0.5 * (1 + math.cos(math.pi * it / steps))
            net.step(cur)
        if it % 100 == 0 or it == steps - 1:
            base_loss, _ = net.loss(bb, tb, with_grad=False)
            l, bl = float(loss.item()), float(base_loss.item())
            hist.append((it, l, bl))
            log(f"step {it} loss {l:.3e} ({psnr(l):.2f} dB) bilinear {bl:.3e} "
                f"({psnr(bl):.2f} dB) lr {cur:.2e} skipped {skipped} "
                f"{time.perf_counter() - t0:.0f}s")
        if time_budget_s and time.perf_counter() - t0 > time_budget_s:
            log(f"time budget reached at step {it}")
            break
    return net, hist


class LearnedRenderer:
    """tvk_paint_learned with a network made from `params` (default: the
    committed weights)."""

    def __init__(self, params=None):
        params = params if params is not None else UNet.load_params()
        flat = np.concatenate([np.concatenate([np.asarray(params[n][0], np.float32).reshape(-1),
                                               np.asarray(params[n][1], np.float32)])
                               for n, *_ in ARCH]).astype(np.float32)
        h = C.c_void_p()
        check(lib().tvk_learned_create(flat.ctypes.data_as(N._f32p), flat.size, C.byref(h)))
        self._h = h

    def close(self):
        if self._h:
            check(lib().tvk_learned_destroy(self._h))
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def Paint(self, renderer, threshold_db=38.0):
        info = N.LearnedInfo()
        check(lib().tvk_paint_learned(renderer.handle, self._h, float(threshold_db),
                                      C.byref(info)))
        return info


def main():
    import argparse
    import torch
    ap = argparse.ArgumentParser(description="train the reconstruction network on the GPU")
    ap.add_argument("--steps", type=int, default=6000)
    ap.add_argument("--crops", type=int, default=8)
    ap.add_argument("--crop", type=int, default=128)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--minutes", type=float, default=None, help="stop after this wall time")
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--resume", action="store_true", help="continue from the weights at --out")
    ap.add_argument("--init", default=None, help="start from these weights (fine-tuning)")
    a = ap.parse_args()
    start = a.init or (a.out if a.resume else None)
    net = UNet(torch, params=UNet.load_params(start), seed=a.seed) if start else None
    net, hist = train(torch, steps=a.steps, crops=a.crops, crop=a.crop, lr=a.lr, seed=a.seed,
                      net=net, time_budget_s=a.minutes * 60 if a.minutes else None)
    net.save(a.out, steps=len(hist) and hist[-1][0] + 1, crops=a.crops, crop=a.crop, lr=a.lr,
             seed=a.seed, last_loss=hist[-1][1] if hist else None)
    print("saved", a.out)


if __name__ == "__main__":
    main()
