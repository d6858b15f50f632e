"""Times the learned reconstruction network's 3x3 convolutions one by one.

Every layer of the U-Net (``learned.ARCH``) runs through ``tvk_cnn_conv3x3`` at
the size the learned frame gives it (the reduced frame, 960 x 540 by default,
halved per level), on seeded BF16 inputs, and is timed with CUDA events on the
stream it runs on.  Prints one JSON line: per layer the shape, microseconds per
launch and TFLOP/s (2 x 9 x cin x cout per output pixel), and the sum.

    python -m tuvok_gb300.profile_conv [--width 960 --height 540 --reps 20]
"""
import argparse
import ctypes as C
import json

import numpy as np

from . import _native as N
from ._native import check, lib
from .learned import ARCH

# the level (0 = full reduced resolution) each layer runs at
LEVEL = {"e0a": 0, "e0b": 0, "e1a": 1, "e1b": 1, "e2a": 2, "e2b": 2, "b": 3, "d2": 2, "d1": 1,
         "d0": 0, "head": 0}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--width", type=int, default=960)
    ap.add_argument("--height", type=int, default=540)
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args(argv)
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("needs a CUDA device")
    torch.cuda.init()
    stream = torch.cuda.Stream()
    s = C.c_void_p(stream.cuda_stream)
    rng = np.random.default_rng(5)
    rows, total_us, total_flop = [], 0.0, 0.0

    def dev(a, dt):
        return torch.tensor(a, dtype=dt, device="cuda").contiguous()

    for name, c1, c2, cout, slope in ARCH:
        h, w = args.height >> LEVEL[name], args.width >> LEVEL[name]
        x1 = dev(rng.normal(size=(1, h, w, c1)), torch.bfloat16)
        x2 = dev(rng.normal(size=(1, h, w, c2)), torch.bfloat16) if c2 else None
        wt = dev(rng.normal(size=(9, cout, c1 + c2)) * 0.05, torch.bfloat16)
        b = dev(rng.normal(size=cout) * 0.1, torch.float32)
        head = name == "head"
        y = None if head else torch.empty((1, h, w, cout), dtype=torch.bfloat16, device="cuda")
        yf = torch.empty((1, h, w, cout), dtype=torch.float32, device="cuda") if head else None

        def ptr(t):
            return C.c_void_p(t.data_ptr()) if t is not None else None
        a = N.CnnConv(x1=ptr(x1), x2=ptr(x2), c1=c1, c2=c2, n=1, h=h, w=w, weights=ptr(wt),
                      bias=ptr(b), cout=cout, slope=slope, y_bf16=ptr(y), y_f32=ptr(yf),
                      y2_f32=None, split=cout, accumulate=0)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for _ in range(3):
                check(lib().tvk_cnn_conv3x3(C.byref(a), s))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.reps):
                check(lib().tvk_cnn_conv3x3(C.byref(a), s))
            e1.record(stream)
        check(lib().tvk_cnn_check(s))
        us = e0.elapsed_time(e1) * 1000.0 / args.reps
        flop = 2.0 * 9 * (c1 + c2) * cout * h * w
        total_us += us
        total_flop += flop
        rows.append(dict(layer=name, h=h, w=w, cin=c1 + c2, cout=cout, us=round(us, 2),
                         tflops=round(flop / us * 1e-6, 1)))
    print(json.dumps(dict(size=[args.width, args.height], reps=args.reps, layers=rows,
                          total_us=round(total_us, 1),
                          total_tflops=round(total_flop / total_us * 1e-6, 1))))


if __name__ == "__main__":
    main()
