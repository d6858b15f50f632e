"""Event counts of the ray march for a workload, from the counting build.

    python -m tuvok_gb300.profile_counts [--workload plain_large_lit] [--poses 4] [--time]

Builds ``_build/libtvk_counts.so`` (the library with TVK_PROFILE_COUNTS=1),
runs the workload's first poses lit and unlit through it in a child process,
and prints one JSON line: per frame, the reference loop steps, the steps
executed (sampled), the samples that took the gradient and lighting, the leap
iterations and the steps they skipped, the candidate-brick slab tests and the
brick marches.  The counting atomics slow the march: these runs are never
timed; --time adds a second line with lit and unlit ms per frame from the
regular library (20 poses after 5 warm-up, CUDA events on the renderer's
stream).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys

NAMES = ["loop_steps", "executed_samples", "bricks_over_step_limit", "gradient_samples",
         "leap_iterations", "steps_leapt", "candidate_slab_tests", "brick_marches"]


def _time(r, poses, warmup: int = 5, frames: int = 20) -> float:
    """Mean ms per frame over `frames` poses after `warmup`: CUDA events on
    the renderer's own stream around the frames, back to back."""
    import torch

    for eye, at, up in poses[:warmup]:
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        r.Paint()
    stream = torch.cuda.ExternalStream(r.GetStream())
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for eye, at, up in poses[warmup:warmup + frames]:
        r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
        r.Paint()
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1) / frames


def _child(workload: str, poses: int, timing: bool) -> dict:
    import numpy as np
    import torch

    from tuvok_gb300 import Renderer, Volume, generate_volume_device
    from tuvok_gb300.workloads import WORKLOADS

    w = WORKLOADS[workload]
    n = w.dims[0] * w.dims[1] * w.dims[2] * np.dtype(w.dtype).itemsize
    raw = torch.empty(n, dtype=torch.uint8, device="cuda")
    generate_volume_device(raw.data_ptr(), w.dims, w.dtype, w.blobs(), w.noise_amp,
                           w.noise_octaves, w.noise_cell, w.seed, int(w.int_noise), w.vmax)
    vol = Volume(raw.data_ptr(), brick_size=w.brick_size, overlap=w.overlap, dims=w.dims,
                 dtype=w.dtype)
    del raw
    out = {"workload": workload, "poses": poses}
    for lit in (True, False):
        r = Renderer()
        r.RegisterDataset(vol)
        r.Set1DTransFloat(w.tf())
        r.SetRendermode(0)
        r.SetUseLighting(lit)
        r.SetLightModel(w.light_model, 0.2, 0.6, 0.2, 32.0)
        r.SetSampleRateModifier(w.srm)
        r.Resize(w.width, w.height)
        key = "lit" if lit else "unlit"
        if timing:
            out[key] = {"ms_per_frame": _time(r, w.poses())}
        else:
            tot = np.zeros(8)
            for eye, at, up in w.poses()[:poses]:
                r.SetViewParameters(50.0, 0.01, 1000.0, eye=eye, at=at, up=up)
                r.Paint()
                tot += np.array(r.GetCounters(), dtype=np.float64)
            out[key] = dict(zip(NAMES, (tot / poses).tolist()))
        del r
    return out


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--workload", default="plain_large_lit")
    ap.add_argument("--poses", type=int, default=4)
    ap.add_argument("--time", action="store_true",
                    help="also time lit and unlit frames with the regular library")
    ap.add_argument("--child", choices=["counts", "time"], help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    if a.child:
        print(json.dumps(_child(a.workload, a.poses, a.child == "time")), flush=True)
        return
    from tuvok_gb300 import build as B
    lib = B.build_counting_library()
    args = [sys.executable, "-m", "tuvok_gb300.profile_counts", "--workload", a.workload,
            "--poses", str(a.poses), "--child"]
    r = subprocess.run(args + ["counts"], env=dict(os.environ, TVK_LIBRARY=str(lib)))
    if r.returncode == 0 and a.time:
        env = {k: v for k, v in os.environ.items() if k != "TVK_LIBRARY"}
        r = subprocess.run(args + ["time"], env=env)
    sys.exit(r.returncode)


if __name__ == "__main__":
    main()
