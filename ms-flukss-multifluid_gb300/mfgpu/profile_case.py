"""Step the heliosphere level (plasma + 3 neutral fluids, GLM, charge
exchange, RK2) a few times in one precision mode and schedule: the case the
committed ncu summaries capture.

    python -m mfgpu.profile_case --n 64 --patch 16 --precision mixed --schedule 0,0,0 --steps 2

--schedule: "auto" runs the autotuner; "0,0,0" the split kernels; x,y,z a
fused tile shape.  --overlap K: the split kernels in K overlapped chunks;
--flux-form lines: the FP64 face fluxes by lines.
Prints the status, the schedule and the step times (CUDA events), and exits
non-zero when a step reports an error."""
import argparse
import sys

import numpy as np

import mfgpu

PRECISIONS = {"fp64": mfgpu.PREC_FP64, "fp64_fast": mfgpu.PREC_FP64_FAST,
              "mixed": mfgpu.PREC_MIXED, "mixed_ce32": mfgpu.PREC_MIXED_CE32}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--patch", type=int, default=16)
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="mixed")
    ap.add_argument("--schedule", default="0,0,0")
    ap.add_argument("--overlap", type=int, default=1,
                    help="chunks of overlapped fluxes and update (mixed precision, split)")
    ap.add_argument("--flux-form", choices=["faces", "lines"], default="faces",
                    help="face fluxes of the FP64 paths per face or by lines")
    ap.add_argument("--steps", type=int, default=2)
    a = ap.parse_args(argv)
    import torch

    boxes = mfgpu.tile_boxes(a.n, a.patch, 3)
    p = mfgpu.helio_params(a.n, precision=PRECISIONS[a.precision])
    ctx = mfgpu.Context(p)
    lev = mfgpu.Level(ctx, boxes)
    flat = np.zeros(lev.ndoubles)
    for i in range(len(boxes)):
        flo, fhi = lev.fab_box(i)
        lev.patch_view(flat, i)[:] = mfgpu.init_host_fab(p, flo, fhi, "helio")
    lev.upload(flat.ctypes.data)
    if a.schedule == "auto":
        lev.autotune(3)
    else:
        lev.set_schedule(tuple(int(v) for v in a.schedule.split(",")))
        if a.overlap > 1:
            lev.set_overlap(a.overlap)
        if a.flux_form == "lines":
            lev.set_flux_form(mfgpu.FLUX_LINES)
    stream = torch.cuda.Stream()
    dt0 = lev.compute_dt()[0]
    lev.seed_dt(0.4 * dt0, 0.4, stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        lev.step_async(stream.cuda_stream)
    e1.record(stream)
    st = lev.result(stream.cuda_stream)[0]
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(1, a.steps)
    print(f"status {st} cells {lev.ncells} patches {len(boxes)} precision {a.precision} "
          f"schedule {lev.schedule()} overlap {lev.overlap()} launches/step {lev.launches_per_step()} ms/step {ms:.3f}")
    lev.close()
    ctx.close()
    return 0 if st == 0 else 1


if __name__ == "__main__":
    sys.exit(main())
