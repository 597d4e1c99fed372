"""bhk_trace_frames_static: the tracer for callers that may not allocate device memory.

Such callers -- a framework that owns the whole device-memory budget through its own pool, or a
per-frame render loop where cudaMalloc/cudaFree would synchronise the device -- hand in their
output buffers and get the same rays the context-based bhk_trace_frames computes, with all working
memory in a fixed array inside libbhk. This file checks, through the C ABI, that two calls in a row
(different frames, so stale contents of the shared array would show) match the existing entry
point to the tolerance the other parity tests use, and that oversized requests are refused. The
test allocates the output buffers itself; the entry point allocates nothing.
"""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from black_simulation_gb300 import bhk

pytestmark = pytest.mark.gpu

FRAMES = [
    [bhk.frame_c1(64, 48)],
    [bhk.Frame(0.998, 1000.0, math.radians(60.0), 96, 54, -20.0, 20.0, -11.25, 11.25, 0.0, 30.0),
     bhk.Frame(0.5, 30.0, 1.2, 17, 9, -10.0, 10.0, -6.0, 6.0, 0.0, 15.0),
     # a naked singularity (a = 1.2) seen from 30 M at 30 degrees, as bhk_trace_frames accepts it
     bhk.Frame(1.2, 30.0, math.radians(30.0), 40, 30, -8.0, 8.0, -6.0, 6.0, 0.0, 20.0)],
]


def _static_call(frames, opts):
    n = sum(f.rays for f in frames)
    out = bhk.alloc_outputs(n, "cuda", extras=True)
    arr = (bhk.FrameDescC * len(frames))(*[f.c() for f in frames])
    oc = opts.c()
    outc = bhk.RaysOutC(*[out[k].data_ptr() for k in bhk.FIELDS + bhk.EXTRA_FIELDS])
    stream = torch.cuda.current_stream().cuda_stream or bhk.CUDA_STREAM_LEGACY
    status = bhk.lib().bhk_trace_frames_static(arr, len(frames), C.byref(oc), C.byref(outc), stream)
    assert status == bhk.OK, bhk.lib().bhk_last_error()
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("prec,sort_buckets,reg_budget",
                         [("fp64", 1, 2), ("fp64", 64, 2), ("mixed", 1, 2), ("mixed", 64, 2), ("mixed", 1, 3),
                          ("mixed", 64, 3)])
def test_static_entry_point_matches_context_entry_point_twice_in_a_row(ctx, prec, sort_buckets, reg_budget):
    """Both the tile order and the cost sort (whose histogram and offsets live in the shared array),
    in the capped and the uncapped FP32 variants, with every RayReport output."""
    opts = bhk.TraceOpts(prec, block=128, chunk=32, sort_buckets=sort_buckets, reg_budget=reg_budget)
    for frames in FRAMES:  # two calls in a row on the shared array
        got = _static_call(frames, opts)
        n = sum(f.rays for f in frames)
        want = ctx.trace_frames(frames, opts, out=bhk.alloc_outputs(n, "cuda", extras=True))
        want = {k: v.cpu().numpy() for k, v in want.items()}
        torch.cuda.synchronize()
        for k in bhk.FIELDS + bhk.EXTRA_FIELDS:
            np.testing.assert_allclose(got[k].astype(float), want[k].astype(float), rtol=1e-12, atol=1e-12,
                                       equal_nan=True, err_msg=f"{prec} {k}")


def test_static_entry_point_refuses_requests_beyond_its_array(cuda):
    too_many_rays = [bhk.frame_c1(257, 256)]
    arr = (bhk.FrameDescC * 1)(*[f.c() for f in too_many_rays])
    oc = bhk.TraceOpts("mixed").c()
    outc = bhk.RaysOutC()
    status = bhk.lib().bhk_trace_frames_static(arr, 1, C.byref(oc), C.byref(outc), None)
    assert status == bhk.EINVAL
    assert b"65536" in bhk.lib().bhk_last_error()
    too_many_frames = [bhk.frame_c1(2, 2)] * 65
    arr = (bhk.FrameDescC * 65)(*[f.c() for f in too_many_frames])
    status = bhk.lib().bhk_trace_frames_static(arr, 65, C.byref(oc), C.byref(outc), None)
    assert status == bhk.EINVAL
    assert b"64 frames" in bhk.lib().bhk_last_error()
