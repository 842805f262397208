"""Reconstruction of a sequence of slices held in (pinned) host memory, with
the host<->device copies overlapped with the device work.

The reference's front ends copy each item in, run the operator and copy the
result out, one after the other (its numpy extension blocks on every call).
``HostStreamer`` keeps a small ring of device buffers and runs three streams:
the input copy of slice k+1 (copy-in stream), the operators of slice k
(compute stream) and the output copy of slice k-1 (copy-out stream), ordered
by CUDA events.  Every slice still makes its own host->device and
device->host copy; only their overlap with the compute is new.
"""
from __future__ import annotations

from typing import Callable, Sequence

import torch


class HostStreamer:
    """Run ``step(din, dout, stream)`` over host slices with overlapped copies.

    ``step`` enqueues the operators of one slice on the CUDA stream handle it
    is given (an int, as ``torch.cuda.Stream.cuda_stream``), reading the device
    tensor ``din`` and writing ``dout``; it must not synchronise.  ``depth``
    device buffer pairs are cycled (2 overlaps one copy in and one copy out
    with each compute step)."""

    def __init__(self, step: Callable, in_shape, out_shape, device, depth: int = 2,
                 in_dtype=torch.float32, out_dtype=torch.float32):
        if depth < 1:
            raise ValueError("depth must be >= 1")
        self.step = step
        self.device = torch.device(device)
        self.depth = depth
        self.din = [torch.empty(in_shape, dtype=in_dtype, device=self.device) for _ in range(depth)]
        self.dout = [torch.empty(out_shape, dtype=out_dtype, device=self.device) for _ in range(depth)]
        self.s_in = torch.cuda.Stream(device=self.device)
        self.s_run = torch.cuda.Stream(device=self.device)
        self.s_out = torch.cuda.Stream(device=self.device)
        self._ev = lambda: torch.cuda.Event()  # noqa: E731  (ordering only, no timing)

    def run(self, inputs: Sequence[torch.Tensor], outputs: Sequence[torch.Tensor]) -> None:
        """Reconstruct inputs[k] into outputs[k] (host tensors, pinned for
        asynchronous copies) for every k; returns when every output is on the
        host."""
        if len(inputs) != len(outputs):
            raise ValueError("inputs and outputs differ in length")
        d = self.depth
        in_free = [None] * d    # compute of the slice that last used din[b] is done
        out_free = [None] * d   # copy-out of the slice that last used dout[b] is done
        for k, (hin, hout) in enumerate(zip(inputs, outputs)):
            b = k % d
            with torch.cuda.stream(self.s_in):
                if in_free[b] is not None:
                    self.s_in.wait_event(in_free[b])
                self.din[b].copy_(hin, non_blocking=True)
                loaded = self._ev()
                loaded.record(self.s_in)
            self.s_run.wait_event(loaded)
            if out_free[b] is not None:
                self.s_run.wait_event(out_free[b])
            self.step(self.din[b], self.dout[b], self.s_run.cuda_stream)
            done = self._ev()
            done.record(self.s_run)
            in_free[b] = done
            with torch.cuda.stream(self.s_out):
                self.s_out.wait_event(done)
                hout.copy_(self.dout[b], non_blocking=True)
                copied = self._ev()
                copied.record(self.s_out)
            out_free[b] = copied
        self.s_out.synchronize()
