"""Host-resident batches streamed through the GPU (no MatX counterpart).

The direct-FIR transforms are independent per row, so a batch that lives in pinned
host memory can be processed in row chunks with the three stages of each chunk on
their own CUDA streams: the host->device copy of chunk c, the transforms of chunk
c-1 and the device->host copies of chunk c-2 run at the same time.  On GB300 the
copies over NVLink-C2C are the slow stage, so the transforms and the copy in the
other direction hide behind them, and the device only holds two chunks.

    pipe = RowPipeline(device, rows_per_chunk=8)
    pipe.run(x_pinned, [y1_pinned, y2_pinned], lambda xd, outs: [
        matx_gb300.resample_poly(xd, h1, 3, 2, out=outs[0]),
        matx_gb300.resample_poly(xd, h2, 4, 5, out=outs[1])])

``fn(x_chunk, out_chunks)`` must write every output chunk (device tensors of
rows_per_chunk or fewer rows) on the current stream, which ``run`` sets to the
compute stream.
"""
from __future__ import annotations

from typing import Callable, Sequence

import torch


class RowPipeline:
    def __init__(self, device: torch.device, rows_per_chunk: int = 8, copy_streams: int = 2):
        """``copy_streams`` device->host streams share each chunk's copies back (row slices
        of every output), so several copy engines drain the results at once."""
        if rows_per_chunk < 1:
            raise ValueError("rows_per_chunk must be >= 1")
        if copy_streams < 1:
            raise ValueError("copy_streams must be >= 1")
        self.device = torch.device(device)
        self.rows = int(rows_per_chunk)
        self.s_in = torch.cuda.Stream(self.device)
        self.s_cmp = torch.cuda.Stream(self.device)
        self.s_outs = [torch.cuda.Stream(self.device) for _ in range(int(copy_streams))]
        self._bufs = None

    def _buffers(self, x: torch.Tensor, outs: Sequence[torch.Tensor]):
        key = (x.shape[1:], x.dtype, tuple((o.shape[1:], o.dtype) for o in outs))
        if self._bufs is None or self._bufs[0] != key:
            xb = [torch.empty((self.rows,) + tuple(x.shape[1:]), dtype=x.dtype, device=self.device) for _ in range(2)]
            ob = [[torch.empty((self.rows,) + tuple(o.shape[1:]), dtype=o.dtype, device=self.device) for o in outs]
                  for _ in range(2)]
            self._bufs = (key, xb, ob)
        return self._bufs[1], self._bufs[2]

    def run(self, x: torch.Tensor, outs: Sequence[torch.Tensor],
            fn: Callable[[torch.Tensor, list], object]) -> None:
        """Stream the rows of pinned host tensor ``x`` through ``fn`` into pinned ``outs``."""
        if x.is_cuda or any(o.is_cuda for o in outs):
            raise ValueError("RowPipeline streams host tensors; pass device tensors to the transforms directly")
        if not x.is_pinned() or not all(o.is_pinned() for o in outs):
            raise ValueError("RowPipeline needs pinned host tensors (tensor.pin_memory())")
        B = x.shape[0]
        if any(o.shape[0] != B for o in outs):
            raise ValueError("every output needs the same number of rows as the input")
        xb, ob = self._buffers(x, outs)
        ns = len(self.s_outs)
        h2d = [torch.cuda.Event() for _ in range(2)]
        cmp = [torch.cuda.Event() for _ in range(2)]
        d2h = [[torch.cuda.Event() for _ in range(ns)] for _ in range(2)]
        used = [False, False]
        caller = torch.cuda.current_stream(self.device)
        # the pipeline's work is ordered after what the caller already queued
        for s in (self.s_in, self.s_cmp, *self.s_outs):
            s.wait_stream(caller)
        for c, r0 in enumerate(range(0, B, self.rows)):
            r1 = min(B, r0 + self.rows)
            n = r1 - r0
            k = c & 1
            if used[k]:
                self.s_in.wait_event(cmp[k])      # chunk c-2 no longer reads xb[k]
            with torch.cuda.stream(self.s_in):
                xb[k][:n].copy_(x[r0:r1], non_blocking=True)
                h2d[k].record(self.s_in)
            self.s_cmp.wait_event(h2d[k])
            if used[k]:
                for e in d2h[k]:
                    self.s_cmp.wait_event(e)      # chunk c-2's outputs have left ob[k]
            with torch.cuda.stream(self.s_cmp):
                fn(xb[k][:n], [b[:n] for b in ob[k]])
                cmp[k].record(self.s_cmp)
            # copy stream j takes the j-th contiguous slice of the chunk's rows
            bounds = [n * j // ns for j in range(ns + 1)]
            for j, so in enumerate(self.s_outs):
                so.wait_event(cmp[k])
                a, b_ = bounds[j], bounds[j + 1]
                with torch.cuda.stream(so):
                    if b_ > a:
                        for o, b in zip(outs, ob[k]):
                            o[r0 + a:r0 + b_].copy_(b[a:b_], non_blocking=True)
                    d2h[k][j].record(so)
            used[k] = True
        # the caller's stream sees every copy back
        for so in self.s_outs:
            caller.wait_stream(so)
