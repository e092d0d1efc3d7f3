"""Ragged batches: many complex64 signals of uneven length, tap count and up/down
resampled in one persistent launch (gbfir_ragged_plan / gbfir_ragged_resample;
no MatX counterpart — MatX needs one resample_poly launch per signal).

    plan = RaggedPlan([(x0, h0, up0, down0), (x1, h1, up1, down1), ...])
    plan.run()                      # outputs in plan.outputs, stream-ordered
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run()                  # capturable: no host synchronisation inside
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib
from . import resample_out_len, _prec, _stream


class RaggedPlan:
    def __init__(self, signals, outputs=None, precision="fp32"):
        """signals: sequence of (x complex64 CUDA 1-D, h float32 CUDA 1-D, up, down).
        ``precision`` selects the arithmetic of the tap contraction as for resample_poly:
        "fp32" (row tiles on the CUDA cores) or a tensor-core form ("bf16", "fp16",
        "bf16x3": column-blocked Toeplitz MMAs); the plan is made for that form."""
        lib = _lib.load()
        self.precision = _prec(precision)
        n = len(signals)
        if n == 0:
            raise ValueError("RaggedPlan: no signals")
        self.inputs = []
        self.filters = []
        self.outputs = []
        descs = (_lib.RaggedDesc * n)()
        for i, (x, h, up, down) in enumerate(signals):
            if x.dtype != torch.complex64 or h.dtype != torch.float32 or x.dim() != 1 or h.dim() != 1:
                raise TypeError("RaggedPlan: complex64 1-D signals and float32 1-D filters")
            if not (x.is_cuda and h.is_cuda):
                raise ValueError("RaggedPlan: CUDA tensors only")
            x = x.contiguous()
            h = h.contiguous()
            olen = resample_out_len(x.shape[0], int(up), int(down))
            y = outputs[i] if outputs is not None else torch.empty(olen, dtype=torch.complex64, device=x.device)
            self.inputs.append(x)
            self.filters.append(h)
            self.outputs.append(y)
            g = math.gcd(int(up), int(down))
            descs[i] = _lib.RaggedDesc(x.data_ptr(), y.data_ptr(), h.data_ptr(), x.shape[0], olen, h.shape[0],
                                       int(up) // g, int(down) // g, 0)
        info = _lib.RaggedPlanInfo()
        cnt = lib.gbfir_ragged_plan_prec(descs, n, self.precision, None, ctypes.byref(info))
        if cnt < 0:
            _lib.check(-cnt)
        table = np.empty((cnt, 4), dtype=np.int64)
        cnt2 = lib.gbfir_ragged_plan_prec(descs, n, self.precision, table.ctypes.data_as(ctypes.c_void_p),
                                          ctypes.byref(info))
        if cnt2 != cnt:
            _lib.check(5 if cnt2 >= 0 else -cnt2)
        dev = self.inputs[0].device
        raw = np.frombuffer(ctypes.string_at(ctypes.addressof(descs), ctypes.sizeof(descs)), dtype=np.uint8)
        self.d_descs = torch.from_numpy(raw.copy()).to(dev)
        self.d_tiles = torch.from_numpy(table).to(dev)
        self.info = info
        self.count = n
        ws = lib.gbfir_ragged_workspace_size(n, cnt)
        self.workspace = torch.zeros(ws, dtype=torch.uint8, device=dev)
        self.num_tiles = int(cnt)

    def run(self):
        """One persistent launch over every signal, in the plan's arithmetic form."""
        lib = _lib.load()
        _lib.check(lib.gbfir_ragged_resample(
            ctypes.c_void_p(self.d_descs.data_ptr()), self.count, ctypes.c_void_p(self.d_tiles.data_ptr()),
            ctypes.byref(self.info), self.precision, ctypes.c_void_p(self.workspace.data_ptr()),
            self.workspace.numel(), _stream()))
        return self.outputs
