"""Utilities (vegasflow utils.py): the per-bin histogram, the mask combiner for
integrands, and the GPU-side helpers of this package (kernel preloading, the
capture guard)."""

from __future__ import annotations

import contextlib
import gc

import torch

from . import _native as nat


def consume_array_into_indices(input_arr, indices, result_size):
    """Accumulate ``input_arr`` into ``result_size`` bins by ``indices``
    (utils.py:17-44), on the GPU.  ``input_arr`` (n,) float64, ``indices`` (n,)
    or (n, 1) integers, both CUDA tensors (or array-likes, copied to the current
    CUDA device).  Returns a (result_size,) float64 CUDA tensor."""
    nat.load()
    dev = input_arr.device if isinstance(input_arr, torch.Tensor) and input_arr.is_cuda \
        else torch.device("cuda", torch.cuda.current_device())
    vals = torch.as_tensor(input_arr, dtype=torch.float64, device=dev).reshape(-1).contiguous()
    idx = torch.as_tensor(indices, device=dev).reshape(-1).to(torch.int32).contiguous()
    if idx.numel() != vals.numel():
        raise ValueError(f"{vals.numel()} values but {idx.numel()} indices")
    out = torch.empty(int(result_size), dtype=torch.float64, device=dev)
    nat.call("vf_consume_array_into_indices", nat.ptr(vals), nat.ptr(idx), int(vals.numel()),
             int(result_size), nat.ptr(out), None, nat.stream_handle())
    return out


def py_consume_array_into_indices(input_arr, indices, result_size):
    """Python-object interface of ``consume_array_into_indices`` (utils.py:47-52)."""
    return consume_array_into_indices(input_arr, indices, int(result_size))


def generate_condition_function(n_mask, condition="and"):
    """A function ``f(*masks) -> (mask, indices)`` combining ``n_mask`` boolean
    tensors with ``condition`` ("and", "or", or a list of n_mask - 1 of them
    applied left to right); ``indices`` are the positions where the combined mask
    is True, int32 of shape (k, 1) (utils.py:55-141, same errors)."""
    allowed = {"and": torch.logical_and, "or": torch.logical_or}
    names = list(allowed)
    if n_mask < 2:
        raise ValueError("At least two masks needed to generate a wrapper")
    if isinstance(condition, str):
        if condition not in allowed:
            raise ValueError(f"Wrong condition {condition}, allowed values are {names}")
        conditions = None
    else:
        conditions = list(condition)
        if len(conditions) != n_mask - 1:
            raise ValueError(f"Wrong number of conditions for {n_mask} masks: {len(conditions)}")
        for cond in conditions:
            if cond not in allowed:
                raise ValueError(f"Wrong condition {cond}, allowed values are {names}")

    def condition_to_idx(*masks):
        masks = [torch.as_tensor(m, dtype=torch.bool) for m in masks]
        if conditions is not None:
            res = masks[0]
            for cond, mask in zip(conditions, masks[1:]):
                res = allowed[cond](res, mask)
        elif condition == "and":
            res = torch.stack(masks).all(dim=0)
        else:
            res = torch.stack(masks).any(dim=0)
        return res, torch.nonzero(res).to(torch.int32)

    return condition_to_idx


_PRELOADED = set()


@contextlib.contextmanager
def capture_guard():
    """Around a CUDA-graph capture: collect Python's cyclic garbage first and
    keep the collector off until the capture ends.  A collection inside the
    capture could run the finalizer of an unreachable CUDA graph, whose reset
    is not permitted while a stream captures and invalidates the capture."""
    gc.collect()
    enabled = gc.isenabled()
    gc.disable()
    try:
        yield
    finally:
        if enabled:
            gc.enable()


def preload_kernels(device):
    """Load, once per device and before the first CUDA-graph capture, every
    kernel of the native library (``vf_preload``) and run the small torch
    operations the integrators, the batch engine and the server use
    around their own kernels (advanced-index writes and gathers, casts,
    concatenation, fills, strided copies) for the dtypes they use.

    With lazy module loading (the default), the first use of a kernel loads its
    module; measured on GB300 with driver 580, a module loaded after a CUDA graph
    has been captured in the process took ~2.2 s (50 ms before), which showed up
    as a 2-second stall in the first admission of a server started after a
    graph-replayed batch.  Loading these modules up front keeps that out of the
    timed paths."""
    dev = torch.device(device)
    if dev.type != "cuda":
        return
    key = (dev.index if dev.index is not None else torch.cuda.current_device())
    if key in _PRELOADED:
        return
    with torch.cuda.device(dev):
        nat.check(nat.load().vf_preload())  # the library's own kernels
    idx = torch.zeros(1, dtype=torch.int64, device=dev)
    for dt in (torch.float64, torch.float32, torch.int32, torch.int64, torch.uint8):
        a = torch.zeros((4, 3, 2), dtype=dt, device=dev)
        a[idx] = torch.ones((1, 3, 2), dtype=dt, device=dev)  # index_put, tensor source
        a[idx] = 0  # index_put, scalar source
        b = a[idx][:, 1:2].reshape(-1)  # gather, strided copy
        c = torch.cat([b, a.reshape(-1)])  # concatenation
        for dt2 in (torch.float64, torch.float32, torch.int32):
            c.to(dt2)  # casts
        a.fill_(1)
        a.copy_(a.clone())
        a.view(4, 6)[:, 2:4].contiguous()
    torch.cuda.synchronize(dev)
    _PRELOADED.add(key)
