"""Utilities (vegasflow utils.py): the per-bin histogram."""

from __future__ import annotations

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
