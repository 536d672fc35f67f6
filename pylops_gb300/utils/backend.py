"""Array-kind helpers: numpy arrays on the host, torch tensors on the device.

Plays the role of ``pylops/utils/backend.py`` (``get_array_module`` at
``:126``, ``to_numpy``) with torch in place of cupy.
"""

import numpy as np

__all__ = ["is_torch", "get_array_module", "to_numpy", "to_device"]


def is_torch(x) -> bool:
    return type(x).__module__.startswith("torch") and hasattr(x, "data_ptr")


def get_array_module(x):
    """numpy for numpy arrays, torch for torch tensors."""
    if is_torch(x):
        import torch

        return torch
    return np


def to_numpy(x):
    if is_torch(x):
        return x.detach().cpu().numpy()
    return np.asarray(x)


def to_device(x, dtype="float32", device="cuda"):
    import torch

    if is_torch(x):
        return x.to(device=device, dtype=getattr(torch, str(np.dtype(dtype))))
    return torch.as_tensor(np.ascontiguousarray(x, dtype=dtype), device=device)
