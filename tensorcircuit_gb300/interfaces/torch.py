"""``torch_interface`` (tensorcircuit/interfaces/torch.py:18-114).

The reference converts torch tensors to the active backend's tensors, runs
the function there and bridges the vector-Jacobian product back through a
``torch.autograd.Function``.  Here the backend *is* torch: arguments pass
through (numpy arrays become tensors), the engine's autograd Functions give
the gradients (adjoint sweep), and ``jit=True`` replays calls that need no
gradient from a captured CUDA graph (``backend.jit``).
"""

from typing import Any, Callable

import numpy as np
import torch

from ..backends import backend


def _as_tensor(x: Any) -> Any:
    if isinstance(x, np.ndarray):
        return torch.as_tensor(x)
    return x


def torch_interface(fun: Callable[..., Any], jit: bool = False, enable_dlpack: bool = False) -> Callable[..., Any]:
    """Wrap ``fun`` (tensor in, tensor out) for torch callers; ``enable_dlpack``
    is accepted for signature compatibility (no conversion happens)."""
    jf = backend.jit(fun) if jit else None

    def wrapper(*args: Any, **kws: Any) -> Any:
        args = tuple(backend.tree_map(_as_tensor, a) for a in args)
        leaves = [t for a in args for t in torch.utils._pytree.tree_flatten(a)[0] if isinstance(t, torch.Tensor)]
        needs_grad = torch.is_grad_enabled() and any(t.requires_grad for t in leaves)
        if jf is not None and not needs_grad and not kws:
            return jf(*args)
        return fun(*args, **kws)

    wrapper.__wrapped__ = fun  # type: ignore
    return wrapper


pytorch_interface = torch_interface
