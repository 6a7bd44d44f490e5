"""``QuantumNet`` / ``TorchLayer`` (tensorcircuit/torchnn.py:16-99): a
``torch.nn.Module`` whose weights are the non-first arguments of a quantum
function; the forward pass is ``vmap``-batched over the inputs and runs on
the engine, the backward pass is the engine's adjoint sweep."""

from typing import Any, Callable, Sequence, Tuple, Union

import torch

from .backends import backend
from .interfaces.torch import torch_interface


class QuantumNet(torch.nn.Module):
    def __init__(self, f: Callable[..., Any], weights_shape: Sequence[Any], initializer: Any = None,
                 use_vmap: bool = True, vectorized_argnums: Union[int, Sequence[int]] = 0,
                 use_interface: bool = True, use_jit: bool = True, enable_dlpack: bool = False) -> None:
        super().__init__()
        if use_vmap:
            f = backend.vmap(f, vectorized_argnums=vectorized_argnums)
        if use_interface:
            f = torch_interface(f, jit=use_jit, enable_dlpack=enable_dlpack)
        self.f = f
        self.q_weights = torch.nn.ParameterList()
        if isinstance(weights_shape[0], int):
            weights_shape = [weights_shape]
        if not isinstance(initializer, (list, tuple)):
            initializer = [initializer] * len(weights_shape)
        for ws, initf in zip(weights_shape, initializer):
            initf = torch.randn if initf is None else initf
            self.q_weights.append(torch.nn.Parameter(initf(tuple(ws))))

    def forward(self, *inputs: torch.Tensor) -> torch.Tensor:
        return self.f(*inputs, *self.q_weights)


TorchLayer = QuantumNet
