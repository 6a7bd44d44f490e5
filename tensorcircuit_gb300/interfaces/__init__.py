"""Framework interfaces (tensorcircuit/interfaces/__init__.py): on this
engine the backend is PyTorch, so the torch interface is the identity on
tensors and gradients flow through the engine's own autograd Functions."""

from .torch import pytorch_interface, torch_interface

__all__ = ["torch_interface", "pytorch_interface"]
