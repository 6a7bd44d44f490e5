"""Global configuration with the reference's entry points
(tensorcircuit/cons.py:36-182): ``set_backend``, ``set_dtype``,
``set_contractor`` and their ``runtime_*`` context managers.

The engine exists for the pytorch backend and complex64 only (the
parameterized-circuit path it replaces); other choices raise instead of
silently falling back to another implementation.
"""

import contextlib
from typing import Any, Iterator, Optional

from .backends import PyTorchBackend, backend

dtypestr = "complex64"
rdtypestr = "float32"
contractor = "statevector-engine"


def set_backend(backend_name: Optional[str] = None, set_global: bool = True) -> PyTorchBackend:
    if backend_name is None or backend_name == "pytorch" or backend_name == "torch" or isinstance(
        backend_name, PyTorchBackend
    ):
        return backend
    raise ValueError(
        "backend %r: this engine implements the pytorch backend only "
        "(GB300 statevector kernels, no multi-backend dispatch)" % (backend_name,)
    )


set_tensornetwork_backend = set_backend


def get_backend(backend_name: Optional[str] = None) -> PyTorchBackend:
    return set_backend(backend_name)


def set_dtype(dtype: Optional[str] = None, set_global: bool = True) -> Any:
    if dtype is None or dtype in ("complex64", "float32", "32"):
        return ("complex64", "float32")
    raise NotImplementedError("the engine computes in complex64 only (got %r)" % (dtype,))


def get_dtype(dtype: Optional[str] = None) -> Any:
    return set_dtype(dtype)


def set_contractor(method: Optional[str] = None, **kws: Any) -> str:
    """Contraction-path settings do not apply: the engine evolves a state
    vector in HBM passes instead of contracting a network."""
    return contractor


@contextlib.contextmanager
def runtime_backend(backend_name: Optional[str] = None) -> Iterator[PyTorchBackend]:
    yield set_backend(backend_name)


@contextlib.contextmanager
def runtime_dtype(dtype: Optional[str] = None) -> Iterator[Any]:
    yield set_dtype(dtype)


@contextlib.contextmanager
def runtime_contractor(method: Optional[str] = None, **kws: Any) -> Iterator[str]:
    yield set_contractor(method, **kws)
