"""The ``backend`` object: the subset of the reference's ``PyTorchBackend``
(tensorcircuit/backends/pytorch_backend.py) that the parameterized-circuit
path uses, with the same names, arguments and return conventions.

``vectorized_value_and_grad`` / ``vvag`` follows the reference exactly
(pytorch_backend.py:673-709): ``torch.func.vmap`` over
``torch.func.grad_and_value`` and a batch sum of the gradients of the
non-vectorised ``argnums``.  Because the engine's autograd Functions carry
vmap rules, the vmapped circuits run as one batched kernel launch per pass
and their gradients come from one batched adjoint sweep.
"""

from functools import partial
from typing import Any, Callable, List, Optional, Sequence, Tuple, Union

import numpy as np
import torch

Tensor = Any


def _tree_map(f: Callable[..., Any], *pytrees: Any) -> Any:
    import torch.utils._pytree as pytree

    return pytree.tree_map(f, *pytrees)


class GraphJit:
    """CUDA-graph compiled callable (see ``PyTorchBackend.jit``)."""

    WARMUP = 3

    def __init__(self, f: Callable[..., Any], static_argnums: Tuple[int, ...]) -> None:
        self.f = f
        self.static = set(static_argnums)
        self.cache: dict = {}
        self.__wrapped__ = f

    def _key(self, args: Tuple[Any, ...]) -> Any:
        import torch.utils._pytree as pytree

        parts = []
        for i, a in enumerate(args):
            if i in self.static:
                parts.append(("s", repr(a)))
                continue
            leaves, spec = pytree.tree_flatten(a)
            sig = []
            for x in leaves:
                if isinstance(x, torch.Tensor):
                    if x.device.type != "cuda":
                        return None
                    sig.append(("t", tuple(x.shape), str(x.dtype), str(x.device)))
                else:
                    sig.append(("v", repr(x)))
            parts.append((str(spec), tuple(sig)))
        return tuple(parts)

    def __call__(self, *args: Any, **kws: Any) -> Any:
        import torch.utils._pytree as pytree

        if kws or torch.cuda.is_current_stream_capturing():
            return self.f(*args, **kws)
        key = self._key(args)
        if key is None:
            return self.f(*args)
        ent = self.cache.setdefault(key, {"calls": 0, "graph": None, "failed": False})
        if ent["failed"] or ent["calls"] < self.WARMUP:
            ent["calls"] += 1
            return self.f(*args)
        if ent["graph"] is None:
            static_args = pytree.tree_map(lambda t: t.clone() if isinstance(t, torch.Tensor) else t, args)
            try:
                torch.cuda.synchronize()
                side = torch.cuda.Stream()
                side.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(side):
                    self.f(*static_args)
                torch.cuda.current_stream().wait_stream(side)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    out = self.f(*static_args)
            except Exception as exc:  # not capturable: stay eager
                torch.cuda.synchronize()
                ent["failed"] = True
                ent["error"] = "%s: %s" % (type(exc).__name__, str(exc)[:300])
                return self.f(*args)
            ent["graph"], ent["inputs"], ent["outputs"] = g, static_args, out
        src_leaves = pytree.tree_flatten(args)[0]
        dst_leaves = pytree.tree_flatten(ent["inputs"])[0]
        for s, d in zip(src_leaves, dst_leaves):
            if isinstance(d, torch.Tensor):
                d.copy_(s, non_blocking=True)
        ent["graph"].replay()
        return pytree.tree_map(lambda t: t.clone() if isinstance(t, torch.Tensor) else t, ent["outputs"])

    def capture_errors(self) -> List[str]:
        """Why capture failed for the argument signatures that stayed eager."""
        return [e["error"] for e in self.cache.values() if e.get("error")]


class PyTorchBackend:
    name = "pytorch"

    # ---------------------------------------------------------- tensor ops
    def convert_to_tensor(self, a: Any, dtype: Optional[Any] = None) -> Tensor:
        t = a if isinstance(a, torch.Tensor) else torch.as_tensor(np.asarray(a))
        if dtype is not None:
            t = self.cast(t, dtype)
        return t

    def numpy(self, a: Tensor) -> np.ndarray:
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
        return np.asarray(a)

    def cast(self, a: Tensor, dtype: Any) -> Tensor:
        if isinstance(dtype, str):
            return a.type(getattr(torch, dtype))
        return a.type(dtype)

    def real(self, a: Tensor) -> Tensor:
        return torch.real(a) if torch.is_complex(a) else a

    def imag(self, a: Tensor) -> Tensor:
        return torch.imag(a) if torch.is_complex(a) else torch.zeros_like(a)

    def abs(self, a: Tensor) -> Tensor:
        return torch.abs(a)

    def conj(self, a: Tensor) -> Tensor:
        return torch.conj(a)

    def sum(self, a: Tensor, axis: Optional[int] = None, keepdims: bool = False) -> Tensor:
        if axis is None:
            return torch.sum(a)
        return torch.sum(a, dim=axis, keepdim=keepdims)

    def mean(self, a: Tensor, axis: Optional[int] = None, keepdims: bool = False) -> Tensor:
        if axis is None:
            return torch.mean(a)
        return torch.mean(a, dim=axis, keepdim=keepdims)

    def reshape(self, a: Tensor, shape: Sequence[int]) -> Tensor:
        return torch.reshape(a, tuple(shape))

    def reshape2(self, a: Tensor) -> Tensor:
        k = int(round(np.log2(int(np.prod(a.shape)))))
        return torch.reshape(a, [2] * k)

    def reshapem(self, a: Tensor) -> Tensor:
        d = int(round(np.sqrt(int(np.prod(a.shape)))))
        return torch.reshape(a, [d, d])

    def stack(self, a: Sequence[Tensor], axis: int = 0) -> Tensor:
        return torch.stack(list(a), dim=axis)

    def concat(self, a: Sequence[Tensor], axis: int = 0) -> Tensor:
        return torch.cat(list(a), dim=axis)

    def zeros(self, shape: Any, dtype: Optional[str] = None) -> Tensor:
        return torch.zeros(shape, dtype=getattr(torch, dtype or "complex64"))

    def ones(self, shape: Any, dtype: Optional[str] = None) -> Tensor:
        return torch.ones(shape, dtype=getattr(torch, dtype or "complex64"))

    def eye(self, n: int, m: Optional[int] = None, dtype: Optional[str] = None) -> Tensor:
        return torch.eye(n, m if m is not None else n, dtype=getattr(torch, dtype or "complex64"))

    def arange(self, start: int, stop: Optional[int] = None, step: int = 1) -> Tensor:
        if stop is None:
            return torch.arange(0, start, step)
        return torch.arange(start, stop, step)

    def cos(self, a: Tensor) -> Tensor:
        return torch.cos(a)

    def sin(self, a: Tensor) -> Tensor:
        return torch.sin(a)

    def exp(self, a: Tensor) -> Tensor:
        return torch.exp(a)

    def sqrt(self, a: Tensor) -> Tensor:
        return torch.sqrt(a)

    def kron(self, a: Tensor, b: Tensor) -> Tensor:
        return torch.kron(a, b)

    def adjoint(self, a: Tensor) -> Tensor:
        return torch.conj(torch.transpose(a, -1, -2))

    def tensordot(self, a: Tensor, b: Tensor, axes: Any) -> Tensor:
        return torch.tensordot(a, b, dims=axes)

    def cumsum(self, a: Tensor, axis: Optional[int] = None) -> Tensor:
        if axis is None:
            return torch.cumsum(a.reshape(-1), dim=0)
        return torch.cumsum(a, dim=axis)

    def searchsorted(self, a: Tensor, v: Tensor, side: str = "left") -> Tensor:
        return torch.searchsorted(self.convert_to_tensor(a), self.convert_to_tensor(v), side=side)

    def shape_tuple(self, a: Tensor) -> Tuple[int, ...]:
        return tuple(a.shape)

    def sizen(self, a: Tensor) -> int:
        return int(a.numel())

    def is_tensor(self, a: Any) -> bool:
        return isinstance(a, torch.Tensor)

    def tree_map(self, f: Callable[..., Any], *pytrees: Any) -> Any:
        return _tree_map(f, *pytrees)

    def i(self, dtype: Any = None) -> Tensor:
        return torch.tensor(1j, dtype=torch.complex64)

    def implicit_randn(self, shape: Any = 1, mean: float = 0.0, stddev: float = 1.0, dtype: str = "32") -> Tensor:
        if isinstance(shape, int):
            shape = (shape,)
        return torch.randn(*shape) * stddev + mean

    def implicit_randu(self, shape: Any = 1, low: float = 0.0, high: float = 1.0, dtype: str = "32") -> Tensor:
        if isinstance(shape, int):
            shape = (shape,)
        return torch.rand(*shape) * (high - low) + low

    def probability_sample(self, shots: int, p: Tensor, status: Optional[Tensor] = None, g: Any = None) -> Tensor:
        from .quantum import probability_sample

        if status is None:
            status = torch.rand(shots, generator=g if isinstance(g, torch.Generator) else None)
        return probability_sample(shots, p, status)

    def set_random_state(self, seed: Optional[int] = None, get_only: bool = False) -> Any:
        g = torch.Generator()
        if seed is not None:
            g.manual_seed(seed)
        if not get_only:
            torch.manual_seed(seed if seed is not None else torch.seed())
        return g

    def get_random_state(self, seed: Optional[int] = None) -> Any:
        return self.set_random_state(seed, get_only=True)

    # ----------------------------------------------------------- transforms
    def jit(self, f: Callable[..., Any], static_argnums: Optional[Union[int, Sequence[int]]] = None,
            jit_compile: Optional[bool] = None, **kws: Any) -> Callable[..., Any]:
        """Compile ``f`` by CUDA-graph capture.

        The reference's pytorch backend returns ``f`` unchanged
        (pytorch_backend.py:659-669) and its jax backend traces with XLA.
        Here the first calls per input signature run eagerly (they build the
        circuit plans and the specialised kernels), then one call is captured
        into a CUDA graph, and later calls copy their tensor arguments into the
        graph's input buffers and replay it -- no Python, autograd or
        functorch work per call.  Outputs are returned as fresh tensors.
        Calls with CPU tensors or keyword arguments, and functions that cannot
        be captured, run eagerly."""
        if isinstance(static_argnums, int):
            static_argnums = (static_argnums,)
        return GraphJit(f, tuple(static_argnums or ()))

    def grad(self, f: Callable[..., Any], argnums: Union[int, Sequence[int]] = 0,
             has_aux: bool = False) -> Callable[..., Any]:
        def wrapper(*args: Any, **kws: Any) -> Any:
            return torch.func.grad(f, argnums=argnums, has_aux=has_aux)(*args, **kws)

        return wrapper

    def value_and_grad(self, f: Callable[..., Any], argnums: Union[int, Sequence[int]] = 0,
                       has_aux: bool = False) -> Callable[..., Tuple[Any, Any]]:
        def wrapper(*args: Any, **kws: Any) -> Any:
            g, v = torch.func.grad_and_value(f, argnums=argnums, has_aux=has_aux)(*args, **kws)
            return v, g

        return wrapper

    def vmap(self, f: Callable[..., Any], vectorized_argnums: Union[int, Sequence[int]] = 0) -> Any:
        if isinstance(vectorized_argnums, int):
            vectorized_argnums = (vectorized_argnums,)

        def wrapper(*args: Any, **kws: Any) -> Tensor:
            in_axes = tuple([0 if i in vectorized_argnums else None for i in range(len(args))])
            return torch.vmap(f, in_axes, 0)(*args, **kws)

        return wrapper

    def vectorized_value_and_grad(self, f: Callable[..., Any], argnums: Union[int, Sequence[int]] = 0,
                                  vectorized_argnums: Union[int, Sequence[int]] = 0,
                                  has_aux: bool = False) -> Callable[..., Tuple[Tensor, Any]]:
        if isinstance(vectorized_argnums, int):
            vectorized_argnums = (vectorized_argnums,)

        def wrapper(*args: Any, **kws: Any) -> Tuple[Tensor, Union[Tensor, Tuple[Tensor, ...]]]:
            jf = self.value_and_grad(f, argnums=argnums, has_aux=has_aux)
            jf = self.vmap(jf, vectorized_argnums=vectorized_argnums)
            vs, gs = jf(*args, **kws)
            if isinstance(argnums, int):
                argnums_list = [argnums]
                gs = [gs]
            else:
                argnums_list = list(argnums)
                gs = list(gs)
            for i, (j, g) in enumerate(zip(argnums_list, gs)):
                if j not in vectorized_argnums:
                    gs[i] = self.tree_map(partial(torch.sum, dim=0), g)
            if isinstance(argnums, int):
                gs = gs[0]
            else:
                gs = tuple(gs)
            return vs, gs

        return wrapper

    vvag = vectorized_value_and_grad

    def __repr__(self) -> str:
        return "pytorch_backend"

    __str__ = __repr__


backend = PyTorchBackend()
