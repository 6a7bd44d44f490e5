"""tensorcircuit_gb300 — a GB300 (sm_103a) statevector engine behind
TensorCircuit's parameterized-circuit API.

Usage mirrors the reference::

    import tensorcircuit_gb300 as tc
    K = tc.set_backend("pytorch")
    c = tc.Circuit(n)
    c.rx(0, theta=t); c.rzz(0, 1, theta=p)
    e = c.expectation_ps(z=[0, 1])
    v, g = K.vvag(f, argnums=0, vectorized_argnums=0)(params)
"""

__version__ = "0.1.0"

from . import channels, gates, interfaces, quantum, torchnn
from .backends import backend
from .circuit import Circuit
from .densitymatrix import DMCircuit, DMCircuit2, DMCircuit_reference
from .cons import (
    dtypestr,
    get_backend,
    get_dtype,
    rdtypestr,
    runtime_backend,
    runtime_contractor,
    runtime_dtype,
    set_backend,
    set_contractor,
    set_dtype,
    set_tensornetwork_backend,
)
from .gates import Gate

__all__ = [
    "Circuit", "DMCircuit", "DMCircuit2", "DMCircuit_reference", "Gate", "backend", "channels", "gates",
    "quantum", "set_backend", "set_dtype", "set_contractor",
    "get_backend", "get_dtype", "runtime_backend", "runtime_dtype", "runtime_contractor", "dtypestr",
    "rdtypestr", "set_tensornetwork_backend",
]


def build() -> str:
    """Compile the native engine library (sm_103a) if its sources changed."""
    from . import _build

    return _build.build()
