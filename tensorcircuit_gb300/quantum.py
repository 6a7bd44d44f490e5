"""Measurement-result formats and Pauli-string helpers.

Restates the reference's converters (tensorcircuit/quantum.py): ``ps2xyz`` /
``xyz2ps`` (:1025-1068), ``sample_int2bin`` / ``sample_bin2int``
(:2104-2134, big-endian: qubit 0 is the most significant bit),
``sample2count`` / ``count_*`` (:2048-2215), ``sample2all`` (:2325-2368),
``measurement_counts`` (:2218-2322) and ``correlation_from_samples`` /
``correlation_from_counts`` (:2400-2445), on torch tensors.
"""

from typing import Any, Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

Tensor = Any


_PS_CODES = (("x", 1), ("y", 2), ("z", 3))


def ps2xyz(ps: List[int]) -> Dict[str, List[int]]:
    """Per-qubit Pauli codes (0 = I, 1 = X, 2 = Y, 3 = Z) to the qubit lists
    of each letter (tensorcircuit/quantum.py:1025-1045)."""
    codes = np.asarray(ps).reshape(-1)
    return {name: [int(i) for i in np.flatnonzero(codes == code)] for name, code in _PS_CODES}


def xyz2ps(xyz: Dict[str, List[int]], n: Optional[int] = None) -> List[int]:
    """Qubit lists per letter to per-qubit codes (tensorcircuit/quantum.py:
    1048-1068).  Only qubits 0..n-1 count; a qubit listed under several
    letters keeps the first of x, y, z."""
    lists = {name: [int(i) for i in xyz.get(name, [])] for name, _ in _PS_CODES}
    if n is None:
        n = max(lists["x"] + lists["y"] + lists["z"]) + 1
    codes = np.zeros(n, dtype=np.int64)
    for name, code in reversed(_PS_CODES):  # x written last, so it wins
        idx = [i for i in lists[name] if 0 <= i < n]
        codes[idx] = code
    return [int(c) for c in codes]


def _t(x: Any) -> torch.Tensor:
    return x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x))


def sample_int2bin(sample: Tensor, n: int) -> Tensor:
    s = _t(sample)
    shifts = torch.arange(n - 1, -1, -1, device=s.device, dtype=s.dtype)
    return torch.bitwise_right_shift(s[..., None], shifts) % 2


def sample_bin2int(sample: Tensor, n: int) -> Tensor:
    s = _t(sample)
    power = torch.tensor([2 ** j for j in reversed(range(n))], device=s.device, dtype=torch.int64)
    return torch.sum(s.to(torch.int64) * power, -1)


def sample2count(sample: Tensor, n: int, jittable: bool = True) -> Tuple[Tensor, Tensor]:
    s = _t(sample)
    return torch.unique(s, return_counts=True)


def count_s2d(srepr: Tuple[Tensor, Tensor], n: int) -> Tensor:
    idx, cnt = _t(srepr[0]), _t(srepr[1])
    out = torch.zeros(2 ** n, dtype=cnt.dtype, device=cnt.device)
    return out.scatter(0, idx.reshape(-1).to(torch.int64), cnt.reshape(-1))


counts_v2t = count_s2d


def count_d2s(drepr: Tensor, eps: float = 1e-7) -> Tuple[Tensor, Tensor]:
    d = _t(drepr)
    mask = torch.abs(d) > eps
    return torch.nonzero(mask).reshape(-1), d[mask]


count_t2v = count_d2s


def count_vector2dict(count: Tensor, n: int, key: str = "bin") -> Dict[Any, int]:
    c = _t(count).detach().cpu().numpy()
    d = {i: c[i].item() for i in range(2 ** n)}
    if key == "int":
        return d
    return {bin(k)[2:].zfill(n): v for k, v in d.items()}


def count_tuple2dict(count: Tuple[Tensor, Tensor], n: int, key: str = "bin") -> Dict[Any, int]:
    a = _t(count[0]).detach().cpu().numpy()
    b = _t(count[1]).detach().cpu().numpy()
    d = {int(i): int(j) for i, j in zip(a, b) if i >= 0}
    if key == "int":
        return d
    return {bin(k)[2:].zfill(n): v for k, v in d.items()}


def sample2all(sample: Tensor, n: int, format: str = "count_vector", jittable: bool = False) -> Any:
    s = _t(sample)
    if s.dim() == 1:
        sample_int = s
        sample_bin = sample_int2bin(s, n)
    elif s.dim() == 2:
        sample_int = sample_bin2int(s, n)
        sample_bin = s
    else:
        raise ValueError("unrecognized tensor shape for sample")
    if format == "sample_int":
        return sample_int
    if format == "sample_bin":
        return sample_bin
    count_tuple = sample2count(sample_int, n, jittable)
    if format == "count_tuple":
        return count_tuple
    if format == "count_vector":
        return count_s2d(count_tuple, n)
    if format == "count_dict_bin":
        return count_tuple2dict(count_tuple, n, key="bin")
    if format == "count_dict_int":
        return count_tuple2dict(count_tuple, n, key="int")
    raise ValueError("unsupported format %s for finite shots measurement" % format)


def measurement_counts(state: Tensor, counts: Optional[int] = 8192, format: str = "count_vector",
                       is_prob: bool = False, random_generator: Optional[Any] = None,
                       status: Optional[Tensor] = None, jittable: bool = False, **kws: Any) -> Any:
    """Sample ``counts`` shots from a state or probability vector with
    torch's ``cumsum``/``searchsorted``, following
    ``backend.probability_sample`` (tensorcircuit/backends/
    abstract_backend.py:1124-1157).  ``Circuit.sample`` uses the engine's
    sampling kernel instead."""
    if "shots" in kws:
        counts = kws.pop("shots")
    st = _t(state)
    if is_prob:
        pi = st / torch.sum(st)
    else:
        st = st / torch.linalg.norm(st)
        pi = torch.real(torch.conj(st) * st)
    pi = pi.reshape(-1)
    d = int(pi.shape[0])
    n = int(np.log(d) / np.log(2) + 1e-8)
    if counts is None or counts <= 0:
        if format == "count_vector":
            return pi
        if format == "count_tuple":
            return count_d2s(pi)
        if format == "count_dict_bin":
            return count_vector2dict(pi, n, key="bin")
        if format == "count_dict_int":
            return count_vector2dict(pi, n, key="int")
        raise ValueError("unsupported format %s for analytical measurement" % format)
    if status is None:
        gen = random_generator if isinstance(random_generator, torch.Generator) else None
        status = torch.rand(counts, generator=gen, device=gen.device if gen is not None else pi.device)
    raw = probability_sample(counts, pi, status)
    return sample2all(raw, n, format=format, jittable=jittable)


measurement_results = measurement_counts


def probability_sample(shots: int, p: Tensor, status: Tensor) -> Tensor:
    """Reference semantics (abstract_backend.py:1124-1157): normalise,
    cumulative sum, ``r = cdf[-1] * (1 - u)``, left ``searchsorted``."""
    p = _t(p)
    u = _t(status).to(device=p.device)
    p = p / torch.sum(p)
    cdf = torch.cumsum(p, 0)
    r = cdf[-1] * (1 - u.to(p.dtype))
    ind = torch.searchsorted(cdf, r)
    return torch.clamp(ind, max=p.shape[0] - 1)


def spin_by_basis(n: int, m: int, elements: Tuple[int, int] = (1, -1)) -> Tensor:
    s = torch.arange(2 ** n)
    bit = torch.bitwise_right_shift(s, n - 1 - m) % 2
    return torch.where(bit == 0, elements[0], elements[1])


def correlation_from_samples(index: Sequence[int], results: Tensor, n: int) -> Tensor:
    r = _t(results)
    if r.dim() == 1:
        r = sample_int2bin(r, n)
    r = 1 - r * 2
    out = r[:, index[0]]
    for i in index[1:]:
        out = out * r[:, i]
    return torch.mean(out.to(torch.float32))


def correlation_from_counts(index: Sequence[int], results: Tensor) -> Tensor:
    r = _t(results).reshape(-1).to(torch.float32)
    r = r / torch.sum(r)
    n = int(np.log(r.shape[0]) / np.log(2))
    for i in index:
        r = r * spin_by_basis(n, i).to(device=r.device, dtype=r.dtype)
    return torch.sum(r)
