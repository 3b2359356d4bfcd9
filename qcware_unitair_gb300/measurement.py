"""Mirror of unitair's measurement module
(src/unitair/simulation/measurement.py:9-140): sampling basis states from
|psi|^2 on the GPU (gbsv_sample) and the histogram type."""
from __future__ import annotations

from collections import OrderedDict
from typing import Optional

import numpy as np
import torch

from . import _core, _lib
from .states import count_qubits


def sample(state: torch.Tensor, num_samples: int,
           seed: Optional[int] = None) -> torch.Tensor:
    """int64 basis indices drawn from |state|^2 (one state, on its device).
    ``seed`` None draws one from torch's CPU generator, so
    torch.manual_seed makes results reproducible."""
    _core.require_cuda(state)
    code = _core.complex_code(state.dtype)
    if state.dim() != 1:
        raise ValueError("measure samples one state; index the batch first")
    if seed is None:
        seed = int(torch.randint(0, 2 ** 62, (1,)).item())
    s = state.contiguous()
    if s.data_ptr() % 16:  # a view at an odd offset: vector loads need 16
        s = s.clone()
    out = torch.empty(int(num_samples), dtype=torch.int64, device=s.device)
    L = _lib.load()
    nbytes = int(L.gbsv_sample_scratch_bytes(s.numel()))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=s.device)
    rc = L.gbsv_sample(s.data_ptr(), code, s.numel(), int(num_samples),
                       int(seed) & (2 ** 64 - 1), out.data_ptr(),
                       scratch.data_ptr(), nbytes, _core.stream_of(s.device))
    _lib.check(rc, "sample")
    return out


def _bits(x: int, n: int) -> str:
    return format(x, f"0{n}b") if n else ""


def measure(state: torch.Tensor, num_samples: int, raw_output: bool = False,
            seed: Optional[int] = None):
    """Draw ``num_samples`` computational-basis outcomes.  Returns a
    MeasurementHistogram (binary-string keys, most frequent first) or, with
    ``raw_output``, a dict {index: count}."""
    n = count_qubits(state)
    idx = sample(state, num_samples, seed).cpu().numpy()
    values, counts = np.unique(idx, return_counts=True)
    if raw_output:
        return {int(v): int(c) for v, c in zip(values, counts)}
    order = np.argsort(-counts, kind="stable")
    hist = MeasurementHistogram(num_qubits=n)
    for i in order:
        hist[_bits(int(values[i]), n)] = int(counts[i])
    return hist


class MeasurementHistogram:
    """Sorted record of measurement outcomes (measurement.py:73-140)."""

    def __init__(self, num_qubits: int,
                 histogram: Optional[OrderedDict] = None):
        self.num_qubits = num_qubits
        self.histogram = OrderedDict() if histogram is None else histogram
        self._int_key_histogram = None

    def __getitem__(self, item: str):
        try:
            return self.histogram[item]
        except KeyError:
            if set(item).issubset({"0", "1"}) and len(item) == self.num_qubits:
                return 0
            raise KeyError(f"Given key {item} is not a valid binary string "
                           f"for {self.num_qubits} bits.") from None

    def __setitem__(self, key, value):
        self.histogram[key] = value

    @property
    def num_distinct_samples(self):
        return len(self.histogram)

    @property
    def observed_samples(self):
        return set(self.histogram)

    def int_key_histogram(self):
        if self._int_key_histogram is None:
            self._int_key_histogram = OrderedDict(
                (int(k, 2) if k else 0, v) for k, v in self.histogram.items())
        return self._int_key_histogram

    def __repr__(self):
        items = list(self.histogram.items())
        short = items[:15] if len(items) >= 50 else items
        text = "\n".join(f"{k}: {v}" for k, v in short)
        if len(items) >= 50:
            text += f"\n ... ({len(items) - 15} lines omitted)"
        return text
