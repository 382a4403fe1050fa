"""Source waveforms evaluated inside the device kernels.

A `Signal` maps time to one value per device. Its parameters are float64
torch tensors with a leading device axis once the signal sits in a source
group (``(N,)``, or ``(B, N)`` for a batch of B circuit instances).

Only the waveforms the Newton hot path evaluates on the GPU are provided:
`Constant`, `Step` and `Pulse` (voltax/signals.py:58-114). Each one has a
fixed kernel code (`kind`) and a fixed parameter order (`fields`) that the
C ABI's device table uses.
"""

from __future__ import annotations

import numpy as np
import torch

_F64 = torch.float64


def _f(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x.to(_F64)
    return torch.as_tensor(np.asarray(x, dtype=np.float64))


class Signal:
    """Base class: ``signal(t) -> value``."""

    kind: int = -1
    fields: tuple[str, ...] = ()

    def params(self) -> list[torch.Tensor]:
        return [getattr(self, f) for f in self.fields]

    def replace_params(self, values) -> "Signal":
        new = object.__new__(type(self))
        for f, v in zip(self.fields, values):
            setattr(new, f, v)
        return new

    def map(self, fn) -> "Signal":
        return self.replace_params([fn(p) for p in self.params()])

    def breakpoints(self, t_stop: float) -> np.ndarray:
        return np.zeros(0)

    def __call__(self, t):  # host-side evaluation (for inspection)
        raise NotImplementedError


class Constant(Signal):
    """A DC value (voltax/signals.py:58-67)."""

    kind = 0
    fields = ("value",)

    def __init__(self, value=0.0):
        self.value = _f(value)

    def __call__(self, t):
        return self.value


class Step(Signal):
    """Linear ramp from `v0` to `v1` starting at `delay`, lasting `rise`
    (voltax/signals.py:70-87)."""

    kind = 1
    fields = ("v0", "v1", "delay", "rise")

    def __init__(self, v0=0.0, v1=1.0, delay=0.0, rise=1e-12):
        self.v0, self.v1, self.delay, self.rise = _f(v0), _f(v1), _f(delay), _f(rise)

    def __call__(self, t):
        frac = torch.clamp((t - self.delay) / self.rise, 0.0, 1.0)
        return self.v0 + (self.v1 - self.v0) * frac

    def breakpoints(self, t_stop):
        d = np.atleast_1d(self.delay.numpy()).ravel()
        r = np.atleast_1d(self.rise.numpy()).ravel()
        times = np.concatenate([d, d + r])
        return np.unique(times[(times >= 0) & (times <= t_stop)])


class Pulse(Signal):
    """SPICE ``PULSE(v1 v2 delay rise fall width period)``
    (voltax/signals.py:90-114)."""

    kind = 2
    fields = ("v1", "v2", "delay", "rise", "fall", "width", "period")

    def __init__(self, v1=0.0, v2=1.0, delay=0.0, rise=1e-9, fall=1e-9, width=1e-6,
                 period=2e-6):
        self.v1, self.v2, self.delay = _f(v1), _f(v2), _f(delay)
        self.rise, self.fall = _f(rise), _f(fall)
        self.width, self.period = _f(width), _f(period)

    def __call__(self, t):
        t = torch.as_tensor(t, dtype=_F64)
        tc = torch.remainder(t - self.delay, self.period)
        up = torch.clamp(tc / (self.rise + 1e-30), 0.0, 1.0)
        t_fall_end = self.rise + self.width + self.fall
        down = torch.clamp((t_fall_end - tc) / (self.fall + 1e-30), 0.0, 1.0)
        value = self.v1 + (self.v2 - self.v1) * torch.minimum(up, down)
        return torch.where(t < self.delay, self.v1, value)

    def breakpoints(self, t_stop):
        """Ramp corners of every period in ``[0, t_stop]``
        (voltax/signals.py:116-125)."""
        out = []
        shape = np.broadcast_shapes(*(np.shape(_np1(x)) for x in
                                      (self.delay, self.rise, self.width, self.fall,
                                       self.period)))
        d, r, w, f, per = (np.broadcast_to(_np1(x), shape).ravel() for x in
                           (self.delay, self.rise, self.width, self.fall, self.period))
        for di, ri, wi, fi, pi in zip(d, r, w, f, per):
            n = max(int((t_stop - di) // pi) + 1, 0) if pi > 0 else 1
            starts = di + pi * np.arange(n)
            for offset in (0.0, ri, ri + wi, ri + wi + fi):
                out.append(starts + offset)
        times = np.concatenate(out) if out else np.zeros(0)
        return np.unique(times[(times >= 0) & (times <= t_stop)])


def _np1(x) -> np.ndarray:
    return np.atleast_1d(torch.as_tensor(x).detach().cpu().numpy().astype(float))


def as_signal(value) -> Signal:
    """Wrap a number as a `Constant`; pass signals through."""
    return value if isinstance(value, Signal) else Constant(value)
