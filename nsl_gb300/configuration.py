"""Configuration: a field dictionary with +, -, scalar * (src/NSL/Configuration/Configuration.tpp:56-191)."""
from __future__ import annotations

from . import tensor as T


class Configuration(dict):
    def copy(self, deep: bool = True) -> "Configuration":
        """Configuration(other, true) deep copy (Configuration.tpp)."""
        out = Configuration()
        for k, v in self.items():
            out[k] = (v.clone() if T.is_torch(v) else v.copy()) if deep else v
        return out

    def __add__(self, other):
        out = Configuration(self)
        for k, v in other.items():
            out[k] = out[k] + v if k in out else v
        return out

    def __iadd__(self, other):
        for k, v in other.items():
            self[k] = self[k] + v if k in self else v
        return self

    def __sub__(self, other):
        out = Configuration(self)
        for k, v in other.items():
            out[k] = out[k] - v if k in out else -v
        return out

    def __mul__(self, s):
        return Configuration({k: v * s for k, v in self.items()})

    __rmul__ = __mul__
