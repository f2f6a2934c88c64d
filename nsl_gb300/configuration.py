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
        """lhs + rhs: a deep copy of lhs, then += (Configuration.tpp:108-115)."""
        out = self.copy()
        out += other
        return out

    def __iadd__(self, other):
        """Fields present in both are added, fields only in other are appended (Configuration.tpp:38-58)."""
        for k, v in other.items():
            self[k] = self[k] + v if k in self else (v.clone() if T.is_torch(v) else v.copy())
        return self

    def __sub__(self, other):
        """lhs - rhs: a deep copy of lhs, then -= (Configuration.tpp:122-129)."""
        out = self.copy()
        out -= other
        return out

    def __isub__(self, other):
        """Fields present in both are subtracted, fields only in other are appended negated (Configuration.tpp:65-84)."""
        for k, v in other.items():
            self[k] = self[k] - v if k in self else -v
        return self

    def __mul__(self, s):
        """Every field times a number, on a deep copy (Configuration.tpp:135-158)."""
        return Configuration({k: v * s for k, v in self.items()})

    __rmul__ = __mul__
