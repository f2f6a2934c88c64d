"""Spatial lattices: the hopping matrix K the fermion matrix is built from (setup, not on the hot path).

Mirrors NSL::Lattice::SpatialLattice (src/NSL/Lattice/lattice.{hpp,tpp}), Ring (Implementations/ring.tpp:8-42) and
Honeycomb (Implementations/honeycomb.tpp:47-138). The honeycomb neighbour search is vectorised over all site pairs
and periodic images instead of the reference's O(N^2) per-pair tensor loop; the rule is the same (minimum squared
distance over the 3x3 images equal to 1 within 1e-4). exp_hopping_matrix(delta) is computed by the GPU library
(scaling and squaring on the device) and memoised per delta like lattice.tpp:52-58.
"""
from __future__ import annotations

import numpy as np


class SpatialLattice:
    def __init__(self, name: str, hops: np.ndarray, sites: np.ndarray):
        self.name = name
        self.hops_ = np.ascontiguousarray(np.asarray(hops, dtype=np.complex128))
        self.sites_ = np.asarray(sites, dtype=np.float64)
        self._exp_memo: dict[complex, np.ndarray] = {}

    def __repr__(self):
        return self.name

    def sites(self) -> int:
        return int(self.hops_.shape[0])

    def hopping_matrix(self, delta: complex = 1.0) -> np.ndarray:
        """lattice.tpp:47-49."""
        return self.hops_ if delta == 1 else self.hops_ * delta

    def adjacency_matrix(self) -> np.ndarray:
        return (np.abs(self.hops_) != 0).astype(np.int32)

    def exp_hopping_matrix(self, delta: complex) -> np.ndarray:
        """exp(delta K), memoised per delta (lattice.tpp:52-58); evaluated on the GPU."""
        d = complex(delta)
        if d not in self._exp_memo:
            from .fermion_matrix import HubbardExp

            fm = HubbardExp(self, 1, beta=1.0)
            self._exp_memo[d] = fm.exp_hopping_matrix(d)
        return self._exp_memo[d]

    def set_exp_hopping_matrix(self, delta: complex, expK: np.ndarray):
        """Installs an externally computed exp(delta K) (e.g. the reference's own memo entry)."""
        self._exp_memo[complex(delta)] = np.ascontiguousarray(np.asarray(expK, dtype=np.complex128))

    def bipartite(self) -> bool:
        """Two-colouring by breadth-first search (lattice.tpp:76-139)."""
        adj = self.adjacency_matrix()
        n = adj.shape[0]
        part = {}
        for head in range(n):
            if head in part:
                continue
            part[head] = 1
            todo = [head]
            while todo:
                cur = todo.pop(0)
                for nb in np.nonzero(adj[cur])[0]:
                    nb = int(nb)
                    if nb == cur:
                        continue
                    if nb not in part:
                        part[nb] = -part[cur]
                        todo.append(nb)
                    elif part[nb] == part[cur]:
                        return False
        return True


class Ring(SpatialLattice):
    """Ring(n, kappa, radius): ring.tpp:8-42."""

    def __init__(self, n: int, kappa: complex = 1.0, radius: float = 1.0):
        n = int(n)
        K = np.zeros((n, n), dtype=np.complex128)
        if n > 1:
            i = np.arange(n - 1)
            K[i, i + 1] = kappa
            K[i + 1, i] = np.conj(kappa)
            K[0, n - 1] = np.conj(kappa)
            K[n - 1, 0] = kappa
        th = 2 * np.pi / n * np.arange(n)
        sites = np.stack([radius * np.cos(th), radius * np.sin(th), np.zeros(n)], axis=1)
        super().__init__(f"Ring({n})", K, sites)


class Honeycomb(SpatialLattice):
    """Honeycomb(L=(L1, L2), kappa): periodic honeycomb of L1*L2 unit cells, 2 sites each (honeycomb.tpp:72-138)."""

    A = np.array([[1.5, 0.8660254037844386], [1.5, -0.8660254037844386]])

    def __init__(self, L=(3, 3), kappa: complex = 1.0):
        L1, L2 = int(L[0]), int(L[1])
        l1, l2 = np.meshgrid(np.arange(L1), np.arange(L2), indexing="ij")
        cell = (l1.T.reshape(-1)[:, None] * self.A[0] + l2.T.reshape(-1)[:, None] * self.A[1])  # i = l1 + L1*l2
        r = np.array([1.0, 0.0])
        sites = np.empty((2 * L1 * L2, 2))
        sites[0::2] = cell + r / 2
        sites[1::2] = cell - r / 2
        T1, T2 = L1 * self.A[0], L2 * self.A[1]
        diff = sites[:, None, :] - sites[None, :, :]
        best = np.full(diff.shape[:2], float((T1 + T2) @ (T1 + T2)))
        for s1 in (-1, 0, 1):
            for s2 in (-1, 0, 1):
                v = diff + s1 * T1 + s2 * T2
                best = np.minimum(best, np.einsum("ijk,ijk->ij", v, v))
        K = np.where(np.abs(best - 1.0) < 1e-4, kappa, 0).astype(np.complex128)
        np.fill_diagonal(K, 0)
        super().__init__(f"Honeycomb({L1}, {L2})", K, sites)
        self.L = (L1, L2)
        self.unit_cells = L1 * L2
