"""CPU oracle for the NSL fermion-matrix hot path: TEST INFRASTRUCTURE ONLY.

A plain numpy (complex128) restatement of the reference algorithms, used by tests/ to check the CUDA path, by
``__graft_entry__.smoke()`` to check its result and by ``bench.py`` as the timed CPU baseline (``kind: "port"``). The
product (``nsl_gb300``) never imports this module.

Parity of this restatement with the reference itself is pinned by tests/test_oracle_golden.py against the fixtures in
tests/golden/, which the reference NSL code produced on libtorch's CPU complex128 path
(oracle/ref_harness/golden_harness.cpp, tests/golden/make_golden.py).

Every function names the reference file:line it follows (paths inside the NSL source tree).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.linalg

PARTICLE, HOLE = 0, 1


# ----------------------------------------------------------------------------------------------------------------
# Lattices (setup only)
# ----------------------------------------------------------------------------------------------------------------
def ring_hops(n: int, kappa: complex = 1.0) -> np.ndarray:
    """Ring hopping matrix: src/NSL/Lattice/Implementations/ring.tpp:8-42."""
    K = np.zeros((n, n), dtype=np.complex128)
    for i in range(n - 1):
        K[i, i + 1] = kappa
    for i in range(1, n):
        K[i, i - 1] = np.conj(kappa)
    if n > 1:
        K[0, n - 1] = np.conj(kappa)
        K[n - 1, 0] = kappa
    return K


def honeycomb_sites(L1: int, L2: int) -> np.ndarray:
    """Site coordinates: src/NSL/Lattice/Implementations/honeycomb.tpp:73-95 (A/B sublattice interleaved)."""
    a = np.array([[1.5, 0.8660254037844386], [1.5, -0.8660254037844386]])
    r = np.array([1.0, 0.0])
    sites = np.zeros((2 * L1 * L2, 2))
    for l1 in range(L1):
        for l2 in range(L2):
            i = l1 + L1 * l2
            base = l1 * a[0] + l2 * a[1]
            sites[2 * i + 0] = base + r / 2
            sites[2 * i + 1] = base - r / 2
    return sites


def honeycomb_hops(L1: int, L2: int, kappa: complex = 1.0) -> np.ndarray:
    """Honeycomb hopping matrix with periodic images: honeycomb.tpp:47-116.

    A pair (i, j) hops when its minimum squared distance over the 3x3 periodic images is 1 (within 1e-4).
    """
    a = np.array([[1.5, 0.8660254037844386], [1.5, -0.8660254037844386]])
    sites = honeycomb_sites(L1, L2)
    T1, T2 = L1 * a[0], L2 * a[1]
    n = len(sites)
    K = np.zeros((n, n), dtype=np.complex128)
    far = float((T1 + T2) @ (T1 + T2))
    for i in range(n):
        for j in range(i, n):
            best = far
            for s1 in (-1, 0, 1):
                for s2 in (-1, 0, 1):
                    v = sites[i] - sites[j] + s1 * T1 + s2 * T2
                    best = min(best, float(v @ v))
            if abs(best - 1.0) < 1e-4:
                K[i, j] = kappa
                K[j, i] = kappa
    return K


def exp_hopping_matrix(K: np.ndarray, delta: complex) -> np.ndarray:
    """exp(delta*K): src/NSL/Lattice/lattice.tpp:52-58 (torch::matrix_exp); here scipy's Pade expm."""
    return scipy.linalg.expm(np.asarray(delta) * K)


# ----------------------------------------------------------------------------------------------------------------
# Fermion matrix, exponential discretisation
# ----------------------------------------------------------------------------------------------------------------
def _roll_t(x: np.ndarray, shift: int, boundary: complex | None) -> np.ndarray:
    """NSL::Tensor::shift along the time axis (dim -2): src/NSL/Tensor/Impl/shift.tpp:59-71.

    roll by `shift`; with a boundary factor, the `shift` wrapped slices at the front (shift>0) or back (shift<0)
    are multiplied by it.
    """
    out = np.roll(x, shift, axis=-2)
    if boundary is not None:
        if shift > 0:
            out[..., :shift, :] *= boundary
        elif shift < 0:
            out[..., out.shape[-2] + shift:, :] *= boundary
    return out


def _udt_product(mats, chunk: int):
    """mats[0] @ mats[1] @ ... @ mats[-1] as (Q, d, T): Q unitary, d > 0 the graded scales, T well conditioned.

    Accumulated from the right end, `chunk` factors multiplied directly per step, then a column-pivoted QR of
    (chunk product) Q diag(d) separates the scales again (the standard stratification of long matrix chains)."""
    n = mats[0].shape[0]
    Q = np.eye(n, dtype=np.complex128)
    d = np.ones(n)
    T = np.eye(n, dtype=np.complex128)
    end = len(mats)
    while end > 0:
        start = max(0, end - chunk)
        C = np.eye(n, dtype=np.complex128)
        for j in range(start, end):
            C = C @ mats[j]
        end = start
        W = (C @ Q) * d[None, :]
        Qn, Rn, P = scipy.linalg.qr(W, pivoting=True)
        dn = np.abs(np.diag(Rn))
        dn[dn == 0] = np.finfo(float).tiny
        Pinv = np.empty_like(P)
        Pinv[P] = np.arange(len(P))
        T = (Rn / dn[:, None])[:, Pinv] @ T
        Q, d = Qn, dn
    return Q, d, T


class HubbardExp:
    """src/NSL/FermionMatrix/Impl/hubbardExp.hpp:33-233 and hubbardExp.tpp:12-211."""

    def __init__(self, K: np.ndarray, Nt: int, beta: complex = 1.0, mu: complex = 0.0, species: int = PARTICLE):
        # hubbardExp.hpp:48-76: delta = beta/Nt, mu_ = delta*mu
        self.K = np.asarray(K, dtype=np.complex128)
        self.Nt = Nt
        self.Nx = self.K.shape[0]
        self.delta = complex(beta) / Nt
        self.mu = complex(beta) / Nt * complex(mu)
        self.species = species
        self.sgn = 1 if species == PARTICLE else -1
        self._memo: dict[complex, np.ndarray] = {}

    # lattice.tpp:52-58 memo keyed by delta
    def expK(self, d: complex) -> np.ndarray:
        d = complex(d)
        if d not in self._memo:
            self._memo[d] = exp_hopping_matrix(self.K, d)
        return self._memo[d]

    def set_expK(self, d: complex, E: np.ndarray):
        self._memo[complex(d)] = np.asarray(E, dtype=np.complex128)

    def populate(self, phi: np.ndarray, species: int | None = None):
        """hubbardExp.hpp:103-128."""
        if species is not None:
            self.species = species
            self.sgn = 1 if species == PARTICLE else -1
        self.phi = np.array(phi, dtype=np.complex128)
        s = self.sgn
        self.phiExp = np.exp(1j * s * self.phi + s * self.mu)
        self.phiExpInv = np.exp(-1j * s * self.phi - s * self.mu)

    def set_phases(self, phiExp: np.ndarray):
        """Replaces phiExp (and phiExpInv) by given values, e.g. another implementation's FP64 rounding of the same
        exponentials, so that both evaluate bit-identical operators."""
        self.phiExp = np.array(phiExp, dtype=np.complex128)
        self.phiExpInv = 1.0 / self.phiExp

    @staticmethod
    def _matvec(E: np.ndarray, v: np.ndarray) -> np.ndarray:
        # mat_vec(E, v^T)^T over the last (space) axis: out[..., t, x] = sum_y E[x, y] v[..., t, y]
        return v @ E.T

    def F_(self, psi):
        """hubbardExp.tpp:13-36."""
        Fpsi = self._matvec(self.expK(self.sgn * self.delta), self.phiExp * psi)
        return _roll_t(Fpsi, 1, -1.0)

    def M(self, psi):
        """hubbardExp.tpp:39-41."""
        return psi - self.F_(psi)

    def Mdagger(self, psi):
        """hubbardExp.tpp:44-75."""
        B = self._matvec(self.expK(self.sgn * np.conj(self.delta)), psi)
        B = _roll_t(B, -1, -1.0)
        return psi - np.conj(self.phiExp) * B

    def MMdagger(self, psi):
        """hubbardExp.tpp:78-104 (4 products, as the reference evaluates it)."""
        S = _roll_t(self.phiExp * np.conj(self.phiExp), 1, None)
        inner = self._matvec(self.expK(self.sgn * np.conj(self.delta)), psi)
        return (self.M(psi) + self.Mdagger(psi) - psi) + self._matvec(self.expK(self.sgn * self.delta), S * inner)

    def MdaggerM(self, psi):
        """hubbardExp.tpp:107-125."""
        E2 = self.expK(self.sgn * (np.conj(self.delta) + self.delta))
        return self.M(psi) + self.Mdagger(psi) - psi + np.conj(self.phiExp) * self._matvec(E2, self.phiExp * psi)

    def time_slices_logdet(self):
        """B_t = exp(sgn delta K) diag(phiExp[(t+1) % Nt]): the `prod` tensor of hubbardExp.tpp:142."""
        E = self.expK(self.sgn * self.delta)
        pe = np.roll(self.phiExp, -1, axis=0)
        return E[None, :, :] * pe[:, None, :]

    def sausage(self):
        """B_{Nt-1} ... B_0 accumulated left to right as in hubbardExp.tpp:145-147."""
        prod = self.time_slices_logdet()
        S = np.eye(self.Nx, dtype=np.complex128)
        for t in range(self.Nt - 1, -1, -1):
            S = S @ prod[t]
        return S

    def logDetM(self):
        """hubbardExp.tpp:129-150 with LinAlg::logdet = log(det(.)) (src/NSL/LinAlg/det.tpp:15-20)."""
        A = np.eye(self.Nx) + self.sausage()
        return complex(np.log(np.linalg.det(A)))

    def logDetM_lu(self):
        """Same matrix, log-determinant as the sum of the logs of the LU pivots (no overflow of det)."""
        A = np.eye(self.Nx) + self.sausage()
        lu, piv = scipy.linalg.lu_factor(A)
        d = np.diag(lu)
        nswap = int(np.sum(piv != np.arange(len(piv))))
        val = np.sum(np.log(d)) + (1j * np.pi if nswap % 2 else 0.0)
        return complex(val)

    def logDetM_stable(self, chunk: int = 4):
        """log det(1 + B_{Nt-1}...B_0) with a QR-stratified (UDT) product, stable at large beta.

        Restates the standard stratification: the product is kept as Q diag(d) T with Q unitary and the scales d
        separated; 1 + Q D T is factored as Q (Q^H T^{-1} D_b^{-1} + D_s) D_b T with D = D_b D_s (big and small
        parts), so no O(exp(beta |K|)) entries are ever summed with O(1) ones.
        """
        prod = self.time_slices_logdet()
        Nx = self.Nx
        Q = np.eye(Nx, dtype=np.complex128)
        d = np.ones(Nx)
        T = np.eye(Nx, dtype=np.complex128)
        t = 0
        while t < self.Nt:
            C = np.eye(Nx, dtype=np.complex128)
            for s in range(t, min(t + chunk, self.Nt)):
                C = prod[s] @ C
            t += chunk
            # new product = C Q D T ; factor (C Q D) = Q' R' with column pivoting -> D' = |diag R'|
            W = (C @ Q) * d[None, :]
            Qn, Rn, P = scipy.linalg.qr(W, pivoting=True)
            dn = np.abs(np.diag(Rn))
            dn[dn == 0] = np.finfo(float).tiny
            Tn = (Rn / dn[:, None])
            Pinv = np.empty_like(P)
            Pinv[P] = np.arange(len(P))
            Tn = Tn[:, Pinv] @ T
            Q, d, T = Qn, dn, Tn
        db = np.maximum(d, 1.0)
        ds = np.minimum(d, 1.0)
        Mid = (Q.conj().T @ np.linalg.inv(T)) / db[None, :] + np.diag(ds)
        s1, l1 = np.linalg.slogdet(Q)
        s2, l2 = np.linalg.slogdet(Mid)
        s3, l3 = np.linalg.slogdet(T)
        return complex(l1 + l2 + l3 + np.sum(np.log(db)) + 1j * (np.angle(s1) + np.angle(s2) + np.angle(s3)))

    def time_slices_force(self):
        """Fk(t) = diag(phiExpInv[(t - 1) mod Nt]) exp(-sgn delta K): the Fk tensor of hubbardExp.tpp:162-168."""
        E = self.expK(-1 * self.sgn * self.delta)
        pinv = np.roll(self.phiExpInv, 1, axis=0)
        return pinv[:, :, None] * E[None, :, :]

    def equal_time_green_stable(self, s: int, chunk: int = 4):
        """G(s) = (1 + C(s))^{-1} with C(s) = Fk(s) Fk(s+1) ... Fk(Nt-1) Fk(0) ... Fk(s-1), QR-stratified.

        Not a reference function: the stable restatement of what hubbardExp.tpp:153-211 evaluates directly. The
        gradient of log det M is i (1 - diag G(t + 1)) at slice t (the reference's pi_dot, by the push-through identity
        S(t+1) (1 + Q(t) S(t+1))^{-1} Q(t) = 1 - (1 + S(t+1) Q(t))^{-1}), and G(t + 1) = 1 - [M^{-1}]_{tt}. The
        product is accumulated from the right as Q diag(d) T, `chunk` factors at a time, with a column-pivoted QR per
        chunk (scales in d, Q unitary, T well conditioned); then 1 + Q D T = Q D_b (D_b^{-1} Q^H T^{-1} + D_s) T
        with D = D_b D_s (parts above and below 1) is inverted without adding O(e^{beta |K|}) to O(1) entries.
        """
        Fk = self.time_slices_force()
        Nt = self.Nt
        mats = [Fk[(s + j) % Nt] for j in range(Nt)]
        Q, d, T = _udt_product(mats, chunk)
        db = np.maximum(d, 1.0)
        ds = np.minimum(d, 1.0)
        Tinv = np.linalg.inv(T)
        Qh = Q.conj().T
        X = (Qh @ Tinv) / db[:, None] + np.diag(ds)
        return Tinv @ np.linalg.solve(X, Qh / db[:, None])

    def gradLogDetM_stable(self, chunk: int = 4, slices=None):
        """d log det M / d phi (Nt, Nx) from the stratified equal-time Green functions (equal_time_green_stable):
        row t = i (1 - diag G(t + 1)). `slices` restricts the rows evaluated (the others are NaN)."""
        Nt = self.Nt
        out = np.full((Nt, self.Nx), np.nan + 0j)
        for t in (range(Nt) if slices is None else slices):
            G = self.equal_time_green_stable((t + 1) % Nt, chunk)
            out[t] = 1j * (1.0 - np.diag(G))
        return out

    def gradLogDetM(self):
        """hubbardExp.tpp:153-211."""
        Nt, Nx = self.Nt, self.Nx
        E = self.expK(-1 * self.sgn * self.delta)
        pinv = np.roll(self.phiExpInv, 1, axis=0)                  # shift(phiExpInv, +1): row t = phiExpInv[t-1]
        Fk = pinv[:, :, None] * E[None, :, :]                      # Fk(t) = diag(pinv[t]) E
        FkFkFk = np.empty_like(Fk)
        FkFkFk[Nt - 1] = Fk[Nt - 1]
        for t in range(Nt - 2, -1, -1):
            FkFkFk[t] = Fk[t] @ FkFkFk[t + 1]
        invAp1F = np.linalg.inv(np.eye(Nx) + FkFkFk[0])
        pi_dot = np.empty((Nt, Nx), dtype=np.complex128)
        pi_dot[Nt - 1] = 1j * np.diag(FkFkFk[0] @ invAp1F)
        for t in range(Nt - 1):
            invAp1F = invAp1F @ Fk[t]
            pi_dot[t] = 1j * np.einsum("xk,kx->x", FkFkFk[t + 1], invAp1F)
        return pi_dot

    def M_dense(self):
        """Dense (Nt,Nx,Nt,Nx) matrix by applying M to unit vectors: src/NSL/FermionMatrix/fermionMatrix.hpp:87-110."""
        n = self.Nt * self.Nx
        I = np.eye(n, dtype=np.complex128).reshape(n, self.Nt, self.Nx)
        cols = self.M(I)                                            # (n, Nt, Nx): column j = M e_j
        return cols.reshape(n, n).T.reshape(self.Nt, self.Nx, self.Nt, self.Nx)


class HubbardDiag(HubbardExp):
    """src/NSL/FermionMatrix/Impl/hubbardDiag.{hpp,tpp}: the diagonal discretisation,
    (M psi)_t = psi_t - sgn delta K psi_t - B_t exp(i sgn phi_{t-1} + sgn mu~) psi_{t-1}, B_0 = -1.

    The reference writes its operators for one (Nt, Nx) vector (shift along dimension 0, slice 0 of dimension 0);
    here the time axis is -2 and a leading batch axis holds independent right-hand sides, which is what the
    reference computes one vector at a time.
    """

    def K_(self, d):
        # SpatialLattice::hopping_matrix(d) = d K (lattice.tpp:47-49)
        return complex(d) * self.K

    def time_slices_force(self):
        raise NotImplementedError("the stratified forms are written for the exponential discretisation")


    def M(self, psi):
        """hubbardDiag.tpp:10-37."""
        out = _roll_t(self.phiExp * psi, 1, -1.0)
        out = out + self._matvec(self.K_(self.sgn * self.delta), psi)
        return psi - out

    def Mdagger(self, psi):
        """hubbardDiag.tpp:40-71."""
        B = np.conj(self.phiExp) * _roll_t(_neg_first(psi), -1, None)
        return psi - self._matvec(self.K_(self.sgn * np.conj(self.delta)), psi) - B

    def MMdagger(self, psi):
        """hubbardDiag.tpp:74-118 (the reference's expanded form)."""
        K1, K2 = self.K_(self.sgn * self.delta), self.K_(self.sgn * np.conj(self.delta))
        out = self.M(psi) + self.Mdagger(psi) - psi + self._matvec(K1, self._matvec(K2, psi))
        out = out + self._matvec(K1, np.conj(self.phiExp) * _roll_t(_neg_first(psi), -1, None))
        B = _roll_t(self.phiExp * self._matvec(K2, psi), 1, -1.0)
        S = _roll_t(self.phiExp * np.conj(self.phiExp), 1, None)
        return out + B + S * psi

    def MdaggerM(self, psi):
        """hubbardDiag.tpp:121-165 (the reference's expanded form)."""
        K1, K2 = self.K_(self.sgn * self.delta), self.K_(self.sgn * np.conj(self.delta))
        out = self.M(psi) + self.Mdagger(psi) - psi + self._matvec(K1, self._matvec(K2, psi))
        out = out + np.conj(self.phiExp) * self._matvec(K1, _roll_t(_neg_first(psi), -1, None))
        B = _roll_t(self._matvec(K2, self.phiExp * psi), 1, -1.0)
        return out + B + (self.phiExp * np.conj(self.phiExp)) * psi

    def slice_matrices(self, shift):
        """(1 - sgn delta K) with its columns (logDetM) or rows (gradLogDetM) scaled by phiExpInv rolled by `shift`."""
        return np.roll(self.phiExpInv, shift, axis=0), np.eye(self.Nx) - self.K_(self.sgn * self.delta)

    def sausage(self):
        """fk_0 fk_1 ... fk_{Nt-1}, fk_t = (1 - sgn delta K) diag(phiExpInv[t+1]) (hubbardDiag.tpp:176-187)."""
        pinv, A = self.slice_matrices(-1)
        S = np.eye(self.Nx, dtype=np.complex128)
        for t in range(self.Nt):
            S = S @ (A * pinv[t][None, :])
        return S

    def logDetM(self):
        """hubbardDiag.tpp:169-193: i sgn sum(phi) + log det(1 + sausage), the second on the principal branch."""
        return complex(1j * self.sgn * np.sum(self.phi) + np.log(np.linalg.det(np.eye(self.Nx) + self.sausage())))

    def gradLogDetM(self):
        """hubbardDiag.tpp:197-250: the HubbardExp algorithm with Fk(t) = diag(phiExpInv[t-1]) (1 - sgn delta K)."""
        Nt, Nx = self.Nt, self.Nx
        pinv, A = self.slice_matrices(1)
        Fk = pinv[:, :, None] * A[None, :, :]
        FkFkFk = np.empty_like(Fk)
        FkFkFk[Nt - 1] = Fk[Nt - 1]
        for t in range(Nt - 2, -1, -1):
            FkFkFk[t] = Fk[t] @ FkFkFk[t + 1]
        invAp1F = np.linalg.inv(np.eye(Nx) + FkFkFk[0])
        pi_dot = np.empty((Nt, Nx), dtype=np.complex128)
        pi_dot[Nt - 1] = 1j * np.diag(FkFkFk[0] @ invAp1F)
        for t in range(Nt - 1):
            invAp1F = invAp1F @ Fk[t]
            pi_dot[t] = 1j * np.einsum("xk,kx->x", FkFkFk[t + 1], invAp1F)
        return pi_dot


def _neg_first(psi):
    """A copy of psi with time slice 0 negated (the reference's `x(0, Slice()) *= -1` on one (Nt, Nx) vector)."""
    out = np.array(psi, dtype=np.complex128, copy=True)
    out[..., 0, :] *= -1.0
    return out


# ----------------------------------------------------------------------------------------------------------------
# Solver
# ----------------------------------------------------------------------------------------------------------------
def inner_product(a, b) -> complex:
    """src/NSL/LinAlg/inner_product.tpp:30-33: sum(conj(a) * b) over every element."""
    return complex(np.sum(np.conj(a) * b))


def cg(op, b, eps: float = 1e-12, max_iter: int = 10000, x0=None):
    """CG exactly as src/NSL/LinAlg/Solver/Impl/CG.tpp:15-113.

    x0 defaults to b (CG.tpp:98-103); stops when the recurrence residual |r|^2 <= eps^2 (CG.tpp:70); on
    exhaustion returns x without raising (CG.tpp:90-93). Returns (x, iterations, converged).
    """
    x = np.array(b if x0 is None else x0, dtype=np.complex128, copy=True)
    errSq = eps * eps
    t = op(x)
    r = b - t
    rsqr_prev = inner_product(r, r).real
    if rsqr_prev <= errSq:
        return x, 0, True
    p = r.copy()
    for count in range(1, max_iter + 1):
        t = op(p)
        alpha = rsqr_prev / inner_product(p, t)
        x += alpha * p
        r -= alpha * t
        rsqr_curr = inner_product(r, r).real
        if rsqr_curr <= errSq:
            return x, count, True
        beta = rsqr_curr / rsqr_prev
        p = r + beta * p
        rsqr_prev = rsqr_curr
    return x, max_iter, False


def cg_per_rhs(op, b, eps: float = 1e-12, max_iter: int = 10000):
    """Independent CG per right-hand side (leading axis), each with the reference's stopping rule."""
    xs, its = [], []
    for i in range(b.shape[0]):
        x, n, _ = cg(lambda v: op(v[None])[0], b[i], eps, max_iter)
        xs.append(x)
        its.append(n)
    return np.stack(xs), its


# ----------------------------------------------------------------------------------------------------------------
# Double-double residuals and the certified CG (not reference functions: they certify true residuals below what FP64
# can hold at low temperature, where |A| |x| / |b| ~ 1e7..1e8)
# ----------------------------------------------------------------------------------------------------------------
_SPLIT = 134217729.0  # 2^27 + 1 (Dekker's splitting constant)


def _two_sum(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _two_prod(a, b):
    """a b = p + e exactly (Dekker 1971, without FMA)."""
    p = a * b
    ca = _SPLIT * a
    ah = ca - (ca - a)
    al = a - ah
    cb = _SPLIT * b
    bh = cb - (cb - b)
    bl = b - bh
    return p, ((ah * bh - p) + ah * bl + al * bh) + al * bl


def _dd_add(ah, al, bh, bl):
    s, e = _two_sum(ah, bh)
    e = e + (al + bl)
    h = s + e
    return h, e - (h - s)


def _dd_mul_c(ph, zh, zl):
    """p z for p complex FP64 and z = zh + zl complex double-double: returns (hi, lo) complex arrays."""
    pr, pi = np.real(ph), np.imag(ph)
    parts = []
    for (a, b, sgn) in ((pr, np.real(zh), 1), (pi, np.imag(zh), -1), (pr, np.imag(zh), 1), (pi, np.real(zh), 1)):
        p, e = _two_prod(a, b)
        parts.append((sgn * p, sgn * e))
    rh, rl = _dd_add(parts[0][0], parts[0][1], parts[1][0], parts[1][1])
    ih, il = _dd_add(parts[2][0], parts[2][1], parts[3][0], parts[3][1])
    # the low part of z times p in FP64 (its error is below 1e-32 of |p z|)
    lo = ph * zl
    rh, rl = _dd_add(rh, rl, np.real(lo), 0.0)
    ih, il = _dd_add(ih, il, np.imag(lo), 0.0)
    return rh + 1j * ih, rl + 1j * il


def _slices(a, nbits: int, count: int):
    """Ozaki splitting of the rows of a real array (last axis = the summation axis): a = sum of `count` slices, each
    a multiple of 2^(e - nbits k) with at most nbits significant bits relative to its row maximum 2^e."""
    out = []
    r = np.array(a, dtype=np.float64, copy=True)
    m = np.max(np.abs(r), axis=-1, keepdims=True)
    e = np.ceil(np.log2(np.where(m > 0, m, 1.0)))
    for k in range(count):
        sigma = np.exp2(e + 52 - nbits * (k + 1) + 1)
        s1 = (r + sigma) - sigma
        out.append(s1)
        r = r - s1
    return out, r


def _matvec_dd(E: np.ndarray, vh: np.ndarray, vl: np.ndarray):
    """out[..., x] = sum_y E[x, y] (vh + vl)[..., y] in double-double: the products of 20-bit slices of E and vh are
    exact in FP64 and so are their sums over <= 2048 sites; the slices are then added with two-sums."""
    assert E.shape[0] <= 2048
    Es = []
    for part in ((E.real,) if not np.iscomplexobj(E) or not np.any(E.imag) else (E.real, E.imag)):
        Es.append(_slices(part, 20, 3))
    real_E = len(Es) == 1

    def real_matvec(Esplit, w):
        # entries far below a row's maximum keep bits beyond the three slices (Erest, wrest); their products are
        # below 2^-60 of the row's scale and are added in FP64
        Esl, Erest = Esplit
        wsl, wrest = _slices(w, 20, 3)
        hi = np.zeros(w.shape[:-1] + (E.shape[0],))
        lo = np.zeros_like(hi)
        for a in range(3):
            for b in range(3):
                hi, lo = _dd_add(hi, lo, wsl[b] @ Esl[a].T, 0.0)
        full = sum(Esl) + Erest
        hi, lo = _dd_add(hi, lo, wrest @ full.T + sum(wsl) @ Erest.T, 0.0)
        return hi, lo

    out = []
    for comp in (vh.real, vh.imag):
        parts = [real_matvec(Esl, comp) for Esl in Es]
        out.append(parts)
    Ef = E.real if real_E else E
    low = vl @ Ef.T  # the low part in FP64
    rr = out[0][0]
    ri = out[1][0]
    if not real_E:  # (Er + i Ei)(vr + i vi) = (Er vr - Ei vi) + i (Er vi + Ei vr)
        ei_vr, ei_vi = out[0][1], out[1][1]
        rr = _dd_add(rr[0], rr[1], -ei_vi[0], -ei_vi[1])
        ri = _dd_add(ri[0], ri[1], ei_vr[0], ei_vr[1])
    rh, rl = _dd_add(rr[0], rr[1], np.real(low), 0.0)
    ih, il = _dd_add(ri[0], ri[1], np.imag(low), 0.0)
    return rh + 1j * ih, rl + 1j * il


def _roll_dd(h, l, shift, boundary):
    return _roll_t(h, shift, boundary), _roll_t(l, shift, boundary)


def apply_dd(hfm: HubbardExp, op: str, xh, xl):
    """(hi, lo) = op (xh + xl) in double-double for op in M, Mdagger, MMdagger, MdaggerM (hubbardExp.tpp:13-125
    with the handle's FP64 exp(delta K) and phases)."""
    if op == "MMdagger":
        return apply_dd(hfm, "M", *apply_dd(hfm, "Mdagger", xh, xl))
    if op == "MdaggerM":
        return apply_dd(hfm, "Mdagger", *apply_dd(hfm, "M", xh, xl))
    xh = np.asarray(xh, dtype=np.complex128)
    xl = np.asarray(xl, dtype=np.complex128)
    if op == "M":
        wh, wl = _dd_mul_c(hfm.phiExp, xh, xl)
        zh, zl = _matvec_dd(hfm.expK(hfm.sgn * hfm.delta), wh, wl)
        zh, zl = _roll_dd(zh, zl, 1, -1.0)
    else:
        zh, zl = _matvec_dd(hfm.expK(hfm.sgn * np.conj(hfm.delta)), xh, xl)
        zh, zl = _roll_dd(zh, zl, -1, -1.0)
        zh, zl = _dd_mul_c(np.conj(hfm.phiExp), zh, zl)
    rh, rl = _dd_add(xh.real, xl.real, -zh.real, -zl.real)
    ih, il = _dd_add(xh.imag, xl.imag, -zh.imag, -zl.imag)
    return rh + 1j * ih, rl + 1j * il


def residual_dd(hfm: HubbardExp, op: str, b, xh, xl):
    """b - op (xh + xl) in double-double, rounded to FP64."""
    th, tl = apply_dd(hfm, op, xh, xl)
    rh, rl = _dd_add(np.real(b), 0.0, -th.real, -tl.real)
    ih, il = _dd_add(np.imag(b), 0.0, -th.imag, -tl.imag)
    return (rh + rl) + 1j * (ih + il)


def _dd_fold(xh, xl, x):
    """(xh + xl) + x for complex double-double (xh, xl) and complex FP64 x."""
    rh, rl = _dd_add(xh.real, xl.real, x.real, 0.0)
    ih, il = _dd_add(xh.imag, xl.imag, x.imag, 0.0)
    return rh + 1j * ih, rl + 1j * il


def cg_certified(hfm: HubbardExp, op: str, b, eps: float, max_iter: int = 200000, update: float = 1e-4,
                 rebase: float = 1e-5):
    """CG on one system (the reference's iteration, CG.tpp:15-95, in FP64) with FP64 reliable updates and
    double-double rebases, stopping when the double-double true residual |b - A (xh + xl)| <= eps.

    The solution is xh + xl + x, x the FP64 increment since the last rebase; a reliable update replaces r by
    bseg - A x (FP64) once |r|^2 fell `update` below its maximum since the last update; a rebase folds x into the pair
    and sets r = bseg = b - A (xh + xl) in double-double once the update's |r| fell `rebase` below |bseg|, stopped
    improving, or met eps. Returns (xh, xl, iterations, rebases, |b - A (xh + xl)|)."""
    A = getattr(hfm, op)
    b = np.asarray(b, dtype=np.complex128)
    xh = np.zeros_like(b)
    xl = np.zeros_like(b)
    x = np.zeros_like(b)
    bseg = b.copy()
    r = b.copy()
    p = r.copy()
    rr = float(np.vdot(r, r).real)
    base = best = maxr = rr
    stall = 0
    it = rebases = 0
    while it < max_iter:
        t = A(p)
        alpha = rr / np.vdot(p, t)
        x += alpha * p
        r -= alpha * t
        rn = float(np.vdot(r, r).real)
        it += 1
        if rn <= eps * eps or rn < update * maxr:
            rt = bseg - A(x)
            rn_t = float(np.vdot(rt, rt).real)
            no_gain = not rn_t < 0.25 * best
            if rn_t <= eps * eps or rn_t <= rebase ** 2 * base or (no_gain and stall >= 1):
                xh, xl = _dd_fold(xh, xl, x)
                x[...] = 0
                rt = residual_dd(hfm, op, b, xh, xl)
                bseg = rt.copy()  # r is updated in place below
                rn_t = float(np.vdot(rt, rt).real)
                rebases += 1
                if rn_t <= eps * eps:
                    return xh, xl, it, rebases, float(np.sqrt(rn_t))
                base = rn_t
            if rn_t < 0.25 * best:
                best, stall = rn_t, 0
            else:
                best, stall = min(best, rn_t), stall + 1
            beta = rn_t / rr
            r = rt
            rr = rn_t
            maxr = rn_t
            p = r + beta * p
            continue
        beta = rn / rr
        rr = rn
        maxr = max(maxr, rn)
        p = r + beta * p
    xh, xl = _dd_fold(xh, xl, x)
    rt = residual_dd(hfm, op, b, xh, xl)
    return xh, xl, it, rebases, float(np.linalg.norm(rt))


# ----------------------------------------------------------------------------------------------------------------
# Actions, integrator, HMC step
# ----------------------------------------------------------------------------------------------------------------
def utilde(beta, Nt, U) -> complex:
    """src/NSL/Action/Implementations/hubbard.tpp:9-19: delta * U."""
    return complex(beta) / Nt * complex(U)


def gauge_eval(phi, Ut):
    """hubbardGaugeAction.tpp:55-57."""
    return complex(np.sum(phi * phi)) / (2 * Ut)


def gauge_force(phi, Ut):
    """hubbardGaugeAction.tpp:59-62."""
    return phi / (-Ut)


def fermion_eval(hfm: HubbardExp, phi, logdet=None):
    """hubbardFermiAction.tpp:68-81: -(logdet M_P + logdet M_H)."""
    logdet = logdet or (lambda h: h.logDetM())
    hfm.populate(phi, PARTICLE)
    v = logdet(hfm)
    hfm.populate(phi, HOLE)
    v += logdet(hfm)
    return -v


def fermion_force(hfm: HubbardExp, phi, grad=None):
    """hubbardFermiAction.tpp:89-113: -(grad_P - grad_H)."""
    grad = grad or (lambda h: h.gradLogDetM())
    hfm.populate(phi, PARTICLE)
    g = grad(hfm)
    hfm.populate(phi, HOLE)
    g = g - grad(hfm)
    return -g


class HubbardAction:
    """HubbardGaugeAction + HubbardFermionAction summed as in src/NSL/Action/action.tpp:72-143. With stable=True the
    fermion terms use the stratified log det and gradient (logDetM_stable, gradLogDetM_stable) instead of the
    reference's direct products."""

    def __init__(self, K, Nt, beta, U, mu=0.0, logdet=None, stable=False):
        self.hfm = HubbardExp(K, Nt, beta, mu)
        self.Ut = utilde(beta, Nt, U)
        self.logdet = logdet or ((lambda h: h.logDetM_stable()) if stable else None)
        self.grad = (lambda h: h.gradLogDetM_stable()) if stable else None

    def eval(self, phi):
        return gauge_eval(phi, self.Ut) + fermion_eval(self.hfm, phi, self.logdet)

    def force(self, phi):
        return gauge_force(phi, self.Ut) + fermion_force(self.hfm, phi, self.grad)


def leapfrog(action, q, p, traj_length: float, nmd: int, backward: bool = False, real_force: bool = False):
    """src/NSL/Integrator/Impl/leapfrog.tpp:35-58 (real_force: leapfrogRealForce.tpp:36-74)."""
    eps = traj_length / nmd * (-1 if backward else 1)
    q = np.array(q, dtype=np.complex128, copy=True)
    p = np.array(p, dtype=np.complex128, copy=True)

    def F(x):
        f = action.force(x)
        return f.real + 0j if real_force else f

    p += (0.5 * eps) * F(q)
    q += eps * p
    for _ in range(nmd - 1):
        p += eps * F(q)
        q += eps * p
    p += (0.5 * eps) * F(q)
    return q, p


def hamiltonian(S, p) -> complex:
    """H = S + 1/2 sum p^2: src/NSL/MarkovChain/HMC.tpp:204-215."""
    return S + 0.5 * complex(np.sum(p * p))


def metropolis_prob(H0, H1) -> float:
    """src/NSL/MarkovChain/HMC.tpp:219: exp(Re(H0 - H1))."""
    return math.exp((H0 - H1).real) if (H0 - H1).real < 700 else math.inf


def two_point_correlator(hfm: HubbardExp, phi, species: int, n_time_sources: int):
    """src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:116-162 with the CG solve replaced by the exact
    inverse of the dense M (small lattices only): corr[t, y, x] averaged over the source times."""
    hfm.populate(phi, species)
    Nt, Nx = hfm.Nt, hfm.Nx
    Minv = np.linalg.inv(hfm.M_dense().reshape(Nt * Nx, Nt * Nx)).reshape(Nt, Nx, Nt, Nx)
    step = Nt // n_time_sources
    corr = np.zeros((Nt, Nx, Nx), dtype=np.complex128)
    for tsrc in range(0, Nt, step):
        invM = np.transpose(Minv[:, :, tsrc, :], (2, 0, 1)).copy()  # (x_src, t, y) = M^{-1} src
        invM = np.roll(invM, -tsrc, axis=1)
        if tsrc > 0:
            invM[:, Nt - tsrc:, :] *= -1.0
        corr += np.transpose(invM, (1, 2, 0))
    return corr / n_time_sources


def two_point_correlator_k(hfm: HubbardExp, phi, species: int, wall, k: int, n_time_sources: int):
    """src/NSL/Measurements/Hubbard/twoPointCorrelationFunction.tpp:169-233 (measureK) with the CG solve replaced by
    the exact dense inverse: for every source time the nb wall sources W[k, s] (placed on that time slice) give
    corrK[s] = M^{-1} src, shifted t -> t - tsrc with the anti-periodic sign and averaged over n_time_sources; the
    block is block[t, s1, s2] = sum_x conj(W[k, s1, x]) corrK[s2, t, x]."""
    hfm.populate(phi, species)
    Nt, Nx = hfm.Nt, hfm.Nx
    Minv = np.linalg.inv(hfm.M_dense().reshape(Nt * Nx, Nt * Nx)).reshape(Nt, Nx, Nt, Nx)
    Wk = np.asarray(wall, dtype=np.complex128)[k]  # (nb, Nx)
    step = Nt // n_time_sources
    corrK = np.zeros((Wk.shape[0], Nt, Nx), dtype=np.complex128)
    for tsrc in range(0, Nt, step):
        invM = np.einsum("tysx,bx->bty", Minv[:, :, tsrc:tsrc + 1, :], Wk)  # (nb, t, y)
        invM = np.roll(invM, -tsrc, axis=1)
        if tsrc > 0:
            invM[:, Nt - tsrc:, :] *= -1.0
        corrK += invM
    corrK /= n_time_sources
    return np.einsum("ax,btx->tab", np.conj(Wk), corrK)


# ----------------------------------------------------------------------------------------------------------------
# Two-body correlators from momentum wall sources
# ----------------------------------------------------------------------------------------------------------------
TWOBODY_CHANNELS = ("I1S1Iz1Sz1", "I1S1Iz1Sz0", "I1S1Iz1Szn1", "I1S1Iz0Sz1", "I1S1Iz0Szn1", "I1S1Izn1Sz1",
                    "I1S1Izn1Sz0", "I1S1Izn1Szn1", "I0S1Iz0Sz1", "I0S1Iz0Szn1", "I1S0Iz1Sz0", "I1S0Izn1Sz0")


def eq_modBZ(k, q, eps: float = 2e-12) -> bool:
    """k == q modulo the honeycomb reciprocal lattice spanned by C = (4 pi/3, 0), D = (-2 pi/3, 2 pi/sqrt 3):
    src/NSL/Measurements/Hubbard/twoBodyCorrelationFunction.tpp:101-135."""
    diff = np.asarray(k, dtype=np.float64) - np.asarray(q, dtype=np.float64)
    C = (4 * math.pi / 3, 0.0)
    D = (-2 * math.pi / 3, 2 * math.pi / math.sqrt(3.0))
    den = C[1] * D[0] - C[0] * D[1]
    m = (diff[1] * D[0] - diff[0] * D[1]) / den
    n = (diff[0] * C[1] - diff[1] * C[0]) / den
    return abs(round(m) - m) < eps and abs(round(n) - n) < eps


def twobody_tuples(momenta) -> np.ndarray:
    """The (w, x, P, Q) keys the reference allocates, map[w][x][P][Q] for k_w + k_x == k_P + k_Q mod BZ
    (twoBodyCorrelationFunction.tpp:196-226; its loop names the third key z and the fourth y), sorted."""
    k = np.asarray(momenta, dtype=np.float64)
    nk = k.shape[0]
    out = [(w, x, P, Q) for w in range(nk) for x in range(nk) for P in range(nk) for Q in range(nk)
           if eq_modBZ(k[w] + k[x], k[P] + k[Q])]
    return np.array(out, dtype=np.int64).reshape(-1, 4)


def two_body_correlator(hfm: HubbardExp, phi, wall, tuples, n_time_sources: int) -> np.ndarray:
    """TwoBodyCorrelator::measure(NumberTimeSources) for one configuration (twoBodyCorrelationFunction.tpp:188-306
    and the channel functions :481-1001), with the CG solves replaced by the exact inverse of the dense M (small
    lattices only): M^dagger (MM^dagger)^{-1} src = M^{-1} src and M (M^dagger M)^{-1} conj(src) = M^{-dagger} conj(src).
    Returns (12, ntuple, Nt, nb^2, nb^2) in the channel order of TWOBODY_CHANNELS, entry [t, i nb + j, l nb + k]."""
    W = np.asarray(wall, dtype=np.complex128)
    nk, nb, Nx = W.shape
    Nt = hfm.Nt
    n = Nt * Nx
    tuples = np.asarray(tuples, dtype=np.int64).reshape(-1, 4)
    step = Nt // n_time_sources
    out = np.zeros((12, len(tuples), Nt, nb * nb, nb * nb), dtype=np.complex128)
    for tsrc in range(0, Nt, step):
        src = np.zeros((nk, nb, Nt, Nx), dtype=np.complex128)
        src[:, :, tsrc, :] = W                                                  # :246
        pool, poolDag = {}, {}
        for sp in (PARTICLE, HOLE):
            hfm.populate(phi, sp)
            Minv = np.linalg.inv(hfm.M_dense().reshape(n, n))
            corrK = (Minv @ src.reshape(nk * nb, n).T).T.reshape(nk, nb, Nt, Nx)
            corrKDag = (Minv.conj().T @ src.conj().reshape(nk * nb, n).T).T.reshape(nk, nb, Nt, Nx)
            corrK = _roll_t(corrK, -tsrc, -1.0)                                 # :264-265
            corrKDag = _roll_t(corrKDag, -tsrc, -1.0)
            # corrKPool[kSink, kSrc, t, sSink, sSrc] = <W[kSink, sSink], corrK[kSrc, sSrc, t]> (:268-282)
            pool[sp] = np.einsum("abx,cdtx->actbd", W.conj(), corrK)
            poolDag[sp] = np.einsum("abx,cdtx->actbd", W, corrKDag).conj()    # :283
        Cp, Ch, Dp, Dh = pool[PARTICLE], pool[HOLE], poolDag[PARTICLE], poolDag[HOLE]

        def d(A, B, w, x, P, Q):   # A(w, z)[i, l] B(x, y)[j, k] with z = P, y = Q -> [t, i nb + j, l nb + k]
            return np.einsum("til,tjk->tijlk", A[w, P], B[x, Q]).reshape(Nt, nb * nb, nb * nb)

        def e(A, B, w, x, P, Q):   # A(w, y)[i, k] B(x, z)[j, l]
            return np.einsum("tik,tjl->tijlk", A[w, Q], B[x, P]).reshape(Nt, nb * nb, nb * nb)

        for u, (w, x, P, Q) in enumerate(tuples):
            a = (w, x, P, Q)
            c = [
                d(Dp, Dp, *a) - e(Dp, Dp, *a),                                                    # :481-522
                -0.5 * (d(Dp, Ch, *a) - e(Dp, Ch, *a) - e(Ch, Dp, *a) + d(Ch, Dp, *a)),           # :529-567
                d(Ch, Ch, *a) - e(Ch, Ch, *a),                                                    # :574-606
                0.5 * (d(Dp, Dh, *a) - e(Dp, Dh, *a) - e(Dh, Dp, *a) + d(Dh, Dp, *a)),            # :613-651
                0.5 * (d(Cp, Ch, *a) - e(Cp, Ch, *a) - e(Ch, Cp, *a) + d(Ch, Cp, *a)),            # :658-696
                d(Dh, Dh, *a) - e(Dh, Dh, *a),                                                    # :703-735
                -0.5 * (d(Cp, Dh, *a) - e(Cp, Dh, *a) - e(Dh, Cp, *a) + d(Dh, Cp, *a)),           # :742-780
                d(Cp, Cp, *a) - e(Cp, Cp, *a),                                                    # :787-819
                0.5 * (d(Dp, Dh, *a) + e(Dp, Dh, *a) + e(Dh, Dp, *a) + d(Dh, Dp, *a)),            # :826-865
                0.5 * (d(Cp, Ch, *a) + e(Cp, Ch, *a) + e(Ch, Cp, *a) + d(Ch, Cp, *a)),            # :872-911
                -0.5 * (d(Dp, Ch, *a) + e(Dp, Ch, *a) + e(Ch, Dp, *a) + d(Ch, Dp, *a)),           # :918-956
                -0.5 * (d(Cp, Dh, *a) + e(Cp, Dh, *a) + e(Dh, Cp, *a) + d(Dh, Cp, *a)),           # :963-1001
            ]
            for ch in range(12):
                out[ch, u] += c[ch] / n_time_sources
    return out


def honeycomb_wall_sources(L1: int, L2: int, ks=None):
    """Plane-wave wall sources on the two sublattices of the honeycomb: momenta k = m1 b1 / L1 + m2 b2 / L2 with the
    reciprocal vectors of honeycomb.tpp:81-84, W[k, s, x] = exp(i k . r_x) / sqrt(L1 L2) on sublattice s (even sites A,
    odd sites B, honeycomb.tpp:91-92), else 0. Returns (momenta (nk, 2), W (nk, 2, Nx)). The reference reads both
    from its YAML input; this is the test inputs' choice."""
    b = np.array([[2 * math.pi / 3, 2 * math.pi / math.sqrt(3.0)], [2 * math.pi / 3, -2 * math.pi / math.sqrt(3.0)]])
    sites = honeycomb_sites(L1, L2)
    allk = [(m1, m2) for m2 in range(L2) for m1 in range(L1)]
    ks = range(len(allk)) if ks is None else ks
    mom = np.array([allk[i][0] * b[0] / L1 + allk[i][1] * b[1] / L2 for i in ks])
    Nx = sites.shape[0]
    W = np.zeros((len(mom), 2, Nx), dtype=np.complex128)
    ph = np.exp(1j * mom @ sites.T) / math.sqrt(L1 * L2)  # (nk, Nx)
    W[:, 0, 0::2] = ph[:, 0::2]
    W[:, 1, 1::2] = ph[:, 1::2]
    return mom, W


def density_double_occupancy(hfm: HubbardExp, phi, n_time_sources: int = 1):
    """n(x) = 1 - G_P(x) + G_H(x) and d(x) = (1 - G_P(x)) G_H(x) from the equal-time diagonal of M^{-1} of both
    species (the two-point correlator at t = 0, two_point_correlator above; the definitions of
    nsl_gb300/observables.py, which the reference does not compute)."""
    gp = np.diagonal(two_point_correlator(hfm, phi, PARTICLE, n_time_sources)[0])
    gh = np.diagonal(two_point_correlator(hfm, phi, HOLE, n_time_sources)[0])
    return 1.0 - gp + gh, (1.0 - gp) * gh
