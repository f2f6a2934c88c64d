"""The split-BF16 operator's digit arithmetic (nsl_gb300/csrc/fm_apply_oz.cu), restated in numpy and checked on the
CPU: balanced base-512 digits are exact in BF16 and reconstruct the rounded operand exactly, the six-digit product
is FP64-class, and the digit-sum bound that proves the FP32 accumulators exact holds for localised exp(delta K) and
fails for a delocalised one (where the GPU operator reports an error instead of a result)."""
import numpy as np
import pytest
import scipy.linalg as sl

W, S = 9, 6          # bits per digit, digits per operand (9 S - 1 = 53 bits)
HALF = 1 << (W - 1)  # |digit| <= 256: exact in BF16 (8 significant bits)


def frexp_exponent(M):
    """|v| < 2^e per row (0 for an all-zero row), from the row maximum."""
    return np.frexp(np.abs(M).max(axis=1))[1].astype(np.int64)


def balanced_digits(V, e):
    """Digits a_k of N = round(v 2^{9S-1-e}) with v = 2^{e-8} sum_k a_k 2^{-9k} (row exponents e)."""
    N = np.rint(V * np.exp2((W * S - 1 - e)[:, None].astype(float))).astype(np.int64)
    a = [None] * S
    for k in range(S - 1, 0, -1):
        d = ((N + HALF) & ((1 << W) - 1)) - HALF
        a[k] = d
        N = (N - d) >> W
    a[0] = N
    return a


def split_product(E, Y):
    """Y E^T from the digit products of order d < S (each order an exact integer sum), recombined in long double."""
    er, ex = frexp_exponent(Y), frexp_exponent(E)
    a, b = balanced_digits(Y, er), balanced_digits(E, ex)
    z = np.zeros((Y.shape[0], E.shape[0]), dtype=np.longdouble)
    for d in range(S):
        G = sum(a[k].astype(np.float64) @ b[d - k].astype(np.float64).T for k in range(d + 1))
        z += G.astype(np.longdouble) * np.longdouble(2.0) ** (-W * d)
    return z * np.exp2(np.longdouble(1) * (er[:, None] + ex[None, :] - 2 * (W - 1)))


def digit_sum_bounds(E):
    """max_x 256 sum_{l<=d} sum_y |b_l(x, y)| per order d: a bound on |G_d| for every operand."""
    b = balanced_digits(E, frexp_exponent(E))
    acc = np.zeros(E.shape[0], dtype=np.int64)
    out = []
    for d in range(S):
        acc = acc + np.abs(b[d]).sum(axis=1)
        out.append(int((HALF * acc).max()))
    return out


def bounds_ok(bounds):
    return all(v < 2 ** 24 for v in bounds[:4]) and all(v < 2 ** 30 for v in bounds[4:])


def honeycomb_K(L):
    from nsl_gb300.lattice import Honeycomb

    return np.asarray(Honeycomb(L).hopping_matrix()).real


def test_digits_exact_in_bf16_and_reconstruct():
    rng = np.random.default_rng(3)
    V = rng.standard_normal((8, 50)) * np.exp2(rng.integers(-30, 30, size=(8, 1))) * np.exp2(
        rng.integers(-20, 1, size=(8, 50)))
    V[0, :5] = 0.0
    e = frexp_exponent(V)
    a = balanced_digits(V, e)
    for k in range(S):
        assert np.abs(a[k]).max() <= HALF
        # an integer of magnitude <= 256 survives a round trip through BF16 (float32 with 16 low bits cleared)
        f = a[k].astype(np.float32).view(np.uint32) & np.uint32(0xFFFF0000)
        assert np.array_equal(f.view(np.float32).astype(np.int64), a[k])
    N = np.rint(V * np.exp2((W * S - 1 - e)[:, None].astype(float))).astype(np.int64)
    rec = sum(a[k] * (1 << (W * (S - 1 - k))) for k in range(S))
    assert np.array_equal(rec, N)
    assert np.abs(N).max() <= 2 ** (W * S - 1)


@pytest.mark.parametrize("delta", [0.125, 0.25, 1.0])
def test_split_product_is_fp64_class(delta):
    K = honeycomb_K((6, 6))
    E = sl.expm(delta * K)
    rng = np.random.default_rng(11)
    w, v = np.linalg.eigh(K)
    rows = {"gauss": rng.standard_normal((12, 72)),
            "smooth": (v[:, :3] @ rng.standard_normal((3, 12))).T + 1e-7 * rng.standard_normal((12, 72))}
    rows["positive"] = np.abs(rows["smooth"])
    for name, Y in rows.items():
        exact = Y.astype(np.longdouble) @ E.astype(np.longdouble).T
        err = float(np.abs(split_product(E, Y) - exact).max() / np.abs(exact).max())
        fp64 = float(np.abs((Y @ E.T) - exact).max() / np.abs(exact).max())
        # within ~10x of an FP64 product's own rounding; both grow where the rows cancel (smooth rows at delta = 1)
        assert err < 20 * max(fp64, 1e-17), (name, err, fp64)
        assert err < (1e-14 if delta < 1 else 1e-13), (name, err)


def test_digit_sum_bound():
    K = honeycomb_K((12, 12))
    for delta in (0.0625, 0.125, 0.5, 1.0):
        assert bounds_ok(digit_sum_bounds(sl.expm(delta * K))), delta
    # delta = 4 (honeycomb 12x12, Nt = 2, beta = 8): too delocalised, the GPU operator refuses it
    assert not bounds_ok(digit_sum_bounds(sl.expm(4.0 * K)))
    # the worst case over operands is attained: one column of digits at their maximum
    E = sl.expm(0.125 * K)
    b = balanced_digits(E, frexp_exponent(E))
    x = int(np.argmax(np.abs(b[0]).sum(axis=1)))
    a0 = np.sign(b[0][x]) * HALF
    assert abs(int(a0 @ b[0][x])) == digit_sum_bounds(E)[0]
