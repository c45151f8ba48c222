"""Accuracy of the fast variants' arithmetic helpers on the GPU.

The fast double path replaces the IEEE divide, cube root and square root by
shorter sequences (step_math.cuh: rcp, rcbrt_pos, sqrt_fast, recip_sqrt).
lulesh_probe_math evaluates each on the device; the results are compared
here with the correctly rounded values computed in long double on the host,
in units in the last place of the double result (ulp). The inputs are seeded
and span the magnitudes a step can meet (and far beyond).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 20


def _ulp_error(got: np.ndarray, ref: np.ndarray) -> float:
    spacing = np.spacing(np.abs(ref.astype(np.float64))).astype(np.longdouble)
    return float((np.abs(got.astype(np.longdouble) - ref) / spacing).max())


def _inputs(lo: int, hi: int, negative: bool = False) -> np.ndarray:
    rng = np.random.default_rng(2024)
    x = np.ldexp(rng.uniform(1.0, 2.0, N), rng.integers(lo, hi, N))
    x[:64] = np.ldexp(1.0, np.arange(64) - 32)  # exact powers of two
    x[64:128] = np.nextafter(np.ldexp(1.0, np.arange(64) - 31), 0.0)  # just below them
    if negative:
        x[N // 2:] *= -1.0
    return x


# (helper, exponent range of the inputs, negative inputs too, reference, bound in ulp)
CASES = [
    ("rcp", (-100, 100), True, lambda x: 1 / x, 0.55),
    ("rcbrt", (-100, 100), False, lambda x: 1 / np.cbrt(x), 1.0),
    ("sqrt", (-1000, 1000), False, np.sqrt, 1.5),
    ("rsqrt", (-1000, 1000), False, lambda x: 1 / np.sqrt(x), 1.0),
]


@pytest.mark.parametrize("name,span,neg,ref,bound", CASES, ids=[c[0] for c in CASES])
def test_helper_within_bound(lulesh, name, span, neg, ref, bound):
    x = _inputs(*span, negative=neg)
    got = lulesh.probe_math(name, x)
    err = _ulp_error(got, ref(x.astype(np.longdouble)))
    assert err <= bound, f"{name}: {err:.3f} ulp"


def test_reciprocal_seed_bound(lulesh):
    """rcp's third-order correction assumes a seed within 2^-19.9 (the
    truncated series term e^3 is then below 2^-59)."""
    x = _inputs(-1000, 1000, negative=True)
    seed = lulesh.probe_math("rcp_seed", x).astype(np.longdouble)
    ref = 1 / x.astype(np.longdouble)
    rel = float((np.abs(seed - ref) / np.abs(ref)).max())
    assert rel <= 2.0 ** -19.9, rel


def test_probe_rejects_bad_arguments(lulesh):
    with pytest.raises(lulesh.LuleshError):
        lulesh.probe_math("rcp", np.empty(0))


def _conversion_inputs() -> np.ndarray:
    """Doubles across float's whole range and beyond it: subnormal floats,
    overflow, ties between two floats, zeros of both signs."""
    rng = np.random.default_rng(31)
    x = np.ldexp(rng.uniform(1.0, 2.0, N), rng.integers(-160, 140, N))
    x[N // 2:] *= -1.0
    ties = np.ldexp(rng.integers(1 << 23, 1 << 24, 4096) * 2.0 + 1.0, rng.integers(-120, 100, 4096) - 24)
    x[:4096] = ties  # exactly halfway between two floats: round to even
    x[4096:4100] = [0.0, -0.0, np.finfo(np.float32).max, -np.finfo(np.float32).max]
    return x


def test_narrow_is_round_to_nearest_even(lulesh):
    """The mixed variant's integer-pipe double-to-float rounding equals the
    conversion bit for bit (signed zeros and infinities included)."""
    x = _conversion_inputs()
    got = lulesh.probe_math("narrow", x)
    with np.errstate(over="ignore"):
        want = x.astype(np.float32).astype(np.float64)
    assert np.array_equal(np.signbit(got), np.signbit(want))
    assert np.array_equal(got, want)


def test_split_is_the_float_pair(lulesh):
    """split(v) = (fl(v), fl(v - fl(v))) bit for bit, where the pair is finite."""
    x = _conversion_inputs()
    x = x[np.abs(x) <= np.finfo(np.float32).max]
    hi = lulesh.probe_math("split_hi", x)
    lo = lulesh.probe_math("split_lo", x)
    want_hi = x.astype(np.float32).astype(np.float64)
    want_lo = (x - want_hi).astype(np.float32).astype(np.float64)
    assert np.array_equal(hi, want_hi)
    assert np.array_equal(lo, want_lo)


def test_integer_pipe_multiply_equals_fp64_pipe(lulesh):
    """dmul_ipipe, the double multiply the fast kernels run on the integer
    pipes, gives the FP64 pipe's bits for every operand pair: seeded random
    bit patterns over the whole exponent range (normal, subnormal, zero,
    infinite and NaN operands; products that overflow, underflow or land on
    a rounding tie), plus products near powers of two and of small integers
    (3 x c, the step's own pattern)."""
    rng = np.random.default_rng(7)
    n = 1 << 22
    bits = rng.integers(0, 2 ** 63, size=(2, n), dtype=np.int64).astype(np.uint64)
    bits[:, : n // 2] |= rng.integers(0, 2, size=(2, n // 2), dtype=np.uint64) << np.uint64(63)
    a, b = bits.view(np.float64)
    # operands in the step's range: exponents near 0, random significands
    k = n // 4
    a[:k] = np.ldexp(rng.uniform(1.0, 2.0, k), rng.integers(-60, 60, k)) * rng.choice([-1.0, 1.0], k)
    b[:k] = np.ldexp(rng.uniform(1.0, 2.0, k), rng.integers(-60, 60, k))
    b[k:k + 4096] = 3.0
    b[k + 4096:k + 8192] = np.ldexp(1.0, rng.integers(-20, 20, 4096))
    # significands whose product is (almost) a tie: a = 1 + 2^-26 j
    a[2 * k:2 * k + 8192] = 1.0 + np.ldexp(rng.integers(1, 2 ** 26, 8192).astype(np.float64), -26)
    b[2 * k:2 * k + 8192] = 1.0 + np.ldexp(rng.integers(1, 2 ** 26, 8192).astype(np.float64), -26)
    # exponents that put the product at the edges of the normal range
    e = rng.integers(-1000, 1000, 8192)
    target = np.where(e > 0, 1024, -1074) + rng.integers(-8, 8, 8192)  # exponent of the product
    a[3 * k:3 * k + 8192] = np.ldexp(rng.uniform(1.0, 2.0, 8192), e)
    b[3 * k:3 * k + 8192] = np.ldexp(rng.uniform(1.0, 2.0, 8192), np.clip(target - e, -1074, 1023))
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.2e-308, 1e308, 1e-308, 1.0, -3.0])
    sa, sb = np.meshgrid(special, special)
    a[-sa.size:], b[-sb.size:] = sa.ravel(), sb.ravel()
    native, ipipe = lulesh.probe_dmul(a, b)
    same = native.view(np.uint64) == ipipe.view(np.uint64)
    both_nan = np.isnan(native) & np.isnan(ipipe)
    assert np.all(same | both_nan), np.flatnonzero(~(same | both_nan))[:8]
    # and both are the IEEE products the host computes
    with np.errstate(all="ignore"):
        host = a * b
    assert np.all((host.view(np.uint64) == native.view(np.uint64)) | (np.isnan(host) & np.isnan(native)))


def test_integer_pipe_add_is_the_fp64_add(lulesh):
    """dadd_ipipe, the integer-pipe double add of the measurement probes (no
    step kernel uses it: it is slower than the FP64 pipe's add), gives the
    FP64 pipe's bits for every operand pair: seeded random bit
    patterns over the whole exponent range (normal, subnormal, zero, infinite
    and NaN operands, both signs), sums that cancel to a few bits, that land
    on a rounding tie, that stay subnormal or become normal, and that
    overflow."""
    rng = np.random.default_rng(11)
    n = 1 << 22
    bits = rng.integers(0, 2 ** 63, size=(2, n), dtype=np.int64).astype(np.uint64)
    bits[:, : n // 2] |= rng.integers(0, 2, size=(2, n // 2), dtype=np.uint64) << np.uint64(63)
    a, b = bits.view(np.float64)
    k = n // 5
    sign = lambda m: rng.choice([-1.0, 1.0], m)  # noqa: E731
    # the step's range: exponents near 0, both signs
    a[:k] = np.ldexp(rng.uniform(1.0, 2.0, k), rng.integers(-60, 60, k)) * sign(k)
    b[:k] = np.ldexp(rng.uniform(1.0, 2.0, k), rng.integers(-60, 60, k)) * sign(k)
    # near cancellation: b = -a (1 + j 2^(e-52))
    j = rng.integers(-2 ** 20, 2 ** 20, k).astype(np.float64)
    with np.errstate(invalid="ignore"):
        b[k:2 * k] = -a[k:2 * k] * (1.0 + np.ldexp(j, -52 + rng.integers(-3, 4, k)))
    # ties: b a power of two half an ulp of a, or below
    a[2 * k:3 * k] = np.ldexp(rng.uniform(1.0, 2.0, k), rng.integers(-100, 100, k)) * sign(k)
    b[2 * k:3 * k] = np.ldexp(sign(k), np.frexp(a[2 * k:3 * k])[1] - 54 - rng.integers(0, 12, k))
    # subnormal operands and sums, and sums at the top of the range
    m = 1 << 16
    a[3 * k:3 * k + m] = np.ldexp(rng.uniform(-2.0, 2.0, m), -1022 - rng.integers(0, 60, m))
    b[3 * k:3 * k + m] = np.ldexp(rng.uniform(-2.0, 2.0, m), -1022 - rng.integers(0, 60, m))
    a[3 * k + m:3 * k + 2 * m] = np.ldexp(rng.uniform(1.0, 2.0, m), 1023) * sign(m)
    b[3 * k + m:3 * k + 2 * m] = np.ldexp(rng.uniform(1.0, 2.0, m), 1023 - rng.integers(0, 60, m)) * sign(m)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, -2.2e-308, 1e308, 1e-308, 1.0,
                        -3.0])
    sa, sb = np.meshgrid(special, special)
    a[-sa.size:], b[-sb.size:] = sa.ravel(), sb.ravel()
    native, ipipe = lulesh.probe_dadd(a, b)
    same = native.view(np.uint64) == ipipe.view(np.uint64)
    both_nan = np.isnan(native) & np.isnan(ipipe)
    assert np.all(same | both_nan), np.flatnonzero(~(same | both_nan))[:8]
    # and both are the IEEE sums the host computes
    with np.errstate(all="ignore"):
        host = a + b
    assert np.all((host.view(np.uint64) == native.view(np.uint64)) | (np.isnan(host) & np.isnan(native)))
