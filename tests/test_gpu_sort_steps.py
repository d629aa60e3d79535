"""The radix sort's counting steps on the GPU against the reference's own
GPU-sort known-answer tests.

The reference implements two steps of its planned GPU sort as compute
shaders and tests them with fixed inputs:
  * histogramOfGlobalDigitCounts.glsl:31-59 — for each of the 32 bit
    positions, how many values have that bit set; cases in
    tests/testsSortGPU/testHistogramCreation.cpp:146-192 (130 values: powers
    of two, zeros, ones, twos, random in [0, 8192]) and
    testHistogramCreationHard.cpp:115 (2^16 random values);
  * prefixSumOfGlobalDigitCounts.glsl:24-69 — the exclusive scan inside
    each group of 4 histogram entries; known answers in
    tests/testsSortGPU/testHistogramPrefixSum.cpp:53-85 and its random case.
The library runs the same steps inside every radix pass: the digit
histogram (with 1-bit digits, entry [b][1] is the per-bit count) and the
exclusive scan over a place's digit counts (with 2-bit digits, a scan inside
each group of 4).  crt_radix_digit_counts / crt_radix_digit_offsets run
those device functions on these inputs; counts are integers, so the check is
exact equality.  Expected values follow the reference tests' own rules.
"""
import numpy as np
import pytest

from realtimeraytracing_gb300 import crt
from realtimeraytracing_gb300 import scenes as S

pytestmark = pytest.mark.gpu


def per_bit_expected(values):
    """initRandomValuesExpectedResults (testHistogramCreation.cpp:30-42)."""
    v = np.asarray(values, np.uint64)
    return np.array([int(((v >> np.uint64(b)) & np.uint64(1)).sum()) for b in range(32)], np.uint32)


def group4_exclusive_expected(counts):
    """initRandomValuesHistogramOutput (testHistogramPrefixSum.cpp:43-51):
    out[j*4 + i] = in[j*4 + i - 1] + out[j*4 + i - 1], out[j*4] = 0."""
    c = np.asarray(counts, np.uint32).reshape(8, 4)
    out = np.zeros_like(c)
    for i in range(1, 4):
        out[:, i] = c[:, i - 1] + out[:, i - 1]
    return out.reshape(-1)


def _bits_histogram(ctx, values):
    counts = ctx.radix_digit_counts(np.asarray(values, np.uint32), 1)   # (32 places, 2 digits)
    assert counts.shape == (32, 2)
    np.testing.assert_array_equal(counts.sum(axis=1), np.full(32, len(values), np.uint32))
    return counts[:, 1]


def test_histogram_creation_cases(ctx):
    n = 130
    pow2 = np.array([1 << (i % 32) for i in range(n)], np.uint32)
    expect_pow2 = np.zeros(32, np.uint32)
    for i in range(n):                       # initPowersOfTwoExpectedResults
        expect_pow2[i % 32] += 1
    np.testing.assert_array_equal(_bits_histogram(ctx, pow2), expect_pow2)
    np.testing.assert_array_equal(_bits_histogram(ctx, np.zeros(n, np.uint32)), np.zeros(32, np.uint32))
    ones = np.zeros(32, np.uint32)
    ones[0] = n                              # initOnesExpectedResults
    np.testing.assert_array_equal(_bits_histogram(ctx, np.ones(n, np.uint32)), ones)
    twos = np.zeros(32, np.uint32)
    twos[1] = n                              # initTwosExpectedResults
    np.testing.assert_array_equal(_bits_histogram(ctx, np.full(n, 2, np.uint32)), twos)
    rnd = (S.splitmix64(7, 1, n) % np.uint64(8193)).astype(np.uint32)   # uniform in [0, 8192]
    np.testing.assert_array_equal(_bits_histogram(ctx, rnd), per_bit_expected(rnd))


def test_histogram_creation_hard(ctx):
    n = 2 << 15
    rnd = (S.splitmix64(8, 1, n) % np.uint64(8193)).astype(np.uint32)
    np.testing.assert_array_equal(_bits_histogram(ctx, rnd), per_bit_expected(rnd))
    full = S.splitmix64(9, 1, n).astype(np.uint32)   # all 32 bits in play
    np.testing.assert_array_equal(_bits_histogram(ctx, full), per_bit_expected(full))


def test_prefix_sum_known_values(ctx):
    """testHistogramPrefixSum.cpp:53-85 (groups 0-2 given, the rest zero)."""
    counts = np.zeros(32, np.uint32)
    counts[0:4] = [37, 41, 49, 53]
    counts[4:8] = [37, 48, 44, 51]
    counts[8:12] = [35, 51, 53, 41]
    expected = np.zeros(32, np.uint32)
    expected[0:4] = [0, 37, 78, 127]
    expected[4:8] = [0, 37, 85, 129]
    expected[8:12] = [0, 35, 86, 139]
    got = ctx.radix_digit_offsets(counts, 2).reshape(-1)
    np.testing.assert_array_equal(got, expected)
    np.testing.assert_array_equal(expected, group4_exclusive_expected(counts))


def test_prefix_sum_random_histogram(ctx):
    """testHistogramPrefixSum.cpp:159-169: the per-bit histogram of 32 random
    values, scanned in groups of 4 — here both steps on the GPU."""
    vals = (S.splitmix64(10, 1, 32) % np.uint64(8193)).astype(np.uint32)
    hist = _bits_histogram(ctx, vals)
    np.testing.assert_array_equal(hist, per_bit_expected(vals))
    got = ctx.radix_digit_offsets(hist, 2).reshape(-1)
    np.testing.assert_array_equal(got, group4_exclusive_expected(hist))


@pytest.mark.parametrize("bits", [4, 8])
def test_digit_steps_at_the_sort_widths(ctx, bits):
    """The widths the sort passes run with: counts and start offsets of every
    digit place against numpy on 300k keys."""
    keys = S.splitmix64(11, bits, 300_000).astype(np.uint32)
    counts = ctx.radix_digit_counts(keys, bits)
    places, radix = counts.shape
    for p in range(places):
        digits = (keys >> np.uint32(p * bits)) & np.uint32(radix - 1)
        np.testing.assert_array_equal(counts[p], np.bincount(digits, minlength=radix).astype(np.uint32))
    offs = ctx.radix_digit_offsets(counts, bits)
    excl = np.concatenate([np.zeros((places, 1), np.uint64), np.cumsum(counts, axis=1, dtype=np.uint64)[:, :-1]], 1)
    np.testing.assert_array_equal(offs, excl.astype(np.uint32))
