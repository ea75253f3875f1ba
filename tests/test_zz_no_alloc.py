"""acdc_debug_sample_noalloc against acdc_debug_sample.  The no-allocation
variant serves callers that must not allocate device memory while they run (a
process whose memory is committed to resident problems, or one checking the
sampler beside running solves that wants no allocation call on their stream).
Through the C-ABI it must return the same draws as the allocating entry point
on two calls in a row (the fixed scratch keeps the previous call's contents),
and refuse counts beyond its scratch.  Collected last, so a run that stops at
the first failure has run every other test before it."""
import numpy as np
import pytest

import acdc

pytestmark = pytest.mark.gpu


def test_two_calls_in_a_row_match_the_allocating_entry_point(ctx):
    cases = [(0xACDC0001, 1000, 4096, 10**7), (12345, 7, acdc.NOALLOC_MAX_SAMPLES, 2**33 + 7)]
    for seed, k0, count, n in cases:
        got = acdc.debug_sample_noalloc(ctx, seed, k0, count, n)
        want = acdc.debug_sample(ctx, seed, k0, count, n)
        np.testing.assert_array_equal(got, want)
        assert got.min() >= 0 and got.max() < n


def test_calls_leave_the_memory_pool_unchanged(ctx):
    # a warm call first: the first call on a device looks up the scratch address
    acdc.debug_sample_noalloc(ctx, 3, 0, 1024, 5000)
    before = ctx.memory()
    for k0 in (0, 10**6):
        acdc.debug_sample_noalloc(ctx, 3, k0, acdc.NOALLOC_MAX_SAMPLES, 5000)
    assert ctx.memory() == before


def test_sizes_beyond_the_scratch_are_refused(ctx):
    with pytest.raises(acdc.AcdcError) as e:
        acdc.debug_sample_noalloc(ctx, 1, 0, acdc.NOALLOC_MAX_SAMPLES + 1, 100)
    assert e.value.code == acdc.EINVAL
    assert len(acdc.debug_sample_noalloc(ctx, 1, 0, 0, 100)) == 0
