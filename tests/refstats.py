"""Assertion shared by the GPU tests: statistics identical to the reference's."""

import oracle as O


def assert_reference_stats(got, ref_map, scale):
    """count, the two sequential f64 sums, mean, SD and max bit-identical to the
    oracle's restatement of nonzero_stats (metrics.rs:204-241, values added one
    after the other in index order); the exact sums against an exact summation."""
    seq = O.nonzero_stats(ref_map, scale)
    assert got.count == seq.count
    assert got.sum == seq.sum and got.sum_of_squares == seq.sum_sq, (got.sum, seq.sum, got.sum_of_squares, seq.sum_sq)
    assert got.mean == seq.mean and got.standard_deviation == seq.sd and got.maximum == seq.max
    n, s, ss, mx = O.exact_moment_sums(ref_map, scale)
    assert got.exact_sum == s and got.exact_sum_of_squares == ss
