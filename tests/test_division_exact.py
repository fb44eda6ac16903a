"""The packed fused kernels divide integer ray sums by integer ray counts with one Markstein
correction step (P. Markstein, IBM J. Res. Dev. 34(1), 1990) instead of a full division:
q0 = RN(s r), rem = RN(s - q0 c), q = RN(q0 + rem r) with r = RN(1 / c).  This checks, over
the whole domain the kernels use (sums 0..65535, counts 1..257), that the result equals the
correctly rounded float32 quotient, with every step emulated exactly in float64 (products of
float32 values are exact there) and the final rounding guarded against double rounding."""
import numpy as np


def test_markstein_quotient_is_correctly_rounded_over_the_domain():
    s = np.arange(0, 65536, dtype=np.float64)
    for c in range(1, 258):
        r = np.float32(1.0 / c)                      # RN32(1/c) (as the plan builds it)
        want = (s / c).astype(np.float32)            # RN32(s/c): s/c is never within 2^-33 of a
        q0 = (s * np.float64(r)).astype(np.float32)  # float32 midpoint unless exactly on one
        rem_exact = s - q0.astype(np.float64) * c
        rem = rem_exact.astype(np.float32)
        assert np.array_equal(rem.astype(np.float64), rem_exact)  # the remainder is exact
        t = q0.astype(np.float64) + rem.astype(np.float64) * np.float64(r)
        q = t.astype(np.float32)
        ulp = np.spacing(q).astype(np.float64)
        qa = q.astype(np.float64)
        near_mid = (np.abs(t - (qa - ulp / 2)) <= np.abs(t) * 2.0 ** -50) | \
                   (np.abs(t - (qa + ulp / 2)) <= np.abs(t) * 2.0 ** -50)
        assert not near_mid.any(), c                 # float64 rounding of t cannot matter
        assert np.array_equal(q, want), (c, s[q != want][:5])
