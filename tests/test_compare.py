"""The two error measures the GPU parity tests assert (oracle/compare.py), on the CPU:
a planted per-value error that the norm-wise measure cannot see is caught element-wise,
and FP64 rounding noise on values that are zero in exact arithmetic is not flagged."""
import numpy as np

from krets_gb300.generators import monte_carlo_values, rlc_ladder
from krets_gb300.table import element_table, is_current_mask
from oracle.compare import elementwise_err, normwise_err


def _ref(oracle_lib, steps=300):
    c = rlc_ladder(30)
    t = element_table(c)
    t["value"] = monte_carlo_values(c, 1, seed=2)[0]
    return c, oracle_lib.tran(t, c.size, 1e-12, steps, method="tr", lag=False)


def test_identical_results_have_zero_error(oracle_lib):
    c, ref = _ref(oracle_lib)
    m = is_current_mask(c)
    assert normwise_err(ref, ref, m) == 0.0 and elementwise_err(ref, ref, m) == 0.0


def test_elementwise_catches_an_error_the_normwise_measure_misses(oracle_lib):
    c, ref = _ref(oracle_lib)
    m = is_current_mask(c)
    v = np.nonzero(~m)[0]
    # a voltage at 1e-2 of the class's largest value, wrong by 5e-8 of itself
    scale = np.abs(ref[:, v]).max()
    mag = np.abs(ref[:, v])
    s, j = np.unravel_index(np.argmin(np.abs(mag - 1e-2 * scale)), mag.shape)
    bad = ref.copy()
    bad[s, v[j]] *= 1.0 + 5e-8
    assert normwise_err(bad, ref, m) < 1e-9          # 5e-10 of the class scale: invisible
    assert elementwise_err(bad, ref, m) > 2e-8       # per value: 5e-8 relative


def test_rounding_noise_on_exact_zeros_is_below_the_floor():
    # one current class with a 2 A value and an exact zero computed as 1e-15 by one side
    ref = np.array([[2.0, 0.0, 1.0]])
    x = np.array([[2.0, 1.7e-15, 1.0]])
    m = np.array([True, True, False])
    assert elementwise_err(x, ref, m) < 1e-9
    # the same noise on a value of 1 mA is a real 1e-12 relative error, also accepted,
    # while 1e-6 relative on it is not
    ref2 = np.array([[2.0, 1e-3, 1.0]])
    assert elementwise_err(ref2 * [1, 1 + 1e-12, 1], ref2, m) < 1e-9
    assert elementwise_err(ref2 * [1, 1 + 1e-6, 1], ref2, m) > 1e-9
