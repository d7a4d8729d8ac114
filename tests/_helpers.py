"""Helpers shared by the test modules (tolerances follow the reference)."""
import numpy as np

# tests/rpp/cpu/single_thread/ops/cpu_typed_ft_ops_test_helper.hpp:33-36 and
# :261-273: |a - e| <= tol * max(1, |a|, |e|), 1e-12 for double, 1e-5 for float.
TOL_F64 = 1e-12
TOL_F32 = 1e-5


def rel_err(actual, expected):
    actual = np.asarray(actual, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    if actual.size == 0:
        return 0.0
    scale = np.maximum(1.0, np.maximum(np.abs(actual), np.abs(expected)))
    return float(np.max(np.abs(actual - expected) / scale))


def scaled_err(actual, expected):
    """Error of a whole array against its own scale: max |a - e| / max(1,
    max |e|).  The reference's metric (above) divides by each coefficient's own
    magnitude with a floor of 1; a gradient coefficient is a sum of O(L) terms
    of either sign and may cancel to near zero, so its error is measured
    against the array's largest coefficient instead (equal to the reference's
    metric wherever that coefficient is at most 1)."""
    actual = np.asarray(actual, dtype=np.float64)
    expected = np.asarray(expected, dtype=np.float64)
    if actual.size == 0:
        return 0.0
    scale = max(1.0, float(np.max(np.abs(expected))))
    return float(np.max(np.abs(actual - expected)) / scale)


def assert_close(actual, expected, tol=TOL_F64, what=""):
    e = rel_err(actual, expected)
    assert np.isfinite(e) and e <= tol, f"{what}: relative error {e:.3e} > {tol:.1e}"


def shuffle_cases(z, op):
    """The cases of one operation in a golden file written as
    `<op>/<i>/<field>` keys, in case order."""
    keys = sorted({k.split("/")[1] for k in z.files if k.startswith(op + "/")}, key=int)
    return [{k.split("/")[2]: z[k] for k in z.files if k.startswith(f"{op}/{i}/")} for i in keys]
