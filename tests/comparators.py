"""Restatement of rulinalg's test comparators (src/macros/comparison.rs,
src/ulp.rs) so that known-answer checks use the reference's own tolerances."""
import numpy as np


def ulp_diff(a, b):
    """ulp.rs:41-65: None for NaN or differing signs, else |bits(a) - bits(b)|."""
    a = np.asarray(a)
    b = np.asarray(b)
    it = np.int64 if a.dtype == np.float64 else np.int32
    if a == b:
        return 0
    if np.isnan(a) or np.isnan(b) or (np.signbit(a) != np.signbit(b)):
        return None
    return abs(int(a.view(it)) - int(b.view(it)))


def float_eq(a, b, eps=None, ulp=4):
    """`comp = float` (comparison.rs:145-197): |a - b| <= eps (default: epsilon of the
    type), else at most `ulp` units in the last place."""
    a = np.asarray(a)
    b = np.asarray(b, dtype=a.dtype)
    if eps is None:
        eps = np.finfo(a.dtype).eps
    if abs(float(a) - float(b)) <= eps:
        return True
    d = ulp_diff(a, b)
    return d is not None and d <= ulp


def assert_matrix_float_eq(x, y, eps=None, ulp=4):
    x = np.asarray(x)
    y = np.asarray(y, dtype=x.dtype)
    assert x.shape == y.shape, (x.shape, y.shape)
    bad = [(i, x.flat[i], y.flat[i]) for i in range(x.size) if not float_eq(x.flat[i], y.flat[i], eps, ulp)]
    assert not bad, f"{len(bad)} elements differ, first: {bad[:3]}"


def assert_ulp_eq(x, y, tol):
    x = np.asarray(x)
    y = np.asarray(y, dtype=x.dtype)
    for i in range(x.size):
        d = ulp_diff(x.flat[i], y.flat[i])
        assert d is not None and d <= tol, (i, x.flat[i], y.flat[i], d)


def assert_abs_eq(x, y, tol):
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    assert x.shape == y.shape
    assert np.max(np.abs(x - y), initial=0.0) <= tol, np.max(np.abs(x - y))


def perm_from_matrix(p):
    """PermutationMatrix::as_matrix inverse: row i has its 1 in column perm[i]."""
    p = np.asarray(p)
    return np.argmax(p, axis=1).astype(np.uint64)


def backward_error(a, x, b):
    """Normwise backward error ||b - A x||_inf / (||A||_inf ||x||_inf + ||b||_inf),
    evaluated in extended precision on the test side; a non-finite x or b gives inf
    (a longdouble max reduction need not propagate NaN on every platform)."""
    if not (np.all(np.isfinite(x)) and np.all(np.isfinite(b))):
        return float("inf")
    a = np.asarray(a, dtype=np.longdouble)
    x = np.asarray(x, dtype=np.longdouble)
    b = np.asarray(b, dtype=np.longdouble)
    r = b - a @ x
    den = np.max(np.sum(np.abs(a), axis=1)) * np.max(np.abs(x)) + np.max(np.abs(b))
    return float(np.max(np.abs(r)) / den) if den > 0 else 0.0
