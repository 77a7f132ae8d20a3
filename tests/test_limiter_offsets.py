"""The CW84 limiter in the offsets u = R - q, v = q - L (the step kernels' form) against the
reference's form (reconstruction_1d.py:102-153, restated in oracle/ppm.py): flatten when
u v <= 0; otherwise move L to 3q - 2R when |v| > 2|u| and R to 3q - 2L when |u| > 2|v|.

Away from the tie lines the two forms take the same branches; on the tie lines (|v| = 2|u|,
|u| = 2|v|) a rounding may send them different ways, where both branches give the same
parabola.  So everywhere the results agree to a few ulps of the cell's values.
"""
import numpy as np


def reference_form(q, L, R):
    """reconstruction_1d.py:102-153 as oracle/ppm.py restates it, on 1-D arrays."""
    L, R = L.copy(), R.copy()
    dq = R - L
    q6 = 6 * q - 3 * (R + L)
    lmax = (R - q) * (q - L) <= 0
    R[lmax] = q[lmax]
    L[lmax] = q[lmax]
    over = np.abs(dq) < np.abs(q6)
    mleft = (R - L) * (q - 0.5 * (R + L)) > ((R - L) ** 2) / 6.0
    mright = -((R - L) ** 2) / 6.0 > (R - L) * (q - 0.5 * (R + L))
    ml = over & mleft
    mr = over & mright
    L[ml] = 3.0 * q[ml] - 2.0 * R[ml]
    R[mr] = 3.0 * q[mr] - 2.0 * L[mr]
    return L, R, lmax, ml, mr


def offset_form(q, L, R):
    """The kernels' form: decisions on u = R - q and v = q - L, moved offsets 2u and 2v."""
    u, v = R - q, q - L
    flat = u * v <= 0
    ml = ~flat & (np.abs(v) > 2 * np.abs(u))
    mr = ~flat & (np.abs(u) > 2 * np.abs(v))
    uo = np.where(flat, 0.0, np.where(mr, 2 * v, u))
    vo = np.where(flat, 0.0, np.where(ml, 2 * u, v))
    return q - vo, q + uo, flat, ml, mr


def cells(n, seed):
    rng = np.random.default_rng(seed)
    q = rng.normal(size=n) * 10.0 ** rng.uniform(-3, 3, size=n)
    scale = np.abs(q) + 10.0 ** rng.uniform(-4, 1, size=n)
    u = rng.normal(size=n) * scale
    v = rng.normal(size=n) * scale
    kind = rng.integers(0, 6, size=n)
    # on and next to the tie lines, flat and one-sided cases
    v = np.where(kind == 1, 2 * u * (1 + rng.normal(size=n) * 1e-15), v)
    u = np.where(kind == 2, 2 * v * (1 + rng.normal(size=n) * 1e-15), u)
    v = np.where(kind == 3, -v, v)
    u = np.where(kind == 4, 0.0, u)
    v = np.where(kind == 5, np.abs(v) * np.sign(u) * 0.5, v)
    return q, q - v, q + u


def test_offset_form_equals_reference_form():
    for seed in range(4):
        q, L, R = cells(200_000, seed)
        Lr, Rr, fr, mlr, mrr = reference_form(q, L, R)
        Lo, Ro, fo, mlo, mro = offset_form(q, L, R)
        size = np.maximum(np.maximum(np.abs(q), np.abs(L)), np.abs(R))
        tol = 8 * np.finfo(float).eps * size
        assert np.all(np.abs(Lo - Lr) <= tol)
        assert np.all(np.abs(Ro - Rr) <= tol)
        np.testing.assert_array_equal(fo, fr)  # the extremum test is the same test
        # branches differ only next to the tie lines
        u, v = R - q, q - L
        near = (np.abs(np.abs(v) - 2 * np.abs(u)) <= 1e-12 * size) | (np.abs(np.abs(u) - 2 * np.abs(v)) <= 1e-12 * size)
        differ = (mlo != mlr) | (mro != mrr)
        assert np.all(near[differ]) and differ.sum() < near.sum()
        assert mlr.sum() > 1000 and mrr.sum() > 1000 and fr.sum() > 1000  # every branch is exercised
