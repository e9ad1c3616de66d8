"""CPU checks of the multigrid set-up's host logic: the coarsest level's dense inverse."""

import numpy as np


def test_coarsest_dense_inverse_paths():
    from warp_gb300.multigrid import _dense_inverse

    rng = np.random.default_rng(0)
    m = rng.standard_normal((40, 40))
    spd = m @ m.T + 40 * np.eye(40)
    spd_rounded = spd + np.triu(rng.standard_normal((40, 40)) * 1e-15, 1)  # symmetric to rounding only
    indefinite = m + m.T
    general = m + 10 * np.eye(40)
    for a, sym in ((spd, True), (spd_rounded, True), (indefinite, True), (general, False)):
        before = a.copy()
        inv = _dense_inverse(a, sym)
        assert np.array_equal(a, before)  # the input is left as it was
        assert np.abs(inv @ a - np.eye(40)).max() < 1e-9 * np.linalg.cond(a)
    # the Cholesky path returns a symmetric inverse
    inv = _dense_inverse(spd, True)
    assert np.array_equal(inv, inv.T)
