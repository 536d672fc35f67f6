"""Host-side parts of the learned preconditioner: the random model generator
and the illumination (Jacobi) diagonal, the latter against explicit column
norms of the oracle operator."""

import types

import numpy as np

from tests.helpers import kwargs_from_golden, load


def test_random_reflectivity_is_seeded_and_layered():
    from pylops_gb300.learned.lsm import random_reflectivity

    a = random_reflectivity(64, 48, np.random.default_rng(3))
    b = random_reflectivity(64, 48, np.random.default_rng(3))
    c = random_reflectivity(64, 48, np.random.default_rng(4))
    assert a.shape == (64, 48) and a.dtype == np.float32
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # every column crosses between 3 and 15 interfaces (plus a few spikes)
    nnz = (np.abs(a) > 0).sum(1)
    assert nnz.min() >= 1 and nnz.max() <= 15 + 10
    assert np.abs(a).max() < 1.0


def test_illumination_diagonal_matches_oracle_column_norms():
    from oracle.kirchhoff_oracle import KirchhoffOracle
    from pylops_gb300.learned.lsm import illumination_diagonal

    g = load("k2d_dyn_noap")
    args, kw = kwargs_from_golden(g)
    # a longer time axis keeps every wavelet inside its trace
    args = args[:2] + (np.arange(300) * 0.004,) + args[3:]
    ora = KirchhoffOracle(*args, **kw)
    op = types.SimpleNamespace(dynamic=True, ni=ora.ni, amp_srcs=ora.amp_srcs, amp_recs=ora.amp_recs,
                               angle_srcs=ora.angle_srcs, angle_recs=ora.angle_recs, vel=ora.vel,
                               wav=g["wav"], angleaperture=ora.angleaperture, aperturetap=ora.aperturetap)
    p = illumination_diagonal(op, eps=0.0).astype(np.float64)
    ratio = []
    for i in range(ora.ni):
        e = np.zeros(ora.ni)
        e[i] = 1.0
        col = ora.matvec(e)
        ratio.append(1.0 / p[i] ** 2 / (col @ col))
    ratio = np.array(ratio)
    # exact up to the per-point spread of interpolation fractions (24 traces here)
    assert abs(np.median(ratio) - 1.0) < 0.02
    assert ratio.min() > 0.88 and ratio.max() < 1.12
