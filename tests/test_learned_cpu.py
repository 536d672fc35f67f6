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


def test_unet_kernel_eligibility_rules():
    """Host-side rules that route a U-Net layer to the resident-weight
    implicit kernels (they mirror the C entry points' checks): the 9-tap
    weights plus three halo rows fit in 227 KB of shared memory, and a
    stride-2 gradient grid splits into 128-pixel tiles (parts of rows of
    128-pixel multiples, or whole rows of 32 or 64 pixels)."""
    from pylops_gb300.learned.unet import _halo_weights_fit, _s2_tiles

    # (C, N): one or two 64-channel blocks with 64 columns, one with 128; not two with 128 or three with 64
    assert _halo_weights_fit(32, 32) and _halo_weights_fit(64, 64) and _halo_weights_fit(128, 64)
    assert _halo_weights_fit(64, 128) and _halo_weights_fit(96, 64)
    assert not _halo_weights_fit(128, 96) and not _halo_weights_fit(192, 64) and not _halo_weights_fit(256, 128)
    for Hg, Wg, ok in [(1, 128, True), (3, 256, True), (4, 64, True), (3, 64, False), (8, 32, True), (6, 32, False),
                       (4, 96, False), (2, 16, False)]:
        assert _s2_tiles(Hg, Wg) is ok, (Hg, Wg)
