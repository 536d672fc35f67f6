"""NonStationaryConvolve2D on the GPU against the reference's golden vectors
(filters interpolated inside the coarse grid, edge filters outside it) and,
at a larger size with PSF-sized filters, against the float64 oracle.
Tolerance 1e-5 relative L2."""

import numpy as np
import pytest

from tests.helpers import load, rel

pytestmark = pytest.mark.gpu


def test_nsconv2d_matches_reference_and_passes_dottest():
    import torch

    from pylops_gb300.signalprocessing import NonStationaryConvolve2D
    from pylops_gb300.utils.dottest import dottest

    g = load("nsconv2d")
    C = NonStationaryConvolve2D(dims=g["x_in"].shape, hs=g["hs"], ihx=g["ihx"], ihz=g["ihz"], engine="cuda",
                                dtype="float32")
    assert rel(C @ g["x_in"].ravel(), g["fwd"]) < 1e-5
    assert rel(C.H @ g["y_in"].ravel(), g["adj"]) < 1e-5
    assert dottest(C, *C.shape, rtol=1e-4)
    x = torch.randn(C.shape[1], device="cuda")
    assert torch.equal(C @ x, C @ x) and torch.equal(C.H @ x, C.H @ x)


def test_nsconv2d_errors_like_reference():
    from pylops_gb300.signalprocessing import NonStationaryConvolve2D

    hs = np.zeros((2, 2, 4, 5))
    with pytest.raises(ValueError):
        NonStationaryConvolve2D(dims=(20, 20), hs=hs, ihx=[2, 10], ihz=[2, 10])
    with pytest.raises(ValueError):
        NonStationaryConvolve2D(dims=(20, 20), hs=np.zeros((3, 2, 5, 5)), ihx=[2, 5, 10], ihz=[2, 10])
    with pytest.raises(ValueError):
        NonStationaryConvolve2D(dims=(20, 20), hs=np.zeros((2, 2, 5, 5)), ihx=[2, 25], ihz=[2, 10])
    with pytest.raises(NotImplementedError):
        NonStationaryConvolve2D(dims=(20, 20), hs=np.zeros((2, 2, 5, 5)), ihx=[2, 10], ihz=[2, 10], engine="x")


def test_nsconv2d_psf_sized_filters_against_oracle():
    from oracle.nsconv2d_oracle import nsconv2d
    from pylops_gb300.signalprocessing import NonStationaryConvolve2D

    rng = np.random.default_rng(3)
    nx, nz = 96, 64
    ihx, ihz = np.arange(8, 96, 20), np.arange(6, 64, 16)
    hs = rng.standard_normal((len(ihx), len(ihz), 31, 25))
    C = NonStationaryConvolve2D(dims=(nx, nz), hs=hs, ihx=ihx, ihz=ihz, dtype="float32")
    x = rng.standard_normal((nx, nz))
    assert rel(C @ x.ravel(), nsconv2d(x, hs, ihx, ihz)) < 1e-5
    assert rel(C.H @ x.ravel(), nsconv2d(x, hs, ihx, ihz, adjoint=True)) < 1e-5
