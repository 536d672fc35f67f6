"""Learned image-domain preconditioner for least-squares migration: a BF16
U-Net trained and run by this package's kernels, and the network-accelerated
LSQR solve that uses it."""

from .lsm import (LearnedLSM, SolveInfo, illumination_diagonal, make_pairs, point_spread_functions,
                  random_reflectivity, train)
from .unet import UNet

__all__ = ["UNet", "LearnedLSM", "SolveInfo", "illumination_diagonal", "make_pairs", "random_reflectivity", "train",
           "point_spread_functions"]
