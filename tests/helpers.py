"""Shared test helpers: build the GB300 operator and the oracle from a golden record."""

import os

import numpy as np

from tests.conftest import GOLDEN


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def kwargs_from_golden(g):
    kw = dict(y=g.get("y"), dynamic=bool(g["dynamic"]))
    if "vel_model" in g:
        vel = g["vel_model"]
        kw.update(mode="byot", trav=(g["trav_in_srcs"], g["trav_in_recs"]),
                  amp=(g["amp_in_srcs"], g["amp_in_recs"]))
    else:
        vel = float(g["vel_scalar"])
        kw.update(mode="analytic")
    if "aperture_in" in g:
        kw["aperture"] = float(g["aperture_in"])
    if "angleaperture_in" in g:
        kw["angleaperture"] = float(g["angleaperture_in"])
    elif bool(g["dynamic"]):
        kw["angleaperture"] = None if np.allclose(g["angleaperture"], np.deg2rad([0.0, 1000.0])) else 90.0
    wav = g["wav"]
    if "wavfilter_in" in g:  # the golden's wav is the reshaped one; the constructor gets the original
        kw["wavfilter"] = True
        wav = g["wav_in"]
    args = (g["z"], g["x"], g["t"], g["srcs"], g["recs"], vel, wav, int(g["wavc"]))
    return args, kw


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


GOLDEN_CASES = ["k2d_kin", "k2d_dyn_ap", "k2d_dyn_noap", "k3d_kin", "k3d_dyn", "k2d_dyn_byot", "k2d_kin_f32",
                "k2d_wavfilter", "k3d_wavfilter"]
