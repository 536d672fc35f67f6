"""bf16 dynamic weights (8-byte table records): the results move by about
1e-3 relative from the reference's float64 values (each weight keeps 8
significant bits); float32 weights stay within 1e-5.  Tolerance for bf16:
5e-3 relative L2, stated here and in the operator's documentation."""

import numpy as np
import pytest

from tests.helpers import kwargs_from_golden, load, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["k2d_dyn_ap", "k2d_dyn_noap", "k3d_dyn", "k2d_dyn_byot"])
def test_bf16_weights_against_reference(name):
    import torch

    from pylops_gb300.waveeqprocessing import Kirchhoff

    g = load(name)
    args, kw = kwargs_from_golden(g)
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    K.set_weight_precision("bfloat16")
    for v in (0, 1):
        K.set_spread_variant(v)
        ef = rel(K @ g["m_in"], g["fwd"])
        assert 1e-6 < ef < 5e-3, (v, ef)
    ea = rel(K.H @ g["d_in"], g["adj"])
    assert 1e-6 < ea < 5e-3, ea
    x = torch.randn(K.ni, device="cuda")
    assert torch.equal(K @ x, K @ x)
    K.set_weight_precision("float32")
    assert rel(K @ g["m_in"], g["fwd"]) < 1e-5 and rel(K.H @ g["d_in"], g["adj"]) < 1e-5


def test_bf16_weights_reject_kinematic_operator():
    from pylops_gb300.waveeqprocessing import Kirchhoff

    args, kw = kwargs_from_golden(load("k2d_kin"))
    K = Kirchhoff(*args, engine="cuda", dtype="float32", **kw)
    with pytest.raises(ValueError):
        K.set_weight_precision("bfloat16")
