"""What the trained network gains: on a reduced version of the learned-LSM
workload (2-D dynamic eikonal, v(z) = 1500 + 0.6 z), a U-Net trained on
operator-generated pairs must bring LSQR to the same 1e-2 data residual in
fewer operator applications than plain LSQR from zero, with a model error
no worse; the residual is recomputed for both, as plain LSQR measures it."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


def test_learned_solve_beats_plain_lsqr_on_held_out_models():
    from pylops_gb300.learned import LearnedLSM, UNet, make_pairs, random_reflectivity, train
    from pylops_gb300.learned.experiment import lsm_operator

    op = lsm_operator(nz=64, nx=128, ns=12, nr=48, nt=500)
    op.autotune()
    X, M = make_pairs(op, 512, seed=1)
    net = UNet(levels=4, base=16, seed=1)
    losses = train(net, X, M, steps=800, batch=8, lr=1e-3)
    assert np.mean(losses[-20:]) < 0.75 * np.mean(losses[:20])
    plain, learned = LearnedLSM(op), LearnedLSM(op, net=net, steps=4)
    rng = np.random.default_rng(77)
    d = torch.empty(op.shape[0], device="cuda")
    pp, lp, pe, le = [], [], [], []
    for _ in range(4):
        m = torch.as_tensor(random_reflectivity(128, 64, rng).reshape(-1), device="cuda")
        op.apply_into(m, d)
        xp, ip = plain.solve(d, tol=1e-2, niter=500)
        xl, il = learned.solve(d, tol=1e-2, niter=500)
        assert ip.residual <= 1.0001e-2 and il.residual <= 1.0001e-2
        assert il.network_steps >= 1 and il.network_residual < 0.5
        pp.append(ip.operator_pairs)
        lp.append(il.operator_pairs)
        mn = float(torch.linalg.norm(m))
        pe.append(float(torch.linalg.norm(xp - m)) / mn)
        le.append(float(torch.linalg.norm(xl - m)) / mn)
    print("operator pairs plain", pp, "learned", lp, "model error plain", pe, "learned", le)
    assert np.median(lp) < 0.8 * np.median(pp)
    assert np.median(le) <= np.median(pe)
    # the host-data path gives the same model
    xh, ih = learned.solve(d.cpu().numpy(), tol=1e-2, niter=500)
    xd, idv = learned.solve(d, tol=1e-2, niter=500)
    assert isinstance(xh, np.ndarray) and np.array_equal(xh, xd.cpu().numpy())
