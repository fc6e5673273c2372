"""Surrogate screening of metasurface placements: the trained MLP must beat
the constant-mean predictor and let annealing rank candidates at >= 10x the
configs/s of the plain ray-trace + adjoint loop."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_surrogate_screening_gains():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import placement, surrogate
    study = placement.PlacementStudy(seed=1, rx=(32, 32), launch=128, pool=2, opt_steps=12)
    Xtr, Ytr, _ = study.dataset(320, seed=1)
    Xva, Yva, Pva = study.dataset(80, seed=2)
    mu, sd = Ytr.mean(0), Ytr.std() + 1e-6
    net = surrogate.MLP([Xtr.shape[1], 512, 512, 512, 512, Ytr.shape[1]], max_batch=512, seed=0)
    hist = net.fit(torch.as_tensor(Xtr).cuda(), torch.as_tensor((Ytr - mu) / sd).cuda(), epochs=150,
                   batch=64, lr=1e-3, lr_decay=0.99)
    assert hist[-1] < 0.5 * hist[0]

    class Denorm:
        def __call__(self, X):
            return net(X) * sd + torch.as_tensor(mu, device="cuda")

    rep = placement.screening_report(study, Denorm(), Pva, Yva, top_frac=0.1)
    print(rep)
    assert rep["surrogate_median_abs_err_db"] < rep["mean_predictor_median_abs_err_db"]
    assert rep["screened_configs_per_s"] >= 5.0 * rep["plain_configs_per_s"]
    # annealing driven by the surrogate visits valid placements
    cands = placement.anneal_candidates(study, 600, np.random.Generator(np.random.PCG64(0)),
                                        surrogate=Denorm())
    assert len(cands) == 600
    net.close()


def test_batched_placements_small():
    """The batched hyper-config driver on a small building: every placement
    is traced and optimised; channels have the expected shapes."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import placement, scenes
    cfg = scenes.batch_config(n_place=4, target_tris=8_000, n_rx=32, launch=96)
    res, wall = placement.batch_evaluate(cfg, workers=2, opt_steps=3)
    assert len(res) == 4 and wall > 0
    for r, p in zip(sorted(res, key=lambda x: x["index"]), cfg["placements"]):
        assert r["M"] == p["size"] ** 2
        assert np.isfinite(r["loss_first"]) and np.isfinite(r["loss_last"])
        assert r["loss_last"] <= r["loss_first"] + 1e-6 * abs(r["loss_first"])
