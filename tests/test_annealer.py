"""Host logic of the placement annealer (automs_gb300/placement.py) with a
fake study and a stub surrogate on the CPU."""
import numpy as np
import torch

from automs_gb300 import placement


class FakeStudy:
    sizes = (8, 24)

    def random_params(self, rng):
        return (int(rng.integers(0, 3)), float(rng.uniform(0.1, 0.9)),
                float(rng.uniform(0.1, 0.9)), int(rng.choice([8, 16, 24])))

    def descriptor(self, p):
        w, u, v, s = p
        return np.array([w, u, v, s / 24.0], np.float32)


def stub_surrogate(X):
    # predicted gain map (4 pooled cells): best near u = 0.7, v = 0.3, wall 2
    u, v, w = X[:, 1], X[:, 2], X[:, 0]
    g = -((u - 0.7) ** 2 + (v - 0.3) ** 2) * 10 + (w == 2).float()
    return g[:, None].repeat(1, 4)


def test_annealer_moves_stay_in_bounds_and_climb():
    rng = np.random.Generator(np.random.PCG64(0))
    study = FakeStudy()
    vis = placement.anneal_candidates(study, 3000, rng, surrogate=stub_surrogate, device="cpu")
    assert len(vis) == 3000
    P = np.array([[w, u, v, s] for w, u, v, s in vis], np.float64)
    assert set(np.unique(P[:, 0])) <= {0, 1, 2}
    assert P[:, 1].min() >= 0.1 and P[:, 1].max() <= 0.9
    assert P[:, 2].min() >= 0.1 and P[:, 2].max() <= 0.9
    assert set(np.unique(P[:, 3])) <= {8, 16, 24}
    sc = placement.score(stub_surrogate(torch.as_tensor(
        np.stack([study.descriptor(q) for q in vis])))).numpy()
    assert sc[-500:].mean() > sc[:500].mean() + 0.3


def test_annealer_without_surrogate_is_a_random_walk():
    rng = np.random.Generator(np.random.PCG64(1))
    vis = placement.anneal_candidates(FakeStudy(), 700, rng)
    assert len(vis) == 700 and len(set(vis)) > 600
