"""CPU: the torch side of the many-body derivatives -- the loss's derivative
along a state tangent (tangent_loss_gradient) against a central difference
of the loss along the same tangent."""
import numpy as np
import pytest

from posidonius_gb300 import adjoint as A
from posidonius_gb300 import ensemble as E, layout as L


@pytest.mark.parametrize("seed", [0, 1])
def test_tangent_loss_gradient_matches_directional_difference(seed):
    pytest.importorskip("torch")
    import torch

    case = E.workload_large(13, seed=seed)
    bf = case["body_f64"].copy()
    n = bf.shape[0]
    for i in range(n):  # spins as posi_large_initialize_physical_values sets them
        bf[i, L.SPIN] = bf[i, L.ANG] / bf[i, L.BF_MOI]
    host, planets = 0, (1, 2)
    idx = [host, *planets]
    t = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64)
    with torch.no_grad():
        a0, _ = A.orbital_elements(t(bf[idx][:, L.POS])[None], t(bf[idx][:, L.VEL])[None],
                                   t(bf[idx][:, L.BF_MASS])[None])
    a0 = a0[0].numpy() * 1.01
    spin0 = np.linalg.norm(bf[1:3, L.ANG], axis=-1) / bf[1:3, L.BF_MOI] * 0.98
    rng = np.random.default_rng(seed)
    tan = np.zeros((2, n, 12))
    for d in range(2):
        tan[d, :, 0:3] = rng.normal(size=(n, 3)) * 1e-3
        tan[d, :, 3:6] = rng.normal(size=(n, 3)) * 1e-5
        tan[d, :, 6:9] = rng.normal(size=(n, 3)) * np.linalg.norm(bf[:, L.ANG], axis=1)[:, None] * 1e-3

    def loss_at(eps, d):
        b = bf.copy()
        b[:, L.POS] += eps * tan[d, :, 0:3]
        b[:, L.VEL] += eps * tan[d, :, 3:6]
        b[:, L.ANG] += eps * tan[d, :, 6:9]
        return A.tangent_loss_gradient(b, tan[:1], host, planets, a0, spin0)[0]

    loss, grad = A.tangent_loss_gradient(bf, tan, host, planets, a0, spin0)
    assert np.isfinite(loss) and loss > 0
    for d in range(2):
        h = 1e-4
        fd = (loss_at(h, d) - loss_at(-h, d)) / (2 * h)
        fd2 = (loss_at(h / 2, d) - loss_at(-h / 2, d)) / h
        assert abs(grad[d] - fd) <= 1e-7 * abs(fd) + 3 * abs(fd - fd2), (d, grad[d], fd)
