"""The FP64 oracle of the adjoint path: the material VJP of the gradient and
the implicit gradient of the equilibrium, both against central differences.
These pin the oracle the GPU adjoint tests compare with."""

import numpy as np
import pytest

from apple_gb300 import meshgen
from oracle import fem_oracle as O


def _potential(material, m, rng, E=1e4):
    lam_e, mu_e = meshgen.lame_converter(E, 0.4)
    mu = mu_e * rng.uniform(0.5, 2.0, m.n_cells)
    lam = lam_e * np.ones(m.n_cells) if material == O.Material.STABLE_NEO_HOOKEAN else None
    return O.FemPotential.from_mesh(material, m.points, m.cells, mu=mu, lam=lam)


@pytest.mark.parametrize("material", [O.Material.STABLE_NEO_HOOKEAN, O.Material.ARAP])
def test_grad_param_vjp_matches_central_difference(material):
    rng = np.random.default_rng(3)
    m = meshgen.grid(2, 2, 3)
    pot = _potential(material, m, rng)
    u = 0.05 * rng.normal(size=(m.n_points, 3))
    w = rng.normal(size=(m.n_points, 3))
    dmu, dlam = pot.grad_param_vjp(u, w)
    for c in (0, 7, m.n_cells - 1):
        def wg(which, h):
            arr = pot.mu if which == "mu" else pot.lam
            old = arr[c]
            arr[c] = old + h
            val = float(np.sum(w * pot.grad(u)))
            arr[c] = old
            return val

        h = 1e-6 * pot.mu[c]
        fd = (wg("mu", h) - wg("mu", -h)) / (2 * h)
        assert dmu[c] == pytest.approx(fd, rel=1e-6, abs=1e-12)
        if dlam is not None:
            h = 1e-6 * pot.lam[c]
            fd = (wg("lam", h) - wg("lam", -h)) / (2 * h)
            assert dlam[c] == pytest.approx(fd, rel=1e-6, abs=1e-12)


def test_implicit_gradient_matches_central_difference_of_forward():
    rng = np.random.default_rng(5)
    m = meshgen.grid(2, 2, 4, h=0.5)
    pot = _potential(O.Material.STABLE_NEO_HOOKEAN, m, rng, E=3e5)
    mask = np.zeros((m.n_points, 3), bool)
    mask[meshgen.face_mask(m, 2, "min")] = True
    f = meshgen.lumped_gravity(m, 1000.0)
    top = meshgen.face_mask(m, 2, "max")
    target = rng.normal(scale=0.01, size=(int(top.sum()), 3))

    def forward():
        model = O.Model(O.DofMap(m.n_points, mask, np.zeros((m.n_points, 3))), [pot],
                        O.ExternalForce(np.arange(m.n_points), f))
        u, st = O.solve_model(model, rtol=1e-13, max_steps=20000)
        return model, u

    def loss(u):
        return 0.5 * float(np.sum((u[top] - target) ** 2))

    model, u = forward()
    dLdu = np.zeros_like(u)
    dLdu[top] = u[top] - target
    dmu, dlam, lam = O.equilibrium_param_grad(model, pot, u, dLdu)
    # the adjoint solves H lam = dL/du on the free DOFs
    r = model.hess_prod(u, lam) - dLdu
    assert np.linalg.norm(r.reshape(-1)[model.dof_map.free_indices]) < 1e-8 * np.linalg.norm(dLdu)
    for c in (1, 11, m.n_cells - 2):
        old = pot.mu[c]
        h = 1e-3 * old
        pot.mu[c] = old + h
        lp = loss(forward()[1])
        pot.mu[c] = old - h
        lm = loss(forward()[1])
        pot.mu[c] = old
        fd = (lp - lm) / (2 * h)
        assert dmu[c] == pytest.approx(fd, rel=1e-3)
