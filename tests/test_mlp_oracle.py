"""CPU pins of the warm-start network's oracle (oracle/mlp.py).

* BF16 rounding: the emulation equals torch's float32 -> bfloat16 conversion
  (round to nearest, ties to even).
* Backward pass: the FP64 gradient equals central finite differences of the
  FP64 loss (no BF16 rounding in this check), relative 1e-6.
* First Jacobi step: t1 from the features equals the first lambda of the
  oracle's own cold solve times 2 (1/m_i + 1/m_j), relative 1e-12.
"""
import numpy as np
import pytest

import mlp
import oracle
from geodesic_cuda import amber


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.normal(size=20000).astype(np.float32),
                        rng.uniform(-1e-3, 1e-3, 5000).astype(np.float32),
                        # exact ties between two BF16 values, both parities
                        (np.arange(1, 2001, dtype=np.uint32) << 16 | 0x8000).view(np.float32)])
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(mlp.bf16(x), ref)


def test_gradient_matches_finite_differences():
    P = mlp.glorot(1).astype(np.float64)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(64, 12)).astype(np.float32)
    t = rng.normal(size=64)
    g, loss = mlp.gradient(P, x, t, emulate_bf16=False)

    def L(Q):
        y, _ = mlp.forward(Q, x, emulate_bf16=False)
        return np.mean((y - t) ** 2)

    assert abs(L(P) - loss) <= 1e-14 * loss
    eps = 1e-6
    for k in list(range(0, 768, 97)) + list(range(768, 832, 13)) + list(range(832, 4928, 401)) + \
            list(range(4928, 5057, 17)) + [5056]:
        Pp, Pm = P.copy(), P.copy()
        Pp[k] += eps
        Pm[k] -= eps
        fd = (L(Pp) - L(Pm)) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(abs(g[k]), 1e-3), (k, fd, g[k])


def test_first_jacobi_step_matches_oracle_solver():
    """t1 of the features is the reference's first lambda (constraint.rs:110-115) x 2 (1/m_i + 1/m_j)."""
    rng = np.random.default_rng(3)
    n = 40
    pos0 = rng.normal(size=(3, n)) * 3.0
    ci = np.arange(0, n, 2, dtype=np.uint32)
    cj = ci + 1
    pos0[:, cj] = pos0[:, ci] + rng.normal(size=(3, len(ci))) * 0.6
    d = pos0[:, ci] - pos0[:, cj]
    dsq = (d * d).sum(0) * (1.0 + rng.uniform(-0.01, 0.01, len(ci)))
    mass = rng.uniform(1.0, 16.0, n)
    atoms = amber.AtomData(np.ones(n), np.ones(n), mass, np.zeros(n), np.ones(n, np.uint8),
                           np.zeros(n, np.uint32), ["C   "] * n)
    topo = amber.BondedTopology.empty()
    topo.constr_i, topo.constr_j, topo.constr_dsq = ci, cj, dsq
    trial = pos0 + rng.normal(size=(3, n)) * 0.01
    f, scale, t1 = mlp.features(ci, cj, dsq, trial, pos0, 1.0 / mass)
    # the summed multipliers of a cold solve stopped after its first sweep
    it, lam1 = oracle.constraint_solve(topo, atoms, pos0, trial.copy(), 1, 1e300, want_lambda=True)
    assert it == 1
    # t1 is the first Jacobi step from FP64 differences rounded once to FP32
    # (numerator, denominator, quotient): within 3 FP32 roundings
    np.testing.assert_allclose(t1, lam1 * scale, rtol=3 * 2.0 ** -24, atol=0)
    assert f.dtype == np.float32 and f.shape == (len(ci), 12)
