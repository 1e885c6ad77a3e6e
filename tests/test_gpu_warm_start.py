"""The constraint warm start on the device, against the oracles (needs a GPU).

Tolerances:
* features: bit-exact (the same FP64 operations, rounded once to FP32);
* warm-started drift: bit-exact against the oracle's constraint::solve given
  the device's own predicted multipliers (positions, velocities, multiplier
  totals, iteration count);
* network output: FP32 sums against the oracle's FP64 sums, relative 1e-5
  for 99 % of samples (a BF16 rounding that falls the other way near a tie
  moves a few samples further, bounded at 5e-2);
* gradient of the training kernels: relative L2 1e-3 against the oracle;
* training: the trained network lowers the mean SHAKE iteration count of a
  different system at the same tolerance, and every solve still converges.
"""
import numpy as np
import pytest

import mlp
import oracle
from geodesic_cuda import amber, backend, synth

pytestmark = pytest.mark.gpu

DT = 0.004  # 4 fs, H bonds constrained
PARAMS = dict(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
              scale14_lj=0.5, scale14_coul=1 / 1.2, max_constr_iter=200, constr_tol=1e-10)


def constrained_system(n, seed):
    """Lattice chain with 40 % hydrogens, H bonds promoted to constraints."""
    atoms, topo, state, _ = synth.generate(n, seed=seed, h_fraction=0.4, temperature=300.0, relax_iters=1000)
    return atoms, amber.promote_hydrogen_bonds(topo, atoms), state


def test_warm_started_drift_matches_oracle():
    atoms, topo, state = constrained_system(1500, 31)
    nc = len(topo.constr_i)
    assert nc > 300
    p = backend.SimParams(**PARAMS)
    be = backend.CudaBackend(atoms, topo, p)
    pos, vel = np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel)
    f, scale, t1 = mlp.features(topo.constr_i, topo.constr_j, topo.constr_dsq, pos + DT * vel, pos,
                                1.0 / atoms.mass)
    sd = f.std(0)
    norm = np.concatenate([f.mean(0), np.where(sd > 0, sd, 1.0), [0.0, 1e-4]]).astype(np.float32)
    P = mlp.glorot(5)
    be.ws_params(P, norm)
    be.ws_enable(True)
    pg, vg = pos.copy(), vel.copy()
    be.geodesic_drift(pg, vg, DT, step=0)
    fd, lam0, lam_sum = be.ws_last(nc)
    assert np.array_equal(fd, f)
    y, _ = mlp.forward(P, mlp.standardize(f, norm))
    lam0_ref = (t1 + (y * norm[25] + norm[24])) / scale
    assert np.max(np.abs(lam0 - lam0_ref) / np.maximum(np.abs(lam0_ref), 1e-6)) < 1e-3
    pr, vr = pos.copy(), vel.copy()
    it, lam = oracle.drift_and_constrain_ws(pr, vr, topo, atoms, DT, PARAMS["max_constr_iter"],
                                            PARAMS["constr_tol"], lam0)
    assert np.array_equal(pg, pr)
    assert np.array_equal(vg, vr)
    assert np.array_equal(lam_sum, lam)
    assert be.counters()["shake_iters"] == it


def test_network_forward_and_gradient_match_oracle():
    atoms, topo, _ = constrained_system(300, 32)
    be = backend.CudaBackend(atoms, topo, backend.SimParams(**PARAMS))
    P = mlp.glorot(7)
    norm = np.array([0.0] * 12 + [1.0] * 12 + [0.0, 1.0], np.float32)
    be.ws_params(P, norm)
    rng = np.random.default_rng(8)
    x = rng.normal(size=(1000, 12)).astype(np.float32)
    t = (rng.normal(size=1000) * 0.5).astype(np.float32)
    y_dev = be.ws_forward(x)
    y_ref, _ = mlp.forward(P, x)
    err = np.abs(y_dev - y_ref) / np.maximum(np.abs(y_ref), 1.0)
    assert np.quantile(err, 0.99) < 1e-5, np.quantile(err, 0.99)
    assert err.max() < 5e-2
    g_dev, loss_dev = be.ws_gradient(x, t)
    g_ref, loss_ref = mlp.gradient(P, x, t)
    assert np.linalg.norm(g_dev - g_ref) / np.linalg.norm(g_ref) < 1e-3
    assert abs(loss_dev - loss_ref) / loss_ref < 1e-4
    # the same call twice: identical bits (fixed-order block sums)
    g2, l2 = be.ws_gradient(x, t)
    assert np.array_equal(g2, g_dev) and l2 == loss_dev


def run_counting(atoms, topo, state, n_steps, params=None, norm=None):
    be = backend.CudaBackend(atoms, topo, backend.SimParams(**PARAMS))
    be.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
    be.forces_resident()
    if params is not None:
        be.ws_params(params, norm)
        be.ws_enable(True)
    be.run_resident(DT, n_steps)
    be.synchronize()
    c = be.counters()
    pos, vel = np.zeros_like(state.pos), np.zeros_like(state.vel)
    be.download_state(pos, vel)
    return c["shake_iter_sum"] / c["constrained_steps"], c["constrained_steps"], pos


def test_trained_network_lowers_shake_iterations():
    """Train on solver multipliers of one system, use on another seed."""
    atoms, topo, state = constrained_system(3000, 41)
    be = backend.CudaBackend(atoms, topo, backend.SimParams(**PARAMS))
    be.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
    be.forces_resident()
    be.ws_record(200, 1)
    be.run_resident(DT, 200)
    be.synchronize()
    be.ws_record(0)
    f, t = be.ws_samples()
    assert len(t) == 200 * len(topo.constr_i)
    loss = be.ws_train(1500, blocks=32, lr=3e-3, seed=3)
    assert loss < 0.1, loss  # standardised: the network explains most of the correction
    P, norm = be.ws_params()
    atoms2, topo2, state2 = constrained_system(3000, 42)
    cold, n_cold, pos_cold = run_counting(atoms2, topo2, state2, 150)
    warm, n_warm, pos_warm = run_counting(atoms2, topo2, state2, 150, P, norm)
    assert n_cold == n_warm == 150
    assert warm < cold - 0.5, (cold, warm)
    # both trajectories satisfy the constraints to the solver's tolerance
    for pos in (pos_cold, pos_warm):
        d = pos[:, topo2.constr_i] - pos[:, topo2.constr_j]
        assert np.max(np.abs((d * d).sum(0) - topo2.constr_dsq)) < 1e-6
