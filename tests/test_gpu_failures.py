"""Device error paths, provoked from the host with valid inputs (needs a GPU).

Neither test faults, traps or hangs the device: the kernels record the
condition in the status word, finish their launches, and the host turns the
word into an error code.

* A neighbour list that outgrows its capacity inside a resident run: a
  resident run cannot grow the list, so the in-graph rebuild stores at most
  `cap` entries per atom (writes stay inside the buffer), sets the overflow
  bit, and the call returns GM_ERR_LIST_OVERFLOW.  The reference grows its
  Vec instead; the code maps to BackendError (geodesic-core/src/error.rs:
  SimError::Backend).  The context stays usable: the next host-side build
  regrows the list.
* A pair force beyond the fixed-point range (|F| >= 2^22 kcal/mol/A): the
  force evaluation returns GM_ERR_FIXED_POINT_OVERFLOW and, since the trait's
  compute_forces is infallible, hands back NaN forces, which the run loop's
  check_forces_finite turns into NumericalError::NanInForce
  (geodesic/src/lib.rs:79-92, geodesic-core/src/error.rs:34-38).
* The persistent step's grid barrier is bounded: with its arrival count
  preset past the grid from the host (gm_stall_next_barrier), no block can
  release it, every block waits out the poll limit (a fraction of a second),
  records the timeout and returns.  gm_steps reports GM_ERR_DEVICE with
  nothing stepped, and the next call steps normally.
"""
import numpy as np
import pytest

import oracle
from geodesic_cuda import amber, backend, synth

pytestmark = pytest.mark.gpu

PARAMS = dict(box_size=(10000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)


def inert_gas(n, density, seed):
    """n atoms without LJ parameters or charges (no forces at all) spread
    uniformly over a ball of the given number density, centred at 5000 A."""
    rng = np.random.default_rng(seed)
    radius = (3.0 * n / (4.0 * np.pi * density)) ** (1.0 / 3.0)
    d = rng.normal(size=(3, n))
    d *= radius * rng.uniform(0.0, 1.0, n) ** (1.0 / 3.0) / np.linalg.norm(d, axis=0)
    atoms = amber.AtomData(np.zeros(n), np.zeros(n), np.full(n, 12.0), np.zeros(n), np.full(n, 5, np.uint8),
                           np.zeros(n, np.uint32), ["C   "] * n)
    return atoms, np.ascontiguousarray(d + 5000.0)


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_list_overflow_inside_a_resident_run(precision):
    n, steps, dt = 1500, 200, 0.002
    atoms, pos = inert_gas(n, 0.0125, seed=4)
    # every atom drifts straight to the centre: after `steps` steps the ball
    # has shrunk to 40 % of its radius, 15.6 times the density it was sized for
    centre = pos.mean(axis=1, keepdims=True)
    vel = np.ascontiguousarray(-(pos - centre) * (0.6 / (steps * dt)))
    be = backend.CudaBackend(atoms, amber.BondedTopology.empty(), backend.SimParams(precision=precision, **PARAMS))
    with pytest.raises(backend.BackendError) as e:
        be.steps(pos, vel, dt, steps)
    assert e.value.status == 7, e.value  # GM_ERR_LIST_OVERFLOW
    # the context is still usable: a host-side build regrows the list and
    # finds the oracle's pairs at the compressed positions
    p2 = np.ascontiguousarray(centre + (pos - centre) * 0.4)
    be.build_neighbor_list(p2)
    gi, gj = be.pairs()
    op = oracle.make_params(box=PARAMS["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)
    ri, rj = oracle.neighbor_build(p2.copy(), atoms, amber.BondedTopology.empty(), op, cells=True)
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    be.close()


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_fixed_point_overflow_gives_nan_forces(precision):
    # sigma 3 A, epsilon 0.2 kcal/mol, 0.2 A apart: |F| ~ 1e15 kcal/mol/A
    atoms = amber.AtomData(np.full(2, 3.0), np.full(2, 0.2), np.full(2, 12.0), np.zeros(2), np.full(2, 5, np.uint8),
                           np.zeros(2, np.uint32), ["C   "] * 2)
    pos = np.ascontiguousarray([[5000.0, 5000.2], [5000.0, 5000.0], [5000.0, 5000.0]])
    be = backend.CudaBackend(atoms, amber.BondedTopology.empty(), backend.SimParams(precision=precision, **PARAMS))
    be.build_neighbor_list(pos)
    with pytest.raises(backend.BackendError) as e:
        be.compute_forces(pos)
    assert e.value.status == 9, e.value  # GM_ERR_FIXED_POINT_OVERFLOW
    assert np.all(np.isnan(be.reduce_forces()))
    # a sane geometry afterwards evaluates normally
    ok = np.ascontiguousarray([[5000.0, 5003.5], [5000.0, 5000.0], [5000.0, 5000.0]])
    be.build_neighbor_list(ok)
    f = be.compute_forces(ok)
    assert np.all(np.isfinite(f)) and f[0, 0] == -f[0, 1]
    be.close()


def test_nonfinite_position_in_a_resident_call():
    """gm_steps checks the caller's positions on the device when the resident
    forces are current: a NaN is NumericalError (lib.rs:94-107), and the
    context carries on with valid positions afterwards."""
    atoms, pos = inert_gas(400, 0.05, seed=9)
    vel = np.ascontiguousarray(np.zeros_like(pos))
    be = backend.CudaBackend(atoms, amber.BondedTopology.empty(), backend.SimParams(**PARAMS))
    be.steps(pos, vel, 0.002, 3)
    bad = pos.copy()
    bad[1, 17] = np.nan
    with pytest.raises(backend.NumericalError):
        be.steps(bad, vel, 0.002, 1)
    be.steps(pos, vel, 0.002, 2)
    assert np.all(np.isfinite(pos))
    be.close()


def test_persistent_barrier_timeout_is_reported_and_recovered():
    atoms, topo, state, _ = synth.generate(2000, seed=12, temperature=300.0, relax_iters=100)
    params = backend.SimParams(precision=backend.PRECISION_MIXED, **PARAMS)
    be = backend.CudaBackend(atoms, topo, params)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    be.steps(pos, vel, 0.002, 5)
    p0, v0 = pos.copy(), vel.copy()
    be.stall_next_barrier()
    with pytest.raises(backend.BackendError) as e:
        be.steps(pos, vel, 0.002, 3)
    assert e.value.status == 4 and "barrier" in str(e.value), e.value  # GM_ERR_DEVICE
    # nothing was stepped: the caller's state is the state it handed in
    assert np.array_equal(pos, p0) and np.array_equal(vel, v0)
    # the context carries on: three steps from there agree with a fresh
    # context's three steps from the same state (lists built at different
    # positions hold the same in-cutoff pairs; only summation order differs)
    be.steps(pos, vel, 0.002, 3)
    fresh = backend.CudaBackend(atoms, topo, params)
    p1, v1 = p0.copy(), v0.copy()
    fresh.steps(p1, v1, 0.002, 3)
    assert np.all(np.isfinite(pos)) and np.allclose(pos, p1, rtol=0, atol=1e-8)
    assert np.allclose(vel, v1, rtol=0, atol=1e-6)
    fresh.close()
    be.close()


def test_barrier_stall_needs_the_persistent_form():
    atoms = amber.AtomData(np.full(2, 3.0), np.full(2, 0.2), np.full(2, 12.0), np.zeros(2), np.full(2, 5, np.uint8),
                           np.zeros(2, np.uint32), ["C   "] * 2)
    be = backend.CudaBackend(atoms, amber.BondedTopology.empty(),
                             backend.SimParams(precision=backend.PRECISION_FP64, **PARAMS))
    with pytest.raises(backend.BackendError) as e:
        be.stall_next_barrier()
    assert e.value.status == 8  # GM_ERR_UNSUPPORTED
    be.close()
