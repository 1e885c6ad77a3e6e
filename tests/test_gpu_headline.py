"""The benchmark's own system against the oracle (needs a GPU).

The seeded 50,000-atom lattice chain of the throughput benchmark: jittered
2.15 A lattice, serpentine bonds / angles / dihedrals, 8 Lorentz-Berthelot
types, charges +-0.5 e with zero net, Coulomb with the LJ switch, 1-4 pairs
scaled by 1/2.0 (LJ) and 1/1.2 (Coulomb), cutoff 10 / switch 8 / list
radius 12 A, non-periodic, FIRE-minimised (1000 iterations), MB 300 K.

Tolerances, per force component, in the form of the reference's own GPU
test (geodesic-gpu/tests/forces_gpu_vs_cpu.rs:7-24):
  |F_gpu - F_oracle| <= tol * max(|F_oracle|, 1)
with tol = 1e-5 for the mixed path and 1e-10 for the FP64 path, plus the
global relative L2 error ||dF|| / ||F|| <= 1e-5 (mixed).  The pair set must
equal the oracle's as a set, and three runs of the resident loop must end in
bit-identical states (geodesic-gpu/tests/gpu_determinism.rs:7-21).
"""
import numpy as np
import pytest

import oracle
from geodesic_cuda import backend, synth

pytestmark = pytest.mark.gpu

N_ATOMS = 50_000
SEED = 20261203
PHYS = dict(box_size=(10000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
            scale14_lj=0.5, scale14_coul=1.0 / 1.2)
STEPS = 1000


@pytest.fixture(scope="module")
def system():
    atoms, topo, state, _ = synth.generate(N_ATOMS, seed=SEED, temperature=300.0, relax_iters=1000)
    return atoms, topo, state


def oracle_reference(atoms, topo, pos):
    op = oracle.make_params(box=PHYS["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0,
                            n_threads=0, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2)
    pi, pj = oracle.neighbor_build(pos.copy(), atoms, topo, op, cells=True)
    ob = oracle.CpuBackend(atoms, topo, op)
    ob.set_pairs(pi, pj, pos)
    f = ob.compute_forces(pos).copy()
    return (pi, pj), f, ob.potential_energy


def device_forces(atoms, topo, pos, precision):
    be = backend.CudaBackend(atoms, topo, backend.SimParams(precision=precision, **PHYS))
    p = np.ascontiguousarray(pos.copy())
    be.build_neighbor_list(p)
    f = be.compute_forces(p).copy()
    out = (be.pairs(), f, be.potential_energy())
    be.close()
    return out


def check_state(atoms, topo, pos, label):
    (ri, rj), f_ref, e_ref = oracle_reference(atoms, topo, pos)
    scale = np.maximum(np.abs(f_ref), 1.0)
    for precision, tol in ((backend.PRECISION_MIXED, 1e-5), (backend.PRECISION_FP64, 1e-10)):
        (gi, gj), f, e = device_forces(atoms, topo, pos, precision)
        assert len(gi) == len(ri) and np.array_equal(gi, ri) and np.array_equal(gj, rj), label
        per = np.abs(f - f_ref) / scale
        assert per.max() <= tol, (label, precision, per.max())
        rel = np.linalg.norm(f - f_ref) / np.linalg.norm(f_ref)
        assert rel <= tol, (label, precision, rel)
        assert abs(e - e_ref) <= tol * abs(e_ref), (label, precision, e, e_ref)


def test_headline_forces_at_minimised_start(system):
    atoms, topo, state = system
    check_state(atoms, topo, np.ascontiguousarray(state.pos), "step 0")


def test_headline_forces_after_run_and_reruns_identical(system):
    """1,000 resident mixed-precision steps at 2 fs (list rebuilds inside
    the graph), three times from the same state: bit-identical end states;
    then both device paths against the oracle at the step-1000 coordinates."""
    atoms, topo, state = system
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **PHYS)
    ends = []
    for _ in range(3):
        be = backend.CudaBackend(atoms, topo, p)
        pos = np.ascontiguousarray(state.pos.copy())
        vel = np.ascontiguousarray(state.vel.copy())
        e, n_reb, _ = be.steps(pos, vel, 0.002, STEPS)
        ends.append((pos, vel, e, n_reb))
        be.close()
    assert ends[0][3] >= 1  # the run rebuilt its list at least once
    for pos, vel, e, n_reb in ends[1:]:
        assert np.array_equal(pos.view(np.uint64), ends[0][0].view(np.uint64))
        assert np.array_equal(vel.view(np.uint64), ends[0][1].view(np.uint64))
        assert e == ends[0][2] and n_reb == ends[0][3]
    check_state(atoms, topo, ends[0][0], f"step {STEPS}")
