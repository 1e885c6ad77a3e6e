"""The persistent step form against the kernel-graph form (needs a GPU).

gm_step_form(GM_STEP_PERSISTENT) issues each unconstrained mixed-precision
step as one cooperative launch: forces at the current positions from one work
queue (pair items and bonded / 1-4 chunks of every system), a grid barrier,
then kick, drift, rebuild check and pack; the rebuild stays in the graph's IF
node.  Its force sums are integer sums and its integrator arithmetic rounds
like the integrator kernels, so it must reproduce the kernel graph's run bit
for bit:
* a single system (non-periodic with Coulomb and 1-4 terms, and periodic
  with and without the nearest image in the bonded terms), resident runs over several
  gm_steps calls with list rebuilds: positions, velocities, potential energy
  and rebuild counts;
* a batch of systems of uneven size: every member's state and the
  per-system energies;
* gm_time_steps (every timed launch evaluates its forces);
* the force phase alone (gm_compute_forces in the persistent form) against
  the force kernels: the same forces, energy and per-system energies;
and it is refused for FP64 and constrained contexts (GM_ERR_UNSUPPORTED).
The potential energy gm_steps returns is the one at the positions it
returns, call after call, in both forms (against the oracle, lib.rs:292-323
reports the energy of the step's closing force evaluation).
"""
import numpy as np
import pytest

import oracle
from geodesic_cuda import amber, backend, synth

pytestmark = pytest.mark.gpu

DT = 0.002
OPEN = dict(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
            scale14_lj=0.5, scale14_coul=1 / 1.2)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def run(atoms, topo, state, params, form, chunks, ensemble=False):
    if ensemble:
        be = backend.CudaBackend.ensemble(atoms, topo, params)
    else:
        be = backend.CudaBackend(atoms, topo, params)
    be.step_form(form)
    pos = np.ascontiguousarray(state[0].copy())
    vel = np.ascontiguousarray(state[1].copy())
    energies, rebuilds = [], 0
    first = 0
    for n in chunks:
        e, nr, _ = be.steps(pos, vel, DT, n, first_step=first)
        energies.append(e)
        rebuilds += nr
        first += n
    sys_e = be.ensemble_energies()[0].copy() if ensemble else None
    be.close()
    return pos, vel, energies, rebuilds, sys_e


def assert_same(a, b):
    pos_a, vel_a, e_a, nr_a, se_a = a
    pos_b, vel_b, e_b, nr_b, se_b = b
    assert np.array_equal(bits(pos_a), bits(pos_b))
    assert np.array_equal(bits(vel_a), bits(vel_b))
    assert e_a == e_b
    assert nr_a == nr_b
    if se_a is not None:
        assert np.array_equal(bits(se_a), bits(se_b))


def test_single_system_bit_identical_over_calls_with_rebuilds():
    atoms, topo, state, _ = synth.generate(5000, seed=77, temperature=600.0, relax_iters=400)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **OPEN)
    chunks = (1, 149, 250)  # a one-step call, then longer ones
    g = run(atoms, topo, (state.pos, state.vel), p, backend.STEP_GRAPH, chunks)
    q = run(atoms, topo, (state.pos, state.vel), p, backend.STEP_PERSISTENT, chunks)
    assert g[3] >= 1  # the run rebuilt its list
    assert_same(g, q)


@pytest.mark.parametrize("form", [backend.STEP_GRAPH, backend.STEP_PERSISTENT])
def test_energy_of_every_call_is_current(form):
    atoms, topo, state, _ = synth.generate(2000, seed=76, temperature=600.0, relax_iters=300)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **OPEN)
    be = backend.CudaBackend(atoms, topo, p)
    be.step_form(form)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    op = oracle.make_params(box=OPEN["box_size"], periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0,
                            n_threads=0, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2)
    seen = []
    for n in (1, 40, 60):
        e, _, _ = be.steps(pos, vel, DT, n)
        pi, pj = oracle.neighbor_build(pos.copy(), atoms, topo, op, cells=True)
        ob = oracle.CpuBackend(atoms, topo, op)
        ob.set_pairs(pi, pj, pos)
        ob.compute_forces(pos.copy())
        assert abs(e - ob.potential_energy) <= 1e-6 * abs(ob.potential_energy), (n, e, ob.potential_energy)
        seen.append(e)
    assert len(set(seen)) == 3
    be.close()


def charged_fluid(side=14, spacing=3.7, seed=5):
    """A periodic charged LJ fluid without bonded terms: a jittered cubic
    lattice near the LJ minimum (sigma 3 A, epsilon 0.2 kcal/mol, charges
    +-0.3 e alternating), Maxwell-Boltzmann velocities at 600 K."""
    rng = np.random.default_rng(seed)
    g = np.arange(side) * spacing + spacing / 2
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1) + rng.uniform(-0.2, 0.2, (3, side ** 3))
    n = pos.shape[1]
    q = np.where(np.arange(n) % 2 == 0, 0.3, -0.3)
    atoms = amber.AtomData(np.full(n, 3.0), np.full(n, 0.2), np.full(n, 12.0), q, np.full(n, 5, np.uint8),
                           np.zeros(n, np.uint32), ["C   "] * n)
    vel = rng.normal(size=(3, n)) * np.sqrt(0.0019872041 * 600.0 / 12.0 * 418.4)
    return atoms, np.ascontiguousarray(pos), np.ascontiguousarray(vel - vel.mean(axis=1, keepdims=True)), side * spacing


@pytest.mark.parametrize("bonded_mi", [False, True])
def test_periodic_system(bonded_mi):
    if bonded_mi:
        atoms, topo, state, _ = synth.generate(4000, seed=78, temperature=600.0, relax_iters=400)
        lo = state.pos.min(axis=1, keepdims=True)
        pos = np.ascontiguousarray(state.pos - lo + 1.0)
        vel = state.vel
        box = float(np.ceil(pos.max())) + 2.0
    else:
        # raw bonded differences across the faces (the reference's
        # behaviour) blow up once a molecule wraps: without the nearest image
        # the run is a fluid without bonded terms (the periodic pair path)
        atoms, pos, vel, box = charged_fluid()
        topo = amber.BondedTopology.empty()
    p = backend.SimParams(precision=backend.PRECISION_MIXED, box_size=(box,) * 3, periodic=True,
                          bonded_min_image=bonded_mi, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
                          scale14_lj=0.5, scale14_coul=1 / 1.2)
    chunks = (120, 180)
    g = run(atoms, topo, (pos, vel), p, backend.STEP_GRAPH, chunks)
    q = run(atoms, topo, (pos, vel), p, backend.STEP_PERSISTENT, chunks)
    assert g[3] >= 1
    assert_same(g, q)


def test_batch_of_uneven_systems():
    syss = [synth.generate(n, seed=s, temperature=600.0, relax_iters=300) for n, s in
            ((600, 81), (2300, 82), (900, 83), (4100, 84), (1300, 85))]
    atoms = [s[0] for s in syss]
    topo = [s[1] for s in syss]
    pos = np.concatenate([s[2].pos for s in syss], axis=1)
    vel = np.concatenate([s[2].vel for s in syss], axis=1)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **OPEN)
    chunks = (50, 250)
    g = run(atoms, topo, (pos, vel), p, backend.STEP_GRAPH, chunks, ensemble=True)
    q = run(atoms, topo, (pos, vel), p, backend.STEP_PERSISTENT, chunks, ensemble=True)
    assert g[3] >= 1
    assert_same(g, q)


def test_timed_steps_evaluate_their_forces():
    atoms, topo, state, _ = synth.generate(3000, seed=79, temperature=300.0, relax_iters=300)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **OPEN)
    out = []
    for form in (backend.STEP_GRAPH, backend.STEP_PERSISTENT):
        be = backend.CudaBackend(atoms, topo, p)
        be.step_form(form)
        be.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
        be.forces_resident()
        ms = be.time_steps(DT, 40)
        assert ms > 0.0
        pos = np.zeros_like(state.pos)
        vel = np.zeros_like(state.vel)
        be.download_state(pos, vel)
        f = be.compute_forces(pos).copy()  # the resident forces at the final positions
        out.append((pos, vel, f))
        be.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(bits(a), bits(b))


@pytest.mark.parametrize("case", ["fp64", "constrained"])
def test_refused_where_it_does_not_apply(case):
    atoms, topo, state, _ = synth.generate(800, seed=80, h_fraction=0.3 if case == "constrained" else 0.0,
                                           relax_iters=100)
    if case == "constrained":
        topo = amber.promote_hydrogen_bonds(topo, atoms)
    prec = backend.PRECISION_FP64 if case == "fp64" else backend.PRECISION_MIXED
    be = backend.CudaBackend(atoms, topo, backend.SimParams(precision=prec, **OPEN))
    with pytest.raises(backend.BackendError) as e:
        be.step_form(backend.STEP_PERSISTENT)
    assert e.value.status == 8  # GM_ERR_UNSUPPORTED
    be.step_form(backend.STEP_GRAPH)
    be.close()


@pytest.mark.parametrize("batch", [False, True])
def test_force_phase_matches_force_kernels(batch):
    if batch:
        syss = [synth.generate(n, seed=s_, relax_iters=200) for n, s_ in ((800, 91), (2600, 92), (1400, 93))]
        atoms, topo = [x[0] for x in syss], [x[1] for x in syss]
        pos = np.ascontiguousarray(np.concatenate([x[2].pos for x in syss], axis=1))
    else:
        atoms, topo, state, _ = synth.generate(4000, seed=94, relax_iters=300)
        pos = np.ascontiguousarray(state.pos)
    p = backend.SimParams(precision=backend.PRECISION_MIXED, **OPEN)
    out = []
    for form in (backend.STEP_GRAPH, backend.STEP_PERSISTENT):
        be = backend.CudaBackend.ensemble(atoms, topo, p) if batch else backend.CudaBackend(atoms, topo, p)
        be.step_form(form)
        q = pos.copy()
        be.build_neighbor_list(q)
        f = be.compute_forces(q).copy()
        e = be.potential_energy()
        sys_e = be.ensemble_energies()[0].copy() if batch else None
        out.append((f, e, sys_e))
        be.close()
    assert np.array_equal(bits(out[0][0]), bits(out[1][0]))
    assert out[0][1] == out[1][1]
    if batch:
        assert np.array_equal(bits(out[0][2]), bits(out[1][2]))
