"""Batches of independent systems in one context (gm_create_ensemble) against
the same systems run one by one (needs a GPU).

A system's grid, sorted order, list order and summation chunks in a batch are
the ones it gets alone, and the batch rebuilds a system's list exactly when
that system needs it, so without constraints the batch reproduces each
system's own run bit for bit:
* pair lists and forces: identical bits;
* per-system potential energies: int64 sums at 2^-32 kcal/mol against the
  single run's FP64 sum, relative 1e-9;
* 100 resident BAB steps: identical positions and velocities, and the same
  number of list rebuilds as the single runs together.
With constraints the batch's SHAKE/RATTLE stop at the batch's largest
iteration count; every solve still meets the tolerance.

Against the oracle (the reference's one-system run, geodesic/src/lib.rs:
187-345, restated): each member's forces (1e-10 * max(|F|, 1) per component
in FP64, 1e-5 mixed) and its positions after 20 resident steps, within
1e-9 A (FP64) or 1e-5 A (mixed).  With constraints a member iterates SHAKE /
RATTLE to the batch's largest count where the oracle stops at its own
(geodesic-engine/src/constraint.rs:62-152, 170-259): the extra iterations
move atoms by less than the 1e-10 tolerance each step, so the FP64 bound is
1e-8 A there.
"""
import numpy as np
import pytest

import oracle
from geodesic_cuda import amber, backend, synth

pytestmark = pytest.mark.gpu

PHYS = dict(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0, coulomb=True,
            scale14_lj=0.5, scale14_coul=1 / 1.2)
SIZES = ((700, 51), (1500, 52), (3100, 53))


def systems(h_fraction=0.0):
    out = []
    for n, seed in SIZES:
        atoms, topo, state, _ = synth.generate(n, seed=seed, h_fraction=h_fraction, relax_iters=400)
        if h_fraction:
            topo = amber.promote_hydrogen_bonds(topo, atoms)
        out.append((atoms, topo, state))
    return out


def concat(arrs):
    return np.ascontiguousarray(np.concatenate(arrs, axis=1))


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_batch_forces_pairs_and_energies_equal_single_runs(precision):
    syss = systems()
    p = backend.SimParams(precision=precision, **PHYS)
    batch = backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p)
    assert batch.n_sys == 3 and batch.n == sum(n for n, _ in SIZES)
    pos = concat([s[2].pos for s in syss])
    batch.build_neighbor_list(pos)
    f_batch = batch.compute_forces(pos).copy()
    e_pot, _ = batch.ensemble_energies()
    bi, bj = batch.pairs()
    off = batch.offsets
    for k, (atoms, topo, state) in enumerate(syss):
        one = backend.CudaBackend(atoms, topo, p)
        pk = np.ascontiguousarray(state.pos.copy())
        one.build_neighbor_list(pk)
        f_one = one.compute_forces(pk)
        assert np.array_equal(f_batch[:, off[k]:off[k + 1]], f_one), k
        e_one = one.potential_energy()
        assert abs(e_pot[k] - e_one) <= 1e-9 * abs(e_one), (k, e_pot[k], e_one)
        oi, oj = one.pairs()
        sel = (bi >= off[k]) & (bi < off[k + 1])
        assert np.array_equal(bi[sel] - off[k], oi) and np.array_equal(bj[sel] - off[k], oj), k
        one.close()
    # no pair crosses systems
    assert np.array_equal(np.searchsorted(off, bi, side="right"), np.searchsorted(off, bj, side="right"))


def test_batch_trajectory_equals_single_runs():
    syss = systems()
    p = backend.SimParams(**PHYS)
    batch = backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p)
    pos, vel = concat([s[2].pos for s in syss]), concat([s[2].vel for s in syss])
    batch.upload_state(pos, vel)
    batch.forces_resident()
    batch.run_resident(0.002, 100)
    batch.synchronize()
    pb, vb = np.zeros_like(pos), np.zeros_like(vel)
    batch.download_state(pb, vb)
    rebuilds = 0
    for k, (atoms, topo, state) in enumerate(syss):
        one = backend.CudaBackend(atoms, topo, p)
        one.upload_state(np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel))
        one.forces_resident()
        one.run_resident(0.002, 100)
        one.synchronize()
        po, vo = np.zeros_like(state.pos), np.zeros_like(state.vel)
        one.download_state(po, vo)
        sl = slice(batch.offsets[k], batch.offsets[k + 1])
        assert np.array_equal(pb[:, sl], po), k
        assert np.array_equal(vb[:, sl], vo), k
        rebuilds += one.counters()["rebuilds"]
        one.close()
    assert batch.counters()["rebuilds"] == rebuilds


def test_batch_with_constraints_converges():
    syss = systems(h_fraction=0.4)
    p = backend.SimParams(max_constr_iter=200, constr_tol=1e-10, **PHYS)
    batch = backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p)
    pos, vel = concat([s[2].pos for s in syss]), concat([s[2].vel for s in syss])
    batch.upload_state(pos, vel)
    batch.forces_resident()
    batch.run_resident(0.004, 50)
    batch.synchronize()
    pb, vb = np.zeros_like(pos), np.zeros_like(vel)
    batch.download_state(pb, vb)
    for k, (atoms, topo, state) in enumerate(syss):
        sl = slice(batch.offsets[k], batch.offsets[k + 1])
        d = pb[:, sl][:, topo.constr_i] - pb[:, sl][:, topo.constr_j]
        assert np.max(np.abs((d * d).sum(0) - topo.constr_dsq)) < 1e-6
    assert batch.counters()["constrained_steps"] == 50


def test_autotuner_keeps_forces_bit_identical():
    """Every autotuner candidate computes the same sums: the forces after
    tuning equal the forces before, for a batch and for a single system."""
    syss = systems()
    p = backend.SimParams(**PHYS)
    for be in (backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p),
               backend.CudaBackend(*syss[2][:2], p)):
        pos = concat([s[2].pos for s in syss]) if be.n_sys > 1 else np.ascontiguousarray(syss[2][2].pos)
        be.build_neighbor_list(pos)
        f0 = be.compute_forces(pos).copy()
        choice = be.autotune(reps=2)
        assert 1 <= choice["split"] <= 16 and choice["warps_per_block"] in (2, 4, 8) and choice["grid"] >= 0
        f1 = be.compute_forces(pos).copy()
        assert np.array_equal(f0, f1)


def oracle_params(p: backend.SimParams):
    return oracle.make_params(box=p.box_size, periodic=p.periodic, r_cutoff=p.r_cutoff, r_skin=p.r_skin,
                              r_switch=p.r_switch, max_constr_iter=p.max_constr_iter, constr_tol=p.constr_tol,
                              n_threads=1, coulomb=p.coulomb, scale14_lj=p.scale14_lj, scale14_coul=p.scale14_coul)


@pytest.mark.parametrize("constrained", [False, True])
@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_batch_members_follow_the_oracle(precision, constrained):
    syss = systems(h_fraction=0.4 if constrained else 0.0)
    p = backend.SimParams(precision=precision, max_constr_iter=200, constr_tol=1e-10, **PHYS)
    op = oracle_params(p)
    fp64 = precision == backend.PRECISION_FP64
    batch = backend.CudaBackend.ensemble([s[0] for s in syss], [s[1] for s in syss], p)
    off = batch.offsets
    pos, vel = concat([s[2].pos for s in syss]), concat([s[2].vel for s in syss])
    # forces of every member at the starting positions
    pf = pos.copy()
    batch.build_neighbor_list(pf)
    f = batch.compute_forces(pf).copy()
    ftol = 1e-10 if fp64 else 1e-5
    for k, (atoms, topo, state) in enumerate(syss):
        ob = oracle.CpuBackend(atoms, topo, op)
        pr = np.ascontiguousarray(state.pos.copy())
        ob.build_neighbor_list(pr)
        fr = ob.compute_forces(pr)
        fk = f[:, off[k]:off[k + 1]]
        assert np.all(np.abs(fk - fr) <= ftol * np.maximum(np.abs(fr), 1.0)), (k, np.abs(fk - fr).max())
    # 20 resident steps at 2 fs after the run loop's initial velocity
    # projection (lib.rs:270-282), against oracle.run per member
    batch.constrain_velocities(pos, vel, 0)
    batch.upload_state(pos, vel)
    batch.forces_resident()
    batch.run_resident(0.002, 20)
    batch.synchronize()
    pb, vb = np.zeros_like(pos), np.zeros_like(vel)
    batch.download_state(pb, vb)
    tol = (1e-8 if constrained else 1e-9) if fp64 else 1e-5
    for k, (atoms, topo, state) in enumerate(syss):
        po, vo = np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.vel.copy())
        oracle.run(atoms, topo, op, po, vo, 0.002, 20, 20)
        err = np.abs(pb[:, off[k]:off[k + 1]] - po).max()
        assert err < tol, (k, err)
    batch.close()
