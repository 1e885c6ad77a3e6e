"""CUDA backend vs the oracle, through the C ABI (needs a GPU).

Tolerances (stated per test):
* pair sets: bit-exact as sets (the reference's FP64 list test);
* FP64 path forces: |dF| <= 1e-10 * max(|F|, 1) per component, energy
  relative 1e-10;
* mixed path: |dF| <= 1e-5 * max(|F|, 1) per component (the form of the
  reference's FP32 kernel test, geodesic-gpu/tests/forces_gpu_vs_cpu.rs:7-34,
  at a tenth of its 1e-4) and ||dF|| / ||F|| <= 1e-5, energy relative 1e-5;
* integrator, SHAKE and RATTLE with given forces: bit-exact;
* reruns: bit-identical.
"""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from geodesic_cuda import amber, backend, synth

pytestmark = pytest.mark.gpu

FIX = dict(box_size=(100.0,) * 3, periodic=True, r_cutoff=12.0, r_skin=14.0, r_switch=10.0)


def oparams(p: backend.SimParams, n_threads=1):
    return oracle.make_params(box=p.box_size, periodic=p.periodic, r_cutoff=p.r_cutoff, r_skin=p.r_skin,
                              r_switch=p.r_switch, max_constr_iter=p.max_constr_iter, constr_tol=p.constr_tol,
                              n_threads=n_threads, coulomb=p.coulomb, scale14_lj=p.scale14_lj,
                              scale14_coul=p.scale14_coul)


def both(atoms, topo, pos, p: backend.SimParams):
    """Builds the list and evaluates forces on both; returns (gpu, ref) dicts."""
    be = backend.CudaBackend(atoms, topo, p)
    ob = oracle.CpuBackend(atoms, topo, oparams(p))
    pg, pr = np.ascontiguousarray(pos.copy()), np.ascontiguousarray(pos.copy())
    be.build_neighbor_list(pg)
    ob.build_neighbor_list(pr)
    fg = be.compute_forces(pg).copy()
    fr = ob.compute_forces(pr)
    out = dict(be=be, pos_g=pg, pos_r=pr, f_g=fg, f_r=fr, e_g=be.potential_energy(), e_r=ob.potential_energy,
               pairs_g=be.pairs(), pairs_r=ob.pairs())
    return out


def assert_pairs_equal(r):
    (gi, gj), (ri, rj) = r["pairs_g"], r["pairs_r"]
    assert len(gi) == len(ri), (len(gi), len(ri))
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def nonbonded_only(topo):
    """The topology with its bonded terms removed but its exclusions kept, so
    compute_forces returns the nonbonded kernel's forces alone."""
    t = amber.BondedTopology.empty()
    t.excl_i, t.excl_j = topo.excl_i, topo.excl_j
    return t


@pytest.mark.parametrize("name", ["lj_pair", "water_box_4", "ala_dipeptide"])
@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_fixture_forces_match_oracle(name, precision, load_fixture):
    """geodesic-gpu/tests/forces_gpu_vs_cpu.rs:7-64 on the same fixtures and
    parameters (box 100 periodic, cutoff 12 / skin 14 / switch 10): full
    mixed-path forces within 1e-5 * max(|F|, 1) per component (the
    reference's FP32 kernel is held to 1e-4), the nonbonded kernel alone as
    well; the FP64 path within 1e-10 * max(|F|, 1)."""
    atoms, topo, state = load_fixture(name)
    p = backend.SimParams(precision=precision, **FIX)
    r = both(atoms, topo, state.pos, p)
    assert_pairs_equal(r)
    assert np.array_equal(r["pos_g"], r["pos_r"])  # wrapped identically
    fg, fr = r["f_g"], r["f_r"]
    if precision == backend.PRECISION_FP64:
        assert np.all(np.abs(fg - fr) <= 1e-10 * np.maximum(np.abs(fr), 1.0)), np.abs(fg - fr).max()
        assert abs(r["e_g"] - r["e_r"]) <= 1e-10 * max(abs(r["e_r"]), 1.0)
        return
    assert rel_l2(fg, fr) <= 1e-5
    assert np.all(np.abs(fg - fr) <= 1e-5 * np.maximum(np.abs(fr), 1.0)), np.abs(fg - fr).max()
    assert abs(r["e_g"] - r["e_r"]) <= 1e-5 * max(abs(r["e_r"]), 1.0)
    nb = both(atoms, nonbonded_only(topo), state.pos, p)
    assert np.all(np.abs(nb["f_g"] - nb["f_r"]) <= 1e-5 * np.maximum(np.abs(nb["f_r"]), 1.0))


def test_lj_pair_pin():
    """lj_pair: sigma 2, epsilon 1 at r = 3 (prmtop_roundtrip.rs:13-17): the
    FP64 path gives the closed-form LJ force."""
    atoms, topo, state, _ = amber.load_npz(os.path.join(GOLDEN, "lj_pair.npz"))
    p = backend.SimParams(precision=backend.PRECISION_FP64, box_size=(1000.0,) * 3, periodic=False,
                          r_cutoff=12.0, r_skin=14.0, r_switch=10.0)
    be = backend.CudaBackend(atoms, topo, p)
    pos = np.ascontiguousarray(state.pos)
    be.build_neighbor_list(pos)
    f = be.compute_forces(pos)
    sr6 = (2.0 / 3.0) ** 6
    f_lj = 24.0 / 3.0 * (2 * sr6 * sr6 - sr6)
    assert abs(f[0, 1] - f_lj) < 1e-12 and abs(f[0, 0] + f_lj) < 1e-12
    assert abs(be.potential_energy() - 4.0 * (sr6 * sr6 - sr6)) < 1e-12


def test_neighbor_list_semantics():
    """geodesic-engine/tests/neighbor_list.rs:48-109 on the device."""
    class A:
        pass
    a = A()
    a.sigma = a.epsilon = a.charge = np.zeros(3)
    a.mass = np.ones(3)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=True, r_cutoff=5.0, r_skin=6.0, r_switch=4.0)
    be = backend.CudaBackend(a, amber.BondedTopology.empty(), p)
    pos = np.ascontiguousarray([[0.0, 3.0, 20.0], [0.0] * 3, [0.0] * 3])
    be.build_neighbor_list(pos)
    pi, pj = be.pairs()
    assert list(pi) == [0] and list(pj) == [1]
    # exclusion filtering
    a2 = A()
    a2.sigma = a2.epsilon = a2.charge = np.zeros(2)
    a2.mass = np.ones(2)
    t = amber.BondedTopology.empty()
    t.excl_i, t.excl_j = np.array([0], np.uint32), np.array([1], np.uint32)
    be2 = backend.CudaBackend(a2, t, p)
    pos2 = np.ascontiguousarray([[0.0, 1.0], [0.0, 0.0], [0.0, 0.0]])
    be2.build_neighbor_list(pos2)
    assert len(be2.pairs()[0]) == 0
    # min-image across the boundary and wrapping
    p10 = backend.SimParams(box_size=(10.0,) * 3, periodic=True, r_cutoff=5.0, r_skin=6.0, r_switch=4.0)
    be3 = backend.CudaBackend(a2, amber.BondedTopology.empty(), p10)
    pos3 = np.ascontiguousarray([[0.5, 9.5], [0.0, 0.0], [0.0, 0.0]])
    be3.build_neighbor_list(pos3)
    pi, pj = be3.pairs()
    assert list(pi) == [0] and list(pj) == [1]
    pos4 = np.ascontiguousarray([[-1.0, 0.5], [11.0, 0.0], [0.0, 0.0]])
    be3.build_neighbor_list(pos4)
    assert abs(pos4[0, 0] - 9.0) < 1e-12 and abs(pos4[1, 0] - 1.0) < 1e-12
    # half-skin rebuild trigger
    a1 = A()
    a1.sigma = a1.epsilon = a1.charge = np.zeros(1)
    a1.mass = np.ones(1)
    be4 = backend.CudaBackend(a1, amber.BondedTopology.empty(), backend.SimParams(
        box_size=(1000.0,) * 3, periodic=True, r_cutoff=5.0, r_skin=6.0, r_switch=4.0))
    z = np.ascontiguousarray(np.zeros((3, 1)))
    be4.build_neighbor_list(z)
    assert not be4.needs_rebuild(np.ascontiguousarray([[0.4], [0.0], [0.0]]))
    assert be4.needs_rebuild(np.ascontiguousarray([[0.6], [0.0], [0.0]]))


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_synthetic_5k_matches_oracle(precision):
    """Seeded 5,000-atom lattice system (cutoff 10 / switch 8 / list radius
    12, non-periodic, 1000 A box): pair set exact, forces and energy within
    the path's tolerance."""
    atoms, topo, state, _ = synth.generate(5000, seed=101)
    p = backend.SimParams(precision=precision, box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0,
                          r_switch=8.0)
    r = both(atoms, topo, state.pos, p)
    assert_pairs_equal(r)
    err = rel_l2(r["f_g"], r["f_r"])
    erel = abs(r["e_g"] - r["e_r"]) / abs(r["e_r"])
    if precision == backend.PRECISION_FP64:
        assert np.all(np.abs(r["f_g"] - r["f_r"]) <= 1e-10 * np.maximum(np.abs(r["f_r"]), 1.0))
        assert erel <= 1e-10
    else:
        assert err <= 1e-5, err
        assert np.all(np.abs(r["f_g"] - r["f_r"]) <= 1e-5 * np.maximum(np.abs(r["f_r"]), 1.0))
        assert erel <= 1e-5, erel


def test_synthetic_coulomb_and_14():
    """Beyond the reference: Coulomb with the LJ switch and scaled 1-4 pairs
    (LJ x 1/2.0, Coulomb x 1/1.2), against the oracle's formulas."""
    atoms, topo, state, _ = synth.generate(3000, seed=7)
    for precision, tol in ((backend.PRECISION_FP64, 1e-10), (backend.PRECISION_MIXED, 1e-5)):
        p = backend.SimParams(precision=precision, box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0,
                              r_skin=12.0, r_switch=8.0, coulomb=True, scale14_lj=0.5, scale14_coul=1 / 1.2)
        r = both(atoms, topo, state.pos, p)
        assert_pairs_equal(r)
        assert rel_l2(r["f_g"], r["f_r"]) <= tol
        assert np.all(np.abs(r["f_g"] - r["f_r"]) <= tol * np.maximum(np.abs(r["f_r"]), 1.0))
        assert abs(r["e_g"] - r["e_r"]) <= tol * abs(r["e_r"])


def test_forces_bit_identical_reruns():
    """gpu_determinism.rs:7-21: repeated evaluations give identical bits (also
    across fresh contexts, whose atomics run in a different order)."""
    atoms, topo, state, _ = synth.generate(4000, seed=3)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)
    outs = []
    for _ in range(3):
        be = backend.CudaBackend(atoms, topo, p)
        pos = np.ascontiguousarray(state.pos.copy())
        be.build_neighbor_list(pos)
        f1 = be.compute_forces(pos).copy()
        f2 = be.compute_forces(pos).copy()
        assert np.array_equal(f1.view(np.uint64), f2.view(np.uint64))
        outs.append((f1, be.potential_energy()))
        be.close()
    for f, e in outs[1:]:
        assert np.array_equal(f.view(np.uint64), outs[0][0].view(np.uint64)) and e == outs[0][1]


def dimer():
    t = amber.BondedTopology.empty()
    t.constr_i, t.constr_j, t.constr_dsq = np.array([0], np.uint32), np.array([1], np.uint32), np.array([1.0])
    a = amber.AtomData(np.zeros(2), np.zeros(2), np.array([1.008, 12.0]), np.zeros(2),
                       np.array([0, 1], np.uint8), np.zeros(2, np.uint32), ["H1  ", "C1  "])
    return a, t


def test_integrator_bit_exact(load_fixture):
    """half_kick, drift + SHAKE + resync and RATTLE on ala_dipeptide with its
    H bonds constrained: the device returns the oracle's exact bits."""
    atoms, topo, state = load_fixture("ala_dipeptide")
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=False, constr_tol=1e-10, max_constr_iter=100)
    be = backend.CudaBackend(atoms, topo, p)
    rng = np.random.default_rng(0)
    vel = np.ascontiguousarray(rng.normal(0, 5.0, (3, atoms.n)))
    force = np.ascontiguousarray(rng.normal(0, 50.0, (3, atoms.n)))
    vg, vr = vel.copy(), vel.copy()
    be.half_kick(vg, force, 0.001)
    oracle.half_kick(vr, force, atoms.mass, 0.001)
    assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64))
    pg, pr = np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.pos.copy())
    be.geodesic_drift(pg, vg, 0.002, step=3)
    oracle.drift_and_constrain(pr, vr, topo, atoms, 0.002, 100, 1e-10, 3)
    assert np.array_equal(pg.view(np.uint64), pr.view(np.uint64))
    assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64))
    be.half_kick(vg, force, 0.001)
    oracle.half_kick(vr, force, atoms.mass, 0.001)
    be.constrain_velocities(pg, vg, step=3)
    oracle.constrain_velocities(topo, atoms, pr, vr, 100, 1e-10, 3)
    assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64))


def test_integrator_bit_exact_mixed_cluster_sizes():
    """SHAKE/RATTLE with single-constraint clusters (one thread each),
    H-star clusters and a 12-bond chain (one warp each) and a 40-bond chain
    (more than 32 constraints: one thread, global memory) in the same system:
    every cluster returns the oracle's exact bits, for 5 steps."""
    atoms, topo, state, _ = synth.generate(400, seed=17, h_fraction=0.3, relax_iters=200)
    t = amber.promote_hydrogen_bonds(topo, atoms)
    # constrain two runs of consecutive chain bonds as well
    heavy = np.flatnonzero(atoms.element != 0)
    chain = [(int(a), int(b)) for a, b in zip(t.bond_i, t.bond_j)]
    runs = set(range(5, 17)) | set(range(40, 80))
    sel = [chain[k] for k in sorted(runs)]
    keep = [k for k in range(len(t.bond_i)) if k not in runs]
    ci = np.concatenate([t.constr_i, np.array([a for a, b in sel], np.uint32)])
    cj = np.concatenate([t.constr_j, np.array([b for a, b in sel], np.uint32)])
    d = state.pos[:, ci] - state.pos[:, cj]
    t.constr_i, t.constr_j, t.constr_dsq = ci, cj, (d * d).sum(0)
    t.bond_i, t.bond_j, t.bond_k, t.bond_r0 = t.bond_i[keep], t.bond_j[keep], t.bond_k[keep], t.bond_r0[keep]
    assert len(heavy) > 80
    # Jacobi converges slowly on the long chain: tolerance 1e-8 within 2000
    # iterations (the oracle needs ~130-195; at 1e-10 / 200 both stop with
    # the same ConvergenceError)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=False, constr_tol=1e-8, max_constr_iter=2000)
    be = backend.CudaBackend(atoms, t, p)
    rng = np.random.default_rng(1)
    pg, pr = np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.pos.copy())
    vg = np.ascontiguousarray(rng.normal(0, 2.0, (3, atoms.n)))
    vr = vg.copy()
    force = np.ascontiguousarray(rng.normal(0, 20.0, (3, atoms.n)))
    for step in range(5):
        be.half_kick(vg, force, 0.001)
        oracle.half_kick(vr, force, atoms.mass, 0.001)
        be.geodesic_drift(pg, vg, 0.002, step=step)
        oracle.drift_and_constrain(pr, vr, t, atoms, 0.002, 2000, 1e-8, step)
        assert np.array_equal(pg.view(np.uint64), pr.view(np.uint64)), step
        be.half_kick(vg, force, 0.001)
        oracle.half_kick(vr, force, atoms.mass, 0.001)
        be.constrain_velocities(pg, vg, step=step)
        oracle.constrain_velocities(t, atoms, pr, vr, 2000, 1e-8, step)
        assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64)), step


def test_constraint_failure_reports_reference_error():
    """constraint_solver.rs:98-120: max_iter = 1 gives ConvergenceError with
    the step and the worst constraint's atoms."""
    a, t = dimer()
    p = backend.SimParams(box_size=(1000.0,) * 3, max_constr_iter=1, constr_tol=1e-10)
    be = backend.CudaBackend(a, t, p)
    pos = np.ascontiguousarray([[0.0, 1.05], [0.0, 0.0], [0.0, 0.0]])
    vel = np.ascontiguousarray(np.zeros((3, 2)))
    # drift with zero velocity keeps the stretched trial positions; the
    # reference vector comes from the same positions
    with pytest.raises(backend.ConvergenceError) as e:
        be.geodesic_drift(pos, vel, 0.1, step=7)
    assert e.value.step == 7 and e.value.max_iter == 1 and (e.value.atom_i, e.value.atom_j) == (0, 1)


def test_nonfinite_position_is_an_error():
    atoms, topo, state, _ = synth.generate(500, seed=1)
    be = backend.CudaBackend(atoms, topo, backend.SimParams(box_size=(1000.0,) * 3, r_cutoff=10.0, r_skin=12.0,
                                                            r_switch=8.0))
    pos = np.ascontiguousarray(state.pos.copy())
    pos[0, 5] = np.nan
    with pytest.raises(backend.NumericalError):
        be.build_neighbor_list(pos)


def test_golden_trajectory_fp64_path(load_fixture):
    """geodesic/tests/golden_reference.rs:27-94 run on the FP64 device path:
    99 BAB steps (1 fs, tolerance 1e-8, H bonds constrained) driven through
    the trait-level entry points like lib.rs:261-333; every float32 frame
    coordinate within 4 ulp of the reference's golden DCD (the device sums
    forces in another order than the reference's single thread)."""
    atoms, topo, state = load_fixture("ala_dipeptide")
    golden = np.load(os.path.join(GOLDEN, "ala_dipeptide_ref_frames.npy"))
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = backend.SimParams(precision=backend.PRECISION_FP64, box_size=(1000.0,) * 3, periodic=False, r_cutoff=12.0,
                          r_skin=14.0, r_switch=10.0, max_constr_iter=100, constr_tol=1e-8)
    be = backend.CudaBackend(atoms, topo, p)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    dt = 0.001
    be.build_neighbor_list(pos)
    f = be.compute_forces(pos).copy()
    be.constrain_velocities(pos, vel, 0)
    frames = [pos.astype(np.float32)]
    for step in range(99):
        be.half_kick(vel, f, dt / 2.0)
        be.geodesic_drift(pos, vel, dt, step)
        if be.needs_rebuild(pos):
            be.build_neighbor_list(pos)
        f = be.compute_forces(pos).copy()
        be.half_kick(vel, f, dt / 2.0)
        be.constrain_velocities(pos, vel, step)
        frames.append(pos.astype(np.float32))
    frames = np.stack(frames)
    ulp = np.abs(frames.view(np.int32).astype(np.int64) - golden.view(np.int32).astype(np.int64))
    assert ulp.max() <= 4, ulp.max()


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_resident_steps_follow_oracle(precision, load_fixture):
    """Device-resident BAB loop (CUDA graph) vs the oracle's run loop on
    ala_dipeptide over 20 steps of 1 fs: positions agree within 1e-9 A (FP64)
    or 1e-5 A (mixed)."""
    atoms, topo, state = load_fixture("ala_dipeptide")
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = backend.SimParams(precision=precision, box_size=(1000.0,) * 3, periodic=False, r_cutoff=12.0, r_skin=14.0,
                          r_switch=10.0, max_constr_iter=100, constr_tol=1e-8)
    be = backend.CudaBackend(atoms, topo, p)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    # the run loop's initial velocity projection (lib.rs:270-282) happens before the loop
    be.constrain_velocities(pos, vel, 0)
    be.steps(pos, vel, 0.001, 20)
    po, vo = np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.vel.copy())
    frames, _, _ = oracle.run(atoms, topo, oparams(p), po, vo, 0.001, 20, 20)
    tol = 1e-9 if precision == backend.PRECISION_FP64 else 1e-5
    assert np.abs(pos - po).max() < tol, np.abs(pos - po).max()


def test_resident_runs_bit_identical():
    """Three runs of the device-resident loop from the same seeded state
    (with list rebuilds) end in bit-identical states."""
    atoms, topo, state, _ = synth.generate(3000, seed=17)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)
    res = []
    for _ in range(3):
        be = backend.CudaBackend(atoms, topo, p)
        pos = np.ascontiguousarray(state.pos.copy())
        vel = np.ascontiguousarray(state.vel.copy())
        e, nreb, _ = be.steps(pos, vel, 0.002, 200)
        res.append((pos, vel, e, nreb))
        be.close()
    for pos, vel, e, nreb in res[1:]:
        assert np.array_equal(pos.view(np.uint64), res[0][0].view(np.uint64))
        assert np.array_equal(vel.view(np.uint64), res[0][1].view(np.uint64))
        assert e == res[0][2] and nreb == res[0][3]


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_resident_unconstrained_steps_equal_trait_loop(precision):
    """Without constraints the resident step folds each step's closing
    half-kick into the next step's first kernel (two additions with the same
    forces, in the same order) and finishes the last one after the loop.
    The result must equal, bit for bit, the loop of lib.rs:292-323 driven
    through the trait-level entry points, list rebuilds included."""
    atoms, topo, state, _ = synth.generate(2000, seed=23, temperature=600.0, relax_iters=200)
    p = backend.SimParams(precision=precision, box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0,
                          r_skin=10.6, r_switch=8.0)
    dt, n = 0.002, 60
    res = backend.CudaBackend(atoms, topo, p)
    pr = np.ascontiguousarray(state.pos.copy())
    vr = np.ascontiguousarray(state.vel.copy())
    _, n_reb, _ = res.steps(pr, vr, dt, n)
    assert n_reb >= 2, n_reb  # the comparison covers rebuilds inside the graph
    res.close()
    be = backend.CudaBackend(atoms, topo, p)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    be.build_neighbor_list(pos)
    f = be.compute_forces(pos).copy()
    for step in range(n):
        be.half_kick(vel, f, dt / 2.0)
        be.geodesic_drift(pos, vel, dt, step)
        if be.needs_rebuild(pos):
            be.build_neighbor_list(pos)
        f = be.compute_forces(pos).copy()
        be.half_kick(vel, f, dt / 2.0)
    be.close()
    assert np.array_equal(pr.view(np.uint64), pos.view(np.uint64))
    assert np.array_equal(vr.view(np.uint64), vel.view(np.uint64))
