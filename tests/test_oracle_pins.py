"""Pins the oracle to the reference's own tests and golden data (CPU only).

Each test restates one reference test with the same inputs and tolerances;
the reference file:line is given in the docstring.  A green run means the
oracle reproduces the reference's behaviour wherever the reference pins it.
"""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN
from geodesic_cuda import amber


class Atoms:
    def __init__(self, sigma, epsilon, mass, charge=None, element=None):
        n = len(mass)
        self.sigma = np.asarray(sigma, float)
        self.epsilon = np.asarray(epsilon, float)
        self.mass = np.asarray(mass, float)
        self.charge = np.zeros(n) if charge is None else np.asarray(charge, float)
        self.element = np.full(n, amber.ELEMENT_C, np.uint8) if element is None else np.asarray(element, np.uint8)


def pos3(x, y=None, z=None):
    n = len(x)
    return np.ascontiguousarray(np.array([x, y if y is not None else [0.0] * n, z if z is not None else [0.0] * n],
                                         dtype=np.float64))


# --------------------------------------------------------------- neighbour

def nb_params(box):
    """geodesic-engine/tests/neighbor_list.rs:30-46"""
    return oracle.make_params(box=box, periodic=True, r_cutoff=5.0, r_skin=6.0, r_switch=4.0)


@pytest.mark.parametrize("cells", [False, True])
def test_finds_pairs_within_skin(cells):
    """neighbor_list.rs:48-58"""
    pos = pos3([0.0, 3.0, 20.0])
    pi, pj = oracle.neighbor_build(pos, Atoms([0] * 3, [0] * 3, [1] * 3), amber.BondedTopology.empty(),
                                   nb_params((1000.0,) * 3), cells=cells)
    assert list(pi) == [0] and list(pj) == [1]


@pytest.mark.parametrize("cells", [False, True])
def test_bonded_exclusions_filtered(cells):
    """neighbor_list.rs:60-71"""
    t = amber.BondedTopology.empty()
    t.excl_i, t.excl_j = np.array([0], np.uint32), np.array([1], np.uint32)
    pi, _ = oracle.neighbor_build(pos3([0.0, 1.0]), Atoms([0] * 2, [0] * 2, [1] * 2), t, nb_params((1000.0,) * 3),
                                  cells=cells)
    assert len(pi) == 0


@pytest.mark.parametrize("cells", [False, True])
def test_min_image_across_boundary(cells):
    """neighbor_list.rs:73-84"""
    pi, pj = oracle.neighbor_build(pos3([0.5, 9.5]), Atoms([0] * 2, [0] * 2, [1] * 2), amber.BondedTopology.empty(),
                                   nb_params((10.0,) * 3), cells=cells)
    assert list(pi) == [0] and list(pj) == [1]


def test_positions_wrapped_into_box():
    """neighbor_list.rs:86-96"""
    pos = pos3([-1.0], [11.0])
    oracle.neighbor_build(pos, Atoms([0], [0], [1]), amber.BondedTopology.empty(), nb_params((10.0,) * 3))
    assert abs(pos[0, 0] - 9.0) < 1e-12 and abs(pos[1, 0] - 1.0) < 1e-12


def test_rebuild_past_half_skin():
    """neighbor_list.rs:98-109"""
    ref = pos3([0.0])
    assert not oracle.needs_rebuild(pos3([0.4]), ref, 6.0, 5.0)
    assert oracle.needs_rebuild(pos3([0.6]), ref, 6.0, 5.0)


def test_cell_build_equals_double_loop():
    """The cell-grid checker path returns the reference's exact pair list."""
    rng = np.random.default_rng(7)
    n = 700
    pos = np.ascontiguousarray(rng.uniform(0, 30, (3, n)))
    t = amber.BondedTopology.empty()
    ii = rng.integers(0, n, 300).astype(np.uint32)
    jj = rng.integers(0, n, 300).astype(np.uint32)
    t.excl_i, t.excl_j = ii, jj
    a = Atoms(np.zeros(n), np.zeros(n), np.ones(n))
    for periodic, box in ((False, 1000.0), (True, 30.0)):
        p = oracle.make_params(box=(box,) * 3, periodic=periodic, r_cutoff=5.0, r_skin=6.0, r_switch=4.0)
        a1 = oracle.neighbor_build(pos.copy(), a, t, p)
        a2 = oracle.neighbor_build(pos.copy(), a, t, p, cells=True)
        assert np.array_equal(a1[0], a2[0]) and np.array_equal(a1[1], a2[1])


# ----------------------------------------------------------- nonbonded

def two_atoms(r):
    return pos3([0.0, r]), Atoms([2.0, 2.0], [1.0, 1.0], [1.0, 1.0])


def lj_potential(r, rc, rs):
    pos, a = two_atoms(r)
    e, _ = oracle.pair_forces(pos, a, [0], [1], rc, rs)
    return e


def lj_fx1(r, rc, rs):
    pos, a = two_atoms(r)
    _, f = oracle.pair_forces(pos, a, [0], [1], rc, rs)
    return f[0, 1]


@pytest.mark.parametrize("r", [2.5, 3.0, 10.5, 11.5])
def test_lj_gradient_matches_fd(r):
    """nonbonded_gradient.rs:173-197"""
    eps = 1e-6
    numeric = -(lj_potential(r + eps, 12.0, 10.0) - lj_potential(r - eps, 12.0, 10.0)) / (2 * eps)
    analytic = lj_fx1(r, 12.0, 10.0)
    assert abs(analytic - numeric) / (abs(numeric) + 1.0) < 1e-5


def test_switch_continuity():
    """nonbonded_gradient.rs:199-210"""
    assert abs(lj_potential(10.0 - 1e-7, 12.0, 10.0) - lj_potential(10.0 + 1e-7, 12.0, 10.0)) < 1e-4
    assert abs(lj_potential(12.0 - 1e-6, 12.0, 10.0)) < 1e-3


def test_repulsion_and_newton():
    """nonbonded_gradient.rs:212-232"""
    assert lj_fx1(1.5, 12.0, 10.0) > 0.0
    pos, a = two_atoms(3.0)
    _, f = oracle.pair_forces(pos, a, [0], [1], 12.0, 10.0)
    assert abs(f[0, 0] + f[0, 1]) < 1e-12


# --------------------------------------------------------------- bonded

def fd_check(pos, kind, topo, tol=1e-4):
    """bonded_gradient.rs:264-300 (central difference, eps 1e-6, rel < 1e-4)."""
    _, f = oracle.bonded_forces(kind, pos, topo)
    eps = 1e-6
    for i in range(pos.shape[1]):
        for ax in range(3):
            p, m = pos.copy(), pos.copy()
            p[ax, i] += eps
            m[ax, i] -= eps
            num = -(oracle.bonded_forces(kind, p, topo)[0] - oracle.bonded_forces(kind, m, topo)[0]) / (2 * eps)
            assert abs(f[ax, i] - num) / (abs(num) + 1.0) < tol, (kind, i, ax, f[ax, i], num)
    return f


def test_bond_gradient():
    """bonded_gradient.rs:314-329"""
    t = amber.BondedTopology.empty()
    t.bond_i, t.bond_j = np.array([0], np.uint32), np.array([1], np.uint32)
    t.bond_k, t.bond_r0 = np.array([300.0]), np.array([1.5])
    fd_check(pos3([0.0, 1.7]), "bond", t)


def test_angle_gradient():
    """bonded_gradient.rs:331-349"""
    t = amber.BondedTopology.empty()
    t.angle_i, t.angle_j, t.angle_k = (np.array([v], np.uint32) for v in (0, 1, 2))
    t.angle_kth, t.angle_th0 = np.array([50.0]), np.array([1.9106])
    fd_check(pos3([1.0, 0.0, 0.3], [0.0, 0.0, 1.0]), "angle", t)


def dihedral_topo(k, n, d):
    t = amber.BondedTopology.empty()
    t.dihed_i, t.dihed_j, t.dihed_k, t.dihed_l = (np.array([v], np.uint32) for v in (0, 1, 2, 3))
    t.dihed_kphi, t.dihed_n, t.dihed_delta = np.array([k]), np.array([n], np.uint32), np.array([d])
    return t


def test_dihedral_gradient_two_geometries():
    """bonded_gradient.rs:351-396"""
    fd_check(pos3([0.0, 0.0, 1.0, 1.5], [0.0, 1.0, 1.0, 2.0], [0.0, 0.0, 0.0, 0.7]), "dihedral",
             dihedral_topo(2.0, 2, 0.0))
    fd_check(pos3([0.3, -0.4, 0.9, 2.1], [-0.6, 0.5, 1.3, 0.8], [1.1, 0.2, -0.3, 1.4]), "dihedral",
             dihedral_topo(3.5, 3, 0.7))


def test_dihedral_forces_sum_to_zero():
    """bonded_gradient.rs:398-418"""
    _, f = oracle.bonded_forces("dihedral", pos3([0.0, 0.0, 1.0, 1.5], [0.0, 1.0, 1.0, 2.0], [0.0, 0.0, 0.0, 0.7]),
                                dihedral_topo(2.0, 2, 0.0))
    assert np.all(np.abs(f.sum(axis=1)) < 1e-10)


# ---------------------------------------------------------- constraints

def dimer():
    """constraint_solver.rs:32-50"""
    t = amber.BondedTopology.empty()
    t.constr_i, t.constr_j, t.constr_dsq = np.array([0], np.uint32), np.array([1], np.uint32), np.array([1.0])
    a = Atoms([0, 0], [0, 0], [1.008, 12.0], element=[amber.ELEMENT_H, amber.ELEMENT_C])
    return t, a


def test_constraint_converges_and_on_manifold():
    """constraint_solver.rs:52-96"""
    t, a = dimer()
    pos = pos3([0.0, 1.05])
    it = oracle.constraint_solve(t, a, pos3([0.0, 1.0]), pos, 50, 1e-10)
    assert 0 < it <= 50
    d = pos[:, 0] - pos[:, 1]
    assert abs(d @ d - 1.0) < 1e-8


def test_constraint_max_iter_one_errors():
    """constraint_solver.rs:98-120"""
    t, a = dimer()
    with pytest.raises(oracle.ConvergenceError) as e:
        oracle.constraint_solve(t, a, pos3([0.0, 1.0]), pos3([0.0, 1.05]), 1, 1e-10, step=7)
    assert e.value.step == 7 and e.value.max_iter == 1 and (e.value.atom_i, e.value.atom_j) == (0, 1)


def test_no_constraints_converges_immediately():
    """constraint_solver.rs:122-142"""
    assert oracle.constraint_solve(amber.BondedTopology.empty(), Atoms([0], [0], [1.0]), pos3([0.0]), pos3([0.0]),
                                   50, 1e-10) == 0


# ----------------------------------------------------------- integrator

def test_half_kick():
    """tests/integrator.rs:50-74"""
    vel = np.zeros((3, 2))
    f = np.array([[10.0, -4.0], [0.0, 2.0], [1.0, 0.0]])
    oracle.half_kick(vel, f, np.array([2.0, 4.0]), 0.5)
    c = 20.455 ** 2
    assert abs(vel[0, 0] - 10.0 * 0.5 / 2.0 * c) < 1e-11
    assert abs(vel[2, 0] - 1.0 * 0.5 / 2.0 * c) < 1e-11
    assert abs(vel[0, 1] - (-4.0) * 0.5 / 4.0 * c) < 1e-11
    assert abs(vel[1, 1] - 2.0 * 0.5 / 4.0 * c) < 1e-11


def test_free_drift_and_constrained_drift():
    """tests/integrator.rs:76-112"""
    pos, vel = pos3([1.0]), pos3([2.0])
    oracle.drift_and_constrain(pos, vel, amber.BondedTopology.empty(), Atoms([0], [0], [1.0]), 0.5, 10, 1e-10)
    assert abs(pos[0, 0] - 2.0) < 1e-14 and abs(vel[0, 0] - 2.0) < 1e-14
    t, a = dimer()
    pos, vel = pos3([0.0, 1.0]), pos3([-0.2, 0.2])
    oracle.drift_and_constrain(pos, vel, t, a, 0.1, 50, 1e-12)
    dx = pos[0, 0] - pos[0, 1]
    assert abs(dx * dx - 1.0) < 1e-9
    assert abs(vel[0, 0] - (pos[0, 0] - 0.0) / 0.1) < 1e-9


def test_free_rigid_rotor():
    """tests/integrator.rs:120-160 (2000 steps, KE drift < 1e-8, bond^2 error < 1e-8)."""
    t, a = dimer()
    pos = pos3([0.0, 1.0])
    vel = pos3([0.1, 0.1], [0.05 + 0.3, 0.05 - 0.3])
    ke = lambda v: float(sum(0.5 * a.mass[i] * (v[:, i] @ v[:, i]) for i in range(2)))  # noqa: E731
    ke0 = ke(vel)
    zero = np.zeros((3, 2))
    for step in range(2000):
        oracle.half_kick(vel, zero, a.mass, 0.002)
        oracle.drift_and_constrain(pos, vel, t, a, 0.004, 50, 1e-12, step)
        oracle.half_kick(vel, zero, a.mass, 0.002)
        oracle.constrain_velocities(t, a, pos, vel, 50, 1e-12, step)
    d = pos[:, 0] - pos[:, 1]
    assert abs(ke(vel) - ke0) < 1e-8 and abs(d @ d - 1.0) < 1e-8


@pytest.mark.slow
def test_harmonic_dimer_energy_conservation(load_fixture):
    """geodesic-engine/tests/energy_conservation.rs:12-77 (100k steps at 4 fs)."""
    atoms, topo, state = load_fixture("harmonic_dimer")
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    assert len(topo.constr_i) == 1 and len(topo.bond_i) == 0
    vel = np.ascontiguousarray([[-0.15, 0.15], [0.08, -0.02], [0.0, 0.0]])
    pos = np.ascontiguousarray(state.pos)
    p = oracle.make_params(box=(1000.0,) * 3, periodic=False, r_cutoff=12.0, r_skin=14.0, r_switch=10.0,
                           max_constr_iter=100, constr_tol=1e-10)
    frames, pot, kin = oracle.run(atoms, topo, p, pos, vel, 0.004, 100_000, frame_interval=100_000)
    e0, e1 = kin[0] + pot[0], kin[-1] + pot[-1]
    assert abs(e1 - e0) / abs(e0) < 1e-4
    d = pos[:, 0] - pos[:, 1]
    assert abs(d @ d - topo.constr_dsq[0]) < 1e-6


# ----------------------------------------------------------- CpuBackend

def lj_cluster():
    """geodesic-engine/tests/cpu_backend.rs:192-217"""
    coords = [(0.0, 0.0, 0.0), (3.0, 0.0, 0.0), (0.0, 3.0, 0.0), (3.0, 3.0, 0.0), (0.0, 0.0, 3.0), (3.0, 0.0, 3.0),
              (0.0, 3.0, 3.0), (3.0, 3.0, 3.0), (1.5, 1.5, 1.5), (4.5, 1.5, 1.5), (1.5, 4.5, 1.5), (1.5, 1.5, 4.5)]
    pos = np.ascontiguousarray(np.array(coords, float).T)
    return pos, Atoms([1.5] * 12, [0.2] * 12, [12.0] * 12)


def cluster_params(n_threads):
    """cpu_backend.rs:174-190"""
    return oracle.make_params(box=(100.0,) * 3, periodic=True, r_cutoff=8.0, r_skin=10.0, r_switch=6.0,
                              constr_tol=1e-10, n_threads=n_threads)


def test_backend_matches_direct_pair_call():
    """cpu_backend.rs:219-243"""
    pos, a = lj_cluster()
    p = cluster_params(1)
    b = oracle.CpuBackend(a, amber.BondedTopology.empty(), p)
    b.build_neighbor_list(pos)
    via = b.compute_forces(pos)
    pos2, _ = lj_cluster()
    pi, pj = oracle.neighbor_build(pos2, a, amber.BondedTopology.empty(), p)
    _, f = oracle.pair_forces(pos2, a, pi, pj, 8.0, 6.0, box=(100.0,) * 3)
    assert np.all(np.abs(via - f) < 1e-12)


def test_backend_repeatable_per_thread_count_and_close_across():
    """cpu_backend.rs:253-297"""
    res = {}
    for t in (1, 4):
        runs = []
        for _ in range(2):
            pos, a = lj_cluster()
            b = oracle.CpuBackend(a, amber.BondedTopology.empty(), cluster_params(t))
            b.build_neighbor_list(pos)
            assert b.n_threads() == t
            runs.append(b.compute_forces(pos))
        assert np.array_equal(runs[0].view(np.uint64), runs[1].view(np.uint64))
        res[t] = runs[0]
    assert np.all(np.abs(res[1] - res[4]) < 1e-10)


def test_backend_geodesic_drift_respects_bond():
    """cpu_backend.rs:316-344"""
    t, a = dimer()
    b = oracle.CpuBackend(a, t, cluster_params(1))
    pos, vel = pos3([0.0, 1.0]), pos3([-0.2, 0.2])
    b.geodesic_drift(pos, vel, 0.1)
    dx = pos[0, 0] - pos[0, 1]
    assert abs(dx * dx - 1.0) < 1e-9


# --------------------------------------------------- H-bond promotion

def test_promote_only_hydrogen_bonds():
    """hydrogen_constraint_promotion.rs:271-330 (host-side ingest logic)."""
    t = amber.BondedTopology.empty()
    t.bond_i = np.array([0, 0, 0, 0], np.uint32)
    t.bond_j = np.array([1, 2, 3, 4], np.uint32)
    t.bond_k = np.array([340.0, 340.0, 340.0, 400.0])
    t.bond_r0 = np.array([1.09, 1.09, 1.09, 1.47])
    H, Cc, N = amber.ELEMENT_H, amber.ELEMENT_C, amber.ELEMENT_N
    a = Atoms([0] * 5, [0] * 5, [12.0, 1.008, 1.008, 1.008, 14.0], element=[Cc, H, H, H, N])
    t2 = amber.promote_hydrogen_bonds(t, a)
    assert list(t2.constr_j) == [1, 2, 3] and np.all(np.abs(t2.constr_dsq - 1.09 ** 2) < 1e-12)
    assert list(t2.bond_i) == [0] and list(t2.bond_j) == [4] and list(t2.bond_k) == [400.0]
    a2 = Atoms([0] * 2, [0] * 2, [12.0, 14.0], element=[Cc, N])
    t3 = amber.BondedTopology.empty()
    t3.bond_i, t3.bond_j = np.array([0], np.uint32), np.array([1], np.uint32)
    t3.bond_k, t3.bond_r0 = np.array([400.0]), np.array([1.47])
    assert len(amber.promote_hydrogen_bonds(t3, a2).constr_i) == 0


def test_water_box_promotes_and_solves(load_fixture):
    """hydrogen_constraint_promotion.rs:336-376"""
    atoms, topo, state = load_fixture("water_box_4")
    assert len(topo.bond_i) == 8 and len(topo.angle_i) == 4
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    assert len(topo.constr_i) == 8 and len(topo.bond_i) == 0 and len(topo.angle_i) == 4
    ref = state.pos.copy()
    pos = np.ascontiguousarray(state.pos.copy())
    pos[0] += 0.01
    it = oracle.constraint_solve(topo, atoms, ref, pos, 100, 1e-10)
    assert 0 < it <= 100
    for n in range(8):
        d = pos[:, topo.constr_i[n]] - pos[:, topo.constr_j[n]]
        assert abs(d @ d - topo.constr_dsq[n]) < 1e-8


# ----------------------------------------------------- prmtop fixtures

def test_prmtop_pins(load_fixture):
    """geodesic-io/tests/prmtop_roundtrip.rs:3-109"""
    atoms, topo, state = load_fixture("lj_pair")
    assert list(atoms.mass) == [1.0, 2.0]
    assert np.all(np.abs(atoms.sigma - 2.0) < 1e-8) and np.all(np.abs(atoms.epsilon - 1.0) < 1e-8)
    assert len(topo.bond_i) == len(topo.angle_i) == len(topo.dihed_i) == len(topo.excl_i) == 0
    atoms, topo, state = load_fixture("ala_dipeptide")
    assert atoms.n == 22 and len(topo.bond_i) == 21
    assert abs(atoms.charge.sum()) < 1e-6
    assert atoms.residue_id[0] == 0 and atoms.residue_id[21] == 2 and atoms.element[0] == amber.ELEMENT_H
    assert abs(state.pos[0, 0] - 2.0000010) < 1e-6 and abs(state.pos[2, 0] + 0.0000013) < 1e-6


FIXTURE_PARAMS = dict(box=(100.0,) * 3, periodic=True, r_cutoff=12.0, r_skin=14.0, r_switch=10.0)


def total_force(pos, atoms, topo):
    """fixture_gradient_check.rs:468-495: bonded + LJ on a wrapped copy."""
    p = oracle.make_params(**FIXTURE_PARAMS)
    e = 0.0
    f = np.zeros(pos.shape)
    for kind in ("bond", "angle", "dihedral"):
        e += oracle.bonded_forces(kind, pos, topo, f)[0]
    w = np.ascontiguousarray(pos.copy())
    pi, pj = oracle.neighbor_build(w, atoms, topo, p)
    e += oracle.pair_forces(pos, atoms, pi, pj, 12.0, 10.0, box=(100.0,) * 3, force=f)[0]
    return e, f


@pytest.mark.parametrize("name", ["lj_pair", "harmonic_dimer", "water_box_4", "ala_dipeptide"])
def test_fixture_newton_and_fd(name, load_fixture):
    """newton_third_law.rs:34-82 and fixture_gradient_check.rs:497-561"""
    atoms, topo, state = load_fixture(name)
    pos = np.ascontiguousarray(state.pos)
    _, f = total_force(pos, atoms, topo)
    n = pos.shape[1]
    assert np.all(np.abs(f.sum(axis=1)) < n * 1e-10)
    eps = 1e-6
    for i in range(n):
        for ax in range(3):
            p, m = pos.copy(), pos.copy()
            p[ax, i] += eps
            m[ax, i] -= eps
            num = -(total_force(p, atoms, topo)[0] - total_force(m, atoms, topo)[0]) / (2 * eps)
            assert abs(f[ax, i] - num) / (abs(num) + 1.0) < 1e-4


# ------------------------------------------------------------ golden DCD

def test_golden_ala_dipeptide_trajectory(load_fixture):
    """geodesic/tests/golden_reference.rs:27-94: 99 BAB steps at 1 fs, T = 1,
    tolerance 1e-8, H bonds constrained.  The golden file is byte-exact only
    with the x86_64 Windows libm; here every float32 coordinate must agree
    within 2 ulp (atan2/acos/cos/sin may differ by one FP64 ulp between libms)."""
    atoms, topo, state = load_fixture("ala_dipeptide")
    with open(os.path.join(GOLDEN, "ala_dipeptide_ref_header.json")) as f:
        hdr = json.load(f)
    golden = np.load(os.path.join(GOLDEN, "ala_dipeptide_ref_frames.npy"))
    assert hdr["nset"] == 100 and golden.shape == (100, 3, 22)
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = oracle.make_params(box=(1000.0,) * 3, periodic=False, r_cutoff=12.0, r_skin=14.0, r_switch=10.0,
                           max_constr_iter=100, constr_tol=1e-8, n_threads=1)
    frames, pot, kin = oracle.run(atoms, topo, p, np.ascontiguousarray(state.pos), np.ascontiguousarray(state.vel),
                                  0.001, 99, 1)
    assert frames.shape == golden.shape
    ulp = np.abs(frames.view(np.int32).astype(np.int64) - golden.view(np.int32).astype(np.int64))
    assert ulp.max() <= 2, f"max float32 ulp difference {ulp.max()}"
