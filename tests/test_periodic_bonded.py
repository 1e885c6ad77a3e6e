"""Nearest-image bonded, 1-4 and constraint terms (`bonded_min_image`, beyond
the reference) on the oracle (CPU only).

With `periodic`, the reference wraps every atom into the box at each list
build (neighbor.rs:8-16) but keeps the bonded and constraint differences raw
(memory.md:140-144), so a molecule that the wrap splits across a face gets
bonds one box long.  With the option, those differences take the reference's
min_image (neighbor.rs:74-76) too.  On a synthetic molecule (400 atoms, 30 %
H, H bonds constrained, about 20 A across) in a 40 A box:

* centred in the box, every term is the same bits with and without the option;
* wrapped atom by atom (split across every face), the terms with the option
  equal those of the whole molecule to rounding, and without it they do not;
* a periodic run started split across the faces follows the run of the
  centred copy, shifted by half a box."""
import numpy as np
import pytest

from geodesic_cuda import amber, synth

import oracle

BOX = 40.0
KINDS = ("bond", "angle", "dihedral")


def system(n=400, seed=71, h=0.3):
    atoms, topo, state, _ = synth.generate(n, seed=seed, h_fraction=h, temperature=300.0, relax_iters=200)
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    pos = state.pos - state.pos.mean(axis=1, keepdims=True)  # centred on the origin, a corner of the box
    centred = np.ascontiguousarray(pos + BOX / 2)
    split = np.ascontiguousarray(pos - BOX * np.floor(pos / BOX))  # wrap_coord per atom
    return atoms, topo, centred, split, np.ascontiguousarray(state.vel)


def p14(topo, n):
    return oracle.pairs14(topo, n)


def params(mi, tol=1e-10):
    return oracle.make_params(box=(BOX,) * 3, periodic=True, r_cutoff=10.0, r_skin=11.0, r_switch=8.0,
                              max_constr_iter=200, constr_tol=tol, n_threads=1, coulomb=True, scale14_lj=0.5,
                              scale14_coul=1 / 1.2, bonded_min_image=mi)


def image_diff(a, b):
    d = a - b
    return d - BOX * np.round(d / BOX)


def test_system_is_split_by_the_wrap():
    atoms, topo, centred, split, _ = system()
    extent = centred.max(axis=1) - centred.min(axis=1)
    assert np.all(extent < BOX - 11.0 - 2.0)  # no atom within the list radius of its own image
    whole = np.abs(centred[:, topo.dihed_l] - centred[:, topo.dihed_i])
    assert whole.max() < BOX / 2 - 4.0  # every bonded distance is well below half a box
    d = np.abs(split[:, topo.bond_j] - split[:, topo.bond_i])
    assert (d > BOX / 2).any(axis=0).sum() > 10  # many bonds cross a face after the wrap


def test_option_changes_no_bit_away_from_the_faces():
    atoms, topo, centred, _, vel = system()
    box = (BOX,) * 3
    for kind in KINDS:
        e0, f0 = oracle.bonded_forces(kind, centred, topo)
        e1, f1 = oracle.bonded_forces(kind, centred, topo, box=box)
        assert e0 == e1 and np.array_equal(f0.view(np.uint64), f1.view(np.uint64)), kind
    pi, pj = p14(topo, atoms.n)
    e0, f0 = oracle.pair14_forces(centred, atoms, pi, pj, 0.5, 1 / 1.2, True)
    e1, f1 = oracle.pair14_forces(centred, atoms, pi, pj, 0.5, 1 / 1.2, True, box=box)
    assert e0 == e1 and np.array_equal(f0.view(np.uint64), f1.view(np.uint64))
    pa, va = centred.copy(), vel.copy()
    pb, vb = centred.copy(), vel.copy()
    ia = oracle.drift_and_constrain(pa, va, topo, atoms, 0.002, 200, 1e-10)
    ib = oracle.drift_and_constrain(pb, vb, topo, atoms, 0.002, 200, 1e-10, box=box)
    assert ia == ib and np.array_equal(pa.view(np.uint64), pb.view(np.uint64))
    assert np.array_equal(va.view(np.uint64), vb.view(np.uint64))
    oracle.constrain_velocities(topo, atoms, pa, va, 200, 1e-10)
    oracle.constrain_velocities(topo, atoms, pb, vb, 200, 1e-10, box=box)
    assert np.array_equal(va.view(np.uint64), vb.view(np.uint64))


def test_terms_of_a_split_molecule_equal_the_whole_molecules():
    atoms, topo, centred, split, vel = system()
    box = (BOX,) * 3
    for kind in KINDS:
        e_whole, f_whole = oracle.bonded_forces(kind, centred, topo)
        e_mi, f_mi = oracle.bonded_forces(kind, split, topo, box=box)
        scale = np.abs(f_whole).max()
        assert abs(e_mi - e_whole) <= 1e-9 * abs(e_whole), kind
        assert np.abs(f_mi - f_whole).max() <= 1e-9 * scale, kind
    e_raw, _ = oracle.bonded_forces("bond", split, topo)
    e_whole, _ = oracle.bonded_forces("bond", centred, topo)
    assert e_raw > 1e3 * e_whole  # the reference's raw differences: bonds one box long
    pi, pj = p14(topo, atoms.n)
    e_whole, f_whole = oracle.pair14_forces(centred, atoms, pi, pj, 0.5, 1 / 1.2, True)
    e_mi, f_mi = oracle.pair14_forces(split, atoms, pi, pj, 0.5, 1 / 1.2, True, box=box)
    assert abs(e_mi - e_whole) <= 1e-9 * abs(e_whole)
    assert np.abs(f_mi - f_whole).max() <= 1e-9 * np.abs(f_whole).max()
    # SHAKE and RATTLE: the same iterations, positions equal modulo the box
    pa, va = centred.copy(), vel.copy()
    pb, vb = split.copy(), vel.copy()
    ia = oracle.drift_and_constrain(pa, va, topo, atoms, 0.002, 200, 1e-10)
    ib = oracle.drift_and_constrain(pb, vb, topo, atoms, 0.002, 200, 1e-10, box=box)
    assert ia == ib
    assert np.abs(image_diff(pb, pa - BOX / 2)).max() <= 1e-11
    assert np.abs(vb - va).max() <= 1e-8 * np.abs(va).max()
    oracle.constrain_velocities(topo, atoms, pa, va, 200, 1e-10)
    oracle.constrain_velocities(topo, atoms, pb, vb, 200, 1e-10, box=box)
    assert np.abs(vb - va).max() <= 1e-8 * np.abs(va).max()
    with pytest.raises(oracle.ConvergenceError):
        oracle.drift_and_constrain(split.copy(), vel.copy(), topo, atoms, 0.002, 200, 1e-10)


def test_run_through_the_faces_follows_the_centred_run():
    atoms, topo, centred, split, vel = system()
    pa, va = centred.copy(), vel.copy()
    pb, vb = split.copy(), vel.copy()
    fa, pot_a, kin_a = oracle.run(atoms, topo, params(True), pa, va, 0.002, 20, 5)
    fb, pot_b, kin_b = oracle.run(atoms, topo, params(True), pb, vb, 0.002, 20, 5)
    assert len(fa) == len(fb) == 5
    assert np.abs(image_diff(pb, pa - BOX / 2)).max() <= 1e-9
    assert np.abs(vb - va).max() <= 1e-7 * np.abs(va).max()
    assert np.allclose(pot_b, pot_a, rtol=1e-9, atol=0) and np.allclose(kin_b, kin_a, rtol=1e-9, atol=0)
    # without the option the reference's solver cannot constrain the split bonds
    with pytest.raises(oracle.ConvergenceError):
        oracle.run(atoms, topo, params(False), split.copy(), vel.copy(), 0.002, 20, 5)
