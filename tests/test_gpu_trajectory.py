"""Trajectory frames recorded on the device during resident steps against the
run loop of geodesic/src/lib.rs:292-331 driven through the trait-level entry
points (needs a GPU).  At every frame step the recorded float32 positions,
kinetic energy and potential energy equal, bit for bit, the loop's
`pos as f32`, `kinetic_energy` and `potential_energy` of the same state;
without and with constraints.  The whole output loop (DCD + energy CSV) runs
end to end."""
import os

import numpy as np
import pytest

from geodesic_cuda import amber, backend, synth, trajectory

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def trait_loop_frames(be, pos, vel, dt, n_steps, every):
    """lib.rs:292-331 through the trait-level calls; frames at step % every == 0."""
    be.build_neighbor_list(pos)
    f = be.compute_forces(pos).copy()
    out = []
    for step in range(n_steps):
        be.half_kick(vel, f, dt / 2.0)
        be.geodesic_drift(pos, vel, dt, step)
        if be.needs_rebuild(pos):
            be.build_neighbor_list(pos)
        f = be.compute_forces(pos).copy()
        e_pot = be.potential_energy()
        be.half_kick(vel, f, dt / 2.0)
        be.constrain_velocities(pos, vel, step)
        if (step + 1) % every == 0:
            out.append((step + 1, pos.astype(np.float32), be.kinetic_energy(vel), e_pot))
    return out


def resident_frames(be, pos, vel, dt, n_steps, every):
    be.frames_enable(every, 64)
    be.upload_state(pos, vel)
    be.forces_resident()
    be.run_resident(dt, n_steps)
    fr = be.frames_take()
    be.frames_enable(0, 0)
    return fr


def check(ref, fr):
    assert len(fr["step"]) == len(ref)
    for k, (step, xyz, e_kin, e_pot) in enumerate(ref):
        assert int(fr["step"][k]) == step
        assert np.array_equal(fr["xyz"][k].view(np.uint32), xyz.view(np.uint32)), step
        assert fr["e_kin"][k] == e_kin, (step, fr["e_kin"][k], e_kin)
        assert fr["e_pot"][k] == e_pot, (step, fr["e_pot"][k], e_pot)


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_frames_without_constraints(precision):
    atoms, topo, state, _ = synth.generate(2000, seed=29, temperature=600.0, relax_iters=200)
    p = backend.SimParams(precision=precision, box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0,
                          r_skin=10.6, r_switch=8.0)
    dt, n, every = 0.002, 40, 5
    res = backend.CudaBackend(atoms, topo, p)
    fr = resident_frames(res, np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.vel.copy()),
                         dt, n, every)
    res.close()
    be = backend.CudaBackend(atoms, topo, p)
    ref = trait_loop_frames(be, np.ascontiguousarray(state.pos.copy()), np.ascontiguousarray(state.vel.copy()),
                            dt, n, every)
    be.close()
    check(ref, fr)


def test_frames_with_constraints(load_fixture):
    atoms, topo, state = load_fixture("ala_dipeptide")
    topo = amber.promote_hydrogen_bonds(topo, atoms)
    p = backend.SimParams(precision=backend.PRECISION_FP64, box_size=(1000.0,) * 3, periodic=False, r_cutoff=12.0,
                          r_skin=14.0, r_switch=10.0, max_constr_iter=100, constr_tol=1e-8)
    dt, n, every = 0.001, 30, 3
    pos0 = np.ascontiguousarray(state.pos.copy())
    vel0 = np.ascontiguousarray(state.vel.copy())
    pre = backend.CudaBackend(atoms, topo, p)
    pre.constrain_velocities(pos0, vel0, 0)  # the run loop's initial projection (lib.rs:270-282)
    pre.close()
    res = backend.CudaBackend(atoms, topo, p)
    fr = resident_frames(res, pos0.copy(), vel0.copy(), dt, n, every)
    res.close()
    be = backend.CudaBackend(atoms, topo, p)
    ref = trait_loop_frames(be, pos0.copy(), vel0.copy(), dt, n, every)
    be.close()
    check(ref, fr)


def test_run_with_output_writes_dcd_and_csv(tmp_path):
    import sys
    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_fixtures import read_dcd

    atoms, topo, state, _ = synth.generate(1500, seed=31, relax_iters=200)
    p = backend.SimParams(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)
    be = backend.CudaBackend(atoms, topo, p)
    pos = np.ascontiguousarray(state.pos.copy())
    vel = np.ascontiguousarray(state.vel.copy())
    pos_in = pos.copy()
    n_frames = trajectory.run_with_output(be, pos, vel, 0.002, 100, 10, tmp_path / "t.dcd", tmp_path / "e.csv",
                                          frames_per_batch=3)
    be.close()
    assert n_frames == 11
    header, frames = read_dcd(tmp_path / "t.dcd")
    assert header["nset"] == 11 and header["natom"] == atoms.n and header["nsavc"] == 10
    assert np.array_equal(frames[0], pos_in.astype(np.float32))
    assert np.array_equal(frames[-1], pos.astype(np.float32))  # the final state handed back
    rows = (tmp_path / "e.csv").read_text().splitlines()
    assert len(rows) == 12 and rows[-1].startswith("100,0.200,")
