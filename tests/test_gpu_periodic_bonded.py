"""Nearest-image bonded, 1-4 and constraint terms (`bonded_min_image`) on the
device against the oracle (needs a GPU), on the system of
tests/test_periodic_bonded.py wrapped atom by atom so that it is split across
every face of a 40 A periodic box:

* list and forces: the oracle's pair set; FP64 forces within 1e-10 per
  component (relative, floor 1), mixed within 1e-5 relative L2; energy alike;
* drift + SHAKE + resync and RATTLE: the oracle's exact bits (single and star
  clusters);
* 20 resident BAB steps through the faces: positions within 1e-9 A (FP64) or
  1e-5 A (mixed) of the oracle's run, compared at the nearest image;
* the SHAKE warm start refuses the option (its features use raw differences)."""
import numpy as np
import pytest

from geodesic_cuda import backend

import oracle
from test_periodic_bonded import BOX, image_diff, params, system

pytestmark = pytest.mark.gpu

BOXES = (BOX,) * 3


def gparams(precision):
    return backend.SimParams(precision=precision, box_size=BOXES, periodic=True, r_cutoff=10.0, r_skin=11.0,
                             r_switch=8.0, max_constr_iter=200, constr_tol=1e-10, coulomb=True, scale14_lj=0.5,
                             scale14_coul=1 / 1.2, bonded_min_image=True)


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_split_system_forces_match_oracle(precision):
    atoms, topo, _, split, _ = system()
    be = backend.CudaBackend(atoms, topo, gparams(precision))
    ob = oracle.CpuBackend(atoms, topo, params(True))
    pg, pr = split.copy(), split.copy()
    be.build_neighbor_list(pg)
    ob.build_neighbor_list(pr)
    (gi, gj), (ri, rj) = be.pairs(), ob.pairs()
    assert np.array_equal(gi, ri) and np.array_equal(gj, rj)
    fg = be.compute_forces(pg).copy()
    fr = ob.compute_forces(pr)
    eg, er = be.potential_energy(), ob.potential_energy
    be.close()
    erel = abs(eg - er) / abs(er)
    if precision == backend.PRECISION_FP64:
        assert np.all(np.abs(fg - fr) <= 1e-10 * np.maximum(np.abs(fr), 1.0))
        assert erel <= 1e-10, erel
    else:
        assert np.linalg.norm(fg - fr) / np.linalg.norm(fr) <= 1e-5
        assert erel <= 1e-5, erel


def test_split_system_constraints_bit_exact():
    atoms, topo, _, split, vel = system()
    be = backend.CudaBackend(atoms, topo, gparams(backend.PRECISION_FP64))
    pg, pr = split.copy(), split.copy()
    vg, vr = vel.copy(), vel.copy()
    be.geodesic_drift(pg, vg, 0.002, step=3)
    oracle.drift_and_constrain(pr, vr, topo, atoms, 0.002, 200, 1e-10, 3, box=BOXES)
    assert np.array_equal(pg.view(np.uint64), pr.view(np.uint64))
    assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64))
    be.constrain_velocities(pg, vg, step=3)
    oracle.constrain_velocities(topo, atoms, pr, vr, 200, 1e-10, 3, box=BOXES)
    be.close()
    assert np.array_equal(vg.view(np.uint64), vr.view(np.uint64))


@pytest.mark.parametrize("precision", [backend.PRECISION_MIXED, backend.PRECISION_FP64])
def test_resident_steps_through_the_faces_follow_oracle(precision):
    atoms, topo, _, split, vel = system()
    be = backend.CudaBackend(atoms, topo, gparams(precision))
    pg, vg = split.copy(), vel.copy()
    be.constrain_velocities(pg, vg, 0)  # the run loop's initial projection (lib.rs:270-282)
    be.steps(pg, vg, 0.002, 20)
    be.close()
    pr, vr = split.copy(), vel.copy()
    oracle.run(atoms, topo, params(True), pr, vr, 0.002, 20, 20)
    tol = 1e-9 if precision == backend.PRECISION_FP64 else 1e-5
    assert np.abs(image_diff(pg, pr)).max() < tol


def test_warm_start_refuses_the_option():
    atoms, topo, _, _, _ = system()
    be = backend.CudaBackend(atoms, topo, gparams(backend.PRECISION_MIXED))
    with pytest.raises(backend.BackendError) as e:
        be.ws_record(10)
    be.close()
    assert e.value.status == 8  # GM_ERR_UNSUPPORTED
