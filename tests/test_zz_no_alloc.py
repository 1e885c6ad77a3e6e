"""gm_build_pairs_static, the allocation-free list build, against the
context's list build (gm_build_list + gm_get_pairs) through the C ABI.

Pair lists are integer data, so the tolerance is exact equality: the same
pairs in the same order (i, then j), and the same wrapped positions.  Each
case calls the static build twice in a row on the same buffers, so leftovers
in its scratch would show up on the second call, and checks that a warm call
leaves the device's free memory unchanged (it allocates nothing) and gives
back the caller's current device.  The module name sorts last so that, in a
full run, it also runs after every other GPU test.
"""
import ctypes as C

import numpy as np
import pytest

from geodesic_cuda import amber, backend, synth

MAX_ATOMS = 16384  # GM_STATIC_MAX_ATOMS


def exclusion_csr(topo, n):
    """Exclusions as a symmetric CSR with ascending rows (self pairs dropped)."""
    rows = [set() for _ in range(n)]
    for i, j in zip(np.asarray(topo.excl_i, np.int64), np.asarray(topo.excl_j, np.int64)):
        if i != j:
            rows[i].add(int(j))
            rows[j].add(int(i))
    start = np.zeros(n + 1, np.int32)
    flat = []
    for i, r in enumerate(rows):
        flat.extend(sorted(r))
        start[i + 1] = len(flat)
    return start, np.asarray(flat, np.int32)


def gas(n, box, seed):
    """n unit LJ atoms scattered over a periodic box, some outside it."""
    rng = np.random.default_rng(seed)
    pos = np.ascontiguousarray(rng.uniform(-0.25 * box, 1.25 * box, (3, n)))
    atoms = amber.AtomData(np.full(n, 3.0), np.full(n, 0.1), np.ones(n), np.zeros(n), np.ones(n, np.uint8),
                           np.zeros(n, np.uint32), ["C   "] * n)
    return atoms, amber.BondedTopology.empty(), pos


def lattice(n, seed):
    atoms, topo, state, _ = synth.generate(n, seed=seed)
    return atoms, topo, np.ascontiguousarray(state.pos)


CASES = {
    # bonded lattice system, non-periodic 1000 A box, exclusions from the topology
    "lattice_5k_open": (lambda: lattice(5000, 101),
                        dict(box_size=(1000.0,) * 3, periodic=False, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)),
    # periodic gas: 6 cells per axis, positions wrapped by the build
    "gas_3k_periodic": (lambda: gas(3000, 40.0, 7),
                        dict(box_size=(40.0, 40.0, 40.0), periodic=True, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)),
    # periodic box with fewer than 5 cells per axis (whole axes searched)
    "gas_500_small_box": (lambda: gas(500, 20.0, 8),
                          dict(box_size=(20.0, 20.0, 20.0), periodic=True, r_cutoff=7.0, r_skin=9.0, r_switch=5.0)),
}


def test_rejects_sizes_beyond_the_static_limit():
    """Checked before any device call, so this runs without a GPU."""
    p = backend.SimParams(box_size=(100.0,) * 3, periodic=True, r_cutoff=10.0, r_skin=12.0, r_switch=8.0)
    with pytest.raises(backend.BackendError) as e:
        backend.build_pairs_static(None, MAX_ATOMS + 1, None, None, p, None, None, 0)
    assert e.value.status == 8  # GM_ERR_UNSUPPORTED
    with pytest.raises(backend.BackendError) as e:
        backend.build_pairs_static(None, -1, None, None, p, None, None, 0)
    assert e.value.status == 1
    L = backend.lib()
    assert L.gm_build_pairs_static(None, 10, None, None, C.byref(p.to_c()), None, None, 0, None, None) == 1


@pytest.mark.gpu
@pytest.mark.parametrize("case", sorted(CASES))
def test_static_build_matches_context_build(case):
    torch = pytest.importorskip("torch")
    make, kw = CASES[case]
    atoms, topo, pos = make()
    n = pos.shape[1]
    p = backend.SimParams(**kw)

    # the existing entry point: a context, its list build and gm_get_pairs
    be = backend.CudaBackend(atoms, topo, p)
    pos_ctx = pos.copy()
    be.build_neighbor_list(pos_ctx)
    ref_i, ref_j = be.pairs()
    assert len(ref_i) > 0

    dev = torch.device("cuda", p.device)
    d_pos = torch.from_numpy(pos.copy()).to(dev)
    if len(topo.excl_i):
        es, ex = exclusion_csr(topo, n)
        d_es, d_ex = torch.from_numpy(es).to(dev), torch.from_numpy(ex).to(dev)
        es_ptr, ex_ptr = d_es.data_ptr(), d_ex.data_ptr()
    else:
        es_ptr = ex_ptr = None
    stream = torch.cuda.current_stream(dev).cuda_stream

    # count only, then the list twice in a row into sentinel-filled buffers
    total = backend.build_pairs_static(d_pos.data_ptr(), n, es_ptr, ex_ptr, p, None, None, 0, stream)
    assert total == len(ref_i)
    d_i = torch.empty(total + 64, dtype=torch.int32, device=dev)
    d_j = torch.empty(total + 64, dtype=torch.int32, device=dev)
    for call in range(2):
        d_i.fill_(-1)
        d_j.fill_(-1)
        got = backend.build_pairs_static(d_pos.data_ptr(), n, es_ptr, ex_ptr, p, d_i.data_ptr(), d_j.data_ptr(),
                                         total + 64, stream)
        torch.cuda.synchronize(dev)
        assert got == total, (call, got, total)
        gi = d_i.cpu().numpy().view(np.uint32)
        gj = d_j.cpu().numpy().view(np.uint32)
        assert np.array_equal(gi[:total], ref_i), call
        assert np.array_equal(gj[:total], ref_j), call
        assert np.all(gi[total:] == np.uint32(0xFFFFFFFF)), call  # nothing past the count
        # positions wrapped in place exactly as the context's build wraps them
        assert np.array_equal(d_pos.cpu().numpy(), pos_ctx), call

    # a warm call allocates nothing: the device's free memory is the same
    # before and after it (no tensor is created in between)
    torch.cuda.synchronize(dev)
    cur = torch.cuda.current_device()
    free0, _ = torch.cuda.mem_get_info(dev)
    got = backend.build_pairs_static(d_pos.data_ptr(), n, es_ptr, ex_ptr, p, d_i.data_ptr(), d_j.data_ptr(),
                                     total + 64, stream)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert got == total and free1 == free0, (free0, free1)
    assert torch.cuda.current_device() == cur

    # a non-finite position: an error, and the pair buffers untouched
    d_i.fill_(-1)
    d_j.fill_(-1)
    bad = d_pos.clone()
    bad[0, n // 2] = float("nan")
    with pytest.raises(backend.BackendError) as e:
        backend.build_pairs_static(bad.data_ptr(), n, es_ptr, ex_ptr, p, d_i.data_ptr(), d_j.data_ptr(),
                                   total + 64, stream)
    assert e.value.status == 6  # GM_ERR_NONFINITE
    torch.cuda.synchronize(dev)
    assert np.all(d_i.cpu().numpy() == -1) and np.all(d_j.cpu().numpy() == -1)

    # a capacity one short: nothing written, the count reported
    d_i.fill_(-1)
    with pytest.raises(backend.BackendError) as e:
        backend.build_pairs_static(d_pos.data_ptr(), n, es_ptr, ex_ptr, p, d_i.data_ptr(), d_j.data_ptr(),
                                   total - 1, stream)
    assert e.value.status == 7 and e.value.n_pairs == total
    torch.cuda.synchronize(dev)
    assert np.all(d_i.cpu().numpy() == -1)
