"""The C-ABI library loads on a host without a GPU and exports every entry
point declared in include/geodesic_cuda.h (no compute calls are made)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT
from geodesic_cuda import _build, backend


def declared_symbols():
    with open(os.path.join(ROOT, "include", "geodesic_cuda.h")) as f:
        text = f.read()
    # function declarations: a return type at the start of the line, then the name
    return sorted(set(re.findall(r"^(?:int32_t|gm_ctx \*|void \*)\s*(gm_[a-z_0-9]+)\(", text, re.M)))


@pytest.fixture(scope="module")
def library():
    path = _build.build_cuda()
    return ctypes.CDLL(path)


def test_header_declares_the_trait_surface():
    syms = declared_symbols()
    for name in ("gm_create", "gm_destroy", "gm_build_list", "gm_compute_forces", "gm_needs_rebuild",
                 "gm_geodesic_drift", "gm_half_kick", "gm_constrain_velocities", "gm_steps", "gm_last_error"):
        assert name in syms


def test_every_declared_symbol_is_exported(library):
    missing = [s for s in declared_symbols() if not hasattr(library, s)]
    assert not missing, missing


def test_python_mirror_binds_every_symbol(library):
    L = backend.lib()
    for s in declared_symbols():
        assert hasattr(L, s), s


def test_invalid_parameters_rejected_before_any_device_call(library):
    """config.rs:213-248: r_switch < r_cutoff < r_skin is validated first."""
    import numpy as np
    from geodesic_cuda import amber
    atoms = amber.AtomData(np.ones(2), np.ones(2), np.ones(2), np.zeros(2), np.ones(2, np.uint8),
                           np.zeros(2, np.uint32), ["C   ", "C   "])
    with pytest.raises(backend.BackendError) as e:
        backend.CudaBackend(atoms, amber.BondedTopology.empty(),
                            backend.SimParams(r_cutoff=10.0, r_skin=9.0, r_switch=8.0))
    assert e.value.status == 1


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes mirrors of gm_atoms, gm_topology, gm_params and
    gm_convergence have the header's size and field offsets (gcc on the header)."""
    import subprocess

    structs = {"gm_atoms": backend.GmAtoms, "gm_topology": backend.GmTopology, "gm_params": backend.GmParams,
               "gm_convergence": backend.GmConvergence}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "geodesic_cuda.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'    printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'    printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                             check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[f"{cname} size"]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname} {fname}"]) == getattr(py, fname).offset, (cname, fname)
