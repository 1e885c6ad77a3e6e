"""Regenerates the golden fixtures in this folder from the reference checkout.

Run in a container that has the reference mounted (the GPU host does not):

    python tests/golden/make_fixtures.py /path/to/GEODESIC-M

It parses the reference's four AMBER test systems
(`geodesic-engine/tests/fixtures/{lj_pair,harmonic_dimer,water_box_4,ala_dipeptide}`)
with `geodesic_cuda.amber` (the restatement of `geodesic-io/src/prmtop.rs` and
`inpcrd.rs`) and stores the parsed arrays as `<name>.npz`.  It also decodes the
reference's golden trajectory `geodesic/tests/golden/ala_dipeptide_ref.dcd`
(100 frames, written by `geodesic-io/src/dcd.rs`) into
`ala_dipeptide_ref_frames.npy` (float32, shape (100, 3, 22)) plus the DCD
header fields in `ala_dipeptide_ref_header.json`.
"""
import hashlib
import json
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "geodesic-m_gb300"))
from geodesic_cuda import amber  # noqa: E402

FIXTURES = ["lj_pair", "harmonic_dimer", "water_box_4", "ala_dipeptide"]


def read_dcd(path):
    """Decodes the CHARMM DCD layout that `dcd.rs:94-136` writes."""
    with open(path, "rb") as f:
        data = f.read()
    off = 0

    def rec():
        nonlocal off
        (n,) = struct.unpack_from("<i", data, off)
        body = data[off + 4: off + 4 + n]
        (n2,) = struct.unpack_from("<i", data, off + 4 + n)
        assert n == n2, "record markers differ"
        off += 8 + n
        return body

    hdr = rec()
    assert hdr[:4] == b"CORD"
    icntrl = struct.unpack_from("<20i", hdr, 4)
    delta = struct.unpack_from("<f", hdr, 4 + 9 * 4)[0]
    title = rec()
    natom = struct.unpack("<i", rec())[0]
    frames = []
    while off < len(data):
        xyz = [np.frombuffer(rec(), dtype="<f4") for _ in range(3)]
        frames.append(np.stack(xyz))
    return {"nset": icntrl[0], "istart": icntrl[1], "nsavc": icntrl[2], "namnf": icntrl[8],
            "delta_akma": float(delta), "charmm_version": icntrl[19], "natom": natom,
            "title": title[4:].decode().rstrip()}, np.stack(frames)


def main(ref_root):
    fx = os.path.join(ref_root, "geodesic-engine", "tests", "fixtures")
    for name in FIXTURES:
        atoms, topo, state = amber.load(os.path.join(fx, f"{name}.prmtop"), os.path.join(fx, f"{name}.inpcrd"))
        amber.save_npz(os.path.join(HERE, f"{name}.npz"), atoms, topo, state)
        print(f"{name}: {atoms.n} atoms, {len(topo.bond_i)} bonds, {len(topo.angle_i)} angles, "
              f"{len(topo.dihed_i)} dihedrals, {len(topo.excl_i)} exclusions")
    dcd_path = os.path.join(ref_root, "geodesic", "tests", "golden", "ala_dipeptide_ref.dcd")
    header, frames = read_dcd(dcd_path)
    with open(dcd_path, "rb") as f:
        raw = f.read()
    # the file's identity, so a writer given the decoded frames can be checked byte for byte
    header["file_bytes"] = len(raw)
    header["file_sha256"] = hashlib.sha256(raw).hexdigest()
    np.save(os.path.join(HERE, "ala_dipeptide_ref_frames.npy"), frames.astype(np.float32))
    with open(os.path.join(HERE, "ala_dipeptide_ref_header.json"), "w") as f:
        json.dump(header, f, indent=1)
    print("golden DCD:", header, frames.shape)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_fixtures.py <path of the GEODESIC-M checkout>")
    main(sys.argv[1])
