"""Convert the reference's committed advection_2d golden HDF5 outputs into
small .npz fixtures (level, i, j, u per leaf cell, in the files' cell order),
with SHA-256 digests of the files' /mesh/points and /mesh/connectivity and
the text of their .xdmf companions, so that the output of samurai::save can be
compared with the reference's files byte for byte without shipping them.

The reference's own pytest compares these files dataset by dataset
(tests/conftest.py:26-194 of hpc-maths/samurai); they are produced by
demos/FiniteVolume/advection_2d.cpp run with --Tf 0.01
(tests/test_demo_finite_volume.py:55-72).  h5py is not available here, so the
few HDF5 structures those files use (superblock v0, v1 object headers, v1
B-tree group nodes, local heaps, contiguous layout) are decoded by hand.

Run once where a checkout of the reference tree is available, giving its root:
    python tests/golden/make_golden.py <path to the samurai checkout>
"""
import hashlib
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from advection_cases import save_mesh_arrays  # noqa: E402
from h5lite import H5  # noqa: E402

NAMES = [
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_0_init",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_0",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_1_init",
    "test_finite_volume_advection_2d_finite-volume-advection-2d-0.01_pred_1",
]


def convert(src_dir, name, out_dir):
    h = H5(os.path.join(src_dir, name + ".h5"))
    pts = h.read("/mesh/points")
    conn = h.read("/mesh/connectivity").astype(np.int64)
    u = h.read("/mesh/fields/u").astype(np.float64)
    p0 = pts[conn[:, 0]]
    p2 = pts[conn[:, 2]]
    length = p2[:, 0] - p0[:, 0]
    level = np.rint(-np.log2(length)).astype(np.int8)
    scale = np.ldexp(1.0, level.astype(np.int64))
    i = np.rint(p0[:, 0] * scale).astype(np.int32)
    j = np.rint(p0[:, 1] * scale).astype(np.int32)
    # corners must be exact dyadic numbers
    assert np.all(i / scale == p0[:, 0]) and np.all(j / scale == p0[:, 1])
    # the restatement of samurai::save's point numbering reproduces the file
    rp, rc = save_mesh_arrays(level, np.stack([i, j], axis=1), 10)
    assert np.array_equal(rp, pts) and np.array_equal(rc, h.read("/mesh/connectivity"))
    pts_sha = hashlib.sha256(np.ascontiguousarray(pts, "<f8").tobytes()).hexdigest()
    conn_sha = hashlib.sha256(np.ascontiguousarray(h.read("/mesh/connectivity"), "<u8").tobytes()).hexdigest()
    xdmf = open(os.path.join(src_dir, name + ".xdmf")).read()
    np.savez_compressed(os.path.join(out_dir, name.split("2d-0.01_")[1] + ".npz"), level=level, i=i, j=j, u=u,
                        points_sha256=pts_sha, connectivity_sha256=conn_sha, n_points=len(pts), xdmf=xdmf, file_name=name)
    return len(u)


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <root of the samurai checkout>")
    ref = sys.argv[1]
    src = os.path.join(ref, "tests", "reference", "finite_volume")
    out = os.path.dirname(os.path.abspath(__file__))
    for name in NAMES:
        n = convert(src, name, out)
        print(name, n, "cells")


if __name__ == "__main__":
    main()
